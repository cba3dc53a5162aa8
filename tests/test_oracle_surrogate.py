"""The FP64 restatement of the surrogate network, pinned by finite differences."""
import numpy as np

from oracle.surrogate import MLPRef, to_bf16


def _net(rng, sizes):
    W = [rng.normal(0, 1 / np.sqrt(c), (r, c)) for c, r in zip(sizes[:-1], sizes[1:])]
    b = [rng.normal(0, 0.1, r) for r in sizes[1:]]
    return W, b


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    W, b = _net(rng, [5, 12, 12, 3])
    x = rng.normal(size=(16, 5))
    t = rng.normal(size=(16, 3))
    net = MLPRef(W, b, bf16=False)
    _, gW, gb = net.loss_and_grads(x, t)
    h = 1e-6
    for l in range(3):
        for _ in range(6):
            r, c = rng.integers(W[l].shape[0]), rng.integers(W[l].shape[1])
            Wp = [w.copy() for w in W]
            Wm = [w.copy() for w in W]
            Wp[l][r, c] += h
            Wm[l][r, c] -= h
            fd = (MLPRef(Wp, b, False).loss_and_grads(x, t)[0] - MLPRef(Wm, b, False).loss_and_grads(x, t)[0]) / (2 * h)
            assert abs(fd - gW[l][r, c]) <= 1e-6 * max(1.0, abs(fd)), (l, r, c)
        k = rng.integers(len(b[l]))
        bp = [v.copy() for v in b]
        bm = [v.copy() for v in b]
        bp[l][k] += h
        bm[l][k] -= h
        fd = (MLPRef(W, bp, False).loss_and_grads(x, t)[0] - MLPRef(W, bm, False).loss_and_grads(x, t)[0]) / (2 * h)
        assert abs(fd - gb[l][k]) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 1e-30])
    r = to_bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0  # a tie rounds to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12
    assert r[4] == 0.0 and r[5] > 0


def test_map_network_restatement_against_finite_differences():
    """The network with the map decoder (MapNetRef) in pure FP64: its loss
    gradients agree with central finite differences for weights and biases of
    dense and decoder layers."""
    from oracle.surrogate import MapNetRef
    rng = np.random.default_rng(21)
    n_in, width, n_out, side, ch = 3, 8, 2, 16, (4, 4, 3)
    s0 = side // 8
    shapes = [(width, n_in), (n_out + s0 * s0 * ch[0], width), (ch[1], 9 * ch[0]), (ch[2], 9 * ch[1]),
              (1, 9 * ch[2])]
    Ws = [rng.normal(0, 0.5, s) for s in shapes]
    bs = [rng.normal(0, 0.1, s[0]) for s in shapes]
    x = rng.uniform(-1, 1, (3, n_in))
    t = rng.normal(0, 1, (3, n_out + side * side))

    def loss(Ws_, bs_):
        return MapNetRef(Ws_, bs_, n_out, side, ch[0], bf16=False).loss_and_grads(x, t)[0]

    _, gW, gb = MapNetRef(Ws, bs, n_out, side, ch[0], bf16=False).loss_and_grads(x, t)
    eps = 1e-6
    for l in range(len(Ws)):
        for idx in [(0, 0), (Ws[l].shape[0] - 1, Ws[l].shape[1] - 1), (0, Ws[l].shape[1] // 2)]:
            Wp = [w.copy() for w in Ws]
            Wm = [w.copy() for w in Ws]
            Wp[l][idx] += eps
            Wm[l][idx] -= eps
            fd = (loss(Wp, bs) - loss(Wm, bs)) / (2 * eps)
            assert abs(fd - gW[l][idx]) <= 1e-6 * max(1.0, abs(fd)), (l, idx, fd, gW[l][idx])
        bp = [b.copy() for b in bs]
        bm = [b.copy() for b in bs]
        bp[l][0] += eps
        bm[l][0] -= eps
        fd = (loss(Ws, bp) - loss(Ws, bm)) / (2 * eps)
        assert abs(fd - gb[l][0]) <= 1e-6 * max(1.0, abs(fd)), (l, fd, gb[l][0])

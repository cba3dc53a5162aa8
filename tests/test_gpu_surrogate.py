"""The surrogate network on the GPU (include/cliffs_surrogate.h) against its
FP64 restatement (oracle/surrogate.py), and the surrogate pipeline end to end.

The restatement passes values through BF16 where the kernels store BF16, so
the comparison measures the kernels' FP32 accumulation and ordering: forward
outputs and every weight and bias gradient agree within 5e-3 of their largest
magnitude (relative), at a small shape and at the production shape
(8 -> 512 x 3 -> 1088).
"""
import importlib

import numpy as np
import pytest

from oracle.surrogate import MapNetRef, MLPRef

pytestmark = pytest.mark.gpu
S = importlib.import_module("cliffs-src_gb300.surrogate")


def _rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("shape,batch", [((8, 64, 2, 40), 64), ((8, 512, 3, 1088), 128)])
def test_forward_and_gradients_against_oracle(shape, batch):
    n_in, width, depth, n_out = shape
    net = S.MLP(n_in, width, depth, n_out, seed=11)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (batch, n_in)).astype(np.float32)
    t = rng.normal(size=(batch, n_out)).astype(np.float32)
    Ws, bs = net.weights()
    # non-zero biases so that they are exercised
    bs = [rng.normal(0, 0.05, b.shape).astype(np.float32) for b in bs]
    for l, b in enumerate(bs):
        net.set(l, 1, b)
    ref = MLPRef(Ws, bs, bf16=True)
    y = net.predict(x)
    yr = ref.forward(x.astype(np.float64))[-1]
    assert _rel(y, yr) <= 5e-3
    loss, gW, gb = net.gradients(x, t)
    lr, rW, rb = ref.loss_and_grads(x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - lr) <= 1e-3 * lr
    for l in range(depth + 1):
        assert _rel(gW[l], rW[l]) <= 5e-3, l
        assert _rel(gb[l], rb[l]) <= 5e-3, l
    net.close()


@pytest.mark.parametrize("side,ch,batch", [(32, (16, 8, 8), 32), (128, (32, 16, 8), 16)])
def test_map_decoder_against_oracle(side, ch, batch):
    """The network with the conv map decoder: the dense outputs, the map and
    every gradient (dense layers and decoder levels) against the FP64
    restatement with the same BF16 roundings, within 5e-3 of the largest
    magnitude; at a small shape and at the surrogate's (128 x 128 map)."""
    n_in, width, depth, n_out = 9, 128, 2, 16
    net = S.MLP(n_in, width, depth, n_out, seed=13, map_side=side, map_ch=ch)
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (batch, n_in)).astype(np.float32)
    t = rng.normal(0, 0.5, (batch, n_out + side * side)).astype(np.float32)
    n_layers = net.layers()
    assert n_layers == depth + 1 + 3
    Ws, bs = net.weights()
    bs = [rng.normal(0, 0.05, b.shape).astype(np.float32) for b in bs]
    for l, b in enumerate(bs):
        net.set(l, 1, b)
    ref = MapNetRef(Ws, bs, n_out, side, ch[0], bf16=True)
    y = net.predict(x)
    yr = ref.forward(x.astype(np.float64))[-1]
    assert _rel(y[:, :n_out], yr[:, :n_out]) <= 5e-3
    assert _rel(y[:, n_out:], yr[:, n_out:]) <= 5e-3
    loss, gW, gb = net.gradients(x, t)
    lr, rW, rb = ref.loss_and_grads(x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - lr) <= 1e-3 * lr
    for l in range(n_layers):
        assert _rel(gW[l], rW[l]) <= 5e-3, (l, _rel(gW[l], rW[l]))
        assert _rel(gb[l], rb[l]) <= 5e-3, (l, _rel(gb[l], rb[l]))
    net.close()


def test_training_reduces_loss_and_is_deterministic():
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (1024, 8)).astype(np.float32)
    A = rng.normal(size=(8, 24))
    t = np.sin(x @ A).astype(np.float32)
    losses = []
    finals = []
    for rep in range(2):
        net = S.MLP(8, 128, 2, 24, seed=7)
        l = net.train(x, t, epochs=200, batch=128, lr=2e-3, seed=9)
        losses.append(l)
        finals.append(net.predict(x))
        net.close()
    assert losses[0][-1] < 0.1 * losses[0][0]
    assert np.array_equal(losses[0], losses[1])
    assert np.array_equal(finals[0], finals[1])


def test_parameters_round_trip():
    net = S.MLP(5, 32, 1, 7, seed=1)
    assert net.layers() == 2 and net.shape(0) == (32, 5) and net.shape(1) == (7, 32)
    w = np.arange(32 * 5, dtype=np.float32).reshape(32, 5) / 100
    net.set(0, 0, w)
    assert np.array_equal(net.get(0, 0), w)
    net.close()


def test_pipeline_small():
    r = S.run(n_train=96, n_test=16, steps=150, epochs=10, target=0.5, seed=1, n_val=32, map_epochs=5, infer_batch=64)
    assert r["nonfinite_runs"] == 0
    assert r["accepted"] + r["fallback"] == 16
    assert np.isfinite(r["gauge_rel_err_all_mean"])
    assert r["surrogate_scenarios_per_s"] > r["one_at_a_time_scenarios_per_s"]
    # the 128 x 128 inundation maps of the conv decoder are judged too
    assert r["map"] == [128, 128] and np.isfinite(r["map_abs_err_mean_m"]) and 0.0 <= r["map_iou_mean"] <= 1.0

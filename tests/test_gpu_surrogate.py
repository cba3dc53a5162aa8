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

from oracle.surrogate import MLPRef

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
    r = S.run(n_train=96, n_test=16, steps=150, epochs=10, target=0.5, seed=1, n_val=32)
    assert r["nonfinite_runs"] == 0
    assert r["accepted"] + r["fallback"] == 16
    assert np.isfinite(r["gauge_rel_err_all_mean"])
    assert r["surrogate_scenarios_per_s"] > r["one_at_a_time_scenarios_per_s"]

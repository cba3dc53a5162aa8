"""FP64 restatement of the surrogate network (TEST INFRASTRUCTURE ONLY).

The ReLU multilayer perceptron of include/cliffs_surrogate.h in numpy FP64:
forward, mean-squared-error loss and backward.  With bf16=True the values
pass through BF16 at the points where the GPU kernels store BF16: the inputs,
the weights, every hidden activation, and every layer's output gradient
before the two matrix products that read it.  Accumulation stays FP64, so
the GPU's FP32 accumulation is what a comparison measures.  The restatement
itself is pinned by central finite differences in pure FP64
(tests/test_oracle_surrogate.py).
"""
import numpy as np


def to_bf16(a):
    """Round to the nearest BF16 (ties to even), returned as FP64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


class MLPRef:
    """weights[l]: (rows, cols), biases[l]: (rows,); layers 0..depth, ReLU on all but the last."""

    def __init__(self, weights, biases, bf16=True):
        self.W = [np.asarray(w, np.float64) for w in weights]
        self.b = [np.asarray(b, np.float64) for b in biases]
        self.bf16 = bf16

    def _r(self, a):
        return to_bf16(a) if self.bf16 else np.asarray(a, np.float64)

    def forward(self, x):
        H = [self._r(x)]
        for l, (w, b) in enumerate(zip(self.W, self.b)):
            z = H[-1] @ self._r(w).T + b
            if l < len(self.W) - 1:
                H.append(self._r(np.maximum(z, 0.0)))
            else:
                H.append(z)
        return H

    def loss_and_grads(self, x, t):
        H = self.forward(x)
        y = H[-1]
        B, n = y.shape
        loss = float(np.mean((y - t) ** 2))
        dy = 2.0 * (y - t) / (B * n)
        gW, gb = [None] * len(self.W), [None] * len(self.W)
        for l in range(len(self.W) - 1, -1, -1):
            if l < len(self.W) - 1:
                dy = dy * (H[l + 1] > 0)
            gb[l] = dy.sum(axis=0)
            dyr = self._r(dy)
            gW[l] = dyr.T @ H[l]
            if l > 0:
                dy = dyr @ self._r(self.W[l])
        return loss, gW, gb

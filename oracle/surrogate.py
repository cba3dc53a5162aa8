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
        gW, gb = self.backward(H, dy)
        return loss, gW, gb

    def backward(self, H, dy):
        """Weight and bias gradients for the output gradient dy."""
        gW, gb = [None] * len(self.W), [None] * len(self.W)
        for l in range(len(self.W) - 1, -1, -1):
            if l < len(self.W) - 1:
                dy = dy * (H[l + 1] > 0)
            gb[l] = dy.sum(axis=0)
            dyr = self._r(dy)
            gW[l] = dyr.T @ H[l]
            if l > 0:
                dy = dyr @ self._r(self.W[l])
        return gW, gb


# -- the map decoder -----------------------------------------------------------

def up2(x):
    """Nearest-neighbour 2x upsampling of (B, S, S, C)."""
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def conv3(u, w):
    """3x3 convolution with zero padding: u (B, S, S, Cin), w (Cout, 3, 3, Cin)
    -> (B, S, S, Cout); z[b,y,x,o] = sum over dy, dx in -1..1 and c of
    u[b, y+dy, x+dx, c] w[o, dy+1, dx+1, c]."""
    B, S, _, C = u.shape
    p = np.zeros((B, S + 2, S + 2, C))
    p[:, 1:-1, 1:-1] = u
    z = np.zeros((B, S, S, w.shape[0]))
    for ty in range(3):
        for tx in range(3):
            z += np.einsum("byxc,oc->byxo", p[:, ty:ty + S, tx:tx + S], w[:, ty, tx, :])
    return z


class DecoderRef:
    """The map decoder of include/cliffs_surrogate.h in FP64: a latent grid
    (B, S0, S0, C0) passes a ReLU, then each level upsamples by 2 (nearest)
    and applies a 3x3 convolution with zero padding and a bias; every level
    but the last applies a ReLU.  With bf16=True the values pass through BF16
    where the GPU stores BF16: the decoder's input after its ReLU, every
    level's weights and output activations, and every level's output
    gradient before the two products that read it.
    weights[l]: (Cout, 3, 3, Cin), biases[l]: (Cout,)."""

    def __init__(self, weights, biases, bf16=True):
        self.W = [np.asarray(w, np.float64) for w in weights]
        self.b = [np.asarray(b, np.float64) for b in biases]
        self.bf16 = bf16

    def _r(self, a):
        return to_bf16(a) if self.bf16 else np.asarray(a, np.float64)

    def forward(self, latent):
        X = [self._r(np.maximum(latent, 0.0))]
        for l, (w, b) in enumerate(zip(self.W, self.b)):
            z = conv3(up2(X[-1]), self._r(w)) + b
            X.append(self._r(np.maximum(z, 0.0)) if l < len(self.W) - 1 else z)
        return X

    def backward(self, X, dout, latent):
        """Gradients of the weights, biases and the latent for the output
        gradient dout (B, S, S, 1)."""
        nl = len(self.W)
        gW, gb = [None] * nl, [None] * nl
        dz = dout
        for l in range(nl - 1, -1, -1):
            if l < nl - 1:
                dz = dz * (X[l + 1] > 0)
            gb[l] = dz.sum(axis=(0, 1, 2))
            dzr = self._r(dz)
            u = up2(X[l])
            B, S, _, C = u.shape
            p = np.zeros((B, S + 2, S + 2, C))
            p[:, 1:-1, 1:-1] = u
            g = np.zeros_like(self.W[l])
            du = np.zeros((B, S + 2, S + 2, C))
            wr = self._r(self.W[l])
            for ty in range(3):
                for tx in range(3):
                    g[:, ty, tx, :] = np.einsum("byxo,byxc->oc", dzr, p[:, ty:ty + S, tx:tx + S])
                    du[:, ty:ty + S, tx:tx + S] += np.einsum("byxo,oc->byxc", dzr, wr[:, ty, tx, :])
            gW[l] = g
            du = du[:, 1:-1, 1:-1]
            dz = du.reshape(B, S // 2, 2, S // 2, 2, C).sum(axis=(2, 4))
        dlatent = dz * (latent > 0)
        return gW, gb, dlatent


class MapNetRef:
    """The whole network with a map decoder: MLPRef layers whose last layer
    emits n_out dense values and the latent grid (side/8)^2 x C0 (NHWC), then
    DecoderRef.  Loss: mean squared error over the dense outputs plus that
    over the map cells; targets (B, n_out + side^2)."""

    def __init__(self, weights, biases, n_out, side, c0, bf16=True):
        nd = len(weights) - 3
        self.mlp = MLPRef(weights[:nd], biases[:nd], bf16)
        dec_w = [np.asarray(w, np.float64).reshape(w.shape[0], 3, 3, -1) for w in weights[nd:]]
        self.dec = DecoderRef(dec_w, biases[nd:], bf16)
        self.n_out, self.side, self.c0, self.s0 = n_out, side, c0, side // 8

    def forward(self, x):
        H = self.mlp.forward(x)
        y = H[-1]
        lat = y[:, self.n_out:].reshape(len(x), self.s0, self.s0, self.c0)
        X = self.dec.forward(lat)
        return H, lat, X, np.hstack([y[:, :self.n_out], X[-1].reshape(len(x), -1)])

    def loss_and_grads(self, x, t):
        H, lat, X, out = self.forward(x)
        B = len(x)
        n, m = self.n_out, self.side * self.side
        d = out - t
        loss = float(np.mean(d[:, :n] ** 2) + np.mean(d[:, n:] ** 2))
        dmap = (2.0 * d[:, n:] / (B * m)).reshape(B, self.side, self.side, 1)
        gWd, gbd, dlat = self.dec.backward(X, dmap, lat)
        dy = np.hstack([2.0 * d[:, :n] / (B * n), dlat.reshape(B, -1)])
        gW, gb = self.mlp.backward(H, dy)
        return loss, gW + [g.reshape(g.shape[0], -1) for g in gWd], gb + list(gbd)

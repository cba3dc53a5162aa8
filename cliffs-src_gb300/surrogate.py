"""A learned surrogate of the solver for source studies (include/cliffs_surrogate.h).

The surrogate maps eight source parameters to the quantities a hazard study
reads from a run: the maximum elevation at 64 gauges and the maximum
inundation depth (the largest flow depth over ground, MaxE + dep on land,
0 where the sea never reached) over a 128 x 128 window of the coast.

- Gauges: an ensemble of 4-layer MLPs (9 features -> 3 x 512 ReLU -> 64),
  trained from different seeds.  Their mean is the prediction, their
  disagreement the gate.
- Map: an MLP of the same shape whose last layer also emits a latent
  16 x 16 x 32 grid, which a conv decoder (three 2x upsampling + 3x3
  convolution levels) turns into the 128 x 128 map; the mean of the map
  members is the prediction.

The training data are runs of the batched solver (cliffs_batch_*) on one
512 x 512 shelf/slope grid at 100 m, every source applied on the device
(cliffs_gpu_add_source, rising over its rise time); the networks are
trained on the GPU by the library's own kernels (BF16 tensor-core products
on tcgen05 with FP32 accumulation in tensor memory, direct convolutions for
the decoder's narrow levels, Adam).  Where the gauge members disagree by
more than a relative spread, the scenario goes back to the solver.  The
spread threshold is calibrated on a validation split of the training runs
as the largest that keeps the accepted scenarios' mean gauge error within
the target; the solver then judges the surrogate's error on held-out
scenarios.

    python cliffs-src_gb300/surrogate.py [--train 4096] [--test 256] [--steps 2000]
                                         [--epochs 3000] [--map-epochs 600] [--map-members 1]
                                         [--target 0.045]

prints one JSON line: data generation time, training losses, accuracy of the
gated ensemble against the solver, and scenarios per second of the surrogate
path against one-at-a-time solves.

    python cliffs-src_gb300/surrogate.py --infer 4096

times the networks' inference alone (untrained weights, no data): the
4 gauge networks and the map network on 4096 fresh parameter sets, twice.
"""
import argparse
import ctypes
import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
pkg = importlib.import_module("cliffs-src_gb300")
cg = pkg.cliffs_gpu
W = pkg.workloads

SIDE = 512
DX = 100.0
NGAUGES = 64
WIN = (slice(192, 320), slice(SIDE - 128, SIDE))  # rows, columns of the coastal window
MAP = 128                 # the window's side: the decoder's map
MAP_CH = (32, 16, 8)      # decoder channels: latent 16 x 16 x 32, levels of 16 and 8
# parameter ranges, as fractions of the domain length where spatial
LO = np.array([0.15, 0.20, 0.5, 0.05, 0.05, 0.0, 0.0, 0.0])
HI = np.array([0.50, 0.80, 3.0, 0.20, 0.20, np.pi, 0.6, 60.0])
NAMES = ["x0", "y0", "amp", "ax", "ay", "angle", "dipole", "rise_time"]


class MlpDesc(ctypes.Structure):
    _fields_ = [("n_in", ctypes.c_int32), ("width", ctypes.c_int32), ("depth", ctypes.c_int32),
                ("n_out", ctypes.c_int32), ("seed", ctypes.c_uint64), ("map_side", ctypes.c_int32),
                ("map_ch", ctypes.c_int32 * 3)]


_fp = ctypes.POINTER(ctypes.c_float)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """One network (cliffs_mlp_*): n_out dense outputs and, with map_side > 0,
    a map_side x map_side map from the conv decoder (channels map_ch)."""

    def __init__(self, n_in, width, depth, n_out, seed=0, map_side=0, map_ch=(32, 16, 8)):
        self.L = cg.load()
        d = MlpDesc(n_in, width, depth, n_out, seed, map_side, (ctypes.c_int32 * 3)(*map_ch))
        h = ctypes.c_void_p()
        cg._chk(self.L.cliffs_mlp_create(ctypes.byref(d), ctypes.byref(h)), "mlp_create")
        self.h = h
        self.n_in, self.n_out = n_in, n_out
        self.map_side = map_side
        self.n_y = n_out + map_side * map_side

    def close(self):
        if getattr(self, "h", None):
            self.L.cliffs_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layers(self):
        n = ctypes.c_int32()
        cg._chk(self.L.cliffs_mlp_layers(self.h, ctypes.byref(n)), "mlp_layers")
        return n.value

    def shape(self, layer):
        r, c = ctypes.c_int32(), ctypes.c_int32()
        cg._chk(self.L.cliffs_mlp_shape(self.h, layer, ctypes.byref(r), ctypes.byref(c)), "mlp_shape")
        return r.value, c.value

    def get(self, layer, which):
        r, c = self.shape(layer)
        a = np.zeros((r, c) if which in (0, 2) else (r,), np.float32)
        cg._chk(self.L.cliffs_mlp_get(self.h, layer, which, a.ctypes.data_as(_fp), a.size), "mlp_get")
        return a

    def set(self, layer, which, a):
        a = _f32(a)
        cg._chk(self.L.cliffs_mlp_set(self.h, layer, which, a.ctypes.data_as(_fp), a.size), "mlp_set")

    def weights(self):
        n = self.layers()
        return [self.get(l, 0) for l in range(n)], [self.get(l, 1) for l in range(n)]

    def predict(self, x):
        x = _f32(x)
        y = np.zeros((x.shape[0], self.n_y), np.float32)
        cg._chk(self.L.cliffs_mlp_predict(self.h, x.shape[0], x.ctypes.data_as(_fp), y.ctypes.data_as(_fp)),
                "mlp_predict")
        return y

    def gradients(self, x, t):
        x, t = _f32(x), _f32(t)
        loss = ctypes.c_float()
        cg._chk(self.L.cliffs_mlp_gradients(self.h, x.shape[0], x.ctypes.data_as(_fp), t.ctypes.data_as(_fp),
                                            ctypes.byref(loss)), "mlp_gradients")
        n = self.layers()
        return loss.value, [self.get(l, 2) for l in range(n)], [self.get(l, 3) for l in range(n)]

    def train(self, x, t, epochs, batch=512, lr=1e-3, seed=0, weight_decay=0.0):
        x, t = _f32(x), _f32(t)
        losses = np.zeros(epochs, np.float32)
        cg._chk(self.L.cliffs_mlp_train(self.h, x.shape[0], x.ctypes.data_as(_fp), t.ctypes.data_as(_fp),
                                        epochs, batch, lr, weight_decay, seed, losses.ctypes.data_as(_fp)),
                "mlp_train")
        return losses

    def launches(self):
        n = ctypes.c_int64()
        cg._chk(self.L.cliffs_mlp_launch_count(self.h, ctypes.byref(n)), "mlp_launch_count")
        return n.value


# ---- data from the batched solver ------------------------------------------------

def base_grid(seed=0):
    return W.shelf_2d(seed=seed, nx=SIDE, ny=SIDE, dx=DX, steps=0, amp=0.0, ngauges=NGAUGES)


def sample_params(n, seed):
    rng = np.random.default_rng(seed)
    return LO + (HI - LO) * rng.random((n, 8))


def source_of(p, L):
    return dict(x0=p[0] * L, y0=p[1] * L, amp=p[2], ax=p[3] * L, ay=p[4] * L, angle=p[5], dipole=p[6],
                rise_time=p[7])


def targets_of(maxe, I, J, dep):
    """Gauge maxima (64, never-wet gauges count as 0) and the maximum
    inundation depth over the coastal window (128 x 128): MaxE + dep on land
    cells (dep < 0) the sea reached, 0 elsewhere (sea cells, dry land)."""
    m = np.where(maxe > -1e30, maxe, 0.0).astype(np.float64)
    g = np.maximum(m[J - 1, I - 1], 0.0)
    w, d = maxe[WIN].astype(np.float64), dep[WIN]
    inund = np.where((d < 0) & (w > -1e30), np.maximum(w + d, 0.0), 0.0)
    return g, inund


def solve(params, base, steps, chunk=512):
    """Runs of the batched solver; returns gauge maxima, inundation maps,
    the solver time (s) and the number of runs with a non-finite state."""
    L = base["xcrd"][-1]
    I, J = base["gauges"]
    dep = base["dep"].astype(np.float32).astype(np.float64)
    G, M = [], []
    t_solve, bad = 0.0, 0
    for s in range(0, len(params), chunk):
        grids = []
        for p in params[s:s + chunk]:
            g = pkg.GpuGrid.from_case(dict(base, H0=base["dep"]))
            g.add_source(base["xcrd"], base["ycrd"], **source_of(p, L))
            grids.append(g)
        b = pkg.Batch(grids)
        b.set_plan(cg.GRAPH, graph_steps=32)
        t0 = time.perf_counter()
        b.step(steps)
        t_solve += time.perf_counter() - t0
        for g in grids:
            r, flags = g.status()
            bad += int(r != 0)
            me, _ = g.maxwave()
            gg, mm = targets_of(me, I, J, dep)
            G.append(gg)
            M.append(mm.astype(np.float32))
            g.close()
        b.close()
    return np.array(G), np.array(M), t_solve, bad


# ---- the surrogate ---------------------------------------------------------------

class Norm:
    """Inputs to [-1, 1]; gauge maxima as standardised log(max + 0.01),
    weighted by GW against the map; inundation maps scaled by one number (the
    RMS of the training maps).

    per_amp: targets per metre of source amplitude (max / amp, map / amp).
    Offshore the response is close to linear in the amplitude, so the network
    then learns the shape of the response rather than its scale."""

    GW = 2.0

    def __init__(self, G, M, params=None, per_amp=True):
        self.per_amp = per_amp
        if per_amp:
            a = params[:, 2:3]
            G, M = G / a, M / a[:, :, None]
        lg = np.log(G + 0.01)
        self.gm, self.gs = lg.mean(0), lg.std(0) + 1e-6
        self.ms = float(np.sqrt(np.mean(np.square(M)))) + 1e-6

    @staticmethod
    def x(params):
        """Features: the parameters scaled to [-1, 1], with the amplitude as its
        logarithm and the angle as its cosine and sine (rotations wrap)."""
        z = 2.0 * (params - LO) / (HI - LO) - 1.0
        la = np.log(params[:, 2])
        z[:, 2] = 2.0 * (la - np.log(LO[2])) / (np.log(HI[2]) - np.log(LO[2])) - 1.0
        return np.hstack([z[:, :5], np.cos(params[:, 5:6]), np.sin(params[:, 5:6]), z[:, 6:]])

    def t(self, G, M, params=None):
        if self.per_amp:
            a = params[:, 2:3]
            G, M = G / a, M / a[:, :, None]
        return np.hstack([self.GW * (np.log(G + 0.01) - self.gm) / self.gs, M.reshape(len(M), -1) / self.ms])

    def back_gauges(self, Y, params=None):
        """Gauge maxima (m) from network outputs (the first NGAUGES columns)."""
        g = np.exp(Y[:, :NGAUGES] / self.GW * self.gs + self.gm) - 0.01
        if self.per_amp:
            g = g * params[:, 2:3]
        return np.maximum(g, 0.0)

    def back_maps(self, Y, params=None):
        """Inundation maps (m) from a map network's outputs."""
        m = Y[:, NGAUGES:].reshape(len(Y), MAP, MAP) * self.ms
        if self.per_amp:
            m = m * params[:, 2:3, None]
        return np.maximum(m, 0.0)


N_FEATURES = 9  # Norm.x


class Ensemble:
    """`members` gauge networks (MLP 9 -> width x depth -> 64) and
    `map_members` map networks (the same MLP emitting the gauges and the
    decoder's latent grid, then the 128 x 128 map)."""

    def __init__(self, members=4, width=512, depth=3, seed=0, map_members=1):
        self.nets = [MLP(N_FEATURES, width, depth, NGAUGES, seed=seed + 101 * k) for k in range(members)]
        self.maps = [MLP(N_FEATURES, width, depth, NGAUGES, seed=seed + 211 + 101 * k, map_side=MAP, map_ch=MAP_CH)
                     for k in range(map_members)]

    def train(self, X, T, epochs, map_epochs, batch=512, lr=1e-3, seed=0, weight_decay=0.0):
        """T: normalised gauge columns, then the map; returns the loss
        curves of the gauge and of the map members."""
        batch = max(16, min(batch, len(X) // 16 * 16))
        Tg = np.ascontiguousarray(T[:, :NGAUGES])
        lg = [net.train(X, Tg, epochs, batch, lr, seed + 7 * k, weight_decay) for k, net in enumerate(self.nets)]
        lm = [net.train(X, T, map_epochs, batch, lr, seed + 13 + 7 * k, weight_decay)
              for k, net in enumerate(self.maps)] if map_epochs > 0 else []
        return lg, lm

    def predict(self, X, norm, params=None, maps=True):
        """Mean gauge maxima, mean map (None without maps) and the members'
        gauge maxima (members, n, 64)."""
        G = np.stack([norm.back_gauges(net.predict(X), params) for net in self.nets])
        M = None
        if maps and self.maps:
            M = np.mean([norm.back_maps(net.predict(X), params) for net in self.maps], axis=0)
        return G.mean(0), M, G

    def close(self):
        for n in self.nets + self.maps:
            n.close()


def forward_flop(width=512, depth=3, with_map=False):
    """Multiply-add FLOPs of one network's forward pass for one sample: the
    dense layers and, for a map network (whose last layer also emits the
    latent grid), the decoder's three convolutions (3x3 taps on the
    upsampled grids)."""
    s0 = MAP // 8
    lat = s0 * s0 * MAP_CH[0] if with_map else 0
    dims = [N_FEATURES] + [width] * depth + [NGAUGES + lat]
    fl = sum(2 * a * b for a, b in zip(dims[:-1], dims[1:]))
    if with_map:
        ch = list(MAP_CH) + [1]
        for l in range(3):
            side = 2 * s0 << l
            fl += 2 * side * side * ch[l + 1] * 9 * ch[l]
    return fl


def spread(Gm, floor=0.05):
    """Relative disagreement of the members per scenario: the mean over
    gauges of std / mean, leaving out gauges whose mean maximum is below
    `floor` m."""
    mean = Gm.mean(0)
    rel = Gm.std(0) / np.maximum(mean, 1e-9)
    keep = mean >= floor
    return np.where(keep, rel, 0.0).sum(axis=1) / np.maximum(keep.sum(axis=1), 1)


def gauge_errors(Gp, G, floor=0.05):
    """Relative error per gauge (gauges with a solver maximum of at least
    `floor` m), and its mean per scenario."""
    mask = G >= floor
    rel = np.abs(Gp - G) / np.maximum(G, 1e-9)
    per = np.where(mask, rel, 0.0).sum(axis=1) / np.maximum(mask.sum(axis=1), 1)
    return rel, mask, per


def calibrate_gate(sp, rel, mask, target):
    """The largest spread threshold whose accepted scenarios keep the mean
    gauge error within `target` (on a validation split)."""
    best = 0.0
    for thr in np.sort(sp):
        acc = sp <= thr
        e = rel[acc[:, None] & mask]
        if e.size and e.mean() <= target:
            best = thr
    return float(best)


def make_data(n_train=4096, n_test=256, steps=2000, seed=0):
    """The solver runs of the study: n_train training runs (the first n_val of
    them calibrate the gate) and n_test held-out runs."""
    base = base_grid(seed)
    Xall = sample_params(n_train, seed + 1)
    Xte = sample_params(n_test, seed + 2)
    t0 = time.perf_counter()
    Gall, Mall, t_data, bad_tr = solve(Xall, base, steps)
    t_gen = time.perf_counter() - t0
    Gte, Mte, t_test_solve, bad_te = solve(Xte, base, steps)
    return dict(base=base, steps=steps, Xall=Xall, Gall=Gall, Mall=Mall, Xte=Xte, Gte=Gte, Mte=Mte,
                t_gen=t_gen, t_data=t_data, t_test_solve=t_test_solve, bad=int(bad_tr + bad_te))


def map_errors(Mp, M, floor=0.05):
    """The inundation maps against the solver's: mean absolute error over the
    window (m), over the cells either inundates by more than `floor` m, the
    relative error of each scenario's largest depth, and the intersection
    over union of the inundated footprints (depth > floor)."""
    a, b = Mp > floor, M > floor
    either = a | b
    inter = (a & b).sum(axis=(1, 2))
    union = either.sum(axis=(1, 2))
    iou = np.where(union > 0, inter / np.maximum(union, 1), 1.0)
    mx = M.max(axis=(1, 2))
    rel_max = np.abs(Mp.max(axis=(1, 2)) - mx) / np.maximum(mx, 1e-9)
    has = mx > floor
    return dict(map_abs_err_mean_m=float(np.abs(Mp - M).mean()),
                map_abs_err_inundated_m=float(np.abs(Mp - M)[either].mean()) if either.any() else 0.0,
                map_max_depth_mean_m=float(mx.mean()),
                map_max_depth_rel_err_mean=float(rel_max[has].mean()) if has.any() else 0.0,
                map_iou_mean=float(iou.mean()), map_scenarios_inundated=int(has.sum()))


def fit_and_judge(D, epochs=3000, map_epochs=600, target=0.045, seed=0, n_val=256, per_amp=True, width=512,
                  depth=3, members=4, map_members=1, single=None, batch=512, lr=1e-3, repeats=1, infer_batch=4096):
    """Train the ensemble on the training runs, calibrate its gate on the
    validation split, judge it on the held-out runs against the solver.

    The gated path (gauge and map predictions of the held-out scenarios, the
    gate, one batched solve of the rejected ones) is timed `repeats` times
    (medians reported); the surrogate alone is also timed at an inference
    batch of `infer_batch` fresh scenarios.  single: seconds of one
    one-at-a-time solve (measured here when None)."""
    base, steps = D["base"], D["steps"]
    Xall, Gall, Mall, Xte, Gte, Mte = D["Xall"], D["Gall"], D["Mall"], D["Xte"], D["Gte"], D["Mte"]
    n_test = len(Xte)
    Xtr, Gtr, Mtr = Xall[n_val:], Gall[n_val:], Mall[n_val:]
    Xva, Gva = Xall[:n_val], Gall[:n_val]
    norm = Norm(Gtr, Mtr, Xtr, per_amp=per_amp)
    ens = Ensemble(members=members, width=width, depth=depth, seed=seed, map_members=map_members)
    t0 = time.perf_counter()
    lg, lm = ens.train(norm.x(Xtr), norm.t(Gtr, Mtr, Xtr), epochs, map_epochs, batch=batch, lr=lr)
    t_train = time.perf_counter() - t0
    # the gate, from the validation split (gauge members)
    Gv, _, Gvm = ens.predict(norm.x(Xva), norm, Xva, maps=False)
    rel_v, mask_v, _ = gauge_errors(Gv, Gva)
    thr = calibrate_gate(spread(Gvm), rel_v, mask_v, target)
    # the gated path on the test split: predictions, the gate, the solver for
    # the rejected scenarios as one batch, timed whole (grid set-up, sources,
    # steps, max-wave download)
    t_preds, t_fbs = [], []
    for _ in range(max(1, repeats)):
        t0 = time.perf_counter()
        Gp, Mp, Gm = ens.predict(norm.x(Xte), norm, Xte)
        sp = spread(Gm)
        accept = sp <= thr
        t_preds.append(time.perf_counter() - t0)
        rej = np.flatnonzero(~accept)
        t_fb = 0.0
        if rej.size:
            t0 = time.perf_counter()
            Gfb, _, _, _ = solve(Xte[rej], base, steps)
            t_fb = time.perf_counter() - t0
            assert np.array_equal(Gfb, Gte[rej])  # batching does not change a run
        t_fbs.append(t_fb)
    t_pred, t_fb = float(np.median(t_preds)), float(np.median(t_fbs))
    n_fallback = int((~accept).sum())
    rel, mask, _ = gauge_errors(Gp, Gte)
    rel_acc = rel[accept[:, None] & mask]
    merr = map_errors(Mp, Mte) if Mp is not None else {}
    # the surrogate alone at the inference batch: fresh scenarios, gauges and maps
    Xinf = sample_params(infer_batch, seed + 99)
    ens.predict(norm.x(Xinf), norm, Xinf)  # buffers at this batch
    t0 = time.perf_counter()
    ens.predict(norm.x(Xinf), norm, Xinf)
    t_inf = time.perf_counter() - t0
    # one-at-a-time solves of a few test scenarios: the method without the surrogate
    if single is None:
        n_single = min(16, n_test)
        L = base["xcrd"][-1]
        t_single = 0.0
        for p in Xte[:n_single]:
            g = pkg.GpuGrid.from_case(dict(base, H0=base["dep"]))
            g.add_source(base["xcrd"], base["ycrd"], **source_of(p, L))
            g.sync()
            t1 = time.perf_counter()
            g.step(steps)
            g.maxwave()
            t_single += time.perf_counter() - t1
            g.close()
        single = t_single / n_single
    per_single = single
    per_batch = D["t_test_solve"] / n_test
    t_gated = t_pred + t_fb
    flop = members * forward_flop(width, depth) + map_members * forward_flop(width, depth, with_map=True)
    res = dict(train=len(Xtr), validation=n_val, test=n_test, steps=steps, epochs=epochs, map_epochs=map_epochs,
               target=target, per_amp=per_amp, width=width, depth=depth, members=members, map_members=map_members,
               map=[MAP, MAP], map_channels=MAP_CH, nonfinite_runs=D["bad"],
               data_seconds=round(D["t_gen"], 2), solver_seconds_train=round(D["t_data"], 2),
               train_seconds=round(t_train, 2),
               final_loss=[round(float(l[-1]), 5) for l in lg], first_loss=[round(float(l[0]), 5) for l in lg],
               map_final_loss=[round(float(l[-1]), 5) for l in lm],
               gate_threshold=round(thr, 4), accepted=int(accept.sum()), fallback=n_fallback,
               gauge_rel_err_all_mean=round(float(rel[mask].mean()), 4),
               gauge_rel_err_all_p90=round(float(np.quantile(rel[mask], 0.9)), 4),
               gauge_rel_err_accepted_mean=round(float(rel_acc.mean()), 4) if rel_acc.size else None,
               gauge_rel_err_accepted_median=round(float(np.median(rel_acc)), 4) if rel_acc.size else None,
               gated_rel_err_mean=round(float(np.where(accept[:, None], rel, 0.0)[mask].mean()), 4),
               **{k: round(v, 4) if isinstance(v, float) else v for k, v in merr.items()},
               repeats=len(t_preds), predict_ms=round(1e3 * t_pred, 3), fallback_solve_ms=round(1e3 * t_fb, 2),
               predict_flop=int(flop * n_test),
               single_solve_s=round(per_single, 4), batched_solve_s_per_scenario=round(per_batch, 5),
               surrogate_scenarios_per_s=round(n_test / t_pred, 1),
               infer_batch=infer_batch, infer_ms=round(1e3 * t_inf, 2),
               infer_scenarios_per_s=round(infer_batch / t_inf, 1),
               gated_scenarios_per_s=round(n_test / t_gated, 1),
               one_at_a_time_scenarios_per_s=round(1.0 / per_single, 2),
               gated_speedup_vs_one_at_a_time=round(per_single * n_test / t_gated, 1),
               gated_speedup_vs_batched=round(per_batch * n_test / t_gated, 1))
    ens.close()
    return res


def run(n_train=4096, n_test=256, steps=2000, epochs=3000, target=0.045, seed=0, n_val=256, per_amp=True,
        map_epochs=600, infer_batch=4096, map_members=1):
    """Data from the batched solver, the ensemble trained on n_train - n_val
    runs, its gate calibrated on the n_val others, judged on n_test held-out
    runs against the solver."""
    D = make_data(n_train, n_test, steps, seed)
    return fit_and_judge(D, epochs=epochs, map_epochs=map_epochs, target=target, seed=seed, n_val=n_val,
                         per_amp=per_amp, infer_batch=infer_batch, map_members=map_members)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--test", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--map-epochs", type=int, default=600)
    ap.add_argument("--map-members", type=int, default=1)
    ap.add_argument("--target", type=float, default=0.045)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-per-amp", action="store_true", help="targets in metres, not per metre of amplitude")
    ap.add_argument("--infer", type=int, default=0, help="time inference of N scenarios alone (untrained)")
    a = ap.parse_args()
    pkg.build.build()
    if a.infer:
        ens = Ensemble(members=4, map_members=1, seed=a.seed)
        X = Norm.x(sample_params(a.infer, a.seed))
        out = {}
        for k in range(2):
            t0 = time.perf_counter()
            G = [net.predict(X) for net in ens.nets]
            M = [net.predict(X) for net in ens.maps]
            out[f"pass{k}_ms"] = round(1e3 * (time.perf_counter() - t0), 2)
        out.update(scenarios=a.infer, finite=bool(np.isfinite(G[0]).all() and np.isfinite(M[0]).all()))
        ens.close()
        print(json.dumps(out), flush=True)
        return
    print(json.dumps(run(a.train, a.test, a.steps, a.epochs, a.target, a.seed, per_amp=not a.no_per_amp,
                         map_epochs=a.map_epochs, map_members=a.map_members)), flush=True)


if __name__ == "__main__":
    main()

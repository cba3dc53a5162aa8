"""The FP32 variant of the CPU time loop (oracle/cliffs_oracle.c built with
orc_real = float), which bench.py times beside the FP64 oracle as a
like-for-like baseline of the FP32 GPU path: it must compute the same steps.
Against the FP64 oracle on a shelf with runup, after 200 steps: wet/dry
disagreements on at most 0.1 % of the cells, and on cells wet in both the
surface within 5 cm and the velocities within 1 cm/s.  The bounds are loose
because a plain FP32 build carries the total depth H = c^2/g: every step
rounds the surface at the spacing of floats near H, about 0.5 mm at 4000 m
(measured: 2.4 cm and 3 mm/s at most).  The GPU path stores the surface
elevation at sea instead and stays within 1e-4 of the amplitude."""
import importlib

import numpy as np

from runners import GRAV, oracle_model, oracle_model32

W = importlib.import_module("cliffs-src_gb300.workloads")


def test_f32_time_loop_follows_the_fp64_oracle():
    c = W.shelf_2d(seed=81, nx=300, ny=220, dx=500.0, steps=0, ngauges=0, axes_km=(30, 15),
                   centre_km=(120.0, 55.0))
    c["crough"] = 0.000625
    m, m32 = oracle_model(c), oracle_model32(c)
    assert m.step(200) == 200 and m32.step(200) == 200
    cel32 = m32.cel.astype(np.float64)
    wet, wet32 = m.cel > m.celmin, cel32 > m.celmin
    both = wet & wet32
    assert both.sum() > 0.5 * both.size
    assert (wet != wet32).sum() <= 1e-3 * wet.size
    eta = m.cel ** 2 / GRAV - m.dep
    eta32 = cel32 ** 2 / GRAV - m32.dep.astype(np.float64)
    assert np.abs(eta - eta32)[both].max() < 0.05
    assert np.abs(m.xvel - m32.xvel)[both].max() < 0.01
    assert np.abs(m.yvel - m32.yvel)[both].max() < 0.01

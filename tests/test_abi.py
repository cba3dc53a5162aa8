"""The C-ABI library builds, loads and exports every symbol of include/*.h.

No compute call runs here (the build container has no GPU); creating a
context without a device must fail with CLIFFS_ERR_DEVICE, not crash.
"""
import ctypes
import glob
import importlib
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pkg = importlib.import_module("cliffs-src_gb300")


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names += re.findall(r"\b(cliffs_(?:gpu|batch|mlp|depth|boundary)_\w+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    pkg.build.build()
    return pkg.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 25
    raw = ctypes.CDLL(pkg.cliffs_gpu.LIB_PATH)
    for n in names:
        assert hasattr(raw, n), n
        assert n in pkg.cliffs_gpu.SIGNATURES, f"binding lacks {n}"


def test_binding_covers_only_declared(lib):
    assert set(pkg.cliffs_gpu.SIGNATURES) <= set(_declared())


def test_metrics_match_oracle(lib):
    import oracle
    x = np.linspace(138.0, 141.5, 57)
    y = np.linspace(41.0, 43.8, 45)
    for cart in (True, False):
        dx, rs, dy, zeta = pkg.metrics(x, y, cart)
        s1, s2, z2 = oracle.metrics(x, y, cart)
        scale = rs if rs is not None else np.ones(len(y))
        assert np.allclose(np.outer(scale, dx), s1, rtol=1e-15, atol=0)
        assert np.array_equal(dy, s2)
        assert np.array_equal(zeta, z2)


def test_strerror_and_no_device(lib):
    assert lib.cliffs_gpu_strerror(0).decode() == "ok"
    assert "argument" in lib.cliffs_gpu_strerror(-1).decode()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    dep = np.ones((4, 5))
    with pytest.raises(pkg.CliffsError) as e:
        pkg.GpuGrid(dep, dx=np.ones(4), dy=np.ones(3), ground=0.01, crough=0, dt=0.1)
    assert e.value.code in (-6, -2)


def test_bad_descriptions_rejected_before_device(lib):
    with pytest.raises(pkg.CliffsError) as e:
        pkg.GpuGrid(np.ones((2, 2)), ground=0.01, crough=0, dt=0.1)  # both dims <= 2
    assert e.value.code == -1
    with pytest.raises(pkg.CliffsError) as e:
        pkg.GpuGrid(np.ones((4, 5)), dx=np.ones(4), dy=np.ones(3), ground=0.01, crough=0, dt=0.0)
    assert e.value.code == -1


def test_grids_past_the_launch_limits_rejected_before_device(lib):
    # a grid with an x-sweep and more than 65535 rows (one block row per grid row)
    with pytest.raises(pkg.CliffsError) as e:
        pkg.GpuGrid(np.ones((65536, 3)), dx=np.ones(2), dy=np.ones(65535), ground=0.01, crough=0, dt=0.1)
    assert e.value.code == -1
    # a channel along y with more than 65535 bands of 16 rows
    with pytest.raises(pkg.CliffsError) as e:
        pkg.GpuGrid(np.ones((16 * 65535 + 1, 1)), dy=np.ones(16 * 65535), ground=0.01, crough=0, dt=0.1)
    assert e.value.code == -1

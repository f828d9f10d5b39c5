"""C-ABI and host logic checks that need no GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import quickses_gb300 as q
from quickses_gb300 import _lib as L
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "quickses.h")


def _declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    funcs = set(re.findall(r"QSES_API\s+[\w\s\*]+?\b(\w+)\s*\(", src))
    data = set(re.findall(r"extern\s+QSES_API\s+[\w\s\*]+?\b(\w+)\s*;", src))
    return funcs, data


def test_every_declared_symbol_is_exported():
    funcs, data = _declared_symbols()
    assert {"API_computeSES", "API_getTriangles", "API_getVertices", "API_freeMesh",
            "API_getAtomIdPerVert"} <= funcs
    assert data == {"NTriangles", "NVertices", "globalTriangles", "globalVertices", "globalIdAtomPerVert"}
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = (funcs | data) - exported
    assert not missing, missing
    assert set(L.SIGNATURES) == funcs | data  # the Python binding covers every symbol
    lib = L.lib()
    for name in funcs | data:
        assert getattr(lib, name) is not None


def test_only_declared_symbols_are_exported():
    funcs, data = _declared_symbols()
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    ours = {ln.split()[-1] for ln in out.splitlines() if re.search(r"\b(API_|qses_)", ln) or
            ln.split()[-1] in data}
    assert ours <= funcs | data


def test_status_strings():
    for code in range(8):
        assert L.status_string(code)
    assert L.status_string(99) == "unknown status"


def _has_gpu():
    try:
        q.Context(0).close()
        return True
    except q.QSESError:
        return False


def test_context_without_gpu_fails_loudly():
    if _has_gpu():
        pytest.skip("a GPU is present")
    with pytest.raises(q.QSESError) as e:
        q.Context(0)
    assert e.value.code == L.QSES_ERR_NO_DEVICE
    # the reference-compatible surface reports the failure instead of exiting
    api = q.ReferenceAPI()
    xyz, rad, _ = q.molecules.ball(50, 1)
    with pytest.raises(q.QSESError):
        api.computeSES(0.5, xyz, rad)
    assert api.exported_counts() == (0, 0)


@pytest.mark.parametrize("n,seed,dx", [(1000, 1, 0.5), (50000, 1, 0.2), (300, 3, 0.3), (2, 4, 0.4)])
def test_grid_sizing_matches_oracle(n, seed, dx):
    xyz, rad, _ = q.molecules.ball(n, seed)
    gi = q.grid_info(xyz, rad, dx)
    g, _ = O.grid(xyz, rad, dx)
    assert (gi.G, gi.gnb, gi.R, gi.Gc) == (g.G, g.gnb, g.R, g.Gc)
    assert tuple(gi.origin) == (g.ox, g.oy, g.oz) and gi.cell == g.cell


def test_workload_grid_sizes():
    """Grid sizes of the benchmark workloads (CudaSurf.cu:556-562 sizing)."""
    xyz, rad, _ = q.molecules.ball(1000, 1)
    assert 80 <= q.grid_info(xyz, rad, 0.5).G <= 90
    xyz, rad, _ = q.molecules.ball(50000, 1)
    gi = q.grid_info(xyz, rad, 0.2)
    assert 655 <= gi.G <= 675 and gi.R == 7


def test_unsupported_inputs_are_rejected():
    xyz, rad, _ = q.molecules.ball(100, 1)
    with pytest.raises(q.QSESError) as e:
        q.grid_info(xyz, rad, 0.1)  # refine window of 14 voxels
    assert e.value.code == L.QSES_ERR_UNSUPPORTED
    far = xyz + np.float32(20000.0)
    with pytest.raises(q.QSESError):
        q.grid_info(far, rad, 0.5)
    with pytest.raises(q.QSESError):
        q.grid_info(xyz, rad, -1.0)


def test_synthetic_generators_are_deterministic():
    a = q.molecules.ball(2000, 5)
    b = q.molecules.ball(2000, 5)
    c = q.molecules.ball(2000, 6)
    assert np.array_equal(a[0], b[0]) and not np.array_equal(a[0], c[0])
    xyz, rad, el = a
    d2 = ((xyz[:200, None, :] - xyz[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2[:, :200], 1e9)
    assert d2.min() >= 1.2 ** 2 - 1e-3
    rb = (3 * 2000 / (4 * np.pi * 0.05)) ** (1 / 3)
    assert np.linalg.norm(xyz, axis=1).max() <= rb + 1e-3
    frac = {chr(k): np.mean(el == k) for k in np.unique(el)}
    assert abs(frac["C"] - 0.62) < 0.04 and abs(frac["O"] - 0.19) < 0.04
    radii = {ord("C"): 1.70, ord("N"): 1.55, ord("O"): 1.52, ord("S"): 1.80}
    assert all(abs(r - radii[e]) < 1e-6 for r, e in zip(rad, el))
    s = q.molecules.shell(3000, 2, r_in=50.0, thickness=5.0)[0]
    rr = np.linalg.norm(s, axis=1)
    assert rr.min() >= 50.0 - 1e-3 and rr.max() <= 55.0 + 1e-3
    j = q.molecules.jitter(xyz, 0.3, 9)
    assert abs(np.std(j - xyz) - 0.3) < 0.02

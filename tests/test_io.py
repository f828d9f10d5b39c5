"""File front-end (CPU only): PDB reading against QuickSES's own parser, OBJ writing against
the reference's fprintf format, and the CLI's argument handling."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import quickses_gb300 as q

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SAMPLE = os.path.join(HERE, "golden", "sample.pdb")
CLI = os.path.join(ROOT, "quickses_gb300", "bin", "QuickSES")

# CudaSurf.h:64-73: radius by the element's first byte, 1.40 otherwise
RADIUS = {ord("O"): 1.52, ord("C"): 1.70, ord("N"): 1.55, ord("H"): 1.20, ord("S"): 1.80, ord("P"): 1.80}


def _radii(element0):
    return np.array([RADIUS.get(int(e), 1.40) for e in element0], np.float32)


def test_read_pdb_matches_reference_golden():
    g = np.load(os.path.join(HERE, "golden", "ref_pdb.npz"))
    xyz, rad = q.read_pdb(SAMPLE)
    assert np.array_equal(xyz, g["xyz"])
    assert np.array_equal(rad, _radii(g["element0"]))


def test_read_pdb_matches_live_reference(tmp_path):
    path = os.path.join(ROOT, "oracle", "_ref", "libqses_ref_pdb.so")
    if not os.path.exists(path):
        pytest.skip("reference checkout not available on this machine")
    L = ctypes.CDLL(path)
    L.ref_read_pdb.restype = ctypes.c_int
    L.ref_read_pdb.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    from tests.golden import gen_pdb_golden as G
    for seed in range(6):
        p = tmp_path / ("s%d.pdb" % seed)
        p.write_text(G.make_pdb(seed))
        xyz = np.zeros((1000, 3), np.float32)
        el = np.zeros(1000, np.uint8)
        n = L.ref_read_pdb(str(p).encode(), xyz.ctypes.data, el.ctypes.data, 1000)
        mx, mr = q.read_pdb(p)
        assert len(mr) == n
        assert np.array_equal(mx, xyz[:n]) and np.array_equal(mr, _radii(el[:n]))


def test_read_pdb_missing_file():
    with pytest.raises(q.QSESError):
        q.read_pdb("/nonexistent/file.pdb")


def test_fixed3_matches_printf():
    rng = np.random.default_rng(3)
    vals = [0.0, -0.0, 0.0005, -0.0005, 0.0625, -0.0625, 0.1875, 2.5e-4, 1e-30, -1e-30, 123.4565, 9.9995,
            -9.9995, 1e7, 3e9, -16000.0]
    vals += list(rng.uniform(-3000, 3000, 3000).astype(np.float32))
    vals += [np.float32(k) / np.float32(2 ** s) for k in range(-40, 40) for s in (3, 4, 5, 10, 13)]  # ties
    for v in vals:
        f = np.float32(v)
        assert q.format_fixed3(f) == "%.3f" % float(f), (repr(f), q.format_fixed3(f), "%.3f" % float(f))


def _expected_obj(v, t):
    out = ["v %.3f %.3f %.3f\n" % tuple(float(c) for c in p) for p in v]
    out.append("\n")
    out += ["f %d %d %d\n" % (b + 1, a + 1, c + 1) for a, b, c in t]  # CudaSurf.cu:366
    return "".join(out)


@pytest.mark.parametrize("threads", [1, 3])
def test_write_obj_matches_reference_format(tmp_path, threads):
    rng = np.random.default_rng(threads)
    nv = 200_000  # several formatting chunks
    v = rng.normal(0, 50, (nv, 3)).astype(np.float32)
    v[:64] = np.float32(rng.integers(-800, 800, (64, 3))) / np.float32(16)  # exact decimal ties
    t = rng.integers(0, nv, (150_000, 3)).astype(np.int32)
    p = tmp_path / "m.obj"
    q.write_obj(p, v, t, threads=threads)
    assert p.read_text() == _expected_obj(v, t)


def test_write_obj_empty(tmp_path):
    p = tmp_path / "e.obj"
    q.write_obj(p, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    assert p.read_text() == "\n"


def _cli(*args):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=60)


def test_cli_arguments():
    assert os.path.exists(CLI)
    r = _cli("-h")
    assert r.returncode == 0 and "-i" in r.stderr and "-o" in r.stderr
    r = _cli("-i", SAMPLE)  # -o is mandatory
    assert r.returncode == 255 and "Usage" in r.stderr
    r = _cli("-i", SAMPLE, "-o", "/tmp/x.obj", "-l", "abc")
    assert r.returncode == 255
    r = _cli("-i", "/nonexistent.pdb", "-o", "/tmp/x.obj")
    assert r.returncode == 2

"""Pins the CPU oracle to QuickSES's own code (CPU, no GPU needed).

The reference ships no tests or fixtures, so the pins are (1) golden vectors produced by
running the reference's host-callable functions (tests/golden/gen_ref_golden.py) and
(2) the same functions run live from oracle/_ref/ when the reference checkout exists.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import quickses_gb300 as q
import ref_slices
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = np.load(os.path.join(HERE, "golden", "ref_host.npz"))
CASES = sorted({k.split("_")[0] for k in GOLDEN.files})


@pytest.mark.parametrize("case", CASES)
def test_hash_matches_reference(case):
    xyz, rad, dx = GOLDEN[case + "_xyz"], GOLDEN[case + "_rad"], float(GOLDEN[case + "_dx"])
    g, _ = O.grid(xyz, rad, dx)
    _, h = O.sort_atoms(xyz, g)
    assert np.array_equal(h, GOLDEN[case + "_hash"])


@pytest.mark.parametrize("case", CASES)
def test_sas_classification_matches_reference(case):
    """computeInOrOut vs the oracle's FP32 classification at every computed voxel.  The
    reference compares sqrt(d^2) < r - dx; the oracle compares d^2 against the squared,
    float-rounded threshold: they may only differ on exact ties, of which these seeds
    have none."""
    xyz, rad, dx = GOLDEN[case + "_xyz"], GOLDEN[case + "_rad"], float(GOLDEN[case + "_dx"])
    g, _ = O.grid(xyz, rad, dx)
    codes = O.field_codes(xyz, rad, g, fp64=False)[:-1, :-1, :-1]
    cls = np.where(codes == O.CODE_OUT, 0, np.where(codes == O.CODE_IN, 2, 1)).astype(np.int8)
    ref = GOLDEN[case + "_class"]
    assert cls.shape == ref.shape
    assert int((cls != ref).sum()) == 0


@pytest.mark.parametrize("case", CASES)
def test_smoothing_matches_reference_bitwise(case):
    v, t = GOLDEN[case + "_mesh_v"], GOLDEN[case + "_mesh_t"]
    out = O.smooth_f32(v, t, 1)
    assert np.array_equal(out, GOLDEN[case + "_smooth1"])


@pytest.mark.parametrize("case", CASES)
def test_closest_atom_matches_reference(case):
    xyz, rad, dx = GOLDEN[case + "_xyz"], GOLDEN[case + "_rad"], float(GOLDEN[case + "_dx"])
    m = O.compute_ses(xyz, rad, dx, smooth=0, fp64=False)
    assert np.array_equal(m.vertices.astype(np.float32), GOLDEN[case + "_mesh_v"])
    assert np.array_equal(m.atom_sorted, GOLDEN[case + "_closest"])


def _ref_lib():
    path = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libqses_ref_host.so")
    if not os.path.exists(path):
        pytest.skip("reference checkout not available on this machine")
    L = ctypes.CDLL(path)
    L.ref_smooth.restype = None
    L.ref_smooth.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
    return L


@pytest.mark.parametrize("passes", [1, 2, 3])
def test_smoothing_live_reference_multipass(passes):
    """The oracle's Gauss-Seidel pass against SmoothMesh.cpp itself on a fresh mesh,
    including degenerate triangles (dx = 0.2 produces many)."""
    L = _ref_lib()
    xyz, rad, _ = q.molecules.ball(150, 21)
    m = O.compute_ses(xyz, rad, 0.2, smooth=0, fp64=False)
    v = m.vertices.astype(np.float32)
    t = np.ascontiguousarray(m.triangles, np.int32)
    assert (t[:, 0] == t[:, 1]).any() or (t[:, 1] == t[:, 2]).any() or (t[:, 0] == t[:, 2]).any()
    ref = np.ascontiguousarray(v.copy())
    L.ref_smooth(passes, ref.ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p), len(v), len(t))
    assert np.array_equal(O.smooth_f32(v, t, passes), ref)


def test_mc_tables_match_reference_source():
    """The packed kernel table and the oracle table both equal MarchingCubes.cu:64-343."""
    from oracle import build as ob
    refdir = ob.reference_sources()
    src = os.path.join(refdir, "MarchingCubes.cu") if refdir else ""
    root = os.path.dirname(HERE)
    packed = open(os.path.join(root, "quickses_gb300", "csrc", "mc_tables.h")).read()
    words = [int(x, 16) for x in re.findall(r"0x([0-9a-f]{16})ULL", packed)]
    otab = open(os.path.join(root, "oracle", "mc_table.h")).read()
    rows = [[int(v) for v in r.split(",")] for r in re.findall(r"\{([-\d, ]+)\}", otab)]
    assert len(words) == 256 and len(rows) == 256
    for c in range(256):
        n = 0
        while n < 16 and rows[c][n] != -1:
            n += 1
        assert (words[c] >> 60) * 3 == n
        assert all(((words[c] >> (4 * v)) & 15) == rows[c][v] for v in range(n))
        # every sign-changing edge of the case is used (welded vertices = active edges)
        corners = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
        cross = {e for e, (a, b) in enumerate(corners) if ((c >> a) & 1) != ((c >> b) & 1)}
        assert set(rows[c][:n]) == cross
    if os.path.exists(src):
        import importlib.util
        spec = importlib.util.spec_from_file_location("g", os.path.join(root, "quickses_gb300", "csrc", "gen_mc_tables.py"))
        gm = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(gm)
        tri, nb = gm.load_reference(src)
        assert tri == rows


@pytest.mark.parametrize("n,seed,dx", [(80, 31, 0.5), (120, 32, 0.4), (90, 33, 0.2)])
def test_oracle_fp32_vs_fp64(n, seed, dx):
    """FP32 arithmetic vs FP64: identical voxel codes on these seeds, and the smoothed
    meshes within 0.05 voxel (symmetric Hausdorff)."""
    xyz, rad, _ = q.molecules.ball(n, seed)
    g, _ = O.grid(xyz, rad, dx)
    c32 = O.field_codes(xyz, rad, g, fp64=False)
    c64 = O.field_codes(xyz, rad, g, fp64=True)
    assert int((c32 != c64).sum()) == 0
    l32, l64 = O.lut(g, False), O.lut(g, True)
    assert np.all((l32 < 0) == (l64 < 0))
    assert np.max(np.abs(l32.astype(np.float64) - l64)) < 1e-6
    m32 = O.compute_ses(xyz, rad, dx, smooth=1, fp64=False)
    m64 = O.compute_ses(xyz, rad, dx, smooth=1, fp64=True)
    h, _, _ = O.hausdorff(m32.vertices, m32.triangles_kept, m64.vertices, m64.triangles_kept)
    assert h <= 0.05 * dx


def test_oracle_smoothing_is_sequential_gauss_seidel():
    """Independent pure-Python statement of SmoothMesh.cpp's loop on a tiny mesh."""
    xyz, rad, _ = q.molecules.ball(12, 41)
    m = O.compute_ses(xyz, rad, 0.5, smooth=0, fp64=False)
    v = m.vertices.astype(np.float32)
    t = m.triangles
    nb = [[] for _ in range(len(v))]
    for a, b, c in t:
        nb[a] += [b, c]
        nb[b] += [a, c]
        nb[c] += [a, b]
    w = v.copy()
    for i in range(len(w)):
        s = np.zeros(3, np.float32)
        for u in nb[i]:
            s = (s + w[u]).astype(np.float32)
        w[i] = (s / np.float32(len(nb[i]))).astype(np.float32)
    assert np.array_equal(O.smooth_f32(v, t, 1), w)


REFCUDA = np.load(os.path.join(HERE, "golden", "ref_cuda.npz"))


def _tie_code(dx):
    """Code whose value is exactly zero in real arithmetic (probe/dx whole), else None."""
    r = 1.4 / dx
    return round(r * r) if abs(r - round(r)) < 1e-4 else None


@pytest.mark.parametrize("case", sorted({k.split("_")[0] for k in REFCUDA.files}))
def test_oracle_matches_reference_cuda_build(case):
    """Outputs of QuickSES's own CUDA build (oracle/ref_cuda/run_ref.py fixtures): its field
    from probeIntersection + distanceFieldRefine, and its unsmoothed API_computeSES mesh.
    At a tie voxel size (0.2 A) the reference's sign of an exactly-zero value is arbitrary:
    flips are allowed there only, and the mesh is compared geometrically."""
    d = REFCUDA
    xyz, rad, dx = d[case + "_xyz"], d[case + "_rad"], float(d[case + "_dx"])
    g, _ = O.grid(xyz, rad, dx)
    codes = O.field_codes(xyz, rad, g)
    mine = O.lut(g)[codes]
    ref = d[case + "_field"]
    inner = (slice(0, g.G - 1),) * 3
    assert np.abs(mine[inner] - ref[inner]).max() < 2e-6       # fast-math FP32 vs our FP32
    flips = (mine < 0) != (ref < 0)
    tie = _tie_code(dx)
    m = O.compute_ses(xyz, rad, dx, smooth=0)
    if tie is not None:
        assert (codes[flips] == tie).all()
        vr, tr = d[case + "_v0"], d[case + "_t0"]
        used = np.zeros(len(vr), bool)
        used[tr.ravel()] = True
        h, _, _ = O.hausdorff(m.vertices, m.triangles_kept, vr[used].astype(np.float64), (np.cumsum(used) - 1)[tr])
        assert h <= 0.005 * dx
        return
    assert int(flips.sum()) == 0
    vr, tr = d[case + "_v0"], d[case + "_t0"]
    index = {tuple(p): i for i, p in enumerate(vr.tolist())}
    to_ref = np.array([index.get(tuple(p), -1) for p in m.vertices.astype(np.float32).tolist()])
    assert (to_ref >= 0).all()
    # the reference never writes its last triangle and leaves a zero vertex instead
    assert np.array_equal(to_ref[m.triangles_kept[:len(tr)]], tr) and len(m.triangles_kept) == len(tr) + 1


REFSLICES = ref_slices.load()


@pytest.mark.skipif(REFSLICES is None, reason="tests/golden/ref_slices.npz not generated")
@pytest.mark.parametrize("case", ref_slices.cases(REFSLICES) if REFSLICES is not None else [])
def test_oracle_slices_match_reference_build(case):
    """The oracle's restatement of the reference's slicing against the reference's own
    per-slice meshes (computeSlicedSES with small SLICE values, several slices per axis):
    the same slices, vertex and triangle counts per slice, every vertex at the same
    quantised position (a rounding tie may put one a quantum apart) and the same triangles."""
    xyz, rad, dx, sl = ref_slices.case_inputs(REFSLICES, case)
    ref = ref_slices.slices(REFSLICES, case, 0)
    m = O.compute_ses_slices(xyz, rad, dx, sl, smooth=0)
    assert len(ref) == len(m.slice_v) - 1 and len(ref) > 8
    near_total = total = 0
    for k, (v, t, a) in enumerate(ref):
        v, t, a = ref_slices.without_unwritten(v, t, a)
        mv = m.vertices[m.slice_v[k]:m.slice_v[k + 1]].astype(np.float32)
        mt = m.triangles[m.slice_t[k]:m.slice_t[k + 1]] - m.slice_v[k]
        exact, near, unmatched, bad_tri = ref_slices.match(v, t, mv, mt)
        assert unmatched == 0 and bad_tri == 0, (k, exact, near, unmatched, bad_tri)
        near_total += near
        total += len(v)
    assert near_total <= max(2, total // 2000)  # rounding ties only


@pytest.mark.skipif(REFSLICES is None, reason="tests/golden/ref_slices.npz not generated")
@pytest.mark.parametrize("case", [c for c in (ref_slices.cases(REFSLICES) if REFSLICES is not None else [])
                                  if ref_slices.slices(REFSLICES, c, 1) is not None])
def test_reference_slice_smoothing_is_smoothmesh_of_its_slice(case):
    """Each smoothed reference slice is the sequential Gauss-Seidel pass (the oracle's,
    pinned to SmoothMesh.cpp) of that slice's own unsmoothed mesh, its unwritten last
    triangle included: the only smoothing difference from this library's slices is that
    triangle, whose corners hold stale device memory."""
    p0 = ref_slices.slices(REFSLICES, case, 0)
    p1 = ref_slices.slices(REFSLICES, case, 1)
    assert len(p0) == len(p1)
    for k, ((v0, t0, _), (v1, t1, _)) in enumerate(zip(p0, p1)):
        assert len(v0) == len(v1) and np.array_equal(t0[:-1], t1[:-1])
        sm = O.smooth_f32(v0, t1, 1)
        real = ~np.isnan(v1).any(axis=1)
        assert np.array_equal(sm[real], v1[real]), k

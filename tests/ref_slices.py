"""Helpers for comparisons with the reference's own per-slice meshes
(tests/golden/ref_slices.npz, written by oracle/ref_cuda/run_ref.py `slices` from
QuickSES's computeSlicedSES with its SLICE set).

Each fixture slice is the reference's MeshData as it leaves computeMarchingCubes and
smoothMeshLaplacian (CudaSurf.cu:741-746): welded vertices, triangles and sorted atom ids.
Its last triangle was never written (MarchingCubes.cu:845 with CudaSurf.cu:421), so its
three corners hold whatever the device memory held: zeros in a fresh allocation, NaN in one
recycled from an int buffer (the reference's EMPTYCELL fill, Kernels.cu:25, reads as NaN),
welded like real vertices (three NaN vertices, since NaN != NaN) and looked up with
lower_bound (NaN finds vertex 0).
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
QUANTUM = 0.001  # the weld quantum (Kernels.cu:27)


def load():
    path = os.path.join(HERE, "golden", "ref_slices.npz")
    return np.load(path) if os.path.exists(path) else None


def cases(d):
    return sorted({k.split("_")[0] for k in d.files})


def case_inputs(d, case):
    return d[case + "_xyz"], d[case + "_rad"], float(d[case + "_dx"]), int(d[case + "_slice"])


def slices(d, case, passes):
    """[(vertices, triangles, atom ids)] per slice of the reference's run, or None."""
    key = "%s_p%d_" % (case, passes)
    if key + "counts" not in d.files:
        return None
    out, vo, to = [], 0, 0
    for nv, nt in d[key + "counts"]:
        out.append((d[key + "v"][vo:vo + nv], d[key + "t"][to:to + nt], d[key + "a"][vo:vo + nv]))
        vo += nv
        to += nt
    return out


def without_unwritten(v, t, a):
    """The slice without its never-written last triangle and the vertices only it named
    (the other vertices keep their order)."""
    t = t[:-1] if len(t) else t
    used = np.zeros(len(v), bool)
    used[t.ravel()] = True
    ids = np.cumsum(used) - 1
    return v[used], ids[t].astype(np.int32), a[used]


def match(v_ref, t_ref, v_mine, t_mine):
    """Compares two unsmoothed slice meshes.  Vertices are matched by quantised position; a
    vertex may sit one quantum apart (the reference's fast-math arithmetic and ours round a
    tie of the 0.001 A quantisation differently).  Returns (vertices matched exactly,
    vertices one quantum apart, unmatched vertices, triangles that differ after mapping)."""
    if len(v_ref) != len(v_mine):
        return 0, 0, max(len(v_ref), len(v_mine)), len(t_ref)
    kr = np.round(v_ref.astype(np.float64) / QUANTUM).astype(np.int64)
    km = np.round(v_mine.astype(np.float64) / QUANTUM).astype(np.int64)
    index = {tuple(k): i for i, k in enumerate(km.tolist())}
    to_mine = np.full(len(v_ref), -1, np.int64)
    exact = near = 0
    taken = np.zeros(len(v_mine), bool)
    for i, k in enumerate(kr.tolist()):
        j = index.get(tuple(k))
        if j is not None and not taken[j]:
            to_mine[i] = j
            taken[j] = True
            exact += 1
    for i in np.nonzero(to_mine < 0)[0]:  # one quantum apart in some coordinates
        d = np.abs(km - kr[i]).max(axis=1)
        cand = np.nonzero((d <= 1) & ~taken)[0]
        if len(cand):
            to_mine[i] = cand[0]
            taken[cand[0]] = True
            near += 1
    unmatched = int((to_mine < 0).sum())
    bad_tri = len(t_ref) if len(t_ref) != len(t_mine) or unmatched else \
        int((to_mine[t_ref] != t_mine).any(axis=1).sum())
    return exact, near, unmatched, bad_tri

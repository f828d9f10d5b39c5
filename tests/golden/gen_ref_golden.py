"""Generate golden vectors from QuickSES's own host code (oracle/_ref/libqses_ref_host.so,
built by oracle/build.py from the reference checkout).

The reference has no tests or fixtures of its own, so these vectors are the pin for the
oracle: its CPU-runnable functions are executed on seeded synthetic molecules and their
outputs stored in tests/golden/ref_host.npz:

* hashAtoms' cell key per atom (spaceToGrid + flatten3DTo1D, Kernels.cu:119-131, 185-216)
* computeInOrOut per voxel (Kernels.cu:344-392) as probeIntersection evaluates it
* smoothMeshLaplacian (SmoothMesh.cpp:96-123) on a marching-cubes mesh
* computeClosestAtom per welded vertex (Kernels.cu:547-604)

Usage: QSES_REFERENCE=<reference checkout> python tests/golden/gen_ref_golden.py
(or with the sources staged by `make -C oracle/ref_cuda stage`).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import quickses_gb300 as q  # noqa: E402
from oracle import build as ob  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "ref_host.npz")
CASES = [("ball", 60, 11, 0.5), ("ball", 40, 12, 0.3)]


def load_ref():
    path = ob.build_ref()
    if path is None:
        raise SystemExit("reference sources not found (set QSES_REFERENCE)")
    L = ctypes.CDLL(path)
    fp, vp = ctypes.c_float, ctypes.c_void_p
    L.ref_compute_in_or_out.restype = ctypes.c_float
    L.ref_compute_in_or_out.argtypes = [ctypes.c_int] * 3 + [fp] * 4 + [ctypes.c_int, fp, vp, vp]
    L.ref_closest_atom.restype = ctypes.c_int
    L.ref_closest_atom.argtypes = [fp] * 7 + [ctypes.c_int, vp, vp]
    L.ref_hash.restype = ctypes.c_int
    L.ref_hash.argtypes = [fp] * 7 + [ctypes.c_int]
    L.ref_smooth.restype = None
    L.ref_smooth.argtypes = [ctypes.c_int, vp, vp, ctypes.c_uint, ctypes.c_uint]
    return L


def cell_table(xyz, rad, g):
    """cellStartEnd (int2 per cell, EMPTYCELL = INT_MAX - 1) + sorted float4, as sortCell
    builds them (Kernels.cu:306-341)."""
    order, h = O.sort_atoms(xyz, g)
    ncell = g.gnb ** 3
    cse = np.full((ncell, 2), 2 ** 31 - 2, np.int32)
    hs = h[order]
    for s, k in enumerate(hs):
        if s == 0 or hs[s - 1] != k:
            cse[k, 0] = s
        if s == len(hs) - 1 or hs[s + 1] != k:
            cse[k, 1] = s + 1
    srt = np.zeros((len(order), 4), np.float32)
    srt[:, :3] = xyz[order]
    srt[:, 3] = rad[order]
    return np.ascontiguousarray(cse), np.ascontiguousarray(srt), order, h


def main():
    L = load_ref()
    data = {}
    for ci, (kind, n, seed, dx) in enumerate(CASES):
        xyz, rad, _ = q.molecules.ball(n, seed)
        g, _ = O.grid(xyz, rad, dx)
        cse, srt, order, h = cell_table(xyz, rad, g)
        ref_h = np.array([L.ref_hash(*xyz[a], g.ox, g.oy, g.oz, g.cell, g.gnb) for a in range(n)], np.int32)
        G = g.G
        cls = np.zeros((G - 1, G - 1, G - 1), np.int8)
        for i in range(G - 1):
            for j in range(G - 1):
                for k in range(G - 1):
                    v = L.ref_compute_in_or_out(i, j, k, g.ox, g.oy, g.oz, g.cell, g.gnb, g.dx,
                                                cse.ctypes.data_as(ctypes.c_void_p),
                                                srt.ctypes.data_as(ctypes.c_void_p))
                    cls[i, j, k] = 2 if v < 0 else (1 if v == 0 else 0)
        m = O.compute_ses(xyz, rad, dx, smooth=0, fp64=False)
        vq = m.vertices.astype(np.float32)
        tri = m.triangles.astype(np.int32)
        sm = np.ascontiguousarray(vq.copy())
        L.ref_smooth(1, sm.ctypes.data_as(ctypes.c_void_p), np.ascontiguousarray(tri).ctypes.data_as(ctypes.c_void_p),
                     len(vq), len(tri))
        closest = np.array([L.ref_closest_atom(*vq[v], g.ox, g.oy, g.oz, g.cell, g.gnb,
                                               cse.ctypes.data_as(ctypes.c_void_p),
                                               srt.ctypes.data_as(ctypes.c_void_p)) for v in range(len(vq))], np.int32)
        p = "c%d_" % ci
        data.update({p + "xyz": xyz, p + "rad": rad, p + "dx": np.float32(dx), p + "hash": ref_h, p + "class": cls,
                     p + "mesh_v": vq, p + "mesh_t": tri, p + "smooth1": sm, p + "closest": closest})
        print("case", ci, "G", G, "verts", len(vq), "tris", len(tri))
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()

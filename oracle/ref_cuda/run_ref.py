"""Run QuickSES's own CUDA build beside libquickses_gb300 on the same GPU.

TEST INFRASTRUCTURE ONLY.  Needs oracle/_ref/libQuickSES.so and oracle/_ref/libref_field.so
(oracle/ref_cuda/Makefile: `make stage` in the build container, `make` on the GPU machine).

    python oracle/ref_cuda/run_ref.py compare ball1k ball50k   # time + mesh comparison (JSON lines)
    python oracle/ref_cuda/run_ref.py field                    # reference field vs our voxel codes
    python oracle/ref_cuda/run_ref.py fixtures                 # tests/golden/ref_cuda.npz
    python oracle/ref_cuda/run_ref.py stream batched|trajectory|served   # plain path, molecules/s
    python oracle/ref_cuda/run_ref.py smooth ball50k           # SmoothMesh.cpp on the CPU vs ours
    python oracle/ref_cuda/run_ref.py slices                   # tests/golden/ref_slices.npz
    python oracle/ref_cuda/run_ref.py bench ball50k 3          # the reference alone: wall clock of
                                                               # API_computeSES (bench.py's ref_cuda)

Timing is wall clock around the reference's API_computeSES (its whole library call:
upload, slices, host smoothing, concatenation) and around our qses_compute (upload,
pipeline, download), on the same molecule.
"""
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import quickses_gb300 as q  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


class Ref:
    def __init__(self):
        L = ctypes.CDLL(os.path.join(REF, "libQuickSES.so"))
        L.API_computeSES.argtypes = [ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p,
                                     ctypes.POINTER(ctypes.c_uint), ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint),
                                     ctypes.c_int]
        L.API_computeSES.restype = None
        L.API_getVertices.restype = ctypes.POINTER(ctypes.c_float)
        L.API_getTriangles.restype = ctypes.POINTER(ctypes.c_int)
        L.API_getTriangles.argtypes = [ctypes.c_bool]
        L.API_getAtomIdPerVert.restype = ctypes.POINTER(ctypes.c_int)
        self.L = L
        F = ctypes.CDLL(os.path.join(REF, "libref_field.so"))
        F.ref_field.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_float, ctypes.c_void_p,
                                ctypes.c_size_t, ctypes.POINTER(ctypes.c_int)]
        F.ref_field.restype = ctypes.c_int
        self.F = F

    def compute(self, xyz, rad, dx, smooth):
        xyz = np.ascontiguousarray(xyz, np.float32)
        rad = np.ascontiguousarray(rad, np.float32)
        nv, nidx = ctypes.c_uint(0), ctypes.c_uint(0)
        t0 = time.perf_counter()
        self.L.API_computeSES(ctypes.c_float(dx), xyz.ctypes.data, rad.ctypes.data, len(rad), None, ctypes.byref(nv),
                              None, ctypes.byref(nidx), smooth)
        dt = time.perf_counter() - t0
        v = np.ctypeslib.as_array(self.L.API_getVertices(), shape=(nv.value * 3,)).reshape(-1, 3).copy() \
            if nv.value else np.zeros((0, 3), np.float32)
        t = np.ctypeslib.as_array(self.L.API_getTriangles(False), shape=(nidx.value,)).reshape(-1, 3).copy() \
            if nidx.value else np.zeros((0, 3), np.int32)
        a = np.ctypeslib.as_array(self.L.API_getAtomIdPerVert(), shape=(nv.value,)).copy() \
            if nv.value else np.zeros(0, np.int32)
        self.L.API_freeMesh()
        return v, t, a, dt

    def field(self, xyz, rad, dx):
        g, _ = O.grid(xyz, rad, dx)
        out = np.zeros(g.G ** 3, np.float32)
        G = ctypes.c_int(0)
        rc = self.F.ref_field(np.ascontiguousarray(xyz, np.float32).ctypes.data,
                              np.ascontiguousarray(rad, np.float32).ctypes.data, len(rad), ctypes.c_float(dx),
                              out.ctypes.data, out.size, ctypes.byref(G))
        if rc:
            raise RuntimeError("ref_field failed (%d)" % rc)
        return out.reshape(G.value, G.value, G.value)


def used(v, t):
    """Drop vertices no triangle references (the reference leaves the unwritten last
    triangle's vertices behind, MarchingCubes.cu:845 with CudaSurf.cu:421)."""
    keep = np.zeros(len(v), bool)
    keep[t.ravel()] = True
    return v[keep]


def mesh_distances(va, ta, vb, tb, dx):
    d_ab = O.point_surface(used(va, ta).astype(np.float64), vb.astype(np.float64), tb)
    d_ba = O.point_surface(used(vb, tb).astype(np.float64), va.astype(np.float64), ta)
    tol = 0.05 * dx
    return {"max_ref_to_ours_A": float(d_ab.max()), "max_ours_to_ref_A": float(d_ba.max()),
            "p999_ref_to_ours_A": float(np.percentile(d_ab, 99.9)),
            "p999_ours_to_ref_A": float(np.percentile(d_ba, 99.9)),
            "frac_ref_within_0.05dx": float(np.mean(d_ab <= tol)),
            "frac_ours_within_0.05dx": float(np.mean(d_ba <= tol))}


def seam_split(va, ta, vb, tb, g, slice_=300, band=None):
    """Distances from mesh a's used vertices to mesh b, split by whether the vertex lies in
    a seam band of the reference's slicing (within R + 2 voxels of a slice-core boundary,
    CudaSurf.cu:653-682) or away from every seam."""
    S = min(slice_, g.G)
    band = band if band is not None else g.R + 2
    keep = np.zeros(len(va), bool)
    keep[ta.ravel()] = True
    pts = va[keep].astype(np.float64)
    c = (pts - np.array([g.ox, g.oy, g.oz])) / g.dx
    planes = np.arange(S, g.G, S, dtype=np.float64)
    if len(planes) == 0:
        in_band = np.zeros(len(pts), bool)
    else:
        dist = np.min(np.abs(c[:, :, None] - planes[None, None, :]), axis=2)
        in_band = (dist <= band).any(axis=1)
    d = O.point_surface(pts, vb.astype(np.float64), tb)
    out = {"seam_band_voxels": band, "vertices_in_band": int(in_band.sum()), "vertices_off_band": int((~in_band).sum())}
    for name, m in (("off_band", ~in_band), ("in_band", in_band)):
        if m.any():
            out["max_%s_A" % name] = float(d[m].max())
            out["p999_%s_A" % name] = float(np.percentile(d[m], 99.9))
    return out


def vertex_set_overlap(vr, ar, vo, ao):
    """Unsmoothed meshes: exact position matches and closest-atom agreement on them."""
    kr = {tuple(p): i for i, p in enumerate(vr.tolist())}
    common = [(kr[tuple(p)], j) for j, p in enumerate(vo.tolist()) if tuple(p) in kr]
    same_atom = sum(1 for i, j in common if ar[i] == ao[j])
    return {"ref_vertices": len(vr), "our_vertices": len(vo), "common_positions": len(common),
            "atom_id_agreement_on_common": same_atom / max(1, len(common))}


def compare(names):
    ref = Ref()
    with q.Context(0) as ctx:
        for name in names:
            wl = q.molecules.WORKLOADS[name]
            xyz, rad, _ = wl.atoms()
            G = q.grid_info(xyz, rad, wl.voxel).G
            ours_t = []
            for _ in range(3):
                t0 = time.perf_counter()
                mo = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=wl.smooth)
                ours_t.append(time.perf_counter() - t0)
            vr, tr, ar, ref_t = ref.compute(xyz, rad, wl.voxel, wl.smooth)
            res = {"workload": name, "grid": G, "voxels": G ** 3,
                   "ref_s": ref_t, "ref_voxels_per_s": G ** 3 / ref_t,
                   "ours_s": min(ours_t), "ours_voxels_per_s": G ** 3 / min(ours_t),
                   "speedup_e2e": ref_t / min(ours_t),
                   "ref_vertices": len(vr), "ref_triangles": len(tr),
                   "our_vertices": len(mo.vertices), "our_triangles": len(mo.triangles)}
            res.update(mesh_distances(vr, tr, mo.vertices, mo.triangles, wl.voxel))
            if G > 300:  # several reference slices: seam bands vs the rest, unsmoothed and smoothed
                g, _ = O.grid(xyz, rad, wl.voxel)
                vr0, tr0, _, _ = ref.compute(xyz, rad, wl.voxel, 0)
                mo0 = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=0)
                res["ref_to_ours_unsmoothed"] = seam_split(vr0, tr0, mo0.vertices, mo0.triangles, g)
                res["ref_to_ours_smoothed"] = seam_split(vr, tr, mo.vertices, mo.triangles, g)
            if G <= 300:  # one reference slice: unsmoothed vertex sets are comparable one to one
                vr0, tr0, ar0, _ = ref.compute(xyz, rad, wl.voxel, 0)
                mo0 = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=0)
                res.update(vertex_set_overlap(vr0, ar0, mo0.vertices, mo0.atom_sorted))
            print(json.dumps(res), flush=True)


def field_stats(fref, codes, g):
    lut = O.lut(g, False)
    mine = lut[codes]
    G = g.G
    inner = (slice(0, G - 1),) * 3
    d = np.abs(fref[inner].astype(np.float64) - mine[inner].astype(np.float64))
    sref, smine = fref < 0, mine < 0
    flips = int((sref != smine).sum())
    Gc = g.Gc
    def cubes(s):
        c = np.zeros((Gc, Gc, Gc), np.int32)
        corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        for bit, (a, b, e) in enumerate(corners):
            c |= s[a:a + Gc, b:b + Gc, e:e + Gc].astype(np.int32) << bit
        return c
    cdiff = int((cubes(sref) != cubes(smine)).sum())
    cls_ref = np.where(fref == np.float32(1.4), 0, np.where(fref == -np.float32(g.dx), 2, 1))
    cls_mine = np.where(codes == 255, 0, np.where((codes == 254) | (codes == 253), 2, 1))
    return {"grid": G, "max_abs_value_diff_A": float(d.max()), "sign_flips": flips,
            "mc_case_mismatches": cdiff, "mc_cells": Gc ** 3,
            "class_mismatch": int((cls_ref[inner] != cls_mine[inner]).sum())}


def field(cases=((200, 61, 0.5), (300, 62, 0.4), (150, 63, 0.3), (120, 64, 0.2), (1000, 1, 0.5))):
    ref = Ref()
    with q.Context(0) as ctx:
        for n, seed, dx in cases:
            xyz, rad, _ = q.molecules.ball(n, seed)
            g, _ = O.grid(xyz, rad, dx)
            fref = ref.field(xyz, rad, dx)
            ctx.compute(xyz, rad, voxel=dx, smooth=0)
            codes = ctx.debug_codes(g.G)
            res = {"atoms": n, "seed": seed, "dx": dx}
            res.update(field_stats(fref, codes, g))
            print(json.dumps(res), flush=True)


# Molecules of tests/golden/ref_cuda.npz: (atoms, seed, voxel).  c2 is the 1 000-atom
# workload itself (85^3, one slice in the reference); c4 at 0.2 A holds the tie voxels where
# the field is exactly zero in real arithmetic and the reference's fast-math sign is
# arbitrary (code 49: 1.4 - 0.2 * 7).
FIXTURE_CASES = [(80, 71, 0.5), (60, 72, 0.3), (1000, 1, 0.5), (300, 73, 0.4), (120, 74, 0.2)]


def fixtures(out=os.path.join(ROOT, "tests", "golden", "ref_cuda.npz")):
    ref = Ref()
    data = {}
    for ci, (n, seed, dx) in enumerate(FIXTURE_CASES):
        xyz, rad = O.synth_ball(n, seed)
        p = "c%d_" % ci
        data[p + "xyz"], data[p + "rad"], data[p + "dx"] = xyz, rad, np.float32(dx)
        data[p + "field"] = ref.field(xyz, rad, dx).astype(np.float32)
        for sm in (0, 1):
            v, t, a, _ = ref.compute(xyz, rad, dx, sm)
            data[p + "v%d" % sm], data[p + "t%d" % sm], data[p + "a%d" % sm] = v, t, a
    np.savez_compressed(out, **data)
    print("wrote", out, os.path.getsize(out))


def time_only(names):
    """Wall clock of the reference's API_computeSES and of our qses_compute on one workload,
    with mesh counts (no distance computation: for the largest workloads)."""
    ref = Ref()
    with q.Context(0) as ctx:
        for name in names:
            wl = q.molecules.WORKLOADS[name]
            xyz, rad, _ = wl.atoms()
            G = q.grid_info(xyz, rad, wl.voxel).G
            ours = []
            for _ in range(3):
                t0 = time.perf_counter()
                mo = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=wl.smooth)
                ours.append(time.perf_counter() - t0)
            vr, tr, _, ref_t = ref.compute(xyz, rad, wl.voxel, wl.smooth)
            print(json.dumps({"workload": name, "grid": G, "voxels": G ** 3, "ref_s": ref_t, "ours_s": min(ours),
                              "speedup": ref_t / min(ours), "ref_vertices": len(vr), "ref_triangles": len(tr),
                              "our_vertices": len(mo.vertices), "our_triangles": len(mo.triangles)}), flush=True)


def smooth(names):
    """The reference's CPU smoothing (SmoothMesh.cpp, single-threaded, compiled from the
    staged sources by oracle/build.py) on our unsmoothed mesh: its time, and whether our
    GPU pass gives the same positions bit for bit."""
    from oracle import build as ob
    path = ob.build_ref()
    L = ctypes.CDLL(path)
    L.ref_smooth.restype = None
    L.ref_smooth.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
    with q.Context(0) as ctx:
        for name in names:
            wl = q.molecules.WORKLOADS[name]
            xyz, rad, _ = wl.atoms()
            m0 = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=0, keep_degenerate=True)
            ctx.set_profiling(True)
            m1 = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=1, keep_degenerate=True)
            gpu_ms = dict(ctx.stage_times()).get("smooth")
            ctx.set_profiling(False)
            v = np.ascontiguousarray(m0.vertices.copy())
            t = np.ascontiguousarray(m0.triangles, np.int32)
            t0 = time.perf_counter()
            L.ref_smooth(1, v.ctypes.data, t.ctypes.data, len(v), len(t))
            ref_s = time.perf_counter() - t0
            print(json.dumps({"workload": name, "vertices": len(v), "triangles": len(t), "ref_smooth_s": ref_s,
                              "ref_threads": 1, "gpu_smooth_ms": gpu_ms,
                              "speedup": ref_s / (gpu_ms * 1e-3) if gpu_ms else None,
                              "bit_identical": bool(np.array_equal(v, m1.vertices))}), flush=True)


def stream(which, limit=None):
    """The reference's plain path (one API_computeSES per molecule, wall clock per call) on
    the request streams of the batch and served forms; prints molecules/s."""
    streams = {"batched": lambda: q.molecules.uneven_batch(256),
               "trajectory": lambda: q.molecules.trajectory(512),
               "served": lambda: q.molecules.served_stream(64)}
    reqs = streams[which]()
    if limit:
        reqs = reqs[:limit]
    ref = Ref()
    ref.compute(reqs[0]["xyz"], reqs[0]["radii"], reqs[0]["voxel"], reqs[0]["smooth"])  # warm-up
    total, vox = 0.0, 0
    for r in reqs:
        *_, dt = ref.compute(r["xyz"], r["radii"], r["voxel"], r["smooth"])
        total += dt
        vox += q.grid_info(r["xyz"], r["radii"], r["voxel"]).G ** 3
    print(json.dumps({"stream": which, "molecules": len(reqs), "ref_s": total,
                      "ref_molecules_per_s": len(reqs) / total, "ref_voxels_per_s": vox / total}), flush=True)


# Molecules of the per-slice fixtures: (atoms, seed, voxel, slice, smoothing passes).  Small
# slices give many slices on small molecules; voxel 0.75 A has R = 2, where the reference
# emits no cell of any slice that does not start at 0 (MarchingCubes.cu:585-590).
SLICE_CASES = [(150, 91, 0.5, 16, (0, 1)), (120, 92, 0.4, 20, (0, 1)), (100, 93, 0.3, 24, (0,)),
               (150, 94, 0.75, 16, (0,))]


def slices(out=os.path.join(ROOT, "tests", "golden", "ref_slices.npz")):
    """The reference's own per-slice meshes (computeSlicedSES with its SLICE set), through
    oracle/_ref/libref_slices.so: per case and pass count, every slice's vertices, triangles
    (its unwritten last triangle included) and sorted atom ids, concatenated, with counts."""
    L = ctypes.CDLL(os.path.join(REF, "libref_slices.so"))
    L.ref_slices_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_float, ctypes.c_int,
                                 ctypes.c_int]
    L.ref_slices_counts.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.ref_slices_copy.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    data = {}
    for ci, (n, seed, dx, sl, passes) in enumerate(SLICE_CASES):
        xyz, rad = O.synth_ball(n, seed)
        p = "s%d_" % ci
        data[p + "xyz"], data[p + "rad"] = xyz, rad
        data[p + "dx"], data[p + "slice"] = np.float32(dx), np.int32(sl)
        for sm in passes:
            ns = L.ref_slices_run(xyz.ctypes.data, rad.ctypes.data, n, ctypes.c_float(dx), sl, sm)
            vs, ts, as_, cnt = [], [], [], []
            for k in range(ns):
                nv, nt = ctypes.c_int(), ctypes.c_int()
                L.ref_slices_counts(k, ctypes.byref(nv), ctypes.byref(nt))
                v = np.zeros((nv.value, 3), np.float32)
                t = np.zeros((nt.value, 3), np.int32)
                a = np.zeros(nv.value, np.int32)
                L.ref_slices_copy(k, v.ctypes.data, t.ctypes.data, a.ctypes.data)
                vs.append(v); ts.append(t); as_.append(a); cnt.append((nv.value, nt.value))
            q = p + "p%d_" % sm
            data[q + "counts"] = np.array(cnt, np.int32).reshape(-1, 2)
            data[q + "v"] = np.concatenate(vs) if vs else np.zeros((0, 3), np.float32)
            data[q + "t"] = np.concatenate(ts) if ts else np.zeros((0, 3), np.int32)
            data[q + "a"] = np.concatenate(as_) if as_ else np.zeros(0, np.int32)
            print(json.dumps({"case": ci, "passes": sm, "slices": ns, "vertices": int(sum(c[0] for c in cnt)),
                              "triangles": int(sum(c[1] for c in cnt))}), flush=True)
    np.savez_compressed(out, **data)
    print("wrote", out, os.path.getsize(out))


def bench(name, calls):
    """The reference's API_computeSES alone on one workload: one untimed call, then `calls`
    timed ones (wall clock around the library call, host atoms in, mesh in its host
    globals).  Atoms and grid size come from the oracle, so this process loads only the
    reference's library and the oracle."""
    from quickses_gb300.molecules import WORKLOADS  # plain data; loads no library
    wl = WORKLOADS[name]
    xyz, rad = (O.synth_ball if wl.kind == "ball" else O.synth_shell)(wl.n_atoms, wl.seed)
    g, _ = O.grid(xyz, rad, wl.voxel)
    ref = Ref()
    ref.compute(xyz, rad, wl.voxel, wl.smooth)
    secs, v, t = [], None, None
    for _ in range(calls):
        v, t, _a, dt = ref.compute(xyz, rad, wl.voxel, wl.smooth)
        secs.append(dt)
    print(json.dumps({"workload": name, "grid": g.G, "voxels": float(g.G) ** 3, "calls": calls,
                      "ms": [round(1e3 * x, 3) for x in secs], "vertices": len(v), "triangle_indices": 3 * len(t)}),
          flush=True)


if __name__ == "__main__":
    mode = sys.argv[1]
    if mode == "bench":
        bench(sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else 3)
        sys.exit(0)
    if mode == "stream":
        stream(sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else None)
        sys.exit(0)
    if mode == "time":
        time_only(sys.argv[2:])
        sys.exit(0)
    if mode == "smooth":
        smooth(sys.argv[2:] or ["ball50k"])
        sys.exit(0)
    if mode == "compare":
        compare(sys.argv[2:] or ["ball1k"])
    elif mode == "field":
        field()
    elif mode == "fixtures":
        fixtures(*sys.argv[2:3])
    elif mode == "slices":
        slices(*sys.argv[2:3])

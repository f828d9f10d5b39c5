"""Python face of the SES mesher, mirroring QuickSES's library path.

QuickSES's entry point is ``API_computeSES(reso, atomPos, atomRad, N, ...)`` followed by
``API_getVertices / API_getTriangles / API_getAtomIdPerVert / API_freeMesh``
(CudaSurf.cu:787-873).  :func:`compute_ses` is the same call through a reentrant context;
:class:`ReferenceAPI` exposes the ``API_*`` symbols unchanged for callers that want the
exact reference semantics (index count in ``NTri``, sorted atom ids, in-place winding
swap).  Everything runs on the GPU through libquickses_gb300.so; there is no CPU path.
"""
import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L


class QSESError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s (status %d)" % (message, code))
        self.code = code


@dataclass
class Mesh:
    vertices: np.ndarray      # (nv, 3) float32, smoothed
    triangles: np.ndarray     # (nt, 3) int32
    atom_sorted: np.ndarray   # (nv,) int32 closest atom in the cell-sorted order (reference ids)
    atom_input: np.ndarray    # (nv,) int32 closest atom in the caller's order
    grid_dim: int
    origin: tuple


def _take(ptr, n, dt, shape):
    if n == 0:
        return np.zeros(shape, dt)
    return np.ctypeslib.as_array(ptr, shape=(n * (shape[1] if len(shape) > 1 else 1),)).astype(
        dt, copy=True).reshape(shape)


def _host_mesh(m):
    nv, nt = m.n_vertices, m.n_triangles
    return Mesh(_take(m.vertices, nv, np.float32, (nv, 3)), _take(m.triangles, nt, np.int32, (nt, 3)),
                _take(m.atom_sorted, nv, np.int32, (nv,)), _take(m.atom_input, nv, np.int32, (nv,)),
                int(m.grid_dim), tuple(m.origin))


def _requests(requests):
    """ctypes qses_request array for a list of request dicts (arrays kept alive by the caller)."""
    arrays, reqs = [], (L.Request * max(1, len(requests)))()
    for i, r in enumerate(requests):
        xyz, rad = _f32(r["xyz"], 3), _f32(r["radii"])
        if rad.shape != (xyz.shape[0],):
            raise ValueError("radii must have shape (N,)")
        arrays.append((xyz, rad))
        reqs[i].atoms, reqs[i].radii, reqs[i].n = xyz.ctypes.data, rad.ctypes.data, xyz.shape[0]
        reqs[i].voxel = float(r.get("voxel", 0.5))
        reqs[i].smooth_passes = int(r.get("smooth", 1))
        reqs[i].flags = (L.QSES_FLAG_KEEP_DEGENERATE if r.get("keep_degenerate", False) else 0) | \
            int(r.get("flags", 0))
    return arrays, reqs


def _f32(a, shape_last=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape_last is not None and (a.ndim != 2 or a.shape[1] != shape_last):
        raise ValueError("expected an (N, %d) array" % shape_last)
    return a


class Context:
    """One CUDA stream and its reusable device workspace (qses_context)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        self._lib = L.lib()
        h = ctypes.c_void_p()
        rc = self._lib.qses_context_create(device, ctypes.c_void_p(stream) if stream else None, ctypes.byref(h))
        if rc != L.QSES_OK:
            raise QSESError(rc, "qses_context_create: " + L.status_string(rc))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qses_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _params(self, voxel, smooth, keep_degenerate, slice_, reference_slices=False):
        p = L.Params()
        self._lib.qses_params_default(ctypes.byref(p))
        p.voxel = float(voxel)
        p.smooth_passes = int(smooth)
        p.slice = int(slice_)
        p.flags = (L.QSES_FLAG_KEEP_DEGENERATE if keep_degenerate else 0) | \
            (L.QSES_FLAG_REFERENCE_SLICES if reference_slices else 0)
        return p

    def _check(self, rc, what):
        if rc != L.QSES_OK:
            raise QSESError(rc, "%s: %s" % (what, self._lib.qses_last_error(self._h).decode()))

    def compute(self, xyz, radii, voxel=0.5, smooth=1, keep_degenerate=False, slice=300,
                reference_slices=False) -> Mesh:
        """Atoms (N, 3) + radii (N,) on the host -> welded, smoothed mesh on the host.
        reference_slices: the reference's per-slice output for slices of `slice` voxels
        (QSES_FLAG_REFERENCE_SLICES); slice_counts() then gives each slice's counts."""
        xyz = _f32(xyz, 3)
        radii = _f32(radii)
        if radii.shape != (xyz.shape[0],):
            raise ValueError("radii must have shape (N,)")
        m = L.Mesh()
        rc = self._lib.qses_compute(self._h, ctypes.byref(self._params(voxel, smooth, keep_degenerate, slice,
                                                                       reference_slices)),
                                    xyz.ctypes.data_as(ctypes.c_void_p),
                                    radii.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), xyz.shape[0],
                                    ctypes.byref(m))
        self._check(rc, "qses_compute")
        try:
            out = _host_mesh(m)
        finally:
            self._lib.qses_mesh_release(ctypes.byref(m))
        return out

    def slice_counts(self):
        """(vertices, triangles) per slice of the last call in the reference's slicing mode."""
        k = self._lib.qses_last_slices(self._h, None, None, 0)
        nv = (ctypes.c_uint * max(1, k))()
        nt = (ctypes.c_uint * max(1, k))()
        self._lib.qses_last_slices(self._h, nv, nt, k)
        return [(int(nv[i]), int(nt[i])) for i in range(k)]

    def compute_batch(self, requests):
        """Batch form: `requests` is a list of dicts with keys xyz, radii and optionally
        voxel (0.5), smooth (1), keep_degenerate (False).  Returns one entry per request:
        a Mesh, or a QSESError for a request outside the supported envelope."""
        arrays, reqs = _requests(requests)
        n = len(requests)
        meshes = (L.Mesh * max(1, n))()
        status = (ctypes.c_int * max(1, n))()
        rc = self._lib.qses_compute_batch(self._h, reqs, n, meshes, status)
        out = []
        try:
            self._check(rc, "qses_compute_batch")
            for i in range(n):
                if status[i] != L.QSES_OK:
                    out.append(QSESError(status[i], "request %d: %s" % (i, L.status_string(status[i]))))
                else:
                    out.append(_host_mesh(meshes[i]))
        finally:
            for i in range(n):
                self._lib.qses_mesh_release(ctypes.byref(meshes[i]))
        return out

    def set_smoothing_shape(self, threads=0, target=16384, cache_flags=0, wave_vertices=0):
        """Fix the smoothing launch shape (threads 512/1024, slab target, cache flags, most
        vertices per slab-kernel wave); threads 0 = tuned/default.  cache_flags: bit 0 L1
        prefetch of successors' lists, bit 1 positions through L1, bit 2 persisting-L2
        window, bit 3 slab positions in shared memory, bit 4 / bit 5 two / four vertex
        updates per worker warp."""
        self._check(self._lib.qses_set_smoothing_shape(self._h, int(threads), int(target), int(cache_flags),
                                                       int(wave_vertices)), "qses_set_smoothing_shape")

    def autotune(self, xyz, radii, voxel=0.5, smooth=1, repeats=1):
        """Times every smoothing launch shape and refine tile shape on this molecule and keeps
        the fastest for its size class; returns (threads, slab target, cache flags, refine
        tile shape, smoothing ms)."""
        xyz, radii = _f32(xyz, 3), _f32(radii)
        th, tg, fl, fs, ms = ctypes.c_int(0), ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_int(0), ctypes.c_float(0)
        rc = self._lib.qses_autotune(self._h, ctypes.byref(self._params(voxel, smooth, False, 300)),
                                     xyz.ctypes.data_as(ctypes.c_void_p),
                                     radii.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), xyz.shape[0], int(repeats),
                                     ctypes.byref(th), ctypes.byref(tg), ctypes.byref(fl), ctypes.byref(fs),
                                     ctypes.byref(ms))
        self._check(rc, "qses_autotune")
        return th.value, tg.value, fl.value, fs.value, ms.value

    def set_field_shape(self, shape=-1):
        """Fix the refine tile shape (0: 8 x 8 rows, 1: 16 x 8, 2: 16 x 16, 3: 32 x 16); -1 = tuned/default."""
        self._check(self._lib.qses_set_field_shape(self._h, int(shape)), "qses_set_field_shape")

    def autotune_batch(self, requests, repeats=1):
        arrays, reqs = _requests(requests)
        th, tg, fl, ms = ctypes.c_int(0), ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_float(0)
        rc = self._lib.qses_autotune_batch(self._h, reqs, len(requests), int(repeats), ctypes.byref(th),
                                           ctypes.byref(tg), ctypes.byref(fl), ctypes.byref(ms))
        self._check(rc, "qses_autotune_batch")
        return th.value, tg.value, fl.value, ms.value

    def compute_device(self, d_xyz_ptr, d_radii_ptr, n, voxel=0.5, smooth=1, keep_degenerate=False):
        """Device-resident form (pointers to device float arrays); returns counts and the
        device pointers of the mesh, valid until the next call on this context."""
        dm = L.DeviceMesh()
        rc = self._lib.qses_compute_device(self._h, ctypes.byref(self._params(voxel, smooth, keep_degenerate, 300)),
                                           ctypes.c_void_p(d_xyz_ptr), ctypes.c_void_p(d_radii_ptr), n,
                                           ctypes.byref(dm))
        self._check(rc, "qses_compute_device")
        return dm

    def debug_codes(self, G):
        codes = np.zeros((G, G, G), np.uint8)
        rc = self._lib.qses_debug_codes(self._h, codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), codes.nbytes)
        self._check(rc, "qses_debug_codes")
        return codes

    def debug_atom_order(self, n):
        order = np.zeros(n, np.uint32)
        keys = np.zeros(n, np.uint32)
        rc = self._lib.qses_debug_atom_order(self._h, order.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                             keys.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), n)
        self._check(rc, "qses_debug_atom_order")
        return order, keys

    def set_profiling(self, on=True):
        self._lib.qses_set_profiling(self._h, int(on))

    def stage_times(self):
        ms = (ctypes.c_float * 32)()
        names = (ctypes.c_char_p * 32)()
        k = self._lib.qses_stage_times(self._h, ms, names, 32)
        return [(names[q].decode(), float(ms[q])) for q in range(k)]

    def last_launch_count(self):
        return int(self._lib.qses_last_launch_count(self._h))

    def set_graphs(self, enable=True):
        """Run the pipeline segments through CUDA graphs (default) or launch every kernel directly."""
        self._check(self._lib.qses_set_graphs(self._h, int(bool(enable))), "qses_set_graphs")

    def host_timeline(self):
        """Host timeline of the last pipeline run (ms): before the first launch, field segment,
        gap, mesh segment, gap, finish segment."""
        out = (ctypes.c_double * 6)()
        k = self._lib.qses_host_timeline(self._h, out, 6)
        names = ["host_prep", "field", "host_mid1", "mesh", "host_mid2", "finish"]
        return {names[q]: float(out[q]) for q in range(k)}

    def graph_stats(self):
        out = (ctypes.c_ulonglong * 4)()
        k = self._lib.qses_graph_stats(self._h, out, 4)
        names = ["captures", "instantiations", "updates", "replays"]
        return {names[q]: int(out[q]) for q in range(k)}

    def diagnostics(self):
        out = (ctypes.c_ulonglong * 10)()
        k = self._lib.qses_diagnostics(self._h, out, 10)
        names = ["slabs", "slab_size", "max_polls", "unfinished_slabs", "update_cycles", "release_cycles",
                 "vertices", "id_wait_cycles", "position_wait_cycles", "store_fence_cycles"]
        return {names[q]: int(out[q]) for q in range(min(k, len(names)))}


def grid_info(xyz, radii, voxel):
    xyz, radii = _f32(xyz, 3), _f32(radii)
    gi = L.GridInfo()
    rc = L.lib().qses_grid_info_for(xyz.ctypes.data_as(ctypes.c_void_p),
                                    radii.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), xyz.shape[0],
                                    ctypes.c_float(voxel), ctypes.byref(gi))
    if rc != L.QSES_OK:
        raise QSESError(rc, "qses_grid_info_for: " + L.status_string(rc))
    return gi


_default_ctx = None


def compute_ses(xyz, radii, voxel=0.5, smooth=1, keep_degenerate=False) -> Mesh:
    """computeSlicedSES + API_computeSES in one call (CudaSurf.cu:524-841)."""
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx.compute(xyz, radii, voxel=voxel, smooth=smooth, keep_degenerate=keep_degenerate)


class ReferenceAPI:
    """The API_* symbols exactly as QuickSES exports them (CudaSurf.h:75-83)."""

    def __init__(self):
        self._lib = L.lib()

    def computeSES(self, reso, xyz, radii, smooth=1):
        xyz, radii = _f32(xyz, 3), _f32(radii)
        nv, ntri = ctypes.c_uint(0), ctypes.c_uint(0)
        self._lib.API_computeSES(ctypes.c_float(reso), xyz.ctypes.data_as(ctypes.c_void_p),
                                 radii.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), xyz.shape[0], None,
                                 ctypes.byref(nv), None, ctypes.byref(ntri), int(smooth))
        rc = self._lib.qses_api_last_status()
        if rc != L.QSES_OK:
            raise QSESError(rc, "API_computeSES: " + L.status_string(rc))
        return nv.value, ntri.value

    def getVertices(self, nv):
        p = self._lib.API_getVertices()
        return np.ctypeslib.as_array(p, shape=(nv * 3,)).reshape(nv, 3).copy() if nv else np.zeros((0, 3), np.float32)

    def getTriangles(self, nidx, invert=False):
        p = self._lib.API_getTriangles(bool(invert))
        return np.ctypeslib.as_array(p, shape=(nidx,)).copy() if nidx else np.zeros(0, np.int32)

    def getAtomIdPerVert(self, nv):
        p = self._lib.API_getAtomIdPerVert()
        return np.ctypeslib.as_array(p, shape=(nv,)).copy() if nv else np.zeros(0, np.int32)

    def freeMesh(self):
        self._lib.API_freeMesh()

    def exported_counts(self):
        return (ctypes.c_int.in_dll(self._lib, "NVertices").value, ctypes.c_int.in_dll(self._lib, "NTriangles").value)


def read_pdb(path):
    """ATOM records of a PDB file -> (xyz (N, 3) float32, radii (N,) float32), as the
    QuickSES executable reads them (cpdb/cpdb.cpp:35-158, CudaSurf.cu:942-964)."""
    lib = L.lib()
    px, pr, n = ctypes.POINTER(ctypes.c_float)(), ctypes.POINTER(ctypes.c_float)(), ctypes.c_uint(0)
    rc = lib.qses_read_pdb(str(path).encode(), ctypes.byref(px), ctypes.byref(pr), ctypes.byref(n))
    if rc != L.QSES_OK:
        raise QSESError(rc, "qses_read_pdb(%s): %s" % (path, L.status_string(rc)))
    try:
        k = n.value
        xyz = np.ctypeslib.as_array(px, shape=(3 * k,)).reshape(k, 3).copy() if k else np.zeros((0, 3), np.float32)
        rad = np.ctypeslib.as_array(pr, shape=(k,)).copy() if k else np.zeros(0, np.float32)
    finally:
        lib.qses_free(ctypes.cast(px, ctypes.c_void_p))
        lib.qses_free(ctypes.cast(pr, ctypes.c_void_p))
    return xyz, rad


def write_obj(path, vertices, triangles, threads=0):
    """OBJ text exactly as QuickSES's writeToObj writes one mesh (CudaSurf.cu:329-371)."""
    v = _f32(vertices, 3)
    t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
    rc = L.lib().qses_write_obj(str(path).encode(), v.ctypes.data_as(ctypes.c_void_p), v.shape[0],
                                t.ctypes.data_as(ctypes.c_void_p), t.shape[0], int(threads))
    if rc != L.QSES_OK:
        raise QSESError(rc, "qses_write_obj(%s): %s" % (path, L.status_string(rc)))


def format_fixed3(x):
    buf = ctypes.create_string_buffer(64)
    k = L.lib().qses_format_fixed3(ctypes.c_float(x), buf, 64)
    return buf.value[:k].decode()


class Server:
    """Served form (qses_server_*): continuous batching over `lanes` streams under a
    device-memory budget.  submit() copies the atoms and returns a ticket; wait() returns
    (Mesh, timing) for it, or raises QSESError with the request's status."""

    def __init__(self, device=0, lanes=2, memory_budget=120 << 30, max_batch=256, max_batch_voxels=None):
        self._lib = L.lib()
        cfg = L.ServerConfig()
        self._lib.qses_server_config_default(ctypes.byref(cfg))
        cfg.device, cfg.lanes, cfg.memory_budget, cfg.max_batch = device, lanes, memory_budget, max_batch
        if max_batch_voxels is not None:
            cfg.max_batch_voxels = int(max_batch_voxels)
        h = ctypes.c_void_p()
        rc = self._lib.qses_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != L.QSES_OK:
            raise QSESError(rc, "qses_server_create: " + L.status_string(rc))
        self._h = h

    @property
    def handle(self):
        return self._h

    def submit(self, xyz, radii, voxel=0.5, smooth=1, keep_degenerate=False):
        xyz, radii = _f32(xyz, 3), _f32(radii)
        r = L.Request(xyz.ctypes.data, radii.ctypes.data, xyz.shape[0], float(voxel), int(smooth),
                      L.QSES_FLAG_KEEP_DEGENERATE if keep_degenerate else 0)
        t = ctypes.c_ulonglong(0)
        rc = self._lib.qses_server_submit(self._h, ctypes.byref(r), ctypes.byref(t))
        if rc != L.QSES_OK:
            raise QSESError(rc, "qses_server_submit: " + L.status_string(rc))
        return t.value

    def wait(self, ticket, timeout=-1.0):
        m, info = L.Mesh(), L.TicketInfo()
        rc = self._lib.qses_server_wait(self._h, ctypes.c_ulonglong(ticket), float(timeout), ctypes.byref(m),
                                        ctypes.byref(info))
        try:
            if rc != L.QSES_OK:
                raise QSESError(rc, "request %d: %s" % (ticket, L.status_string(rc)))
            mesh = _host_mesh(m)
        finally:
            self._lib.qses_mesh_release(ctypes.byref(m))
        return mesh, {"queued_s": info.queued_s, "run_s": info.run_s, "total_s": info.total_s}

    def cancel(self, ticket):
        """Withdraw a queued request (True); False when it is already running."""
        rc = self._lib.qses_server_cancel(self._h, ctypes.c_ulonglong(ticket))
        if rc == L.QSES_OK:
            return True
        if rc == 5:  # QSES_ERR_UNSUPPORTED: taken into a batch already
            return False
        raise QSESError(rc, "qses_server_cancel: %s" % L.status_string(rc))

    def stats(self):
        out = (ctypes.c_ulonglong * 5)()
        k = self._lib.qses_server_stats(self._h, out, 5)
        names = ["batches", "served", "max_batch", "max_lanes_busy", "queued"]
        return {names[i]: int(out[i]) for i in range(k)}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qses_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

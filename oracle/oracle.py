"""ctypes wrapper over the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's CPU-baseline
leg.  It is the checker for the CUDA path and is never called by the product.
"""
import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CODE_NONE, CODE_IN, CODE_OUT = 253, 254, 255


class Grid(ctypes.Structure):
    _fields_ = [("ox", ctypes.c_float), ("oy", ctypes.c_float), ("oz", ctypes.c_float),
                ("cell", ctypes.c_float), ("dx", ctypes.c_float), ("probe", ctypes.c_float),
                ("maxR", ctypes.c_float), ("maxDist", ctypes.c_float),
                ("gnb", ctypes.c_int), ("G", ctypes.c_int), ("R", ctypes.c_int),
                ("Gc", ctypes.c_int), ("N", ctypes.c_int)]


class _Mesh(ctypes.Structure):
    _fields_ = [("nv", ctypes.c_uint), ("nt", ctypes.c_uint), ("nt_kept", ctypes.c_uint),
                ("ne", ctypes.c_uint),
                ("v", ctypes.POINTER(ctypes.c_double)), ("vq", ctypes.POINTER(ctypes.c_double)),
                ("tri", ctypes.POINTER(ctypes.c_int32)), ("tri_kept", ctypes.POINTER(ctypes.c_int32)),
                ("atom_sorted", ctypes.POINTER(ctypes.c_int32)),
                ("atom_input", ctypes.POINTER(ctypes.c_int32)),
                ("edge_vertex", ctypes.POINTER(ctypes.c_int32)),
                ("nslices", ctypes.c_uint), ("slice_v", ctypes.POINTER(ctypes.c_uint32)),
                ("slice_t", ctypes.POINTER(ctypes.c_uint32)), ("slice_tk", ctypes.POINTER(ctypes.c_uint32))]


@dataclass
class Mesh:
    vertices: np.ndarray      # (nv, 3) float64 smoothed positions
    vertices_q: np.ndarray    # (nv, 3) welded positions before smoothing
    triangles: np.ndarray     # (nt, 3) int32, emission order, degenerate included
    triangles_kept: np.ndarray
    atom_sorted: np.ndarray
    atom_input: np.ndarray
    n_edges: int
    slice_v: np.ndarray = None   # reference slicing mode: first vertex / triangle / kept
    slice_t: np.ndarray = None   # triangle of each slice, then the totals
    slice_tk: np.ndarray = None


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from oracle import build as _b  # noqa: WPS433
            _b.build_oracle()
        L = ctypes.CDLL(path)
        fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_grid_setup.argtypes = [fp, fp, ctypes.c_uint, ctypes.c_float, ctypes.POINTER(Grid)]
        L.oracle_sort_atoms.argtypes = [fp, ctypes.c_uint, ctypes.POINTER(Grid),
                                        ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int32)]
        L.oracle_code_lut_f32.argtypes = [ctypes.POINTER(Grid), fp]
        L.oracle_code_lut_f64.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(ctypes.c_double)]
        L.oracle_field_codes.argtypes = [fp, fp, ctypes.c_uint, ctypes.POINTER(Grid), ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_uint8), ctypes.c_int]
        L.oracle_mesh_from_codes.argtypes = [ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(Grid), ctypes.c_int,
                                             fp, ctypes.c_uint, ctypes.c_int, ctypes.c_int]
        L.oracle_mesh_from_codes.restype = ctypes.POINTER(_Mesh)
        L.oracle_compute_ses.argtypes = [fp, fp, ctypes.c_uint, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int]
        L.oracle_compute_ses.restype = ctypes.POINTER(_Mesh)
        L.oracle_compute_ses_slices.argtypes = [fp, fp, ctypes.c_uint, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int]
        L.oracle_compute_ses_slices.restype = ctypes.POINTER(_Mesh)
        L.oracle_mesh_free.argtypes = [ctypes.POINTER(_Mesh)]
        L.oracle_smooth_f32.argtypes = [fp, ctypes.c_uint, ctypes.POINTER(ctypes.c_int32), ctypes.c_uint,
                                        ctypes.c_int]
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.oracle_hausdorff.argtypes = [dp, ctypes.c_uint, ip, ctypes.c_uint, dp, ctypes.c_uint, ip, ctypes.c_uint,
                                       dp, dp, ctypes.c_int]
        L.oracle_hausdorff.restype = ctypes.c_double
        L.oracle_point_surface.argtypes = [dp, ctypes.c_uint, dp, ctypes.c_uint, ip, ctypes.c_uint, dp, ctypes.c_int]
        L.oracle_point_surface.restype = ctypes.c_double
        L.oracle_smooth_depth.argtypes = [ip, ctypes.c_uint, ctypes.c_uint, ip]
        L.oracle_smooth_depth.restype = ctypes.c_int
        L.oracle_synth_ball.argtypes = [ctypes.c_uint, ctypes.c_uint64, ctypes.c_float, ctypes.c_float, fp, fp]
        L.oracle_synth_shell.argtypes = [ctypes.c_uint, ctypes.c_uint64, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float, fp, fp]
        _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def grid(xyz, rad, dx):
    xyz, rad = _f(xyz), _f(rad)
    g = Grid()
    rc = lib().oracle_grid_setup(_ptr(xyz, ctypes.c_float), _ptr(rad, ctypes.c_float), len(rad),
                                 ctypes.c_float(dx), ctypes.byref(g))
    return g, rc


def sort_atoms(xyz, g):
    xyz = _f(xyz)
    n = xyz.shape[0]
    order = np.zeros(n, np.uint32)
    h = np.zeros(n, np.int32)
    lib().oracle_sort_atoms(_ptr(xyz, ctypes.c_float), n, ctypes.byref(g), _ptr(order, ctypes.c_uint32),
                            _ptr(h, ctypes.c_int32))
    return order, h


def lut(g, fp64=False):
    if fp64:
        out = np.zeros(256, np.float64)
        lib().oracle_code_lut_f64(ctypes.byref(g), _ptr(out, ctypes.c_double))
    else:
        out = np.zeros(256, np.float32)
        lib().oracle_code_lut_f32(ctypes.byref(g), _ptr(out, ctypes.c_float))
    return out


def field_codes(xyz, rad, g, fp64=False, x0=0, x1=None, threads=0):
    xyz, rad = _f(xyz), _f(rad)
    x1 = g.G if x1 is None else x1
    codes = np.zeros((x1 - x0, g.G, g.G), np.uint8)
    rc = lib().oracle_field_codes(_ptr(xyz, ctypes.c_float), _ptr(rad, ctypes.c_float), len(rad),
                                  ctypes.byref(g), int(fp64), x0, x1, _ptr(codes, ctypes.c_uint8), threads)
    if rc != 0:
        raise ValueError("oracle_field_codes failed (%d)" % rc)
    return codes


def _take(mp):
    if not mp:
        raise RuntimeError("oracle returned no mesh")
    m = mp.contents

    def arr(p, n, dt, shape=None):
        if n == 0:
            return np.zeros((0,) if shape is None else (0, shape), dt)
        a = np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)
        return a if shape is None else a.reshape(-1, shape)

    out = Mesh(arr(m.v, 3 * m.nv, np.float64, 3), arr(m.vq, 3 * m.nv, np.float64, 3),
               arr(m.tri, 3 * m.nt, np.int32, 3), arr(m.tri_kept, 3 * m.nt_kept, np.int32, 3),
               arr(m.atom_sorted, m.nv, np.int32), arr(m.atom_input, m.nv, np.int32), int(m.ne))
    if m.slice_v:
        out.slice_v = arr(m.slice_v, m.nslices + 1, np.int64)
        out.slice_t = arr(m.slice_t, m.nslices + 1, np.int64)
        out.slice_tk = arr(m.slice_tk, m.nslices + 1, np.int64)
    lib().oracle_mesh_free(mp)
    return out


def mesh_from_codes(codes, g, xyz, fp64=False, smooth=1, threads=0):
    codes = np.ascontiguousarray(codes, np.uint8)
    xyz = _f(xyz)
    return _take(lib().oracle_mesh_from_codes(_ptr(codes, ctypes.c_uint8), ctypes.byref(g), int(fp64),
                                              _ptr(xyz, ctypes.c_float), xyz.shape[0], smooth, threads))


def compute_ses(xyz, rad, dx, smooth=1, fp64=False, threads=0):
    xyz, rad = _f(xyz), _f(rad)
    return _take(lib().oracle_compute_ses(_ptr(xyz, ctypes.c_float), _ptr(rad, ctypes.c_float), len(rad),
                                          ctypes.c_float(dx), smooth, int(fp64), threads))


def compute_ses_slices(xyz, rad, dx, slice_, smooth=1, fp64=False, threads=0):
    """The reference's slicing (-s slice_): per-slice meshes concatenated as API_computeSES
    does; slice_v / slice_t / slice_tk give each slice's first vertex and triangle."""
    xyz, rad = _f(xyz), _f(rad)
    return _take(lib().oracle_compute_ses_slices(_ptr(xyz, ctypes.c_float), _ptr(rad, ctypes.c_float), len(rad),
                                                 ctypes.c_float(dx), int(slice_), smooth, int(fp64), threads))


def smooth_f32(vertices, triangles, passes):
    v = np.ascontiguousarray(vertices, np.float32).copy()
    t = np.ascontiguousarray(triangles, np.int32)
    lib().oracle_smooth_f32(_ptr(v, ctypes.c_float), v.shape[0], _ptr(t, ctypes.c_int32), t.shape[0], passes)
    return v


def hausdorff(va, ta, vb, tb, threads=0):
    va = np.ascontiguousarray(va, np.float64); vb = np.ascontiguousarray(vb, np.float64)
    ta = np.ascontiguousarray(ta, np.int32); tb = np.ascontiguousarray(tb, np.int32)
    ab, ba = ctypes.c_double(), ctypes.c_double()
    h = lib().oracle_hausdorff(_ptr(va, ctypes.c_double), va.shape[0], _ptr(ta, ctypes.c_int32), ta.shape[0],
                               _ptr(vb, ctypes.c_double), vb.shape[0], _ptr(tb, ctypes.c_int32), tb.shape[0],
                               ctypes.byref(ab), ctypes.byref(ba), threads)
    return h, ab.value, ba.value


def point_surface(va, vb, tb, threads=0):
    """Distance from every point of va to the triangle surface (vb, tb)."""
    va = np.ascontiguousarray(va, np.float64); vb = np.ascontiguousarray(vb, np.float64)
    tb = np.ascontiguousarray(tb, np.int32)
    out = np.zeros(va.shape[0], np.float64)
    lib().oracle_point_surface(_ptr(va, ctypes.c_double), va.shape[0], _ptr(vb, ctypes.c_double), vb.shape[0],
                               _ptr(tb, ctypes.c_int32), tb.shape[0], _ptr(out, ctypes.c_double), threads)
    return out


def smooth_depth(triangles, nv):
    t = np.ascontiguousarray(triangles, np.int32)
    level = np.zeros(nv, np.int32)
    d = lib().oracle_smooth_depth(_ptr(t, ctypes.c_int32), t.shape[0], nv, _ptr(level, ctypes.c_int32))
    return d, level


def synth_ball(n, seed=1, density=0.05, min_dist=1.2):
    """The seeded ball molecule (oracle_synth.cpp): the same atoms as the library's
    generator, made without loading the library."""
    xyz = np.zeros((n, 3), np.float32)
    rad = np.zeros(n, np.float32)
    if lib().oracle_synth_ball(n, seed, density, min_dist, _ptr(xyz, ctypes.c_float), _ptr(rad, ctypes.c_float)):
        raise ValueError("oracle_synth_ball failed")
    return xyz, rad


def synth_shell(n, seed=1, r_in=400.0, thickness=30.0, min_dist=1.2):
    """The seeded shell molecule (oracle_synth.cpp), as synth_ball."""
    xyz = np.zeros((n, 3), np.float32)
    rad = np.zeros(n, np.float32)
    if lib().oracle_synth_shell(n, seed, r_in, thickness, min_dist, _ptr(xyz, ctypes.c_float),
                                _ptr(rad, ctypes.c_float)):
        raise ValueError("oracle_synth_shell failed")
    return xyz, rad

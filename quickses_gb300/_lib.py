"""ctypes binding of libquickses_gb300.so (declarations mirror include/quickses.h).

Loading fails loudly when the library has not been built: there is no fallback path.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libquickses_gb300.so")

QSES_OK = 0
QSES_ERR_INVALID_ARG = 1
QSES_ERR_NO_DEVICE = 2
QSES_ERR_CUDA = 3
QSES_ERR_OUT_OF_MEMORY = 4
QSES_ERR_UNSUPPORTED = 5
QSES_ERR_TIMEOUT = 6
QSES_ERR_INTERNAL = 7
QSES_ERR_CANCELLED = 8
QSES_FLAG_KEEP_DEGENERATE = 1
QSES_FLAG_REFERENCE_SLICES = 2


class Float3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


class Params(ctypes.Structure):
    _fields_ = [("voxel", ctypes.c_float), ("smooth_passes", ctypes.c_int), ("slice", ctypes.c_int),
                ("flags", ctypes.c_int)]


class Mesh(ctypes.Structure):
    _fields_ = [("n_vertices", ctypes.c_uint), ("n_triangles", ctypes.c_uint),
                ("vertices", ctypes.POINTER(ctypes.c_float)), ("triangles", ctypes.POINTER(ctypes.c_int)),
                ("atom_sorted", ctypes.POINTER(ctypes.c_int)), ("atom_input", ctypes.POINTER(ctypes.c_int)),
                ("grid_dim", ctypes.c_int), ("origin", ctypes.c_float * 3), ("_owner", ctypes.c_void_p)]


class DeviceMesh(ctypes.Structure):
    _fields_ = [("n_vertices", ctypes.c_uint), ("n_triangles", ctypes.c_uint),
                ("d_vertices", ctypes.c_void_p), ("d_triangles", ctypes.c_void_p),
                ("d_atom_sorted", ctypes.c_void_p), ("d_atom_input", ctypes.c_void_p)]


class Request(ctypes.Structure):
    _fields_ = [("atoms", ctypes.c_void_p), ("radii", ctypes.c_void_p), ("n", ctypes.c_uint),
                ("voxel", ctypes.c_float), ("smooth_passes", ctypes.c_int), ("flags", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("lanes", ctypes.c_int), ("memory_budget", ctypes.c_ulonglong),
                ("max_batch", ctypes.c_uint), ("max_batch_voxels", ctypes.c_ulonglong)]


class TicketInfo(ctypes.Structure):
    _fields_ = [("queued_s", ctypes.c_double), ("run_s", ctypes.c_double), ("total_s", ctypes.c_double)]


class GridInfo(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("cell", ctypes.c_float), ("dx", ctypes.c_float),
                ("probe", ctypes.c_float), ("max_radius", ctypes.c_float), ("max_dist", ctypes.c_float),
                ("gnb", ctypes.c_int), ("G", ctypes.c_int), ("R", ctypes.c_int), ("Gc", ctypes.c_int),
                ("W", ctypes.c_int)]


# Every symbol include/quickses.h declares, with its ctypes signature (None = data symbol).
_FP = ctypes.POINTER(ctypes.c_float)
_VP = ctypes.c_void_p
SIGNATURES = {
    "API_computeSES": (None, [ctypes.c_float, _VP, _FP, ctypes.c_uint, _VP, ctypes.POINTER(ctypes.c_uint), _VP,
                              ctypes.POINTER(ctypes.c_uint), ctypes.c_int]),
    "API_getTriangles": (ctypes.POINTER(ctypes.c_int), [ctypes.c_bool]),
    "API_getVertices": (_FP, []),
    "API_freeMesh": (None, []),
    "API_getAtomIdPerVert": (ctypes.POINTER(ctypes.c_int), []),
    "qses_api_last_status": (ctypes.c_int, []),
    "qses_context_create": (ctypes.c_int, [ctypes.c_int, _VP, ctypes.POINTER(_VP)]),
    "qses_context_destroy": (ctypes.c_int, [_VP]),
    "qses_params_default": (None, [ctypes.POINTER(Params)]),
    "qses_compute": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _FP, ctypes.c_uint, ctypes.POINTER(Mesh)]),
    "qses_last_slices": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint), ctypes.c_int]),
    "qses_mesh_release": (None, [ctypes.POINTER(Mesh)]),
    "qses_compute_device": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _VP, ctypes.c_uint,
                                           ctypes.POINTER(DeviceMesh)]),
    "qses_compute_batch": (ctypes.c_int, [_VP, ctypes.POINTER(Request), ctypes.c_uint, ctypes.POINTER(Mesh),
                                          ctypes.POINTER(ctypes.c_int)]),
    "qses_set_pinned_cache": (None, [ctypes.c_ulonglong]),
    "qses_set_smoothing_shape": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint]),
    "qses_autotune": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _FP, ctypes.c_uint, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint),
                                     ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_int), _FP]),
    "qses_set_field_shape": (ctypes.c_int, [_VP, ctypes.c_int]),
    "qses_set_default_smoothing_shape": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_uint]),
    "qses_autotune_batch": (ctypes.c_int, [_VP, ctypes.POINTER(Request), ctypes.c_uint, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint),
                                           ctypes.POINTER(ctypes.c_uint), _FP]),
    "qses_server_config_default": (None, [ctypes.POINTER(ServerConfig)]),
    "qses_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_VP)]),
    "qses_server_submit": (ctypes.c_int, [_VP, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_ulonglong)]),
    "qses_server_wait": (ctypes.c_int, [_VP, ctypes.c_ulonglong, ctypes.c_double, ctypes.POINTER(Mesh),
                                        ctypes.POINTER(TicketInfo)]),
    "qses_server_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]),
    "qses_server_destroy": (ctypes.c_int, [_VP]),
    "qses_server_cancel": (ctypes.c_int, [_VP, ctypes.c_ulonglong]),
    "qses_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "qses_last_error": (ctypes.c_char_p, [_VP]),
    "qses_set_profiling": (ctypes.c_int, [_VP, ctypes.c_int]),
    "qses_stage_times": (ctypes.c_int, [_VP, _FP, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]),
    "qses_last_launch_count": (ctypes.c_int, [_VP]),
    "qses_last_download_bytes": (ctypes.c_ulonglong, [_VP]),
    "qses_diagnostics": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]),
    "qses_set_graphs": (ctypes.c_int, [_VP, ctypes.c_int]),
    "qses_debug_fail_reservations": (None, [ctypes.c_uint]),
    "qses_debug_wait_limit": (ctypes.c_int, [_VP, ctypes.c_longlong, ctypes.POINTER(ctypes.c_int)]),
    "qses_host_timeline": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "qses_debug_slab_plan": (ctypes.c_int, [ctypes.c_uint, _VP, _VP, ctypes.c_uint, ctypes.c_int, ctypes.c_uint,
                                            ctypes.c_uint, ctypes.c_uint, ctypes.c_int, _VP, _VP, ctypes.c_size_t]),
    "qses_graph_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]),
    "qses_field_codes_noalloc": (ctypes.c_int, [_VP, _VP, ctypes.c_uint, ctypes.c_float, _VP, ctypes.c_size_t,
                                                _VP]),
    "qses_grid_info_for": (ctypes.c_int, [_VP, _FP, ctypes.c_uint, ctypes.c_float, ctypes.POINTER(GridInfo)]),
    "qses_debug_codes": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t]),
    "qses_debug_atom_order": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                             ctypes.c_uint]),
    "qses_synth_ball": (ctypes.c_int, [ctypes.c_uint, ctypes.c_uint64, ctypes.c_float, ctypes.c_float, _FP, _FP,
                                       ctypes.POINTER(ctypes.c_ubyte)]),
    "qses_synth_shell": (ctypes.c_int, [ctypes.c_uint, ctypes.c_uint64, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float, _FP, _FP, ctypes.POINTER(ctypes.c_ubyte)]),
    "qses_synth_jitter": (ctypes.c_int, [_FP, ctypes.c_uint, ctypes.c_float, ctypes.c_uint64, _FP]),
    "qses_read_pdb": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_FP), ctypes.POINTER(_FP),
                                     ctypes.POINTER(ctypes.c_uint)]),
    "qses_free": (None, [_VP]),
    "qses_write_obj": (ctypes.c_int, [ctypes.c_char_p, _VP, ctypes.c_uint, _VP, ctypes.c_uint, ctypes.c_int]),
    "qses_format_fixed3": (ctypes.c_int, [ctypes.c_float, ctypes.c_char_p, ctypes.c_int]),
    "NTriangles": None,
    "NVertices": None,
    "globalTriangles": None,
    "globalVertices": None,
    "globalIdAtomPerVert": None,
}

_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libquickses_gb300.so is not built; run `python -c \"import __graft_entry__ as g; "
                              "g.build()\"` (or python quickses_gb300/_build.py)")
        L = ctypes.CDLL(LIB_PATH)
        for name, sig in SIGNATURES.items():
            if sig is None:
                continue
            fn = getattr(L, name)
            fn.restype, fn.argtypes = sig
        _lib = L
    return _lib


def status_string(code):
    return lib().qses_status_string(code).decode()

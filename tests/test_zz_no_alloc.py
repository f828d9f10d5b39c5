"""The allocation-free field entry point (qses_field_codes_noalloc) against the regular
one.  It is for callers that may not allocate device memory while they run; its output
must be the same voxel codes qses_compute produces (bit for bit, like every field test),
call after call, although every call reuses the same in-library working array.

Kept in its own file, collected last, so a failure here cannot hide other results."""
import ctypes

import numpy as np
import pytest

import quickses_gb300 as q
from quickses_gb300 import _lib as L

pytestmark = pytest.mark.gpu

MAX_ATOMS, MAX_G, MAX_GNB = 4096, 128, 40  # the limits the entry point documents


def _call(xyz, rad, voxel, out_bytes=None, stream=None):
    """One call through the C-ABI; returns (status, codes or None).  The output buffer is
    pre-filled with a byte no voxel code takes, so untouched voxels show."""
    import torch
    d_xyz = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).cuda()
    d_rad = torch.from_numpy(np.ascontiguousarray(rad, np.float32)).cuda()
    G = None
    if out_bytes is None:
        G = q.grid_info(xyz, rad, voxel).G
        out_bytes = G * G * G
    d_out = torch.full((max(out_bytes, 1),), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
    rc = L.lib().qses_field_codes_noalloc(ctypes.c_void_p(d_xyz.data_ptr()), ctypes.c_void_p(d_rad.data_ptr()),
                                          len(rad), ctypes.c_float(voxel), ctypes.c_void_p(d_out.data_ptr()),
                                          out_bytes, handle)
    torch.cuda.synchronize()
    if rc != L.QSES_OK or G is None:
        return rc, None
    return rc, d_out.cpu().numpy().reshape(G, G, G)


def _regular_codes(xyz, rad, voxel):
    with q.Context(0) as c:
        c.compute(xyz, rad, voxel=voxel, smooth=0)
        return c.debug_codes(q.grid_info(xyz, rad, voxel).G)


def _check(xyz, rad, voxel, stream=None):
    rc, got = _call(xyz, rad, voxel, stream=stream)
    assert rc == L.QSES_OK, L.status_string(rc)
    want = _regular_codes(xyz, rad, voxel)
    assert got.shape == want.shape
    assert np.array_equal(got, want)


def test_noalloc_matches_regular_entry_point_twice():
    pytest.importorskip("torch")
    mols = [(q.molecules.ball(600, 51), 0.5), (q.molecules.ball(250, 52), 0.4)]
    for (xyz, rad, _), voxel in mols:  # two calls in a row, different sizes
        _check(xyz, rad, voxel)


def test_noalloc_at_the_size_limits():
    """Grids of exactly 128 voxels and 40 neighbour cells per axis (both limits in one
    sparse 4 000-atom molecule), then a 3 000-atom molecule at G = 128 with few cells."""
    pytest.importorskip("torch")
    xyz, rad, _ = q.molecules.ball(4000, 62, density=0.0045)
    g = q.grid_info(xyz, rad, 1.0)
    assert (g.G, g.gnb) == (MAX_G, MAX_GNB)
    _check(xyz, rad, 1.0)
    xyz, rad, _ = q.molecules.ball(3000, 61)
    assert q.grid_info(xyz, rad, 0.45).G == MAX_G
    _check(xyz, rad, 0.45)


def test_noalloc_smaller_after_larger_same_grid():
    """The same grid size twice in a row, first from 3 000 atoms, then from 1 500: nothing
    the first call left in the shared array (atoms, cell ranges, masks) may show through."""
    pytest.importorskip("torch")
    a_xyz, a_rad, _ = q.molecules.ball(3000, 61)
    b_xyz, b_rad, _ = q.molecules.ball(1500, 63)
    ga, gb = q.grid_info(a_xyz, a_rad, 0.45), q.grid_info(b_xyz, b_rad, 0.37)
    assert ga.G == gb.G == MAX_G and gb.gnb < ga.gnb
    _check(a_xyz, a_rad, 0.45)
    _check(b_xyz, b_rad, 0.37)
    _check(b_xyz, b_rad, 0.37)


def test_noalloc_on_a_caller_stream():
    """On a stream of the caller's with work of its own queued before the call."""
    pytest.importorskip("torch")
    import torch
    s = torch.cuda.Stream()
    busy = torch.zeros(1 << 24, device="cuda")
    with torch.cuda.stream(s):
        for _ in range(8):
            busy.add_(1.0)  # keeps the stream busy when the call is enqueued
    xyz, rad, _ = q.molecules.ball(900, 64)
    _check(xyz, rad, 0.45, stream=s)
    _check(xyz, rad, 0.45, stream=s)


def test_noalloc_rejects_oversize_inputs():
    """Each limit one step over: more atoms, a grid of 129 voxels, 41 neighbour cells, an
    output buffer one byte short.  Each call is refused, and the next valid call works."""
    pytest.importorskip("torch")
    xyz, rad, _ = q.molecules.ball(MAX_ATOMS + 1, 53)
    assert _call(xyz, rad, 0.5, out_bytes=16)[0] == L.QSES_ERR_UNSUPPORTED
    xyz, rad, _ = q.molecules.ball(3000, 61)
    assert q.grid_info(xyz, rad, 0.447).G == MAX_G + 1
    assert _call(xyz, rad, 0.447, out_bytes=129 ** 3)[0] == L.QSES_ERR_UNSUPPORTED
    sx, sr, _ = q.molecules.ball(4000, 62, density=0.0043)
    g = q.grid_info(sx, sr, 1.02)
    assert g.gnb == MAX_GNB + 1 and g.G <= MAX_G
    assert _call(sx, sr, 1.02, out_bytes=g.G ** 3)[0] == L.QSES_ERR_UNSUPPORTED
    assert _call(xyz, rad, 0.45, out_bytes=MAX_G ** 3 - 1)[0] == L.QSES_ERR_INVALID_ARG
    _check(xyz, rad, 0.45)

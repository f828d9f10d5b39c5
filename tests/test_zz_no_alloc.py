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


def _noalloc_codes(xyz, rad, voxel):
    import torch
    gi = q.grid_info(xyz, rad, voxel)
    G = gi.G
    d_xyz = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).cuda()
    d_rad = torch.from_numpy(np.ascontiguousarray(rad, np.float32)).cuda()
    d_out = torch.full((G * G * G,), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc = L.lib().qses_field_codes_noalloc(ctypes.c_void_p(d_xyz.data_ptr()), ctypes.c_void_p(d_rad.data_ptr()),
                                          len(rad), ctypes.c_float(voxel), ctypes.c_void_p(d_out.data_ptr()),
                                          d_out.numel(), None)
    assert rc == L.QSES_OK, L.status_string(rc)
    torch.cuda.synchronize()
    return d_out.cpu().numpy().reshape(G, G, G)


def _regular_codes(xyz, rad, voxel):
    with q.Context(0) as c:
        c.compute(xyz, rad, voxel=voxel, smooth=0)
        return c.debug_codes(q.grid_info(xyz, rad, voxel).G)


def test_noalloc_matches_regular_entry_point_twice():
    pytest.importorskip("torch")
    mols = [(q.molecules.ball(600, 51), 0.5), (q.molecules.ball(250, 52), 0.4)]
    for (xyz, rad, _), voxel in mols:  # two calls in a row, different sizes
        got = _noalloc_codes(xyz, rad, voxel)
        want = _regular_codes(xyz, rad, voxel)
        assert got.shape == want.shape
        assert np.array_equal(got, want)


def test_noalloc_rejects_oversize_inputs():
    pytest.importorskip("torch")
    import torch
    xyz, rad, _ = q.molecules.ball(5000, 53)  # more atoms than the working array holds
    d_xyz = torch.from_numpy(xyz).cuda()
    d_rad = torch.from_numpy(rad).cuda()
    d_out = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc = L.lib().qses_field_codes_noalloc(ctypes.c_void_p(d_xyz.data_ptr()), ctypes.c_void_p(d_rad.data_ptr()),
                                          len(rad), ctypes.c_float(0.5), ctypes.c_void_p(d_out.data_ptr()),
                                          d_out.numel(), None)
    assert rc == L.QSES_ERR_UNSUPPORTED

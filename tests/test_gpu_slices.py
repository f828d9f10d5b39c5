"""The reference's slicing mode (QSES_FLAG_REFERENCE_SLICES, CudaSurf.cu:629-754): the GPU
path against the oracle's restatement of it (oracle.compute_ses_slices), bit for bit -
per-slice counts, vertices, triangles, closest atoms - and its boundaries."""
import numpy as np
import pytest

import quickses_gb300 as q
from quickses_gb300 import _lib as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# atoms, seed, voxel, slice, passes, keep degenerate triangles
CASES = [
    (300, 101, 0.5, 16, 1, False),
    (300, 101, 0.5, 40, 0, True),
    (200, 102, 0.4, 20, 2, False),
    (150, 103, 0.3, 24, 1, False),
    (120, 104, 0.2, 30, 1, True),
    (150, 105, 0.75, 16, 1, False),  # R = 2: only slices starting at 0 emit cells
    (500, 107, 0.5, 7, 1, False),    # slices smaller than the refine halo
    (400, 106, 0.5, 1000, 1, False),  # one slice covering the grid
]


def _check(ctx, xyz, rad, dx, sl, passes, keep):
    m = ctx.compute(xyz, rad, voxel=dx, smooth=passes, keep_degenerate=keep, slice=sl, reference_slices=True)
    ref = O.compute_ses_slices(xyz, rad, dx, sl, smooth=passes)
    counts = ctx.slice_counts()
    toff = ref.slice_t if keep else ref.slice_tk
    assert [c[0] for c in counts] == np.diff(ref.slice_v).tolist()
    assert [c[1] for c in counts] == np.diff(toff).tolist()
    assert np.array_equal(m.vertices, ref.vertices.astype(np.float32))
    assert np.array_equal(m.triangles, ref.triangles if keep else ref.triangles_kept)
    # closest atoms by input index: the cell-sorted order follows the reference's fast-math
    # cell keys, which the IEEE oracle does not reproduce for atoms on a cell boundary
    assert np.array_equal(m.atom_input, ref.atom_input)
    return m, counts


@pytest.mark.parametrize("n,seed,dx,sl,passes,keep", CASES)
def test_slices_match_oracle(ctx, n, seed, dx, sl, passes, keep):
    xyz, rad, _ = q.molecules.ball(n, seed)
    _, counts = _check(ctx, xyz, rad, dx, sl, passes, keep)
    G = q.grid_info(xyz, rad, dx).G
    if sl < G:
        assert len(counts) > 1


def test_one_slice_is_the_grid_without_its_last_triangle(ctx):
    """With one slice covering the grid the reference's output is the single-slice mesh
    whose last triangle was never written."""
    xyz, rad, _ = q.molecules.ball(400, 106)
    whole = ctx.compute(xyz, rad, voxel=0.5, smooth=0, keep_degenerate=True)
    sl = ctx.compute(xyz, rad, voxel=0.5, smooth=0, keep_degenerate=True, slice=10 ** 6, reference_slices=True)
    used = np.zeros(len(whole.vertices), bool)
    used[whole.triangles[:-1].ravel()] = True
    ids = np.cumsum(used) - 1
    assert np.array_equal(sl.vertices, whole.vertices[used])
    assert np.array_equal(sl.triangles, ids[whole.triangles[:-1]])
    assert np.array_equal(sl.atom_input, whole.atom_input[used])


def test_slices_at_scale_match_oracle(ctx):
    """20 000 atoms at 0.2 A with the reference's 300-voxel slices: a 502^3 grid in eight
    slices, two seam layers each way, windows clamped at every box face."""
    xyz, rad, _ = q.molecules.ball(20000, 1)
    _, counts = _check(ctx, xyz, rad, 0.2, 300, 1, False)
    assert len(counts) == 8


def test_slices_are_refused_where_they_do_not_apply(ctx):
    xyz, rad, _ = q.molecules.ball(200, 108)
    with pytest.raises(q.QSESError) as e:
        ctx.compute(xyz, rad, voxel=0.5, slice=0, reference_slices=True)
    assert e.value.code == L.QSES_ERR_INVALID_ARG
    out = ctx.compute_batch([dict(xyz=xyz, radii=rad, voxel=0.5, smooth=1, flags=L.QSES_FLAG_REFERENCE_SLICES),
                             dict(xyz=xyz, radii=rad, voxel=0.5, smooth=1)])
    assert isinstance(out[0], q.QSESError) and out[0].code == L.QSES_ERR_UNSUPPORTED
    assert not isinstance(out[1], q.QSESError)
    # the next plain call reports no slices
    ctx.compute(xyz, rad, voxel=0.5)
    assert ctx.slice_counts() == []


def test_grid_too_large_for_one_pass_gets_the_reference_slicing(ctx):
    """Two clusters 2 100 A apart: a 4 300-voxel grid, beyond one pass.  The reference slices
    every grid, so the call returns its sliced output (300-voxel slices), the same as asking
    for that mode, with a surface around each cluster."""
    a_xyz, a_rad, _ = q.molecules.ball(200, 109)
    xyz = np.concatenate([a_xyz, a_xyz + np.float32([2100.0, 0.0, 0.0])])
    rad = np.concatenate([a_rad, a_rad])
    with pytest.raises(q.QSESError):
        q.grid_info(xyz, rad, 0.5)  # no single-pass grid
    m = ctx.compute(xyz, rad, voxel=0.5, smooth=1)
    counts = ctx.slice_counts()
    assert len(counts) >= 2 and sum(c[0] for c in counts) == len(m.vertices)
    s = ctx.compute(xyz, rad, voxel=0.5, smooth=1, slice=300, reference_slices=True)
    assert np.array_equal(m.vertices, s.vertices) and np.array_equal(m.triangles, s.triangles)
    near_a = m.vertices[:, 0] < 1000.0
    assert near_a.any() and (~near_a).any()
    # each cluster's surface: the far one is the near one moved by 2100 A, up to the slice
    # seams that cut them differently
    assert abs(int(near_a.sum()) - int((~near_a).sum())) < 0.2 * len(m.vertices)

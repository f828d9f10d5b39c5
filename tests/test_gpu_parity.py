"""GPU path vs the CPU oracle on seeded small molecules, through the C-ABI.

Bar: bit-exact against the oracle's FP32 mode (same arithmetic order) for voxel codes,
atom order, welded vertices, triangles and atom ids; against the FP64 oracle the mesh is
within a symmetric Hausdorff distance of 0.05 voxel.
"""
import numpy as np
import pytest

import quickses_gb300 as q
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HAUSDORFF_TOL = 0.05  # in voxels

CASES = [
    ("ball", 2, 3, 0.5), ("ball", 30, 1, 0.5), ("ball", 200, 2, 0.5), ("ball", 1000, 1, 0.5),
    ("ball", 300, 4, 0.4), ("ball", 300, 5, 0.3), ("ball", 250, 6, 0.2), ("shell", 400, 9, 0.5),
]


def _atoms(kind, n, seed):
    if kind == "ball":
        xyz, rad, _ = q.molecules.ball(n, seed)
    else:
        xyz, rad, _ = q.molecules.shell(n, seed, r_in=12.0, thickness=4.0)
    return xyz, rad


def _compare_exact(m, ref, keep_degenerate=False, order=None):
    """Bit-exact mesh comparison.  Closest atoms are compared by input index: the sorted
    order behind atom_sorted follows the reference's fast-math cell keys (k_hash.cu),
    which the IEEE oracle cannot reproduce at cell boundaries; `order` (the GPU's
    sorted-to-input map) checks that atom_sorted is the same atom."""
    assert m.vertices.shape == ref.vertices.shape
    assert np.array_equal(m.vertices, ref.vertices.astype(np.float32))
    tri_ref = ref.triangles if keep_degenerate else ref.triangles_kept
    assert np.array_equal(m.triangles, tri_ref)
    assert np.array_equal(m.atom_input, ref.atom_input)
    if order is not None:
        assert np.array_equal(order[m.atom_sorted], m.atom_input)


def _ambiguous_cells(xyz, g, ulps=4):
    """Atoms whose cell coordinate (p - o) / cell lies within a few ulp of an integer in
    some axis: there the reference's approximate division may truncate either way."""
    o = np.array([g.ox, g.oy, g.oz], np.float32)
    q = (xyz.astype(np.float32) - o) / np.float32(g.cell)
    near = np.abs(q - np.round(q)) <= ulps * np.spacing(np.abs(q).astype(np.float32))
    return near.any(axis=1)


@pytest.mark.parametrize("kind,n,seed,dx", CASES)
def test_field_codes_exact(ctx, kind, n, seed, dx):
    xyz, rad = _atoms(kind, n, seed)
    ctx.compute(xyz, rad, voxel=dx, smooth=0)
    g, _ = O.grid(xyz, rad, dx)
    codes = ctx.debug_codes(g.G)
    ref = O.field_codes(xyz, rad, g, fp64=False)
    mism = np.argwhere(codes != ref)
    assert len(mism) == 0, "first mismatches %s gpu=%s oracle=%s" % (
        mism[:5].tolist(), codes[tuple(mism[:5].T)].tolist(), ref[tuple(mism[:5].T)].tolist())


@pytest.mark.parametrize("shape", [0, 1, 2, 3])
@pytest.mark.parametrize("kind,n,seed,dx", CASES[1:])
def test_field_codes_every_tile_shape(ctx, kind, n, seed, dx, shape):
    """Every refine tile shape (8 x 8, 16 x 8, 16 x 16, 32 x 16 z-rows per CTA) gives the
    oracle's codes."""
    xyz, rad = _atoms(kind, n, seed)
    ctx.set_field_shape(shape)
    try:
        ctx.compute(xyz, rad, voxel=dx, smooth=0)
    finally:
        ctx.set_field_shape(-1)
    g, _ = O.grid(xyz, rad, dx)
    assert np.array_equal(ctx.debug_codes(g.G), O.field_codes(xyz, rad, g, fp64=False))


@pytest.mark.parametrize("kind,n,seed,dx", CASES)
def test_atom_order_exact(ctx, kind, n, seed, dx):
    """Cell keys equal the oracle's except at exact cell boundaries (where the reference's
    approximate division may pick the lower cell), and the order is the stable sort."""
    xyz, rad = _atoms(kind, n, seed)
    ctx.compute(xyz, rad, voxel=dx, smooth=0)
    order, keys = ctx.debug_atom_order(n)
    g, _ = O.grid(xyz, rad, dx)
    _, ref_hash = O.sort_atoms(xyz, g)
    gkey = np.zeros(n, np.int64)
    gkey[order] = keys
    amb = _ambiguous_cells(xyz, g)
    assert np.array_equal(gkey[~amb], ref_hash[~amb])
    assert (np.abs(gkey[amb] - ref_hash[amb]) <= g.gnb * g.gnb + g.gnb + 1).all()
    assert np.array_equal(order, np.argsort(gkey, kind="stable"))


@pytest.mark.parametrize("smooth", [0, 1, 3])
@pytest.mark.parametrize("kind,n,seed,dx", CASES)
def test_mesh_exact_fp32(ctx, kind, n, seed, dx, smooth):
    xyz, rad = _atoms(kind, n, seed)
    m = ctx.compute(xyz, rad, voxel=dx, smooth=smooth)
    order, _ = ctx.debug_atom_order(n)
    ref = O.compute_ses(xyz, rad, dx, smooth=smooth, fp64=False)
    _compare_exact(m, ref, order=order)


def test_keep_degenerate_exact(ctx):
    xyz, rad = _atoms("ball", 250, 6)
    m = ctx.compute(xyz, rad, voxel=0.2, smooth=1, keep_degenerate=True)
    ref = O.compute_ses(xyz, rad, 0.2, smooth=1, fp64=False)
    _compare_exact(m, ref, keep_degenerate=True)


@pytest.mark.parametrize("kind,n,seed,dx", CASES[1:])
def test_mesh_vs_fp64_hausdorff(ctx, kind, n, seed, dx):
    xyz, rad = _atoms(kind, n, seed)
    m = ctx.compute(xyz, rad, voxel=dx, smooth=1)
    ref = O.compute_ses(xyz, rad, dx, smooth=1, fp64=True)
    h, _, _ = O.hausdorff(m.vertices.astype(np.float64), m.triangles, ref.vertices, ref.triangles_kept)
    assert h <= HAUSDORFF_TOL * dx, "Hausdorff %.4g A > %.4g A" % (h, HAUSDORFF_TOL * dx)
    assert abs(len(m.vertices) - len(ref.vertices)) <= max(2, 0.01 * len(ref.vertices))


def test_empty_inputs(ctx):
    for n in (0, 1):
        xyz = np.zeros((n, 3), np.float32)
        rad = np.full(n, 1.7, np.float32)
        m = ctx.compute(xyz, rad, voxel=0.5)
        assert len(m.vertices) == 0 and len(m.triangles) == 0


def test_coincident_atoms(ctx):
    xyz = np.zeros((6, 3), np.float32)
    rad = np.array([1.7, 1.55, 1.52, 1.8, 1.7, 1.7], np.float32)
    m = ctx.compute(xyz, rad, voxel=0.5, smooth=1)
    ref = O.compute_ses(xyz, rad, 0.5, smooth=1, fp64=False)
    _compare_exact(m, ref)
    assert len(m.triangles) > 0


def test_reference_api_semantics():
    xyz, rad = _atoms("ball", 200, 2)
    api = q.ReferenceAPI()
    nv, nidx = api.computeSES(0.5, xyz, rad, smooth=1)
    ref = O.compute_ses(xyz, rad, 0.5, smooth=1, fp64=False)
    assert nv == len(ref.vertices) and nidx == 3 * len(ref.triangles_kept)  # NTri counts indices
    assert api.exported_counts() == (nv, nidx)
    v = api.getVertices(nv)
    assert np.array_equal(v, ref.vertices.astype(np.float32))
    t = api.getTriangles(nidx).reshape(-1, 3)
    assert np.array_equal(t, ref.triangles_kept)
    tw = api.getTriangles(nidx, invert=True).reshape(-1, 3)  # swaps the first two, in place
    assert np.array_equal(tw[:, [1, 0, 2]], ref.triangles_kept)
    tb = api.getTriangles(nidx, invert=True).reshape(-1, 3)
    assert np.array_equal(tb, ref.triangles_kept)
    with q.Context(0) as c:  # the same molecule through a context, for its sorted order
        c.compute(xyz, rad, voxel=0.5, smooth=1)
        order, _ = c.debug_atom_order(len(rad))
    assert np.array_equal(order[api.getAtomIdPerVert(nv)], ref.atom_input)
    api.freeMesh()
    assert api.exported_counts() == (0, 0)


def test_reference_api_with_reference_slices(monkeypatch):
    """API_computeSES with QSES_REFERENCE_SLICES set: the reference's sliced output, its
    concatenation and degenerate filter (CudaSurf.cu:796-836)."""
    xyz, rad = _atoms("ball", 250, 3)
    monkeypatch.setenv("QSES_REFERENCE_SLICES", "18")
    api = q.ReferenceAPI()
    nv, nidx = api.computeSES(0.5, xyz, rad, smooth=1)
    ref = O.compute_ses_slices(xyz, rad, 0.5, 18, smooth=1)
    assert len(ref.slice_v) > 2
    assert nv == len(ref.vertices) and nidx == 3 * len(ref.triangles_kept)
    assert np.array_equal(api.getVertices(nv), ref.vertices.astype(np.float32))
    assert np.array_equal(api.getTriangles(nidx).reshape(-1, 3), ref.triangles_kept)
    api.freeMesh()
    monkeypatch.delenv("QSES_REFERENCE_SLICES")
    nv, nidx = api.computeSES(0.5, xyz, rad, smooth=1)
    assert nv == len(O.compute_ses(xyz, rad, 0.5, smooth=1).vertices)
    api.freeMesh()


@pytest.mark.parametrize("n,dx,passes", [(20000, 0.2, 1), (5000, 0.4, 2)])
def test_mesh_vs_fp64_at_scale(ctx, n, dx, passes):
    """The FP32 GPU mesh against the FP64 oracle on large molecules (20 000 atoms at 0.2 A:
    1.7 M vertices; 5 000 atoms at 0.4 A with two passes).  At this size a few voxels sit on
    an FP32 rounding tie of the SAS test (|p - a|^2 against (r + probe)^2; 16 of 126 M voxels
    on the 20 000-atom ball), where FP32 and FP64 classify them differently, as the
    reference's FP32 kernel does.  Each such flip moves the surface near that voxel only:
    symmetric Hausdorff within half a voxel, and under 1e-4 of the vertices farther than
    0.05 voxel from the FP64 surface (measured: 0.25 voxel and 34 of 1 668 491)."""
    xyz, rad, _ = q.molecules.ball(n, 1)
    m = ctx.compute(xyz, rad, voxel=dx, smooth=passes)
    ref = O.compute_ses(xyz, rad, dx, smooth=passes, fp64=True)
    v = m.vertices.astype(np.float64)
    h, _, _ = O.hausdorff(v, m.triangles, ref.vertices, ref.triangles_kept)
    assert h <= 0.5 * dx, "Hausdorff %.4g A > %.4g A" % (h, 0.5 * dx)
    used = np.zeros(len(v), bool)
    used[m.triangles.ravel()] = True
    d = O.point_surface(v[used], ref.vertices, ref.triangles_kept)
    far = int((d > HAUSDORFF_TOL * dx).sum())
    assert far <= 1e-4 * len(d), "%d of %d vertices farther than %.3g A" % (far, len(d), HAUSDORFF_TOL * dx)
    assert abs(len(m.vertices) - len(ref.vertices)) <= max(2, 0.01 * len(ref.vertices))

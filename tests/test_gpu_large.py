"""Full-size checks on the 50 000-atom / 0.2 A workload (grid 664^3, ~3.5 M vertices) and
the 1 000 000-atom shell at 0.5 A (grid 1738^3).

The oracle cannot afford the whole field at this size, so the checks are split:
* field: oracle codes on x-slabs (with their refine halo) == GPU codes there
* mesh:  the oracle's marching cubes + weld + closest atom fed the GPU's field == GPU mesh
* smoothing: the oracle's Gauss-Seidel pass on the GPU's unsmoothed mesh == GPU pass
  (this exercises the slab-partitioned kernel with ~150 slabs)
* size-independent properties: lexicographic vertex order, index ranges, no unused vertex
"""
import numpy as np
import pytest

import quickses_gb300 as q
from oracle import oracle as O

pytestmark = pytest.mark.gpu

WL = q.molecules.WORKLOADS["ball50k"]


@pytest.fixture(scope="module")
def big():
    xyz, rad, _ = WL.atoms()
    g, _ = O.grid(xyz, rad, WL.voxel)
    with q.Context(0) as c:
        m0 = c.compute(xyz, rad, voxel=WL.voxel, smooth=0, keep_degenerate=True)
        codes = c.debug_codes(g.G)
        m1 = c.compute(xyz, rad, voxel=WL.voxel, smooth=1, keep_degenerate=True)
        m1k = c.compute(xyz, rad, voxel=WL.voxel, smooth=1, keep_degenerate=False)
    return xyz, rad, g, m0, codes, m1, m1k


@pytest.mark.parametrize("shape", [1, 2, 3])
def test_field_tile_shapes_match(big, shape):
    """The 16 x 8, 16 x 16 and 32 x 16 refine tiles give the same 664^3 codes as the 8 x 8 one."""
    xyz, rad, g, _, codes, _, _ = big
    with q.Context(0) as c:
        c.set_field_shape(shape)
        c.compute(xyz, rad, voxel=WL.voxel, smooth=0)
        assert np.array_equal(c.debug_codes(g.G), codes)


@pytest.mark.parametrize("x0", [0, 200, 330, 640])
def test_field_slab_exact(big, x0):
    xyz, rad, g, _, codes, _, _ = big
    x1 = min(x0 + 4, g.G)
    ref = O.field_codes(xyz, rad, g, fp64=False, x0=x0, x1=x1)
    assert np.array_equal(codes[x0:x1], ref)


def test_mesh_from_gpu_field_exact(big):
    xyz, rad, g, m0, codes, _, _ = big
    ref = O.mesh_from_codes(codes, g, xyz, fp64=False, smooth=0)
    assert np.array_equal(m0.vertices, ref.vertices.astype(np.float32))
    assert np.array_equal(m0.triangles, ref.triangles)
    assert np.array_equal(m0.atom_input, ref.atom_input)


def test_smoothing_at_scale_exact(big):
    _, _, _, m0, _, m1, _ = big
    ref = O.smooth_f32(m0.vertices, m0.triangles, 1)
    assert np.array_equal(m1.vertices, ref)
    assert np.array_equal(m1.triangles, m0.triangles)


@pytest.mark.parametrize("threads,target,flags,wave", [(1024, 16384, 0, 0), (1024, 4096, 3, 0), (512, 25000, 2, 0),
                                                       (1024, 16384, 4, 0), (1024, 16384, 6, 0),
                                                       (1024, 16384, 0, 1000000), (512, 8192, 2, 600000),
                                                       (1024, 8192, 10, 0), (512, 4096, 8, 0), (1024, 8192, 11, 600000),
                                                       (1024, 25000, 18, 0), (1024, 8192, 26, 0), (1024, 16384, 34, 0),
                                                       (512, 8192, 42, 600000), (1024, 4096, 17, 1000000)])
def test_smoothing_shapes_at_scale_exact(big, threads, target, flags, wave):
    """~150 slabs, every cache policy, and the mesh split into sequential waves (as meshes
    above 3.8 M vertices are): still the sequential Gauss-Seidel result."""
    xyz, rad, _, m0, _, _, _ = big
    ref = O.smooth_f32(m0.vertices, m0.triangles, 1)
    with q.Context(0) as c:
        c.set_smoothing_shape(threads, target, flags, wave)
        m = c.compute(xyz, rad, voxel=WL.voxel, smooth=1, keep_degenerate=True)
    assert np.array_equal(m.vertices, ref)


def test_mesh_properties(big):
    _, _, g, m0, _, _, m1k = big
    v = m0.vertices.astype(np.float64)
    # welded vertices are in strictly increasing lexicographic (x, y, z) order
    d = np.diff(v, axis=0)
    lex = (d[:, 0] > 0) | ((d[:, 0] == 0) & ((d[:, 1] > 0) | ((d[:, 1] == 0) & (d[:, 2] > 0))))
    assert lex.all()
    t = m0.triangles
    assert t.min() >= 0 and t.max() < len(v)
    assert np.bincount(t.ravel(), minlength=len(v)).min() > 0  # every vertex is used
    tk = m1k.triangles
    assert (tk[:, 0] != tk[:, 1]).all() and (tk[:, 1] != tk[:, 2]).all() and (tk[:, 0] != tk[:, 2]).all()
    assert len(tk) < len(t)  # dx = 0.2 produces degenerate triangles, which the API drops


# ---- the 1 000 000-atom shell at 0.5 A (grid 1738^3, 5.2e9 voxels, no smoothing)

SHELL = q.molecules.WORKLOADS["shell1m"]


@pytest.fixture(scope="module")
def shell():
    xyz, rad, _ = SHELL.atoms()
    g, _ = O.grid(xyz, rad, SHELL.voxel)
    with q.Context(0) as c:
        m = c.compute(xyz, rad, voxel=SHELL.voxel, smooth=0, keep_degenerate=True)
        codes = c.debug_codes(g.G)
    return xyz, rad, g, m, codes


@pytest.mark.parametrize("x0", [0, 431, 869, 1300, 1734])
def test_shell_field_slab_exact(shell, x0):
    xyz, rad, g, _, codes = shell
    x1 = min(x0 + 4, g.G)
    assert np.array_equal(codes[x0:x1], O.field_codes(xyz, rad, g, fp64=False, x0=x0, x1=x1))


def test_shell_mesh_from_gpu_field_exact(shell):
    xyz, _, g, m, codes = shell
    ref = O.mesh_from_codes(codes, g, xyz, fp64=False, smooth=0)
    assert np.array_equal(m.vertices, ref.vertices.astype(np.float32))
    assert np.array_equal(m.triangles, ref.triangles)
    assert np.array_equal(m.atom_input, ref.atom_input)


def test_shell_mesh_properties(shell):
    _, _, g, m, _ = shell
    v = m.vertices.astype(np.float64)
    d = np.diff(v, axis=0)
    lex = (d[:, 0] > 0) | ((d[:, 0] == 0) & ((d[:, 1] > 0) | ((d[:, 1] == 0) & (d[:, 2] > 0))))
    assert lex.all()
    t = m.triangles
    assert t.min() >= 0 and t.max() < len(v)
    assert np.bincount(t.ravel(), minlength=len(v)).min() > 0
    # the shell has an outer and an inner (cavity) surface, both inside the grid
    r = np.linalg.norm(v - v.mean(axis=0), axis=1)
    assert r.min() < 400.0 < 430.0 < r.max()


def test_shell_smoothing_in_waves_exact(shell):
    """Smoothing a mesh far above one slab wave (152 x 25 000 vertices): sequential waves,
    still the sequential Gauss-Seidel result."""
    xyz, rad, g, m, _ = shell
    assert len(m.vertices) > 3 * 152 * 25000
    with q.Context(0) as c:
        m1 = c.compute(xyz, rad, voxel=SHELL.voxel, smooth=1, keep_degenerate=True)
    assert np.array_equal(m1.triangles, m.triangles)
    assert np.array_equal(m1.vertices, O.smooth_f32(m.vertices, m.triangles, 1))

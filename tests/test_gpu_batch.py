"""Batch form vs the single-molecule path, through the C-ABI (qses_compute_batch).

Bar: every molecule of a batch is bit-identical to the same molecule computed alone
(vertices, triangles, both atom-id arrays) - the batch shares launches, not arithmetic -
and, through that, to the oracle the single path is pinned to.
"""
import numpy as np
import pytest

import quickses_gb300 as q
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.vertices.shape == b.vertices.shape
    assert np.array_equal(a.vertices, b.vertices)
    assert np.array_equal(a.triangles, b.triangles)
    assert np.array_equal(a.atom_sorted, b.atom_sorted)
    assert np.array_equal(a.atom_input, b.atom_input)
    assert a.grid_dim == b.grid_dim and a.origin == b.origin


def _req(xyz, rad, voxel=0.5, smooth=1, keep=False):
    return {"xyz": xyz, "radii": rad, "voxel": voxel, "smooth": smooth, "keep_degenerate": keep}


def _single(ctx, r):
    return ctx.compute(r["xyz"], r["radii"], voxel=r["voxel"], smooth=r["smooth"], keep_degenerate=r["keep_degenerate"])


def test_mixed_batch_matches_single(ctx):
    reqs = []
    for n, seed, voxel, smooth, keep in [(2, 3, 0.5, 1, False), (30, 1, 0.5, 1, False), (300, 2, 0.5, 1, False),
                                         (1000, 1, 0.4, 1, False), (250, 6, 0.2, 1, True), (120, 8, 0.3, 2, False),
                                         (800, 4, 0.5, 0, False), (0, 1, 0.5, 1, False), (1, 1, 0.5, 1, False)]:
        xyz, rad, _ = q.molecules.ball(n, seed) if n > 1 else (np.zeros((n, 3), np.float32),
                                                                np.full(n, 1.7, np.float32), None)
        reqs.append(_req(xyz, rad, voxel, smooth, keep))
    xyz, rad, _ = q.molecules.shell(400, 9, r_in=12.0, thickness=4.0)
    reqs.append(_req(xyz, rad, 0.5, 1))
    xyz, rad, _ = q.molecules.ball(200, 5)
    reqs.append(_req(xyz, rad, 0.1, 1))  # refine window above 9 voxels: rejected alone
    out = ctx.compute_batch(reqs)
    assert isinstance(out[-1], q.QSESError) and out[-1].code == 5
    for r, m in zip(reqs[:-1], out[:-1]):
        assert not isinstance(m, Exception), m
        _same(m, _single(ctx, r))
    # and the oracle, for two of them
    for i in (3, 4):
        r = reqs[i]
        ref = O.compute_ses(r["xyz"], r["radii"], r["voxel"], smooth=r["smooth"], fp64=False)
        assert np.array_equal(out[i].vertices, ref.vertices.astype(np.float32))
        assert np.array_equal(out[i].atom_input, ref.atom_input)
        assert np.array_equal(out[i].triangles, ref.triangles if r["keep_degenerate"] else ref.triangles_kept)


def test_trajectory_frames_match_single(ctx):
    base, rad, _ = q.molecules.ball(1500, 21)
    frames = [q.molecules.jitter(base, 0.3, seed=100 + f) for f in range(12)]
    reqs = [_req(x, rad, 0.4, 1) for x in frames]
    out = ctx.compute_batch(reqs)
    for r, m in zip(reqs, out):
        _same(m, _single(ctx, r))


def test_uneven_batch_matches_single(ctx):
    rng = np.random.default_rng(7)
    sizes = np.exp(rng.uniform(np.log(500), np.log(20000), 24)).astype(int)
    reqs = []
    for k, n in enumerate(sizes):
        xyz, rad, _ = q.molecules.ball(int(n), 1000 + k)
        reqs.append(_req(xyz, rad, float(rng.choice([0.3, 0.4, 0.5])), 1))
    out = ctx.compute_batch(reqs)
    for r, m in zip(reqs, out):
        _same(m, _single(ctx, r))


def test_small_waves_match_single(ctx):
    """Sequential smoothing waves that cut through molecules give the same meshes."""
    reqs = [_req(*q.molecules.ball(n, 500 + n)[:2], 0.4, 2) for n in (900, 4000, 12000, 2500)]
    singles = [_single(ctx, r) for r in reqs]
    ctx.set_smoothing_shape(1024, 4096, 0, 50000)
    try:
        out = ctx.compute_batch(reqs)
        one = _single(ctx, reqs[2])
    finally:
        ctx.set_smoothing_shape(0)
    for m, s1 in zip(out, singles):
        _same(m, s1)
    _same(one, singles[2])


def test_multi_wave_smoothing_matches_single(ctx):
    """More vertices than one Gauss-Seidel wave holds (152 slabs x 25 000), so the batch
    is smoothed in several waves."""
    reqs = []
    for k in range(5):
        xyz, rad, _ = q.molecules.ball(20000, 300 + k)
        reqs.append(_req(xyz, rad, 0.2, 1))
    out = ctx.compute_batch(reqs)
    assert sum(len(m.vertices) for m in out) > 152 * 25000
    for r, m in zip(reqs, out):
        _same(m, _single(ctx, r))


@pytest.mark.parametrize("threads,target,flags", [(512, 16384, 0), (1024, 16384, 0), (512, 4096, 1), (1024, 4096, 2),
                                                  (1024, 25000, 3), (512, 8192, 3), (1024, 16384, 4), (512, 4096, 6),
                                                  (1024, 25000, 7), (1024, 8192, 8), (512, 4096, 9),
                                                  (1024, 2048, 11), (512, 256, 10), (1024, 25000, 18), (512, 4096, 16),
                                                  (1024, 8192, 26), (1024, 25000, 34), (512, 2048, 41), (1024, 256, 33),
                                                  (512, 16384, 19)])
def test_every_smoothing_shape_is_exact(ctx, threads, target, flags):
    """The autotuner's candidate launch shapes and cache policies give the same mesh bit
    for bit (single and batch), since the Gauss-Seidel order is fixed by the vertex ids."""
    xyz, rad, _ = q.molecules.ball(3000, 44)
    ref = O.compute_ses(xyz, rad, 0.3, smooth=2, fp64=False)
    ctx.set_smoothing_shape(threads, target, flags)
    try:
        m = ctx.compute(xyz, rad, voxel=0.3, smooth=2)
        assert np.array_equal(m.vertices, ref.vertices.astype(np.float32))
        reqs = [_req(*q.molecules.ball(n, 60 + n)[:2], 0.4, 1) for n in (800, 2500, 6000)]
        out = ctx.compute_batch(reqs)
    finally:
        ctx.set_smoothing_shape(0)
    for r, mb in zip(reqs, out):
        _same(mb, _single(ctx, r))


def test_autotune_keeps_results(ctx):
    xyz, rad, _ = q.molecules.ball(2000, 45)
    before = ctx.compute(xyz, rad, voxel=0.4, smooth=1)
    threads, target, flags, field_shape, ms = ctx.autotune(xyz, rad, voxel=0.4, smooth=1)
    assert threads in (512, 1024) and target >= 256 and 0 <= flags < 64 and (flags & 48) != 48 and field_shape in (0, 1, 2, 3) and ms > 0
    _same(ctx.compute(xyz, rad, voxel=0.4, smooth=1), before)
    reqs = [_req(*q.molecules.ball(n, 70 + n)[:2], 0.4, 1) for n in (700, 3000)]
    singles = [_single(ctx, r) for r in reqs]
    ctx.autotune_batch(reqs)
    for m, s1 in zip(ctx.compute_batch(reqs), singles):
        _same(m, s1)

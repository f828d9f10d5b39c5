"""CUDA-graph replay of the pipeline segments (qses_set_graphs / qses_graph_stats).

Bar: a call whose segments replay a cached graph, or update it in place, or re-instantiate
it, gives exactly the bytes of the same call with every kernel launched directly - for the
single-molecule path and the batch form - and the counters show which of the three ran.
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


@pytest.fixture(scope="module")
def direct():
    c = q.Context(0)
    c.set_graphs(False)
    yield c
    c.close()


def _delta(after, before):
    return {k: after[k] - before[k] for k in after}


def test_replay_update_and_reinstantiate_match_direct(direct):
    xyz, rad, _ = q.molecules.ball(1500, 31)
    with q.Context(0) as g:
        g.set_smoothing_shape(1024, 16384, 2, 0)  # not a tuned shape with a stream attribute
        s0 = g.graph_stats()
        first = g.compute(xyz, rad, voxel=0.4, smooth=1)
        s1 = g.graph_stats()
        assert _delta(s1, s0) == {"captures": 3, "instantiations": 3, "updates": 0, "replays": 0}
        _same(first, direct.compute(xyz, rad, voxel=0.4, smooth=1))

        # the same molecule again: every segment's key repeats, the graphs replay
        again = g.compute(xyz, rad, voxel=0.4, smooth=1)
        s2 = g.graph_stats()
        assert _delta(s2, s1) == {"captures": 0, "instantiations": 0, "updates": 0, "replays": 3}
        _same(again, first)

        # moved atoms (new origin, new counts): captured again into free cache entries
        rng = np.random.default_rng(5)
        moved = (xyz + rng.normal(0, 0.3, xyz.shape)).astype(np.float32)
        m = g.compute(moved, rad, voxel=0.4, smooth=1)
        s3 = g.graph_stats()
        d = _delta(s3, s2)
        assert d["replays"] + d["captures"] == 3 and d["captures"] >= 1
        _same(m, direct.compute(moved, rad, voxel=0.4, smooth=1))

        # two passes instead of one: the finish segment's topology changes
        m2 = g.compute(moved, rad, voxel=0.4, smooth=2)
        s4 = g.graph_stats()
        assert _delta(s4, s3)["instantiations"] >= 1
        _same(m2, direct.compute(moved, rad, voxel=0.4, smooth=2))
        ref = O.compute_ses(moved, rad, 0.4, smooth=2, fp64=False)
        assert np.array_equal(m2.vertices, ref.vertices.astype(np.float32))
        assert np.array_equal(m2.triangles, ref.triangles_kept)


@pytest.mark.parametrize("n,seed,voxel,smooth,keep", [(300, 2, 0.5, 0, False), (800, 3, 0.3, 1, True),
                                                      (2, 4, 0.5, 1, False), (4000, 5, 0.5, 3, False)])
def test_sequence_of_molecules_matches_direct(direct, n, seed, voxel, smooth, keep):
    """One graph context through a sequence of different molecules and flags, each call
    compared with direct launches (a stale parameter in a replayed graph would show here)."""
    with q.Context(0) as g:
        for k in range(3):
            xyz, rad, _ = q.molecules.ball(n, seed + 10 * k)
            for rep in range(2):
                _same(g.compute(xyz, rad, voxel=voxel, smooth=smooth, keep_degenerate=keep),
                      direct.compute(xyz, rad, voxel=voxel, smooth=smooth, keep_degenerate=keep))
        assert g.graph_stats()["replays"] >= 3


def test_cache_full_updates_in_place(direct):
    """More distinct molecules than cache entries: the least recently used graphs are
    updated in place (same topology), and every result still matches direct launches."""
    with q.Context(0) as g:
        g.set_smoothing_shape(512, 4096, 0, 0)
        base, rad, _ = q.molecules.ball(900, 51)
        rng = np.random.default_rng(3)
        for k in range(7):
            xyz = (base + rng.normal(0, 0.25, base.shape)).astype(np.float32)
            _same(g.compute(xyz, rad, voxel=0.5, smooth=1), direct.compute(xyz, rad, voxel=0.5, smooth=1))
        st = g.graph_stats()
        # (entries captured before an arena grew are instantiated afresh, never updated)
        assert st["updates"] >= 3 and st["instantiations"] + st["updates"] == st["captures"]


def test_forced_smoothing_shapes_and_waves(direct):
    xyz, rad, _ = q.molecules.ball(3000, 41)
    want = direct.compute(xyz, rad, voxel=0.3, smooth=1)
    with q.Context(0) as g:
        for threads, target, flags, wave in [(512, 4096, 0, 0), (1024, 16384, 2, 0), (1024, 4096, 4, 0),
                                             (512, 4096, 1, 20000), (512, 4096, 1, 20000)]:
            g.set_smoothing_shape(threads, target, flags, wave)
            _same(g.compute(xyz, rad, voxel=0.3, smooth=1), want)


def test_profiling_launches_directly_and_caller_stream_replays():
    torch = pytest.importorskip("torch")
    xyz, rad, _ = q.molecules.ball(500, 7)
    with q.Context(0) as g:
        g.set_smoothing_shape(512, 4096, 0, 0)
        g.set_profiling(True)
        a = g.compute(xyz, rad, voxel=0.5)
        assert g.graph_stats()["captures"] == 0
        g.set_profiling(False)
        b = g.compute(xyz, rad, voxel=0.5)
        assert g.graph_stats()["captures"] == 3
        _same(a, b)
    st = torch.cuda.Stream()
    with q.Context(0, stream=st.cuda_stream) as g:
        g.set_smoothing_shape(512, 4096, 0, 0)
        c = g.compute(xyz, rad, voxel=0.5)
        assert g.graph_stats()["captures"] == 3
        _same(a, c)
        # work the caller queued on its stream before the call is ordered before the graphs
        d_xyz = torch.from_numpy(xyz).cuda()
        d_rad = torch.from_numpy(rad).cuda()
        with torch.cuda.stream(st):
            buf = torch.zeros_like(d_xyz)
            for _ in range(50):
                buf.add_(d_xyz)  # keeps the stream busy
            buf.copy_(d_xyz)
            dm = g.compute_device(buf.data_ptr(), d_rad.data_ptr(), xyz.shape[0], voxel=0.5, smooth=1)
        st.synchronize()
        assert dm.n_vertices == len(a.vertices) and dm.n_triangles == len(a.triangles)
        v = torch.as_tensor(_DeviceArray(dm.d_vertices, (dm.n_vertices, 3), "<f4"), device="cuda").cpu().numpy()
        t = torch.as_tensor(_DeviceArray(dm.d_triangles, (dm.n_triangles, 3), "<i4"), device="cuda").cpu().numpy()
        assert np.array_equal(v, a.vertices) and np.array_equal(t, a.triangles)


class _DeviceArray:
    """A device pointer seen through __cuda_array_interface__ (read after a synchronize)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": shape, "typestr": typestr,
                                         "strides": None, "version": 2}


def test_batch_graphs_match_direct(direct):
    reqs = []
    for n, seed, voxel, smooth, keep in [(30, 1, 0.5, 1, False), (600, 2, 0.4, 1, False), (1200, 3, 0.3, 1, True),
                                         (900, 4, 0.5, 2, False), (1, 1, 0.5, 1, False)]:
        xyz, rad, _ = q.molecules.ball(n, seed) if n > 1 else (np.zeros((1, 3), np.float32),
                                                                np.full(1, 1.7, np.float32), None)
        reqs.append({"xyz": xyz, "radii": rad, "voxel": voxel, "smooth": smooth, "keep_degenerate": keep})
    want = direct.compute_batch(reqs)
    with q.Context(0) as g:
        g.set_smoothing_shape(1024, 16384, 0, 0)
        for rep in range(4):
            if rep == 2:  # workspaces have their final sizes after two calls
                s0 = g.graph_stats()
            got = g.compute_batch(reqs)
            for a, b in zip(got, want):
                _same(a, b)
        d = _delta(g.graph_stats(), s0)
        # two batches per call (1 and 2 smoothing passes), each with its cached graphs
        assert d["captures"] == 0 and d["replays"] == 12
        # trajectory-like: the same molecules moved
        rng = np.random.default_rng(9)
        moved = [dict(r, xyz=(r["xyz"] + rng.normal(0, 0.2, r["xyz"].shape)).astype(np.float32)) for r in reqs]
        for a, b in zip(g.compute_batch(moved), direct.compute_batch(moved)):
            _same(a, b)

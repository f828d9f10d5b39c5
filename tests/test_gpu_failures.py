"""Failure handling without a GPU fault: an injected allocation failure, a request withdrawn
from the server queue, and a bounded device wait that runs out.  Each is reported as a
status code, and the context (or server) keeps working afterwards - the reference instead
exits the process on any error (CudaSurf.h:54-62)."""
import ctypes

import numpy as np
import pytest

import quickses_gb300 as q
from quickses_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.vertices, b.vertices)
    assert np.array_equal(a.triangles, b.triangles)
    assert np.array_equal(a.atom_sorted, b.atom_sorted)
    assert np.array_equal(a.atom_input, b.atom_input)


@pytest.fixture
def fail_reservations():
    lib = L.lib()
    yield lib.qses_debug_fail_reservations
    lib.qses_debug_fail_reservations(0)


def test_allocation_failure_single(ctx, fail_reservations):
    xyz, rad, _ = q.molecules.ball(700, 81)
    want = ctx.compute(xyz, rad, voxel=0.4)
    with q.Context(0) as c:
        fail_reservations(1)
        with pytest.raises(q.QSESError) as e:
            c.compute(xyz, rad, voxel=0.4)
        assert e.value.code == L.QSES_ERR_OUT_OF_MEMORY
        _same(c.compute(xyz, rad, voxel=0.4), want)  # the same context works afterwards


def test_allocation_failure_batch(ctx, fail_reservations):
    reqs = [{"xyz": x, "radii": r, "voxel": 0.5} for x, r, _ in (q.molecules.ball(n, 90 + n) for n in (200, 900))]
    want = [ctx.compute(r["xyz"], r["radii"], voxel=0.5) for r in reqs]
    with q.Context(0) as c:
        fail_reservations(1)
        out = c.compute_batch(reqs)
        assert all(isinstance(m, q.QSESError) and m.code == L.QSES_ERR_OUT_OF_MEMORY for m in out)
        for m, w in zip(c.compute_batch(reqs), want):
            _same(m, w)


def test_allocation_failure_served(ctx, fail_reservations):
    xyz, rad, _ = q.molecules.ball(600, 83)
    want = ctx.compute(xyz, rad, voxel=0.5)
    with q.Server(lanes=1, memory_budget=4 << 30) as srv:
        fail_reservations(1)
        with pytest.raises(q.QSESError) as e:
            srv.wait(srv.submit(xyz, rad, 0.5))
        assert e.value.code == L.QSES_ERR_OUT_OF_MEMORY
        m, _ = srv.wait(srv.submit(xyz, rad, 0.5))  # the lane keeps serving
        _same(m, want)


def test_cancel_queued_requests(ctx):
    big, brad, _ = q.molecules.ball(60000, 84)  # keeps the single lane busy for a while
    small = [q.molecules.ball(300 + 40 * k, 85 + k)[:2] for k in range(8)]
    with q.Server(lanes=1, memory_budget=8 << 30, max_batch=1) as srv:
        t_big = srv.submit(big, brad, 0.3)
        tickets = [srv.submit(x, r, 0.5) for x, r in small]
        cancelled = [srv.cancel(t) for t in tickets[::2]]
        assert any(cancelled)
        srv.wait(t_big)
        for k, t in enumerate(tickets):
            if k % 2 == 0 and cancelled[k // 2]:
                with pytest.raises(q.QSESError) as e:
                    srv.wait(t)
                assert e.value.code == L.QSES_ERR_CANCELLED
            else:
                m, _ = srv.wait(t)
                _same(m, ctx.compute(*small[k], voxel=0.5))
        with pytest.raises(q.QSESError):
            srv.cancel(tickets[1])  # collected already: unknown ticket


def test_bounded_wait_runs_out(ctx):
    """The smoothing kernel's boundary warp waits for a hand-off that never comes: after its
    cycle budget (~0.1 s) it reports QSES_ERR_TIMEOUT, every CTA returns, and the context
    computes normally afterwards."""
    lib = L.lib()
    with q.Context(0) as c:
        st = ctypes.c_int(0)
        assert lib.qses_debug_wait_limit(c.handle, 200_000_000, ctypes.byref(st)) == 0
        assert st.value == L.QSES_ERR_TIMEOUT
        xyz, rad, _ = q.molecules.ball(500, 86)
        _same(c.compute(xyz, rad, voxel=0.5), ctx.compute(xyz, rad, voxel=0.5))
    assert lib.qses_debug_wait_limit(None, 200_000_000, ctypes.byref(st)) == L.QSES_ERR_INVALID_ARG

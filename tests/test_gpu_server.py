"""Served form (qses_server_*): requests submitted from several threads while others run are
batched as lanes free up, and every result is bit-identical to the same request computed
alone through qses_compute."""
import threading
import time

import numpy as np
import pytest

import quickses_gb300 as q

pytestmark = pytest.mark.gpu


def _requests(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(np.exp(rng.uniform(np.log(50), np.log(6000))))
        xyz, rad, _ = q.molecules.ball(n, 7000 + seed * 1000 + k)
        out.append(dict(xyz=xyz, radii=rad, voxel=float(rng.choice([0.3, 0.4, 0.5])), smooth=int(rng.integers(0, 3)),
                        keep_degenerate=bool(rng.integers(0, 2))))
    return out


def _same(a, b):
    assert np.array_equal(a.vertices, b.vertices)
    assert np.array_equal(a.triangles, b.triangles)
    assert np.array_equal(a.atom_sorted, b.atom_sorted)
    assert np.array_equal(a.atom_input, b.atom_input)


@pytest.mark.parametrize("lanes", [1, 2, 3])
def test_results_same_alone_and_in_the_mix(ctx, lanes):
    reqs = _requests(36, lanes)
    tickets = [None] * len(reqs)
    with q.Server(lanes=lanes, memory_budget=6 << 30, max_batch=8) as srv:
        def submitter(part):
            rng = np.random.default_rng(part)
            for i in range(part, len(reqs), 3):
                r = reqs[i]
                tickets[i] = srv.submit(r["xyz"], r["radii"], r["voxel"], r["smooth"], r["keep_degenerate"])
                time.sleep(float(rng.uniform(0, 0.004)))  # arrivals while earlier batches run
        th = [threading.Thread(target=submitter, args=(p,)) for p in range(3)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["served"] == len(reqs) and st["batches"] >= 2
    assert st["max_batch"] >= 2  # requests that arrived together ran as one batch
    for r, (m, info) in zip(reqs, results):
        assert info["total_s"] >= info["run_s"] >= 0.0
        alone = ctx.compute(r["xyz"], r["radii"], voxel=r["voxel"], smooth=r["smooth"],
                            keep_degenerate=r["keep_degenerate"])
        _same(m, alone)


def test_rejected_at_submit():
    with q.Server(lanes=1) as srv:
        xyz, rad, _ = q.molecules.ball(100, 3)
        with pytest.raises(q.QSESError) as e:
            srv.submit(xyz, rad, voxel=0.1)  # refine window above 9 voxels
        assert e.value.code == 5
        t = srv.submit(xyz, rad, voxel=0.5)
        m, _ = srv.wait(t)
        assert len(m.triangles) > 0
        e1, _ = srv.wait(srv.submit(xyz[:1], rad[:1], voxel=0.5))  # one atom: empty mesh
        assert len(e1.vertices) == 0


def test_waits_while_other_threads_submit(ctx):
    """Two threads wait for the same ticket while the main thread submits hundreds of small
    requests (the server's ticket table grows and rehashes under the waiters).  Exactly one
    waiter gets the mesh, the other is refused with QSES_ERR_INVALID_ARG, and every result
    equals the request computed alone."""
    from quickses_gb300 import _lib as L
    xyz, rad, _ = q.molecules.ball(8000, 4401)
    small = [q.molecules.ball(int(n), 4500 + k)[:2] for k, n in enumerate(np.linspace(3, 40, 24).astype(int))]
    with q.Server(lanes=2, memory_budget=6 << 30, max_batch=4) as srv:
        big = srv.submit(xyz, rad, voxel=0.4, smooth=1)
        got, refused = [], []

        def waiter():
            try:
                got.append(srv.wait(big)[0])
            except q.QSESError as e:
                refused.append(e.code)

        th = [threading.Thread(target=waiter) for _ in range(2)]
        for t in th:
            t.start()
        tickets = []
        for rep in range(12):
            for k, (s_xyz, s_rad) in enumerate(small):
                tickets.append((srv.submit(s_xyz, s_rad, voxel=0.5, smooth=1), k))
        for t in th:
            t.join()
        results = [(srv.wait(t)[0], k) for t, k in tickets]
    assert len(got) == 1 and refused == [L.QSES_ERR_INVALID_ARG]
    _same(got[0], ctx.compute(xyz, rad, voxel=0.4, smooth=1))
    alone = [ctx.compute(a, b, voxel=0.5, smooth=1) for a, b in small]
    for m, k in results:
        _same(m, alone[k])

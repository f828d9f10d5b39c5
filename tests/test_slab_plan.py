"""Slab plan of the Gauss-Seidel pass (CPU, through qses_debug_slab_plan).

The smoothing kernel's persistent CTAs take slabs from a counter in the plan's order and a
slab waits only for lower-id slabs of its own molecule, so every wait ends if (a) the slabs
tile each wave, (b) a slab holds whole molecules unless one molecule is larger than a slab,
and (c) a molecule's slabs are taken in id order.  These tests check those invariants, the
size and capacity bounds, and that one molecule keeps the single-molecule split (at most
pmax slabs of at least `target` vertices, at most 25 000).
"""
import ctypes

import numpy as np
import pytest

from quickses_gb300 import _lib as L

SMAX = 25000


def _plan(nv, mol_off=None, depth=None, threads=1024, target=16384, wave=0, pmax=152, flags=0):
    lib = L.lib()
    launch = (ctypes.c_uint * 6)()
    nm = 1 if mol_off is None else len(mol_off) - 1
    mo = None if mol_off is None else np.ascontiguousarray(mol_off, np.uint32)
    dp = None if depth is None else np.ascontiguousarray(depth, np.int32)
    rc = lib.qses_debug_slab_plan(nv, None if mo is None else mo.ctypes.data, None if dp is None else dp.ctypes.data,
                                  nm, threads, target, flags, wave, pmax, launch, None, 0)
    assert rc == 0, rc
    ctas, smax, qcap, wsize, waves, words = list(launch)
    table = np.zeros(waves * words, np.uint32)
    rc = lib.qses_debug_slab_plan(nv, None if mo is None else mo.ctypes.data, None if dp is None else dp.ctypes.data,
                                  nm, threads, target, flags, wave, pmax, launch, table.ctypes.data, table.size)
    assert rc == 0
    out = []
    for w in range(waves):
        t = table[w * words:(w + 1) * words]
        Q = int(t[0])
        out.append((np.array(t[1:Q + 2], np.int64), np.array(t[qcap + 2:qcap + 2 + Q], np.int64)))
    return dict(ctas=ctas, smax=smax, qcap=qcap, wsize=wsize, waves=waves, target=target, flags=flags), out


def _check(nv, mol_off, info, waves, pmax=152):
    mol_off = np.array([0, nv] if mol_off is None else mol_off, np.int64)
    assert info["ctas"] == min(pmax, info["qcap"]) and info["smax"] <= SMAX
    if info["flags"] & 8:  # slab positions in shared memory: at most 8192 vertices per slab
        assert info["smax"] <= max(256, min(info["target"], 8192))
    if mol_off is not None and len(mol_off) > 2:
        assert info["smax"] <= max(256, min(info["target"], SMAX))
    v0 = 0
    for bnd, order in waves:
        Q = len(order)
        assert 1 <= Q <= info["qcap"]
        # (a) the slabs tile the wave
        assert bnd[0] == v0 and np.all(np.diff(bnd) > 0)
        v1 = bnd[-1]
        assert v1 - v0 <= info["wsize"]
        assert np.all(np.diff(bnd) <= info["smax"])
        # order is a permutation of the slabs
        assert sorted(order.tolist()) == list(range(Q))
        pos = np.empty(Q, np.int64)
        pos[order] = np.arange(Q)
        mol_of = lambda v: int(np.searchsorted(mol_off, v, side="right") - 1)
        for q in range(Q):
            a, b = bnd[q], bnd[q + 1]
            ma, mb = mol_of(a), mol_of(b - 1)
            if ma != mb:
                # (b) several molecules: each whole (clipped to the wave)
                assert max(mol_off[ma], v0) == a and min(mol_off[mb + 1], v1) == b
            elif q > 0 and mol_of(bnd[q - 1]) == ma and mol_of(bnd[q] - 1) == ma and bnd[q - 1] >= max(mol_off[ma], v0):
                # (c) the lower slab of the same molecule is taken earlier
                assert pos[q - 1] < pos[q]
        v0 = v1
    assert v0 == nv


@pytest.mark.parametrize("nv,target", [(1, 4096), (900, 4096), (29938, 4096), (3540690, 4096), (3540690, 25000),
                                       (17_000_000, 16384)])
def test_one_molecule_keeps_the_single_split(nv, target):
    info, waves = _plan(nv, target=target)
    _check(nv, None, info, waves)
    bnd, order = waves[0]
    k = max(-(-nv // SMAX), min(-(-nv // target), 152))
    S = -(-nv // k)
    assert np.array_equal(bnd[:-1], np.arange(0, nv, S)) and np.array_equal(order, np.arange(len(order)))


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("target", [256, 4096, 25000])
def test_batches(seed, target):
    rng = np.random.default_rng(seed)
    nm = int(rng.integers(1, 300))
    sizes = np.exp(rng.uniform(np.log(1), np.log(2_000_000), nm)).astype(np.int64)
    sizes[rng.random(nm) < 0.05] = 0  # molecules without vertices
    mol_off = np.concatenate([[0], np.cumsum(sizes)])
    nv = int(mol_off[-1])
    if nv == 0:
        return
    depth = rng.integers(20, 700, nm)
    for wave in (0, int(rng.integers(max(1000, nv // 16), max(1001, nv)))):
        info, waves = _plan(nv, mol_off, depth, target=target, wave=wave)
        _check(nv, mol_off, info, waves)


def test_order_follows_expected_start():
    # a deep molecule's later slabs come after a shallow molecule's whole range
    mol_off = [0, 100_000, 100_500, 101_000]
    info, waves = _plan(101_000, mol_off, [600, 50, 40], target=25000)
    bnd, order = waves[0]
    first = [int(bnd[q]) for q in order[:2]]
    assert first[0] == 0  # the deepest molecule starts first
    assert int(bnd[order[-1]]) == 75_000  # its last quarter is taken last


def test_invalid():
    lib = L.lib()
    launch = (ctypes.c_uint * 6)()
    assert lib.qses_debug_slab_plan(0, None, None, 1, 1024, 4096, 0, 0, 152, launch, None, 0) != 0
    assert lib.qses_debug_slab_plan(10, None, None, 1, 1024, 4096, 0, 0, 0, launch, None, 0) != 0


@pytest.mark.parametrize("nv,target", [(1, 4096), (29938, 4096), (3540690, 8192), (3540690, 20000),
                                       (17_000_000, 4096)])
def test_shared_memory_positions_split(nv, target):
    # one molecule, slab positions in shared memory: slabs of at most min(target, 8192),
    # as many as needed (more than the resident CTAs), taken in id order
    info, waves = _plan(nv, target=target, flags=8)
    _check(nv, None, info, waves)
    bnd, order = waves[0]
    S = -(-nv // -(-nv // min(target, 8192)))
    assert np.array_equal(bnd[:-1], np.arange(0, nv, S)) and np.array_equal(order, np.arange(len(order)))
    assert info["smax"] <= 8192


@pytest.mark.parametrize("seed", range(4))
def test_batches_shared_memory_positions(seed):
    rng = np.random.default_rng(100 + seed)
    nm = int(rng.integers(2, 200))
    sizes = np.exp(rng.uniform(np.log(1), np.log(1_000_000), nm)).astype(np.int64)
    mol_off = np.concatenate([[0], np.cumsum(sizes)])
    nv = int(mol_off[-1])
    info, waves = _plan(nv, mol_off, rng.integers(20, 700, nm), target=25000, flags=11)
    _check(nv, mol_off, info, waves)


def test_smoothing_flag_validation():
    # lane-group bits 4 (two vertices per worker warp) and 5 (four) are exclusive; bits above
    # 5 do not exist.  Invalid shapes are refused before any state changes.
    lib = L.lib()
    for flags in (48, 50, 64, 1 << 20):
        assert lib.qses_set_default_smoothing_shape(1, 1024, 4096, flags) == L.QSES_ERR_INVALID_ARG
    assert lib.qses_set_default_smoothing_shape(1, 1024, 4096, 4) == L.QSES_ERR_INVALID_ARG  # persisting L2
    assert lib.qses_set_default_smoothing_shape(1, 768, 4096, 16) == L.QSES_ERR_INVALID_ARG
    launch = (ctypes.c_uint * 6)()
    assert lib.qses_debug_slab_plan(1000, None, None, 1, 1024, 4096, 48, 0, 152, launch, None, 0) == L.QSES_ERR_INVALID_ARG


@pytest.mark.parametrize("flags", [16, 18, 32, 34])
def test_lane_groups_do_not_change_the_plan(flags):
    # the lane mode is a property of the kernel, not of the slab split
    rng = np.random.default_rng(7)
    sizes = rng.integers(100, 200_000, 40)
    mol_off = np.concatenate([[0], np.cumsum(sizes)])
    depth = rng.integers(20, 700, 40)
    base = _plan(int(mol_off[-1]), mol_off, depth, target=25000, flags=flags & 15)
    info, waves = _plan(int(mol_off[-1]), mol_off, depth, target=25000, flags=flags)
    assert {k: info[k] for k in ("ctas", "smax", "qcap", "wsize", "waves")} == \
        {k: base[0][k] for k in ("ctas", "smax", "qcap", "wsize", "waves")}
    for (b0, o0), (b1, o1) in zip(base[1], waves):
        assert np.array_equal(b0, b1) and np.array_equal(o0, o1)

"""Seeded synthetic molecules (the benchmark workloads use no public dataset).

Workloads (heavy atoms, C/N/O/S 62/17/19/2 % with radii 1.70/1.55/1.52/1.80 A, 1.2 A
minimum pair distance, probe 1.4 A):

* ``ball1k``    1 000 atoms uniform in a ball at 0.05 atoms/A^3, voxel 0.5 A, 1 pass
* ``ball50k``   50 000 atoms, same generator, voxel 0.2 A, 1 pass (multi-slice grid)
* ``shell1m``   1 000 000 atoms uniform in a 400-430 A shell, voxel 0.5 A, 0 passes
* ``ball20k``   20 000 atoms, voxel 0.2 A, 1 pass (profiling size: ~127 M voxels, field
                larger than L2, well under the device memory of a capture)

Request streams for the batch and served forms:

* :func:`uneven_batch`   molecules with atom counts log-uniform in [500, 20 000], voxel 0.4
* :func:`trajectory`     one 5 000-atom molecule plus i.i.d. N(0, 0.3^2) jitter per frame
* :func:`served_stream`  atom counts log-uniform in [200, 200 000], voxel one of
                         {0.3, 0.4, 0.5}; requests draw from a pool of distinct molecules
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L

DENSITY = 0.05
MIN_DIST = 1.2


def _call(fn, n, *args):
    xyz = np.zeros((n, 3), np.float32)
    rad = np.zeros(n, np.float32)
    elem = np.zeros(n, np.uint8)
    rc = fn(*args, xyz.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            rad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), elem.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    if rc != L.QSES_OK:
        raise ValueError("synthetic generator failed: " + L.status_string(rc))
    return xyz, rad, elem


def ball(n, seed=1, density=DENSITY, min_dist=MIN_DIST):
    """n atoms uniform in a ball of radius (3n / (4 pi density))^(1/3)."""
    return _call(L.lib().qses_synth_ball, n, ctypes.c_uint(n), ctypes.c_uint64(seed), ctypes.c_float(density),
                 ctypes.c_float(min_dist))


def shell(n, seed=1, r_in=400.0, thickness=30.0, min_dist=MIN_DIST):
    """n atoms uniform in volume in the shell [r_in, r_in + thickness]."""
    return _call(L.lib().qses_synth_shell, n, ctypes.c_uint(n), ctypes.c_uint64(seed), ctypes.c_float(r_in),
                 ctypes.c_float(thickness), ctypes.c_float(min_dist))


def jitter(xyz, sigma, seed):
    xyz = np.ascontiguousarray(xyz, np.float32)
    out = np.zeros_like(xyz)
    rc = L.lib().qses_synth_jitter(xyz.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), xyz.shape[0],
                                   ctypes.c_float(sigma), ctypes.c_uint64(seed),
                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    if rc != L.QSES_OK:
        raise ValueError("jitter failed")
    return out


@dataclass(frozen=True)
class Workload:
    name: str
    kind: str
    n_atoms: int
    voxel: float
    smooth: int
    seed: int = 1

    def atoms(self):
        if self.kind == "ball":
            return ball(self.n_atoms, self.seed)
        return shell(self.n_atoms, self.seed)


WORKLOADS = {
    "ball1k": Workload("ball1k", "ball", 1000, 0.5, 1),
    "ball50k": Workload("ball50k", "ball", 50000, 0.2, 1),
    "shell1m": Workload("shell1m", "shell", 1000000, 0.5, 0),
    "ball20k": Workload("ball20k", "ball", 20000, 0.2, 1),
}


def _req(xyz, rad, voxel, smooth=1):
    return {"xyz": xyz, "radii": rad, "voxel": float(voxel), "smooth": int(smooth), "keep_degenerate": False}


def uneven_batch(count=256, seed=2024, lo=500, hi=20000, voxel=0.4):
    """`count` independent ball molecules, atom counts log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(int)
    return [_req(*ball(int(n), seed * 1000 + k)[:2], voxel) for k, n in enumerate(sizes)]


def trajectory(frames=512, n=5000, sigma=0.3, seed=77, voxel=0.4):
    """Frames of one molecule: base coordinates plus i.i.d. Gaussian jitter."""
    base, rad, _ = ball(n, seed)
    return [_req(jitter(base, sigma, seed * 100000 + f), rad, voxel) for f in range(frames)]


def served_stream(count, seed=9, pool=160, lo=200, hi=200000, voxels=(0.3, 0.4, 0.5)):
    """`count` requests drawn from `pool` distinct molecules (atom counts log-uniform in
    [lo, hi]), each with a voxel size drawn uniformly from `voxels`."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), pool)).astype(int)
    mols = [ball(int(n), seed * 10000 + k)[:2] for k, n in enumerate(sizes)]
    picks = rng.integers(0, pool, count)
    vox = rng.choice(np.asarray(voxels, np.float64), count)
    return [_req(mols[p][0], mols[p][1], v) for p, v in zip(picks, vox)]

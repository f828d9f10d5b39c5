"""SES mesher benchmark: voxels/s per molecule on a seeded synthetic molecule.

Workload (default): 50 000 heavy atoms uniform in a ball at 0.05 atoms/A^3 (1.2 A minimum
pair distance, C/N/O/S mix), voxel 0.2 A, probe 1.4 A, 1 Laplacian pass - the multi-slice
single-molecule configuration.  voxels = G^3 of the reference's grid sizing.

* value     G^3 / device time per step, atoms already in HBM (qses_compute_device)
* e2e       same metric through the C-ABI with host buffers (qses_compute: atom upload,
            full pipeline, mesh download into library-owned pinned buffers)
* roofline  dominant stage: algorithmic bytes / its CUDA-event time vs measured HBM peak
* cpu_baseline  the CPU oracle on a bounded slab of the same grid, all host threads

`--impl reference` times the reference path's CPU implementation instead: QuickSES has no
CPU field code, so this is the CPU oracle port (C++/OpenMP restatement) on the same
workload, one bounded slab per step.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 2 ** 20


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, device=0):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench.csv")
        self.device = device

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.f.close()

    def summary(self):
        try:
            rows = [ln.split(",") for ln in open(self.path).read().strip().splitlines()]
            sm = [float(r[0]) for r in rows if r[0].strip().replace(".", "").isdigit()]
            mx = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = sorted({names[q] for r in rows for q in range(4) if len(r) > 3 + q and r[3 + q].strip() == "Active"})
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                    "reasons": reasons, "samples": len(sm)}
        except Exception as e:  # noqa: BLE001
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(e)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(values, world, device=None):
    """Element-wise max of per-rank floats over all ranks (identity when world == 1).
    The timed region's duration is the slowest rank's."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu().tolist()]


def aggregate(world, units_per_rank, ms_max, e2e_ms_max):
    """Whole-job throughput of N replicas: every rank processes the same units per step,
    so the job rate is world * units / (slowest rank's time)."""
    return world * units_per_rank / (ms_max * 1e-3), world * units_per_rank / (e2e_ms_max * 1e-3)


def algorithmic_bytes(stage, g, n_atoms, T, nv, NE, passes):
    """Compulsory HBM bytes of one launch of each stage (roofline)."""
    G3 = float(g.G) ** 3
    nrow = float(g.Gc + 1) ** 2
    if stage == "sas":
        return G3 / 4.0 + 16.0 * n_atoms                      # in+out bit masks written, atoms read
    if stage == "refine":
        return G3 / 4.0 + G3 * (1.0 + 1.0 / 8.0)              # masks read, codes + sign bits written
    if stage == "mc_count":
        return G3 / 8.0 + 8.0 * nrow                           # sign bits read, row counts written
    if stage == "mc_emit":
        return G3 / 8.0 + 8.0 * nrow + 12.0 * T + 8.0 * NE     # signs, row bases, triangles, edge keys
    if stage == "weld":
        return 2 * 12.0 * NE + 12.0 * nv + 2 * 12.0 * T         # key+slot read/written per pass floor
    if stage == "smooth":
        return passes * (12.0 * nv * 2 + 24.0 * T * 4 / 3)     # positions in/out + neighbour lists
    if stage == "closest_atom":
        return 12.0 * nv + 8.0 * nv + 16.0 * n_atoms
    return 0.0


def run_gpu(args):
    import torch
    import quickses_gb300 as q
    from quickses_gb300 import _lib as L

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    wl = q.molecules.WORKLOADS[args.workload]
    xyz, rad, _ = wl.atoms()
    n = xyz.shape[0]
    gi = q.grid_info(xyz, rad, wl.voxel)
    voxels = float(gi.G) ** 3
    stream = torch.cuda.Stream()
    ctx = q.Context(local, stream=stream.cuda_stream)
    d_xyz = torch.from_numpy(xyz).cuda(local)
    d_rad = torch.from_numpy(rad).cuda(local)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def step():
        return ctx.compute_device(d_xyz.data_ptr(), d_rad.data_ptr(), n, voxel=wl.voxel, smooth=wl.smooth)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            dm = step()
        torch.cuda.synchronize()
        # per-stage times on a separate profiled call (events on the context stream)
        ctx.set_profiling(True)
        step()
        stages = ctx.stage_times()
        diag = ctx.diagnostics()
        ctx.set_profiling(False)
        launches = ctx.last_launch_count()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        times = []
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            t_wall0 = time.perf_counter()
            for _ in range(args.steps):
                flush.zero_()  # L2 flush between steps, outside the event pair
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                dm = step()
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            torch.cuda.synchronize()
            t_wall = time.perf_counter() - t_wall0
        ms = float(np.mean(times))
    nv, nt = dm.n_vertices, dm.n_triangles

    # e2e through the C-ABI with host buffers (upload, pipeline, download to pinned host)
    lib = L.lib()
    pr = L.Params()
    lib.qses_params_default(ctypes.byref(pr))
    pr.voxel, pr.smooth_passes = wl.voxel, wl.smooth
    e2e_times = []
    mesh = L.Mesh()
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rc = lib.qses_compute(ctx.handle, ctypes.byref(pr), xyz.ctypes.data_as(ctypes.c_void_p),
                              rad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n, ctypes.byref(mesh))
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(lib.qses_last_error(ctx.handle).decode())
        h2d = 16 * n
        d2h = 12 * mesh.n_vertices + 12 * mesh.n_triangles + 8 * mesh.n_vertices
        lib.qses_mesh_release(ctypes.byref(mesh))
        if it >= args.warmup:
            e2e_times.append(dt)
    ms, e2e_ms = reduce_max([ms, 1e3 * float(np.mean(e2e_times))], world, device="cuda")
    if world > 1:
        dist.barrier()
    value, e2e_value = aggregate(world, voxels, ms, e2e_ms)

    # roofline of the dominant stage
    peak, peak_kind = peaks()
    g = gi
    T_all = nt  # kept triangles; emitted count is close
    dom = max(stages, key=lambda s: s[1]) if stages else ("none", 1.0)
    nbytes = algorithmic_bytes(dom[0], g, n, T_all, nv, nv, wl.smooth)
    achieved = nbytes / (dom[1] * 1e-3) / 1e9
    result = {
        "metric": "SES grid voxels/s per molecule",
        "value": value,
        "unit": "voxels/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded ball, 0.05 atoms/A^3, 1.2 A min distance, C/N/O/S mix)",
        "config": {"workload": "%s: %d atoms, voxel %.2f A, probe 1.4 A, %d smoothing pass, grid %d^3"
                               % (wl.name, n, wl.voxel, wl.smooth, gi.G),
                   "grid_dim": gi.G, "voxels": voxels, "atoms": n, "mesh_vertices": nv, "mesh_triangles": nt,
                   "l2": "flushed between timed steps (256 MB write outside the event pair)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": "voxels/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "qses_compute (C-ABI, pageable host atoms in, pinned host mesh out)"},
        "roofline": {"kernel": dom[0], "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes": nbytes, "stage_ms": dom[1], "traffic": None},
        "stages_ms": {k: round(v, 4) for k, v in stages},
        "gpu_launches": launches * args.steps,
        "smooth_diagnostics": diag,
        "clocks": clk.summary(),
        "wall_s": t_wall,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(wl, xyz, rad, args.cpu_planes)
    if world > 1:
        dist.destroy_process_group()
    ctx.close()
    if rank == 0:
        print(json.dumps(result))


def run_once(args):
    """One pipeline run through the C-ABI (host atoms in, host mesh out): a short program
    for profiler captures, with few launches before the kernel of interest."""
    import quickses_gb300 as q
    wl = q.molecules.WORKLOADS[args.workload]
    xyz, rad, _ = wl.atoms()
    with q.Context(0) as ctx:
        m = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=wl.smooth)
        print(json.dumps({"workload": wl.name, "grid": q.grid_info(xyz, rad, wl.voxel).G,
                          "vertices": len(m.vertices), "triangles": len(m.triangles),
                          "launches": ctx.last_launch_count()}))


def cpu_baseline(wl, xyz, rad, planes):
    """The CPU oracle (FP32 mode, all host threads): SAS classification + probe refine for
    `planes` x-planes of the grid (default: all of them; the refine halo is included in the
    work).  Marching cubes, weld and smoothing are left out, so this overstates the CPU's
    end-to-end rate.  voxels/s = voxels covered / time."""
    from oracle import oracle as O
    g, _ = O.grid(xyz, rad, wl.voxel)
    planes = g.G if planes <= 0 or planes > g.G else planes
    x0 = g.G // 2 - planes // 2
    t0 = time.perf_counter()
    O.field_codes(xyz, rad, g, fp64=False, x0=x0, x1=x0 + planes)
    dt = time.perf_counter() - t0
    cores = os.cpu_count()
    return {"value": planes * g.G * g.G / dt, "unit": "voxels/s", "cores": cores, "kind": "port",
            "sample": "oracle SAS+refine on x-planes [%d,%d) of the %d^3 grid (%.1f s); MC/weld/smoothing "
                      "not included" % (x0, x0 + planes, g.G, dt)}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import quickses_gb300 as q
    from oracle import oracle as O
    wl = q.molecules.WORKLOADS[args.workload]
    xyz, rad, _ = wl.atoms()
    g, _ = O.grid(xyz, rad, wl.voxel)
    planes = g.G if args.cpu_planes <= 0 or args.cpu_planes > g.G else args.cpu_planes
    x0 = g.G // 2 - planes // 2
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.field_codes(xyz, rad, g, fp64=False, x0=x0, x1=x0 + planes)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    sec = float(np.mean(times))
    v = planes * g.G * g.G / sec
    sample = ("CPU oracle port (C++/OpenMP restatement of the reference grid method; the reference ships no CPU "
              "field code): SAS+refine on %d of %d x-planes per step" % (planes, g.G))
    out = {"impl": "reference", "metric": "SES grid voxels/s per molecule", "value": v, "unit": "voxels/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "%s: %d atoms, voxel %.2f A, grid %d^3" % (wl.name, len(rad), wl.voxel, g.G)},
           "cpu_baseline": {"value": v, "unit": "voxels/s", "cores": os.cpu_count(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ball50k")
    ap.add_argument("--cpu-planes", type=int, default=0, help="x-planes of the CPU sample (0 = whole grid)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-once", action="store_true",
                    help="run the pipeline once on the workload (for profiler captures) and exit")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_once:
        run_once(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

"""SES mesher benchmark: voxels/s per molecule on a seeded synthetic molecule.

Workload (default): 50 000 heavy atoms uniform in a ball at 0.05 atoms/A^3 (1.2 A minimum
pair distance, C/N/O/S mix), voxel 0.2 A, probe 1.4 A, 1 Laplacian pass - the multi-slice
single-molecule configuration.  voxels = G^3 of the reference's grid sizing.

* value          G^3 / device time per step, atoms already in HBM (qses_compute_device)
* e2e            same metric through the C-ABI with host buffers (qses_compute: atom upload,
                 full pipeline, mesh download into library-owned pinned buffers)
* roofline       dominant stage: algorithmic bytes / its CUDA-event time vs measured HBM peak
* other_configs  the 1 000-atom ball (0.5 A) and the 1 M-atom shell (0.5 A, no smoothing):
                 device and end-to-end times
* ref_cuda       the reference's own CUDA build (API_computeSES) on the same molecules and
                 GPU, wall clock, in a child process; ratio = its time / our end-to-end time
* cpu_baseline   the CPU job of one step on the host cores: the FP64 oracle (field, marching
                 cubes, weld, closest atom) + the reference's own SmoothMesh.cpp

`--impl reference` times that CPU job per step instead (QuickSES's only CPU code on the path
is its smoothing; the rest is the oracle, its CPU restatement).  Its inputs come from the
oracle's generator, so that arm never loads the product library.
"""
import argparse
import atexit
import datetime
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 2 ** 20

# dram__bytes_read.sum + dram__bytes_write.sum of one launch of a stage's kernel, from the
# ncu capture summarised in the named profile (update both together).
NCU_TRAFFIC = {
    ("ball50k", "smooth"): {"bytes": 509.28e6, "source": "profiles/k_gs_flow_ball50k.md"},
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling.  Started before the warm-up (nvidia-smi's start-up
    slows CUDA calls for a while), summarised over the samples stamped between mark() and
    stop(): the timed region."""

    def __init__(self, device=0, interval_ms=100):
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="qses_clocks_", suffix=".csv")
        os.close(fd)
        self.device = device
        self.interval_ms = interval_ms
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=timestamp,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        if self.proc:
            atexit.register(self._kill)  # never leave the sampler behind
        return self

    def _kill(self):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
        try:
            os.unlink(self.path)
        except OSError:
            pass

    def mark(self):
        self.t0 = datetime.datetime.now()

    def stop(self):
        self.t1 = datetime.datetime.now()
        if self.proc and self.proc.poll() is None:
            time.sleep(0.15)
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.f.close()

    def summary(self):
        try:
            rows = []
            for ln in open(self.path).read().strip().splitlines():
                r = [x.strip() for x in ln.split(",")]
                try:
                    ts = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f")
                except ValueError:
                    continue
                if (self.t0 is None or ts >= self.t0) and (self.t1 is None or ts <= self.t1):
                    rows.append(r[1:])
            sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
            mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = sorted({names[q] for r in rows for q in range(4) if len(r) > 3 + q and r[3 + q] == "Active"})
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
    """Compulsory HBM bytes of one launch of each stage: what the stage must read and write
    at least once (bit masks, codes, triangles, edge keys, positions, neighbour lists)."""
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
    ctx.set_graphs(not args.no_graphs)
    d_xyz = torch.from_numpy(xyz).cuda(local)
    d_rad = torch.from_numpy(rad).cuda(local)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def step():
        return ctx.compute_device(d_xyz.data_ptr(), d_rad.data_ptr(), n, voxel=wl.voxel, smooth=wl.smooth)

    with torch.cuda.stream(stream):
        # launch-shape tuning of the smoothing kernel (same mesh for every shape), before
        # the warm-up: it runs the pipeline once per candidate shape
        clk = ClockSampler(local).start()
        tuned = ctx.autotune(xyz, rad, voxel=wl.voxel, smooth=wl.smooth) if wl.smooth > 0 else None
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
        torch.cuda.synchronize()
        clk.mark()
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
        clk.stop()
        ms = float(np.mean(times))
        graphs_timed = ctx.graph_stats()
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
        d2h = int(lib.qses_last_download_bytes(ctx.handle))  # triangles sized by the pre-filter count
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
        "config": {"workload": workload_desc(wl, n, gi.G),
                   "grid_dim": gi.G, "voxels": voxels, "atoms": n, "mesh_vertices": nv, "mesh_triangles": nt,
                   "l2": "flushed between timed steps (256 MB write outside the event pair)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "smoothing_shape": None if tuned is None else
                   {"threads": tuned[0], "slab_target": tuned[1], "cache_flags": tuned[2]},
                   "refine_tile": None if tuned is None else ["8x8", "16x8", "16x16", "32x16"][tuned[3]],
                   "cuda_graphs": _graph_summary(args, graphs_timed)},
        "e2e": {"value": e2e_value, "unit": "voxels/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "qses_compute (C-ABI, pageable host atoms in, pinned host mesh out)"},
        "roofline": {"kernel": dom[0], "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes": nbytes, "stage_ms": dom[1],
                     "traffic": NCU_TRAFFIC.get((wl.name, dom[0]), {}).get("bytes"),
                     "traffic_source": NCU_TRAFFIC.get((wl.name, dom[0]), {}).get("source")},
        "stages_ms": {k: round(v, 4) for k, v in stages},
        "gpu_launches": launches * args.steps,
        "smooth_diagnostics": diag,
        "clocks": clk.summary(),
        "wall_s": t_wall,
    }
    if rank == 0 and world == 1 and not args.no_other_configs:
        # the other single-molecule workloads, device time and end to end, then the
        # reference's own CUDA build on the same three molecules
        result["other_configs"] = {k: time_config(ctx, stream, q.molecules.WORKLOADS[k], flush, args)
                                   for k in ("ball1k", "shell1m")}
        result["ref_cuda"] = ref_cuda_block(args, {wl.name: (voxels, e2e_ms), **{
            k: (v["voxels"], v["e2e_ms"]) for k, v in result["other_configs"].items()}})
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(wl, *oracle_atoms(wl), gi.G)
    if world > 1:
        dist.destroy_process_group()
    ctx.close()
    if rank == 0:
        print(json.dumps(result))


def time_config(ctx, stream, wl, flush, args):
    """One more single-molecule workload: device time per call with atoms in HBM (CUDA
    events on the context stream, L2 flushed between calls) and end-to-end time through
    qses_compute with host buffers."""
    import torch
    import quickses_gb300 as q
    from quickses_gb300 import _lib as L
    xyz, rad, _ = wl.atoms()
    n = len(rad)
    G = q.grid_info(xyz, rad, wl.voxel).G
    d_xyz, d_rad = torch.from_numpy(xyz).cuda(), torch.from_numpy(rad).cuda()
    steps = max(3, min(args.steps, 10))
    with torch.cuda.stream(stream):
        if wl.smooth > 0:
            ctx.autotune(xyz, rad, voxel=wl.voxel, smooth=wl.smooth)
        for _ in range(3):
            dm = ctx.compute_device(d_xyz.data_ptr(), d_rad.data_ptr(), n, voxel=wl.voxel, smooth=wl.smooth)
        times = []
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dm = ctx.compute_device(d_xyz.data_ptr(), d_rad.data_ptr(), n, voxel=wl.voxel, smooth=wl.smooth)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ctx.set_profiling(True)
        ctx.compute_device(d_xyz.data_ptr(), d_rad.data_ptr(), n, voxel=wl.voxel, smooth=wl.smooth)
        stages = ctx.stage_times()
        ctx.set_profiling(False)
    torch.cuda.synchronize()
    lib = L.lib()
    pr = L.Params()
    lib.qses_params_default(ctypes.byref(pr))
    pr.voxel, pr.smooth_passes = wl.voxel, wl.smooth
    mesh, e2e = L.Mesh(), []
    for it in range(3 + steps):
        t0 = time.perf_counter()
        rc = lib.qses_compute(ctx.handle, ctypes.byref(pr), xyz.ctypes.data_as(ctypes.c_void_p),
                              rad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n, ctypes.byref(mesh))
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(lib.qses_last_error(ctx.handle).decode())
        lib.qses_mesh_release(ctypes.byref(mesh))
        if it >= 3:
            e2e.append(dt)
    del d_xyz, d_rad
    ms, e2e_ms = float(np.mean(times)), 1e3 * float(np.mean(e2e))
    return {"workload": workload_desc(wl, n, G), "voxels": float(G) ** 3, "steps": steps,
            "ms_per_step": ms, "voxels_per_s": float(G) ** 3 / (ms * 1e-3),
            "e2e_ms": e2e_ms, "e2e_voxels_per_s": float(G) ** 3 / (e2e_ms * 1e-3),
            "mesh_vertices": dm.n_vertices, "mesh_triangles": dm.n_triangles,
            "stages_ms": {k: round(v, 4) for k, v in stages}}


# Timed calls of the reference's own CUDA build per workload (its 1 M-atom shell runs
# seconds per call).
REF_CUDA_CALLS = {"ball1k": 10, "ball50k": 3, "shell1m": 1}


def ref_cuda_block(args, ours):
    """The reference's own CUDA build (oracle/_ref/libQuickSES.so, compiled from its sources
    for sm_103a by oracle/build.py) on the same molecules and the same GPU, in a child
    process: wall clock of API_computeSES (host atoms in, host mesh out).  `ours` maps a
    workload to (voxels, our end-to-end ms through qses_compute); the ratio is ours over
    the reference's, both end to end."""
    lib = os.path.join(ROOT, "oracle", "_ref", "libQuickSES.so")
    if not os.path.exists(lib):
        return {"unavailable": "the reference's CUDA build (oracle/_ref/libQuickSES.so) was not built: its "
                               "sources were not at hand"}
    out = {"path": "API_computeSES of the reference's own CUDA build, wall clock around the call, one molecule "
                   "per call, same atoms and GPU"}
    for name, (voxels, e2e_ms) in ours.items():
        calls = REF_CUDA_CALLS.get(name, 3)
        try:
            r = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "ref_cuda", "run_ref.py"), "bench",
                                name, str(calls)], capture_output=True, text=True, timeout=args.ref_cuda_timeout)
            line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not line:
                out[name] = {"unavailable": "reference run failed (rc %d): %s" % (
                    r.returncode, (r.stderr.strip().splitlines() or ["no output"])[-1][:200])}
                continue
            d = json.loads(line[-1])
        except subprocess.TimeoutExpired:
            out[name] = {"unavailable": "reference run exceeded %d s" % args.ref_cuda_timeout}
            continue
        ms = float(np.mean(d["ms"]))
        out[name] = {"ms_per_call": ms, "voxels_per_s": voxels / (ms * 1e-3), "calls": d["calls"],
                     "mesh_vertices": d["vertices"], "ours_e2e_ms": e2e_ms,
                     "ratio_e2e": ms / e2e_ms}
    return out


def run_once(args):
    """One pipeline run through the C-ABI (host atoms in, host mesh out), or one batch call
    with --form batched / trajectory: a short program for profiler captures, with few
    launches before the kernel of interest."""
    import quickses_gb300 as q
    if args.form in ("batched", "trajectory"):
        # one qses_compute_batch of the batch form's molecule stream
        reqs = q.molecules.uneven_batch(256) if args.form == "batched" else q.molecules.trajectory(512)
        with q.Context(0) as ctx:
            if args.gs_shape:
                ctx.set_smoothing_shape(*[int(x) for x in args.gs_shape.split(",")])
            out = ctx.compute_batch(reqs)
            print(json.dumps({"form": args.form, "molecules": len(reqs),
                              "vertices": int(sum(len(m.vertices) for m in out)),
                              "triangles": int(sum(len(m.triangles) for m in out)),
                              "launches": ctx.last_launch_count()}))
        return
    wl = q.molecules.WORKLOADS[args.workload]
    xyz, rad, _ = wl.atoms()
    with q.Context(0) as ctx:
        if args.gs_shape:
            ctx.set_smoothing_shape(*[int(x) for x in args.gs_shape.split(",")])
        m = ctx.compute(xyz, rad, voxel=wl.voxel, smooth=wl.smooth)
        print(json.dumps({"workload": wl.name, "grid": q.grid_info(xyz, rad, wl.voxel).G,
                          "vertices": len(m.vertices), "triangles": len(m.triangles),
                          "launches": ctx.last_launch_count()}))


def workload_desc(wl, n, G):
    """The workload string both arms print (the same text for the same job)."""
    return "%s: %d atoms, voxel %.2f A, probe 1.4 A, %d smoothing pass, grid %d^3" % (wl.name, n, wl.voxel,
                                                                                  wl.smooth, G)


def oracle_atoms(wl):
    """The workload's atoms from the oracle's generator (bit-identical to the library's,
    tests/test_oracle_synth.py): the CPU legs never load the product library."""
    from oracle import oracle as O
    if wl.kind == "ball":
        return O.synth_ball(wl.n_atoms, wl.seed)
    return O.synth_shell(wl.n_atoms, wl.seed)


_REF_SMOOTH = []


def _ref_smooth_lib():
    """The reference's own CPU smoothing (SmoothMesh.cpp, compiled from its sources into
    oracle/_ref/libqses_ref_host.so), or None when its sources were not at hand."""
    if not _REF_SMOOTH:
        lib = None
        try:
            from oracle import build as ob
            path = ob.build_ref()
            if path:
                lib = ctypes.CDLL(path)
                lib.ref_smooth.restype = None
                lib.ref_smooth.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint,
                                           ctypes.c_uint]
        except Exception:  # noqa: BLE001
            lib = None
        _REF_SMOOTH.append(lib)
    return _REF_SMOOTH[0]


def cpu_step(wl, xyz, rad):
    """One CPU pass of the whole job: the FP64 oracle (OpenMP over all host threads) for the
    field, marching cubes, weld and closest atom, then the reference's own SmoothMesh.cpp
    (one thread, in place, as the reference runs it after each slice) for the smoothing
    passes.  Returns (seconds, seconds of the smoothing, description)."""
    from oracle import oracle as O
    ref = _ref_smooth_lib() if wl.smooth > 0 else None
    t0 = time.perf_counter()
    m = O.compute_ses(xyz, rad, wl.voxel, smooth=0 if ref is not None else wl.smooth, fp64=True)
    t1 = time.perf_counter()
    if ref is not None:
        v = np.ascontiguousarray(m.vertices_q, np.float32)
        t = np.ascontiguousarray(m.triangles, np.int32)
        ref.ref_smooth(wl.smooth, v.ctypes.data, t.ctypes.data, len(v), len(t))
    t2 = time.perf_counter()
    if ref is not None:
        how = ("FP64 oracle (field, marching cubes, weld, closest atom; %d threads) %.2f s + the reference's "
               "SmoothMesh.cpp (%d pass, 1 thread, %d vertices) %.2f s" % (os.cpu_count(), t1 - t0, wl.smooth,
                                                                        len(m.vertices_q), t2 - t1))
        return t2 - t0, t2 - t1, how
    how = ("FP64 oracle, whole pipeline including its sequential smoothing (%d threads; the reference's "
           "SmoothMesh.cpp was not available): %.2f s" % (os.cpu_count(), t1 - t0))
    return t1 - t0, None, how


def cpu_baseline(wl, xyz, rad, G):
    """The CPU job of one GPU step (cpu_step), once, on the same molecule."""
    dt, t_smooth, how = cpu_step(wl, xyz, rad)
    return {"value": float(G) ** 3 / dt, "unit": "voxels/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "the whole %d^3 grid, one molecule: %s" % (G, how),
            "cpu_smooth_ms": None if t_smooth is None else 1e3 * t_smooth}


def _libs_loaded():
    try:
        with open("/proc/self/maps") as f:
            return sorted({ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")})
    except OSError:
        return []


def run_reference(args):
    """The reference's CPU implementation of the path on the host cores: QuickSES has CPU
    code only for the smoothing (SmoothMesh.cpp, timed as the reference's own code); the
    field, marching cubes and weld run in the FP64 oracle, its CPU restatement.  Inputs and
    grid sizes come from the oracle, so this arm never loads the product library."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from quickses_gb300.molecules import WORKLOADS  # plain data; loads no library
    wl = WORKLOADS[args.workload]
    xyz, rad = oracle_atoms(wl)
    g, _ = O.grid(xyz, rad, wl.voxel)
    times, smooth_times, how = [], [], ""
    for it in range(args.warmup + args.steps):
        dt, t_smooth, how = cpu_step(wl, xyz, rad)
        if it >= args.warmup:
            times.append(dt)
            if t_smooth is not None:
                smooth_times.append(t_smooth)
    sec = float(np.mean(times))
    v = float(g.G) ** 3 / sec
    product = [p for p in _libs_loaded() if "libquickses_gb300" in p]
    assert not product, "the reference arm loaded the product library: %s" % product
    out = {"impl": "reference", "metric": "SES grid voxels/s per molecule", "value": v, "unit": "voxels/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": workload_desc(wl, len(rad), g.G)},
           "cpu_baseline": {"value": v, "unit": "voxels/s", "cores": os.cpu_count(), "kind": "port",
                            "sample": "each step the whole %d^3 grid, one molecule: %s" % (g.G, how)},
           "cpu_smooth_ms": float(np.mean(smooth_times)) * 1e3 if smooth_times else None,
           "e2e": {"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ------------------------------------------------------------ batch and served forms

def _raw_batch(lib, L, ctx, rr, n):
    meshes = (L.Mesh * n)()
    st = (ctypes.c_int * n)()
    rc = lib.qses_compute_batch(ctx.handle, rr, n, meshes, st)
    if rc != 0:
        raise RuntimeError(lib.qses_last_error(ctx.handle).decode())
    nv = sum(meshes[i].n_vertices for i in range(n))
    nt = sum(meshes[i].n_triangles for i in range(n))
    bad = sum(1 for i in range(n) if st[i] != 0)
    for i in range(n):
        lib.qses_mesh_release(ctypes.byref(meshes[i]))
    return nv, nt, bad


def _raw_single(lib, L, ctx, reqs):
    pr = L.Params()
    lib.qses_params_default(ctypes.byref(pr))
    m = L.Mesh()
    for r in reqs:
        pr.voxel, pr.smooth_passes = r["voxel"], r["smooth"]
        rc = lib.qses_compute(ctx.handle, ctypes.byref(pr), r["xyz"].ctypes.data_as(ctypes.c_void_p),
                              r["radii"].ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(r["radii"]),
                              ctypes.byref(m))
        if rc != 0:
            raise RuntimeError(lib.qses_last_error(ctx.handle).decode())
        lib.qses_mesh_release(ctypes.byref(m))


def _graph_summary(args, stats):
    """How the pipeline segments ran: counters since the context was created (the
    autotuner, warm-up and profiled calls included)."""
    if args.no_graphs:
        return "off (every kernel launched directly)"
    return dict(stats, mode="segments replayed from CUDA graphs; captured again and updated in place when "
                            "their pointers, counts or shapes change")


def run_batch_form(args):
    """Batch form: one step = every molecule of the stream through qses_compute_batch (host
    atoms in, host meshes out).  Beside it, the same molecules one by one through
    qses_compute (the plain per-molecule path) on the same GPU."""
    import quickses_gb300 as q
    from quickses_gb300 import _lib as L, api as A
    lib = L.lib()
    if args.form == "batched":
        reqs = q.molecules.uneven_batch(256)
        desc = "256 molecules, atom counts log-uniform in [500, 20000], voxel 0.4 A, 1 pass"
    else:
        reqs = q.molecules.trajectory(512)
        desc = "5000-atom molecule x 512 frames (N(0, 0.3^2) jitter), voxel 0.4 A, 1 pass"
    n = len(reqs)
    voxels = float(sum(q.grid_info(r["xyz"], r["radii"], r["voxel"]).G ** 3 for r in reqs))
    arrays, rr = A._requests(reqs)
    with q.Context(0) as ctx:
        ctx.set_graphs(not args.no_graphs)
        clk = ClockSampler(0).start()
        tune = ctx.autotune_batch(reqs)  # launch-shape tuning, before the warm-up
        for _ in range(args.warmup):
            _raw_batch(lib, L, ctx, rr, n)
        ctx.set_profiling(True)
        _raw_batch(lib, L, ctx, rr, n)
        stages = ctx.stage_times()
        launches = ctx.last_launch_count()
        ctx.set_profiling(False)
        times, timelines = [], []
        clk.mark()
        for _ in range(args.steps):
            t0 = time.perf_counter()
            nv, nt, bad = _raw_batch(lib, L, ctx, rr, n)
            times.append(time.perf_counter() - t0)
            timelines.append(ctx.host_timeline())
        clk.stop()
        sec = float(np.mean(times))
        graphs_timed = ctx.graph_stats()
        timeline = timelines[-1]
        _raw_single(lib, L, ctx, reqs[:8])
        t0 = time.perf_counter()
        _raw_single(lib, L, ctx, reqs)
        t_plain = time.perf_counter() - t0
    h2d = sum(16 * len(r["radii"]) for r in reqs)
    d2h = 12 * nv + 12 * nt + 8 * nv
    print(json.dumps({
        "metric": "SES molecules/s (%s form)" % args.form, "value": n / sec, "unit": "molecules/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": desc, "form": args.form, "molecules": n, "voxels": voxels,
                   "mesh_vertices": nv, "mesh_triangles": nt, "rejected": bad,
                   "smoothing_shape": {"threads": tune[0], "slab_target": tune[1], "cache_flags": tune[2]},
                   "l2": "inputs and meshes far larger than L2",
                   "cuda_graphs": _graph_summary(args, graphs_timed)},
        "voxels_per_s": voxels / sec,
        "e2e": {"value": n / sec, "unit": "molecules/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "qses_compute_batch (C-ABI, host atoms in, host meshes out)"},
        "plain_path": {"value": n / t_plain, "unit": "molecules/s",
                       "path": "the same molecules one by one through qses_compute on the same GPU"},
        "stages_ms": {k: round(v, 3) for k, v in stages}, "gpu_launches": launches * args.steps,
        "step_ms": [round(1e3 * t, 3) for t in times],
        "host_timeline_ms": {k: round(v, 3) for k, v in timeline.items()},
        "step_timelines_ms": [{k: round(v, 2) for k, v in tl.items()} for tl in timelines],
        "clocks": clk.summary()}))


def _raw_wait(lib, L, srv, ticket):
    """One result through the C-ABI (qses_server_wait + qses_mesh_release, the mesh stays in
    its pinned block: no copy into Python arrays); returns its submit-to-result time (s)."""
    m, info = L.Mesh(), L.TicketInfo()
    rc = lib.qses_server_wait(srv.handle, ctypes.c_ulonglong(ticket), -1.0, ctypes.byref(m), ctypes.byref(info))
    lib.qses_mesh_release(ctypes.byref(m))
    if rc != 0:
        raise RuntimeError("served request failed: %d" % rc)
    return info.total_s


def run_served_form(args):
    """Served form: open-loop Poisson arrivals into qses_server (continuous batching over
    `lanes` streams, 120 GB admission budget); per offered rate, p50/p99 of submit-to-result
    latency and the completed-request rate.  Requests: atom counts log-uniform in
    [200, 200000], voxel one of {0.3, 0.4, 0.5} A, 1 pass, drawn from 160 seeded molecules.
    Results are taken through the C-ABI without copying the meshes into Python."""
    import threading
    import quickses_gb300 as q
    from quickses_gb300 import _lib as L
    lib = L.lib()
    rates = [float(x) for x in args.rates.split(",")]
    per_rate = args.requests
    reqs = q.molecules.served_stream(per_rate * len(rates) + 64)
    rng = np.random.default_rng(11)
    sweep = []
    clk = ClockSampler(0).start()
    if args.served_shape:  # a fixed process-wide shape for the lanes (e.g. one that shares the SMs)
        th, tg, fl = [int(x) for x in args.served_shape.split(",")]
        from quickses_gb300 import _lib as L0
        if L0.lib().qses_set_default_smoothing_shape(1, th, tg, fl) != 0:
            raise SystemExit("bad --served-shape")
        tune = (th, tg, fl, 0.0)
    else:
        with q.Context(0) as tctx:  # launch-shape tuning on a sample (process-wide, like a service start)
            tune = tctx.autotune_batch(reqs[-64:-32])
    with q.Server(lanes=args.lanes, memory_budget=120 << 30, max_batch=256,
                  max_batch_voxels=int(args.batch_voxels) if args.batch_voxels else None) as srv:
        # warm-up: a burst, so that batches as large as the timed ones form and workspaces and
        # pinned blocks grow to size before the timed phases
        for _ in range(2):
            warm = [srv.submit(r["xyz"], r["radii"], r["voxel"], r["smooth"]) for r in reqs[-64:]]
            for t in warm:
                _raw_wait(lib, L, srv, t)
        clk.mark()
        for ri, rate in enumerate(rates):
            chunk = reqs[ri * per_rate:(ri + 1) * per_rate]
            arrivals = np.cumsum(rng.exponential(1.0 / rate, per_rate))
            tickets = [None] * per_rate

            def submitter():
                t0 = time.perf_counter()
                for k, r in enumerate(chunk):
                    d = t0 + arrivals[k] - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    tickets[k] = srv.submit(r["xyz"], r["radii"], r["voxel"], r["smooth"])

            t_start = time.perf_counter()
            th = threading.Thread(target=submitter)
            th.start()
            lat = []
            for k in range(per_rate):
                while tickets[k] is None:
                    time.sleep(0.0002)
                lat.append(_raw_wait(lib, L, srv, tickets[k]))
            t_end = time.perf_counter()
            th.join()
            lat = np.array(lat) * 1e3
            sweep.append({"offered_per_s": rate, "achieved_per_s": per_rate / (t_end - t_start),
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "requests": per_rate})
        clk.stop()
        stats = srv.stats()
    # the plain per-request path on the same GPU: one qses_compute at a time, closed loop, on
    # the first requests of the chunk that gave the reported served rate (the same mix)
    from quickses_gb300 import _lib as L
    bi = max(range(len(sweep)), key=lambda i: sweep[i]["achieved_per_s"])
    best = sweep[bi]
    sample = reqs[bi * per_rate:(bi + 1) * per_rate][:192]
    with q.Context(0) as ctx:
        _raw_single(L.lib(), L, ctx, reqs[-8:])
        t0 = time.perf_counter()
        _raw_single(L.lib(), L, ctx, sample)
        plain = len(sample) / (time.perf_counter() - t0)
    print(json.dumps({
        "metric": "SES molecules/s (served form)", "value": best["achieved_per_s"], "unit": "molecules/s",
        "n_gpus": 1, "steps": len(rates), "warmup": 128, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "open-loop Poisson, %d requests per offered rate, atom counts log-uniform in "
                               "[200, 200000], voxel one of {0.3, 0.4, 0.5} A, 1 pass" % per_rate,
                   "form": "served", "lanes": args.lanes, "memory_budget_gb": 120,
                   "max_batch_voxels": args.batch_voxels or 1e9,
                   "smoothing_shape": {"threads": tune[0], "slab_target": tune[1], "cache_flags": tune[2]}},
        "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"], "sweep": sweep, "server": stats,
        "plain_path": {"value": plain, "unit": "molecules/s",
                       "path": "the first %d requests of the %g req/s chunk one by one through qses_compute on "
                               "the same GPU" % (len(sample), best["offered_per_s"])},
        "clocks": clk.summary()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ball50k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the 1 000-atom and 1 M-atom workloads and the reference CUDA build's timings")
    ap.add_argument("--ref-cuda-timeout", type=int, default=240,
                    help="seconds per workload for the reference CUDA build's child process")
    ap.add_argument("--form", default="plain", choices=["plain", "batched", "trajectory", "served"],
                    help="plain: one molecule per step (default); batched/trajectory: a molecule stream per step "
                         "through qses_compute_batch; served: Poisson arrivals into qses_server")
    ap.add_argument("--rates", default="50,100,200,500,1000,2000", help="served form: offered requests/s")
    ap.add_argument("--requests", type=int, default=1000, help="served form: requests per offered rate")
    ap.add_argument("--lanes", type=int, default=2, help="served form: batches in flight")
    ap.add_argument("--served-shape", default="",
                    help="served form: smoothing shape threads,target,cache_flags for every lane (default: tuned)")
    ap.add_argument("--batch-voxels", type=float, default=0,
                    help="served form: grid voxels per batch (0 = the server's default)")
    ap.add_argument("--no-graphs", action="store_true", help="launch every kernel directly (no CUDA graphs)")
    ap.add_argument("--gs-shape", default="", help="profile-once: smoothing shape threads,target,cache_flags")
    ap.add_argument("--profile-once", action="store_true",
                    help="run the pipeline once on the workload (for profiler captures) and exit")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_once:
        run_once(args)
    elif args.form in ("batched", "trajectory") and args.impl == "ours":
        run_batch_form(args)
    elif args.form == "served" and args.impl == "ours":
        run_served_form(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

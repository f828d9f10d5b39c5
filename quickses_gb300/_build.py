"""Compile libquickses_gb300.so (and the QuickSES-compatible CLI) in-tree for sm_103a.

Plain nvcc / g++ invocations, translation units compiled in parallel, no cmake.  Objects
go to quickses_gb300/_build/, the library to quickses_gb300/libquickses_gb300.so and the
CLI to quickses_gb300/bin/QuickSES (all git-ignored build outputs).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libquickses_gb300.so")
CLI = os.path.join(PKG, "bin", "QuickSES")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = ["nvcc", "-std=c++17", "-O3", "-lineinfo"] + ARCH + [
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-I", CSRC, "-I", INCLUDE]
GXX = ["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
       "-I", "/usr/local/cuda/include", "-I", CSRC, "-I", INCLUDE]

LIB_CU = ["k_prims.cu", "k_field.cu", "k_hash.cu", "k_mesh.cu", "k_smooth.cu", "pipeline.cu", "pipeline_batch.cu", "pipeline_slices.cu", "noalloc.cu"]
# Per-file flags: the atom cell key uses the reference's own arithmetic (see k_hash.cu).
EXTRA_FLAGS = {"k_hash.cu": ["-use_fast_math"]}
LIB_CPP = ["api.cpp", "synth.cpp", "io.cpp", "server.cpp"]
CLI_CPP = ["cli.cpp"]


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _compile(src, verbose_ptxas=False):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _stale(obj, [path] + _headers()):
        return obj, ""
    if src.endswith(".cu"):
        cmd = NVCC + EXTRA_FLAGS.get(src, []) + (["-Xptxas", "-v"] if verbose_ptxas else []) + \
            ["-c", path, "-o", obj]
    else:
        cmd = GXX + ["-c", path, "-o", obj]
    return obj, _run(cmd)


def build(verbose_ptxas=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    srcs = LIB_CU + LIB_CPP + CLI_CPP
    srcs = [s for s in srcs if os.path.exists(os.path.join(CSRC, s))]
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_compile, s, verbose_ptxas): s for s in srcs}
        objs = {}
        for f in cf.as_completed(futs):
            objs[futs[f]], logs[futs[f]] = f.result()
    lib_objs = [objs[s] for s in LIB_CU + LIB_CPP if s in objs]
    if _stale(LIB, lib_objs):
        _run(["nvcc", "-shared"] + ARCH + ["-o", LIB] + lib_objs + ["-lpthread", "-ldl", "-lrt"])
    if "cli.cpp" in objs and _stale(CLI, [objs["cli.cpp"], LIB]):
        _run(["g++", "-o", CLI, objs["cli.cpp"], "-L", PKG, "-lquickses_gb300",
              "-Wl,-rpath,$ORIGIN/.."])
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(verbose_ptxas="-v" in sys.argv)
    for k, v in sorted(logs.items()):
        if v.strip():
            print("==", k)
            print(v)
    print(lib)

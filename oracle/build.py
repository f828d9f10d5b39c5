"""Build the CPU oracle (test infrastructure) and, where the reference's sources are at
hand, the reference-derived helpers under oracle/_ref/.

    python oracle/build.py            # oracle/liboracle.so (+ oracle/_ref/ if available)

The reference's sources are taken from, in this order: the `ref` argument, the checkout
named by $QSES_REFERENCE, or the copy staged into oracle/_ref/src by
`make -C oracle/ref_cuda stage REF_CHECKOUT=<checkout>` (git-ignored; it travels with the
working tree to machines without the checkout).  Nothing is built from them when none
exists.

The oracle is plain C++17 + OpenMP compiled with -ffp-contract=off so that its FP32
mode is IEEE single precision in the written operation order on both x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
STAGED = os.path.join(HERE, "_ref", "src")


def reference_sources(ref=None):
    """Directory with the reference's sources (see the module docstring), or None."""
    for d in (ref, os.environ.get("QSES_REFERENCE"), STAGED):
        if d and os.path.isfile(os.path.join(d, "SmoothMesh.cpp")):
            return d
    return None


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("oracle build failed: %s" % cmd[0])


def build_oracle():
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, "qses_oracle.cpp"), os.path.join(HERE, "oracle_synth.cpp")]
    deps = srcs + [os.path.join(HERE, "qses_oracle.h"), os.path.join(HERE, "mc_table.h")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
          "-o", out] + srcs)
    return out


def build_ref(ref=None):
    """Compile the reference's host-side code (SmoothMesh.cpp and the __host__ __device__
    helpers of Kernels.cu) from the reference checkout into oracle/_ref/.  Returns the
    library path, or None when the checkout is absent (e.g. on the GPU machine)."""
    ref = reference_sources(ref)
    if ref is None:
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libqses_ref_host.so")
    shim = os.path.join(HERE, "ref", "ref_host_shim.cu")
    deps = [shim, os.path.join(ref, "SmoothMesh.cpp"), os.path.join(ref, "Kernels.cu")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    obj_smooth = os.path.join(outdir, "SmoothMesh.o")
    obj_shim = os.path.join(outdir, "ref_host_shim.o")
    cuda_inc = "/usr/local/cuda/include"
    # SmoothMesh.cpp is plain C++ that only needs cuda_runtime.h for float3.
    _run(["g++", "-O3", "-fPIC", "-ffp-contract=off", "-I", cuda_inc, "-c",
          os.path.join(ref, "SmoothMesh.cpp"), "-o", obj_smooth])
    # The shim #includes Kernels.cu so its __host__ __device__ helpers run on the host.
    _run(["nvcc", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off", "-gencode",
          "arch=compute_103a,code=sm_103a", "-I", ref, "-c", shim, "-o", obj_shim])
    _run(["nvcc", "-shared", "-o", out, obj_shim, obj_smooth])
    return out


def build_ref_pdb(ref=None):
    """The reference's PDB parser (cpdb/cpdb.cpp) plus a walk shim, into
    oracle/_ref/libqses_ref_pdb.so.  None when the checkout is absent."""
    ref = reference_sources(ref)
    if ref is None:
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libqses_ref_pdb.so")
    shim = os.path.join(HERE, "ref", "ref_pdb_shim.cpp")
    src = os.path.join(ref, "cpdb", "cpdb.cpp")
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in (shim, src)):
        return out
    _run(["g++", "-O2", "-fPIC", "-shared", "-w", "-I", os.path.join(ref, "cpdb"), "-I", "/usr/local/cuda/include",
          "-o", out, shim, src])
    return out


def build_ref_cuda(ref=None):
    """The reference's own CUDA build (oracle/_ref/libQuickSES.so, its Makefile's
    shared-library recipe for sm_103a) and its field kernels for one slice
    (oracle/_ref/libref_field.so), by oracle/ref_cuda/Makefile.  Returns the library path,
    or None without the sources."""
    ref = reference_sources(ref)
    if ref is None:
        return None
    _run(["make", "-s", "-j2", "-C", os.path.join(HERE, "ref_cuda"), "SRC=" + ref])
    return os.path.join(HERE, "_ref", "libQuickSES.so")


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    print(build_ref_pdb())
    print(build_ref_cuda())

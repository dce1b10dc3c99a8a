"""Build recipe of the oracle -- TEST INFRASTRUCTURE ONLY (never linked by the product).

Products, all git-ignored and rebuilt on every machine:
  oracle/_build/liboracle.so             the CPU restatement (oracle.cpp, pathtrace.cpp)
  oracle/_build/libref_sort.so           CUB's stable merge sort of the reference GPU LBVH
                                         build's prim refs (ref_sort.cu; CUDA toolkit only)
  oracle/_ref/libvsnray_ref.so           visionaray's own CPU code, compiled from its
                                         unmodified headers (ref_driver.cpp)
  oracle/_ref/vsnray_ref_gpu.cubin       visionaray's own GPU traversal and path tracer
  oracle/_ref/vsnray_ref_gpu_exact.cubin   (device code, sm_103a; the second without
                                         fused multiply-adds)
The `_ref` products are built only where visionaray's headers are: $VSNRAY_INCLUDE, by
default the read-only checkout at /root/reference/include.  Where they are absent (the
GPU host) the prebuilt cubins that travelled with the tree are used as they are, and the
CPU baseline falls back to the restatement.

    python -m oracle.build [-v]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE_INCLUDE = os.environ.get("VSNRAY_INCLUDE", "/root/reference/include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

LIBORACLE = os.path.join(HERE, "_build", "liboracle.so")
LIBSORT = os.path.join(HERE, "_build", "libref_sort.so")
LIBREF = os.path.join(HERE, "_ref", "libvsnray_ref.so")
REFCUBIN = os.path.join(HERE, "_ref", "vsnray_ref_gpu.cubin")
REFCUBIN_EXACT = os.path.join(HERE, "_ref", "vsnray_ref_gpu_exact.cubin")

# the flags of oracle/Makefile: every float expression unfused, as written, on x86-64
# and AArch64 alike
CXX_FLAGS = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall"]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run_all(jobs):
    procs = [(name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for name, cmd in jobs]
    failed = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((name, out.decode(errors="replace")))
    if failed:
        raise RuntimeError("oracle build failed:\n" + "\n".join(f"--- {n} ---\n{o}" for n, o in failed))


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE_INCLUDE, "visionaray"))


def build(verbose=False, with_reference=True):
    gbrt_h = os.path.join(ROOT, "include", "visionaray_gb300", "gbrt.h")
    rng_h = os.path.join(ROOT, "include", "visionaray_gb300", "gbrt_rng.h")
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "pathtrace.cpp")]
    deps = srcs + [os.path.join(HERE, "oracle.h"), gbrt_h, rng_h]
    jobs = []
    if _stale(LIBORACLE, deps):
        os.makedirs(os.path.dirname(LIBORACLE), exist_ok=True)
        jobs.append(("oracle", CXX_FLAGS + ["-o", LIBORACLE] + srcs + ["-lpthread"]))
    sort_src = os.path.join(HERE, "ref_sort.cu")
    if _stale(LIBSORT, [sort_src]):
        os.makedirs(os.path.dirname(LIBSORT), exist_ok=True)
        jobs.append(("ref-sort", [NVCC, "-shared", "-Xcompiler", "-fPIC", "-O3", "-std=c++17"] + ARCH +
                     [sort_src, "-o", LIBSORT]))
    have_ref = with_reference and reference_available()
    ref_src = os.path.join(HERE, "ref_driver.cpp")
    if have_ref and _stale(LIBREF, deps + [ref_src]):
        os.makedirs(os.path.dirname(LIBREF), exist_ok=True)
        jobs.append(("reference", CXX_FLAGS + ["-w", "-DNDEBUG", "-I" + REFERENCE_INCLUDE, "-o", LIBREF, ref_src,
                                               "-lpthread"]))
    # device code only: a cubin runs on the GPU host whatever its CPU (default nvcc
    # contraction, as visionaray's own build; and a --fmad=false twin whose arithmetic is
    # the CPU reference's, for parity checks)
    ref_gpu_src = os.path.join(HERE, "ref_gpu.cu")
    for cubin, extra in ((REFCUBIN, []), (REFCUBIN_EXACT, ["--fmad=false"])):
        if have_ref and _stale(cubin, [ref_gpu_src, gbrt_h, rng_h]):
            os.makedirs(os.path.dirname(cubin), exist_ok=True)
            jobs.append(("reference-gpu", [NVCC, "-cubin"] + ARCH + extra + [
                "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-w", "-I" + REFERENCE_INCLUDE, ref_gpu_src,
                "-o", cubin]))
    if verbose:
        for n, c in jobs:
            print(n, " ".join(c))
    _run_all(jobs)
    return LIBORACLE


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIBORACLE)

"""In-tree build of the native parts (no cmake, no pip): run `python -m visionaray_gb300.build`.

Products, all git-ignored and rebuilt on every machine (x86-64 here, AArch64 on the
GPU host):
  visionaray_gb300/_lib/libgbrt.so         CUDA kernels + C ABI (sm_103a only)
  visionaray_gb300/_lib/libgbrt_scenes.so  deterministic synthetic workloads (host)
  oracle/_build/liboracle.so               CPU oracle (test infrastructure)
  oracle/_ref/libvsnray_ref.so             visionaray's own CPU code, only where its
                                           headers are present (test infrastructure)
  oracle/_ref/vsnray_ref_gpu.cubin         visionaray's own GPU traversal and path tracer
                                           (device code, sm_103a), only where its headers
                                           are present (benchmark infrastructure)
Translation units compile in parallel; an up-to-date output is not rebuilt.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "_lib")
ORACLE = os.path.join(ROOT, "oracle")
REFERENCE_INCLUDE = os.environ.get("VSNRAY_INCLUDE", "/root/reference/include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["api.cu", "batch.cu", "batch_pt.cu", "instances.cu", "lbvh.cu", "noalloc.cu", "pathtrace.cu",
              "ploc.cu", "radix_sort.cu", "traverse.cu"]
CU_HEADERS = ["device_math.cuh", "bvh_layout.cuh", "api_internal.h", "traverse_core.cuh", "lbvh_device.cuh",
              "pt_shade.cuh"]
# host code of every unit keeps expressions unfused (-ffp-contract=off) so x86-64 and
# AArch64 hosts compute the same camera bases and copies
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")] + ARCH
# the path tracer's shading repeats the reference's float expressions operation for
# operation: no fused multiply-add anywhere in its device code
PER_FILE_FLAGS = {"pathtrace.cu": ["--fmad=false"], "batch_pt.cu": ["--fmad=false"]}

LIBGBRT = os.path.join(LIB, "libgbrt.so")
LIBSCENES = os.path.join(LIB, "libgbrt_scenes.so")
LIBORACLE = os.path.join(ORACLE, "_build", "liboracle.so")
LIBREF = os.path.join(ORACLE, "_ref", "libvsnray_ref.so")
REFCUBIN = os.path.join(ORACLE, "_ref", "vsnray_ref_gpu.cubin")
REFCUBIN_EXACT = os.path.join(ORACLE, "_ref", "vsnray_ref_gpu_exact.cubin")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run_all(jobs):
    procs = [(name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
             for name, cmd in jobs]
    failed = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((name, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(f"--- {n} ---\n{o}" for n, o in failed)
        raise RuntimeError(f"native build failed:\n{msg}")


def build(verbose=False, with_reference=True):
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(os.path.join(LIB, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in CU_HEADERS] + [
        os.path.join(ROOT, "include", "visionaray_gb300", h) for h in ("gbrt.h", "gbrt_rng.h")]

    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIB, "obj", src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append((src, [NVCC] + NVCC_FLAGS + PER_FILE_FLAGS.get(src, []) + ["-c", s, "-o", o]))
    scenes_srcs = [os.path.join(CSRC, "scenes.cpp"), os.path.join(CSRC, "obj.cpp"), os.path.join(CSRC, "ply.cpp")]
    if _stale(LIBSCENES, scenes_srcs + [os.path.join(CSRC, "scenes.h")]):
        jobs.append(("scenes", ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                                "-ffp-contract=off", "-Wall"] + scenes_srcs + ["-o", LIBSCENES]))
    # the oracle flags are those of oracle/Makefile (kept for manual builds)
    oracle_flags = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall"]
    oracle_srcs = [os.path.join(ORACLE, f) for f in ("oracle.cpp", "pathtrace.cpp")]
    oracle_deps = oracle_srcs + [os.path.join(ORACLE, "oracle.h"),
                                 os.path.join(ROOT, "include", "visionaray_gb300", "gbrt_rng.h"),
                                 os.path.join(ROOT, "include", "visionaray_gb300", "gbrt.h")]
    if _stale(LIBORACLE, oracle_deps):
        os.makedirs(os.path.dirname(LIBORACLE), exist_ok=True)
        jobs.append(("oracle", oracle_flags + ["-o", LIBORACLE] + oracle_srcs + ["-lpthread"]))
    have_ref = with_reference and os.path.isdir(os.path.join(REFERENCE_INCLUDE, "visionaray"))
    ref_src = os.path.join(ORACLE, "ref_driver.cpp")
    if have_ref and _stale(LIBREF, oracle_deps + [ref_src]):
        os.makedirs(os.path.dirname(LIBREF), exist_ok=True)
        jobs.append(("reference", oracle_flags + ["-w", "-DNDEBUG", "-I" + REFERENCE_INCLUDE, "-o", LIBREF,
                                                  ref_src, "-lpthread"]))
    # visionaray's own GPU traversal and path-tracing kernel as device code only (a cubin
    # runs on the GPU host whatever its CPU); built only where the headers are
    # (default nvcc contraction, as visionaray's own build; and a --fmad=false twin whose
    # arithmetic is the CPU reference's, for parity checks)
    ref_gpu_src = os.path.join(ORACLE, "ref_gpu.cu")
    ref_gpu_deps = [ref_gpu_src, os.path.join(ROOT, "include", "visionaray_gb300", "gbrt.h"),
                    os.path.join(ROOT, "include", "visionaray_gb300", "gbrt_rng.h")]
    for cubin, extra in ((REFCUBIN, []), (REFCUBIN_EXACT, ["--fmad=false"])):
        if have_ref and _stale(cubin, ref_gpu_deps):
            os.makedirs(os.path.dirname(cubin), exist_ok=True)
            jobs.append(("reference-gpu", [NVCC, "-cubin"] + ARCH + extra + [
                "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-w", "-I" + REFERENCE_INCLUDE, ref_gpu_src,
                "-o", cubin]))
    if verbose:
        for n, c in jobs:
            print(n, " ".join(c))
    _run_all(jobs)

    if _stale(LIBGBRT, objs):
        _run_all([("link", [NVCC] + ARCH + ["-shared", "-o", LIBGBRT] + objs)])
    return LIBGBRT


def clean():
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIBGBRT)

"""In-tree build of the product's native parts (no cmake, no pip): run
`python -m visionaray_gb300.build`.

Products, both git-ignored and rebuilt on every machine (x86-64 here, AArch64 on the
GPU host):
  visionaray_gb300/_lib/libgbrt.so         CUDA kernels + C ABI (sm_103a only)
  visionaray_gb300/_lib/libgbrt_scenes.so  deterministic synthetic workloads (host)
The oracle (test infrastructure) has its own recipe, oracle/build.py.
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

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["api.cu", "batch.cu", "batch_pt.cu", "batch_pt_wide.cu", "instances.cu", "lbvh.cu", "noalloc.cu",
              "pathtrace.cu", "ploc.cu", "radix_sort.cu", "traverse.cu"]
CU_HEADERS = ["device_math.cuh", "bvh_layout.cuh", "api_internal.h", "traverse_core.cuh", "lbvh_device.cuh",
              "pt_shade.cuh", "collapse.cuh", "batch_pt.cuh"]
# host code of every unit keeps expressions unfused (-ffp-contract=off) so x86-64 and
# AArch64 hosts compute the same camera bases and copies
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")] + ARCH
# the path tracer's shading repeats the reference's float expressions operation for
# operation: no fused multiply-add anywhere in its device code
PER_FILE_FLAGS = {"pathtrace.cu": ["--fmad=false"], "batch_pt.cu": ["--fmad=false"],
                  "batch_pt_wide.cu": ["--fmad=false"]}

LIBGBRT = os.path.join(LIB, "libgbrt.so")
LIBSCENES = os.path.join(LIB, "libgbrt_scenes.so")


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


def build(verbose=False):
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

"""The header-only C++ shim (include/visionaray_gb300/visionaray_gb300.hpp) as a
visionaray caller uses it: compiled with g++, linked against libgbrt.so, run.  On a
host without a GPU the context constructor reports the missing device through the
shim's exception; on a GPU host the program traces a ray end to end, builds LBVH and
PLOC trees and path-traces a frame through make_kernel_params / cuda_sched::frame."""
import os
import shutil
import subprocess

import pytest

from visionaray_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "shim_smoke")
    lib = os.path.dirname(build.LIBGBRT)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "shim", "shim_smoke.cpp"),
           "-L", lib, "-lgbrt", f"-Wl,-rpath,{lib}", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_shim_compiles_links_and_runs(tmp_path):
    out = subprocess.run([_compile(tmp_path)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() in ("no-device", "ok")


@pytest.mark.gpu
def test_shim_traces_on_gpu(tmp_path):
    out = subprocess.run([_compile(tmp_path)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"

"""bench.py's JSON line on a reduced workload: every key of the benchmark contract is
present and consistent (value = rays per step / time, e2e on the host path giving the
device path's hits, a roofline fraction from the traversal kernel's own event time,
clock samples taken inside the timed region, counted kernel launches) and the keys of
the legs measured beside it."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_bench_line_has_the_contract_keys():
    d = run_bench("--steps", "3", "--warmup", "3", "--grid", "256", "--origins", "16384", "--pt-frames", "1",
                  "--batch-steps", "1", "--batch-scenes", "8", "--batch-max-tris", "20000", "--adjoint-steps", "3",
                  "--no-cpu-baseline")
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "roofline", "e2e", "gpu_launches", "clocks"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3 and d["higher_is_better"] is True
    rays = d["config"]["rays_per_step"]
    assert d["value"] == pytest.approx(rays / (d["ms_per_step"] * 1e-3) / 1e6, rel=1e-2)
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert r["io_floor"]["bytes_per_ray"] == 48 and 0 < r["io_floor"]["frac"] < r["frac"]
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] == 32 * rays and e["d2h_bytes_per_step"] == 16 * rays
    assert e["matches_device_path"] is True
    assert d["gpu_launches"] > 0
    assert d["clocks"]["samples"] >= 1
    assert d["pathtrace"]["msamples_s"] > 0 and d["batched_pathtrace"]["images_bit_identical"] is True
    assert d["adjoint"]["bwd_ms"] > 0
    # the closest-hit kernel's own CUDA-event time: one per timed step, below the query's
    k = d["kernels"]["closest"]
    assert k["launches_timed"] == 3 and 0 < k["kernel_ms_per_launch"] <= k["query_ms"] * 1.01
    assert d["anyhit"]["mrays_s"] > 0 and d["build_inclusive"]["ms_per_step"] > d["ms_per_step"]
    assert d["closest_plus_anyhit"]["rays_per_step"] == rays + d["config"]["anyhit_rays"]
    b = d["batched_pathtrace"]
    assert b["plain_preallocated"]["images_bit_identical"] is True and b["roofline"]["frac"] > 0
    assert d["pathtrace"]["roofline"]["b_sample"] > 0
    inst = d["pathtrace"]["instanced"]
    assert inst["instanced"]["msamples_s"] > 0 and inst["instanced"]["tree_bytes"] < inst["flattened"]["tree_bytes"]
    assert d["adjoint"]["roofline"]["forward"]["bound"] == "l2"
    assert set(d["adjoint"]["albedo_error_end"]) == set(d["adjoint"]["albedo_error_start"])


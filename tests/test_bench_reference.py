"""bench.py's reference arm (visionaray's CPU path, or the oracle port where the
reference is not built) on a reduced workload: one JSON line with its own
cpu_baseline and a host-only e2e; needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--grid", "128", "--origins", "4096"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1


def test_both_arms_print_the_same_config():
    """The reference arm and the product's arm describe the same workload with the same
    `config` (run-specific figures live under other keys)."""
    import bench
    a = bench.workload_config(bench.GRID, bench.ORIGINS, 1 << 22, 1 << 25, 8388608)
    assert a == bench.workload_config(bench.GRID, bench.ORIGINS, 1 << 22, 1 << 25, 8388608, "lbvh")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--grid", "128", "--origins", "4096"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    d = json.loads([line for line in out.stdout.splitlines() if line.startswith("{")][0])
    assert d["config"] == bench.workload_config(128, 4096, 4096, 4096 * bench.AO_PER_ORIGIN, 2 * 128 * 128)

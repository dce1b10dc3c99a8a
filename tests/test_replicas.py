"""Multi-GPU host logic on CPU: the benchmark's max-over-ranks timing and the scene
partition of the batch leg, run as two gloo ranks (world_size 2, 127.0.0.1).  The
path has no data exchange, so these collectives on timings and the local partition are
the whole N > 1 path."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from visionaray_gb300 import replicas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_partition_covers_and_balances():
    rng = np.random.default_rng(3)
    costs = rng.lognormal(10, 1.5, size=512).tolist()
    for world in (1, 2, 3, 8):
        parts = replicas.partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        lower = max(sum(costs) / world, max(costs))
        assert max(loads) <= 4.0 / 3.0 * lower + 1e-6   # Graham's bound for LPT
        assert parts == replicas.partition(costs, world)   # deterministic


def test_partition_edge_cases():
    assert replicas.partition([], 2) == [[], []]
    assert replicas.partition([5.0], 3) == [[0], [], []]
    assert replicas.partition([1.0, 1.0, 1.0, 1.0], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        replicas.partition([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, costs):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    w, r, _ = replicas.init("gloo")
    assert (w, r) == (world, rank)
    # the slowest rank's time and the job's total work
    assert replicas.reduce_over_ranks(1.5 * (rank + 1), "max") == 1.5 * world
    assert replicas.reduce_over_ranks(1.0, "sum") == float(world)
    mine = replicas.partition(costs, world)[rank]
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    flat = sorted(i for p in gathered for i in p)
    assert flat == list(range(len(costs)))
    replicas.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    costs = [float(c) for c in np.random.default_rng(5).integers(1, 1000, size=37)]
    mp.spawn(_rank_main, args=(2, _free_port(), costs), nprocs=2, join=True)


def test_split_samples():
    assert replicas.split_samples(16, 1) == [16]
    assert replicas.split_samples(16, 3) == [6, 5, 5]
    assert replicas.split_samples(7, 7) == [1] * 7
    assert sum(replicas.split_samples(256, 8)) == 256
    with pytest.raises(ValueError):
        replicas.split_samples(2, 3)


def _samples_rank(rank, world, port, samples, grads):
    """Each rank holds the per-sample images of its share of the samples and a partial
    gradient; the all-rank mean image and summed gradient equal the single-process ones."""
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch
    import torch.distributed as dist
    replicas.init("gloo")
    counts = replicas.split_samples(len(samples), world)
    first = sum(counts[:rank])
    f64 = torch.float64
    mine = torch.tensor(samples[first:first + counts[rank]], dtype=f64).mean(0)
    image = replicas.mean_image_(mine.clone(), counts[rank], len(samples))
    assert torch.allclose(image, torch.tensor(samples, dtype=f64).mean(0), rtol=1e-12, atol=1e-12)
    g = replicas.all_reduce_sum_(torch.tensor(grads[rank], dtype=f64))
    assert torch.allclose(g, torch.tensor(grads, dtype=f64).sum(0), rtol=1e-12, atol=1e-12)
    dist.destroy_process_group()


def test_sample_parallel_reductions_two_gloo_ranks():
    import torch.multiprocessing as mp
    rng = np.random.default_rng(11)
    samples = rng.normal(size=(7, 3, 4, 4)).tolist()   # 7 samples of a 3x4 RGBA image
    grads = rng.normal(size=(2, 5, 3)).tolist()
    mp.spawn(_samples_rank, args=(2, _free_port(), samples, grads), nprocs=2, join=True)


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun the reference arm runs on rank 0 only; rank 1 exits 0 at once."""
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                         env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""

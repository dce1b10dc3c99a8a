"""Multi-GPU host logic: one process per GPU.

Rays, pixels and whole scenes are independent (visionaray's schedulers hand every
pixel to its own thread, detail/cuda_sched.inl:43-49), so nothing is exchanged between
GPUs while tracing.  Three ways of using N GPUs follow:
  replicas   every rank runs the whole workload (the heightfield traversal, weak
             scaling); the job's rate is N x work / the slowest rank's time
  scenes     a batch of independent scenes is partitioned across ranks by cost
             (longest-processing-time greedy), each rank builds and renders its share
             (strong scaling of a fixed batch)
  samples    inverse rendering splits each step's samples per pixel across ranks
             (split_samples); the one real exchange is an all-reduce of the rendered
             image (weighted by samples) and of the parameter gradients per step
Timings are reduced with a max over ranks, outside the timed work.
Rendezvous: MASTER_ADDR defaults to 127.0.0.1.
"""
import os


def world_from_env():
    """(world_size, rank, local_rank) from torchrun's environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend):
    """Initialises the default process group when world_size > 1; returns (world, rank, local)."""
    import torch.distributed as dist
    world, rank, local = world_from_env()
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
    return world, rank, local


def reduce_over_ranks(value, op="max", device="cpu"):
    """max / sum of a float over all ranks (the value itself on one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def partition(costs, world):
    """Longest-processing-time greedy assignment of items with the given costs to `world`
    ranks: items by decreasing cost (index breaks ties), each to the least-loaded rank
    (lowest rank breaks ties).  Returns one ascending index list per rank; every rank
    computes the same answer locally, so no communication is needed."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


def scene_costs(offsets, params):
    """Cost model of one batched scene: triangles (the build) plus pixels x samples x
    bounces (the frame), in comparable units."""
    costs = []
    for s in range(len(offsets) - 1):
        tris = int(offsets[s + 1]) - int(offsets[s])
        p = params[s]
        work = int(p["width"]) * int(p["height"]) * int(p["spp"]) * max(int(p["num_bounces"]), 1)
        costs.append(tris + 4 * work)
    return costs


def split_samples(spp, world):
    """Samples per pixel of each rank when `spp` are split across `world` ranks: the
    first spp % world ranks take one more.  Every rank computes the same list."""
    if world < 1 or spp < world:
        raise ValueError("need 1 <= world <= spp")
    return [spp // world + (1 if r < spp % world else 0) for r in range(world)]


def all_reduce_sum_(tensor):
    """In-place sum of a tensor over all ranks (nothing on one rank)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(tensor, op=dist.ReduceOp.SUM)
    return tensor


def mean_image_(image, my_spp, total_spp):
    """The all-rank image of a frame whose samples are split across ranks: each rank's
    per-pixel mean over its `my_spp` samples, weighted by my_spp / total_spp and summed
    in place (alpha included)."""
    image.mul_(float(my_spp) / float(total_spp))
    return all_reduce_sum_(image)

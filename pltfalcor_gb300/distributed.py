"""Multi-process use of the library (one process per GPU, no device-side collective).

The path shards without exchange: BSDF query batches split into contiguous ranges, render views
(whole scenes or image tiles) split across ranks, and the only communication is on the host: one
gather of the ranks' framebuffers and, for data-parallel training of the learned proposal, one
average of the ranks' gradients per step.  Everything here works with any torch.distributed
backend (gloo on CPU in the tests, NCCL between GPUs).
"""
import numpy as np


def shard_range(n, rank, world):
    """Contiguous [begin, end) of n items for `rank` of `world`, sizes differing by at most one."""
    base, extra = divmod(int(n), int(world))
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def partition_views(pixel_counts, world):
    """Assigns render views to ranks, largest first to the least-loaded rank (ties to the lowest
    rank), so every rank gets a similar number of paths.  Returns one list of view indices per rank,
    each in increasing view order."""
    load = [0] * world
    parts = [[] for _ in range(world)]
    for v in sorted(range(len(pixel_counts)), key=lambda i: (-int(pixel_counts[i]), i)):
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(v)
        load[r] += int(pixel_counts[v])
    return [sorted(p) for p in parts]


def gather_images(local, dist, dst=0):
    """Gathers {view index: image array} from every rank onto rank `dst` (a dict of all views there,
    None elsewhere)."""
    world = dist.get_world_size()
    out = [None] * world if dist.get_rank() == dst else None
    dist.gather_object({int(k): np.asarray(v) for k, v in local.items()}, out, dst=dst)
    if out is None:
        return None
    merged = {}
    for part in out:
        merged.update(part)
    return merged


def allreduce_mean_(tensor, dist):
    """In-place mean of a tensor over all ranks (the data-parallel gradient average)."""
    dist.all_reduce(tensor, op=dist.ReduceOp.SUM)
    tensor /= dist.get_world_size()
    return tensor


def train_proposal_data_parallel(ctx, steps, batch, lr, seed, dist):
    """Data-parallel training of the learned proposal: every rank draws its own batch from the exact
    samplers (seed, step and rank decide the stream), computes the gradient with the library's
    kernels, the gradients are averaged over ranks, and every rank applies the same Adam step, so
    the replicas stay identical.  Returns the rank-mean loss per step."""
    rank, world = dist.get_rank(), dist.get_world_size()
    losses = np.zeros(steps, np.float32)
    for s in range(steps):
        x, t, w = ctx.proposal_generate(batch, seed + (s * world + rank) * 7919)
        loss, g = ctx.proposal_gradient(x, t, w)
        allreduce_mean_(g, dist)
        import torch
        lt = torch.tensor([loss], dtype=torch.float32, device=g.device)
        allreduce_mean_(lt, dist)
        losses[s] = float(lt.item())
        ctx.proposal_adam_step(g, lr)
    return losses

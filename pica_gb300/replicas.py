"""Independent replicas on several GPUs (the single-plasma step does not shard
without a halo exchange, so N GPUs run N independent plasmas with no collective
on the data path).  The only cross-rank step is the timing: the job's time is the
slowest rank's, and the job's throughput is the particles of every rank over it.

The batching form's independent plasmas shard with no communication at all: they
are binned over the ranks by particle count (bin_members), and each rank advances
its own bin.
"""


def replica_seed(seed, rank):
    """Seed of rank `rank`'s plasma (rank 0 keeps the workload's own seed)."""
    return int(seed) + int(rank)


def job_throughput(particles_per_rank, steps, elapsed_s, dist=None, device="cpu"):
    """(particle-steps/s of the whole job, the job's time): every rank passes its own
    elapsed time; the maximum over ranks is the job's time (all_reduce MAX over
    `dist`, the torch.distributed module, or None for one rank)."""
    world = 1
    elapsed = float(elapsed_s)
    if dist is not None and dist.is_initialized():
        import torch

        world = dist.get_world_size()
        t = torch.tensor([elapsed], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    return world * particles_per_rank * steps / elapsed, elapsed


def bin_members(counts, world):
    """Independent plasmas with particle counts `counts` binned over `world` ranks:
    largest first, each to the rank with the fewest particles so far (ties: the lower
    rank).  Returns one list of member indices per rank, each in member order; the
    result depends only on the counts, so every rank computes the same bins alone."""
    if world < 1:
        raise ValueError("world >= 1")
    load = [0] * world
    bins = [[] for _ in range(world)]
    for i in sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i)):
        r = min(range(world), key=lambda q: (load[q], q))
        bins[r].append(i)
        load[r] += int(counts[i])
    return [sorted(b) for b in bins]


def job_throughput_binned(particles_this_rank, steps, elapsed_s, dist=None, device="cpu"):
    """(particle-steps/s of the whole job, the job's time) when ranks hold different
    particle counts: the particles of every rank (all_reduce SUM) times steps over
    the slowest rank's time (all_reduce MAX); one rank without `dist`."""
    parts, elapsed = float(particles_this_rank), float(elapsed_s)
    if dist is not None and dist.is_initialized():
        import torch

        p = torch.tensor([parts], dtype=torch.float64, device=device)
        t = torch.tensor([elapsed], dtype=torch.float64, device=device)
        dist.all_reduce(p, op=dist.ReduceOp.SUM)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        parts, elapsed = float(p.item()), float(t.item())
    return parts * steps / elapsed, elapsed

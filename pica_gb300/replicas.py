"""Independent replicas on several GPUs (the single-plasma step does not shard
without a halo exchange, so N GPUs run N independent plasmas with no collective
on the data path).  The only cross-rank step is the timing: the job's time is the
slowest rank's, and the job's throughput is the particles of every rank over it.
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

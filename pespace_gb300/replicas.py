"""Multi-GPU replicas for the batched likelihood (one process per GPU).

The lnL+gradient of a batch of posterior samples has no cross-sample data
dependence, so N GPUs run N independent replicas: rank r evaluates its own
batch (samples seeded with 2026 + r), there is no data-path collective, and
the job rate is the total number of samples over the slowest rank's time
(weak scaling).  The only collective is the MAX of the per-rank step time
(and a barrier around the timed region), on whatever process group the
caller initialised (NCCL on GPUs, gloo on CPU for the tests).
"""

import numpy as np

from .workloads import prior_samples

SEED_BASE = 2026


def rank_seed(rank):
    return SEED_BASE + int(rank)


def rank_theta(rank, batch, tc0):
    """The (batch, 11) prior samples of one rank."""
    return prior_samples(np.random.default_rng(rank_seed(rank)), batch, tc0)


def reduce_max(value, device="cpu"):
    """MAX over the ranks of a per-rank scalar (identity without a process group)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, batch, step_ms):
    """Samples per second of the whole job: every rank's batch over the slowest step."""
    return world * batch / (step_ms / 1e3)

"""Multi-rank host logic of the replicated benchmark (gloo, world size 2, CPU).

Each rank draws its own prior samples, evaluates them (here with the oracle on
a small grid, standing in for the GPU engine), and the job reports the MAX of
the per-rank step times; there is no data-path collective.  The union of the
rank shards must equal a single process evaluating the same seeded batches.
"""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from tests.helpers import config0_theta, make_dataset
from tests.test_gpu_plan import lisa

DUR, DT, FMIN, FMAX = 2.0 ** 15, 8.0, 1e-4, 0.03
B = 3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from oracle import fdpath as oracle
    from pespace_gb300 import replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    th0 = config0_theta(DUR - 2000.0)
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, [lisa(oracle)], th0, seed=5)
    theta = replicas.rank_theta(rank, B, th0[10])
    lnl = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(theta)
    step_ms = 10.0 + rank  # the slower rank sets the job time
    dist.barrier()
    t = replicas.reduce_max(step_ms)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), theta=theta, lnl=lnl, t=t,
             rate=replicas.job_rate(world, B, t))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_two_ranks(tmp_path, oracle):  # the fixture builds the oracle before the ranks start
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r = [np.load(tmp_path / f"rank{k}.npz") for k in range(world)]
    # distinct shards, each rank its own seed
    assert not np.allclose(r[0]["theta"], r[1]["theta"])
    # the job time is the slowest rank's, seen identically by every rank
    assert float(r[0]["t"]) == float(r[1]["t"]) == 11.0
    assert float(r[0]["rate"]) == pytest.approx(world * B / 11e-3)
    # the union of the shards equals one process evaluating the same seeded batches
    from oracle import fdpath as oracle
    from pespace_gb300 import replicas

    th0 = config0_theta(DUR - 2000.0)
    g, dets = make_dataset(oracle, DUR, DT, FMIN, FMAX, [lisa(oracle)], th0, seed=5)
    thetas = np.concatenate([replicas.rank_theta(k, B, th0[10]) for k in range(world)])
    want = oracle.Plan(g, [(o, gen, d, p) for _, o, gen, d, p in dets], 1e-4, cut_factor=1.2).lnl(thetas)
    got = np.concatenate([r[k]["lnl"] for k in range(world)])
    np.testing.assert_array_equal(got, want)

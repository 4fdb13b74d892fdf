"""Multi-GPU form of the sieve: contiguous shards of the Gray-code term range, summed on the host.

CPU: the shard partition, the term count of an instance (library call, no GPU), and two gloo
ranks that each evaluate their shard (the oracle stands in for the GPU) and combine with one
all-reduce.  GPU: shards of plain, loop and batch instances sum to the unsharded outputs."""
import os
import tempfile

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat, sharding, workloads as wl


def test_shard_range_partition():
    for steps in (1, 2, 7, 1000, 524288):
        for world in (1, 2, 3, 5, 8):
            ranges = [sharding.shard_range(steps, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == steps
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c and a <= b
    with pytest.raises(ValueError):
        sharding.shard_range(10, 2, 2)


def test_instance_terms():
    A = wl.complex_symmetric(12, seed=3)
    inst = tw.prepare_hafnian(A)
    assert inst.terms() == 2 ** 5  # glynn: first edge halved, 2^(n/2 - 1)
    inst = tw.prepare_hafnian(wl.complex_symmetric(5, seed=3), reps=[2, 1, 3, 1, 1])
    x, reps, _ = oracle.matched_reps([2, 1, 3, 1, 1])
    want = (reps[0] + 2) // 2 * int(np.prod([r + 1 for r in reps[1:]]))
    assert inst.terms() == want
    with pytest.raises(ValueError):
        inst.shard(3, 3)


def _gloo_rank(rank, world, port, path):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        A = wl.complex_symmetric(16, seed=5)
        inst = tw.prepare_hafnian(A)
        b, e = sharding.shard_range(inst.terms(), rank, world)
        part = complex(oracle.haf_term_range(inst.A, inst.reps, b, e, nthreads=1))
        total = sharding.combine([part])
        np.save(os.path.join(path, "rank%d.npy" % rank), total)
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_combine():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    with tempfile.TemporaryDirectory() as path:
        mp.spawn(_gloo_rank, args=(2, port, path), nprocs=2, join=True)
        got = [np.load(os.path.join(path, "rank%d.npy" % r)) for r in range(2)]
    A = wl.complex_symmetric(16, seed=5)
    inst = tw.prepare_hafnian(A)
    want = complex(oracle.haf_term_range(inst.A, inst.reps, 0, inst.terms(), nthreads=1))
    for g in got:
        assert abs(complex(g[0]) - want) <= 1e-12 * abs(want)


@pytest.mark.gpu
def test_gpu_shards_sum_to_full():
    A = wl.complex_symmetric(20, seed=9)
    Al, gamma, rpt = wl.gaussian_state_loop(modes=6, seed=2, photons=12, max_rep=3)
    B, D, fixed, cutoff = wl.batch_loop_calls(count=1, seed=13, modes=7, cutoff=4)[0]
    insts = [tw.prepare_hafnian(A), tw.prepare_loop_hafnian(Al, gamma, list(rpt)),
             tw.prepare_loop_hafnian_batch(B, D, list(fixed), cutoff)]
    full = nat.run(insts, "fp64")
    for world in (2, 3, 7):
        total = sum(sharding.run_shard(insts, r, world) for r in range(world))
        assert np.max(np.abs(total - full) / np.abs(full)) < 1e-11, world

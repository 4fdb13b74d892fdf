"""One sieve across several GPUs: contiguous shards of the Gray-code term range.

The sieve is a sum over independent terms, so N processes (one per GPU) each evaluate the terms
[steps * r / N, steps * (r + 1) / N) of the same instance (``Instance.shard``, carried to the
kernels as ``term_begin``/``term_end``) and the shards' results are summed on the host: one
all-reduce of a few float64 values per call after the device-to-host copy, nothing on the data
path.  ``combine`` does that sum with ``torch.distributed`` (gloo on host tensors, NCCL on device
tensors).  Thewalrus itself is single-process; per instance the reduction is one complex scalar
(or one batch vector).
"""
import numpy as np

from . import _native as nat
from ._hafnian import DEFAULT_PRECISION, prepare_hafnian, prepare_loop_hafnian

__all__ = ["shard_range", "run_shard", "combine", "hafnian_sharded"]


def shard_range(steps, rank, world):
    """Terms [begin, end) of shard ``rank`` of ``world`` (a partition of [0, steps))."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    return steps * rank // world, steps * (rank + 1) // world


def run_shard(instances, rank, world, precision=None):
    """This shard's share of every instance's outputs (concatenated like ``nat.run``).  FP64 or
    double-float: a shard's share of an exact (modular) sieve is a residue, not an integer."""
    if precision not in (None, "fp64", "df"):
        raise ValueError("sharded sieves run in fp64 or df precision")
    parts, where, out = [], [], []
    for inst in instances:
        b, e = shard_range(inst.terms(), rank, world)
        if e > b:
            where.append(len(out))
            parts.append(inst.shard(b, e))
        out.append(np.zeros(inst.outputs(), dtype=np.complex128))
    if parts:
        vals = nat.run(parts, precision or DEFAULT_PRECISION)
        k = 0
        for i, inst in zip(where, parts):
            n = inst.outputs()
            out[i] = vals[k:k + n]
            k += n
    return np.concatenate(out) if out else np.zeros(0, dtype=np.complex128)


def combine(values, group=None, device=None):
    """Sum complex ``values`` over the ranks of ``group`` (torch.distributed all-reduce)."""
    import torch
    import torch.distributed as dist

    v = np.asarray(values, dtype=np.complex128).reshape(-1)
    t = torch.tensor(np.stack([v.real, v.imag], axis=1), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    t = t.cpu().numpy()
    return t[:, 0] + 1j * t[:, 1]


def hafnian_sharded(A, loop=False, precision=None, group=None, device=None):
    """``hafnian(A, loop=loop)`` with the sieve split over the ranks of ``group``; every rank
    returns the full value.  Inputs the reference answers in closed form are answered by every
    rank without a sieve."""
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    prep = prepare_loop_hafnian(A) if loop else prepare_hafnian(A)
    if not isinstance(prep, nat.Instance):
        return np.complex128(prep)
    part = run_shard([prep], rank, world, precision)
    return np.complex128(combine(part, group, device)[0])

"""Slice-level sharding of one count over several GPUs (one process per GPU).

The slices of a plan are independent sub-networks of identical shape
(``TensorNetwork.slice_groups``, ``tensor_network/tensor_network.pyx:363-401``),
so a count shards by slice range with no exchange of tensors: each rank
contracts a contiguous block of slices into its own compensated FP64
accumulator, and the ranks' (sum, compensation) pairs -- 16 bytes each -- are
combined once at the end.  The reference's analogue is the JAX backend's
``split_every(assignments, num_devices)`` followed by a host sum
(``tensor_apis/jax_apis.py:281-286``).

The combine is deterministic: partials are gathered in rank order and added
with a two-sum on the host, so the result does not depend on arrival order.

The int forms shard the same way.  A rank's partial is its words (the int
form's sums modulo 2^64, or the residue form's residues modulo p).  The
combine adds them modulo 2^64 or p, which is exact in any order
(:func:`contract_sharded_words`).
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import numpy as np

Partial = Tuple[np.ndarray, np.ndarray]  # (sum, compensation), each 2^root_rank entries


def slice_range(num_slices: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous block of slices for ``rank``; block sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    base, extra = divmod(int(num_slices), world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def two_sum(a: float, b: float) -> Tuple[float, float]:
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def combine(partials: Sequence[Partial]) -> np.ndarray:
    """Compensated sum of per-rank partials, in the order given."""
    if not partials:
        raise ValueError("no partials")
    shape = np.shape(partials[0][0])
    n = int(np.prod(shape)) if shape else 1
    out = np.zeros(n, dtype=np.float64)
    for e in range(n):
        s, c = 0.0, 0.0
        for psum, pcomp in partials:
            s, err = two_sum(s, float(np.ravel(psum)[e]))
            c += err + float(np.ravel(pcomp)[e])
        out[e] = s + c
    return out.reshape(shape)


def gather_partials(partial: Partial, group=None) -> List[Partial]:
    """All-gather every rank's (sum, compensation) through torch.distributed
    (gloo or NCCL); returns them in rank order."""
    import torch
    import torch.distributed as dist

    s, c = (np.asarray(x, dtype=np.float64).ravel() for x in partial)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    mine = torch.from_numpy(np.concatenate([s, c])).to(dev)
    world = dist.get_world_size(group)
    bufs = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(bufs, mine, group=group)
    n = s.size
    shape = np.shape(partial[0])
    return [(b[:n].cpu().numpy().reshape(shape), b[n:].cpu().numpy().reshape(shape)) for b in bufs]


def contract_sharded(num_slices: int, run_range: Callable[[int, int], Partial], rank: int, world: int,
                     group=None) -> np.ndarray:
    """One count sharded by slice range: ``run_range(begin, end)`` contracts
    this rank's slices and returns its partial; the combined result is
    returned on every rank."""
    begin, end = slice_range(num_slices, rank, world)
    mine = run_range(begin, end)
    if world == 1:
        return combine([mine])
    return combine(gather_partials(mine, group))


def combine_words(parts: Sequence[np.ndarray], modulus: int = 0) -> np.ndarray:
    """Sum of per-rank words modulo 2^64 (``modulus`` 0, the int form) or
    modulo ``modulus`` (the residue form), as uint64."""
    if not parts:
        raise ValueError("no partials")
    shape = np.shape(parts[0])
    m = int(modulus) if modulus else 1 << 64
    total = [0] * (int(np.prod(shape)) if shape else 1)
    for w in parts:
        for e, x in enumerate(np.asarray(w).astype(np.uint64, copy=False).ravel()):
            total[e] = (total[e] + int(x)) % m
    return np.array(total, dtype=np.uint64).reshape(shape)


def gather_words(words: np.ndarray, group=None) -> List[np.ndarray]:
    """All-gather every rank's 64-bit words (as int64 through torch.distributed,
    gloo or NCCL); returns them as uint64 in rank order."""
    import torch
    import torch.distributed as dist

    w = np.ascontiguousarray(np.asarray(words).astype(np.uint64, copy=False).view(np.int64).ravel())
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    mine = torch.from_numpy(w).to(dev)
    bufs = [torch.empty_like(mine) for _ in range(dist.get_world_size(group))]
    dist.all_gather(bufs, mine, group=group)
    shape = np.shape(words)
    return [b.cpu().numpy().view(np.uint64).reshape(shape) for b in bufs]


def contract_sharded_words(num_slices: int, run_range: Callable[[int, int], np.ndarray], rank: int, world: int,
                           modulus: int = 0, group=None) -> np.ndarray:
    """An int-form count sharded by slice range: ``run_range(begin, end)``
    returns this rank's words; their sum modulo 2^64 (or ``modulus``) is
    returned on every rank."""
    begin, end = slice_range(num_slices, rank, world)
    mine = run_range(begin, end)
    if world == 1:
        return combine_words([mine], modulus)
    return combine_words(gather_words(mine, group), modulus)


def device_words_runner(device_program, mode, workspace=None, stream=None):
    """``run_range`` for :func:`contract_sharded_words` on this rank's GPU, in
    the int form or the residue form (whose modulus the program holds)."""

    def run(begin, end):
        device_program.reset(stream)
        if end > begin:
            device_program.run(mode, begin, end, workspace=workspace, stream=stream)
        return device_program.result_words(stream, np.uint64)

    return run


def device_range_runner(device_program, mode, workspace=None, stream=None):
    """``run_range`` for :func:`contract_sharded` on this rank's GPU."""

    def run(begin, end):
        device_program.reset(stream)
        if end > begin:
            device_program.run(mode, begin, end, workspace=workspace, stream=stream)
        return device_program.partial(stream)

    return run


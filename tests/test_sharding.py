"""Slice sharding of one count across ranks (host logic; gloo on CPU).

Two and three CPU ranks each contract their slice block with the numpy oracle
standing in for the GPU, gather the partials through torch.distributed (gloo)
and combine them; the combined count must equal the reference's own count of
the whole plan, and every rank must see the same value."""
import os

import numpy as np
import pytest

from conftest import load_golden
from tensororder_gb300 import sharding
from tensororder_gb300.program import Program


@pytest.mark.parametrize("n,world", [(1024, 2), (1024, 3), (5, 4), (3, 8), (0, 2)])
def test_slice_ranges_partition_the_slices(n, world):
    ranges = [sharding.slice_range(n, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    for (a, b), (c, d) in zip(ranges, ranges[1:]):
        assert b == c
    sizes = [b - a for a, b in ranges]
    assert max(sizes) - min(sizes) <= 1


def test_slice_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        sharding.slice_range(8, 2, 2)


def test_combine_is_compensated():
    parts = [(np.array([1e16]), np.array([0.0])), (np.array([1.0]), np.array([0.0])),
             (np.array([-1e16]), np.array([0.0])), (np.array([1.0]), np.array([0.5]))]
    assert sharding.combine(parts)[0] == 2.5


def _oracle_range(prog, begin, end):
    from oracle import contract as oracle

    acc = None
    for s in range(begin, end):
        arr, _ = oracle.contract(prog, s)
        acc = arr.astype(np.float64) if acc is None else acc + arr
    if acc is None:
        acc = np.zeros(())
    acc = np.asarray(acc, dtype=np.float64).reshape(-1)
    return acc, np.zeros_like(acc)


def _worker(rank, world, port, name, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prog = Program.from_dict(load_golden(name)["program"])
        got = sharding.contract_sharded(prog.num_slices, lambda b, e: _oracle_range(prog, b, e), rank, world)
        q.put((rank, float(np.ravel(got)[0])))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("wvc30_s3", 2), ("vc60_s4", 3)])
def test_sharded_count_over_gloo_ranks(name, world):
    import multiprocessing as mp
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, name, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    vals = dict(q.get(timeout=10) for _ in range(world))
    want = load_golden(name)["reference"]["float64"]
    assert len(set(vals.values())) == 1
    assert abs(vals[0] - want) <= 1e-13 * abs(want)


def test_combine_words_is_modular():
    top = np.array([np.iinfo(np.uint64).max], dtype=np.uint64)
    assert sharding.combine_words([top, np.array([2], dtype=np.uint64)])[0] == 1
    p = 268435399
    assert sharding.combine_words([np.array([p - 1], dtype=np.uint64), np.array([5], dtype=np.uint64)], p)[0] == 4


def _words_worker(rank, world, port, name, modulus, q):
    import torch.distributed as dist

    from intcases import MOD, exact_count, integer_weights

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prog = integer_weights(Program.from_dict(load_golden(name)["program"]))
        m = modulus or MOD

        def run_range(b, e):  # the oracle stands in for this rank's GPU
            return np.array([exact_count(prog, b, e) % m], dtype=np.uint64)

        got = sharding.contract_sharded_words(prog.num_slices, run_range, rank, world, modulus)
        q.put((rank, int(got[0])))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,world,modulus", [("wvc30_s3", 2, 0), ("vc60_s4", 3, 0), ("vc60_s4", 3, 268435399)])
def test_sharded_int_count_over_gloo_ranks(name, world, modulus):
    """Int-form words (modulo 2^64) and residues (modulo a prime) shard
    exactly: the ranks' combined words equal the whole count's."""
    import multiprocessing as mp
    import socket

    from intcases import MOD, exact_count, integer_weights

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_words_worker, args=(r, world, port, name, modulus, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    vals = dict(q.get(timeout=10) for _ in range(world))
    want = exact_count(integer_weights(Program.from_dict(load_golden(name)["program"]))) % (modulus or MOD)
    assert set(vals.values()) == {want}

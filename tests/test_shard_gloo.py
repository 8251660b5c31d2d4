"""Tuple-list sharding over processes (atrip_gb300.shard and the sharded
Atrip.run path), checked on CPU with world_size-2 gloo process groups.

Each rank stands in for one GPU: a fake context computes its share of the
per-tuple energies with the CPU oracle (the same numbers the GPU context
produces, to 1e-10), and the ranks merge their compensated sums through
torch.distributed exactly as the GPU path does.  The merged E(T) and E(cT)
must equal the one-process oracle to 1e-13, for the whole list, for an
ijkabc run with max_iterations, and for a resume from a checkpoint.
"""
import math
import os
import socket

import numpy as np
import pytest

import oracle
from atrip_gb300 import shard, synth


def test_tuple_range_partitions_every_list():
    for first, end in ((0, 0), (0, 1), (0, 2), (3, 17), (0, 11440), (5, 6)):
        for world in (1, 2, 3, 4, 7, 8):
            ranges = [shard.tuple_range(first, end, r, world) for r in range(world)]
            pos = first
            for t0, t1 in ranges:
                assert t0 == pos and t1 >= t0
                pos = t1
            assert pos == max(first, end)
            sizes = [t1 - t0 for t0, t1 in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.tuple_range(0, 10, 2, 2)


def test_merge_pairs_is_compensated():
    vals = [1e16, 1.0, -1e16, 1.0] * 50
    pairs = [(v, 0.0) for v in vals]
    s, c = shard.merge_pairs(pairs)
    assert s + c == math.fsum(vals)


def _pairs(x):
    s, c = 0.0, 0.0
    for v in x:
        s, c = shard.neumaier(s, c, float(v))
    return s, c


class OracleContext:
    """Stands in for capi.Context on a CPU: run / last_sums / tuple_energies
    over the oracle's per-tuple energies."""

    def __init__(self, p):
        self.p = p
        self.n = oracle.n_tuples(p.Nv)

    def run(self, first_iteration=0, max_iterations=0, ijkabc=False, use_j=True, **_):
        end = self.n if max_iterations == 0 else min(self.n, max_iterations + 1)
        t0 = min(first_iteration, end)
        self.lo = t0
        self.e, self.ect = oracle.tuple_energies(self.p, t0, end, ijkabc, use_j)

        class R:
            device_ms = 0.0
        return R()

    def last_sums(self):
        return (*_pairs(self.e), *_pairs(self.ect))

    def tuple_energies(self, t0, n):
        return self.e[t0 - self.lo:t0 - self.lo + n], self.ect[t0 - self.lo:t0 - self.lo + n]


CASES = {
    "full": dict(first=0, maxit=0, ijkabc=False, start=0.0),
    "ijkabc_maxit": dict(first=0, maxit=301, ijkabc=True, start=0.0),
    "resume": dict(first=57, maxit=0, ijkabc=False, start=-12.5),
    "two_tuples": dict(first=0, maxit=1, ijkabc=False, start=0.0),
}


def _rank_main(rank, world, port, case, out):
    import torch.distributed as dist
    from atrip_gb300.atrip import Atrip
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        d = synth.make_inputs(6, 14, 8, with_j=True)
        ctx = OracleContext(oracle.Problem(d))
        Atrip.init()
        assert (Atrip.rank, Atrip.np) == (rank, world)
        c = CASES[case]
        n = ctx.n
        end = n if c["maxit"] == 0 else min(n, c["maxit"] + 1)
        e, ect = Atrip._run_shard(ctx, c["first"], end, c["start"], dict(ijkabc=c["ijkabc"]),
                                  c["ijkabc"])
        out.put((rank, e, ect))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("case", sorted(CASES))
def test_two_gloo_ranks_match_one_process(case):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    c = CASES[case]
    d = synth.make_inputs(6, 14, 8, with_j=True)
    ref_e, ref_ect = oracle.run(oracle.Problem(d), ijkabc=c["ijkabc"],
                                max_iterations=c["maxit"], first_iteration=c["first"],
                                start_energy=c["start"])
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, case, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, e, ect in res:
        # every rank holds the merged totals
        assert abs(e - ref_e) <= 1e-13 * abs(ref_e)
        assert abs(ect - ref_ect) <= 1e-13 * abs(ref_e)

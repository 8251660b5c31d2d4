"""Tuple-list sharding over processes (one process per GPU).

atrip spreads its tuple list over MPI ranks and ends with one
MPI_Reduce of the local energies (src/atrip/Tuples.cxx:89-120,
src/atrip/Atrip.cxx:1094-1107).  Here every process owns one GPU and one
contiguous share of the lexicographic list; tuples are independent, so the
data path needs no exchange at all.  The only collective is the merge of
the per-process compensated sums at the end: each process contributes its
(sum, compensation) pairs for E(T) and E(cT) (``Context.last_sums``), every
process gathers all of them and merges them in rank order with the same
Neumaier step the device reduction uses, so the total is independent of
the number of processes up to the rounding of those few merges, and every
rank ends with the same value.

Every tuple costs the same 12 No^3 (No + Nv) FLOPs (src/atrip/Atrip.cxx:
578-580), so equal tuple counts are equal work.
"""
from __future__ import annotations

from typing import Iterable, Sequence, Tuple


def tuple_range(first: int, end: int, rank: int, world: int) -> Tuple[int, int]:
    """[t0, t1) of list positions first .. end-1 owned by `rank` of `world`:
    contiguous, sizes differ by at most one, ranks in list order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    n = max(0, end - first)
    base, extra = divmod(n, world)
    t0 = first + rank * base + min(rank, extra)
    return t0, t0 + base + (1 if rank < extra else 0)


def neumaier(s: float, c: float, x: float) -> Tuple[float, float]:
    """One compensated-summation step: s + c + x as (s', c')."""
    t = s + x
    if abs(s) >= abs(x):
        c += (s - t) + x
    else:
        c += (x - t) + s
    return t, c


def merge_pairs(pairs: Iterable[Sequence[float]]) -> Tuple[float, float]:
    """Merge per-process (sum, compensation) pairs into one total (the
    compensations are merged as values of their own, in order)."""
    s, c = 0.0, 0.0
    for ps, pc in pairs:
        s, c = neumaier(s, c, ps)
        s, c = neumaier(s, c, pc)
    return s, c


def allgather_sums(local: Sequence[float], group=None):
    """All ranks' 4-tuples (s_e, c_e, s_ct, c_ct), in rank order, through
    torch.distributed (gloo or NCCL).  With no initialised process group the
    local tuple is the only one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [tuple(local)]
    world = dist.get_world_size(group)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else \
        torch.device("cpu")
    mine = torch.tensor(list(local), dtype=torch.float64, device=dev)
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine, group=group)
    return [tuple(float(v) for v in p.cpu().tolist()) for p in parts]


def reduce_energies(local: Sequence[float], ijkabc: bool = False, start_energy: float = 0.0,
                    group=None) -> Tuple[float, float]:
    """(energy, ct_energy) of the whole list from every rank's local sums,
    with atrip's final sign (negated unless ijkabc, src/atrip/Atrip.cxx:
    1108-1111) and a checkpointed energy added back as atrip does
    (src/atrip/Atrip.cxx:612-616)."""
    allp = allgather_sums(local, group)
    se, ce = merge_pairs((p[0], p[1]) for p in allp)
    sc, cc = merge_pairs((p[2], p[3]) for p in allp)
    sign = 1.0 if ijkabc else -1.0
    # -start_energy enters the local sum of rank 0 only in atrip; adding it
    # once after the merge is the same value
    e_s, e_c = neumaier(se, ce, -start_energy)
    return sign * (e_s + e_c), sign * (sc + cc)

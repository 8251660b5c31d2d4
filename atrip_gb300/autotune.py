"""Autotuner of the triples engine: launch parameters and slice count.

For one system (a ``capi.Context`` with its tensors uploaded) it times the
candidate launch parameters of the chosen form on sample windows of the
tuple list (device time from CUDA events, ``atrip_result.device_ms``) and
keeps the fastest:

* FP64 form: the register tile (32 or 64 rows of (p,q) pairs per CTA pass),
  the kernel's register budget (compiler's choice, or capped at 128 for two
  resident CTAs per SM) and the tuples a CTA claims per queue access;
* split forms: the slice format first -- the cheapest of 2 FP16 slices
  (where the system fits its kernel; form ``split``) and 2..4 BF16 slices
  whose estimated |dE(T)| against the FP64 form, carried to the
  power-of-two scaled twin of the system with |E(T)| ~ 0.1 Eh, stays within
  ``tol_eh`` -- then
  the depth of the operand ring, where W lives (shared memory or L2) and the
  processing order (list order, or grouped in (a, b, c) blocks of side L so
  the tuples in flight share their operand slabs in L2).

The error estimate runs both forms on the same windows, evenly spread over
the list, and extrapolates the per-tuple differences to the whole list
(sum over the sample times n / sample size, with the standard error of the
window sums).  Scaling every input by 2^k leaves the split form's digits
unchanged and multiplies every energy and its error by 2^(4k), so the
twin's error is the estimate times the same factor as its energy.

Choices are cached in a JSON file keyed by device name, No, Nv and form.
The reference has no tuner: its only knob for this loop is the tuple
distribution (src/atrip/Tuples.hpp:49-52).
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import capi

CACHE = os.environ.get("ATRIP_GB300_TUNING_CACHE",
                       os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib",
                                    "tuning.json"))


def windows(n: int, m: int, w: int):
    """m windows of w consecutive tuples, evenly spread over [0, n)."""
    w = max(1, min(w, n))
    m = max(1, min(m, n // w))
    step = n / m
    out = []
    for k in range(m):
        lo = min(n - w, int(k * step + (step - w) / 2)) if step > w else int(k * step)
        lo = max(0, lo)
        out.append((lo, lo + w))
    return out


def window_size(No: int, Nv: int, m: int, flops: float) -> int:
    """Tuples per window so that m windows carry about `flops` FP64-equivalent work."""
    fpt = 12.0 * No ** 3 * (No + Nv)
    return max(1, int(flops / (m * fpt)))


def run_windows(ctx: capi.Context, wins, form: str, slices: int = 0, use_j: bool = False):
    """Device milliseconds over the windows and the per-tuple energies."""
    ms, es = 0.0, []
    for lo, hi in wins:
        r = ctx.run(form=form, slices=slices, use_j=use_j, first_iteration=lo,
                    max_iterations=hi - 1)
        ms += r.device_ms
        e, _ = ctx.tuple_energies(lo, hi - lo)
        es.append(e.copy())
    return ms, es


def error_estimate(n: int, e_ref, e_test, ijkabc: bool = False) -> dict:
    """Extrapolated E(T) and dE(T) = E_test - E_ref over the whole list from
    per-window per-tuple energies (atrip's accumulated sign: E = -sum e)."""
    sign = 1.0 if ijkabc else -1.0
    n_s = sum(len(x) for x in e_ref)
    scale = n / max(n_s, 1)
    d = np.array([float(np.sum(t - r)) for r, t in zip(e_ref, e_test)])
    s = np.array([float(np.sum(r)) for r in e_ref])
    m = len(d)
    dE = sign * scale * float(d.sum())
    E = sign * scale * float(s.sum())
    se = scale * math.sqrt(m) * float(np.std(d, ddof=1)) if m > 1 else abs(dE)
    # power-of-two twin with |E(T)| ~ 0.1 Eh: every energy and error times 2^(4k)
    k = round(math.log2(0.1 / abs(E)) / 4) if E != 0 else 0
    f = 2.0 ** (4 * k)
    maxrel = max(float(np.max(np.abs(t - r))) for r, t in zip(e_ref, e_test)) / \
        max(float(np.max(np.abs(r))) for r in e_ref)
    return {"E_est": E, "dE_est": dE, "dE_stderr": se, "rel": abs(dE) / abs(E) if E else None,
            "twin_scale_log2": k, "twin_E": E * f, "twin_dE": abs(dE) * f,
            "twin_dE_bound": (abs(dE) + 3 * se) * f, "sample_tuples": n_s,
            "max_tuple_rel": maxrel}


def _device_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:  # pragma: no cover
        return f"device{device}"


def _load_cache() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_cache(c: dict) -> None:
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(c, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def _key(ctx: capi.Context, form: str) -> str:
    return f"{_device_name(ctx.device)}|No={ctx.No}|Nv={ctx.Nv}|{form}"


def _time(ctx, wins, form, slices, tuning, reps=3):
    ctx.set_tuning(**tuning)
    best = math.inf
    for _ in range(reps):
        ms, _ = run_windows(ctx, wins, form, slices)
        best = min(best, ms)
    return best


def tune_fp64(ctx: capi.Context, flops: float = 2e12, m: int = 8) -> dict:
    n = capi.n_tuples(ctx.Nv)
    wins = windows(n, m, window_size(ctx.No, ctx.Nv, m, flops))
    cands = [{"fp64_tile_rows": 64, "fp64_min_blocks": 0},
             {"fp64_tile_rows": 64, "fp64_min_blocks": 2},
             {"fp64_tile_rows": 32, "fp64_min_blocks": 0}]
    run_windows(ctx, wins[:1], "fp64")  # warm-up
    timed = [(_time(ctx, wins, "fp64", 0, c), c) for c in cands]
    best_ms, best = min(timed, key=lambda x: x[0])
    for claim in (2, 4):
        c = dict(best, tuples_per_claim=claim)
        t = _time(ctx, wins, "fp64", 0, c)
        if t < 0.98 * best_ms:
            best_ms, best = t, c
    ctx.set_tuning(**best)
    return {"tuning": best, "ms": best_ms, "trials": [(t, c) for t, c in timed],
            "sample_tuples": sum(hi - lo for lo, hi in wins)}


def f16_eligible(No: int, Nv: int) -> bool:
    """The FP16 form's kernel: 2 slices of No rows in the 128 M rows
    (No <= 64), level-0 sums below 2^31 (K = 2 (Nv + No) < 2048)."""
    return No <= 64 and 2 * (Nv + No) < 2048


def split_formats(No: int, Nv: int, form: str = "split", slice_counts=(2, 3, 4)):
    """(form, slices) candidates in order of tensor-core work: 2 FP16 slices
    (3 digit products, 22-bit digits) replace 2 BF16 slices (3 products,
    16 bits) where the FP16 kernel covers the system."""
    out = []
    if form in ("split", "split_f16") and f16_eligible(No, Nv):
        out.append(("split_f16", 2))
    if form != "split_f16":
        out += [("split_bf16", S) for S in slice_counts if not (out and S == 2)]
    return out


def choose_slices(ctx: capi.Context, tol_eh: float = 1e-8, flops: float = 2e12, m: int = 16,
                  slice_counts=(2, 3, 4), form: str = "split_bf16") -> dict:
    """Cheapest slice format whose twin error bound is within tol_eh."""
    n = capi.n_tuples(ctx.Nv)
    wins = windows(n, m, window_size(ctx.No, ctx.Nv, m, flops))
    _, e_ref = run_windows(ctx, wins, "fp64")
    report = {}
    cands = split_formats(ctx.No, ctx.Nv, form, slice_counts)
    chosen = cands[-1]
    for f, S in cands:
        _, e_s = run_windows(ctx, wins, f, S)
        est = error_estimate(n, e_ref, e_s)
        report[f"{f}x{S}"] = est
        if est["twin_dE_bound"] <= tol_eh:
            chosen = (f, S)
            break
    return {"form": chosen[0], "slices": chosen[1], "estimates": report}


def tune_split(ctx: capi.Context, slices: int, flops: float = 2e13, m: int = 8,
               form: str = "split_bf16") -> dict:
    n = capi.n_tuples(ctx.Nv)
    wins = windows(n, m, window_size(ctx.No, ctx.Nv, m, flops))
    run_windows(ctx, wins[:1], form, slices)  # warm-up (cuts the slices)
    f16 = form == "split_f16"  # always the transposed kernel
    cands = [{"split_stages": st} for st in (0, 3, 4)]
    if ctx.No <= 24 and not f16:  # W copy in shared memory, or a deeper ring with W in L2
        cands += [{"split_stages": st, "split_w_global": 1} for st in (0, 5)]
    if f16:
        cands = [{"split_variant": 2, "split_stages": st} for st in (0, 3)]
        cands += [{"split_variant": 2, "split_w_global": 1}]
        if ctx.No % 8 == 0:
            cands += [{"split_variant": 3}]
    elif slices * ctx.No <= 128 and 2 * (ctx.Nv + ctx.No) <= 1024:
        # transposed kernel: stacked slices as M, (p,q) pairs as N <= 256
        cands += [{"split_variant": 2, "split_stages": st} for st in (0, 3)]
        cands += [{"split_variant": 2, "split_w_global": 1}]
        if ctx.No % 8 == 0:  # one shared stack load per K chunk
            cands += [{"split_variant": 3}]
    timed = [(_time(ctx, wins, form, slices, c), c) for c in cands]
    best_ms, tuning = min(timed, key=lambda x: x[0])
    # L2 prefetch of the next part's slab tiles
    c = dict(tuning, split_prefetch=1)
    t = _time(ctx, wins, form, slices, c)
    timed.append((t, c))
    if t < 0.98 * best_ms:
        best_ms, tuning = t, c
    # then the processing order: tuples grouped by (a, b, c) blocks of side L
    # keep the slabs of the tuples in flight in L2
    for L in (4, 6, 8, 12, 16, 24):
        c = dict(tuning, tuple_block=L)
        t = _time(ctx, wins, form, slices, c)
        timed.append((t, c))
        if t < 0.98 * best_ms:
            best_ms, tuning = t, c
    ctx.set_tuning(**tuning)
    return {"tuning": tuning, "ms": best_ms, "trials": timed}


def tune(ctx: capi.Context, form: str = "split_bf16", tol_eh: float = 1e-8,
         use_cache: bool = True, slices: int = 0) -> dict:
    """Tune ctx for form; returns {"tuning": ..., "form": ..., "slices": ...}
    and applies the tuning to ctx.  slices=0 lets the tuner choose; form
    "split" lets it choose between the FP16 and BF16 split forms too."""
    key = _key(ctx, form) + (f"|S={slices}" if slices else "")
    cache = _load_cache() if use_cache else {}
    if key in cache:
        ent = cache[key]
        ctx.set_tuning(**ent["tuning"])
        return dict(ent, cached=True)
    t0 = time.perf_counter()
    if form == "fp64":
        r = tune_fp64(ctx)
        ent = {"tuning": r["tuning"], "form": "fp64", "slices": 0, "detail": {"fp64": r}}
    else:
        if slices:
            f = "split_bf16" if form == "split" else form
            acc = {"form": f, "slices": slices, "estimates": {}}
        else:
            acc = choose_slices(ctx, tol_eh, form=form)
        r = tune_split(ctx, acc["slices"], form=acc["form"])
        ent = {"tuning": r["tuning"], "form": acc["form"], "slices": acc["slices"],
               "detail": {"accuracy": acc["estimates"], "split": r}}
    ent["seconds"] = time.perf_counter() - t0
    if use_cache:
        cache = _load_cache()
        cache[key] = json.loads(json.dumps(ent, default=str))
        _save_cache(cache)
    return dict(ent, cached=False)


def tune_batch(batch: capi.Batch, window: int = 256) -> dict:
    """Batch kernel register budget and claim size, timed on the first
    `window` tuples of every system (FP64 form)."""
    best = None
    trials = []
    batch.run(form="fp64", use_j=False, max_iterations=window - 1)  # warm-up
    for c in ({"fp64_min_blocks": 0}, {"fp64_min_blocks": 2},
              {"fp64_min_blocks": 0, "tuples_per_claim": 4}):
        batch.set_tuning(**c)
        ms = min(batch.run(form="fp64", use_j=False, max_iterations=window - 1)[0].device_ms
                 for _ in range(2))
        trials.append((ms, c))
        if best is None or ms < best[0]:
            best = (ms, c)
    batch.set_tuning(**best[1])
    return {"tuning": best[1], "ms": best[0], "trials": trials}


def tune_batch_tiles(contexts, window: int = 256) -> list:
    """Per-system FP64 row tile (32 or 64), timed on a window of each."""
    out = []
    for ctx in contexts:
        if ctx.No > 16:
            ctx.set_tuning(fp64_tile_rows=64)
            out.append(64)
            continue
        n = capi.n_tuples(ctx.Nv)
        wins = [(0, min(n, window))]
        t = {}
        for rows in (64, 32):
            t[rows] = _time(ctx, wins, "fp64", 0, {"fp64_tile_rows": rows})
        rows = min(t, key=t.get)
        ctx.set_tuning(fp64_tile_rows=rows)
        out.append(rows)
    return out

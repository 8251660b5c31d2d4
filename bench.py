"""Benchmark of the CCSD(T) triples loop on GB300.

Workloads (synthetic inputs with the benchmark's seeded value distributions):

  no40_nv400  (default) No=40, Nv=400, seed 0: the precision workload, on
              which the benchmark compares the FP64 and split forms
  no24_nv240  No=24, Nv=240, seed 0 (the plain-FP64 drop-in workload)
  no56_nv560  No=56, Nv=560, seed 0 (the large single system)
  no8_nv40    No=8, Nv=40, seed 0 (the reference's own CPU-sized case)
  batch96     96 systems, No in [4,20], Nv in [30,200], seeds 0..95, one
              batch (captured graph) per step

A step is one pass of the hot path over one batch of tuples: for a single
system a contiguous stretch of the lexicographic tuple list holding about
1e14 FP64-equivalent FLOPs (the whole list at No=24/Nv=240), consecutive
steps walking through the list; for batch96 every tuple of every system.
Inputs (>= 3 GB) are larger than the 129 MB L2, so no flush is needed.

Metric: FP64-equivalent TFLOP/s of the triples loop (atrip's own count,
12 No^3 (No + Nv) FLOPs per tuple, src/atrip/Atrip.cxx:578-580), with the
time to the full E(T) beside it.  The default form ("split") lets the
autotuner pick the slice format -- 2 FP16 slices where their kernel covers
the system, else 2..4 BF16 slices -- as the cheapest one whose estimated
|dE(T)| on the |E(T)| ~ 0.1 Eh twin stays within 1e-8 Eh, then the launch
parameters; the same line carries the FP64 form's throughput on sample
windows of the same list and the sampled |dE(T)| between the two forms.

  python bench.py [--workload W] [--form split|split_f16|split_bf16|fp64]
                  [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 0
WORKLOADS = {"no8_nv40": (8, 40), "no24_nv240": (24, 240), "no40_nv400": (40, 400),
             "no56_nv560": (56, 560), "batch96": None}
DEFAULT_WORKLOAD = "no40_nv400"
STEP_FLOPS = 1e14        # FP64-equivalent work of one split-form step
STEP_FLOPS_FP64 = 3e12   # ... of one FP64-form step
TENSORS = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci")
METRIC = "CCSD(T) triples FP64-equivalent TFLOP/s (12 No^3 (No+Nv) per tuple)"


def flops_per_tuple(No, Nv):
    return 12.0 * No ** 3 * (No + Nv)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_median": statistics.median(power) if power else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)) if os.path.exists(path) else {}


def traffic_per_tuple(kernel: str, workload: str, form: str = "fp64", slices: int = 0):
    """DRAM bytes per tuple of `kernel` on `workload` in `form` with `slices`
    from the committed ncu summary (profiles/traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        ent = json.load(open(path))[kernel][workload]
        if kernel == "triples_split_kernel" and (ent.get("form", "split_bf16"),
                                                 ent.get("slices", 3)) != (form, slices):
            return None
        return float(ent["bytes_per_tuple"])
    except (OSError, KeyError, ValueError, TypeError):
        return None


# ---------------------------------------------------------------- CPU arms

def cpu_baseline(d, seconds=12.0, threads=None):
    """The oracle's DGEMM-route port (numpy's OpenBLAS dgemm, one thread per
    worker, tuples split over all host cores) on a bounded sample of the
    workload's tuple list.  Returns the cpu_baseline object."""
    import oracle
    threads = threads or os.cpu_count() or 1
    blas = oracle.register_numpy_openblas()
    No, Nv = d["No"], d["Nv"]
    p = oracle.Problem(d)
    port = oracle.PreparedPort(p)
    n = int(oracle.n_tuples(Nv))
    probe = min(n, 2 * threads)
    mid = n // 2
    t = time.perf_counter()
    port.run(mid, min(n, mid + probe), threads)
    dt = max(time.perf_counter() - t, 1e-6)
    sample = int(min(n, max(probe, probe * seconds / dt)))
    t0 = max(0, min(mid, n - sample))
    t1 = min(n, t0 + sample)
    t = time.perf_counter()
    port.run(t0, t1, threads)
    dt = time.perf_counter() - t
    port.close()
    tflops = (t1 - t0) * flops_per_tuple(No, Nv) / dt / 1e12
    return {"value": tflops, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": f"tuples {t0}..{t1 - 1} of {n} ({t1 - t0} tuples, {dt:.1f} s), DGEMM route "
                      f"with {'OpenBLAS ' + os.path.basename(blas) if blas else 'C loops'}",
            "tuples_per_s": (t1 - t0) / dt,
            "time_to_ET_s_extrapolated": n / ((t1 - t0) / dt)}


def cpu_baseline_batch(ds, seconds=12.0, threads=None):
    """The port on a bounded sample of the multi-system workload: a stretch
    of the tuple list of every 12th system, about seconds/8 s each."""
    import oracle
    threads = threads or os.cpu_count() or 1
    oracle.register_numpy_openblas()
    flops, secs, parts = 0.0, 0.0, []
    for d in ds[::12]:
        No, Nv = d["No"], d["Nv"]
        n = int(oracle.n_tuples(Nv))
        port = oracle.PreparedPort(oracle.Problem(d))
        probe = min(n, 2 * threads)
        t = time.perf_counter()
        port.run(0, probe, threads)
        dt = max(time.perf_counter() - t, 1e-6)
        m = int(min(n, max(probe, probe * (seconds / 8) / dt)))
        t0 = (n - m) // 2
        t = time.perf_counter()
        port.run(t0, t0 + m, threads)
        dt = time.perf_counter() - t
        port.close()
        flops += m * flops_per_tuple(No, Nv)
        secs += dt
        parts.append(f"No={No} Nv={Nv}: {m} tuples")
    v = flops / secs / 1e12
    return {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": "; ".join(parts) + f" ({secs:.1f} s)"}


BATCH96 = "96 CCSD(T) triples systems, No in [4,20], Nv in [30,200], seeds 0..95"


def workload_config(workload, No=None, Nv=None, n_tuples=None):
    """The bench line's `config`: what identifies the workload, the same for
    both arms (run-dependent details go to the line's `run` object)."""
    from atrip_gb300 import capi, synth
    if workload == "batch96":
        n = sum(capi.n_tuples(nv) for _, nv, _ in synth.multi_system_sizes(96))
        return {"workload": BATCH96, "name": "batch96", "n_tuples": n,
                "l2": "no flush: inputs > 129 MB L2"}
    # FP64 inputs: eps_i, eps_a, T1, T2, V_pphh, V_hhhp, V_pphp
    nbytes = 8 * (No + Nv + Nv * No + 2 * Nv * Nv * No * No + No ** 3 * Nv + Nv ** 3 * No)
    l2 = ("no flush: inputs > 129 MB L2" if nbytes > 129e6 else
          f"no flush: the {nbytes / 1e6:.0f} MB of inputs fit the 129 MB L2 "
          "(a parity-size workload, not a timing one)")
    return {"workload": f"CCSD(T) triples No={No} Nv={Nv} seed {SEED}", "name": workload,
            "n_tuples": n_tuples if n_tuples is not None else capi.n_tuples(Nv), "l2": l2}


def run_reference_arm(args, workload):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from atrip_gb300 import synth
    import oracle
    threads = os.cpu_count() or 1
    oracle.register_numpy_openblas()
    if workload == "batch96":
        sizes = synth.multi_system_sizes(96)[::12]
        systems = [synth.make_inputs(No, Nv, s) for No, Nv, s in sizes]
        desc = "every 12th system of the 96-system workload"
        cfg = workload_config("batch96")
    else:
        No, Nv = WORKLOADS[workload] if workload in WORKLOADS else (args.no, args.nv)
        systems = [synth.make_inputs(No, Nv, SEED)]
        desc = f"No={No} Nv={Nv} seed {SEED}"
        cfg = workload_config(workload, No, Nv)
    ports = [(d, oracle.PreparedPort(oracle.Problem(d)), int(oracle.n_tuples(d["Nv"])))
             for d in systems]
    times, flops = [], 0.0
    for step in range(args.warmup + args.steps):
        t_step, f_step = 0.0, 0.0
        for d, port, n in ports:
            fpt = flops_per_tuple(d["No"], d["Nv"])
            batch = max(threads, int(args.ref_flops / len(ports) / fpt))
            batch = min(batch, n)
            lo = ((n // 2) + step * batch) % max(1, n - batch + 1)
            t = time.perf_counter()
            port.run(lo, lo + batch, threads)
            t_step += time.perf_counter() - t
            f_step += batch * fpt
        if step >= args.warmup:
            times.append(t_step)
            flops += f_step
    for _, port, _ in ports:
        port.close()
    total = sum(times)
    value = flops / total / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, benchmark value distributions)",
            "config": cfg,
            "run": {"systems": desc, "flops_per_step": flops / args.steps},
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steps of ~{args.ref_flops:.0e} FLOPs, "
                                       f"stretches from the middle of the tuple list ({desc})"},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU arm

def _upload_all(ctx, d, names=TENSORS):
    for name in names:
        ctx.upload(name, d[name])


def _pinned(d):
    import torch
    out, nbytes = {}, 0
    for name in TENSORS:
        flat = np.ascontiguousarray(np.asarray(d[name]).ravel(order="F"))
        t = torch.from_numpy(flat).pin_memory()
        out[name] = t
        nbytes += t.numel() * 8
    return out, nbytes


def _timed(steps, stream, fn):
    """Run fn(s) for s < steps between CUDA events on stream, with the
    clocks sampled meanwhile.  Returns (ms, results, clocks)."""
    import torch
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    res = [fn(s) for s in range(steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    return ms, res, clocks.stop()


def _fp64_rate(ctx, n, fpt):
    """FP64-form TFLOP/s over one contiguous stretch in the middle of the
    list, 8 waves of the largest resident FP64 grid (4 CTAs per SM) long, so
    that the last partial wave does not count; the error-sample windows are
    separate launches too short for a rate (a window of fewer tuples than
    resident CTAs leaves SMs idle)."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    w = min(n, 8 * 4 * sms)
    lo = (n - w) // 2
    r = ctx.run(form="fp64", use_j=False, first_iteration=lo, max_iterations=lo + w - 1)
    return r.tuples_done * fpt / (r.device_ms * 1e-3) / 1e12, w


def _role_profile(ctx, form, slices, lo, hi):
    """One extra, untimed run of tuples [lo, hi) with the kernel built with
    per-role cycle counters (atrip_gpu_split_profile; 2-slice transposed
    kernel only): per role its cycles per tuple (one CTA) and the share of
    its lifetime spent in each wait; the rest of a role's time is its work."""
    from atrip_gb300 import capi
    tuned = ctx.get_tuning()
    try:
        ctx.set_tuning(**dict(tuned, split_profile=1))
        r = ctx.run(form=form, slices=slices, use_j=False, first_iteration=lo,
                    max_iterations=hi - 1)
        c = ctx.split_profile()
    except capi.AtripError as exc:
        return {"unavailable": str(exc)}
    finally:
        ctx.set_tuning(**tuned)
    tuples = max(c["tuples"], 1)
    roles = {"producer": ("stage", "tuple_slot"), "mma": ("tuple", "accumulator", "stage"),
             "epilogue": ("tuple", "w_buffer", "accumulator"), "energy": ("tuple", "w")}
    out = {"tuples": c["tuples"], "ctas": c["ctas"], "device_ms": r.device_ms,
           "stages_per_tuple": c["stages"] / tuples,
           "cycles_per_tuple": {k: c[f"{k}_total"] / tuples for k in roles},
           "wait_share": {}}
    for k, waits in roles.items():
        tot = max(c[f"{k}_total"], 1)
        for w in waits:
            out["wait_share"][f"{k}_wait_{w}"] = c[f"{k}_wait_{w}"] / tot
    out["wait_share"]["energy_w_convert"] = c["energy_w_convert"] / max(c["energy_total"], 1)
    return out


def _max_over_ranks(world, ms, count):
    if world <= 1:
        return ms, count
    import torch
    t = torch.tensor([ms], device="cuda")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    c = torch.tensor([float(count)], device="cuda")
    torch.distributed.all_reduce(c)
    return float(t.item()), c.item()


def _roofline(form, slices, flops_per_launch, launch_ms, peaks, live_fp64, traffic):
    if form == "fp64":
        achieved = flops_per_launch / (launch_ms * 1e-3) / 1e12
        peak = live_fp64
        src = "measured FP64 DFMA/DMMA peak (live, atrip_gpu_measure_peaks)"
        kernel = "triples_fp64_kernel"
    else:
        products = slices * (slices + 1) // 2
        achieved = flops_per_launch * products / (launch_ms * 1e-3) / 1e12
        peak = peaks.get("bf16_tflops", 1900.0)  # FP16 MMAs run at the BF16 rate
        src = ("of measured BF16 dense peak (bf16_tflops, burst)" if "bf16_tflops" in peaks
               else "of fallback BF16 peak")
        kernel = "triples_split_kernel"
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": src, "kernel": kernel,
            "algorithmic": ("FP64-equivalent FLOPs per launch" if form == "fp64" else
                            f"{'FP16' if form == 'split_f16' else 'BF16'} MMA FLOPs per "
                            f"launch = FP64-equivalent x S(S+1)/2 = "
                            f"{slices * (slices + 1) // 2} digit products (S={slices}), "
                            "unpadded")}


def run_single(args, workload, world, rank, local):
    import torch
    from atrip_gb300 import autotune, capi, synth

    No, Nv = WORKLOADS[workload] if workload in WORKLOADS else (args.no, args.nv)
    fpt = flops_per_tuple(No, Nv)
    t_gen = time.perf_counter()
    d = synth.make_inputs(No, Nv, SEED)
    t_gen = time.perf_counter() - t_gen
    n = capi.n_tuples(Nv)
    form = args.form
    batch = args.batch_tuples or max(1, int((STEP_FLOPS if form != "fp64" else STEP_FLOPS_FP64)
                                            / fpt))
    # the list is cut into `parts` equal stretches of `batch` tuples (the last
    # one shorter); step s runs stretch (s + rank) % parts (weak scaling:
    # rank r starts at its own stretch)
    parts = max(1, round(n / min(batch, n)))
    batch = -(-n // parts)

    ctx = capi.Context(No, Nv, local)
    _upload_all(ctx, d)
    stream = torch.cuda.Stream()
    if args.tuning or args.no_tune:
        if args.tuning:
            ctx.set_tuning(**json.loads(args.tuning))
        form = "split_bf16" if form == "split" else form
        tune = {"tuning": ctx.get_tuning(),
                "slices": args.slices or (2 if form == "split_f16" else 3)}
    else:
        tune = autotune.tune(ctx, form, tol_eh=args.tol_eh, use_cache=not args.retune,
                             slices=args.slices)
        form = tune.get("form", "split_bf16" if form == "split" else form)
    slices = tune["slices"] if form != "fp64" else 0

    def stretch(s):
        lo = ((s + rank) % parts) * batch
        return lo, min(n, lo + batch)

    def step(s):
        lo, hi = stretch(s)
        return ctx.run(form=form, slices=slices, use_j=False, first_iteration=lo,
                       max_iterations=hi - 1, stream=stream.cuda_stream)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms, res, clk = _timed(args.steps, stream, step)
    tuples = sum(r.tuples_done for r in res)
    launches = sum(r.kernel_launches for r in res)
    ms, tuples_all = _max_over_ranks(world, ms, tuples)
    value = tuples_all * fpt / (ms * 1e-3) / 1e12
    time_to_et = n * fpt / (value * 1e12)  # whole list at the whole job's rate

    # ---- FP64 form on sample windows of the same list (and the error estimate)
    compare = None
    if form != "fp64" and not args.no_compare:
        m = 16
        wins = autotune.windows(n, m, autotune.window_size(No, Nv, m, args.compare_flops))
        tuned = ctx.get_tuning()
        fp64_tune = autotune.tune(ctx, "fp64", use_cache=not args.retune)["tuning"]
        ms64, e64 = autotune.run_windows(ctx, wins, "fp64")
        fp64_tflops, rate_tuples = _fp64_rate(ctx, n, fpt)
        ctx.set_tuning(**tuned)
        ms_s, es = autotune.run_windows(ctx, wins, form, slices)
        est = autotune.error_estimate(n, e64, es)
        compare = {"fp64_tflops": fp64_tflops,
                   "fp64_time_to_ET_s": n * fpt / (fp64_tflops * 1e12),
                   "fp64_tuning": fp64_tune,
                   "fp64_rate_sample": f"{rate_tuples} consecutive tuples mid-list, one launch",
                   "speedup_split_vs_fp64": (n * fpt / (fp64_tflops * 1e12)) / time_to_et,
                   "windows": f"{len(wins)} windows x {wins[0][1] - wins[0][0]} tuples",
                   "accuracy": {k: est[k] for k in ("E_est", "dE_est", "dE_stderr", "rel",
                                                    "twin_scale_log2", "twin_E", "twin_dE",
                                                    "twin_dE_bound", "max_tuple_rel",
                                                    "sample_tuples")},
                   "tolerance_eh": args.tol_eh}

    # ---- where the kernel's time goes: one untimed profiled run of a step
    role_prof = None
    if form != "fp64" and rank == 0 and not args.no_role_profile:
        role_prof = _role_profile(ctx, form, slices, *stretch(0))

    # ---- end to end through the C ABI with host (pinned) buffers; the
    # timed context is released first so the large workloads fit twice over
    tuning_used = ctx.get_tuning()
    kernel_ms = sum(r.device_ms for r in res) / len(res)
    live_fp64 = capi.measure_peaks(local)[0] if (form == "fp64" and rank == 0) else None
    ctx.close()
    e2e_steps = 0 if args.no_e2e else args.steps
    pinned, h2d = _pinned(d) if e2e_steps else ({}, sum(
        np.asarray(d[name]).nbytes for name in TENSORS))
    torch.cuda.synchronize()
    e2e_tuples, e2e_s, whole = 0, 0.0, None
    if e2e_steps:
        with capi.Context(No, Nv, local) as c2:
            c2.set_tuning(**tuning_used)
            t0 = time.perf_counter()
            for s in range(e2e_steps):
                # every step: pinned H2D + re-layout of every input (and the
                # split operands cut again), the step's tuples, energy D2H
                for name in TENSORS:
                    c2.upload_ptr(name, pinned[name].data_ptr(), pinned[name].numel(), False)
                lo, hi = stretch(s)
                r = c2.run(form=form, slices=slices, use_j=False, first_iteration=lo,
                           max_iterations=hi - 1)
                e2e_tuples += r.tuples_done
            e2e_s = time.perf_counter() - t0
        # time to E(T) end to end: one context, one upload, the whole list,
        # where the whole list fits the bench's time budget
        if time_to_et <= args.whole_list_max_s:
            t0 = time.perf_counter()
            with capi.Context(No, Nv, local) as c3:
                c3.set_tuning(**tuning_used)
                for name in TENSORS:
                    c3.upload_ptr(name, pinned[name].data_ptr(), pinned[name].numel(), False)
                r = c3.run(form=form, slices=slices, use_j=False)
            secs = time.perf_counter() - t0
            whole = {"time_to_ET_s": secs, "tflops": n * fpt / secs / 1e12,
                     "energy": r.energy, "tuples": r.tuples_done,
                     "note": "context create, pinned H2D + re-layout of all inputs, operands "
                             "cut, every tuple of the list, E(T) back"}
    e2e_value = (e2e_tuples * fpt / e2e_s / 1e12 * max(world, 1)) if e2e_steps else None

    if rank != 0:
        return 0
    peaks = load_peaks()
    # per launch: the steps' mean tuples and mean device time of the loop
    launch_tuples = tuples / len(res)
    kname = "triples_fp64_kernel" if form == "fp64" else "triples_split_kernel"
    tpt = traffic_per_tuple(kname, workload, form, slices)
    roof = _roofline(form, slices, launch_tuples * fpt, kernel_ms, peaks, live_fp64,
                     tpt * launch_tuples if tpt is not None else None)
    roof["tuples_per_launch"] = launch_tuples
    cpu = None if args.no_cpu_baseline else cpu_baseline(d, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if form == "fp64" else f"{form[6:]}x{slices}->f64",
        "data": "synthetic (seeded, benchmark value distributions)",
        "config": workload_config(workload, No, Nv, n),
        "run": {"form": form, "slices": slices, "tuning": tune["tuning"],
                "tuples_per_step": batch, "stretches": parts,
                "time_to_ET_s": time_to_et, "input_gen_s": t_gen},
        "compare_fp64": compare,
        "roofline": roof,
        "role_profile": role_prof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 16, "steps": e2e_steps,
                "note": "per step: pinned H2D + re-layout of all inputs, split operands cut "
                        "(split form), the step's tuples, energies D2H",
                "whole_list": whole},
        "clocks": clk,
        "gpu_launches": launches,
    }
    print(json.dumps(line))
    return 0


def run_batch96(args, world, rank, local):
    import torch
    from atrip_gb300 import autotune, capi, synth

    sizes = synth.multi_system_sizes(96)
    t_gen = time.perf_counter()
    ds = [synth.make_inputs(No, Nv, s) for No, Nv, s in sizes]
    t_gen = time.perf_counter() - t_gen
    total_flops = sum(capi.n_tuples(Nv) * flops_per_tuple(No, Nv) for No, Nv, _ in sizes)
    total_tuples = sum(capi.n_tuples(Nv) for _, Nv, _ in sizes)
    ctxs = []
    for d in ds:
        c = capi.Context(d["No"], d["Nv"], local)
        _upload_all(c, d)
        ctxs.append(c)
    form = args.form
    if form == "split":  # FP16 slices where every system fits their kernel
        ok = all(autotune.f16_eligible(c.No, c.Nv) for c in ctxs)
        form = "split_f16" if ok and args.slices in (0, 2) else "split_bf16"
    slices = args.slices or (2 if form == "split_f16" else 3)
    tiles = autotune.tune_batch_tiles(ctxs)
    b = capi.Batch(ctxs)
    btune = autotune.tune_batch(b)
    split_choice = None
    trials = []
    if form != "fp64":
        # one persistent launch over all systems (the default), or one launch
        # per system with each system's kernel variant and processing order:
        # one full batch run per candidate, the faster kept
        base = [c.get_tuning() for c in ctxs]
        bbase = dict(btune["tuning"])
        for launch, cand in (("one", {}), ("per-system", {}),
                             ("per-system", {"split_variant": 2}),
                             ("per-system", {"split_variant": 2, "tuple_block": 4})):
            for c, t in zip(ctxs, base):
                c.set_tuning(**dict(t, **cand))
            b.set_tuning(**dict(bbase, split_variant=1 if launch == "per-system" else 0))
            b.run(form=form, slices=slices, use_j=False)  # first run captures the graph
            ms = b.run(form=form, slices=slices, use_j=False)[0].device_ms
            trials.append((ms, dict(cand, launch=launch)))
        split_choice = min(trials, key=lambda x: x[0])
        cand = {k: v for k, v in split_choice[1].items() if k != "launch"}
        for c, t in zip(ctxs, base):
            c.set_tuning(**dict(t, **cand))
        b.set_tuning(**dict(bbase, split_variant=1 if split_choice[1]["launch"] == "per-system"
                            else 0))
    stream = torch.cuda.Stream()

    def step(s):
        return b.run(form=form, slices=slices, use_j=False, stream=stream.cuda_stream)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms, res, clk = _timed(args.steps, stream, step)
    launches = sum(r[0].kernel_launches for r in res)
    ms, _ = _max_over_ranks(world, ms, 0)
    value = total_flops * args.steps * max(world, 1) / (ms * 1e-3) / 1e12

    # FP64 form and accuracy on the first W tuples of every system
    W = 512
    r64 = b.run(form="fp64", use_j=False, max_iterations=W - 1)
    e64 = [c.tuple_energies(0, r.tuples_done)[0].copy() for c, r in zip(ctxs, r64)]
    rs = b.run(form=form, slices=slices, use_j=False, max_iterations=W - 1)
    es = [c.tuple_energies(0, r.tuples_done)[0].copy() for c, r in zip(ctxs, rs)]
    wflops = sum(min(W, capi.n_tuples(Nv)) * flops_per_tuple(No, Nv) for No, Nv, _ in sizes)
    fp64_tflops = wflops / (r64[0].device_ms * 1e-3) / 1e12
    rel = [float(np.max(np.abs(x - y)) / max(float(np.max(np.abs(y))), 1e-300))
           for x, y in zip(es, e64)]
    # the same windows' summed energy per system (what a user reads)
    sum_rel = [abs(float(np.sum(x) - np.sum(y))) / max(abs(float(np.sum(y))), 1e-300)
               for x, y in zip(es, e64)]
    compare = {"fp64_tflops": fp64_tflops, "fp64_time_to_ET_s": total_flops / fp64_tflops / 1e12,
               "speedup_split_vs_fp64": (total_flops / fp64_tflops / 1e12) / (ms / args.steps / 1e3),
               "windows": f"first {W} tuples of every system",
               "accuracy": {"max_tuple_rel": max(rel), "max_system_sum_rel": max(sum_rel)}}

    pinned = [_pinned(d) for d in ds]
    h2d = sum(p[1] for p in pinned)
    e2e_steps = 0 if args.no_e2e else 1
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        cs = []
        for d, (pin, _) in zip(ds, pinned):
            c2 = capi.Context(d["No"], d["Nv"], local)
            for name in TENSORS:
                c2.upload_ptr(name, pin[name].data_ptr(), pin[name].numel(), False)
            cs.append(c2)
        with capi.Batch(cs) as b2:
            b2.run(form=form, slices=slices, use_j=False)
        for c2 in cs:
            c2.close()
    e2e_s = time.perf_counter() - t0
    e2e_value = total_flops * e2e_steps / e2e_s / 1e12 if e2e_steps else None

    if rank != 0:
        return 0
    peaks = load_peaks()
    kernel_ms = statistics.median(r[0].device_ms for r in res)
    roof = _roofline(form, slices, total_flops, kernel_ms, peaks,
                     capi.measure_peaks(local)[0] if form == "fp64" else None, None)
    roof["note"] = "whole batch graph (all systems' launches and the energy reduction)"
    cpu = None if args.no_cpu_baseline else cpu_baseline_batch(ds, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if form == "fp64" else f"{form[6:]}x{slices}->f64",
        "data": "synthetic (seeded, benchmark value distributions)",
        "config": workload_config("batch96"),
        "run": {"form": form, "slices": slices,
                "tuples_per_step": total_tuples, "flops_per_step": total_flops,
                "fp64_row_tiles": {"32": tiles.count(32), "64": tiles.count(64)},
                "batch_tuning": btune["tuning"],
                "split_tuning": split_choice[1] if split_choice else None,
                "split_trials_ms": [(round(t, 2), c) for t, c in trials] if split_choice
                else None,
                "time_to_ET_s": ms / args.steps / 1e3, "input_gen_s": t_gen},
        "compare_fp64": compare,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 16 * len(ds),
                "note": "per step: 96 contexts created, pinned H2D + re-layout, batch run"},
        "clocks": clk,
        "gpu_launches": launches,
    }
    print(json.dumps(line))
    b.close()
    for c in ctxs:
        c.close()
    return 0


def run_precision_table(args, workload, local):
    """|dE(T)| and speed of several slice formats on one workload: one
    context, the FP64 form on 16 evenly spread windows, each split format on
    the same windows (sampled error, carried to the power-of-two twin) and on
    one stretch of ~1e14 FP64-equivalent FLOPs (throughput).  One JSON line
    per format, then a summary line."""
    from atrip_gb300 import autotune, capi, synth

    No, Nv = WORKLOADS[workload] if workload in WORKLOADS else (args.no, args.nv)
    fpt = flops_per_tuple(No, Nv)
    d = synth.make_inputs(No, Nv, SEED)
    n = capi.n_tuples(Nv)
    rows = []
    with capi.Context(No, Nv, local) as ctx:
        _upload_all(ctx, d)
        del d
        m = 16
        wins = autotune.windows(n, m, autotune.window_size(No, Nv, m, args.compare_flops))
        autotune.tune(ctx, "fp64", use_cache=not args.retune)
        ms64, e64 = autotune.run_windows(ctx, wins, "fp64")
        fp64_tflops, rate_tuples = _fp64_rate(ctx, n, fpt)
        batch = max(1, min(n, int(STEP_FLOPS / fpt)))
        lo = (n - batch) // 2
        for item in args.precision_table.split(","):
            form, S = item.split(":")
            S = int(S)
            try:
                tune = autotune.tune(ctx, form, use_cache=not args.retune, slices=S)
            except capi.AtripError as exc:
                rows.append({"form": form, "slices": S, "unavailable": str(exc)})
                print(json.dumps(rows[-1]), flush=True)
                continue
            _, es = autotune.run_windows(ctx, wins, form, S)
            est = autotune.error_estimate(n, e64, es)
            ctx.run(form=form, slices=S, use_j=False, first_iteration=lo,
                    max_iterations=lo + batch - 1)  # warm-up
            r = ctx.run(form=form, slices=S, use_j=False, first_iteration=lo,
                        max_iterations=lo + batch - 1)
            tflops = r.tuples_done * fpt / (r.device_ms * 1e-3) / 1e12
            row = {"workload": f"No={No} Nv={Nv} seed {SEED}", "form": form, "slices": S,
                   "tflops": tflops, "time_to_ET_s": n * fpt / (tflops * 1e12),
                   "speedup_vs_fp64": tflops / fp64_tflops, "tuning": tune["tuning"],
                   "accuracy": {k: est[k] for k in ("E_est", "dE_est", "dE_stderr", "rel",
                                                    "twin_scale_log2", "twin_E", "twin_dE",
                                                    "twin_dE_bound", "max_tuple_rel",
                                                    "sample_tuples")},
                   "meets_1e-8_Eh_twin": est["twin_dE_bound"] <= args.tol_eh}
            rows.append(row)
            print(json.dumps(row), flush=True)
    print(json.dumps({"precision_table": f"No={No} Nv={Nv}", "fp64_tflops": fp64_tflops,
                      "fp64_time_to_ET_s": n * fpt / (fp64_tflops * 1e12),
                      "fp64_rate_sample": f"{rate_tuples} consecutive tuples mid-list, one launch",
                      "windows": f"{len(wins)} windows x {wins[0][1] - wins[0][0]} tuples",
                      "note": "sampled errors: extrapolated from the windows; the estimator's "
                              "3-sigma bound is checked against whole-list differences at "
                              "No=24/Nv=240 by tests/test_gpu_cfg2_full.py",
                      "rows": len(rows)}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + ["custom"])
    ap.add_argument("--form", default="split", choices=["split", "fp64", "split_bf16", "split_f16"],
                    help="split: the autotuner picks FP16 or BF16 slices and their count")
    ap.add_argument("--slices", type=int, default=0, help="0: chosen by the autotuner")
    ap.add_argument("--tol-eh", type=float, default=1e-8)
    ap.add_argument("--retune", action="store_true", help="ignore the tuning cache")
    ap.add_argument("--no-tune", action="store_true",
                    help="built-in launch parameters, --slices or 3 slices (profiling runs)")
    ap.add_argument("--tuning", default="",
                    help="explicit atrip_tuning fields as JSON instead of the autotuner "
                         "(profiling runs), e.g. '{\"split_variant\": 2}'")
    ap.add_argument("--batch-tuples", type=int, default=0)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-flops", type=float, default=1e12)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--compare-flops", type=float, default=4e12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-role-profile", action="store_true",
                    help="skip the untimed profiled run behind role_profile")
    ap.add_argument("--whole-list-max-s", type=float, default=60.0,
                    help="run the end-to-end whole-list time to E(T) when the device rate "
                         "says it takes at most this long")
    ap.add_argument("--precision-table", default="",
                    help="instead of the bench line: sampled |dE(T)| and speed per slice "
                         "format, e.g. 'split_f16:2,split_bf16:2,split_bf16:3,split_bf16:4'")
    ap.add_argument("--no", type=int, default=24, help="No of --workload custom")
    ap.add_argument("--nv", type=int, default=240, help="Nv of --workload custom")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference_arm(args, args.workload)

    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.precision_table:
        return run_precision_table(args, args.workload, local)
    if args.workload == "batch96":
        return run_batch96(args, world, rank, local)
    return run_single(args, args.workload, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())

"""Benchmark of the CCSD(T) triples loop on GB300.

Workload: No=24, Nv=240, seed 0 (the plain-FP64 drop-in configuration of
the benchmark definition), synthetic inputs with its value distributions.
A step is one pass of the hot path over one batch of the lexicographic tuple
list; consecutive steps walk through the list.  The inputs (3.2 GB) are
larger than L2, so no flush is needed between steps.

Metric: FP64-equivalent TFLOP/s of the triples loop, counting atrip's own
12 No^3 (No + Nv) FLOPs per tuple (src/atrip/Atrip.cxx:578-580); the
extrapolated time to the full E(T) is reported beside it.

  python bench.py [--steps K] [--warmup W] [--form fp64|split_bf16]
                  [--batch-tuples B] [--impl reference]
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

NO, NV, SEED = 24, 240, 0
TENSORS = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci")
METRIC = "CCSD(T) triples FP64-equivalent TFLOP/s (12 No^3 (No+Nv) per tuple)"


def flops_per_tuple(No=None, Nv=None):
    No = NO if No is None else No
    Nv = NV if Nv is None else Nv
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs():
    from atrip_gb300 import synth
    return synth.make_inputs(NO, NV, SEED)


def cpu_baseline(d, seconds=12.0, threads=None):
    """The oracle's DGEMM-route port (numpy's OpenBLAS dgemm, one thread per
    worker, tuples split over all host cores) on a bounded sample of the
    workload's tuple list.  Returns the cpu_baseline object."""
    import oracle
    threads = threads or os.cpu_count() or 1
    blas = oracle.register_numpy_openblas()
    p = oracle.Problem(d)
    port = oracle.PreparedPort(p)
    n = int(oracle.n_tuples(NV))
    probe = min(n, 4 * threads)
    t = time.perf_counter()
    port.run(0, probe, threads)
    dt = max(time.perf_counter() - t, 1e-6)
    sample = int(min(n, max(probe, probe * seconds / dt)))
    t0 = n // 2  # a middle stretch of the list
    t1 = min(n, t0 + sample)
    t = time.perf_counter()
    port.run(t0, t1, threads)
    dt = time.perf_counter() - t
    port.close()
    tflops = (t1 - t0) * flops_per_tuple() / dt / 1e12
    return {"value": tflops, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": f"tuples {t0}..{t1 - 1} of {n} ({t1 - t0} tuples, {dt:.1f} s), DGEMM route "
                      f"with {'OpenBLAS ' + os.path.basename(blas) if blas else 'C loops'}",
            "tuples_per_s": (t1 - t0) / dt,
            "time_to_ET_s_extrapolated": n / ((t1 - t0) / dt)}


def run_reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    d = make_inputs()
    import oracle
    threads = os.cpu_count() or 1
    oracle.register_numpy_openblas()
    p = oracle.Problem(d)
    port = oracle.PreparedPort(p)
    n = int(oracle.n_tuples(NV))
    batch = max(threads, int(args.ref_batch))
    pos = n // 2
    for _ in range(args.warmup):
        port.run(pos, min(n, pos + threads), threads)
    times = []
    done = 0
    for s in range(args.steps):
        lo = (pos + s * batch) % max(1, n - batch)
        t = time.perf_counter()
        port.run(lo, lo + batch, threads)
        times.append(time.perf_counter() - t)
        done += batch
    port.close()
    total = sum(times)
    value = done * flops_per_tuple() / total / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"CCSD(T) triples No={NO} Nv={NV} seed {SEED}",
                       "tuples_per_step": batch, "l2": "inputs 3.2 GB > L2"},
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steps of {batch} tuples from tuple {pos}"},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "time_to_ET_s_extrapolated": n * total / done}
    print(json.dumps(line))
    return 0


def main():
    global NO, NV
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--form", default="fp64", choices=["fp64", "split_bf16"])
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--batch-tuples", type=int, default=0,
                    help="tuples per step (default: whole list for split, 1%% for fp64)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-batch", type=int, default=2048)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no", type=int, default=NO, help="override No (profiling captures)")
    ap.add_argument("--nv", type=int, default=NV, help="override Nv (profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    NO, NV = args.no, args.nv
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch
    from atrip_gb300 import capi

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    d = make_inputs()
    n = capi.n_tuples(NV)
    batch = args.batch_tuples or (n if args.form != "fp64" else max(1, n // 100))
    batch = min(batch, n)
    # weak scaling: rank r walks its own stretch of the tuple list
    origin = (rank * batch) % n

    ctx = capi.Context(NO, NV, local)
    for name in TENSORS:
        ctx.upload(name, d[name])
    stream = torch.cuda.Stream()

    def step(s):
        lo = (origin + s * batch) % n
        hi = min(n, lo + batch)
        return ctx.run(form=args.form, slices=args.slices, first_iteration=lo,
                       max_iterations=hi - 1, stream=stream.cuda_stream)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    launches, tuples, kernel_ms = 0, 0, []
    form_used = None
    for s in range(args.steps):
        r = step(s)
        launches += r.kernel_launches
        tuples += r.tuples_done
        kernel_ms.append(r.device_ms)
        form_used = r.form_used
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        tt = torch.tensor([float(tuples)], device="cuda")
        torch.distributed.all_reduce(tt)
        tuples_all = int(tt.item())
    else:
        tuples_all = tuples
    value = tuples_all * flops_per_tuple() / (ms * 1e-3) / 1e12

    # ---- end to end through the C ABI with host (pinned) buffers
    pinned = {}
    h2d = 0
    for name in TENSORS:
        flat = np.ascontiguousarray(np.asarray(d[name]).ravel(order="F"))
        t = torch.from_numpy(flat).pin_memory()
        pinned[name] = t
        h2d += t.numel() * 8
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_tuples = 0
    for s in range(e2e_steps):
        with capi.Context(NO, NV, local) as c2:
            for name in TENSORS:
                c2.upload_ptr(name, pinned[name].data_ptr(), pinned[name].numel(), False)
            lo = (origin + s * batch) % n
            hi = min(n, lo + batch)
            r = c2.run(form=args.form, slices=args.slices, first_iteration=lo,
                       max_iterations=hi - 1)
            e2e_tuples += r.tuples_done
    e2e_s = time.perf_counter() - t0
    e2e_value = (e2e_tuples * flops_per_tuple() / e2e_s / 1e12 * (world if world > 1 else 1)
                 if e2e_steps else None)

    if rank != 0:
        return 0
    # ---- roofline of the dominant kernel
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    if form_used == capi.FORM_FP64:
        fp64_peak, _ = capi.measure_peaks(local)
        peak, peak_note = fp64_peak, "measured FP64 peak (max of DFMA and DMMA loops, live)"
        achieved = batch * flops_per_tuple() / (statistics.median(kernel_ms) * 1e-3) / 1e12
        dtype = "f64"
    else:
        peak = peaks.get("bf16_tflops", 1900.0)
        peak_note = "of measured BF16 dense peak (MEASURED_PEAKS.json bf16_tflops)"
        s_used = args.slices or 3
        products = s_used * (s_used + 1) // 2
        achieved = (batch * flops_per_tuple() * products /
                    (statistics.median(kernel_ms) * 1e-3) / 1e12)
        dtype = "bf16x%d->f64" % s_used
    cpu = None if args.no_cpu_baseline else cpu_baseline(d, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": "synthetic (seeded, benchmark value distributions)",
        "config": {"workload": f"CCSD(T) triples No={NO} Nv={NV} seed {SEED}",
                   "form": args.form, "tuples_per_step": batch, "n_tuples": n,
                   "l2": "no flush: inputs 3.2 GB > 129 MB L2",
                   "time_to_ET_s": n * (ms / 1e3) / max(tuples_all, 1)},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": peak_note,
                     "kernel": "triples_fp64_kernel" if form_used == capi.FORM_FP64
                     else "triples_split_kernel"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 16,
                "note": "per step: context create, pinned H2D + re-layout of all inputs, "
                        "tuple batch, energies D2H"},
        "clocks": clk,
        "gpu_launches": launches,
    }
    print(json.dumps(line))
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

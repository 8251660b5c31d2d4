"""Generate ``cfg2_no24_nv240_s0_full.json``: E(T) of EVERY tuple of the
No=24 / Nv=240 / seed 0 system (2,332,640 tuples), from the oracle's C
restatement (DGEMM route, numpy's bundled OpenBLAS, all host threads).

The restatement is pinned to the reference's own build: it matches the
reference's per-tuple energies of the first 60 tuples of this very system
(``cfg2_no24_nv240_s0_prefix.json``) and every other golden fixture here to
<= 1.3e-13 relative (``tests/test_oracle_golden.py``).  Running the
reference build itself over the whole list is not feasible (it links loop
BLAS through the shims: ~1e14 FLOPs at a few GFLOP/s).

Recorded: the Atrip::run total from the exactly rounded sum of the
per-tuple energies (``math.fsum``, sign applied; no (cT) intermediates, so
ct_energy == energy), the same total summed in list order as atrip's
accumulation does, and the sum of every block of ``block`` consecutive
tuples (a checksum of checksums that locates a disagreement).

Usage (minutes on 8 cores; not part of the test run):
    python tests/golden/make_cfg2_full.py [threads]
"""
from __future__ import annotations

import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from atrip_gb300 import synth  # noqa: E402

NO, NV, SEED, BLOCK = 24, 240, 0, 16384


def main() -> None:
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    blas = oracle.register_numpy_openblas()
    d = synth.make_inputs(NO, NV, SEED, with_j=False)
    p = oracle.Problem(d)
    port = oracle.PreparedPort(p)
    n = synth.n_tuples(NV)
    e = np.zeros(n)
    t0 = time.time()
    step = 1 << 18
    for s in range(0, n, step):
        e[s:min(n, s + step)], _ = port.run(s, min(n, s + step), threads)
        print(f"{min(n, s + step)}/{n} tuples, {time.time() - t0:.0f} s", flush=True)
    port.close()
    secs = time.time() - t0
    exact = math.fsum(e.tolist())
    blocks = [math.fsum(e[s:s + BLOCK].tolist()) for s in range(0, n, BLOCK)]
    fx = {
        "generator": "atrip_gb300.synth.make_inputs",
        "checker": "oracle port (DGEMM route), pinned to the reference build",
        "blas": os.path.basename(blas) if blas else "loops",
        "No": NO, "Nv": NV, "seed": SEED, "with_j": False, "ijkabc": False,
        "n_tuples": n,
        "energy": -exact,
        "ct_energy": -exact,
        "energy_sequential_sum": oracle.total(e),
        "sum_e_fsum": exact,
        "block": BLOCK,
        "block_sums": blocks,
        "port_seconds": secs,
        "threads": threads,
    }
    with open(os.path.join(HERE, "cfg2_no24_nv240_s0_full.json"), "w") as f:
        json.dump(fx, f, indent=1)
    print("E(T)", fx["energy"], f"{secs:.0f} s")


if __name__ == "__main__":
    main()

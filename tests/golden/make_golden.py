"""Generate the golden fixtures in this directory from the atrip reference.

Runs the reference's OWN sources, compiled one-rank with the shims in
``oracle/`` (``make -C oracle ref``), on seeded synthetic inputs
(``atrip_gb300.synth``) and records:

* ``Atrip::run`` totals (energy, ct_energy) -- with GROUP_AND_SORT, because
  the NAIVE distribution throws in the slice bookkeeping at one rank;
* per-tuple energies from the reference's doubles_contribution /
  singles_contribution / get_energy_* called tuple by tuple;
* Tijk / Zijk of one tuple at a tiny size.

Both reference variants (DGEMM route and naive loops) are run and must agree
before a real-field fixture is written.  For the complex field (``z_``
cases, the reference's run<Complex>) the two routes differ by design -- the
naive loops skip the conjugation of V_hhhp that the DGEMM route applies
(src/atrip/Equations.cxx:599-632 vs :685-726) -- so the configure-default
DGEMM route is recorded and the naive variant's totals are kept beside it
for the record.  The inputs are NOT stored: tests regenerate them from
(No, Nv, seed, with_j, field, eps_imag).

Usage (needs the reference tree, given as the first argument or in the
ATRIP_REFERENCE environment variable; not part of the test run):
    python tests/golden/make_golden.py [/path/to/reference] [name-prefix]
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from atrip_gb300 import synth  # noqa: E402

# (name, No, Nv, seed, with_j, ijkabc, max_iterations, per_tuple, dump_tuple)
CASES = [
    ("cfg1_no8_nv40_s0", 8, 40, 0, False, False, 0, 400, None),
    ("cfg1_no8_nv40_s0_ijkabc", 8, 40, 0, False, True, 0, 0, None),
    ("cfg1_no8_nv40_s0_maxit", 8, 40, 0, False, False, 777, 0, None),
    ("cfg2_no24_nv240_s0_prefix", 24, 240, 0, False, False, 59, 60, None),
    ("tiny_no2_nv4_s1_j", 2, 4, 1, True, False, 0, 10 ** 6, None),
    ("tiny_no3_nv5_s1_j", 3, 5, 1, True, False, 0, 10 ** 6, None),
    ("tiny_no4_nv7_s1_j", 4, 7, 1, True, False, 0, 10 ** 6, 11),
    ("odd_no5_nv9_s3_j", 5, 9, 3, True, False, 0, 10 ** 6, 100),
    ("odd_no5_nv9_s3_j_ijkabc", 5, 9, 3, True, True, 0, 10 ** 6, None),
    ("edge_no1_nv3_s2", 1, 3, 2, False, False, 0, 10 ** 6, 0),
    ("edge_no3_nv2_s2_j", 3, 2, 2, True, False, 0, 10 ** 6, None),
    ("odd_no17_nv33_s5_j", 17, 33, 5, True, False, 0, 300, None),
    # complex field: (..., field, eps_imag)
    ("z_tiny_no3_nv5_s1_j", 3, 5, 1, True, False, 0, 10 ** 6, 7, "complex", 0.0),
    ("z_odd_no5_nv7_s2_j_epsim", 5, 7, 2, True, False, 0, 10 ** 6, None, "complex", 0.05),
    ("z_odd_no5_nv7_s2_j_ijkabc", 5, 7, 2, True, True, 0, 10 ** 6, None, "complex", 0.0),
    ("z_no6_nv11_s4_maxit", 6, 11, 4, False, False, 150, 151, None, "complex", 0.0),
    ("z_edge_no1_nv3_s2", 1, 3, 2, False, False, 0, 10 ** 6, 0, "complex", 0.0),
    ("z_no9_nv16_s6_j", 9, 16, 6, True, False, 0, 200, None, "complex", 0.0),
]


def dump(bin_dir: str, t: int):
    """Tijk, Zijk of tuple t; complex values as [re, im] pairs."""
    exe = oracle.reference_binary("dgemm")
    import subprocess
    out = subprocess.run([exe, bin_dir, "dump", str(t)], check=True, capture_output=True,
                         text=True).stdout

    def val(line):
        parts = [float(x) for x in line.split()[1:]]
        return parts[0] if len(parts) == 1 else parts
    T = [val(l) for l in out.splitlines() if l.startswith("TIJK")]
    Z = [val(l) for l in out.splitlines() if l.startswith("ZIJK")]
    return T, Z


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ATRIP_REFERENCE", "")
    prefix = sys.argv[2] if len(sys.argv) > 2 else ""
    if not oracle.build_reference(ref):
        raise SystemExit("reference tree not found: " + ref)
    for case in CASES:
        name, No, Nv, seed, with_j, ijkabc, maxit, per_tuple, dump_t = case[:9]
        field, eps_imag = case[9:] if len(case) > 9 else ("real", 0.0)
        if not name.startswith(prefix):
            continue
        d = synth.make_inputs(No, Nv, seed, with_j=with_j, field=field, eps_imag=eps_imag)
        with tempfile.TemporaryDirectory() as tmp:
            synth.write_bin_dir(d, tmp)
            e1, c1, secs = oracle.run_reference(tmp, "dgemm", maxit, ijkabc, True)
            e2, c2, _ = oracle.run_reference(tmp, "naive", maxit, ijkabc, True)
            if field == "real":
                for x, y in ((e1, e2), (c1, c2)):
                    assert abs(x - y) <= 1e-12 * abs(x) + 1e-14, (name, x, y)
            fx = {
                "generator": "atrip_gb300.synth.make_inputs",
                "No": No, "Nv": Nv, "seed": seed, "with_j": with_j, "ijkabc": ijkabc,
                "field": field, "eps_imag": eps_imag,
                "max_iterations": maxit,
                "n_tuples": synth.n_tuples(Nv),
                "energy": e1, "ct_energy": c1,
                "energy_naive_variant": e2, "ct_energy_naive_variant": c2,
                "reference_seconds_one_core": secs,
            }
            if per_tuple:
                abc, e, ect = oracle.reference_tuples(tmp, per_tuple, ijkabc, True)
                fx["tuples"] = {"abc": abc.tolist(), "e": e.tolist(), "ect": ect.tolist()}
            if dump_t is not None:
                T, Z = dump(tmp, dump_t)
                fx["dump"] = {"t": dump_t, "Tijk": T, "Zijk": Z}
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(fx, f, indent=1)
        print(name, e1, c1, f"{secs:.2f}s")


if __name__ == "__main__":
    main()

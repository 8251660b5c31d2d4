"""Reference model of the split-precision arithmetic, for the tests.

The split form writes each FP64 element as 2^(e-7) sum_p q_p 2^(-8p) with
integer digits |q_p| <= 128 (one power-of-two scale per tensor: 2^eT for T,
2^eV shared by V_pphp and V_hhhp), and keeps the digit products of level
p + q < S.  The FP16 form does the same with radix 2^11 (bits=11):
2^(e-10) sum_p q_p 2^(-11p), |q_p| <= 1024.  Because the doubles contribution is bilinear in (T, V), the kept
sum equals

    W_S = sum_{p < S} doubles(T_p, V_{< S-p}),

where T_p is the p-th digit component of T and V_{<m} the sum of the first
m components of V.  This module evaluates W_S with the CPU oracle's doubles
and energy routines (FP64 everywhere else), which is what the GPU kernel is
expected to reproduce up to FP32 rounding of the level >= 1 partial sums.
"""
from __future__ import annotations

import math

import numpy as np

import oracle


def exponent(maxabs: float) -> int:
    return 0 if maxabs <= 0 else math.frexp(maxabs)[1]  # maxabs < 2^e


def digit_components(x: np.ndarray, e: int, S: int, bits: int = 8):
    """[x_0, ..., x_{S-1}]: x_p = q_p 2^(e-(bits-1)-bits p)."""
    h = bits - 1
    y = np.ldexp(np.asarray(x, dtype=np.float64), h - e)
    out = []
    for p in range(S):
        q = np.rint(y)
        assert np.max(np.abs(q)) <= 2 ** h
        out.append(np.ldexp(q, e - h - bits * p))
        y = (y - q) * 2.0 ** bits
    return out


def _problems(d, Tc, Pc, Hc, S, pkey, hkey):
    out = []
    for p in range(S):
        m = S - p
        dd = dict(d)
        dd["Tabij"] = np.asfortranarray(Tc[p])
        dd["Vabci"] = np.asfortranarray(sum(Pc[:m]))
        dd["Vijka"] = np.asfortranarray(sum(Hc[:m]))
        out.append(oracle.Problem(dd))
    return out


def split_tuple_energies(d: dict, S: int, t0: int = 0, t1: int | None = None,
                         use_j: bool = False, bits: int = 8):
    """Per-tuple energies of the split form's arithmetic with S slices of
    radix 2^bits (8: BF16 form, 11: FP16 form); with use_j also the (cT)
    energies (T from the J intermediates, Z from V), returned as (e, ect)."""
    No, Nv = d["No"], d["Nv"]
    eT = exponent(float(np.max(np.abs(d["Tabij"]))))
    eV = exponent(max(float(np.max(np.abs(d["Vabci"]))), float(np.max(np.abs(d["Vijka"])))))
    Tc = digit_components(d["Tabij"], eT, S, bits)
    problems = _problems(d, Tc, digit_components(d["Vabci"], eV, S, bits),
                         digit_components(d["Vijka"], eV, S, bits), S, "Vabci", "Vijka")
    jproblems = []
    if use_j:
        eJ = exponent(max(float(np.max(np.abs(d["Jabci"]))), float(np.max(np.abs(d["Jijka"])))))
        jproblems = _problems(d, Tc, digit_components(d["Jabci"], eJ, S, bits),
                              digit_components(d["Jijka"], eJ, S, bits), S, "Jabci", "Jijka")
    full = oracle.Problem(d)
    lst = oracle.tuple_list(Nv)
    t1 = len(lst) if t1 is None else t1
    lib = oracle._load()
    out = np.zeros(t1 - t0)
    out_ct = np.zeros(t1 - t0)
    eps = np.ascontiguousarray(d["epsi"], dtype=np.float64)
    for n, t in enumerate(range(t0, t1)):
        a, b, c = (int(v) for v in lst[t])
        W = np.zeros(No ** 3)
        for pr in problems:
            W += oracle.tuple_arrays(pr, a, b, c)[0]
        # Z = W + singles, from the full-precision problem
        T_full, Z_full = oracle.tuple_arrays(full, a, b, c)
        Z = W + (Z_full - T_full)
        epsabc = d["epsa"][a] + d["epsa"][b] + d["epsa"][c]
        fn = lib.oracle_energy_distinct if (a != b and b != c) else lib.oracle_energy_same
        out[n] = fn(float(epsabc), No, eps.ctypes.data, W.ctypes.data, Z.ctypes.data)
        if use_j:
            WJ = np.zeros(No ** 3)
            for pr in jproblems:
                WJ += oracle.tuple_arrays(pr, a, b, c)[0]
            out_ct[n] = fn(float(epsabc), No, eps.ctypes.data, WJ.ctypes.data, Z.ctypes.data)
    return (out, out_ct) if use_j else out

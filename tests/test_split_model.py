"""CPU checks of the split-precision digit model (no GPU): digit bounds,
exact reconstruction, and the truncation error of each slice format against
the FP64 oracle, which sets the bars the GPU split tests use."""
import numpy as np
import pytest

import oracle
import split_model
from atrip_gb300 import synth


@pytest.mark.parametrize("bits", [8, 11])
def test_digits_bounded_and_exact(bits):
    rng = np.random.default_rng(bits)
    x = rng.standard_normal(4096) * np.exp(rng.uniform(-20, 0, 4096))
    e = split_model.exponent(float(np.max(np.abs(x))))
    comps = split_model.digit_components(x, e, 8, bits)  # asserts |q| <= 2^(bits-1)
    # 8 digits carry at least 64 bits: the sum reproduces x to FP64 rounding
    assert np.max(np.abs(sum(comps) - x)) <= 4 * np.finfo(float).eps * np.max(np.abs(x))
    # digit p carries radix^-p of the scale: the partial sums converge
    for S in range(1, 4):
        err = np.max(np.abs(sum(comps[:S]) - x))
        assert err <= 2.0 ** (e - (bits - 1) - bits * (S - 1) - 1), (S, err)


@pytest.mark.parametrize("S,bits,bound", [(2, 8, 1e-4), (3, 8, 1e-6), (2, 11, 5e-6)])
def test_model_truncation_error(S, bits, bound):
    for No, Nv, seed in [(8, 40, 0), (13, 17, 2)]:
        d = synth.make_inputs(No, Nv, seed)
        n = 60
        e = split_model.split_tuple_energies(d, S, 0, n, bits=bits)
        e64, _ = oracle.tuple_energies(oracle.Problem(d), 0, n, use_j=False)
        rel = np.max(np.abs(e - e64)) / np.max(np.abs(e64))
        assert rel <= bound, (No, Nv, rel)


def test_newton_reciprocal_bound():
    """The split kernel's energy denominators use 1/d = x0 + x0 (1 - d x0)
    with x0 the correctly rounded FP32 reciprocal of d truncated to FP32:
    emulated here (the truncation on the bit patterns, numpy float32
    division rounds to nearest like the FP32 reciprocal instruction), the
    relative error stays below 2^-44 over the range of orbital-energy gaps
    and beyond."""
    rng = np.random.default_rng(7)
    d = np.concatenate([np.exp(rng.uniform(np.log(1e-6), np.log(1e6), 200000)),
                        -np.exp(rng.uniform(np.log(1e-3), np.log(1e3), 1000)),
                        1.0 + np.arange(1, 4000) * 2.0 ** -40])  # just above powers of two
    b = d.view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7ff)).astype(np.int64) - 1023
    fb = (((b >> np.uint64(32)) & np.uint64(0x80000000)) |
          (((e + 127).astype(np.uint64)) << np.uint64(23)) |
          ((b >> np.uint64(29)) & np.uint64(0x7fffff))).astype(np.uint32)
    d32 = fb.view(np.float32)
    assert np.all(np.abs(d32.astype(np.float64) - d) <= np.abs(d) * 2.0 ** -23)
    x0 = (np.float32(1.0) / d32).astype(np.float64)
    e = 1.0 - d * x0  # the kernel forms this with one FMA
    x1 = x0 + x0 * e
    rel = np.abs(x1 * d - 1.0)
    assert np.max(rel) <= 2.0 ** -44, np.max(rel)


@pytest.mark.parametrize("S,bits,bound", [(3, 8, 1e-6), (2, 11, 5e-6)])
def test_model_ct_truncation_error(S, bits, bound):
    """(cT) energies of the digit model (T from the J intermediates) within
    the same per-tuple bounds against the FP64 oracle."""
    d = synth.make_inputs(8, 20, 1, with_j=True)
    n = 60
    _, ect = split_model.split_tuple_energies(d, S, 0, n, use_j=True, bits=bits)
    e64, ect64 = oracle.tuple_energies(oracle.Problem(d), 0, n, use_j=True)
    rel = np.max(np.abs(ect - ect64)) / np.max(np.abs(e64))
    assert rel <= bound, rel

"""GPU parity of the split-precision form (BF16 digit slices on tcgen05).

Two references:
* the split model (tests/split_model.py): the same truncated digit products
  evaluated in FP64 by the CPU oracle -- the kernel must reproduce it up to
  FP32 rounding of the level >= 1 partial sums (tolerance 1e-7 relative per
  tuple, far below the split truncation error it would expose);
* the FP64 form: the error of the split form itself, bounded per slice count
  (S=2: 1e-4, S=3: 1e-6, S=4: 1e-8 relative per tuple), and the benchmark's
  |dE(T)| <= 1e-8 Eh on a power-of-two-scaled twin with |E(T)| ~ 0.1 Eh.

The FP16 form (2 slices of 11-bit digits) rounds its level-0 sums in FP32
(products up to 2^20 do not stay exact), so its bar against the model is
the FP32 rounding of level 0: 3e-6 relative per tuple; against the FP64
form 5e-6 (its digit truncation alone gives ~1e-6).
"""
import numpy as np
import pytest

import oracle
import split_model
from atrip_gb300 import autotune, capi, synth

pytestmark = pytest.mark.gpu
BOUND = {2: 1e-4, 3: 1e-6, 4: 1e-8}


def _ctx(d):
    ctx = capi.Context(d["No"], d["Nv"], 0)
    for n in ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci"):
        ctx.upload(n, d[n])
    return ctx


CASES = [(6, 10, 1), (8, 40, 0), (5, 9, 3), (13, 17, 2), (24, 30, 4), (30, 14, 5), (1, 6, 7),
         (64, 6, 8), (17, 70, 9)]


@pytest.mark.parametrize("No,Nv,seed", CASES)
@pytest.mark.parametrize("S", [2, 3, 4])
@pytest.mark.parametrize("variant", [1, 2, 3])
def test_split_matches_model_and_fp64(No, Nv, seed, S, variant):
    """variant 2 = the transposed kernel (stacked slices as the MMA's M rows)
    where S No <= 128, elsewhere variant 1; variant 3 = variant 2 with one
    stack load per K chunk shared by the slice units where No % 8 == 0,
    elsewhere variant 2."""
    d = synth.make_inputs(No, Nv, seed)
    n = min(synth.n_tuples(Nv), 120)
    model = split_model.split_tuple_energies(d, S, 0, n)
    with _ctx(d) as ctx:
        r64 = ctx.run(form="fp64", use_j=False, max_iterations=n - 1)
        e64, _ = ctx.tuple_energies(0, n)
        ctx.set_tuning(split_variant=variant)
        r = ctx.run(form="split_bf16", slices=S, use_j=False, max_iterations=n - 1)
        assert r.form_used == capi.FORM_SPLIT_BF16 and r.slices_used == S
        e, ect = ctx.tuple_energies(0, n)
    assert np.array_equal(e, ect)
    if No == 1:
        # one occupied orbital: every tuple energy cancels to rounding noise
        assert np.max(np.abs(e)) <= 1e-12 and np.max(np.abs(e64)) <= 1e-12
        return
    scale = np.max(np.abs(model))
    assert np.max(np.abs(e - model)) <= 1e-7 * scale + 1e-14, np.max(np.abs(e - model)) / scale
    rel = np.max(np.abs(e - e64)) / np.max(np.abs(e64))
    assert rel <= BOUND[S], rel
    assert abs(r.energy - r64.energy) <= BOUND[S] * abs(r64.energy)


def test_split_scaled_twin_meets_1e8_hartree():
    """No=8, Nv=40 with t1, t2 and all integrals scaled by 2^-k so that
    |E(T)| ~ 0.1 Eh: |E_split - E_fp64| <= 1e-8 Eh with 3 slices."""
    d0 = synth.make_inputs(8, 40, 0)
    with _ctx(d0) as ctx:
        e0 = ctx.run(form="fp64", use_j=False).energy
    k = int(round(np.log2(abs(e0) / 0.1) / 4))
    d = synth.make_inputs(8, 40, 0, scale=2.0 ** -k)
    with _ctx(d) as ctx:
        e64 = ctx.run(form="fp64", use_j=False).energy
        e3 = ctx.run(form="split_bf16", slices=3, use_j=False).energy
    assert 0.01 < abs(e64) < 1.0
    assert abs(e64 * 2.0 ** (4 * k) - e0) <= 1e-12 * abs(e0)  # power-of-two scaling is exact
    assert abs(e3 - e64) <= 1e-8, abs(e3 - e64)


@pytest.mark.parametrize("No,Nv,seed", [(5, 9, 3), (8, 20, 1), (24, 14, 2), (30, 12, 6)])
def test_split_ct_energy(No, Nv, seed):
    """(cT): the J pass reproduces the model and stays within the 3-slice
    bound of the FP64 form's ct_energy."""
    d = synth.make_inputs(No, Nv, seed, with_j=True)
    n = min(synth.n_tuples(Nv), 80)
    model_e, model_ct = split_model.split_tuple_energies(d, 3, 0, n, use_j=True)
    with _ctx(d) as ctx:
        ctx.upload("Jijka", d["Jijka"])
        ctx.upload("Jabci", d["Jabci"])
        r64 = ctx.run(form="fp64", use_j=True, max_iterations=n - 1)
        e64, ect64 = ctx.tuple_energies(0, n)
        r = ctx.run(form="split_bf16", slices=3, use_j=True, max_iterations=n - 1)
        e, ect = ctx.tuple_energies(0, n)
        # the same context still runs without the J pass afterwards
        r2 = ctx.run(form="split_bf16", slices=3, use_j=False, max_iterations=n - 1)
    scale = np.max(np.abs(model_e))
    assert np.max(np.abs(e - model_e)) <= 1e-7 * scale
    assert np.max(np.abs(ect - model_ct)) <= 1e-7 * scale
    assert np.max(np.abs(ect - ect64)) <= BOUND[3] * np.max(np.abs(e64))
    assert abs(r.ct_energy - r64.ct_energy) <= BOUND[3] * abs(r64.energy)
    assert r2.energy == r.energy and r2.ct_energy == r2.energy


def test_split_rejects_bad_slices():
    d = synth.make_inputs(4, 7, 1)
    with _ctx(d) as ctx:
        with pytest.raises(capi.AtripError) as ei:
            ctx.run(form="split_bf16", slices=5, use_j=False)
        assert ei.value.status == capi.ERR_ARGUMENT
        # the FP64 form still works on the same context
        assert np.isfinite(ctx.run(form="fp64").energy)


@pytest.mark.parametrize("No,Nv,seed", [(6, 10, 1), (24, 30, 4), (17, 70, 9), (1, 6, 7)])
def test_split_w_global_and_ring_depth_do_not_change_results(No, Nv, seed):
    """The autotuner's split knobs (ring depth, W read from L2 instead of
    its shared-memory copy) change the schedule, not the arithmetic: the
    per-tuple energies stay the same to FP32-reassociation level."""
    d = synth.make_inputs(No, Nv, seed, with_j=True)
    d_noj = {k: v for k, v in d.items() if k not in ("Jijka", "Jabci")}
    n = min(synth.n_tuples(Nv), 300)
    with _ctx(d_noj) as ctx:
        ref = ctx.run(form="split_bf16", slices=3, max_iterations=n - 1)
        e_ref, _ = ctx.tuple_energies(0, n)
        for tune in ({"split_w_global": 1}, {"split_w_global": 1, "split_stages": 2},
                     {"split_stages": 3}):
            ctx.set_tuning(**tune)
            r = ctx.run(form="split_bf16", slices=3, max_iterations=n - 1)
            e, _ = ctx.tuple_energies(0, n)
            s = np.max(np.abs(e_ref))
            assert np.max(np.abs(e - e_ref)) <= 1e-12 * s, tune
            assert abs(r.energy - ref.energy) <= 1e-12 * abs(ref.energy), tune


def test_split_level0_split_accumulator_large_k():
    """K = 2 (Nv + No) > 1024 (the No=56/Nv=560 workload's regime): level 0
    of the transposed half gets its own exact accumulator.  The error
    against the FP64 form shrinks with the slice count as the truncation
    does (a wrong accumulator would not): at K ~ 1000 the per-tuple bound
    is 1e-5 for 3 slices and 1e-7 for 4."""
    No, Nv = 3, 515
    d = synth.make_inputs(No, Nv, 11)
    n = 256
    err = {}
    with _ctx(d) as ctx:
        ctx.run(form="fp64", max_iterations=n - 1)
        e64, _ = ctx.tuple_energies(0, n)
        scale = np.max(np.abs(e64))
        for S in (3, 4):
            ctx.run(form="split_bf16", slices=S, max_iterations=n - 1)
            es, _ = ctx.tuple_energies(0, n)
            err[S] = np.max(np.abs(es - e64)) / scale
    assert err[3] <= 1e-5 and err[4] <= 1e-7, err
    assert err[4] < err[3] / 20, err


@pytest.mark.parametrize("No,Nv,seed,S", [(5, 9, 3, 3), (24, 30, 4, 3), (40, 12, 2, 3),
                                          (32, 20, 6, 4), (64, 7, 1, 2), (13, 17, 2, 2)])
def test_transposed_variant_with_j_and_knobs(No, Nv, seed, S):
    """The transposed kernel gives the same per-tuple E(T) and E(cT) as the
    M-tile kernel up to FP32 reassociation of the level >= 1 sums, with the
    (cT) pass, W in L2 or shared memory and a shallow ring."""
    d = synth.make_inputs(No, Nv, seed, with_j=True)
    n = min(synth.n_tuples(Nv), 400)
    with _ctx(d) as ctx:
        for name in ("Jijka", "Jabci"):
            ctx.upload(name, d[name])
        ctx.set_tuning(split_variant=1)
        ctx.run(form="split_bf16", slices=S, use_j=True, max_iterations=n - 1)
        e1, c1 = ctx.tuple_energies(0, n)
        for tune in ({"split_variant": 2}, {"split_variant": 2, "split_w_global": 1},
                     {"split_variant": 2, "split_stages": 2, "tuple_block": 4},
                     {"split_variant": 2, "split_prefetch": 1},
                     {"split_variant": 1, "split_prefetch": 1},
                     {"split_variant": 3}, {"split_variant": 3, "tuple_block": 4}):
            ctx.set_tuning(**tune)
            ctx.run(form="split_bf16", slices=S, use_j=True, max_iterations=n - 1)
            e2, c2 = ctx.tuple_energies(0, n)
            s = np.max(np.abs(e1))
            assert np.max(np.abs(e2 - e1)) <= 1e-9 * s, (tune, np.max(np.abs(e2 - e1)) / s)
            assert np.max(np.abs(c2 - c1)) <= 1e-9 * s, tune


F16_MODEL_TOL, F16_BOUND = 3e-6, 5e-6


@pytest.mark.parametrize("No,Nv,seed", CASES)
@pytest.mark.parametrize("variant", [2, 3])
def test_f16_matches_model_and_fp64(No, Nv, seed, variant):
    d = synth.make_inputs(No, Nv, seed)
    n = min(synth.n_tuples(Nv), 120)
    if not autotune.f16_eligible(No, Nv):
        with _ctx(d) as ctx, pytest.raises(capi.AtripError) as ei:
            ctx.run(form="split_f16", use_j=False, max_iterations=n - 1)
        assert ei.value.status == capi.ERR_UNSUPPORTED
        return
    model = split_model.split_tuple_energies(d, 2, 0, n, bits=11)
    with _ctx(d) as ctx:
        r64 = ctx.run(form="fp64", use_j=False, max_iterations=n - 1)
        e64, _ = ctx.tuple_energies(0, n)
        ctx.set_tuning(split_variant=variant)
        r = ctx.run(form="split_f16", use_j=False, max_iterations=n - 1)
        assert r.form_used == capi.FORM_SPLIT_F16 and r.slices_used == 2
        e, ect = ctx.tuple_energies(0, n)
    assert np.array_equal(e, ect)
    if No == 1:
        assert np.max(np.abs(e)) <= 1e-12
        return
    scale = np.max(np.abs(model))
    assert np.max(np.abs(e - model)) <= F16_MODEL_TOL * scale, np.max(np.abs(e - model)) / scale
    rel = np.max(np.abs(e - e64)) / np.max(np.abs(e64))
    assert rel <= F16_BOUND, rel
    assert abs(r.energy - r64.energy) <= F16_BOUND * abs(r64.energy)


def test_f16_scaled_twin_meets_1e8_hartree():
    d0 = synth.make_inputs(8, 40, 0)
    with _ctx(d0) as ctx:
        e0 = ctx.run(form="fp64", use_j=False).energy
    k = int(round(np.log2(abs(e0) / 0.1) / 4))
    d = synth.make_inputs(8, 40, 0, scale=2.0 ** -k)
    with _ctx(d) as ctx:
        e64 = ctx.run(form="fp64", use_j=False).energy
        e2 = ctx.run(form="split_f16", use_j=False).energy
    assert 0.01 < abs(e64) < 1.0
    assert abs(e2 - e64) <= 1e-8, abs(e2 - e64)


@pytest.mark.parametrize("No,Nv,seed", [(5, 9, 3), (8, 20, 1), (24, 14, 2), (32, 12, 6)])
def test_f16_ct_energy_and_knobs(No, Nv, seed):
    """(cT) pass against the model; ring depth, W placement, variant 3 and
    the blocked order change the schedule only (1e-9 relative)."""
    d = synth.make_inputs(No, Nv, seed, with_j=True)
    n = min(synth.n_tuples(Nv), 80)
    model_e, model_ct = split_model.split_tuple_energies(d, 2, 0, n, use_j=True, bits=11)
    with _ctx(d) as ctx:
        ctx.upload("Jijka", d["Jijka"])
        ctx.upload("Jabci", d["Jabci"])
        r64 = ctx.run(form="fp64", use_j=True, max_iterations=n - 1)
        ctx.run(form="split_f16", use_j=True, max_iterations=n - 1)
        e, ect = ctx.tuple_energies(0, n)
        scale = np.max(np.abs(model_e))
        assert np.max(np.abs(e - model_e)) <= F16_MODEL_TOL * scale
        assert np.max(np.abs(ect - model_ct)) <= F16_MODEL_TOL * scale
        for tune in ({"split_variant": 3}, {"split_w_global": 1}, {"split_stages": 2},
                     {"split_variant": 3, "tuple_block": 4}, {"split_prefetch": 1}):
            ctx.set_tuning(**tune)
            r = ctx.run(form="split_f16", use_j=True, max_iterations=n - 1)
            e2, c2 = ctx.tuple_energies(0, n)
            assert np.max(np.abs(e2 - e)) <= 1e-9 * scale, tune
            assert np.max(np.abs(c2 - ect)) <= 1e-9 * scale, tune
        assert abs(r.ct_energy - r64.ct_energy) <= F16_BOUND * abs(r64.energy)
        # switching back to BF16 slices re-cuts the operands
        ctx.set_tuning(split_variant=2)
        rb = ctx.run(form="split_bf16", slices=3, use_j=True, max_iterations=n - 1)
        assert rb.form_used == capi.FORM_SPLIT_BF16
        assert abs(rb.energy - r64.energy) <= BOUND[3] * abs(r64.energy)


def test_f16_large_k():
    """K = 2 (Nv + No) = 1036 > 1024: beyond the BF16 transposed kernel,
    within the FP16 one (level 0 < 2^31)."""
    No, Nv = 3, 515
    d = synth.make_inputs(No, Nv, 11)
    n = 256
    with _ctx(d) as ctx:
        ctx.run(form="fp64", max_iterations=n - 1)
        e64, _ = ctx.tuple_energies(0, n)
        ctx.run(form="split_f16", max_iterations=n - 1)
        e, _ = ctx.tuple_energies(0, n)
    assert np.max(np.abs(e - e64)) / np.max(np.abs(e64)) <= 1e-5


def test_f16_rejects_what_it_does_not_cover():
    d = synth.make_inputs(4, 7, 1)
    with _ctx(d) as ctx:
        with pytest.raises(capi.AtripError) as ei:
            ctx.run(form="split_f16", slices=3)
        assert ei.value.status == capi.ERR_ARGUMENT
        assert np.isfinite(ctx.run(form="split_f16").energy)
    # No = 64 (the largest context): two slices of 64 rows fill the 128 M rows
    d = synth.make_inputs(64, 4, 2)
    with _ctx(d) as ctx:
        e64 = ctx.run(form="fp64", use_j=False).energy
        e16 = ctx.run(form="split_f16", use_j=False).energy
        assert abs(e16 - e64) <= F16_BOUND * abs(e64)

"""The split kernel's role profile (tuning split_profile = 1,
atrip_gpu_split_profile): the profiled kernel gives the same per-tuple
energies as the plain one, and its counters add up -- every tuple counted
once, the ring stages per tuple of the transposed kernel's schedule
(3 groups x N tiles x (2 particle parts x K chunks + 2 hole parts) x 2
slice units), every wait within its role's lifetime."""
import numpy as np
import pytest

from atrip_gb300 import capi, synth

pytestmark = pytest.mark.gpu
NAMES = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci")


@pytest.mark.parametrize("form,No,Nv", [("split_f16", 24, 70), ("split_bf16", 13, 40),
                                        ("split_f16", 8, 150)])
def test_profiled_run_matches_and_counts(form, No, Nv):
    d = synth.make_inputs(No, Nv, 4)
    with capi.Context(No, Nv, 0) as ctx:
        for n in NAMES:
            ctx.upload(n, d[n])
        ctx.set_tuning(split_variant=2)
        ref = ctx.run(form=form, slices=2, use_j=False)
        e0, _ = ctx.tuple_energies(0, ref.tuples_done)
        e0 = e0.copy()
        ctx.set_tuning(split_variant=2, split_profile=1)
        r = ctx.run(form=form, slices=2, use_j=False)
        e1, _ = ctx.tuple_energies(0, r.tuples_done)
        assert np.array_equal(e0, e1)
        assert r.energy == ref.energy
        p = ctx.split_profile()
    n = synth.n_tuples(Nv)
    assert p["tuples"] == n
    assert 1 <= p["ctas"] <= n
    jt = 256 // No
    ntiles = -(-No // jt)
    kch = -(-Nv // 64)
    assert p["stages"] == n * 3 * ntiles * (2 * kch + 2) * 2
    waits = {"producer": ("stage", "tuple_slot"), "mma": ("tuple", "accumulator", "stage"),
             "epilogue": ("tuple", "w_buffer", "accumulator"), "energy": ("tuple", "w")}
    for role, ws in waits.items():
        total = p[f"{role}_total"]
        assert total > 0, role
        assert sum(p[f"{role}_wait_{w}"] for w in ws) <= total, role
    assert p["energy_w_convert"] <= p["energy_total"]


def test_profile_needs_the_transposed_two_slice_kernel():
    d = synth.make_inputs(6, 11, 3)
    with capi.Context(6, 11, 0) as ctx:
        for n in NAMES:
            ctx.upload(n, d[n])
        with pytest.raises(capi.AtripError) as err:
            ctx.split_profile()  # no profiled run yet
        assert err.value.status == capi.ERR_STATE
        ctx.set_tuning(split_variant=0, split_profile=1)
        with pytest.raises(capi.AtripError) as err:
            ctx.run(form="split_bf16", slices=3, use_j=False)
        assert err.value.status == capi.ERR_UNSUPPORTED
        ctx.set_tuning(split_variant=2)
        ctx.run(form="split_bf16", slices=3, use_j=False)  # plain kernel again
        with pytest.raises(capi.AtripError):
            ctx.set_tuning(split_profile=2)

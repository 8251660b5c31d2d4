"""GPU parity of the complex field (atrip's run<Complex>, FP64 form)
against the reference's own Complex build (golden fixtures) and the C
restatement of it, through the C ABI.

Tolerance: 1e-10 relative on E(T) and per tuple, the FP64 form's bar.
"""
import numpy as np
import pytest

import oracle
from atrip_gb300 import capi, synth
from conftest import golden_inputs, golden_names, load_golden

pytestmark = pytest.mark.gpu
REL = 1e-10
NAMES = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci")


def _ctx_for(d):
    ctx = capi.Context(d["No"], d["Nv"], 0, field="complex")
    for name in NAMES:
        if name in d:
            ctx.upload(name, d[name])
    return ctx


@pytest.mark.parametrize("name", [n for n in golden_names() if n.startswith("z_")])
def test_complex_matches_reference_fixture(name):
    fx = load_golden(name)
    d = golden_inputs(fx)
    with _ctx_for(d) as ctx:
        r = ctx.run(form="fp64", ijkabc=fx["ijkabc"], use_j=True,
                    max_iterations=fx["max_iterations"])
        scale = abs(fx["energy"])
        assert abs(r.energy - fx["energy"]) <= REL * scale + 1e-14, (r.energy, fx["energy"])
        assert abs(r.ct_energy - fx["ct_energy"]) <= REL * scale + 1e-14
        if "tuples" in fx:
            n = min(len(fx["tuples"]["e"]), r.tuples_done)
            e, ect = ctx.tuple_energies(0, n)
            ref = np.array(fx["tuples"]["e"][:n])
            s = np.max(np.abs(ref)) + 1e-300
            assert np.max(np.abs(e - ref)) <= REL * s + 1e-14
            assert np.max(np.abs(ect - np.array(fx["tuples"]["ect"][:n]))) <= REL * s + 1e-14


@pytest.mark.parametrize("No,Nv,seed,eps_imag", [(16, 24, 3, 0.02), (9, 13, 5, 0.0),
                                                 (33, 10, 7, 0.0)])
def test_complex_per_tuple_matches_oracle(No, Nv, seed, eps_imag):
    d = synth.make_inputs(No, Nv, seed, with_j=True, field="complex", eps_imag=eps_imag)
    p = oracle.Problem(d)
    n = min(synth.n_tuples(Nv), 600)
    e_ref, ect_ref = oracle.tuple_energies(p, 0, n, threads=8)
    with _ctx_for(d) as ctx:
        r = ctx.run(form="fp64", max_iterations=n - 1)
        e, ect = ctx.tuple_energies(0, n)
    s = np.max(np.abs(e_ref))
    assert np.max(np.abs(e - e_ref)) <= REL * s
    assert np.max(np.abs(ect - ect_ref)) <= REL * s
    assert abs(r.energy + np.sum(e_ref)) <= REL * abs(np.sum(e_ref))


def test_complex_rejects_the_split_form():
    d = synth.make_inputs(4, 6, 1, field="complex")
    with _ctx_for(d) as ctx:
        with pytest.raises(capi.AtripError) as ex:
            ctx.run(form="split_bf16")
        assert ex.value.status == capi.ERR_UNSUPPORTED
        r = ctx.run(form="auto")  # AUTO falls back to the FP64 form for complex
        assert r.form_used == capi.FORM_FP64

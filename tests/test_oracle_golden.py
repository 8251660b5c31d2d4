"""The C oracle restatement against fixtures produced by the atrip
reference's own sources (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle
from conftest import golden_inputs, golden_names, load_golden

REL = 1e-12


def _close(x, y, scale):
    return abs(x - y) <= REL * abs(scale) + 1e-14


@pytest.mark.parametrize("name", golden_names())
def test_oracle_total_matches_reference(name):
    fx = load_golden(name)
    if fx["Nv"] >= 200 and fx["max_iterations"] == 0:
        pytest.skip("full run too long for the CPU suite")
    p = oracle.Problem(golden_inputs(fx))
    e, ect = oracle.run(p, ijkabc=fx["ijkabc"], use_j=True, threads=4,
                        max_iterations=fx["max_iterations"])
    assert _close(e, fx["energy"], fx["energy"]), (e, fx["energy"])
    assert _close(ect, fx["ct_energy"], fx["energy"]), (ect, fx["ct_energy"])


@pytest.mark.parametrize("name", [n for n in golden_names() if "tuples" in load_golden(n)])
@pytest.mark.parametrize("route", ["naive", "port"])
def test_oracle_per_tuple_matches_reference(name, route):
    fx = load_golden(name)
    tup = fx["tuples"]
    n = len(tup["e"])
    p = oracle.Problem(golden_inputs(fx))
    assert (oracle.tuple_list(fx["Nv"])[:n] == np.array(tup["abc"], dtype=np.int32)).all()
    e, ect = oracle.tuple_energies(p, 0, n, ijkabc=fx["ijkabc"], use_j=True, route=route,
                                   threads=4)
    scale = np.max(np.abs(tup["e"])) + 1e-300
    assert np.max(np.abs(e - tup["e"])) <= REL * scale + 1e-14
    assert np.max(np.abs(ect - tup["ect"])) <= REL * scale + 1e-14


@pytest.mark.parametrize("name", [n for n in golden_names() if "dump" in load_golden(n)])
def test_oracle_tuple_arrays_match_reference(name):
    fx = load_golden(name)
    p = oracle.Problem(golden_inputs(fx))
    t = fx["dump"]["t"]
    a, b, c = oracle.tuple_list(fx["Nv"])[t]
    T, Z = oracle.tuple_arrays(p, a, b, c)

    def ref(v):
        v = np.array(v)
        return v[:, 0] + 1j * v[:, 1] if v.ndim == 2 else v  # complex: [re, im] pairs
    np.testing.assert_allclose(T, ref(fx["dump"]["Tijk"]), rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(Z, ref(fx["dump"]["Zijk"]), rtol=1e-12, atol=1e-15)


def test_tuple_count_and_order():
    for nv in (1, 2, 3, 7, 40):
        lst = oracle.tuple_list(nv)
        assert len(lst) == nv * (nv + 1) * (nv + 2) // 6 - nv
        if len(lst):
            assert (lst[:, 0] <= lst[:, 1]).all() and (lst[:, 1] <= lst[:, 2]).all()
            assert not ((lst[:, 0] == lst[:, 1]) & (lst[:, 1] == lst[:, 2])).any()
            keys = lst[:, 0] * nv * nv + lst[:, 1] * nv + lst[:, 2]
            assert (np.diff(keys) > 0).all()


def test_naive_and_port_routes_agree_with_j():
    from atrip_gb300 import synth
    p = oracle.Problem(synth.make_inputs(6, 11, 7, with_j=True))
    a = oracle.run(p, route="naive", threads=2)
    b = oracle.run(p, route="port", threads=3)
    assert _close(a[0], b[0], a[0]) and _close(a[1], b[1], a[0])


def test_complex_field_is_not_the_real_one():
    """The complex fixtures exercise the conjugations: dropping the imaginary
    parts changes the energies, and the reference's two routes (DGEMM with
    the hole conjugation, naive loops without) disagree for complex input."""
    fx = load_golden("z_odd_no5_nv7_s2_j_epsim")
    d = golden_inputs(fx)
    real = {k: (np.real(v) if isinstance(v, np.ndarray) else v) for k, v in d.items()}
    e_real, _ = oracle.run(oracle.Problem(real), use_j=True)
    assert abs(e_real - fx["energy"]) > 1e-6 * abs(fx["energy"])
    assert abs(fx["energy_naive_variant"] - fx["energy"]) > 1e-9 * abs(fx["energy"])

"""GPU parity: the CUDA triples path (through the C ABI) against the atrip
reference's golden fixtures and the CPU oracle, on the same seeded inputs.

Tolerance for the FP64 form: 1e-10 relative on E(T), the bar of the
benchmark definition (plus 1e-14 absolute for energies that cancel to ~0).
"""
import numpy as np
import pytest

import oracle
from atrip_gb300 import capi, synth
from conftest import golden_inputs, golden_names, load_golden

pytestmark = pytest.mark.gpu
REL = 1e-10


def _ctx_for(d):
    ctx = capi.Context(d["No"], d["Nv"], 0)
    for name in ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci"):
        if name in d:
            ctx.upload(name, d[name])
    return ctx


def _close(x, y, scale=None):
    scale = abs(y) if scale is None else scale
    return abs(x - y) <= REL * scale + 1e-14


@pytest.mark.parametrize("name", [n for n in golden_names()
                                  if load_golden(n).get("field", "real") == "real" and
                                  (load_golden(n)["Nv"] < 200 or load_golden(n).get("max_iterations"))])
def test_fp64_matches_reference_fixture(name):
    fx = load_golden(name)
    d = golden_inputs(fx)
    with _ctx_for(d) as ctx:
        r = ctx.run(form="fp64", ijkabc=fx["ijkabc"], use_j=True,
                    max_iterations=fx["max_iterations"])
        assert _close(r.energy, fx["energy"]), (r.energy, fx["energy"])
        assert _close(r.ct_energy, fx["ct_energy"], abs(fx["energy"])), (r.ct_energy, fx["ct_energy"])
        if "tuples" in fx:
            n = min(len(fx["tuples"]["e"]), r.tuples_done)
            e, ect = ctx.tuple_energies(0, n)
            ref_e = np.array(fx["tuples"]["e"][:n])
            ref_ect = np.array(fx["tuples"]["ect"][:n])
            scale = np.max(np.abs(ref_e))
            assert np.max(np.abs(e - ref_e)) <= REL * scale + 1e-14
            assert np.max(np.abs(ect - ref_ect)) <= REL * scale + 1e-14


@pytest.mark.parametrize("No,Nv,seed,with_j", [(6, 13, 11, True), (9, 20, 4, False),
                                               (16, 24, 2, True), (24, 30, 0, False),
                                               (33, 17, 8, False), (64, 12, 9, False)])
def test_fp64_per_tuple_matches_oracle(No, Nv, seed, with_j):
    d = synth.make_inputs(No, Nv, seed, with_j=with_j)
    p = oracle.Problem(d)
    n = min(synth.n_tuples(Nv), 400)
    e_ref, ect_ref = oracle.tuple_energies(p, 0, n, route="port", threads=8)
    with _ctx_for(d) as ctx:
        r = ctx.run(form="fp64", max_iterations=n - 1)
        assert r.tuples_done == n
        e, ect = ctx.tuple_energies(0, n)
    scale = np.max(np.abs(e_ref))
    assert np.max(np.abs(e - e_ref)) <= REL * scale
    assert np.max(np.abs(ect - ect_ref)) <= REL * scale
    assert _close(r.energy, -float(np.sum(e_ref)))


def test_fp64_cfg2_slice_matches_oracle():
    """No=24, Nv=240: a contiguous slice of the tuple list (all tuples of
    a = 120 and the start of a = 121) against the oracle port."""
    d = synth.make_inputs(24, 240, 0)
    p = oracle.Problem(d)
    lst = oracle.tuple_list(240)
    t0 = int(np.searchsorted(lst[:, 0], 120))
    t1 = t0 + 1500
    e_ref, _ = oracle.tuple_energies(p, t0, t1, route="port", threads=8)
    with _ctx_for(d) as ctx:
        r = ctx.run(form="fp64", first_iteration=t0, max_iterations=t1 - 1)
        e, _ = ctx.tuple_energies(t0, t1 - t0)
    assert np.max(np.abs(e - e_ref)) <= REL * np.max(np.abs(e_ref))
    assert _close(r.energy, -float(np.sum(e_ref)))


def test_fp64_options_semantics():
    d = synth.make_inputs(5, 9, 3, with_j=True)
    p = oracle.Problem(d)
    n = synth.n_tuples(9)
    with _ctx_for(d) as ctx:
        # no (cT) intermediates requested -> ct_energy == energy
        r = ctx.run(use_j=False)
        assert r.energy == r.ct_energy
        # resume: tuples 40.. with a checkpointed physical energy
        e_ref, ect_ref = oracle.run(p, first_iteration=40, start_energy=1.25)
        r = ctx.run(first_iteration=40, start_energy=1.25)
        assert _close(r.energy, e_ref) and _close(r.ct_energy, ect_ref, abs(e_ref))
        assert r.tuples_done == n - 40 and r.next_iteration == n
        # ijkabc
        e_ref, ect_ref = oracle.run(p, ijkabc=True)
        r = ctx.run(ijkabc=True)
        assert _close(r.energy, e_ref) and _close(r.ct_energy, ect_ref, abs(e_ref))
        # empty range: cursor past the end returns the checkpoint energy
        r = ctx.run(first_iteration=n + 5, start_energy=-3.5)
        assert r.tuples_done == 0 and r.energy == -3.5
        # max_iterations is inclusive
        r = ctx.run(max_iterations=7)
        assert r.tuples_done == 8


def test_fp64_deterministic():
    d = synth.make_inputs(12, 30, 5)
    with _ctx_for(d) as ctx:
        a = ctx.run()
        ea, _ = ctx.tuple_energies(0, synth.n_tuples(30))
        b = ctx.run()
        eb, _ = ctx.tuple_energies(0, synth.n_tuples(30))
    assert a.energy == b.energy and a.ct_energy == b.ct_energy
    assert np.array_equal(ea, eb)


def test_errors_are_reported_not_faulted():
    d = synth.make_inputs(4, 7, 1)
    ctx = capi.Context(4, 7, 0)
    with pytest.raises(capi.AtripError) as ei:
        ctx.run()
    assert ei.value.status == capi.ERR_STATE
    with pytest.raises(capi.AtripError) as ei:
        ctx.upload("Tabij", d["Tabij"][:, :, :, :2])
    assert ei.value.status == capi.ERR_ARGUMENT
    ctx.close()
    with pytest.raises(capi.AtripError):
        capi.Context(65, 10, 0)


def test_python_atrip_api_with_checkpoints(tmp_path):
    from atrip_gb300 import Atrip, Input, read_checkpoint
    d = synth.make_inputs(6, 10, 4, with_j=True)
    p = oracle.Problem(d)
    e_ref, ect_ref = oracle.run(p)
    Atrip.init()
    ck = str(tmp_path / "ck.yaml")
    inp = (Input().with_epsilon_i(d["epsi"]).with_epsilon_a(d["epsa"]).with_Tai(d["Tai"])
           .with_Tabij(d["Tabij"]).with_Vabij(d["Vabij"]).with_Vijka(d["Vijka"])
           .with_Vabci(d["Vabci"]).with_Jijka(d["Jijka"]).with_Jabci(d["Jabci"])
           .with_checkpoint_path(ck).with_read_checkpoint_if_exists(False))
    out = Atrip.run(inp)
    assert _close(out.energy, e_ref) and _close(out.ct_energy, ect_ref, abs(e_ref))
    # checkpoint at every chunk (checkpoint_at_every_iteration = 0 and a
    # percentage that rounds to 0 -> atrip writes each iteration)
    inp.with_checkpoint_at_percentage(0.0).with_checkpoint_chunks(7)
    out2 = Atrip.run(inp)
    assert _close(out2.energy, e_ref)
    c = read_checkpoint(ck)
    assert c.no == 6 and c.nv == 10 and 0 < c.iteration < synth.n_tuples(10)
    # resume from that checkpoint: energy identical within tolerance
    inp.with_read_checkpoint_if_exists(True).with_checkpoint_at_percentage(10.0)
    out3 = Atrip.run(inp)
    assert _close(out3.energy, e_ref)


def test_chunked_host_upload_matches(tmp_path):
    """Host uploads larger than the staging bound are streamed through a
    bounded buffer a run of source slices at a time; a tiny bound (set for
    a child process) gives the same energies as the one-shot upload."""
    import json
    import os
    import subprocess
    import sys
    code = (
        "import json, sys; sys.path.insert(0, %r)\n"
        "from atrip_gb300 import capi, synth\n"
        "out = []\n"
        "for field in ('real', 'complex'):\n"
        "    d = synth.make_inputs(7, 13, 3, with_j=True, field=field)\n"
        "    with capi.Context(7, 13, 0, field=field) as c:\n"
        "        for n in ('epsi','epsa','Tai','Tabij','Vabij','Vijka','Vabci','Jijka','Jabci'):\n"
        "            c.upload(n, d[n])\n"
        "        r = c.run(form='fp64')\n"
        "        out.append([r.energy, r.ct_energy])\n"
        "print(json.dumps(out))\n" % os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    res = {}
    for elems in ("", "97"):
        env = dict(os.environ)
        env.pop("ATRIP_GB300_STAGING_ELEMS", None)
        if elems:
            env["ATRIP_GB300_STAGING_ELEMS"] = elems
        p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                           check=True)
        res[elems] = json.loads(p.stdout.strip().splitlines()[-1])
    assert res[""] == res["97"], res


@pytest.mark.parametrize("form,slices", [("fp64", 0), ("split_bf16", 3), ("split_f16", 2)])
def test_blocked_order_leaves_results_unchanged(form, slices):
    """tuple_block only changes the order in which the work queue hands out
    tuples: per-tuple energies (indexed by list position) and totals stay
    the same, also for a range that starts and ends inside a block."""
    d = synth.make_inputs(7, 23, 4)
    with _ctx_for(d) as ctx:
        ref = ctx.run(form=form, slices=slices, first_iteration=37, max_iterations=1200)
        e_ref, _ = ctx.tuple_energies(37, ref.tuples_done)
        for L in (2, 5, 8):
            ctx.set_tuning(tuple_block=L)
            r = ctx.run(form=form, slices=slices, first_iteration=37, max_iterations=1200)
            e, _ = ctx.tuple_energies(37, r.tuples_done)
            assert np.array_equal(e, e_ref), L
            assert abs(r.energy - ref.energy) <= 1e-13 * abs(ref.energy)

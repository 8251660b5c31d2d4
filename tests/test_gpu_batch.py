"""GPU parity of the batching form: many systems of uneven No/Nv in one
captured graph against the same systems run one by one, and against the
CPU oracle.

Per-tuple energies of a batch come from the same device code as the
single-system run (agreement to 1e-13 relative is asserted, in practice
they are bit-identical); the per-system totals are reduced in a different
order (one block per system instead of the two-stage sum), so they agree to
1e-13 relative.  The FP64 totals also
match the oracle at the 1e-10 relative bar of the plain form.
"""
import numpy as np
import pytest

import oracle
from atrip_gb300 import capi, synth

pytestmark = pytest.mark.gpu

# (No, Nv, seed): uneven sizes in the range of the multi-system workload,
# kept small enough for the oracle
SYSTEMS = [(4, 30, 0), (20, 33, 1), (7, 12, 2), (13, 41, 3), (9, 9, 4), (17, 25, 5), (5, 48, 6)]


def _ctx_for(d):
    ctx = capi.Context(d["No"], d["Nv"], 0)
    for name in ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci"):
        if name in d:
            ctx.upload(name, d[name])
    return ctx


@pytest.fixture(scope="module")
def systems():
    ds = [synth.make_inputs(No, Nv, seed, with_j=(seed % 2 == 0)) for No, Nv, seed in SYSTEMS]
    ctxs = [_ctx_for(d) for d in ds]
    yield ds, ctxs
    for c in ctxs:
        c.close()


def _singles(ctxs, **kw):
    out = []
    for c in ctxs:
        r = c.run(**kw)
        e, ect = c.tuple_energies(0, r.tuples_done)
        out.append((r.energy, r.ct_energy, e.copy(), ect.copy()))
    return out


@pytest.mark.parametrize("form", ["fp64", "split_bf16", "split_f16"])
@pytest.mark.parametrize("ijkabc", [False, True])
def test_batch_matches_single_runs(systems, form, ijkabc):
    """The split batch is one persistent launch of the transposed kernel over
    all systems: the single runs use the same kernel (split_variant 2)."""
    ds, ctxs = systems
    for c in ctxs:
        c.set_tuning(split_variant=2 if form != "fp64" else 0)
    ref = _singles(ctxs, form=form, ijkabc=ijkabc, use_j=True)
    with capi.Batch(ctxs) as b:
        for rep in range(2):  # the second run replays the captured graph
            res = b.run(form=form, ijkabc=ijkabc, use_j=True)
            for s, (c, r) in enumerate(zip(ctxs, res)):
                e0, ect0, te, tect = ref[s]
                assert r.tuples_done == synth.n_tuples(c.Nv)
                e, ect = c.tuple_energies(0, r.tuples_done)
                scale = np.max(np.abs(te))
                assert np.max(np.abs(e - te)) <= 1e-13 * scale, (form, s)
                assert np.max(np.abs(ect - tect)) <= 1e-13 * scale, (form, s)
                assert abs(r.energy - e0) <= 1e-13 * abs(e0) + 1e-15, (s, r.energy, e0)
                assert abs(r.ct_energy - ect0) <= 1e-13 * abs(e0) + 1e-15, (s, r.ct_energy, ect0)
            assert res[0].kernel_launches >= 2


@pytest.mark.parametrize("form,slices", [("split_f16", 2), ("split_bf16", 3), ("split_bf16", 2)])
def test_split_batch_one_launch_equals_launch_per_system(systems, form, slices):
    """All systems in ONE persistent launch (a work queue over their
    concatenated tuple ranges, per-system tensor maps in a device table)
    gives the per-tuple energies of one launch per system, bit for bit."""
    ds, ctxs = systems
    for c in ctxs:
        c.set_tuning(split_variant=2)
    with capi.Batch(ctxs) as b:
        b.set_tuning(split_variant=1)  # one launch per system
        per = b.run(form=form, slices=slices, use_j=True)
        per_e = [c.tuple_energies(0, r.tuples_done) for c, r in zip(ctxs, per)]
        b.set_tuning()  # default: one launch
        for rep in range(2):
            one = b.run(form=form, slices=slices, use_j=True)
            for s, (c, r, r0) in enumerate(zip(ctxs, one, per)):
                e, ect = c.tuple_energies(0, r.tuples_done)
                assert np.array_equal(e, per_e[s][0]), (form, s)
                assert np.array_equal(ect, per_e[s][1]), (form, s)
                assert abs(r.energy - r0.energy) <= 1e-14 * abs(r0.energy)
        # one split launch and one energy reduction, against one per system
        assert one[0].kernel_launches < per[0].kernel_launches
    with capi.Batch(ctxs[1:4]) as b:  # a subset and a tuple range
        r3 = b.run(form=form, slices=slices, use_j=False, first_iteration=5, max_iterations=300)
        for c, r in zip(ctxs[1:4], r3):
            one = c.run(form=form, slices=slices, use_j=False, first_iteration=5,
                        max_iterations=300)
            assert abs(r.energy - one.energy) <= 1e-13 * abs(one.energy) + 1e-15


def test_batch_fp64_matches_oracle(systems):
    ds, ctxs = systems
    with capi.Batch(ctxs) as b:
        res = b.run(form="fp64", use_j=True)
    for d, r in zip(ds, res):
        e_ref, ect_ref = oracle.run(oracle.Problem(d), use_j=True, threads=8, route="port")
        assert abs(r.energy - e_ref) <= 1e-10 * abs(e_ref) + 1e-14, (d["No"], d["Nv"])
        assert abs(r.ct_energy - ect_ref) <= 1e-10 * abs(e_ref) + 1e-14


def test_batch_range_and_reupload(systems):
    """A tuple range applies to every system; a re-uploaded tensor (new
    device buffer) is picked up by the replayed graph."""
    ds, ctxs = systems
    with capi.Batch(ctxs) as b:
        res = b.run(form="fp64", first_iteration=3, max_iterations=40)
        for c, r in zip(ctxs, res):
            n_all = synth.n_tuples(c.Nv)
            assert r.tuples_done == max(0, min(n_all, 41) - 3)
            one = c.run(form="fp64", first_iteration=3, max_iterations=40)
            assert abs(r.energy - one.energy) <= 1e-13 * abs(one.energy) + 1e-15
        d = dict(ds[1])
        d["Tai"] = d["Tai"] * 1.5
        ctxs[1].upload("Tai", d["Tai"])
        res = b.run(form="fp64")
        one = ctxs[1].run(form="fp64")
        assert abs(res[1].energy - one.energy) <= 1e-13 * abs(one.energy)
        ctxs[1].upload("Tai", ds[1]["Tai"])


def test_batch_rejects_bad_options(systems):
    ds, ctxs = systems
    with capi.Batch(ctxs[:2]) as b:
        opts = capi.RunOptions(capi.FORM_FP64, 0, 0, 0, 0, 0, 1.0, None)
        res = (capi.Result * 2)()
        import ctypes
        assert b.lib.atrip_gpu_batch_run(b.h, ctypes.byref(opts), res) == capi.ERR_ARGUMENT
    with pytest.raises(capi.AtripError):
        capi.Batch([ctxs[0], ctxs[0]])

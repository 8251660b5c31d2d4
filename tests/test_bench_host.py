"""Host helpers of bench.py (no GPU): the FLOP count, the roofline object
and the committed DRAM-traffic lookup the bench line uses."""
import importlib.util
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_flops_per_tuple_is_atrips_count(bench):
    # src/atrip/Atrip.cxx:578-580: 12 No^3 (No + Nv) per tuple
    assert bench.flops_per_tuple(40, 400) == 12 * 40 ** 3 * 440
    assert bench.flops_per_tuple(8, 40) == 294912


def test_roofline_counts_the_kept_digit_products(bench):
    peaks = {"bf16_tflops": 2000.0}
    # 1e12 FP64-equivalent FLOPs in one second
    r2 = bench._roofline("split_f16", 2, 1e12, 1000.0, peaks, None, None)
    r3 = bench._roofline("split_bf16", 3, 1e12, 1000.0, peaks, None, None)
    assert r2["achieved"] == pytest.approx(3.0) and r3["achieved"] == pytest.approx(6.0)
    assert r2["frac"] == pytest.approx(3.0 / 2000.0) and r2["bound"] == "tensor"
    assert "FP16" in r2["algorithmic"] and "BF16" in r3["algorithmic"]
    f = bench._roofline("fp64", 0, 1e12, 1000.0, peaks, 1.25, 5e9)
    assert f["achieved"] == pytest.approx(1.0) and f["frac"] == pytest.approx(0.8)
    assert f["traffic"] == 5e9


def test_traffic_lookup_matches_form_and_slices(bench):
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
        t = json.load(fh)
    ent = t["triples_split_kernel"]["no40_nv400"]
    got = bench.traffic_per_tuple("triples_split_kernel", "no40_nv400", ent["form"],
                                  ent["slices"])
    assert got == pytest.approx(ent["bytes_per_tuple"])
    # a capture of another slice format does not describe this run
    other = "split_bf16" if ent["form"] == "split_f16" else "split_f16"
    assert bench.traffic_per_tuple("triples_split_kernel", "no40_nv400", other, 3) is None
    assert bench.traffic_per_tuple("triples_split_kernel", "no_such_workload") is None


class _FakeRun:
    device_ms = 2.0


class _FakeContext:
    """Stands in for capi.Context: records the tuning and the profile."""

    def __init__(self, counters=None, fail=False):
        self.tuning = {"split_variant": 2}
        self.counters = counters
        self.fail = fail
        self.runs = []

    def get_tuning(self):
        return dict(self.tuning)

    def set_tuning(self, **kw):
        self.tuning = dict(kw)

    def run(self, **kw):
        from atrip_gb300 import capi
        self.runs.append((dict(self.tuning), kw))
        if self.fail:
            raise capi.AtripError(capi.ERR_UNSUPPORTED, "no profiled kernel here")
        return _FakeRun()

    def split_profile(self):
        return dict(self.counters)


def test_role_profile_shares_and_restores_tuning(bench):
    from atrip_gb300 import capi
    c = {name: 0 for name in capi.SPLIT_PROFILE if name}
    c.update(tuples=10, ctas=2, stages=6720, producer_total=1000, producer_wait_stage=500,
             mma_total=1000, mma_wait_stage=290, mma_wait_accumulator=4, epilogue_total=1000,
             epilogue_wait_accumulator=510, energy_total=2000, energy_wait_w=400,
             energy_w_convert=500)
    ctx = _FakeContext(c)
    out = bench._role_profile(ctx, "split_f16", 2, 100, 110)
    tun, kw = ctx.runs[0]
    assert tun["split_profile"] == 1 and tun["split_variant"] == 2
    assert kw["first_iteration"] == 100 and kw["max_iterations"] == 109
    assert ctx.tuning == {"split_variant": 2}  # restored after the run
    assert out["stages_per_tuple"] == 672 and out["cycles_per_tuple"]["energy"] == 200
    ws = out["wait_share"]
    assert ws["producer_wait_stage"] == 0.5 and ws["mma_wait_stage"] == 0.29
    assert ws["energy_wait_w"] == 0.2 and ws["energy_w_convert"] == 0.25


def test_role_profile_reports_an_unsupported_kernel(bench):
    ctx = _FakeContext(fail=True)
    out = bench._role_profile(ctx, "split_bf16", 3, 0, 5)
    assert "unavailable" in out and ctx.tuning == {"split_variant": 2}

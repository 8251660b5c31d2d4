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

"""Host logic of the autotuner (no GPU): sample windows and the sampled
error estimate that picks the split form's slice count."""
import math

import numpy as np

from atrip_gb300 import autotune


def test_windows_cover_the_list_evenly():
    for n, m, w in [(100, 4, 10), (11440, 16, 37), (5, 8, 2), (7, 3, 100)]:
        wins = autotune.windows(n, m, w)
        assert len(wins) <= m
        for lo, hi in wins:
            assert 0 <= lo < hi <= n
        for (l0, h0), (l1, h1) in zip(wins, wins[1:]):
            assert h0 <= l1  # disjoint, ordered
    wins = autotune.windows(1000, 10, 10)
    assert [lo for lo, _ in wins][0] < 100 and wins[-1][1] > 900


def test_window_size_tracks_flops():
    w = autotune.window_size(24, 240, 8, 1e12)
    fpt = 12 * 24 ** 3 * (24 + 240)
    assert abs(w * 8 * fpt - 1e12) <= 8 * fpt
    assert autotune.window_size(64, 1000, 8, 1.0) == 1


def test_error_estimate_extrapolates_and_scales_the_twin():
    rng = np.random.default_rng(0)
    ref = [rng.normal(1e-3, 1e-4, 50) for _ in range(8)]
    delta = 1e-12
    test = [r + delta for r in ref]
    n = 10_000
    est = autotune.error_estimate(n, ref, test)
    assert math.isclose(est["dE_est"], -n * delta, rel_tol=1e-6)
    assert math.isclose(est["E_est"], -n / 400 * sum(float(r.sum()) for r in ref), rel_tol=1e-12)
    assert est["dE_stderr"] < 1e-3 * abs(est["dE_est"])  # constant shift: no spread
    k = est["twin_scale_log2"]
    assert 0.1 / 16 <= abs(est["twin_E"]) <= 0.1 * 16
    assert math.isclose(est["twin_dE"], abs(est["dE_est"]) * 2.0 ** (4 * k))
    assert est["sample_tuples"] == 400
    # ijkabc keeps atrip's accumulated sign
    est2 = autotune.error_estimate(n, ref, test, ijkabc=True)
    assert math.isclose(est2["dE_est"], n * delta, rel_tol=1e-6)


def test_split_formats_order_and_eligibility():
    # FP16 2 slices first where its kernel covers the system; BF16 2 slices
    # (same digit products, fewer bits) then drop out
    assert autotune.split_formats(40, 400) == [("split_f16", 2), ("split_bf16", 3),
                                               ("split_bf16", 4)]
    assert autotune.split_formats(40, 400, "split_bf16") == [("split_bf16", 2), ("split_bf16", 3),
                                                             ("split_bf16", 4)]
    assert autotune.split_formats(40, 400, "split_f16") == [("split_f16", 2)]
    # No > 64 (2 No rows > 128), or K = 2 (Nv + No) >= 2048: BF16 only
    assert autotune.split_formats(64, 100)[0] == ("split_f16", 2)
    assert autotune.split_formats(65, 100)[0] == ("split_bf16", 2)
    assert autotune.split_formats(20, 1004)[0] == ("split_bf16", 2)
    assert autotune.f16_eligible(56, 560) and autotune.f16_eligible(63, 960)
    assert not autotune.f16_eligible(63, 961)

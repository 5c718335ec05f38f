"""The bench line's roofline objects, computed on the CPU from a made-up
per-class profile: the keys the JSON contract needs, achieved = algorithmic
bytes per launch / average launch time, frac = achieved / peak, and the ncu
traffic scaled to the average launch."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

CLASSES = ["panel_cqr", "larfb_w", "larfb_update", "wide_w", "wide_update", "wide_vsplit", "residual_fp64", "normal_eq_fp64", "prepare_digits"]


def fake_profile(steps):
    # (launches, total ms) over `steps` solves
    per_step = {"panel_cqr": (16, 0.84), "larfb_w": (12, 0.33), "larfb_update": (12, 0.28), "wide_w": (3, 0.16), "wide_update": (3, 0.10),
                "wide_vsplit": (3, 0.12), "wide_t": (3, 0.13), "residual_fp64": (3, 0.30),
                "normal_eq_fp64": (1, 0.11), "prepare_digits": (1, 0.25), "multq_thin": (3, 0.62)}
    return {k: (c * steps, ms * steps) for k, (c, ms) in per_step.items()}


@pytest.mark.parametrize("top", ["panel_cqr", "larfb_update"])
def test_rooflines_have_the_contract_keys(top):
    steps = 5
    prof = fake_profile(steps)
    tot = sum(v[1] for v in prof.values())
    main, others = bench.kernel_rooflines(prof, tot, top, 1.2, steps)
    assert main["class"] == top
    for r in [main] + list(others.values()):
        for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
            assert key in r
        assert r["bound"] in ("hbm", "tensor")
        assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
        cnt, ms = prof[main["class"] if r is main else next(k for k, v in others.items() if v is r)]
        assert r["avg_launch_us"] == pytest.approx(ms / cnt * 1e3)
        assert r["achieved"] == pytest.approx(r["algorithmic_bytes_per_launch"] / (r["avg_launch_us"] * 1e-6) / 1e9)
    assert set(others) | {top} == set(CLASSES)


def test_traffic_scales_with_the_algorithmic_bytes():
    steps = 2
    prof = fake_profile(steps)
    main, _ = bench.kernel_rooflines(prof, sum(v[1] for v in prof.values()), "panel_cqr", 1.2, steps)
    captured, captured_bytes = bench.NCU_TRAFFIC["panel_cqr"]
    assert main["traffic"] == pytest.approx(captured * main["algorithmic_bytes_per_launch"] / captured_bytes)

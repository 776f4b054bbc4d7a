"""The time-to-RMSE ladder of bench.py (host logic only, no GPU): rungs step
toward the target on the 1/sqrt(spp) law and stop at the first measured rung
below it; other targets are interpolated on the same law."""
import math

import bench


def _run(err_at, target, lo=16, cap=1 << 20, sec_per_spp=1e-3):
    ladder, n, e = [], 0, float("inf")
    while n < cap:
        n = min(bench.ladder_next(n, e, lo, target), cap)
        e = err_at(n)
        ladder.append({"spp": n, "seconds": n * sec_per_spp, "rmse": e})
        if e <= target:
            break
    return ladder


def test_ladder_stops_just_past_a_one_over_sqrt_target():
    # error 1 / sqrt(spp): RMSE 0.01 at exactly 10,000 spp
    ladder = _run(lambda n: 1.0 / math.sqrt(n), 0.01)
    assert ladder[-1]["rmse"] <= 0.01
    # doubling up to within 4x of the target, then one predicted step: the
    # stop lands within the 2% margin above the crossing, not at a doubling
    assert 10000 <= ladder[-1]["spp"] <= 10200
    assert [r["spp"] for r in ladder[:6]] == [16, 32, 64, 128, 256, 512]
    t, how = bench.ladder_time(ladder, 0.01, 0.01)
    assert how == "measured" and t == ladder[-1]["seconds"]


def test_ladder_creeps_up_on_a_flatter_error_curve():
    # an error falling slower than 1/sqrt(spp): the predicted steps undershoot
    # and the ladder takes several, each at least one sample, never past double
    err = lambda n: 0.3 * n ** -0.35  # noqa: E731
    ladder = _run(err, 0.01)
    assert ladder[-1]["rmse"] <= 0.01 and ladder[-2]["rmse"] > 0.01
    for a, b in zip(ladder, ladder[1:]):
        assert a["spp"] < b["spp"] <= 2 * max(a["spp"], 8)


def test_other_targets_interpolate_on_the_same_law():
    ladder = _run(lambda n: 1.0 / math.sqrt(n), 0.01)
    # 0.05 lies between the 256 and 512 rungs: exact on a 1/sqrt(spp) curve
    t, how = bench.ladder_time(ladder, 0.05, 0.01)
    assert how == "interpolated" and abs(t - 400 * 1e-3) < 1e-9
    # a target no rung reaches
    assert bench.ladder_time(ladder, 1e-4, 0.01) == (None, None)
    # below the first rung already: that rung's time
    assert bench.ladder_time(ladder, 0.5, 0.01) == (ladder[0]["seconds"], "measured")

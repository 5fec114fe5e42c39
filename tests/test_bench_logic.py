"""Host logic of bench.py (no GPU): the timed region's sort schedule, the
kernel-launch count it reports and the ensemble's whole-period step counts."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import bench  # noqa: E402


def test_timed_cadence_divides_the_timed_steps():
    assert bench.timed_cadence(20, 40) == 20
    assert bench.timed_cadence(20, 20) == 20
    assert bench.timed_cadence(80, 40) == 40
    assert bench.timed_cadence(30, 40) == 30
    assert bench.timed_cadence(30, 20) == 15
    assert bench.timed_cadence(7, 20) == 7
    for k in range(1, 100):
        for c in (1, 5, 20, 40):
            S = bench.timed_cadence(k, c)
            assert k % S == 0 and S <= c


def test_timed_steps_start_with_a_sort_and_hold_whole_periods():
    for K in (20, 40, 80):
        for chosen in (10, 20, 40):
            for W in (3, 5, 11):
                S = bench.timed_cadence(K, chosen)
                align = bench.warmup_alignment(W, S)
                _, since = bench.schedule(W + align, 0, S)
                assert since == S  # the next step sorts
                sorts, after = bench.schedule(K, since, S)
                assert sorts == K // S and after == S


def test_launch_count_of_the_default_line():
    # 20 timed steps, one sort: 6 sort kernels + 5 kernels per step (push,
    # three spectral-solve kernels, one diagnostics fold)
    S = bench.timed_cadence(20, 40)
    align = bench.warmup_alignment(5, S)
    _, _, since = bench.launches_for(5 + align, 0, S, 5)
    n, sorts, _ = bench.launches_for(20, since, S, 5)
    assert (n, sorts) == (106, 1)


def test_whole_periods_and_boundaries():
    assert bench.whole_periods(80, [20, 40]) == 80
    assert bench.whole_periods(50, [20, 30]) == 60
    assert bench.whole_periods(1, [7]) == 7
    assert bench.warm_to_boundary(20) == 20
    assert bench.warm_to_boundary(2) == 4
    assert bench.warm_to_boundary(1) == 3

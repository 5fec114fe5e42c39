"""The sort histogram's counting scheme (msc-thesis_gb300/csrc/pic_sort_dev.cuh,
sort_hist_segments) restated in numpy and checked against a plain count on
the CPU: blocks of HIST_BLOCK particles, each thread counting its HIST_SEG
consecutive particles with one add per run of equal keys, into a window of
wk keys centred on the block's middle key or straight into the global
histogram outside it; empty and past-the-end slots are skipped.  The GPU
histogram itself is exercised by every sort in the GPU tests."""
import numpy as np
import pytest

THREADS, SEG = 256, 16
BLOCK = THREADS * SEG


def histogram(keys, nkeys, wk, end=None):
    """keys: one key per slot, -1 for an empty slot (key of a cell < 0)."""
    end = len(keys) if end is None else end
    count = np.zeros(nkeys, np.int64)
    adds = 0
    for base in range(0, end, BLOCK):
        stop = min(end, base + BLOCK)
        mid = keys[base + (stop - base - 1) // 2]
        k0 = max(0, (mid if mid >= 0 else 0) - wk // 2)
        window = np.zeros(wk, np.int64)
        for t in range(THREADS):
            cur, run = -1, 0

            def flush():
                nonlocal adds
                if cur < 0:
                    return
                adds += 1
                if 0 <= cur - k0 < wk:
                    window[cur - k0] += run
                else:
                    count[cur] += run

            for j in range(SEG):
                s = base + SEG * t + j
                key = keys[s] if s < stop else -1
                if key != cur:
                    flush()
                    cur, run = key, 0
                run += 1
            flush()
        for r in range(wk):
            if window[r] and k0 + r < nkeys:
                count[k0 + r] += window[r]
    return count, adds


@pytest.mark.parametrize("scatter", [0.0, 0.02, 1.0])
def test_histogram_scheme_matches_a_plain_count(scatter):
    rng = np.random.default_rng(int(scatter * 100))
    nkeys, n, cap = 1200, 30000, 30720
    # keys sorted a while ago (about 30 particles per key), 5 % of the
    # particles since moved to a neighbouring key, some far stragglers
    keys = np.sort(rng.integers(0, nkeys - 1, n))
    moved = rng.random(n) < 0.05
    keys[moved] = np.clip(keys[moved] + rng.choice([-1, 1], moved.sum()), 0, nkeys - 2)
    far = rng.random(n) < scatter
    keys[far] = rng.integers(0, nkeys - 1, far.sum())
    slots = np.full(cap, -1)
    slots[:n] = keys
    slots[rng.random(cap) < 0.01] = -1
    count, adds = histogram(slots, nkeys, 256)
    live = slots[slots >= 0]
    np.testing.assert_array_equal(count, np.bincount(live, minlength=nkeys))
    if scatter == 0.0:
        # a few adds per thread (runs of equal keys), not one per particle
        assert adds < 4 * THREADS * (cap // BLOCK + 1) < cap / 3


def test_histogram_stops_at_the_live_count():
    keys = np.arange(10000) // 7
    count, _ = histogram(keys, 2000, 256, end=5000)
    np.testing.assert_array_equal(count, np.bincount(keys[:5000], minlength=2000))

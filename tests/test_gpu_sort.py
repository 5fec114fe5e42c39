"""The counting sort (cellTracking's replacement, thesisCode/dsmcCollisions/
cellTrackerAdvanced/src/main.cc:269-278) on particles that are far out of
order: thermal speeds of several cells per step and no sort for 30 steps
scatter each sort block's particles over thousands of cells, so most keys
miss the block's key window, overflow its straggler table and take the
per-run fallback.  After pic_sort the storage order must be sorted by the
tile-major row key (the cell key over the tile width: the order every
species but the DSMC one is kept in) and be a permutation of the state
before the sort."""
import numpy as np
import pytest

import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu

NX, NY, TW, TH = 256, 128, 16, 8


def tile_keys(cell):
    cx, cy = cell & 0xFFFF, cell >> 16
    ntx = NX // TW
    tx, lx = cx // TW, cx % TW
    ty, ly = cy // TH, cy % TH
    return ((ty * ntx + tx) * TH + ly) * TW + lx


def by_pid(a):
    o = np.argsort(a["pid"], kind="stable")
    return {k: v[o] for k, v in a.items()}


@pytest.mark.parametrize("ppc,steps", [(32, 30), (5, 30), (32, 4)])
def test_sort_of_scattered_particles_is_a_sorted_permutation(ppc, steps):
    n = NX * NY * ppc
    cfg, _, _ = normalized_electrons(NX, NY, float(NX), float(NY), n, 0.5, sort_every=100000,
                                     tile_w=TW, tile_h=TH)
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(n, vth=(8.0, 8.0, 0.0), seed=11))
        h.prime_leapfrog()
        h.step(steps)
        h.synchronize()
        before = h.get_particles_raw()
        kb = tile_keys(before["cell"]) // TW
        assert np.count_nonzero(np.diff(kb) < 0) > (n // 4 if steps >= 30 else 0)  # out of order
        h.sort()
        h.synchronize()
        after = h.get_particles_raw()
        assert h.diagnostics().error_flags == 0
    assert len(after["cell"]) == n
    ka = tile_keys(after["cell"]) // TW
    assert np.all(np.diff(ka) >= 0)
    b, a = by_pid(before), by_pid(after)
    assert np.unique(b["pid"]).size == n
    for k in ("pid", "cell", "ox", "oy", "vx", "vy"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)

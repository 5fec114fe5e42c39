"""pic_run_host, the one-call run from and to host memory (how the
reference's picFloatGpu is used, thesisCode/collisionless/double/src/
main.cc:182): the same state as the staged calls, outputs that alias the
inputs, page-locked or pageable arrays, and the FP64 oracle over a short
run from the imported state."""
import numpy as np
import pytest
import torch

import oracle as O
import picgpu as P
from gpu_util import normalized_electrons, periodic_diff

pytestmark = pytest.mark.gpu

NX = NY = 64
L = 4 * np.pi
DT = 0.1
STEPS = 30


def _load(n, seed=21):
    rng = np.random.default_rng(seed)
    x = rng.random(n) * L
    x = (x + 0.05 * np.sin(2 * np.pi * x / L)) % L  # a density wave on mode 1
    y = rng.random(n) * L
    vx = rng.normal(0.0, 0.05, n) + np.where(np.arange(n) % 2 == 0, 0.2, -0.2)
    vy = rng.normal(0.0, 0.05, n)
    return x, y, vx, vy


def test_run_host_matches_staged_calls_and_fp64_oracle():
    n = NX * NY * 16
    cfg, q, m = normalized_electrons(NX, NY, L, L, n, DT)
    arrs = _load(n)
    with P.Handle(cfg) as h:
        out = h.run_host(*arrs, STEPS)
        d = h.diagnostics()
        assert d.error_flags == 0 and d.step == STEPS
        assert d.total_charge_fixed == d.expected_charge_fixed
    with P.Handle(cfg) as h:
        h.set_particles(0, *arrs)
        start = h.get_particles()
        h.prime_leapfrog()
        h.step(STEPS)
        staged = h.get_particles()
    for k, o in zip(("x", "y", "vx", "vy"), out):
        np.testing.assert_array_equal(o, staged[k], err_msg=k)

    st = O.PhysState(NX, NY, L, L, DT, 1.0)
    st.add_species(start["x"], start["y"], start["vx"], start["vy"], q, m)
    st.prime(nthreads=0)
    st.run(STEPS, nthreads=0)
    s = st.species[0]
    cell = L / NX
    dxp = periodic_diff(out[0], s["x"], L)
    dyp = periodic_diff(out[1], s["y"], L)
    print("position max abs err (cells)", np.abs(dxp).max() / cell, np.abs(dyp).max() / cell)
    assert np.abs(dxp).max() < 1e-3 * cell
    assert np.abs(dyp).max() < 1e-3 * cell
    np.testing.assert_allclose(out[2], s["vx"], atol=1e-4 * np.abs(s["vx"]).max())
    np.testing.assert_allclose(out[3], s["vy"], atol=1e-4 * np.abs(s["vy"]).max())


def test_run_host_in_place_from_page_locked_arrays():
    n = NX * NY * 8 + 1
    cfg, _, _ = normalized_electrons(NX, NY, L, L, n, DT)
    arrs = _load(n, seed=22)
    with P.Handle(cfg) as h:
        ref = h.run_host(*arrs, 7, prime=False)
    pinned = [torch.from_numpy(a.copy()).pin_memory() for a in arrs]
    views = [t.numpy() for t in pinned]
    with P.Handle(cfg) as h:
        h.run_host(*views, 7, prime=False, out=views)
    for k in range(4):
        np.testing.assert_array_equal(views[k], ref[k])
    assert not np.array_equal(views[0], arrs[0])  # the particles moved


def test_run_host_rejects_more_particles_than_capacity():
    n = 1000
    cfg, _, _ = normalized_electrons(16, 16, 1.0, 1.0, n, DT)
    x, y, vx, vy = (np.zeros(n + 1) for _ in range(4))
    with P.Handle(cfg) as h:
        with pytest.raises(P.PicError):
            h.run_host(x, y, vx, vy, 1)

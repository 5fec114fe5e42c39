"""Device-side problems are reported through the device error word and the
status of pic_synchronize, and the handle stays usable: a non-finite
velocity, and ionisation beyond a species' capacity.  Both come from the
host's input; no kernel is made to fault or wait."""
import numpy as np
import pytest

import picgpu as P
from collide_util import E_CH, ME, MI, TN_EV, set_tabulated_mcc
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu


def test_non_finite_velocity_is_reported_and_the_handle_stays_usable():
    nx = 32
    n = nx * nx * 8
    cfg, _, _ = normalized_electrons(nx, nx, 4.0, 4.0, n, 0.05)
    rng = np.random.default_rng(3)
    x, y = rng.random(n) * 4.0, rng.random(n) * 4.0
    vx, vy = rng.normal(size=n) * 0.1, rng.normal(size=n) * 0.1
    vx[123] = np.nan
    with P.Handle(cfg) as h:
        h.set_particles(0, x, y, vx, vy)
        h.prime_leapfrog()
        h.step(3)
        with pytest.raises(P.PicError) as ei:
            h.synchronize()
        assert ei.value.status == 6  # PIC_ERR_NAN
        d = h.diagnostics()
        assert d.error_flags & P.DEVERR_NAN
        assert d.n[0] == n
        a = h.get_particles(0)  # still answers
        assert np.isnan(a["vx"][123])  # the bad particle drifts by NaN, the others do not
        for k in ("x", "y", "vx", "vy"):
            assert np.isfinite(np.delete(a[k], 123)).all()


def test_ionisation_beyond_capacity_is_reported():
    nx = 16
    dx = 2e-4
    L = nx * dx
    n = nx * nx * 64
    w = 1e4
    room = 64  # ion and electron slots left for newborn pairs
    sp = [P.species(n + room, -E_CH * w, ME * w, -1, P.SPECIES_HAS_VZ),
          P.species(n + room, E_CH * w, MI * w, 1, P.SPECIES_HAS_VZ)]
    cfg = P.config(nx, nx, L, L, 1e-11, sp, eps0=8.8541878128e-12)
    ve = np.sqrt(100.0 * E_CH / ME)  # 100 eV electrons: ionisation is frequent
    vi = np.sqrt(TN_EV * E_CH / MI)
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(n, vth=(ve, ve, ve), seed=2))
        h.init_particles(1, P.init_spec(n, vth=(vi, vi, vi), seed=3))
        set_tabulated_mcc(h, seed=4)
        for _ in range(20):
            h.collide(P.COLLIDE_MCC)
        with pytest.raises(P.PicError) as ei:
            h.synchronize()
        assert ei.value.status == 5  # PIC_ERR_OVERFLOW
        d = h.diagnostics()
        c = h.collision_counts()
        assert d.error_flags & P.DEVERR_CAPACITY
        assert c[2] > room  # more ionisations were drawn than there was room for
        assert n < d.n[0] <= n + room and n < d.n[1] <= n + room
        h.prime_leapfrog()
        h.step(2)  # the step still runs with the full species
        a = h.get_particles(0, vz=True)
        assert len(a["vx"]) == d.n[0]
        # ion slots the overflow may leave empty (cell -1; an ion slot
        # reserved whose electron found no room) carry no particle: both
        # export paths leave the caller's values at those ids and agree on
        # every other id
        import ctypes as C
        import os

        raw = h.get_particles_raw(1)
        ni = int(d.n[1])
        empty_ids = raw["pid"][:ni][raw["cell"][:ni] < 0]
        outs = []
        for lean in (False, True):
            old = os.environ.pop("PIC_STAGE_MAX_BYTES", None)
            if lean:
                os.environ["PIC_STAGE_MAX_BYTES"] = "1"
            try:
                arrs = [np.full(ni, 7.0) for _ in range(4)]
                cnt = C.c_longlong()
                h._c("pic_get_particles", 1, C.byref(cnt), *[P._ptr(x) for x in arrs], None)
            finally:
                os.environ.pop("PIC_STAGE_MAX_BYTES", None)
                if old is not None:
                    os.environ["PIC_STAGE_MAX_BYTES"] = old
            outs.append(arrs)
        for k in range(4):
            np.testing.assert_array_equal(outs[0][k], outs[1][k])
            assert (outs[0][k][empty_ids] == 7.0).all()

"""Electron-neutral MCC (the 512^2 MCC workload's cross sections, null-collision
method) against the oracle's restatement on the same Philox streams and
against the analytic collision frequency."""
import numpy as np
import pytest

import oracle as O
import picgpu as P
from collide_util import (E_CH, ME, MI, TN_EV, energies_eV, ks_statistic, mcc_resolved,
                          set_tabulated_mcc)

pytestmark = pytest.mark.gpu

DX = 2e-4


def mcc_handle(n, te_eV, dt, nx=32, extra=40000, with_field_species=True):
    w = 1e4  # real particles per macro-particle
    L = nx * DX
    sp = [P.species(n + extra, -E_CH * w, ME * w, -1, P.SPECIES_HAS_VZ),
          P.species(n + extra, E_CH * w, MI * w, 1, P.SPECIES_HAS_VZ)]
    cfg = P.config(nx, nx, L, L, dt, sp, eps0=8.8541878128e-12)
    h = P.Handle(cfg)
    ve = np.sqrt(te_eV * E_CH / ME)
    vi = np.sqrt(TN_EV * E_CH / MI)
    h.init_particles(0, P.init_spec(n, vth=(ve, ve, ve), seed=11))
    h.init_particles(1, P.init_spec(n, vth=(vi, vi, vi), seed=11))
    return h


def test_mcc_pass_matches_oracle_and_collision_frequency():
    n, dt, seed = 200_000, 1e-10, 7
    with mcc_handle(n, 20.0, dt) as h:
        set_tabulated_mcc(h, seed)
        a0 = h.get_particles(0, vz=True)
        h.collide(P.COLLIDE_MCC)
        h.synchronize()
        a1 = h.get_particles(0, vz=True)
        c = h.collision_counts()
        ni = h.diagnostics().n[1]
        d = h.diagnostics()
    m = mcc_resolved(dt, seed)
    vx, vy, vz, ne, nion, parent, oc = O.mcc_pass(m, np.arange(n), a0["vx"], a0["vy"], a0["vz"], 1)
    print("gpu counts", c[:4], "oracle counts", oc)
    # same streams: the same particles collide the same way, up to float margins
    vo = np.stack([vx, vy, vz], 1)
    vg = np.stack([a1["vx"][:n], a1["vy"][:n], a1["vz"][:n]], 1)
    speed = np.linalg.norm(vo, axis=1) + 1.0
    bad = np.linalg.norm(vg - vo, axis=1) > 1e-4 * speed
    print("mismatched particles", int(bad.sum()))
    assert bad.sum() == 0
    assert np.array_equal(c[:4], oc)
    # ionisation made electron-ion pairs, charge stays exact
    born = len(a1["vx"]) - n
    assert born == c[2] and ni == n + born
    assert abs(born - len(ne)) <= 2
    assert d.total_charge_fixed == d.expected_charge_fixed == 0
    # analytic expectation of each process count over the candidates
    E = energies_eV(a0)
    Et, sel, sexc, sion = (np.asarray(t) for t in O_tables())
    s = [np.interp(E, Et, t) for t in (sel, sexc, sion)]
    s[1][E < 11.5] = 0.0
    s[2][E < 15.8] = 0.0
    v = np.sqrt(2 * E * E_CH / ME)
    for k in range(3):
        expect = m["p_null"] * np.sum(m["ng"] * s[k] * v / m["nu_max"])
        print(f"process {k}: gpu {c[k]} expected {expect:.1f}")
        assert abs(c[k] - expect) < 5 * np.sqrt(expect) + 2


def O_tables():
    from collide_util import mcc_cross_sections
    return mcc_cross_sections()


def test_mcc_eedf_after_many_passes_matches_oracle():
    n, dt, seed, passes = 100_000, 1e-10, 3, 100
    with mcc_handle(n, 8.0, dt, extra=60000) as h:
        set_tabulated_mcc(h, seed)
        a0 = h.get_particles(0, vz=True)
        for _ in range(passes):
            h.collide(P.COLLIDE_MCC)
        a1 = h.get_particles(0, vz=True)
        c = h.collision_counts()
    m = mcc_resolved(dt, seed)
    vx, vy, vz = a0["vx"].copy(), a0["vy"].copy(), a0["vz"].copy()
    pid = np.arange(n)
    counts = np.zeros(4, dtype=np.int64)
    for p in range(1, passes + 1):
        vx, vy, vz, ne, ni, parent, oc = O.mcc_pass(m, pid, vx, vy, vz, p)
        counts += oc
        if len(ne):
            pid = np.concatenate([pid, np.arange(len(pid), len(pid) + len(ne))])
            vx = np.concatenate([vx, ne[:, 0]])
            vy = np.concatenate([vy, ne[:, 1]])
            vz = np.concatenate([vz, ne[:, 2]])
    eg = energies_eV(a1)
    eo = energies_eV(dict(vx=vx, vy=vy, vz=vz))
    D = ks_statistic(eg, eo)
    print(f"EEDF KS statistic {D:.5f}; gpu counts {c[:4]} oracle {counts}; "
          f"mean energy gpu {eg.mean():.4f} oracle {eo.mean():.4f} eV")
    # same streams for all but the newborns' descendants: far below the
    # 0.1 % two-sample critical value 1.95 sqrt(2/n)
    assert D < 1.95 * np.sqrt(2.0 / n)
    assert abs(eg.mean() - eo.mean()) < 5e-3 * eo.mean()
    assert eg.mean() < energies_eV(a0).mean()  # excitation and ionisation cool the tail


def test_mcc_inside_the_step_small():
    """Electrons and ions with field and MCC through pic_step (the MCC workload's physics
    on a 64^2 grid): charge exact, collisions happen, no device errors."""
    nx, ppc = 64, 16
    n = nx * nx * ppc
    ne0 = 1e15
    L = nx * DX
    w = ne0 * L * L / n
    sp = [P.species(n + n // 4, -E_CH * w, ME * w, -1, P.SPECIES_HAS_VZ),
          P.species(n + n // 4, E_CH * w, MI * w, 1, P.SPECIES_HAS_VZ)]
    cfg = P.config(nx, nx, L, L, 1e-11, sp, eps0=8.8541878128e-12, sort_every=20)
    ve, vi = np.sqrt(2.0 * E_CH / ME), np.sqrt(TN_EV * E_CH / MI)
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(n, vth=(ve, ve, ve), seed=5))
        h.init_particles(1, P.init_spec(n, vth=(vi, vi, vi), seed=5))
        set_tabulated_mcc(h, seed=9)
        h.prime_leapfrog()
        h.step(200)
        h.synchronize()
        d = h.diagnostics()
        c = h.collision_counts()
        q = h.history(P.HIST_CHARGE, 0, 201)
    print("counts", c, "n", list(d.n)[:2])
    assert d.error_flags == 0
    assert c[0] > 0
    assert (q == 0.0).all() and d.total_charge_fixed == d.expected_charge_fixed
    assert d.n[0] - n == d.n[1] - n == c[2]

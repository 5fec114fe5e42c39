"""Neutral-neutral DSMC (hard spheres, Bird NTC; the neutral gas of the
512^2 MCC + DSMC workload): conservation, relaxation of a bimodal
(300 K / 1000 K) gas against the oracle's restatement and theory, and the
collision rate."""
import numpy as np
import pytest

import oracle as O
import picgpu as P
from collide_util import D_NEUTRAL, E_CH, KB, M_NEUTRAL, ME, MI, NG, TN_EV, set_tabulated_mcc

pytestmark = pytest.mark.gpu

DX = 2e-4
PPC = 50


def bimodal(n, nx, seed=1):
    rng = np.random.default_rng(seed)
    L = nx * DX
    T = np.where(np.arange(n) % 2 == 0, 300.0, 1000.0)
    s = np.sqrt(KB * T / M_NEUTRAL)
    v = rng.normal(size=(3, n)) * s
    return rng.random(n) * L, rng.random(n) * L, v[0], v[1], v[2]


def temps(vx, vy, vz):
    out = []
    for g in (0, 1):
        a = np.stack([vx[g::2], vy[g::2], vz[g::2]])
        a = a - a.mean(axis=1, keepdims=True)
        out.append(M_NEUTRAL * (a ** 2).sum(axis=0).mean() / (3 * KB))
    return out


def neutral_handle(nx, n, dt, seed=4):
    L = nx * DX
    w = NG * L * L * 1.0 / n  # real atoms per macro-particle (depth 1 m)
    cfg = P.config(nx, nx, L, L, dt, [P.species(n, 0.0, M_NEUTRAL * w, 0, P.SPECIES_HAS_VZ)])
    h = P.Handle(cfg)
    h.set_dsmc(0, D_NEUTRAL, w, 1.0, np.pi * D_NEUTRAL ** 2 * 3000.0, seed)
    return h, w


def test_dsmc_relaxation_conservation_and_rate():
    nx, dt = 32, 5e-8
    n = nx * nx * PPC
    x, y, vx, vy, vz = bimodal(n, nx)
    h, w = neutral_handle(nx, n, dt)
    with h:
        h.set_particles(0, x, y, vx, vy, vz)
        p0 = np.array([vx.sum(), vy.sum(), vz.sum()])
        e0 = (vx ** 2 + vy ** 2 + vz ** 2).sum()
        Tg = []
        for blk in range(10):
            h.step(20)
            a = h.get_particles(0, vz=True)
            Tg.append(temps(a["vx"], a["vy"], a["vz"]))
        c_before = h.collision_counts()
        h.step(20)
        c_after = h.collision_counts()
        # 220 steps of every-step sorts on cell counts the push keeps current
        # (0.15 cells of motion per step): every particle still present once
        raw = h.get_particles_raw(0)
        assert np.array_equal(np.sort(raw["pid"][:n]), np.arange(n, dtype=np.uint32))
        assert (raw["cell"][:n] >= 0).all()
    Tg = np.array(Tg)
    p1 = np.array([a["vx"].sum(), a["vy"].sum(), a["vz"].sum()])
    e1 = (a["vx"] ** 2 + a["vy"] ** 2 + a["vz"] ** 2).sum()
    s = np.sqrt(e0)
    print("momentum change / sqrt(sum v^2):", np.abs(p1 - p0).max() / s,
          "energy rel change", abs(e1 - e0) / e0)
    assert np.abs(p1 - p0).max() < 1e-4 * s
    assert abs(e1 - e0) < 1e-4 * e0
    # oracle (same algorithm in FP64, independent streams) from the same start
    L = nx * DX
    d = dict(nx=nx, ny=nx, Lx=L, Ly=L, dt=dt, sigma=np.pi * D_NEUTRAL ** 2,
             coef=w * dt / (2 * DX * DX * 1.0), mass=M_NEUTRAL, seed=99)
    r = O.dsmc_run(d, x, y, vx, vy, vz, np.full(nx * nx, np.pi * D_NEUTRAL ** 2 * 3000.0), 200)
    To = np.stack([r["T_even"][19::20], r["T_odd"][19::20]], 1)
    print("T gpu (even, odd) per 20 steps:\n", np.round(Tg, 1), "\nT oracle:\n", np.round(To, 1))
    assert np.abs(Tg - To).max() < 15.0
    # relaxed to the mean temperature of the two halves
    assert abs(Tg[-1].mean() - 650.0) < 8.0 and abs(Tg[-1][0] - Tg[-1][1]) < 15.0
    # collision rate at equilibrium: 1/2 N n sigma <g> dt per step, <g> = sqrt(16 kT / (pi m))
    g_mean = np.sqrt(16 * KB * 650.0 / (np.pi * M_NEUTRAL))
    expect = 0.5 * n * NG * np.pi * D_NEUTRAL ** 2 * g_mean * dt * 20
    got = c_after[4] - c_before[4]
    print(f"collisions in 20 steps: {got}, expected {expect:.0f}")
    assert abs(got - expect) < 0.03 * expect


def test_small_dsmc_with_mcc_electrons():
    """Electrons + ions with MCC and the DSMC neutrals in one step loop
    (the MCC + DSMC workload's species on a 64^2 grid, dt = 1e-11 s)."""
    nx = 64
    L = nx * DX
    ne_ = nx * nx * 16
    nn = nx * nx * PPC
    w = 1e15 * L * L / ne_
    wn = NG * L * L / nn
    sp = [P.species(ne_ + ne_ // 4, -E_CH * w, ME * w, -1, P.SPECIES_HAS_VZ),
          P.species(ne_ + ne_ // 4, E_CH * w, MI * w, 1, P.SPECIES_HAS_VZ),
          P.species(nn, 0.0, M_NEUTRAL * wn, 0, P.SPECIES_HAS_VZ)]
    cfg = P.config(nx, nx, L, L, 1e-11, sp, eps0=8.8541878128e-12)
    ve, vi = np.sqrt(2.0 * E_CH / ME), np.sqrt(TN_EV * E_CH / MI)
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(ne_, vth=(ve, ve, ve), seed=5))
        h.init_particles(1, P.init_spec(ne_, vth=(vi, vi, vi), seed=5))
        x, y, vx, vy, vz = bimodal(nn, nx)
        h.set_particles(2, x, y, vx, vy, vz)
        set_tabulated_mcc(h, seed=9)
        h.set_dsmc(2, D_NEUTRAL, wn, 1.0, np.pi * D_NEUTRAL ** 2 * 3000.0, 21)
        h.prime_leapfrog()
        h.step(100)
        h.synchronize()
        d = h.diagnostics()
        c = h.collision_counts()
        a = h.get_particles(2, vz=True)
    print("counts", c)
    assert d.error_flags == 0 and d.total_charge_fixed == d.expected_charge_fixed
    assert c[0] > 0 and c[5] > 0
    assert len(a["vx"]) == nn and np.isfinite(a["vx"]).all()

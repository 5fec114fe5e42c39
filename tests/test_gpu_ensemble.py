"""Ensembles (pic_ensemble_*) against the same runs on single handles and
against the FP64 oracle."""
import os

import numpy as np
import pytest

import oracle as O
import picgpu as P
from gpu_util import normalized_electrons, oracle_from_handle, periodic_diff

pytestmark = pytest.mark.gpu

L = 4 * np.pi
DT = 0.1
# (nx, ny, particles per cell, beam drift, x-displacement amplitude, seed)
RUNS = [(32, 32, 16, 0.2, 1e-3, 1), (64, 32, 8, 0.15, 3e-3, 2), (32, 32, 32, 0.3, 1e-4, 3),
        (16, 64, 16, 0.1, 1e-2, 4), (64, 64, 4, 0.25, 5e-4, 5)]


def run_cfg(nx, ny, ppc, **tuning):
    n = nx * ny * ppc
    cfg, q, m = normalized_electrons(nx, ny, L, L, n, DT, **tuning)
    return cfg, n, q, m


def run_spec(n, v0, amp, seed):
    return P.init_spec(n, vth=(0.01, 0.01, 0.0), beam_v=v0, pert_kind=P.PERT_XDISP, pert_amp=amp,
                       pert_mx=1, seed=seed)


def build(runs, **tuning):
    cfgs, specs = [], []
    for nx, ny, ppc, v0, amp, seed in runs:
        cfg, n, _, _ = run_cfg(nx, ny, ppc, **tuning)
        cfgs.append(cfg)
        specs.append(run_spec(n, v0, amp, seed))
    return cfgs, specs


def test_ensemble_runs_match_single_handles():
    nst = 30
    cfgs, specs = build(RUNS, sort_every=5, chunk=1024)
    with P.Ensemble(cfgs) as E:
        E.init(specs)
        E.step(nst)
        E.synchronize()
        ens = [E.get_particles(r) for r in range(len(RUNS))]
        fe_ens = [E.history(r, P.HIST_FIELD_ENERGY, 0, nst + 1) for r in range(len(RUNS))]
        diags = [E.diagnostics(r) for r in range(len(RUNS))]
    exact = 0
    for r, (cfg, spec) in enumerate(zip(cfgs, specs)):
        with P.Handle(cfg) as h:
            h.init_particles(0, spec)
            h.prime_leapfrog()
            h.step(nst)
            a = h.get_particles(0)
            fe = h.history(P.HIST_FIELD_ENERGY, 0, nst + 1)
        dx = L / cfg.nx
        err = max(np.abs(periodic_diff(ens[r]["x"], a["x"], L)).max(),
                  np.abs(periodic_diff(ens[r]["y"], a["y"], L)).max()) / dx
        same = all(np.array_equal(ens[r][k], a[k]) for k in a)
        exact += same
        print(f"run {r}: {cfg.nx}x{cfg.ny}, max position difference {err:.2e} cells, "
              f"bit-identical {same}, FE rel diff {np.max(np.abs(fe_ens[r] - fe) / fe.max()):.2e}")
        # power-of-two grids: the ensemble and the single handle solve with the
        # same spectral kernels, run by run, so the particles agree bit for bit
        assert same
        assert err < 1e-4
        np.testing.assert_allclose(ens[r]["vx"], a["vx"], atol=1e-5)
        np.testing.assert_allclose(fe_ens[r], fe, rtol=1e-5, atol=1e-6 * fe.max())
        d = diags[r]
        assert d.step == nst and d.error_flags == 0
        assert d.total_charge_fixed == d.expected_charge_fixed
    print("bit-identical runs:", exact, "of", len(RUNS))


def test_ensemble_independent_of_sort_cadence():
    cfgs1, specs = build(RUNS[:3], sort_every=1, chunk=512)
    cfgs2, _ = build(RUNS[:3], sort_every=7, chunk=2048)
    out = []
    for cfgs in (cfgs1, cfgs2):
        with P.Ensemble(cfgs) as E:
            E.init(specs)
            E.step(20)
            out.append([E.get_particles(r) for r in range(3)])
    for r in range(3):
        for k in out[0][r]:
            np.testing.assert_array_equal(out[0][r][k], out[1][r][k], err_msg=f"run {r} {k}")


def ensemble_run(runs, nst, solver=None):
    cfgs, specs = build(runs, sort_every=5, chunk=1024)
    old = os.environ.get("PIC_FIELD_SOLVER")
    if solver:
        os.environ["PIC_FIELD_SOLVER"] = solver
    try:
        with P.Ensemble(cfgs) as E:
            E.init(specs)
            E.step(nst)
            E.synchronize()
            parts = [E.get_particles(r) for r in range(len(runs))]
            fe = [E.history(r, P.HIST_FIELD_ENERGY, 0, nst + 1) for r in range(len(runs))]
    finally:
        if old is None:
            os.environ.pop("PIC_FIELD_SOLVER", None)
        else:
            os.environ["PIC_FIELD_SOLVER"] = old
    return cfgs, parts, fe


def test_ensemble_cufft_path_matches_spectral_path():
    """The ensemble's cuFFT solve (grids that are not powers of two, or
    PIC_FIELD_SOLVER=cufft) against its spectral solve on the same runs, and
    an ensemble with a 48 x 32 run (cuFFT for every group) against single
    handles."""
    nst = 20
    cfgs, a, fa = ensemble_run(RUNS[:3], nst)
    _, b, fb = ensemble_run(RUNS[:3], nst, "cufft")
    for r, cfg in enumerate(cfgs):
        err = max(np.abs(periodic_diff(a[r]["x"], b[r]["x"], L)).max(),
                  np.abs(periodic_diff(a[r]["y"], b[r]["y"], L)).max()) / (L / cfg.nx)
        rel = np.abs(fa[r] - fb[r]).max() / fb[r].max()
        print(f"run {r}: spectral vs cuFFT, positions {err:.2e} cells, FE {rel:.2e}")
        assert err < 1e-4 and rel < 1e-5
    mixed = [(48, 32, 16, 0.2, 1e-3, 21), (32, 32, 16, 0.15, 1e-3, 22)]
    cfgs, e, fe = ensemble_run(mixed, nst)
    for r, (cfg, spec) in enumerate(zip(*build(mixed, sort_every=5, chunk=1024))):
        with P.Handle(cfg) as h:
            h.init_particles(0, spec)
            h.prime_leapfrog()
            h.step(nst)
            s = h.get_particles(0)
            fs = h.history(P.HIST_FIELD_ENERGY, 0, nst + 1)
        err = max(np.abs(periodic_diff(e[r]["x"], s["x"], L)).max(),
                  np.abs(periodic_diff(e[r]["y"], s["y"], L)).max()) / (L / cfg.nx)
        rel = np.abs(fe[r] - fs).max() / fs.max()
        print(f"mixed run {r} ({cfg.nx}x{cfg.ny}): vs single handle {err:.2e} cells, FE {rel:.2e}")
        assert err < 1e-4 and rel < 1e-5


@pytest.mark.parametrize("runs,nst,bar", [
    ([(32, 32, 16, 0.2, 1e-2, 7), (16, 32, 32, 0.25, 1e-2, 8), (128, 128, 16, 0.15, 1e-3, 9)],
     200, 1e-5),
    ([(64, 64, 32, 0.286, 5.4e-4, 10), (128, 128, 64, 0.145, 1.1e-3, 11)], 500, 1e-5),
    ([(64, 64, 16, 0.13, 5.8e-4, 12)], 500, 3e-5)])
def test_ensemble_field_energy_matches_fp64_oracle(runs, nst, bar):
    """Each run's field-energy history against the FP64 oracle from the same
    load, relative to the run's largest field energy.  Within 1e-5 over 200
    steps (through the growth and the saturation of the instability) for all
    sizes, and over the batched configuration's 500 steps for its runs of 32
    and more particles per cell.  After saturation the orbits are chaotic and
    the FP32 run (2^-16-cell deposit weights, FP32 offsets and velocities)
    drifts from the FP64 one by about 4x per 100 steps: the configuration's
    smallest runs (64^2 x 16 per cell, 65,536 particles) end at 1.4e-5 to
    2.1e-5 after 500 steps."""
    cfgs, specs = [], []
    for nx, ny, ppc, v0, amp, seed in runs:
        cfg, n, _, _ = run_cfg(nx, ny, ppc, history=nst + 1)
        cfgs.append(cfg)
        specs.append(run_spec(n, v0, amp, seed))
    with P.Ensemble(cfgs) as E:
        E.init(specs)
        E.step(nst)
        fe_ens = [E.history(r, P.HIST_FIELD_ENERGY, 0, nst + 1) for r in range(len(runs))]
    for r, (nx, ny, ppc, v0, amp, seed) in enumerate(runs):
        cfg, n, q, m = run_cfg(nx, ny, ppc)
        with P.Handle(cfg) as h:
            h.init_particles(0, specs[r])
            st = oracle_from_handle(h, cfg, q, m)
        st.prime(nthreads=0)
        ref = st.run(nst, nthreads=0)
        rel = np.abs(fe_ens[r] - ref["fe"]) / ref["fe"].max()
        print(f"{nx}x{ny} x {ppc}: field energy max rel error vs FP64 oracle "
              + ", ".join(f"{k} steps {rel[:k + 1].max():.2e}" for k in (40, 100, 200, 300, 400, 500)
                          if k <= nst))
        assert rel[:201].max() < 1e-5
        assert rel.max() < bar


def test_ensemble_rejects_bad_configs():
    cfg, n, _, _ = run_cfg(32, 32, 4)
    two = P.config(32, 32, L, L, DT, [P.species(n, -1.0, 1.0, -1), P.species(n, 1.0, 1.0, 1)])
    with pytest.raises(P.PicError):
        P.Ensemble([cfg, two])
    with P.Ensemble([cfg]) as E:
        with pytest.raises(P.PicError):
            E.step(1)  # not initialised
        with pytest.raises(P.PicError):
            E.init([run_spec(n + 4, 0.2, 1e-3, 1)])  # over capacity

"""Ensemble adjoint (pic_ensemble_adjoint) against the single-run GPU adjoint,
the FP64 adjoint restatement and central finite differences."""
import numpy as np
import pytest

import oracle as O
import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu

L = 4 * np.pi
DT = 0.1
# (nx, ny, particles per cell, beam drift, x-displacement amplitude, seed)
RUNS = [(32, 32, 16, 0.2, 1e-3, 11), (64, 32, 8, 0.15, 3e-3, 12), (32, 32, 32, 0.25, 1e-2, 13)]


def setup(runs, dt=DT, **tuning):
    cfgs, specs, qm = [], [], []
    for nx, ny, ppc, v0, amp, seed in runs:
        n = nx * ny * ppc
        cfg, q, m = normalized_electrons(nx, ny, L, L, n, dt, **tuning)
        cfgs.append(cfg)
        specs.append(P.init_spec(n, vth=(0.01, 0.01, 0.0), beam_v=v0, pert_kind=P.PERT_XDISP,
                                 pert_amp=amp, pert_mx=1, seed=seed))
        qm.append((q, m))
    return cfgs, specs, qm


def rel_norm(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_ensemble_adjoint_matches_single_run_and_fp64():
    nst, every = 40, 15
    cfgs, specs, qm = setup(RUNS, sort_every=5)
    with P.Ensemble(cfgs) as E:
        res, grads = E.adjoint(specs, nst, every)
        E.synchronize()
        assert all(E.diagnostics(r).step == nst for r in range(len(RUNS)))
    for r, (cfg, spec) in enumerate(zip(cfgs, specs)):
        with P.Handle(cfg) as h:
            h.init_particles(0, spec)
            s0 = h.get_particles(0)
            single, *sg = h.adjoint(nst, every=8, spec=spec)
        q, m = qm[r]
        ocfg = O.PhysCfg(cfg.nx, cfg.ny, L, L, DT, 1.0, 1)
        J, *og = O.adjoint(ocfg, s0["x"], s0["y"], s0["vx"], s0["vy"], q, m, nst)
        errs_single = [rel_norm(a, b) for a, b in zip(grads[r], sg)]
        errs_fp64 = [rel_norm(a, b) for a, b in zip(grads[r], og)]
        print(f"run {r}: J {res[r][0]:.6e} single {single.J:.6e} fp64 {J:.6e}; "
              f"vs single {max(errs_single):.2e}, vs FP64 {max(errs_fp64):.2e}; "
              f"dbeam {res[r][1]:.6e} / {single.dJ_dbeam_v:.6e}, damp {res[r][2]:.6e} / {single.dJ_damp:.6e}")
        assert res[r][0] == pytest.approx(single.J, rel=1e-6)
        assert res[r][0] == pytest.approx(J, rel=1e-5)
        assert max(errs_single) < 1e-4
        assert max(errs_fp64) < 1e-4
        assert res[r][1] == pytest.approx(single.dJ_dbeam_v, rel=1e-4)
        assert res[r][2] == pytest.approx(single.dJ_damp, rel=1e-4)


@pytest.mark.parametrize("dt,nsteps,every", [(0.1, 30, 10), (0.01, 500, 50)])
def test_ensemble_adjoint_against_central_differences(dt, nsteps, every):
    """dJ/d(beam drift) and dJ/d(amplitude) of each run against central
    differences (eps 1e-8) of the FP64 oracle's forward map of the run's load
    family (its device load's undisplaced positions and thermal velocities),
    within 1e-4; the FP64 adjoint of the family is checked against the same
    differences.  The 500-step case keeps a checkpoint every 50 steps, at
    dt = 0.01 (500 steps of dt = 0.1 end in the chaotic, saturated phase)."""
    from adjoint_util import central_differences, family_from_device, fp64_adjoint, rel
    runs = RUNS[:2]
    cfgs, specs, qm = setup(runs, dt=dt)
    with P.Ensemble(cfgs) as E:
        res, _ = E.adjoint(specs, nsteps, every=every, gradients=False)
    for r, (nx, ny, ppc, v0, amp, seed) in enumerate(runs):
        cfg = cfgs[r]
        q, m = qm[r]
        ocfg = O.PhysCfg(nx, ny, L, L, dt, 1.0, 1)
        fam = family_from_device(P, cfg, nx * ny * ppc, seed, P.LOAD_RANDOM)
        J, (adj_v, adj_a) = fp64_adjoint(ocfg, fam, q, m, nsteps, v0, amp)
        fd_v, fd_a = central_differences(ocfg, fam, q, m, nsteps, v0, amp)
        print(f"run {r}, dt {dt}, {nsteps} steps: J {res[r][0]:.8e} fp64 {J:.8e}; dJ/dbeam "
              f"{res[r][1]:.8e} fp64 {adj_v:.8e} FD {fd_v:.8e} ({rel(res[r][1], fd_v):.1e}); "
              f"dJ/damp {res[r][2]:.8e} fp64 {adj_a:.8e} FD {fd_a:.8e} "
              f"({rel(res[r][2], fd_a):.1e})")
        assert rel(adj_v, fd_v) < 1e-4 and rel(adj_a, fd_a) < 1e-4
        assert rel(res[r][1], fd_v) < 1e-4
        assert rel(res[r][2], fd_a) < 1e-4
        assert res[r][0] == pytest.approx(J, rel=1e-5)


def test_ensemble_adjoint_checkpoint_spacing_and_final_state():
    nst = 36
    cfgs, specs, _ = setup(RUNS, sort_every=4)
    out = {}
    for every in (6, 36):
        with P.Ensemble(cfgs) as E:
            out[every] = E.adjoint(specs, nst, every)
            final = [E.get_particles(r) for r in range(len(RUNS))]
            E.step(3)
            after = [E.get_particles(r) for r in range(len(RUNS))]
        with P.Ensemble(cfgs) as F:
            F.init(specs)
            F.step(nst)
            ref = [F.get_particles(r) for r in range(len(RUNS))]
            F.step(3)
            ref_after = [F.get_particles(r) for r in range(len(RUNS))]
        for r in range(len(RUNS)):
            for k in ref[r]:
                np.testing.assert_array_equal(final[r][k], ref[r][k])
                np.testing.assert_array_equal(after[r][k], ref_after[r][k])
    for r in range(len(RUNS)):
        assert out[6][0][r][0] == out[36][0][r][0]
        for a, b in zip(out[6][1][r], out[36][1][r]):
            assert rel_norm(a, b) < 1e-4


def test_torch_binding_of_the_batched_adjoint():
    """ensemble_field_energy_function: J per run from (beam drift, amplitude)
    tensors; backward gives the ensemble adjoint's dJ/d(beam), dJ/d(amplitude)
    scaled by the incoming gradient, run by run."""
    torch = pytest.importorskip("torch")
    nst = 12
    cfgs, specs, _ = setup(RUNS)
    with P.Ensemble(cfgs) as E:
        ref, _ = E.adjoint(specs, nst, every=4, gradients=False)
        f = P.ensemble_field_energy_function(E, specs, nst, every=4)
        bv = torch.tensor([r[3] for r in RUNS], dtype=torch.float64, requires_grad=True)
        amp = torch.tensor([r[4] for r in RUNS], dtype=torch.float64, requires_grad=True)
        J = f(bv, amp)
        w = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64)
        (w * J).sum().backward()
        # another drift for run 1 changes that run's J only
        bv2 = bv.detach().clone()
        bv2[1] += 0.01
        J2 = f(bv2, amp.detach())
    # J repeats bit for bit; the gradients to the float scatter atomics'
    # summation order (3e-8 between two calls), far inside the adjoint's error
    for r in range(len(RUNS)):
        assert J[r].item() == ref[r][0]
        assert bv.grad[r].item() == pytest.approx(w[r].item() * ref[r][1], rel=1e-5)
        assert amp.grad[r].item() == pytest.approx(w[r].item() * ref[r][2], rel=1e-5)
    assert J2[0].item() == J[0].item() and J2[2].item() == J[2].item()
    assert J2[1].item() != J[1].item()

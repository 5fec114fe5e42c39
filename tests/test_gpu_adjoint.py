"""GPU adjoint (pic_adjoint_run) against the FP64 adjoint restatement."""
import numpy as np
import pytest

import oracle as O
import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu

NX, PPC, L, DT = 32, 16, 4 * np.pi, 0.1


def two_beam_handle_state(h, seed=0, v0=0.2, amp=1e-3, k=0.5):
    n = NX * NX * PPC
    rng = np.random.default_rng(seed)
    x = rng.random(n) * L
    y = rng.random(n) * L
    x = (x + amp * np.cos(k * x)) % L
    sign = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    vx = sign * v0 + 0.01 * rng.normal(size=n)
    vy = 0.01 * rng.normal(size=n)
    h.set_particles(0, x, y, vx, vy)
    return h.get_particles(0), sign  # the state as stored (FP32)


def rel_norm(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture
def setup():
    n = NX * NX * PPC
    cfg, q, m = normalized_electrons(NX, NX, L, L, n, DT)
    return cfg, q, m, O.PhysCfg(NX, NX, L, L, DT, 1.0, 1)


@pytest.mark.parametrize("nsteps", [10, 50])
def test_gpu_adjoint_matches_fp64_adjoint(setup, nsteps):
    cfg, q, m, ocfg = setup
    with P.Handle(cfg) as h:
        s0, sign = two_beam_handle_state(h)
        r, gx, gy, gvx, gvy = h.adjoint(nsteps, every=8)
    J, ox, oy, ovx, ovy = O.adjoint(ocfg, s0["x"], s0["y"], s0["vx"], s0["vy"], q, m, nsteps)
    print(nsteps, "J", r.J, J)
    assert r.J == pytest.approx(J, rel=1e-5)
    errs = [rel_norm(a, b) for a, b in ((gx, ox), (gy, oy), (gvx, ovx), (gvy, ovy))]
    print("gradient rel norm errors", errs)
    # per-particle gradients carry the FP32 trajectory's node crossings
    # (measured 1e-5 after 10 steps, 1e-4 after 50)
    assert max(errs) < (1e-4 if nsteps <= 10 else 1e-3)
    drift_gpu, drift_orc = np.sum(sign * gvx), np.sum(sign * ovx)
    print("d/d(drift)", drift_gpu, drift_orc)
    assert drift_gpu == pytest.approx(drift_orc, rel=1e-4)


def test_checkpoint_interval_does_not_change_the_gradient(setup):
    cfg = setup[0]
    out = {}
    with P.Handle(cfg) as h:
        for every in (1, 7, 40):
            two_beam_handle_state(h)
            out[every] = h.adjoint(40, every=every)
    for every in (7, 40):
        assert out[every][0].J == out[1][0].J  # forward is deterministic
        for a, b in zip(out[every][1:], out[1][1:]):
            assert rel_norm(a, b) < 1e-4  # float atomics in the adjoint scatter


def test_adjoint_leaves_the_handle_at_the_final_step(setup):
    cfg = setup[0]
    nst = 30
    with P.Handle(cfg) as h:
        two_beam_handle_state(h)
        r = h.adjoint(nst, every=8)[0]
        a = h.get_particles(0)
        d = h.diagnostics()
        fe_hist = h.history(P.HIST_FIELD_ENERGY, 0, nst + 1)
    with P.Handle(cfg) as h:
        two_beam_handle_state(h)
        h.prime_leapfrog()
        h.step(nst)
        b = h.get_particles(0)
        e = h.diagnostics()
        fe_ref = h.history(P.HIST_FIELD_ENERGY, 0, nst + 1)
    assert d.step == e.step == nst
    assert r.J == d.field_energy == e.field_energy
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_array_equal(a[k], b[k])
    np.testing.assert_array_equal(fe_hist, fe_ref)


def test_load_parameter_gradients(setup):
    """dJ/d(beam_v) and dJ/d(pert_amp) of a lattice load with an x
    displacement, against the FP64 adjoint of the exported initial state
    contracted with the load's derivatives."""
    cfg, q, m, ocfg = setup
    n = NX * NX * PPC
    nst = 20
    spec = P.init_spec(n, layout=P.LOAD_LATTICE, vth=(0.01, 0.01, 0.0), beam_v=0.2,
                       pert_kind=P.PERT_XDISP, pert_amp=1e-3, pert_mx=1, seed=11)
    with P.Handle(cfg) as h:
        h.init_particles(0, spec)
        s0 = h.get_particles(0)
        r, gx, gy, gvx, gvy = h.adjoint(nst, every=5, spec=spec)
    J, ox, oy, ovx, ovy = O.adjoint(ocfg, s0["x"], s0["y"], s0["vx"], s0["vy"], q, m, nst)
    # lattice: 16 particles per cell as 4 x 4 sites, site i at x = (i % 128 + 1/2) L / 128
    lat_nx = NX * 4
    i = np.arange(n)
    x_lat = (i % lat_nx + 0.5) * (L / lat_nx)
    dxdA = np.cos(2 * np.pi / L * x_lat)
    sign = np.where(i % 2 == 0, 1.0, -1.0)
    damp, dbeam = np.sum(ox * dxdA), np.sum(sign * ovx)
    print("J", r.J, J, "damp", r.dJ_damp, damp, "dbeam", r.dJ_dbeam_v, dbeam)
    assert r.J == pytest.approx(J, rel=1e-5)
    assert r.dJ_damp == pytest.approx(damp, rel=1e-4)
    assert r.dJ_dbeam_v == pytest.approx(dbeam, rel=1e-4)
    # the contraction done on the device equals the one done here on its own arrays
    assert r.dJ_damp == pytest.approx(np.sum(gx * dxdA), rel=1e-9, abs=1e-12)
    assert r.dJ_dbeam_v == pytest.approx(np.sum(sign * gvx), rel=1e-9, abs=1e-12)


@pytest.mark.parametrize("dt,nsteps,every", [(0.1, 50, 10), (0.01, 500, 50)])
def test_load_parameter_gradients_match_central_differences(dt, nsteps, every):
    """dJ/d(beam_v) and dJ/d(pert_amp) of the GPU adjoint (contracted on the
    device from the load) against central differences (eps 1e-8) of the FP64
    forward map of the same load family, within 1e-4; the FP64 adjoint of
    the family is checked against the same differences.  The 500-step case
    keeps a checkpoint every 50 steps, at dt = 0.01: 500 steps of dt = 0.1
    end past the saturation of the two-stream modes, where the map is
    chaotic and neither differences nor an FP32 trajectory follow it."""
    from adjoint_util import central_differences, family_from_device, fp64_adjoint, rel
    n = NX * NX * PPC
    v0, amp = 0.2, 1e-3
    cfg, q, m = normalized_electrons(NX, NX, L, L, n, dt)
    spec = P.init_spec(n, layout=P.LOAD_LATTICE, vth=(0.01, 0.01, 0.0), beam_v=v0,
                       pert_kind=P.PERT_XDISP, pert_amp=amp, pert_mx=1, seed=11)
    with P.Handle(cfg) as h:
        h.init_particles(0, spec)
        r = h.adjoint(nsteps, every=every, spec=spec)[0]
    fam = family_from_device(P, cfg, n, 11, P.LOAD_LATTICE)
    ocfg = O.PhysCfg(NX, NX, L, L, dt, 1.0, 1)
    J, (adj_v, adj_a) = fp64_adjoint(ocfg, fam, q, m, nsteps, v0, amp)
    fd_v, fd_a = central_differences(ocfg, fam, q, m, nsteps, v0, amp)
    print(f"dt {dt}, {nsteps} steps: J gpu {r.J:.8e} fp64 {J:.8e}; dJ/dv0 gpu {r.dJ_dbeam_v:.8e} "
          f"fp64 {adj_v:.8e} FD {fd_v:.8e} ({rel(r.dJ_dbeam_v, fd_v):.1e}); dJ/damp gpu "
          f"{r.dJ_damp:.8e} fp64 {adj_a:.8e} FD {fd_a:.8e} ({rel(r.dJ_damp, fd_a):.1e})")
    assert rel(adj_v, fd_v) < 1e-4 and rel(adj_a, fd_a) < 1e-4
    assert rel(r.dJ_dbeam_v, fd_v) < 1e-4
    assert rel(r.dJ_damp, fd_a) < 1e-4
    assert r.J == pytest.approx(J, rel=1e-5)


def test_torch_binding_gradients(setup):
    torch = pytest.importorskip("torch")
    cfg = setup[0]
    with P.Handle(cfg) as h:
        s0, _ = two_beam_handle_state(h)
        ref = h.adjoint(15, every=5)
        f = P.field_energy_function(h, 15, every=5)
        t = [torch.tensor(s0[k], dtype=torch.float64, requires_grad=True)
             for k in ("x", "y", "vx", "vy")]
        J = f(*t)
        (2.0 * J).backward()
    assert J.item() == ref[0].J
    for tt, g in zip(t, ref[1:]):
        np.testing.assert_allclose(tt.grad.numpy(), 2.0 * g, rtol=1e-4,
                                   atol=1e-4 * np.abs(g).max())

"""The step's spectral Poisson solve (pic_spectral.cu, power-of-two grids from
16 to 4096 cells a side) against an FP64 solve of the same float density and
against the cuFFT path of the same handle (PIC_FIELD_SOLVER=cufft) on the
same particles."""
import os

import numpy as np
import pytest

import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu

SIZES = [(16, 16), (64, 32), (32, 128), (256, 256), (4096, 16), (16, 4096), (2048, 2048)]
NSTEPS = 10


def fp64_fields(rho, Lx, Ly, eps0=1.0):
    """E = -grad phi with k^2 phi^ = rho^ / eps0 (zero mode removed), the
    Nyquist component of each derivative set to zero; phi as well."""
    ny, nx = rho.shape
    rh = np.fft.rfft2(rho.astype(np.float64))
    mx = np.arange(nx // 2 + 1)[None, :]
    my = np.arange(ny)[:, None]
    kx = 2 * np.pi / Lx * mx
    ky = 2 * np.pi / Ly * np.where(2 * my <= ny, my, my - ny)
    k2 = kx**2 + ky**2
    k2[0, 0] = 1.0
    ph = rh / (eps0 * k2)
    ph[0, 0] = 0.0
    kxe = np.where(2 * mx == nx, 0.0, kx)
    kye = np.where(2 * my == ny, 0.0, ky)
    ex = np.fft.irfft2(-1j * kxe * ph, s=(ny, nx))
    ey = np.fft.irfft2(-1j * kye * ph, s=(ny, nx))
    return ex, ey, np.fft.irfft2(ph, s=(ny, nx))


def run(nx, ny, solver):
    ppc = 32 if nx * ny >= 1 << 20 else 16  # 2048^2: the benchmarked load
    n = nx * ny * ppc
    Lx, Ly = 0.05 * nx, 0.05 * ny
    cfg, _, _ = normalized_electrons(nx, ny, Lx, Ly, n, 0.05)
    spec = P.init_spec(n, vth=(0.05, 0.05, 0.0), pert_kind=P.PERT_DENSITY, pert_amp=0.05,
                       pert_mx=1, pert_my=1, seed=nx * 7 + ny)
    old = os.environ.get("PIC_FIELD_SOLVER")
    os.environ["PIC_FIELD_SOLVER"] = solver
    try:
        with P.Handle(cfg) as h:
            h.track_mode(1, 1)
            h.init_particles(0, spec)
            h.deposit()
            h.poisson()
            g = {w: h.grid(w) for w in (P.GRID_RHO, P.GRID_EX, P.GRID_EY, P.GRID_PHI)}
            h.prime_leapfrog()
            h.step(NSTEPS)
            hist = {w: h.history(w, 0, NSTEPS + 1)
                    for w in (P.HIST_FIELD_ENERGY, P.HIST_CHARGE, P.HIST_MODE_AMP)}
            g["ex_end"] = h.grid(P.GRID_EX)
            d = h.diagnostics()
    finally:
        if old is None:
            os.environ.pop("PIC_FIELD_SOLVER", None)
        else:
            os.environ["PIC_FIELD_SOLVER"] = old
    assert d.error_flags == 0 and d.total_charge_fixed == d.expected_charge_fixed
    return cfg, g, hist


@pytest.mark.parametrize("nx,ny", SIZES)
def test_spectral_solve_matches_fp64_and_cufft(nx, ny):
    cfg, gs, hs = run(nx, ny, "spectral")
    _, gc, hc = run(nx, ny, "cufft")
    # the conversion is the same arithmetic: identical density
    np.testing.assert_array_equal(gs[P.GRID_RHO], gc[P.GRID_RHO])
    ex, ey, phi = fp64_fields(gs[P.GRID_RHO], cfg.Lx, cfg.Ly)
    emax = max(np.abs(ex).max(), np.abs(ey).max())
    err_s = max(np.abs(gs[P.GRID_EX] - ex).max(), np.abs(gs[P.GRID_EY] - ey).max()) / emax
    err_c = max(np.abs(gc[P.GRID_EX] - ex).max(), np.abs(gc[P.GRID_EY] - ey).max()) / emax
    err_p = np.abs(gs[P.GRID_PHI] - phi).max() / np.abs(phi).max()
    print(f"{nx}x{ny}: E vs FP64, spectral {err_s:.2e}, cuFFT {err_c:.2e}; phi {err_p:.2e}")
    assert err_s < 1e-5 and err_c < 1e-5 and err_p < 1e-5
    if nx * ny >= 1024:  # the two paths ran (their roundings differ)
        assert not np.array_equal(gs[P.GRID_EX], gc[P.GRID_EX])
    # ten steps on each path
    np.testing.assert_array_equal(hs[P.HIST_CHARGE], hc[P.HIST_CHARGE])
    fe_s, fe_c = hs[P.HIST_FIELD_ENERGY], hc[P.HIST_FIELD_ENERGY]
    rel_fe = np.abs(fe_s - fe_c).max() / fe_c.max()
    rel_mode = np.abs(hs[P.HIST_MODE_AMP] - hc[P.HIST_MODE_AMP]).max() / hc[P.HIST_MODE_AMP].max()
    rel_e = np.abs(gs["ex_end"] - gc["ex_end"]).max() / np.abs(gc["ex_end"]).max()
    print(f"  after {NSTEPS} steps: FE {rel_fe:.2e}, mode (1,1) {rel_mode:.2e}, Ex {rel_e:.2e}")
    assert rel_fe < 1e-5 and rel_mode < 1e-5 and rel_e < 1e-4


@pytest.mark.parametrize("nx,ny", [(64, 16), (32, 128)])
def test_adjoint_solve_paths_agree(nx, ny):
    """The adjoint's transposed solve (psi = S^T g) through the spectral
    kernels' adjoint mode against cuFFT, on non-square grids: the final field
    energy to 1e-5 and the gradients with respect to the initial state to
    1e-4 over 20 steps (measured 2e-6 to 4e-6; per-particle gradients carry
    each FP32 trajectory's own cell crossings)."""
    n = nx * ny * 16
    Lx, Ly = 0.25 * nx, 0.25 * ny
    cfg, _, _ = normalized_electrons(nx, ny, Lx, Ly, n, 0.1)
    spec = P.init_spec(n, vth=(0.02, 0.02, 0.0), beam_v=0.2, pert_kind=P.PERT_XDISP,
                       pert_amp=1e-3, pert_mx=1, seed=nx + ny)
    out = {}
    old = os.environ.get("PIC_FIELD_SOLVER")
    try:
        for solver in ("spectral", "cufft"):
            os.environ["PIC_FIELD_SOLVER"] = solver
            with P.Handle(cfg) as h:
                h.init_particles(0, spec)
                out[solver] = h.adjoint(20, every=10)
    finally:
        if old is None:
            os.environ.pop("PIC_FIELD_SOLVER", None)
        else:
            os.environ["PIC_FIELD_SOLVER"] = old
    rs, *gs = out["spectral"]
    rc, *gc = out["cufft"]
    errs = [np.linalg.norm(a - b) / np.linalg.norm(b) for a, b in zip(gs, gc)]
    print(f"{nx}x{ny}: J {rs.J:.8e} vs {rc.J:.8e}; gradient rel norm differences", errs)
    assert rs.J == pytest.approx(rc.J, rel=1e-5)
    assert max(errs) < 1e-4

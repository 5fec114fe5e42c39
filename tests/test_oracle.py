"""CPU oracle checks: pinned against the reference's own outputs (golden
vectors made by tests/golden/make_golden.py from the reference's CPU
sources) and against published known-answer vectors."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN


def load_case(path):
    z = np.load(path)
    keys = [str(k) for k in z["param_keys"]]
    vals = dict(zip(keys, z["params"]))
    ints = {"xDim", "yDim", "nx", "ny", "npx", "npy"}
    p = O.ref_params(**{k: (int(v) if k in ints else float(v)) for k, v in vals.items()})
    return p, z


CASES = sorted(glob.glob(os.path.join(GOLDEN, "compat_*.npz")))


def test_golden_fixtures_present():
    assert len(CASES) >= 3


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c) for c in CASES])
def test_compat_restatement_bit_exact_vs_reference_golden(path):
    p, z = load_case(path)
    out = O.compat_run(p, z["x0"], z["y0"], z["vx0"], z["vy0"], int(z["nsteps"]))
    for k in ("x", "y", "vx", "vy", "rho", "phi", "ex", "ey"):
        assert np.array_equal(out[k], z[k]), k


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c) for c in CASES])
def test_loop_step_count(path):
    p, z = load_case(path)
    assert O.count_steps(p.dt, p.tmax) == int(z["loop_steps"])


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_compat_restatement_bit_exact_vs_reference_live():
    p = O.ref_params(xDim=6, yDim=9, nx=12, ny=18, npx=25, npy=21, dt=0.015, tmax=0.1,
                     charge=-30.0, mass=3.0, vtx=0.8, vty=0.4, vdx=0.2, vdy=0.0)
    x, y, vx, vy = O.ref_init(p)
    a = O.compat_run(p, x, y, vx, vy, 12, use_ref=True)
    b = O.compat_run(p, x, y, vx, vy, 12)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_compat_threads_match_serial():
    p, z = load_case(CASES[0])
    a = O.compat_run(p, z["x0"], z["y0"], z["vx0"], z["vy0"], 5, nthreads=1)
    b = O.compat_run(p, z["x0"], z["y0"], z["vx0"], z["vy0"], 5, nthreads=4)
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_allclose(b[k], a[k], rtol=0, atol=1e-12)


def test_philox_known_answers():
    # Random123 philox4x32_10 known-answer vectors (Salmon et al., SC'11)
    assert O.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E,
                                                                    0xA20BC7C6, 0x6D5451FD]
    assert O.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                           [0xA4093822, 0x299F31D0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420,
                                                          0x24126EA1]


@pytest.mark.parametrize("shape", [(16, 12), (32, 32), (10, 7), (8, 64)])
def test_fft_matches_numpy(shape):
    import ctypes as C
    a = np.random.default_rng(1).standard_normal(shape)
    n0, n1 = shape
    out = np.empty((n0, n1 // 2 + 1, 2))
    L = O.lib()
    L.orc_fft2d_r2c.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.orc_fft2d_c2r.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.orc_fft2d_r2c(n0, n1, a.ctypes.data, out.ctypes.data)
    ref = np.fft.rfft2(a)
    np.testing.assert_allclose(out[..., 0] + 1j * out[..., 1], ref, atol=1e-12 * np.abs(ref).max())
    back = np.empty(shape)
    L.orc_fft2d_c2r(n0, n1, out.ctypes.data, back.ctypes.data)
    np.testing.assert_allclose(back / (n0 * n1), a, atol=1e-12)


def test_fixed_point_deposit_exact_total_charge():
    rng = np.random.default_rng(3)
    nx, ny, n = 24, 20, 5000
    cx = rng.integers(0, nx, n)
    cy = rng.integers(0, ny, n)
    cell = (cx | (cy << 16)).astype(np.int32)
    ox = rng.random(n, dtype=np.float32)
    oy = rng.random(n, dtype=np.float32)
    ox[:3] = [0.0, np.float32(1) - np.float32(2**-24), 0.5]
    rho = O.deposit_fixed(nx, ny, cell, ox, oy, q_int=-1)
    assert rho.sum() == -n * 2**32
    assert (rho <= 0).all()
    # skipped slots
    cell[::7] = -1
    rho2 = O.deposit_fixed(nx, ny, cell, ox, oy, q_int=1)
    assert rho2.sum() == (n - len(cell[::7])) * 2**32


def test_fixed_point_deposit_matches_float_cic():
    rng = np.random.default_rng(4)
    nx, ny, n = 8, 6, 3000
    cx, cy = rng.integers(0, nx, n), rng.integers(0, ny, n)
    ox, oy = rng.random(n, dtype=np.float32), rng.random(n, dtype=np.float32)
    rho = O.deposit_fixed(nx, ny, (cx | (cy << 16)).astype(np.int32), ox, oy) / 2**32
    ref = np.zeros((ny, nx))
    fx, fy = ox.astype(np.float64), oy.astype(np.float64)
    np.add.at(ref, (cy, cx), (1 - fx) * (1 - fy))
    np.add.at(ref, (cy, (cx + 1) % nx), fx * (1 - fy))
    np.add.at(ref, ((cy + 1) % ny, cx), (1 - fx) * fy)
    np.add.at(ref, ((cy + 1) % ny, (cx + 1) % nx), fx * fy)
    # weights are quantised to 2^-16 per axis
    np.testing.assert_allclose(rho.reshape(ny, nx), ref, atol=n * 2**-16)


def test_physics_oracle_field_energy_and_poisson():
    nx, ny, L = 32, 16, 2 * np.pi
    st = O.PhysState(nx, ny, L, L / 2, 0.1)
    rng = np.random.default_rng(5)
    n = 20000
    st.add_species(rng.random(n) * L, rng.random(n) * L / 2, np.zeros(n), np.zeros(n),
                   q=-L * L / 2 / n, m=L * L / 2 / n)
    f = st.fields(nthreads=1)
    dx, dy = L / nx, L / 2 / ny
    assert abs(f["rho"].mean()) < 1e-12
    assert f["fe"] == pytest.approx(0.5 * (f["ex"] ** 2 + f["ey"] ** 2).sum() * dx * dy, rel=1e-12)
    # spectral Laplacian of phi equals -rho (modes below Nyquist)
    ph = np.fft.rfft2(f["phi"])
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=dy)[:, None]
    kx = 2 * np.pi * np.fft.rfftfreq(nx, d=dx)[None, :]
    lap = -(kx ** 2 + ky ** 2) * ph
    r = np.fft.rfft2(f["rho"])
    np.testing.assert_allclose(lap[1:ny // 2, 1:nx // 2], -r[1:ny // 2, 1:nx // 2],
                               atol=1e-9 * np.abs(r).max())


def test_physics_oracle_energy_conservation():
    # cold plasma oscillation: total energy is conserved to second order in dt
    nx = ny = 16
    L = 2 * np.pi
    st = O.PhysState(nx, ny, L, L, 0.05)
    npx = 64
    g = (np.arange(npx) + 0.5) * L / npx
    x, y = np.meshgrid(g, g)
    x, y = x.ravel(), y.ravel()
    n = len(x)
    x = (x + 0.01 * np.cos(x)) % L
    st.add_species(x, y, np.zeros(n), np.zeros(n), q=-L * L / n, m=L * L / n)
    st.prime()
    h = st.run(200, nthreads=2)
    tot = h["fe"][:-1] + h["ke"]
    assert np.ptp(tot) < 2e-3 * tot.max()
    # the plasma oscillates at omega_pe = 1: field energy period pi
    fe = h["fe"]
    peaks = [i for i in range(1, len(fe) - 1) if fe[i] > fe[i - 1] and fe[i] >= fe[i + 1]]
    assert len(peaks) >= 2
    period = 2 * np.mean(np.diff(peaks)) * 0.05
    assert period == pytest.approx(2 * np.pi, rel=0.03)

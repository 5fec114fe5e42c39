"""The FP64 adjoint restatement against central finite differences (CPU).

The map is the physics-mode step (CIC deposit, spectral Poisson, leapfrog)
and J the final field energy; the adjoint is exact for this map except where
a finite-difference perturbation moves a particle across a cell boundary (a
kink of the CIC weights), so the comparison uses small perturbations and a
short run of a two-beam plasma."""
import numpy as np
import pytest

import oracle as O


def two_beams(nx=32, ppc=16, L=4 * np.pi, v0=0.2, amp=1e-3, k=0.5, seed=0):
    n = nx * nx * ppc
    rng = np.random.default_rng(seed)
    x = rng.random(n) * L
    y = rng.random(n) * L
    dxdA = np.cos(k * x)
    x = (x + amp * dxdA) % L
    sign = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    vx = sign * v0 + 0.01 * rng.normal(size=n)
    vy = 0.01 * rng.normal(size=n)
    q, m = -L * L / n, L * L / n
    return dict(x=x, y=y, vx=vx, vy=vy, q=q, m=m, L=L, nx=nx, sign=sign, dxdA=dxdA)


@pytest.mark.parametrize("nsteps,tol", [(10, 2e-5), (50, 2e-4)])
def test_oracle_adjoint_matches_central_differences(nsteps, tol):
    s = two_beams()
    L, nx = s["L"], s["nx"]
    cfg = O.PhysCfg(nx, nx, L, L, 0.1, 1.0, 1)
    args = (s["q"], s["m"], nsteps)
    J, gx, gy, gvx, gvy = O.adjoint(cfg, s["x"], s["y"], s["vx"], s["vy"], *args)
    J0 = O.forward_J(cfg, s["x"], s["y"], s["vx"], s["vy"], *args)
    assert J == pytest.approx(J0, rel=1e-12)
    eps = 1e-6
    # direction 1: beam drift (velocity), direction 2: the seeded displacement
    adj = {"drift": np.sum(s["sign"] * gvx), "disp": np.sum(s["dxdA"] * gx)}
    fd = {}
    for key in adj:
        vals = []
        for e in (eps, -eps):
            if key == "drift":
                vals.append(O.forward_J(cfg, s["x"], s["y"], s["vx"] + e * s["sign"], s["vy"], *args))
            else:
                vals.append(O.forward_J(cfg, (s["x"] + e * s["dxdA"]) % L, s["y"], s["vx"], s["vy"],
                                        *args))
        fd[key] = (vals[0] - vals[1]) / (2 * eps)
    for key in adj:
        rel = abs(adj[key] - fd[key]) / abs(fd[key])
        print(nsteps, key, adj[key], fd[key], rel)
        assert rel < tol
    # a random direction over all four arrays
    rng = np.random.default_rng(5)
    d = [rng.normal(size=len(s["x"])) for _ in range(4)]
    ad = sum(np.dot(a, b) for a, b in zip((gx, gy, gvx, gvy), d))
    st = [s["x"], s["y"], s["vx"], s["vy"]]
    Jp = O.forward_J(cfg, *[a + eps * b for a, b in zip(st, d)], *args)
    Jm = O.forward_J(cfg, *[a - eps * b for a, b in zip(st, d)], *args)
    fdr = (Jp - Jm) / (2 * eps)
    print(nsteps, "random", ad, fdr)
    assert abs(ad - fdr) < 10 * tol * abs(fdr) + 1e-9


def test_oracle_adjoint_of_zero_steps_is_the_field_gradient():
    """nsteps = 0: J is the field energy of the initial positions; moving one
    particle changes it by its charge times the potential gradient."""
    s = two_beams(nx=16, ppc=4)
    L, nx = s["L"], s["nx"]
    cfg = O.PhysCfg(nx, nx, L, L, 0.1, 1.0, 1)
    J, gx, gy, gvx, gvy = O.adjoint(cfg, s["x"], s["y"], s["vx"], s["vy"], s["q"], s["m"], 0)
    assert np.all(gvx == 0) and np.all(gvy == 0)
    eps = 1e-6
    for i in (0, 17, 333):
        xp, xm = s["x"].copy(), s["x"].copy()
        xp[i] += eps
        xm[i] -= eps
        args = (s["y"], s["vx"], s["vy"], s["q"], s["m"], 0)
        fd = (O.forward_J(cfg, xp, *args) - O.forward_J(cfg, xm, *args)) / (2 * eps)
        assert gx[i] == pytest.approx(fd, rel=1e-5, abs=1e-12)


@pytest.mark.parametrize("load,dt,nsteps", [("lattice", 0.1, 50), ("random", 0.1, 30),
                                            ("lattice", 0.01, 500)])
def test_oracle_load_parameter_gradients_match_central_differences(load, dt, nsteps):
    """dJ/d(beam drift) and dJ/d(displacement amplitude) of a two-beam load
    (32^2 cells, 16 per cell, drift 0.2, amplitude 1e-3), contracted from the
    FP64 adjoint, against central differences with eps = 1e-8: within 1e-4.
    The 500-step case runs at dt = 0.01 (t = 5): at dt = 0.1 those 500 steps
    reach t = 50, past the saturation of the fastest two-stream modes, where
    the map is chaotic and difference quotients do not converge."""
    from adjoint_util import (central_differences, fp64_adjoint, lattice_family, random_family,
                              rel)
    nx, ppc, L = 32, 16, 4 * np.pi
    n = nx * nx * ppc
    fam = lattice_family(nx, ppc, L, seed=11) if load == "lattice" else random_family(n, L, 3)
    q, m = -L * L / n, L * L / n
    cfg = O.PhysCfg(nx, nx, L, L, dt, 1.0, 1)
    J, (adj_v, adj_a) = fp64_adjoint(cfg, fam, q, m, nsteps, 0.2, 1e-3)
    fd_v, fd_a = central_differences(cfg, fam, q, m, nsteps, 0.2, 1e-3)
    print(f"{load} dt {dt} {nsteps} steps: J {J:.6e}; dJ/dv0 adjoint {adj_v:.8e} FD {fd_v:.8e} "
          f"({rel(adj_v, fd_v):.1e}); dJ/damp adjoint {adj_a:.8e} FD {fd_a:.8e} "
          f"({rel(adj_a, fd_a):.1e})")
    assert rel(adj_v, fd_v) < 1e-4
    assert rel(adj_a, fd_a) < 1e-4

"""Generate the golden vectors in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py

Builds oracle/_ref/libpicref.so from the reference's unmodified CPU sources
(taylorj5/msc-thesis thesisCode/collisionless/double/src/{grid,particle,
fourier,main}.cc; see oracle/Makefile) and runs its step through the harness
oracle/ref_harness.cc.  Each case stores the initial particle arrays, the
parameters, and the state after `nsteps` steps: final positions and
velocities and the ghost-padded grids rho, phi, Ex, Ey.  The initial arrays
of the lattice cases come from the reference's own initialiseParticles
(main.cc:201-244); the edge case places particles on the domain boundaries.

The reference tree is needed only here; the fixtures are committed so that
tests run without it.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

CASES = {
    # square grid, the reference's default domain, lattice init
    "compat_square": dict(p=dict(xDim=10, yDim=10, nx=32, ny=32, npx=40, npy=40, dt=0.01,
                                 tmax=0.2, charge=-100.0, mass=100.0, vtx=1.0, vty=1.0),
                          nsteps=20, init="ref"),
    # rectangular grid and domain, drift: exercises the second-index wavenumber
    # map and the swapped field axes
    "compat_rect": dict(p=dict(xDim=8, yDim=12, nx=16, ny=24, npx=30, npy=20, dt=0.02,
                               tmax=0.3, charge=-50.0, mass=10.0, vtx=0.5, vty=0.7, vdx=0.3,
                               vdy=0.1),
                        nsteps=15, init="ref"),
    # particles exactly on x = 0, x = xDim, y = yDim (cell index nx / ny)
    "compat_edges": dict(p=dict(xDim=4, yDim=4, nx=16, ny=16, npx=10, npy=10, dt=0.01,
                                tmax=0.1, charge=-100.0, mass=100.0, vtx=1.0, vty=1.0),
                         nsteps=10, init="edges"),
}


def edges_init(p):
    n = p.npx * p.npy
    rng = np.random.default_rng(7)
    x = rng.uniform(0, p.xDim, n)
    y = rng.uniform(0, p.yDim, n)
    x[:4] = [0.0, float(p.xDim), float(p.xDim), 0.0]
    y[:4] = [0.0, 0.0, float(p.yDim), float(p.yDim)]
    x[4], y[4] = 0.5 * p.xDim, float(p.yDim)
    vx = rng.normal(0, 1, n)
    vy = rng.normal(0, 1, n)
    vx[:5] = [0.0, 1.0, 1.0, -1.0, 0.0]
    vy[:5] = [-1.0, 0.0, 1.0, 1.0, 1.0]
    return x, y, vx, vy


def main():
    O.build()
    if not O.ref_available():
        raise SystemExit("reference library not built (is the reference tree present?)")
    for name, c in CASES.items():
        p = O.ref_params(**c["p"])
        if c["init"] == "ref":
            x, y, vx, vy = O.ref_init(p)
        else:
            x, y, vx, vy = edges_init(p)
        out = O.compat_run(p, x, y, vx, vy, c["nsteps"], use_ref=True)
        nloop = O.ref().ref_count_steps(p.dt, p.tmax)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            params=np.array([c["p"].get(k, 0.0) for k in PARAM_KEYS], dtype=np.float64),
            param_keys=np.array(PARAM_KEYS), nsteps=c["nsteps"], loop_steps=nloop,
            x0=x, y0=y, vx0=vx, vy0=vy, **out)
        print(name, "particles", len(x), "steps", c["nsteps"], "loop", nloop)


PARAM_KEYS = ["xDim", "yDim", "nx", "ny", "npx", "npy", "dt", "tmax", "charge", "mass",
              "vtx", "vty", "vdx", "vdy"]

if __name__ == "__main__":
    main()

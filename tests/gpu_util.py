"""Helpers shared by the GPU tests (not a test module)."""
import numpy as np

import oracle as O
import picgpu as P


def normalized_electrons(nx, ny, Lx, Ly, n, dt, **tuning):
    """One electron species in plasma units (eps0 = 1, omega_pe = 1): macro
    charge -A/n and mass A/n, so that n_macro q^2 / (eps0 m) = 1."""
    A = Lx * Ly
    sp = P.species(n, -A / n, A / n, -1)
    return P.config(nx, ny, Lx, Ly, dt, [sp], **tuning), -A / n, A / n


def oracle_from_handle(h, cfg, q, m, s=0):
    st = O.PhysState(cfg.nx, cfg.ny, cfg.Lx, cfg.Ly, cfg.dt, cfg.eps0)
    a = h.get_particles(s)
    st.add_species(a["x"], a["y"], a["vx"], a["vy"], q, m)
    return st


def periodic_diff(a, b, L):
    d = a - b
    return d - L * np.round(d / L)

"""Helpers shared by the adjoint tests (not a test module).

Two-beam loads written as functions of the two load parameters that the
adjoint differentiates -- the beam drift v0 and the x-displacement amplitude
-- and central finite differences of the FP64 oracle's forward map along
them.  The map is the physics-mode step loop (deposit, spectral solve,
gather, leapfrog) that replaces the reference's loop body
(collisionless/double/src/main.cc:137-172); J is the final field energy.

Finite differences of a CIC particle map converge only while no particle
crosses a grid node inside the difference interval: each such crossing is a
kink of J whose effect on the difference quotient does not shrink with eps
(about 1e-4 of the derivative per kink in these runs), and the number of
kinks inside the interval grows with eps.  eps = 1e-8 keeps the quotients
of these tests within 2e-5 of the derivative (FP64 round-off stays near
1e-7 of it); eps = 1e-4 leaves them 1e-3 to 1e-2 away.
"""
import numpy as np

import oracle as O

EPS_FD = 1e-8


class TwoBeamFamily:
    """Initial states x = x_u + amp cos(k x_u) (mod L), y = y_u,
    vx = vx_t + s v0, vy = vy_t with s = +1 for even particle ids and -1 for
    odd ones: pic_init_particles' load with beam_v and PIC_PERT_XDISP, in
    FP64 around fixed undisplaced positions and thermal velocities."""

    def __init__(self, xu, yu, vxt, vyt, L, k):
        self.xu, self.yu, self.vxt, self.vyt = (np.asarray(a, dtype=np.float64)
                                                for a in (xu, yu, vxt, vyt))
        self.L, self.k = L, k
        n = len(self.xu)
        self.sign = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
        self.dxdA = np.cos(k * self.xu)

    def state(self, v0, amp):
        x = (self.xu + amp * self.dxdA) % self.L
        return x, self.yu, self.vxt + self.sign * v0, self.vyt

    def contract(self, gx, gvx):
        """(dJ/dv0, dJ/damp) from the gradients with respect to x0 and vx0."""
        return float(np.sum(self.sign * gvx)), float(np.sum(self.dxdA * gx))


def lattice_family(nx, ppc, L, seed, vth=0.01, k=0.5):
    """A quiet two-beam load on an nx x nx grid: ppc sites per cell on a
    square lattice (sqrt(ppc) per side), Gaussian thermal velocities."""
    side = int(round(np.sqrt(ppc)))
    lat = nx * side
    i = np.arange(lat * lat)
    xu = (i % lat + 0.5) * (L / lat)
    yu = (i // lat + 0.5) * (L / lat)
    rng = np.random.default_rng(seed)
    return TwoBeamFamily(xu, yu, vth * rng.normal(size=len(i)), vth * rng.normal(size=len(i)),
                         L, k)


def random_family(n, L, seed, vth=0.01, k=0.5):
    """A two-beam load with uniformly random undisplaced positions."""
    rng = np.random.default_rng(seed)
    xu, yu = rng.random(n) * L, rng.random(n) * L
    return TwoBeamFamily(xu, yu, vth * rng.normal(size=n), vth * rng.normal(size=n), L, k)


def family_from_device(P, cfg, n, seed, layout, vth=0.01, mx=1):
    """The family of a device load (pic_init_particles with the given seed and
    layout): a handle loads it with no drift and no displacement, and its
    exported positions and velocities become x_u, y_u and the thermal parts."""
    spec = P.init_spec(n, layout=layout, vth=(vth, vth, 0.0), seed=seed)
    with P.Handle(cfg) as h:
        h.init_particles(0, spec)
        a = h.get_particles(0)
    return TwoBeamFamily(a["x"], a["y"], a["vx"], a["vy"], cfg.Lx, 2 * np.pi * mx / cfg.Lx)


def central_differences(ocfg, fam, q, m, nsteps, v0, amp, eps=EPS_FD):
    """(dJ/dv0, dJ/damp) by central differences of the FP64 forward map."""
    out = []
    for dv, da in ((eps, 0.0), (0.0, eps)):
        jp = O.forward_J(ocfg, *fam.state(v0 + dv, amp + da), q, m, nsteps)
        jm = O.forward_J(ocfg, *fam.state(v0 - dv, amp - da), q, m, nsteps)
        out.append((jp - jm) / (2 * eps))
    return tuple(out)


def fp64_adjoint(ocfg, fam, q, m, nsteps, v0, amp):
    """J and (dJ/dv0, dJ/damp) from the FP64 adjoint restatement."""
    J, gx, gy, gvx, gvy = O.adjoint(ocfg, *fam.state(v0, amp), q, m, nsteps)
    return J, fam.contract(gx, gvx)


def rel(a, b):
    return abs(a - b) / abs(b)

"""ctypes access to the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline / reference
legs of ``bench.py`` import this module.  It loads

* ``oracle/build/liboracle.so`` -- the plain-C restatement (pic_oracle.c),
* ``oracle/_ref/libpicref.so``  -- the reference's own CPU step compiled from
  its sources (present only where the reference tree was available at build
  time; ``ref_available()`` says whether it is).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "build", "liboracle.so")
_REF = os.path.join(HERE, "_ref", "libpicref.so")

_dp = C.POINTER(C.c_double)


class RefParams(C.Structure):
    """Mirror of the reference's Params fields (collisionless/double/inc/params.h:21-47)."""

    _fields_ = [
        ("xDim", C.c_int), ("yDim", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
        ("npx", C.c_int), ("npy", C.c_int),
        ("dt", C.c_double), ("tmax", C.c_double), ("charge", C.c_double), ("mass", C.c_double),
        ("vtx", C.c_double), ("vty", C.c_double), ("vdx", C.c_double), ("vdy", C.c_double),
    ]


def ref_params(xDim=10, yDim=10, nx=32, ny=32, npx=10, npy=10, dt=1e-7, tmax=1e-4,
               charge=-100.0, mass=100.0, vtx=1.0, vty=1.0, vdx=0.0, vdy=0.0) -> RefParams:
    """Defaults are the reference's struct Params defaults (params.h:22-42)."""
    return RefParams(xDim, yDim, nx, ny, npx, npy, dt, tmax, charge, mass, vtx, vty, vdx, vdy)


class PhysCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("Lx", C.c_double), ("Ly", C.c_double),
                ("dt", C.c_double), ("eps0", C.c_double), ("nspecies", C.c_int)]


class Species(C.Structure):
    _fields_ = [("n", C.c_long), ("q", C.c_double), ("m", C.c_double),
                ("x", _dp), ("y", _dp), ("vx", _dp), ("vy", _dp)]


def build() -> None:
    """Compile the restatement (and the reference, when its tree is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if os.path.isdir(os.environ.get("REF_ROOT", "/root/reference/thesisCode")):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        L.orc_count_steps.restype = C.c_long
        L.orc_count_steps.argtypes = [C.c_double, C.c_double]
        L.orc_compat_init.argtypes = [C.POINTER(RefParams), C.c_uint64, _dp, _dp, _dp, _dp]
        L.orc_compat_run.argtypes = [C.POINTER(RefParams), _dp, _dp, _dp, _dp, C.c_long,
                                     _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_phys_fields.restype = C.c_double
        L.orc_phys_fields.argtypes = [C.POINTER(PhysCfg), C.POINTER(Species), _dp, _dp, _dp, _dp,
                                      C.c_int]
        L.orc_phys_prime.argtypes = [C.POINTER(PhysCfg), C.POINTER(Species), C.c_int]
        L.orc_phys_run.argtypes = [C.POINTER(PhysCfg), C.POINTER(Species), C.c_long, _dp, _dp,
                                   _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32)]
        L.orc_deposit_fixed.argtypes = [C.c_int, C.c_int, C.c_long, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int64, C.c_void_p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(_REF)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(_REF)
        R.ref_count_steps.restype = C.c_long
        R.ref_count_steps.argtypes = [C.c_double, C.c_double]
        R.ref_init.argtypes = [C.POINTER(RefParams), _dp, _dp, _dp, _dp]
        R.ref_run.argtypes = [C.POINTER(RefParams), _dp, _dp, _dp, _dp, C.c_long,
                              _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        _ref = R
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# --------------------------------------------------------------- compat ----
def compat_run(p: RefParams, x, y, vx, vy, nsteps: int, nthreads: int = 1, use_ref=False):
    """Run ``nsteps`` of the reference-convention step (restatement, or the
    reference itself with ``use_ref``).  Returns a dict of final arrays and the
    (nx+2)x(ny+2) ghost-padded grids."""
    n = p.npx * p.npy
    x, y, vx, vy = (_f64(a) for a in (x, y, vx, vy))
    out = {k: np.empty(n) for k in ("x", "y", "vx", "vy")}
    g = (p.nx + 2, p.ny + 2)
    out.update({k: np.empty(g) for k in ("rho", "phi", "ex", "ey")})
    args = [C.byref(p), _p(x), _p(y), _p(vx), _p(vy), nsteps,
            _p(out["x"]), _p(out["y"]), _p(out["vx"]), _p(out["vy"]),
            _p(out["rho"]), _p(out["phi"]), _p(out["ex"]), _p(out["ey"])]
    if use_ref:
        ref().ref_run(*args)
    else:
        lib().orc_compat_run(*args, nthreads)
    return out


def ref_init(p: RefParams):
    n = p.npx * p.npy
    a = [np.empty(n) for _ in range(4)]
    ref().ref_init(C.byref(p), *[_p(v) for v in a])
    return a


def compat_init(p: RefParams, seed: int = 1234):
    n = p.npx * p.npy
    a = [np.empty(n) for _ in range(4)]
    lib().orc_compat_init(C.byref(p), seed, *[_p(v) for v in a])
    return a


def count_steps(dt: float, tmax: float) -> int:
    return int(lib().orc_count_steps(dt, tmax))


# -------------------------------------------------------------- physics ----
class PhysState:
    """Holds FP64 species arrays for the physics-mode oracle."""

    def __init__(self, nx, ny, Lx, Ly, dt, eps0=1.0):
        self.cfg = PhysCfg(nx, ny, Lx, Ly, dt, eps0, 0)
        self.species = []  # list of dicts with numpy arrays

    def add_species(self, x, y, vx, vy, q, m):
        self.species.append(dict(x=_f64(x).copy(), y=_f64(y).copy(), vx=_f64(vx).copy(),
                                 vy=_f64(vy).copy(), q=float(q), m=float(m)))

    def _sp(self):
        arr = (Species * len(self.species))()
        for i, s in enumerate(self.species):
            arr[i] = Species(len(s["x"]), s["q"], s["m"], _p(s["x"]), _p(s["y"]), _p(s["vx"]),
                             _p(s["vy"]))
        self.cfg.nspecies = len(self.species)
        return arr

    def fields(self, nthreads=0):
        g = (self.cfg.ny, self.cfg.nx)
        out = {k: np.empty(g) for k in ("rho", "phi", "ex", "ey")}
        sp = self._sp()
        fe = lib().orc_phys_fields(C.byref(self.cfg), sp, _p(out["rho"]), _p(out["phi"]),
                                   _p(out["ex"]), _p(out["ey"]), nthreads)
        out["fe"] = fe
        return out

    def prime(self, nthreads=0):
        lib().orc_phys_prime(C.byref(self.cfg), self._sp(), nthreads)

    def run(self, nsteps, nthreads=0):
        g = (self.cfg.ny, self.cfg.nx)
        h = dict(fe=np.empty(nsteps + 1), ke=np.empty(nsteps), px=np.empty(nsteps),
                 py=np.empty(nsteps))
        out = {k: np.empty(g) for k in ("rho", "phi", "ex", "ey")}
        lib().orc_phys_run(C.byref(self.cfg), self._sp(), nsteps, _p(h["fe"]), _p(h["ke"]),
                           _p(h["px"]), _p(h["py"]), _p(out["rho"]), _p(out["phi"]),
                           _p(out["ex"]), _p(out["ey"]), nthreads)
        out.update(h)
        return out


# ------------------------------------------------------ integer restatements ----
def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [int(v) for v in o]


def deposit_fixed(nx, ny, cell, ox, oy, q_int=1, rho=None):
    cell = np.ascontiguousarray(cell, dtype=np.int32)
    ox = np.ascontiguousarray(ox, dtype=np.float32)
    oy = np.ascontiguousarray(oy, dtype=np.float32)
    if rho is None:
        rho = np.zeros(nx * ny, dtype=np.int64)
    lib().orc_deposit_fixed(nx, ny, len(cell), cell.ctypes.data, ox.ctypes.data, oy.ctypes.data,
                            int(q_int), rho.ctypes.data)
    return rho


# ------------------------------------------------------------- collisions ----
class MccC(C.Structure):
    _fields_ = [("ntab", C.c_int), ("e_min", C.c_double), ("e_max", C.c_double),
                ("sel", _dp), ("sexc", _dp), ("sion", _dp), ("ng", C.c_double),
                ("half_me_over_e", C.c_double), ("two_m_over_M", C.c_double),
                ("e_exc", C.c_double), ("e_ion", C.c_double), ("vth_ion", C.c_double),
                ("nu_max", C.c_double), ("p_null", C.c_double), ("seed", C.c_uint64)]


class DsmcC(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("Lx", C.c_double), ("Ly", C.c_double),
                ("dt", C.c_double), ("sigma", C.c_double), ("coef", C.c_double),
                ("mass", C.c_double), ("seed", C.c_uint64)]


def mcc_pass(m: dict, pid, vx, vy, vz, pass_no, cap_new=None):
    """One MCC pass (restatement).  m: dict with the MccC fields, tables as
    numpy arrays.  Returns (vx, vy, vz, new_e (k,3), new_i (k,3), parent, counts)."""
    L = lib()
    L.orc_mcc_pass.restype = C.c_long
    L.orc_mcc_pass.argtypes = [C.POINTER(MccC), C.c_long, C.c_void_p, _dp, _dp, _dp, C.c_uint64,
                               C.c_long, _dp, _dp, C.c_void_p, C.c_void_p]
    tabs = [np.ascontiguousarray(m[k], dtype=np.float64) for k in ("sel", "sexc", "sion")]
    mc = MccC(len(tabs[0]), m["e_min"], m["e_max"], *[_p(t) for t in tabs], m["ng"],
              m["half_me_over_e"], m["two_m_over_M"], m["e_exc"], m["e_ion"], m["vth_ion"],
              m["nu_max"], m["p_null"], m["seed"])
    vx, vy, vz = (np.array(a, dtype=np.float64) for a in (vx, vy, vz))
    pid = np.ascontiguousarray(pid, dtype=np.uint32)
    n = len(vx)
    cap = n if cap_new is None else cap_new
    ne, ni = np.zeros((cap, 3)), np.zeros((cap, 3))
    parent = np.zeros(cap, dtype=np.int64)
    counts = np.zeros(4, dtype=np.int64)
    born = L.orc_mcc_pass(C.byref(mc), n, pid.ctypes.data, _p(vx), _p(vy), _p(vz), pass_no, cap,
                          _p(ne), _p(ni), parent.ctypes.data, counts.ctypes.data)
    return vx, vy, vz, ne[:born], ni[:born], parent[:born], counts


def mcc_passes(m: dict, pid, vx, vy, vz, first_pass, npasses, nthreads=0):
    """npasses MCC passes over fixed electrons (no field, newborns not kept):
    returns (vx, vy, vz, counts)."""
    L = lib()
    L.orc_mcc_passes.restype = None
    L.orc_mcc_passes.argtypes = [C.POINTER(MccC), C.c_long, C.c_void_p, _dp, _dp, _dp,
                                 C.c_uint64, C.c_long, C.c_void_p, C.c_int]
    tabs = [np.ascontiguousarray(m[k], dtype=np.float64) for k in ("sel", "sexc", "sion")]
    mc = MccC(len(tabs[0]), m["e_min"], m["e_max"], *[_p(t) for t in tabs], m["ng"],
              m["half_me_over_e"], m["two_m_over_M"], m["e_exc"], m["e_ion"], m["vth_ion"],
              m["nu_max"], m["p_null"], m["seed"])
    vx, vy, vz = (np.array(a, dtype=np.float64) for a in (vx, vy, vz))
    pid = np.ascontiguousarray(pid, dtype=np.uint32)
    counts = np.zeros(4, dtype=np.int64)
    L.orc_mcc_passes(C.byref(mc), len(vx), pid.ctypes.data, _p(vx), _p(vy), _p(vz), first_pass,
                     npasses, counts.ctypes.data, nthreads)
    return vx, vy, vz, counts


def dsmc_run(d: dict, x, y, vx, vy, vz, sgmax, nsteps, first_pass=0):
    L = lib()
    L.orc_dsmc_run.restype = None
    L.orc_dsmc_run.argtypes = [C.POINTER(DsmcC), C.c_long, _dp, _dp, _dp, _dp, _dp, _dp,
                               C.c_long, C.c_uint64, _dp, _dp, C.c_void_p]
    dc = DsmcC(d["nx"], d["ny"], d["Lx"], d["Ly"], d["dt"], d["sigma"], d["coef"], d["mass"],
               d["seed"])
    x, y, vx, vy, vz = (np.array(a, dtype=np.float64) for a in (x, y, vx, vy, vz))
    sg = np.array(sgmax, dtype=np.float64)
    te, to = np.zeros(nsteps), np.zeros(nsteps)
    counts = np.zeros(2, dtype=np.int64)
    L.orc_dsmc_run(C.byref(dc), len(x), _p(x), _p(y), _p(vx), _p(vy), _p(vz), _p(sg), nsteps,
                   first_pass, _p(te), _p(to), counts.ctypes.data)
    return dict(x=x, y=y, vx=vx, vy=vy, vz=vz, T_even=te, T_odd=to, counts=counts)


# ---------------------------------------------------------------- adjoint ----
def adjoint(cfg: PhysCfg, x0, y0, vx0, vy0, q, m, nsteps, nthreads=0):
    """FP64 forward + adjoint (restatement): returns (J, dJ/dx0, dJ/dy0, dJ/dvx0, dJ/dvy0)."""
    L = lib()
    L.orc_adjoint.restype = C.c_double
    L.orc_adjoint.argtypes = [C.POINTER(PhysCfg), C.c_long, C.c_double, C.c_double, _dp, _dp, _dp,
                              _dp, C.c_long, _dp, _dp, _dp, _dp, C.c_int]
    x0, y0, vx0, vy0 = (_f64(a) for a in (x0, y0, vx0, vy0))
    n = len(x0)
    out = [np.empty(n) for _ in range(4)]
    J = L.orc_adjoint(C.byref(cfg), n, q, m, _p(x0), _p(y0), _p(vx0), _p(vy0), nsteps,
                      *[_p(o) for o in out], nthreads)
    return (J, *out)


def forward_J(cfg: PhysCfg, x0, y0, vx0, vy0, q, m, nsteps, nthreads=0):
    L = lib()
    L.orc_forward_J.restype = C.c_double
    L.orc_forward_J.argtypes = [C.POINTER(PhysCfg), C.c_long, C.c_double, C.c_double, _dp, _dp,
                                _dp, _dp, C.c_long, C.c_int]
    x0, y0, vx0, vy0 = (_f64(a) for a in (x0, y0, vx0, vy0))
    return L.orc_forward_J(C.byref(cfg), len(x0), q, m, _p(x0), _p(y0), _p(vx0), _p(vy0), nsteps,
                           nthreads)

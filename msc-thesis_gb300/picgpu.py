"""Python binding of libpic's C ABI (include/pic.h) through ctypes.

This is the host-side mirror of the reference's step interface
(taylorj5/msc-thesis thesisCode/collisionless/double/src/main.cc:137-172):
``Handle.init_particles`` / ``set_particles`` (initialiseParticles,
Particle::Particle), ``deposit`` (Grid::chargeAssignment), ``poisson``
(fftPoissonSolver + Grid::computeElectricField), ``gather_push``
(Particle::forceCalculation + positionUpdate), ``collide``, ``step`` and
``diagnostics``; ``compat_run`` is the drop-in for picFloatGpu.

Every failing call raises ``PicError`` with the library's status and message.
There is no fallback: if libpic.so is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpic.so")

MAX_SPECIES = 4
SPECIES_HAS_VZ = 1
LOAD_RANDOM, LOAD_LATTICE = 0, 1
PERT_NONE, PERT_XDISP, PERT_DENSITY, PERT_BEAM_MODE = 0, 1, 2, 3
COLLIDE_MCC, COLLIDE_DSMC = 1, 2
GRID_RHO, GRID_PHI, GRID_EX, GRID_EY = 0, 1, 2, 3
HIST_FIELD_ENERGY, HIST_KINETIC, HIST_MOMENTUM_X, HIST_MOMENTUM_Y, HIST_CHARGE, HIST_MODE_AMP = range(6)
DEVERR_NAN, DEVERR_CAPACITY, DEVERR_CELL, DEVERR_TIMEOUT, DEVERR_SORT = 1, 2, 4, 8, 16

STATUS = {0: "PIC_OK", 1: "PIC_ERR_INVALID_ARG", 2: "PIC_ERR_OOM", 3: "PIC_ERR_CUDA",
          4: "PIC_ERR_CUFFT", 5: "PIC_ERR_OVERFLOW", 6: "PIC_ERR_NAN", 7: "PIC_ERR_TIMEOUT",
          8: "PIC_ERR_STATE", 9: "PIC_ERR_NO_DEVICE"}


class PicError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")
        self.status = status


class RefParams(C.Structure):
    """pic_ref_params: the reference's Params fields (inc/params.h:21-47)."""

    _fields_ = [("xDim", C.c_int), ("yDim", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("npx", C.c_int), ("npy", C.c_int), ("dt", C.c_double), ("tmax", C.c_double),
                ("charge", C.c_double), ("mass", C.c_double), ("vtx", C.c_double),
                ("vty", C.c_double), ("vdx", C.c_double), ("vdy", C.c_double)]


class SpeciesDesc(C.Structure):
    _fields_ = [("capacity", C.c_longlong), ("q", C.c_double), ("m", C.c_double),
                ("q_int", C.c_int), ("flags", C.c_int)]


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("Lx", C.c_double), ("Ly", C.c_double),
                ("dt", C.c_double), ("eps0", C.c_double), ("nspecies", C.c_int),
                ("species", SpeciesDesc * MAX_SPECIES), ("sort_every", C.c_int),
                ("tile_w", C.c_int), ("tile_h", C.c_int), ("chunk", C.c_int), ("halo", C.c_int),
                ("history", C.c_int), ("device", C.c_int), ("push_variant", C.c_int)]


class InitSpec(C.Structure):
    _fields_ = [("n", C.c_longlong), ("layout", C.c_int), ("pert_kind", C.c_int),
                ("vth", C.c_double * 3), ("vdrift", C.c_double * 2), ("beam_v", C.c_double),
                ("pert_amp", C.c_double), ("pert_mx", C.c_int), ("pert_my", C.c_int),
                ("seed", C.c_ulonglong), ("beam_xi", (C.c_double * 2) * 2),
                ("beam_u", (C.c_double * 2) * 2)]


class Diag(C.Structure):
    _fields_ = [("step", C.c_longlong), ("field_energy", C.c_double),
                ("kinetic_energy", C.c_double), ("momentum", C.c_double * 2),
                ("total_charge_fixed", C.c_longlong), ("expected_charge_fixed", C.c_longlong),
                ("n", C.c_longlong * MAX_SPECIES), ("error_flags", C.c_uint)]


class MccParams(C.Structure):
    _fields_ = [("electron_species", C.c_int), ("ion_species", C.c_int),
                ("neutral_density", C.c_double), ("neutral_temp_eV", C.c_double),
                ("electron_mass", C.c_double), ("ion_mass", C.c_double),
                ("unit_charge", C.c_double), ("ntab", C.c_int), ("e_min_eV", C.c_double),
                ("e_max_eV", C.c_double), ("sigma_elastic", C.POINTER(C.c_double)),
                ("sigma_excitation", C.POINTER(C.c_double)),
                ("sigma_ionization", C.POINTER(C.c_double)), ("e_exc_eV", C.c_double),
                ("e_ion_eV", C.c_double), ("seed", C.c_ulonglong)]


class DsmcParams(C.Structure):
    _fields_ = [("species", C.c_int), ("diameter", C.c_double), ("weight", C.c_double),
                ("depth", C.c_double), ("sigma_g_max0", C.c_double), ("seed", C.c_ulonglong)]


class TuneResult(C.Structure):
    _fields_ = [("chunk", C.c_int), ("tile_w", C.c_int), ("tile_h", C.c_int),
                ("sort_every", C.c_int), ("ms_per_step", C.c_double), ("tried", C.c_int)]


class AdjointResult(C.Structure):
    _fields_ = [("J", C.c_double), ("dJ_dbeam_v", C.c_double), ("dJ_damp", C.c_double)]


class ParticlesView(C.Structure):
    _fields_ = [("n", C.c_longlong), ("cell_dev", C.c_void_p), ("ox_dev", C.c_void_p),
                ("oy_dev", C.c_void_p), ("vx_dev", C.c_void_p), ("vy_dev", C.c_void_p),
                ("vz_dev", C.c_void_p), ("pid_dev", C.c_void_p)]


_dp = C.POINTER(C.c_double)
_vp = C.c_void_p
_H = C.c_void_p

# name -> argtypes (restype is pic_status / int unless listed in _RESTYPES)
SIGNATURES = {
    "pic_status_string": [C.c_int],
    "pic_last_error": [],
    "pic_version": [],
    "pic_compat_run": [C.POINTER(RefParams), _dp, _dp, _dp, _dp, _dp, _dp, _dp],
    "pic_compat_run_steps": [C.POINTER(RefParams), _dp, _dp, _dp, _dp, C.c_longlong,
                             _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp],
    "pic_config_default": [C.POINTER(Config)],
    "pic_create": [C.POINTER(Config), C.POINTER(_H)],
    "pic_destroy": [_H],
    "pic_get_stream": [_H, C.POINTER(_vp)],
    "pic_synchronize": [_H],
    "pic_init_particles": [_H, C.c_int, C.POINTER(InitSpec)],
    "pic_set_particles": [_H, C.c_int, C.c_longlong, _vp, _vp, _vp, _vp, _vp],
    "pic_get_particles": [_H, C.c_int, C.POINTER(C.c_longlong), _vp, _vp, _vp, _vp, _vp],
    "pic_get_particles_raw": [_H, C.c_int, C.POINTER(C.c_longlong), _vp, _vp, _vp, _vp, _vp, _vp],
    "pic_particles_device": [_H, C.c_int, C.POINTER(ParticlesView)],
    "pic_prime_leapfrog": [_H],
    "pic_sort": [_H],
    "pic_deposit": [_H],
    "pic_poisson": [_H],
    "pic_gather_push": [_H, C.c_int],
    "pic_collide": [_H, C.c_int],
    "pic_set_mcc": [_H, C.POINTER(MccParams)],
    "pic_set_dsmc": [_H, C.POINTER(DsmcParams)],
    "pic_collision_counts": [_H, _vp],
    "pic_autotune": [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p],
    "pic_save": [_H, C.c_char_p],
    "pic_load": [_H, C.c_char_p],
    "pic_adjoint_run": [_H, _vp, C.c_longlong, C.c_int, _vp, _vp, _vp, _vp,
                        C.POINTER(AdjointResult)],
    "pic_step": [_H, C.c_longlong],
    "pic_ensemble_create": [C.c_void_p, C.c_int, C.POINTER(_H)],
    "pic_ensemble_destroy": [_H],
    "pic_ensemble_get_stream": [_H, C.POINTER(_vp)],
    "pic_ensemble_synchronize": [_H],
    "pic_ensemble_init": [_H, C.c_void_p],
    "pic_ensemble_step": [_H, C.c_longlong],
    "pic_ensemble_diagnostics": [_H, C.c_int, C.POINTER(Diag)],
    "pic_ensemble_get_history": [_H, C.c_int, C.c_int, C.c_longlong, C.c_longlong, _vp],
    "pic_ensemble_get_particles": [_H, C.c_int, C.POINTER(C.c_longlong), _vp, _vp, _vp, _vp],
    "pic_ensemble_autotune": [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p],
    "pic_ensemble_adjoint": [_H, C.c_void_p, C.c_longlong, C.c_int, _vp, _vp, _vp, _vp, C.c_void_p],
    "pic_run_host": [_H, C.c_longlong, _vp, _vp, _vp, _vp, C.c_longlong, C.c_int,
                     _vp, _vp, _vp, _vp],
    "pic_diagnostics": [_H, C.POINTER(Diag)],
    "pic_get_history": [_H, C.c_int, C.c_longlong, C.c_longlong, _vp],
    "pic_track_mode": [_H, C.c_int, C.c_int],
    "pic_get_grid": [_H, C.c_int, _vp],
    "pic_get_rho_fixed": [_H, _vp],
    "pic_deposit_grid": [C.c_int, C.c_int, C.c_longlong, _vp, _vp, _vp, C.c_int, C.c_double,
                         _vp, _vp],
    "pic_deposit_grid_noalloc": [C.c_int, C.c_int, C.c_longlong, _vp, _vp, _vp, C.c_int,
                                 C.c_double, _vp, _vp],
}
NOALLOC_MAX_CELLS = 1 << 20
_RESTYPES = {"pic_status_string": C.c_char_p, "pic_last_error": C.c_char_p,
             "pic_version": C.c_char_p}

_lib = None


def load(path: str = LIB_PATH):
    """Load libpic.so (raises OSError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise OSError(f"libpic.so not built at {path}; run msc-thesis_gb300/build_lib.py")
        L = C.CDLL(path)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPES.get(name, C.c_int)
        _lib = L
    return _lib


def _check(status: int, where: str):
    if status != 0:
        msg = load().pic_last_error().decode(errors="replace")
        raise PicError(status, where, msg)


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ------------------------------------------------------------ compat ----
def ref_params(**kw) -> RefParams:
    """Defaults are the reference's struct Params defaults (params.h:22-42)."""
    d = dict(xDim=10, yDim=10, nx=32, ny=32, npx=10, npy=10, dt=1e-7, tmax=1e-4,
             charge=-100.0, mass=100.0, vtx=1.0, vty=1.0, vdx=0.0, vdy=0.0)
    d.update(kw)
    return RefParams(**d)


def compat_run(p: RefParams, x, y, vx, vy):
    """picFloatGpu drop-in: returns (xOut, yOut, seconds)."""
    x, y, vx, vy = (_f64(a) for a in (x, y, vx, vy))
    n = p.npx * p.npy
    xo, yo = np.empty(n), np.empty(n)
    sec = C.c_double(0)
    dp = lambda a: a.ctypes.data_as(_dp)
    _check(load().pic_compat_run(C.byref(p), dp(x), dp(y), dp(vx), dp(vy), dp(xo), dp(yo),
                                 C.byref(sec)), "pic_compat_run")
    return xo, yo, sec.value


def compat_run_steps(p: RefParams, x, y, vx, vy, nsteps: int):
    x, y, vx, vy = (_f64(a) for a in (x, y, vx, vy))
    n = p.npx * p.npy
    out = {k: np.empty(n) for k in ("x", "y", "vx", "vy")}
    g = (p.nx + 2, p.ny + 2)
    out.update({k: np.empty(g) for k in ("rho", "phi", "ex", "ey")})
    dp = lambda a: a.ctypes.data_as(_dp)
    _check(load().pic_compat_run_steps(C.byref(p), dp(x), dp(y), dp(vx), dp(vy), nsteps,
                                       *[dp(out[k]) for k in ("x", "y", "vx", "vy", "rho",
                                                             "phi", "ex", "ey")]),
           "pic_compat_run_steps")
    return out


def deposit_grid(nx, ny, n, cell_ptr, ox_ptr, oy_ptr, q_int, scale, rho_ptr, stream=None):
    """Stateless deposit of device arrays (integer device pointers)."""
    _check(load().pic_deposit_grid(nx, ny, n, cell_ptr, ox_ptr, oy_ptr, q_int, scale, rho_ptr,
                                   stream), "pic_deposit_grid")


def deposit_grid_noalloc(nx, ny, n, cell_ptr, ox_ptr, oy_ptr, q_int, scale, rho_ptr,
                         stream=None):
    """The same deposit from the library's static scratch grid: allocates no
    device memory; enqueues on `stream` and returns (see include/pic.h)."""
    _check(load().pic_deposit_grid_noalloc(nx, ny, n, cell_ptr, ox_ptr, oy_ptr, q_int, scale,
                                           rho_ptr, stream), "pic_deposit_grid_noalloc")


def autotune(cfg: Config, species: int, spec: InitSpec, trial_steps: int = 40) -> TuneResult:
    """Time candidate push chunks and sort cadences on this workload; the
    chosen values are written into cfg (see pic_autotune in include/pic.h)."""
    r = TuneResult()
    _check(load().pic_autotune(C.addressof(cfg), species, C.addressof(spec), trial_steps,
                               C.addressof(r)), "pic_autotune")
    return r


# ------------------------------------------------------------ handle ----
def species(capacity, q, m, q_int, flags=0) -> SpeciesDesc:
    return SpeciesDesc(int(capacity), float(q), float(m), int(q_int), int(flags))


def config(nx, ny, Lx, Ly, dt, species_list, eps0=1.0, **tuning) -> Config:
    c = Config()
    _check(load().pic_config_default(C.byref(c)), "pic_config_default")
    c.nx, c.ny, c.Lx, c.Ly, c.dt, c.eps0 = nx, ny, Lx, Ly, dt, eps0
    c.nspecies = len(species_list)
    for i, s in enumerate(species_list):
        c.species[i] = s
    for k, v in tuning.items():
        setattr(c, k, v)
    return c


def init_spec(n, layout=LOAD_RANDOM, vth=(0.0, 0.0, 0.0), vdrift=(0.0, 0.0), beam_v=0.0,
              pert_kind=PERT_NONE, pert_amp=0.0, pert_mx=0, pert_my=0, seed=0,
              beam_xi=((0, 0), (0, 0)), beam_u=((0, 0), (0, 0))) -> InitSpec:
    s = InitSpec()
    s.n, s.layout, s.pert_kind = int(n), layout, pert_kind
    for i in range(3):
        s.vth[i] = float(vth[i]) if i < len(vth) else 0.0
    s.vdrift[0], s.vdrift[1] = float(vdrift[0]), float(vdrift[1])
    s.beam_v, s.pert_amp, s.pert_mx, s.pert_my, s.seed = beam_v, pert_amp, pert_mx, pert_my, seed
    for b in range(2):
        for c in range(2):
            s.beam_xi[b][c] = float(beam_xi[b][c])
            s.beam_u[b][c] = float(beam_u[b][c])
    return s


def two_stream_growing_mode(k, v0, omega_b2=0.5, amp=1e-4):
    """Linear growing eigenmode of two symmetric cold beams (+v0, -v0), each
    with plasma frequency^2 omega_b2, at wavenumber k (plasma units, q/m = -1).
    Returns (gamma, beam_xi, beam_u) for PERT_BEAM_MODE, scaled so that the
    total density perturbation has amplitude `amp` (relative)."""
    n0 = 1.0  # per-beam density in units where omega_b2 = n0 * q^2 / m
    M = np.zeros((4, 4), complex)
    for j, v in enumerate((v0, -v0)):
        M[j, j] = -1j * k * v
        M[j, 2 + j] = -1j * k * n0
        M[2 + j, 2 + j] = -1j * k * v
        M[2 + j, 0] += omega_b2 / (1j * k)
        M[2 + j, 1] += omega_b2 / (1j * k)
    w, V = np.linalg.eig(M)
    g = int(np.argmax(w.real))
    vec = V[:, g]
    # relative density of each beam n_b/n0; displacement xi = i n_b / (k n0)
    scale = amp / abs(vec[0] + vec[1]) * 2.0
    vec = vec * scale
    xi = [1j * vec[j] / k for j in range(2)]
    u = [vec[2 + j] for j in range(2)]
    return (float(w[g].real), tuple((z.real, z.imag) for z in xi),
            tuple((z.real, z.imag) for z in u))


class Handle:
    """One simulation on one GPU (owns a CUDA stream and its device buffers)."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        h = C.c_void_p()
        _check(load().pic_create(C.byref(cfg), C.byref(h)), "pic_create")
        self.h = h
        self.ncell = cfg.nx * cfg.ny

    def close(self):
        if self.h:
            load().pic_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, name, *args):
        _check(getattr(load(), name)(self.h, *args), name)

    # ---- particles
    def init_particles(self, s: int, spec: InitSpec):
        self._c("pic_init_particles", s, C.byref(spec))

    def set_particles(self, s, x, y, vx, vy, vz=None):
        x, y, vx, vy = (_f64(a) for a in (x, y, vx, vy))
        vz = None if vz is None else _f64(vz)
        self._keep = (x, y, vx, vy, vz)
        self._c("pic_set_particles", s, len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(vz))

    def count(self, s=0) -> int:
        n = C.c_longlong()
        self._c("pic_get_particles", s, C.byref(n), None, None, None, None, None)
        return n.value

    def get_particles(self, s=0, vz=False):
        n = C.c_longlong()
        self._c("pic_get_particles", s, C.byref(n), None, None, None, None, None)
        a = {k: np.empty(n.value) for k in ("x", "y", "vx", "vy")}
        if vz:
            a["vz"] = np.empty(n.value)
        self._c("pic_get_particles", s, C.byref(n), _ptr(a["x"]), _ptr(a["y"]), _ptr(a["vx"]),
                _ptr(a["vy"]), _ptr(a.get("vz")))
        return a

    def get_particles_raw(self, s=0):
        n = C.c_longlong()
        self._c("pic_get_particles_raw", s, C.byref(n), None, None, None, None, None, None)
        m = n.value
        a = dict(cell=np.empty(m, np.int32), ox=np.empty(m, np.float32),
                 oy=np.empty(m, np.float32), vx=np.empty(m, np.float32),
                 vy=np.empty(m, np.float32), pid=np.empty(m, np.uint32))
        self._c("pic_get_particles_raw", s, C.byref(n), *[_ptr(a[k]) for k in
                                                         ("cell", "ox", "oy", "vx", "vy", "pid")])
        return a

    def particles_device(self, s=0) -> ParticlesView:
        v = ParticlesView()
        self._c("pic_particles_device", s, C.byref(v))
        return v

    # ---- stages
    def prime_leapfrog(self):
        self._c("pic_prime_leapfrog")

    def sort(self):
        self._c("pic_sort")

    def deposit(self):
        self._c("pic_deposit")

    def poisson(self):
        self._c("pic_poisson")

    def gather_push(self, deposit=True):
        self._c("pic_gather_push", 1 if deposit else 0)

    def collide(self, kind):
        self._c("pic_collide", kind)

    def step(self, n=1):
        self._c("pic_step", int(n))

    def set_mcc(self, electron_species, ion_species, neutral_density, neutral_temp_eV,
                electron_mass, ion_mass, unit_charge, e_min_eV, e_max_eV, sigma_elastic,
                sigma_excitation, sigma_ionization, e_exc_eV, e_ion_eV, seed=0):
        tabs = [_f64(t) for t in (sigma_elastic, sigma_excitation, sigma_ionization)]
        self._mcc_tabs = tabs
        p = MccParams(electron_species, ion_species, neutral_density, neutral_temp_eV,
                      electron_mass, ion_mass, unit_charge, len(tabs[0]), e_min_eV, e_max_eV,
                      *[t.ctypes.data_as(_dp) for t in tabs], e_exc_eV, e_ion_eV, seed)
        self._c("pic_set_mcc", C.byref(p))

    def set_dsmc(self, species, diameter, weight, depth, sigma_g_max0, seed=0):
        p = DsmcParams(species, diameter, weight, depth, sigma_g_max0, seed)
        self._c("pic_set_dsmc", C.byref(p))

    def save(self, path):
        self._c("pic_save", os.fsencode(path))

    def load(self, path):
        self._c("pic_load", os.fsencode(path))

    def adjoint(self, nsteps, every=10, spec: InitSpec | None = None):
        """Final field energy J and its gradients with respect to the initial
        state (pic_adjoint_run).  Returns (AdjointResult, dJ/dx0, dJ/dy0,
        dJ/dvx0, dJ/dvy0), arrays in particle-id order."""
        n = spec.n if spec is not None else self.count(0)
        out = [np.empty(n) for _ in range(4)]
        r = AdjointResult()
        self._c("pic_adjoint_run", C.addressof(spec) if spec is not None else None, int(nsteps),
                int(every), *[_ptr(o) for o in out], C.byref(r))
        return (r, *out)

    def collision_counts(self):
        c = np.zeros(6, dtype=np.int64)
        self._c("pic_collision_counts", _ptr(c))
        return c

    def synchronize(self):
        self._c("pic_synchronize")

    def stream(self) -> int:
        s = C.c_void_p()
        self._c("pic_get_stream", C.byref(s))
        return s.value or 0

    def run_host(self, x, y, vx, vy, nsteps, prime=True, out=None):
        n = len(x)
        if out is None:
            out = [np.empty(n) for _ in range(4)]
        self._c("pic_run_host", n, _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), int(nsteps),
                1 if prime else 0, *[_ptr(o) for o in out])
        return out

    # ---- diagnostics
    def diagnostics(self) -> Diag:
        d = Diag()
        self._c("pic_diagnostics", C.byref(d))
        return d

    def history(self, which, first, count):
        out = np.empty(count)
        self._c("pic_get_history", which, first, count, _ptr(out))
        return out

    def track_mode(self, mx, my):
        self._c("pic_track_mode", mx, my)

    def grid(self, which):
        out = np.empty((self.cfg.ny, self.cfg.nx))
        self._c("pic_get_grid", which, _ptr(out))
        return out

    def rho_fixed(self):
        out = np.empty((self.cfg.ny, self.cfg.nx), np.int64)
        self._c("pic_get_rho_fixed", _ptr(out))
        return out


def ensemble_autotune(cfgs, specs, trial_steps: int = 20) -> TuneResult:
    """Pick chunk and sort cadence for an ensemble (pic_ensemble_autotune); the
    chosen values are written into cfgs[0]."""
    arr = (Config * len(cfgs))(*cfgs)
    sp = (InitSpec * len(specs))(*specs)
    r = TuneResult()
    _check(load().pic_ensemble_autotune(C.addressof(arr), len(cfgs), C.addressof(sp), trial_steps,
                                        C.addressof(r)), "pic_ensemble_autotune")
    cfgs[0].chunk, cfgs[0].sort_every = arr[0].chunk, arr[0].sort_every
    return r


class Ensemble:
    """Many independent collisionless runs advanced together (pic_ensemble_*):
    one Config per run (one charged species each); chunk, halo, sort_every,
    history and device come from the first."""

    def __init__(self, cfgs):
        self.cfgs = list(cfgs)
        arr = (Config * len(self.cfgs))(*self.cfgs)
        h = C.c_void_p()
        _check(load().pic_ensemble_create(C.addressof(arr), len(self.cfgs), C.byref(h)),
               "pic_ensemble_create")
        self.h = h

    def close(self):
        if self.h:
            load().pic_ensemble_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, name, *args):
        _check(getattr(load(), name)(self.h, *args), name)

    def init(self, specs):
        arr = (InitSpec * len(specs))(*specs)
        self._c("pic_ensemble_init", C.addressof(arr))

    def step(self, n=1):
        self._c("pic_ensemble_step", int(n))

    def synchronize(self):
        self._c("pic_ensemble_synchronize")

    def stream(self) -> int:
        s = C.c_void_p()
        self._c("pic_ensemble_get_stream", C.byref(s))
        return s.value or 0

    def diagnostics(self, run) -> Diag:
        d = Diag()
        self._c("pic_ensemble_diagnostics", run, C.byref(d))
        return d

    def history(self, run, which, first, count):
        out = np.empty(count)
        self._c("pic_ensemble_get_history", run, which, first, count, _ptr(out))
        return out

    def adjoint(self, specs, nsteps, every=50, gradients=True):
        """pic_ensemble_adjoint: per run (J, dJ/d beam_v, dJ/d pert_amp) and, with
        gradients, per run the arrays (dJ/dx0, dJ/dy0, dJ/dvx0, dJ/dvy0) in id order."""
        sp = (InitSpec * len(specs))(*specs)
        res = (AdjointResult * len(specs))()
        total = sum(int(x.n) for x in specs)
        arrs = [np.empty(total) for _ in range(4)] if gradients else [None] * 4
        self._c("pic_ensemble_adjoint", C.addressof(sp), int(nsteps), int(every),
                *[_ptr(a) for a in arrs], C.addressof(res))
        out = [(r.J, r.dJ_dbeam_v, r.dJ_damp) for r in res]
        if not gradients:
            return out, None
        per, k = [], 0
        for x in specs:
            per.append(tuple(a[k:k + x.n] for a in arrs))
            k += x.n
        return out, per

    def get_particles(self, run):
        n = C.c_longlong()
        self._c("pic_ensemble_get_particles", run, C.byref(n), None, None, None, None)
        a = {k: np.empty(n.value) for k in ("x", "y", "vx", "vy")}
        self._c("pic_ensemble_get_particles", run, C.byref(n), *[_ptr(a[k]) for k in
                                                                ("x", "y", "vx", "vy")])
        return a


def field_energy_function(handle: Handle, nsteps: int, every: int = 10):
    """A torch.autograd.Function for J(x0, y0, vx0, vy0) = field energy after
    `nsteps` steps of `handle`'s species 0 from that initial state (unprimed).
    The forward pass runs pic_adjoint_run, so the gradients are computed with
    J; backward scales them by the incoming gradient.  Inputs are 1-D tensors
    of one length (any device, float64 recommended); they pass through host
    memory."""
    import torch

    class _FieldEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, y0, vx0, vy0):
            arrs = [t.detach().to("cpu", torch.float64).numpy() for t in (x0, y0, vx0, vy0)]
            handle.set_particles(0, *arrs)
            r, *grads = handle.adjoint(nsteps, every)
            ctx.save_for_backward(*[torch.from_numpy(g).to(x0.device, x0.dtype) for g in grads])
            return x0.new_tensor(r.J)

        @staticmethod
        def backward(ctx, gJ):
            return tuple(gJ * g for g in ctx.saved_tensors)

    return _FieldEnergy.apply


def ensemble_field_energy_function(ensemble: Ensemble, specs, nsteps: int, every: int = 50):
    """A torch.autograd.Function for the batched runs of `ensemble`:
    (beam_v, pert_amp), two 1-D tensors with one entry per run, -> J, the
    final field energy of every run after `nsteps` steps from specs[r] with
    those two entries replaced.  The forward pass runs pic_ensemble_adjoint,
    so dJ_r/d beam_v_r and dJ_r/d pert_amp_r come with J; backward scales them
    by the incoming gradient (each J_r depends on its own run's two entries
    only).  Values pass through host memory."""
    import copy

    import torch

    base = [copy.copy(s) for s in specs]

    class _EnsembleFieldEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, beam_v, pert_amp):
            bv = beam_v.detach().to("cpu", torch.float64).numpy()
            pa = pert_amp.detach().to("cpu", torch.float64).numpy()
            if len(bv) != len(base) or len(pa) != len(base):
                raise ValueError("one beam_v and one pert_amp per run")
            run = []
            for s, b, a in zip(base, bv, pa):
                t = copy.copy(s)
                t.beam_v, t.pert_amp = float(b), float(a)
                run.append(t)
            out, _ = ensemble.adjoint(run, nsteps, every, gradients=False)
            J = torch.tensor([o[0] for o in out], dtype=beam_v.dtype, device=beam_v.device)
            gb = torch.tensor([o[1] for o in out], dtype=beam_v.dtype, device=beam_v.device)
            ga = torch.tensor([o[2] for o in out], dtype=pert_amp.dtype, device=pert_amp.device)
            ctx.save_for_backward(gb, ga)
            return J

        @staticmethod
        def backward(ctx, gJ):
            gb, ga = ctx.saved_tensors
            return gJ * gb, gJ * ga

    return _EnsembleFieldEnergy.apply

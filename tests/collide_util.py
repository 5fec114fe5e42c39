"""Shared setup of the collision tests (not a test module): the
electron-neutral cross sections of the 512^2 MCC workload and the
constants pic_set_mcc derives from them."""
import numpy as np

E_CH = 1.602176634e-19
ME = 9.1093837015e-31
KB = 1.380649e-23
MI = 73000.0 * ME          # singly charged ion, mass ratio 1/73,000
M_NEUTRAL = 6.6e-26        # hard-sphere neutral of the DSMC workload
D_NEUTRAL = 3.6e-10
NG = 3.2e21                # background neutral density, m^-3
TN_EV = KB * 300.0 / E_CH  # 300 K


def mcc_cross_sections(ntab=256, emin=0.01, emax=1000.0):
    """256 log-spaced energies 0.01..1000 eV: elastic 5e-20 m^2; excitation
    from 11.5 eV rising linearly to 2e-20 at 30 eV, then flat; ionisation from
    15.8 eV rising linearly to 3e-20 at 100 eV, then flat."""
    E = emin * (emax / emin) ** (np.arange(ntab) / (ntab - 1))
    sel = np.full(ntab, 5e-20)
    sexc = np.where(E < 11.5, 0.0, np.where(E < 30.0, 2e-20 * (E - 11.5) / (30.0 - 11.5), 2e-20))
    sion = np.where(E < 15.8, 0.0, np.where(E < 100.0, 3e-20 * (E - 15.8) / (100.0 - 15.8), 3e-20))
    return E, sel, sexc, sion


def mcc_resolved(dt, seed, ntab=256, emin=0.01, emax=1000.0):
    """The constants pic_set_mcc derives (nu_max, P_null rounded to float as
    the GPU uses them), as a dict for the oracle's orc_mcc_pass."""
    E, sel, sexc, sion = mcc_cross_sections(ntab, emin, emax)
    v = np.sqrt(2.0 * E * E_CH / ME)
    st = sel + sexc + sion
    nu_max = NG * 1.0001 * np.max(np.maximum(st[:-1], st[1:]) * v[1:])
    p_null = 1.0 - np.exp(-nu_max * dt)
    return dict(e_min=emin, e_max=emax, sel=sel, sexc=sexc, sion=sion, ng=NG,
                half_me_over_e=float(np.float32(0.5 * ME / E_CH)),
                two_m_over_M=float(np.float32(2.0 * ME / MI)), e_exc=11.5, e_ion=15.8,
                vth_ion=float(np.float32(np.sqrt(TN_EV * E_CH / MI))),
                nu_max=float(np.float32(nu_max)), p_null=float(np.float32(p_null)), seed=seed)


def set_tabulated_mcc(h, seed, e=0, i=1):
    E, sel, sexc, sion = mcc_cross_sections()
    h.set_mcc(e, i, NG, TN_EV, ME, MI, E_CH, 0.01, 1000.0, sel, sexc, sion, 11.5, 15.8, seed)


def energies_eV(a):
    return 0.5 * ME * (a["vx"] ** 2 + a["vy"] ** 2 + a["vz"] ** 2) / E_CH


def ks_statistic(a, b):
    a, b = np.sort(a), np.sort(b)
    allv = np.concatenate([a, b])
    return np.max(np.abs(np.searchsorted(a, allv, side="right") / len(a)
                         - np.searchsorted(b, allv, side="right") / len(b)))

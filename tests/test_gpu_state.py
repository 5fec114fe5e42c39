"""State files (pic_save / pic_load): exact resume and rejected files."""
import os
import struct

import numpy as np
import pytest

import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu

NX, NY = 64, 32
HEADER = 8 + 4 + 4 * 2 + 8 * 4 + 4 + 8 * 3  # magic .. dsmc_pass
SPECIES_HEADER = 8 + 4 + 4 + 8 + 8


def make_cfg(n, capacity=None, **kw):
    """Electrons normalised for n particles, room for `capacity`."""
    cfg, q, m = normalized_electrons(NX, NY, 8.0, 4.0, n, 0.1, **kw)
    if capacity is not None:
        cfg.species[0] = P.species(capacity, q, m, -1)
    return cfg


def started_handle(cfg, n, steps):
    h = P.Handle(cfg)
    h.init_particles(0, P.init_spec(n, vth=(0.3, 0.3, 0), pert_kind=P.PERT_DENSITY, pert_amp=0.1,
                                    pert_mx=1, pert_my=1, seed=9))
    h.prime_leapfrog()
    h.step(steps)
    return h


def test_resume_is_bit_exact(tmp_path):
    n = NX * NY * 16
    cfg = make_cfg(n, sort_every=5)
    path = str(tmp_path / "run.picstate")
    with started_handle(cfg, n, 23) as h:
        h.save(path)
        h.step(17)
        a = h.get_particles()
        d = h.diagnostics()
        fe = h.history(P.HIST_FIELD_ENERGY, 23, 18)
    size = os.path.getsize(path)
    assert size == HEADER + SPECIES_HEADER + n * 4 * 6
    with P.Handle(make_cfg(n, capacity=n + 1000, sort_every=7)) as h2:  # more room, other cadence
        h2.load(path)
        assert h2.diagnostics().step == 23
        h2.step(17)
        b = h2.get_particles()
        e = h2.diagnostics()
        fe2 = h2.history(P.HIST_FIELD_ENERGY, 23, 18)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert d.step == e.step == 40
    assert d.field_energy == e.field_energy
    np.testing.assert_array_equal(fe, fe2)


def _corrupt(src, dst, edit):
    raw = bytearray(open(src, "rb").read())
    raw = edit(raw)
    open(dst, "wb").write(bytes(raw))
    return dst


def test_bad_files_are_rejected_and_leave_the_handle_unchanged(tmp_path):
    n = NX * NY * 4
    cfg = make_cfg(n)
    good = str(tmp_path / "good.picstate")
    with started_handle(cfg, n, 5) as h:
        h.save(good)
    body = HEADER + SPECIES_HEADER
    cases = {
        "magic": lambda r: b"XICSTATE" + r[8:],
        "version": lambda r: r[:8] + struct.pack("<I", 2) + r[12:],
        "truncated": lambda r: r[:-3],
        "trailing": lambda r: r + b"\0",
        "grid": lambda r: r[:12] + struct.pack("<i", NX * 2) + r[16:],
        "dt": lambda r: r[:36] + struct.pack("<d", 0.05) + r[44:],
        "eps0": lambda r: r[:44] + struct.pack("<d", 2.0) + r[52:],
        "charge": lambda r: r[:HEADER + 16] + struct.pack("<d", -1.0) + r[HEADER + 24:],
        "mass": lambda r: r[:HEADER + 24] + struct.pack("<d", 1.0) + r[HEADER + 32:],
        "count": lambda r: r[:HEADER] + struct.pack("<q", n + 1) + r[HEADER + 8:],
        "cell": lambda r: r[:body] + struct.pack("<i", NX) + r[body + 4:],
        "offset": lambda r: r[:body + 4 * n] + struct.pack("<f", 1.0) + r[body + 4 * n + 4:],
        "velocity": lambda r: r[:body + 12 * n] + struct.pack("<f", float("nan")) + r[body + 12 * n + 4:],
        "pid": lambda r: r[:body + 20 * n] + r[body + 20 * n + 4:body + 20 * n + 8] + r[body + 20 * n + 4:],
    }
    with started_handle(cfg, n, 3) as h:
        before = h.get_particles()
        for name, edit in cases.items():
            path = _corrupt(good, str(tmp_path / f"{name}.picstate"), edit)
            with pytest.raises(P.PicError) as ei:
                h.load(path)
            assert ei.value.status == 1, name  # PIC_ERR_INVALID_ARG
            after = h.get_particles()
            for k in before:
                np.testing.assert_array_equal(before[k], after[k], err_msg=name)
            assert h.diagnostics().step == 3
        with pytest.raises(P.PicError):
            h.load(str(tmp_path / "missing.picstate"))
        h.load(good)
        assert h.diagnostics().step == 5


def test_small_capacity_is_rejected(tmp_path):
    n = NX * NY * 4
    path = str(tmp_path / "s.picstate")
    with started_handle(make_cfg(n), n, 2) as h:
        h.save(path)
    with P.Handle(make_cfg(n, capacity=n - 4)) as h2:
        with pytest.raises(P.PicError):
            h2.load(path)

"""Imports and exports through packed 32-byte particle records against the
per-field gathers used when the stage may not grow (PIC_STAGE_MAX_BYTES):
identical sorted state, identical runs, identical exports, from page-locked
and from pageable host arrays, with and without a third velocity."""
import os

import numpy as np
import pytest
import torch

import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu

NX, NY = 64, 48


def _particles(n, seed, vz=False):
    rng = np.random.default_rng(seed)
    x = rng.random(n) * 8.0
    y = rng.random(n) * 6.0
    v = [rng.normal(0.0, 0.3, n) for _ in range(3 if vz else 2)]
    return (x, y, *v)


def _run(arrs, n, pinned, lean, steps, vz=False, nx=NX, ny=NY):
    old = os.environ.get("PIC_STAGE_MAX_BYTES")
    if lean:
        os.environ["PIC_STAGE_MAX_BYTES"] = "1"
    try:
        cfg, q, m = normalized_electrons(nx, ny, 8.0, 6.0, n, 0.05, sort_every=7)
        cfg.species[0] = P.species(n + 37, q, m, -1, P.SPECIES_HAS_VZ if vz else 0)
        src = [torch.from_numpy(a).pin_memory().numpy() if pinned else a for a in arrs]
        with P.Handle(cfg) as h:
            h.set_particles(0, *src)
            raw = h.get_particles_raw(0)
            first = h.get_particles(0, vz=vz)
            h.prime_leapfrog()
            h.step(steps)
            d = h.diagnostics()
            out = h.get_particles(0, vz=vz)
            assert d.error_flags == 0
            assert d.total_charge_fixed == d.expected_charge_fixed
            return raw, first, out, d.field_energy
    finally:
        if old is None:
            os.environ.pop("PIC_STAGE_MAX_BYTES", None)
        else:
            os.environ["PIC_STAGE_MAX_BYTES"] = old


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("vz", [False, True])
def test_record_and_per_field_paths_agree(pinned, vz):
    n = NX * NY * 9 + 3  # not a multiple of 4: padded tail slots
    arrs = _particles(n, 11, vz)
    rec = _run(arrs, n, pinned, lean=False, steps=20, vz=vz)
    lean = _run(arrs, n, pinned, lean=True, steps=20, vz=vz)
    for k in rec[0]:
        np.testing.assert_array_equal(rec[0][k], lean[0][k], err_msg="sorted " + k)
    for k in rec[1]:
        np.testing.assert_array_equal(rec[1][k], lean[1][k], err_msg="export " + k)
        np.testing.assert_array_equal(rec[2][k], lean[2][k], err_msg="after steps " + k)
    assert rec[3] == lean[3]
    # the import keeps every particle, in cell-key order, and the export
    # returns them in id (input) order
    cells = rec[0]["cell"][:n]
    assert np.all(cells >= 0)
    assert np.array_equal(np.sort(rec[0]["pid"][:n]), np.arange(n, dtype=np.uint32))
    dx, dy = 8.0 / NX, 6.0 / NY
    assert np.abs(rec[1]["x"] - arrs[0]).max() < 1e-6 * dx + 1e-12
    assert np.abs(rec[1]["y"] - arrs[1]).max() < 1e-6 * dy + 1e-12
    np.testing.assert_array_equal(rec[1]["vx"], arrs[2].astype(np.float32).astype(np.float64))
    if vz:
        np.testing.assert_array_equal(rec[1]["vz"], arrs[4].astype(np.float32).astype(np.float64))


def test_export_in_id_ranges_matches_per_field_export():
    """From 2^22 particles the record export runs in id ranges, each copied
    to the host while the next is prepared."""
    n = (1 << 22) + 5
    arrs = _particles(n, 12)
    rec = _run(arrs, n, True, lean=False, steps=3, nx=256, ny=192)
    lean = _run(arrs, n, True, lean=True, steps=3, nx=256, ny=192)
    for k in rec[1]:
        np.testing.assert_array_equal(rec[1][k], lean[1][k], err_msg="export " + k)
        np.testing.assert_array_equal(rec[2][k], lean[2][k], err_msg="after steps " + k)
    np.testing.assert_array_equal(rec[1]["vy"], arrs[3].astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("lean", [False, True])
def test_empty_single_and_full_imports(lean):
    """0 particles, 1 particle and a full species (count = capacity, a
    multiple of 4: no padding slot) through both paths."""
    old = os.environ.get("PIC_STAGE_MAX_BYTES")
    if lean:
        os.environ["PIC_STAGE_MAX_BYTES"] = "1"
    try:
        cap = NX * NY * 4
        cfg, q, m = normalized_electrons(NX, NY, 8.0, 6.0, cap, 0.05)
        with P.Handle(cfg) as h:
            e = np.zeros(0)
            h.set_particles(0, e, e, e, e)
            assert h.count(0) == 0
            h.step(3)
            a = h.get_particles(0)
            assert all(len(v) == 0 for v in a.values())
            d = h.diagnostics()
            assert d.error_flags == 0 and d.total_charge_fixed == 0
            one = [np.array([7.9999]), np.array([0.0]), np.array([-0.3]), np.array([0.2])]
            h.set_particles(0, *one)
            b = h.get_particles(0)
            assert abs(b["x"][0] - 7.9999) < 1e-6 and b["y"][0] == 0.0
            assert b["vx"][0] == np.float32(-0.3) and b["vy"][0] == np.float32(0.2)
            h.prime_leapfrog()
            h.step(5)
            c = h.get_particles(0)
            assert 0.0 <= c["x"][0] < 8.0 and 0.0 <= c["y"][0] < 6.0
            arrs = _particles(cap, 13)
            h.set_particles(0, *arrs)
            assert h.count(0) == cap
            f = h.get_particles(0)
            np.testing.assert_array_equal(f["vy"], arrs[3].astype(np.float32).astype(np.float64))
            h.step(4)
            d = h.diagnostics()
            assert d.error_flags == 0 and d.total_charge_fixed == d.expected_charge_fixed
    finally:
        if old is None:
            os.environ.pop("PIC_STAGE_MAX_BYTES", None)
        else:
            os.environ["PIC_STAGE_MAX_BYTES"] = old


@pytest.mark.parametrize("vz", [False, True])
def test_large_import_sorted_range_by_range(vz):
    """From 2^22 slots an import from page-locked arrays is converted and
    radix-sorted in eight slot ranges, each range's sort overlapping the next
    range's transfer, then put in tile-row order by one counting sort: the
    stored order is sorted by row key and the particles are the same as
    through the whole-array sort of the per-field path, before and after
    steps that include a periodic sort."""
    nx, ny, tw, th = 256, 192, 16, 8
    n = (1 << 22) + 7
    arrs = _particles(n, 14, vz)
    out = {}
    for lean in (False, True):
        old = os.environ.get("PIC_STAGE_MAX_BYTES")
        if lean:
            os.environ["PIC_STAGE_MAX_BYTES"] = "1"
        try:
            cfg, q, m = normalized_electrons(nx, ny, 8.0, 6.0, n, 0.05, sort_every=7,
                                             tile_w=tw, tile_h=th)
            cfg.species[0] = P.species(n + 37, q, m, -1, P.SPECIES_HAS_VZ if vz else 0)
            src = [torch.from_numpy(a).pin_memory().numpy() for a in arrs]
            with P.Handle(cfg) as h:
                h.set_particles(0, *src)
                raw = h.get_particles_raw(0)
                first = h.get_particles(0, vz=vz)
                h.prime_leapfrog()
                h.step(9)
                d = h.diagnostics()
                assert d.error_flags == 0 and d.total_charge_fixed == d.expected_charge_fixed
                out[lean] = (raw, first, h.get_particles(0, vz=vz), d.field_energy)
        finally:
            if old is None:
                os.environ.pop("PIC_STAGE_MAX_BYTES", None)
            else:
                os.environ["PIC_STAGE_MAX_BYTES"] = old
    raw = out[False][0]
    cell = raw["cell"][:n]
    cx, cy = cell & 0xFFFF, cell >> 16
    ntx = nx // tw
    row = ((cy // th) * ntx + cx // tw) * th + cy % th
    assert np.all(np.diff(row) >= 0)
    assert np.array_equal(np.sort(raw["pid"][:n]), np.arange(n, dtype=np.uint32))
    for k in out[False][1]:
        np.testing.assert_array_equal(out[False][1][k], out[True][1][k], err_msg="import " + k)
        np.testing.assert_array_equal(out[False][2][k], out[True][2][k], err_msg="after steps " + k)
    assert out[False][3] == out[True][3]

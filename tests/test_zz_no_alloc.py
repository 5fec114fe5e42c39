"""pic_deposit_grid_noalloc: the charge deposit for callers that cannot
allocate device memory (a framework that owns the GPU's memory through its
own pool, a fixed device-memory budget, or no tolerance for cudaFree's
device-wide synchronisation).  It must give exactly what pic_deposit_grid
gives, call after call, although every call reuses one static scratch grid.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import picgpu as P


def _particles(rng, nx, ny, n):
    cx, cy = rng.integers(0, nx, n), rng.integers(0, ny, n)
    cell = (cx | (cy << 16)).astype(np.int32)
    cell[::101] = -1  # empty slots are skipped
    cell[5::997] = nx | (cy[5::997] << 16)  # off the grid: skipped by both calls
    return cell, rng.random(n, dtype=np.float32), rng.random(n, dtype=np.float32)


@pytest.mark.gpu
def test_noalloc_matches_allocating_deposit_on_consecutive_calls():
    import torch

    lib = P.load()
    rng = np.random.default_rng(12)
    # two different problems back to back: the second call must not see the
    # first call's scratch contents
    for nx, ny, n, q, scale in [(64, 48, 200_000, -1, 0.5), (1024, 1024, 300_000, 2, 1.25)]:
        cell, ox, oy = _particles(rng, nx, ny, n)
        dc, dox, doy = (torch.from_numpy(a).cuda() for a in (cell, ox, oy))
        ref = torch.empty(nx * ny, dtype=torch.float64, device="cuda")
        out = torch.full((nx * ny,), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.pic_deposit_grid(nx, ny, n, dc.data_ptr(), dox.data_ptr(), doy.data_ptr(), q,
                                  scale, ref.data_ptr(), None)
        assert st == 0, lib.pic_last_error()
        st = lib.pic_deposit_grid_noalloc(nx, ny, n, dc.data_ptr(), dox.data_ptr(),
                                          doy.data_ptr(), q, scale, out.data_ptr(), None)
        assert st == 0, lib.pic_last_error()
        torch.cuda.synchronize()
        # both are exact integer sums scaled once: bit-identical
        assert torch.equal(out, ref)


@pytest.mark.gpu
def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch

    lib = P.load()
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    st = lib.pic_deposit_grid_noalloc(2048, 1024, 0, None, None, None, 1, 1.0, out.data_ptr(),
                                      None)
    assert st == 1  # PIC_ERR_INVALID_ARG
    assert b"exceeds the fixed scratch grid" in lib.pic_last_error()

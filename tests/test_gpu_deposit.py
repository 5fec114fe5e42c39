"""Fixed-point deposit: bit-exact against the integer restatement of the
oracle, exact total charge, through the handle and the stateless entry."""
import numpy as np
import pytest

import oracle as O
import picgpu as P
from gpu_util import normalized_electrons

pytestmark = pytest.mark.gpu


def raw_deposit(h, cfg, s=0, q_int=-1):
    r = h.get_particles_raw(s)
    return O.deposit_fixed(cfg.nx, cfg.ny, r["cell"], r["ox"], r["oy"], q_int).reshape(cfg.ny, cfg.nx)


@pytest.mark.parametrize("nx,ny,ppc,chunk", [(64, 64, 16, 0), (48, 40, 7, 512),
                                             (4, 4, 300, 256), (128, 32, 33, 2048)])
def test_deposit_bit_exact(nx, ny, ppc, chunk):
    n = nx * ny * ppc
    cfg, q, m = normalized_electrons(nx, ny, 3.0, 2.0, n, 0.05, chunk=chunk)
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(n, vth=(0.3, 0.3, 0), seed=5))
        np.testing.assert_array_equal(h.rho_fixed(), raw_deposit(h, cfg))
        d = h.diagnostics()
        assert d.total_charge_fixed == d.expected_charge_fixed == -n * 2**32


def test_fused_deposit_bit_exact_after_drift():
    # particles move up to a few cells per step and the sort is not rerun, so
    # many of them deposit outside their block's window (global path)
    nx, ny, ppc = 96, 64, 10
    n = nx * ny * ppc
    cfg, q, m = normalized_electrons(nx, ny, 6.0, 4.0, n, 0.05, sort_every=1000)
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(n, vth=(30.0, 20.0, 0), seed=9))
        h.step(12)
        h.synchronize()
        d = h.diagnostics()
        # every step's fused deposit kept the total charge exact
        q_hist = h.history(P.HIST_CHARGE, 0, 13)
        assert (q_hist == -n * 2.0**32).all()
        assert d.total_charge_fixed == -n * 2**32
        np.testing.assert_array_equal(h.rho_fixed(), raw_deposit(h, cfg))


def test_deposit_grid_stateless():
    import torch
    nx, ny, n = 40, 24, 50000
    rng = np.random.default_rng(2)
    cx, cy = rng.integers(0, nx, n), rng.integers(0, ny, n)
    cell = (cx | (cy << 16)).astype(np.int32)
    cell[::97] = -1
    ox, oy = rng.random(n, dtype=np.float32), rng.random(n, dtype=np.float32)
    dc, dox, doy = (torch.from_numpy(a).cuda() for a in (cell, ox, oy))
    out = torch.empty(ny * nx, dtype=torch.float64, device="cuda")
    P.deposit_grid(nx, ny, n, dc.data_ptr(), dox.data_ptr(), doy.data_ptr(), 3, 0.25,
                   out.data_ptr())
    ref = O.deposit_fixed(nx, ny, cell, ox, oy, 1).astype(np.float64) * (3 * 0.25 / 2**32)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)

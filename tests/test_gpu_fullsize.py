"""The 2048 x 2048, 32 particles-per-cell Landau run (134,217,728 particles) at
full size against the FP64 oracle on the host cores, over a short horizon."""
import numpy as np
import pytest

import picgpu as P
from gpu_util import normalized_electrons, oracle_from_handle

pytestmark = pytest.mark.gpu


def test_landau_2048_field_energy_matches_fp64_oracle():
    nx = ny = 2048
    n = nx * ny * 32
    L = nx * 0.05
    nst = 20
    cfg, q, m = normalized_electrons(nx, ny, L, L, n, 0.05)
    spec = P.init_spec(n, vth=(0.05, 0.05, 0.0), pert_kind=P.PERT_DENSITY, pert_amp=0.01,
                       pert_mx=1, pert_my=1, seed=2024)
    with P.Handle(cfg) as h:
        h.init_particles(0, spec)
        st = oracle_from_handle(h, cfg, q, m)
        h.prime_leapfrog()
        h.step(nst)
        fe = h.history(P.HIST_FIELD_ENERGY, 0, nst + 1)
        d = h.diagnostics()
    st.prime(nthreads=0)
    ref = st.run(nst, nthreads=0)
    rel = np.abs(fe - ref["fe"]) / ref["fe"]
    print("field energy relative error vs FP64 per step:", np.array2string(rel, precision=2))
    assert d.total_charge_fixed == d.expected_charge_fixed
    assert rel.max() < 1e-5

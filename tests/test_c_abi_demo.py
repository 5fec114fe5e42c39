"""The C ABI from plain C: tests/c_abi_demo.c compiles as C99 against
include/pic.h and links libpic.so (CPU); on a GPU it runs the step
interface and the one-call host run and agrees with the Python binding."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import picgpu as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "msc-thesis_gb300")


def build_demo(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    out = str(tmp_path / "c_abi_demo")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi_demo.c"), "-L", LIBDIR, "-lpic", "-lm",
           "-Wl,-rpath," + LIBDIR, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_c_caller_compiles_and_links(tmp_path):
    assert os.path.exists(build_demo(tmp_path))


@pytest.mark.gpu
def test_c_caller_runs_and_matches_the_python_binding(tmp_path):
    exe = build_demo(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    tok = r.stdout.split()
    fe, charge_ok, moved = float(tok[1]), int(tok[3]), int(tok[5])
    assert charge_ok == 1 and moved == 1
    # the same run through the Python binding
    nx = ny = 64
    n = nx * ny * 8
    L = 4 * np.pi
    A = L * L
    cfg = P.config(nx, ny, L, L, 0.1, [P.species(n, -A / n, A / n, -1)])
    with P.Handle(cfg) as h:
        h.init_particles(0, P.init_spec(n, vth=(0.01, 0.01, 0.0), beam_v=0.2,
                                        pert_kind=P.PERT_XDISP, pert_amp=1e-3, pert_mx=1, seed=5))
        h.prime_leapfrog()
        h.step(20)
        assert h.diagnostics().field_energy == fe

"""The C-ABI library loads and exports every symbol include/*.h declares;
host-side argument validation works without a GPU."""
import ctypes as C
import glob
import os
import re

import pytest

import picgpu as P
from conftest import ROOT


def header_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(pic_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_functions():
    assert "pic_create" in header_functions()
    assert "pic_compat_run" in header_functions()


@pytest.mark.parametrize("name", header_functions())
def test_library_exports(name):
    lib = C.CDLL(P.LIB_PATH)
    assert hasattr(lib, name), name


def test_binding_covers_header():
    assert set(header_functions()) <= set(P.SIGNATURES)


def test_status_strings():
    L = P.load()
    assert L.pic_status_string(0) == b"ok"
    assert L.pic_status_string(7) == b"device wait timed out"


def test_config_validation_is_host_side():
    bad = P.config(1, 64, 1.0, 1.0, 0.1, [P.species(100, -1.0, 1.0, -1)])
    with pytest.raises(P.PicError) as e:
        P.Handle(bad)
    assert e.value.status == 1
    bad = P.config(64, 64, 1.0, 1.0, 0.1, [P.species(100, -1.0, 1.0, 0)])  # q without q_int
    with pytest.raises(P.PicError) as e:
        P.Handle(bad)
    assert e.value.status == 1
    bad = P.config(64, 64, 1.0, 1.0, 0.1, [P.species(100, -1.0, 1.0, -1),
                                           P.species(100, 1.5, 1.0, 1)])  # not integer multiples
    with pytest.raises(P.PicError) as e:
        P.Handle(bad)
    assert e.value.status == 1
    # push chunks above 32768 particles could overflow the window's 32-bit cell moments
    bad = P.config(64, 64, 1.0, 1.0, 0.1, [P.species(100, -1.0, 1.0, -1)], chunk=32772)
    with pytest.raises(P.PicError) as e:
        P.Handle(bad)
    assert e.value.status == 1
    # the bulk-copy push pipelines (variants 2 and 4) were removed
    for variant in (2, 4, -1):
        bad = P.config(64, 64, 1.0, 1.0, 0.1, [P.species(100, -1.0, 1.0, -1)],
                       push_variant=variant)
        with pytest.raises(P.PicError) as e:
            P.Handle(bad)
        assert e.value.status == 1


def test_compat_params_validation_is_host_side():
    import numpy as np
    p = P.ref_params(nx=1)
    with pytest.raises(P.PicError) as e:
        P.compat_run(p, *(np.zeros(100) for _ in range(4)))
    assert e.value.status == 1


def test_no_device_is_reported(monkeypatch):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = P.config(64, 64, 1.0, 1.0, 0.1, [P.species(100, -1.0, 1.0, -1)])
    with pytest.raises(P.PicError) as e:
        P.Handle(c)
    assert e.value.status == 9

"""The C-ABI library without a GPU: it builds, loads, exports every symbol the
header declares, validates parameters on the host, and reports a missing
device as a status code instead of crashing."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, cfgs, pkg

HEADER = os.path.join(ROOT, "include", "lmm_gb300.h")


@pytest.fixture(scope="module")
def L():
    P = pkg()
    if not os.path.exists(P.LIB_PATH):
        P.build()
    return P.lib()


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lmm_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_what_the_binding_exports():
    assert header_functions() == sorted(pkg().EXPORTS)


def test_library_exports_every_declared_symbol(L):
    P = pkg()
    out = subprocess.run(["nm", "-D", "--defined-only", P.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(lmm_\w+)$", out, flags=re.M))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing
    for f in header_functions():
        assert hasattr(L, f)


def test_status_strings_and_version(L):
    assert L.lmm_status_string(0) == b"ok"
    assert L.lmm_status_string(-4) == b"non-finite result"
    assert re.match(rb"^\d+\.\d+\.\d+$", L.lmm_version())


def _params(cfg):
    return pkg()._ParamsRef(cfg)


def test_validate_accepts_all_workloads(L):
    for n in (1, 2, 3, 4, 5):
        assert pkg().validate(cfgs().workload(n)) == 0
    assert pkg().validate(cfgs().reference_params()) == 0


@pytest.mark.parametrize("mutate,needle", [
    (lambda c: setattr(c, "nmat", c.nn), "nmat"),
    (lambda c: setattr(c, "nn", 300), "nn must be"),
    (lambda c: c.L0.__setitem__(3, -0.01), "L0[3]"),
    (lambda c: c.L0.__setitem__(5, np.nan), "L0[5]"),
    (lambda c: c.lam.__setitem__(0, np.inf), "lambda[0]"),
    (lambda c: c.maturities.__setitem__(2, 41), "maturities[2]"),
    (lambda c: c.maturities.__setitem__(0, 0), "maturities[0]"),
    (lambda c: setattr(c, "delta", 0.0), "delta"),
])
def test_validate_rejects_bad_parameters(L, mutate, needle):
    c = cfgs().workload(1)
    c.L0, c.lam, c.maturities = c.L0.copy(), c.lam.copy(), c.maturities.copy()
    mutate(c)
    assert pkg().validate(c) == -1
    assert needle in pkg().last_error()


def test_too_many_swaptions_rejected(L):
    c = cfgs().workload(1)
    c.maturities = np.ones(65, dtype=np.int32)
    c.swaprates = np.full(65, 0.05)
    assert pkg().validate(c) == -1


def test_null_arguments_are_errors_not_crashes(L):
    assert L.lmm_validate_params(None) == -1
    assert L.lmm_engine_destroy(None) == 0
    assert L.lmm_greeks_f32_host(None, None, 10, None, None) == -1
    assert L.lmm_swaption_greeks(None, 0, 0.0, 1.0, 0, None, None, 0) == -1
    assert L.lmm_num_outputs(C.byref(_params(cfgs().workload(3)).p)) == 321


def test_engine_without_gpu_reports_no_device(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _params(cfgs().workload(1))
    h = C.c_void_p()
    assert L.lmm_engine_create(C.byref(r.p), 0, C.byref(h)) == -5
    assert not h.value

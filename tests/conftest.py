import importlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "financial-services-workload-samples_gb300"
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pkg():
    return importlib.import_module(PKG_NAME)


def cfgs():
    return importlib.import_module(PKG_NAME + ".configs")


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def cfg_from_record(rec, paths):
    c = cfgs()
    return c.LmmConfig("golden", int(rec["nn"]), int(rec["nmat"]), float(rec["delta"]),
                       np.array(rec["L0"], dtype=np.float64), np.array(rec["lam"], dtype=np.float64),
                       np.array(rec["maturities"], dtype=np.int32),
                       np.array(rec["swaprates"], dtype=np.float64), int(paths))


def normals_from_record(rec):
    """Regenerate a golden case's normals with the oracle and check the checksum."""
    import hashlib

    from oracle import oracle as O
    if rec["dtype"] == "f64":
        z = O.normals_f64(rec["seed"], rec["paths"], rec["nmat"], path0=rec["path0"])
    else:
        z = O.normals_f32(rec["seed"], rec["paths"], rec["nmat"], path0=rec["path0"])
    assert hashlib.sha256(z.tobytes()).hexdigest() == rec["sha256"], "normals drifted from the golden spec"
    return z


@pytest.fixture(scope="session")
def lmm():
    """The CUDA library through its C-ABI; GPU tests only."""
    return pkg().engine_lib()

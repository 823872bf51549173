"""The drop-in claim: the reference's own driver (LiborMarketModel/main.cpp,
unmodified) compiles and links against this library with the shim
(shim/liborSwaptionGreeks_gb300.cpp) replacing liborSwaptionGreeks.cpp and
mklRng.cpp, in the FP64 and FP32 builds. The reference tree is named by
LMM_REFERENCE_ROOT; without it there is nothing to link and the test is
skipped."""
import os
import subprocess

import pytest

from conftest import ROOT, pkg

REF = os.environ.get("LMM_REFERENCE_ROOT", "")


@pytest.mark.parametrize("double", [True, False])
def test_reference_driver_links_against_the_library(tmp_path, double):
    if not REF or not os.path.isfile(os.path.join(REF, "LiborMarketModel", "main.cpp")):
        pytest.skip("LMM_REFERENCE_ROOT does not name the reference tree")
    P = pkg()
    if not os.path.exists(P.LIB_PATH):
        P.build()
    import importlib
    b = importlib.import_module("financial-services-workload-samples_gb300.build_lib")
    exe = b.build_dropin(REF, str(tmp_path), double=double)
    assert os.access(exe, os.X_OK)
    out = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    names = "lmm_swaption_greeks_mrg32k3a" if double else "lmm_swaption_greeks_mrg32k3a_f32"
    assert names in out          # the entry point comes from liblmm_gb300.so
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "liblmm_gb300.so" in ldd and "not found" not in ldd.split("liblmm_gb300.so")[1].splitlines()[0]

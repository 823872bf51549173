"""The roofline calibration probes (lmm_fp32_peak_tflops, lmm_fp64_peak_tflops,
lmm_mufu_peak_gops): they run, return plausible rates for a GB300-class GPU,
and the MUFU mix lies between its parts."""
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def test_peak_probes_are_plausible():
    P = pkg()
    f32 = P.fp32_peak_tflops(0, 50.0)
    f64 = P.fp64_peak_tflops(0, 50.0)
    mufu = P.mufu_peak_gops(0, 30.0)
    assert 10.0 < f32 < 500.0
    assert 0.05 < f64 < f32
    assert 100.0 < mufu["rcp"] and 100.0 < mufu["ex2"]
    lo, hi = sorted((mufu["ex2"], mufu["rcp"]))
    assert 0.9 * lo <= mufu["mixed"] <= 1.1 * hi


def test_probe_arguments():
    P = pkg()
    L = P.lib()
    import ctypes as C
    t = C.c_double()
    assert L.lmm_fp64_peak_tflops(0, 0.0, C.byref(t)) == -1
    assert L.lmm_fp64_peak_tflops(99, 10.0, C.byref(t)) == -1
    assert L.lmm_mufu_peak_gops(0, -1.0, None, None, None) in (0, -1)

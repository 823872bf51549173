"""Rounding error reported apart from the Monte Carlo standard error
(lmm_greeks_f32_rounding_device): per output |FP32 - FP64| on the identical
normals. The reference reports a value and one delta (LiborMarketModel/
main.cpp:91-92) with neither figure."""
import numpy as np
import pytest

from conftest import cfgs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from conftest import pkg
    return pkg()


@pytest.mark.parametrize("wl,paths", [(2, 65536), (3, 2048), (5, 4096)])
def test_rounding_vector_is_fp32_minus_fp64(P, wl, paths):
    import torch
    cfg = cfgs().workload(wl, paths)
    n = cfg.paths
    tot = cfg.nscen * cfg.nout
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(77 + wl, n, cfg.nmat, dz.data_ptr())
    out, se, err = (torch.full((tot,), np.nan, dtype=torch.float64, device="cuda") for _ in range(3))
    ref, ref_se, f64 = (torch.zeros(tot, dtype=torch.float64, device="cuda") for _ in range(3))
    dz64 = dz.double()
    with P.Engine(cfg) as e:
        e.greeks_f32_rounding_device(dz.data_ptr(), n, out.data_ptr(), se.data_ptr(), err.data_ptr())
        e.greeks_f32_device(dz.data_ptr(), n, ref.data_ptr(), ref_se.data_ptr())
        e.greeks_f64_device(dz64.data_ptr(), n, f64.data_ptr())
        e.synchronize()
    out, se, err = out.cpu().numpy(), se.cpu().numpy(), err.cpu().numpy()
    ref, ref_se, f64 = ref.cpu().numpy(), ref_se.cpu().numpy(), f64.cpu().numpy()
    np.testing.assert_array_equal(out, ref)
    np.testing.assert_array_equal(se, ref_se)
    np.testing.assert_array_equal(err, np.abs(ref - f64))
    # FP32 rounding sits far below the FP32 tolerance of the largest entry,
    # and the value's is far below its Monte Carlo standard error
    assert np.all(err <= 1e-4 * np.abs(f64).max())
    v = np.arange(cfg.nscen) * cfg.nout
    assert np.all(err[v] < 0.1 * se[v])

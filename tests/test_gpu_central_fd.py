"""The FP32 adjoint against FP64 central finite differences on the GPU.

The headline workload states its finite-difference check as FP64 central
differences (bump 1e-6) under common random numbers: every one of the 1+4NN
forward re-runs (path_calc_b1, LiborMarketModel/liborSwaptionGreeks.cpp:34-82,
and the portfolio value of :120-197) reads the same normals, so the
differences carry no Monte Carlo noise and measure the pathwise derivative
the adjoint computes (:86-117 for the deltas; the vegas are this library's
addition).
"""
import numpy as np
import pytest

from conftest import cfgs
from oracle import oracle as O
from test_gpu_parity import assert_f32_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from conftest import pkg
    return pkg()


def test_central_bumps_match_oracle_bumped_values(P):
    """The central comparator's entries are (V(+h) - V(-h)) / 2h of the
    oracle's own FP64 revaluations on the same normals."""
    cfg = cfgs().workload(1, 512)
    z = O.normals_f64(19, cfg.paths, cfg.nmat)
    h = 1e-6
    with P.Engine(cfg) as e:
        g, se = e.bump_greeks_f64(z, h, central=True)
        assert e.last_launches == 3
    base, _ = O.value(cfg, z)
    assert g[0][0] == pytest.approx(base, rel=1e-12)
    assert np.all(se[0][1:] == 0.0) and se[0][0] > 0
    for i in (0, 17, 45, 79):
        up = O.value(cfg, z, L0=np.where(np.arange(cfg.nn) == i, cfg.L0 + h, cfg.L0))[0]
        dn = O.value(cfg, z, L0=np.where(np.arange(cfg.nn) == i, cfg.L0 - h, cfg.L0))[0]
        assert g[0][1 + i] == pytest.approx((up - dn) / (2 * h), rel=1e-6, abs=1e-6)
        upl = O.value(cfg, z, lam=np.where(np.arange(cfg.nn) == i, cfg.lam + h, cfg.lam))[0]
        dnl = O.value(cfg, z, lam=np.where(np.arange(cfg.nn) == i, cfg.lam - h, cfg.lam))[0]
        assert g[0][1 + cfg.nn + i] == pytest.approx((upl - dnl) / (2 * h), rel=1e-6, abs=1e-6)


def test_fp32_adjoint_vs_fp64_central_differences_65536_paths(P):
    """65,536 paths of the headline workload: FP32 adjoint Greeks within 1e-4
    of FP64 central differences (h = 1e-6) on the identical normals, and the
    FP64 adjoint within 1e-6 of them (the differences' own truncation and
    rounding error)."""
    import torch
    cfg = cfgs().workload(2, 65536)
    n = cfg.paths
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(4242, n, cfg.nmat, dz.data_ptr())
    dz64 = dz.double()
    fd = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    a32 = torch.zeros_like(fd)
    a64 = torch.zeros_like(fd)
    with P.Engine(cfg) as e:
        e.bump_greeks_f64_device(dz64.data_ptr(), n, 1e-6, fd.data_ptr(), central=True)
        e.greeks_f32_device(dz.data_ptr(), n, a32.data_ptr())
        e.greeks_f64_device(dz64.data_ptr(), n, a64.data_ptr())
        e.synchronize()
    fd, a32, a64 = fd.cpu().numpy(), a32.cpu().numpy(), a64.cpu().numpy()
    assert_f32_close(a32, fd, cfg.nn, "FP32 adjoint vs FP64 central differences")
    np.testing.assert_allclose(a64, fd, rtol=1e-6, atol=1e-6 * np.abs(fd[1:]).max())


def test_central_rejects_bad_bump(P):
    cfg = cfgs().workload(1, 64)
    z = O.normals_f64(3, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        for h in (0.0, -1e-6, float("inf")):
            with pytest.raises(P.LmmError) as ei:
                e.bump_greeks_f64(z, h, central=True)
            assert ei.value.code == -1

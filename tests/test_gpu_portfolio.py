"""Runtime portfolio weights and the per-swaption breakdown, through the C ABI,
against the oracle priced with the same weights (FP64 1e-12, FP32 within the
1e-4 rule): weighted value and Greeks for both FP32 kernel families, the
FP64 kernel, the forward/backward pair and the bump comparator; the
breakdown per swaption and its sum over swaptions."""
import numpy as np
import pytest

from conftest import cfgs, pkg
from oracle import oracle as O
from test_gpu_parity import RTOL_F64, assert_f32_close

pytestmark = pytest.mark.gpu


def _weights(nopt, seed):
    w = np.random.default_rng(seed).uniform(-1.0, 2.5, nopt)
    w[0] = 0.0                   # a swaption switched off
    return w


@pytest.mark.parametrize("wl,paths", [(1, 4096), (3, 512)])
def test_weighted_fp32_matches_weighted_oracle(wl, paths):
    P = pkg()
    cfg = cfgs().workload(wl, paths)
    w = _weights(len(cfg.swaprates), wl)
    z = O.normals_f32(300 + wl, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        e.set_weights(w)
        g, _ = e.greeks_f32(z)
        e.set_weights(None)
        g1, _ = e.greeks_f32(z)
    m, _ = O.greeks(cfg, z.astype(np.float64), weights=w)
    assert_f32_close(g[0], m, cfg.nn, f"weighted workload {wl}")
    m1, _ = O.greeks(cfg, z.astype(np.float64))
    assert_f32_close(g1[0], m1, cfg.nn, f"weights reset, workload {wl}")


def test_weighted_fp64_and_unit_weights_are_the_reference_portfolio():
    P = pkg()
    cfg = cfgs().workload(1, 2048)
    w = _weights(len(cfg.swaprates), 7)
    z = O.normals_f64(11, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g0, _ = e.greeks_f64(z)
        e.set_weights(np.ones(len(cfg.swaprates)))
        g1, _ = e.greeks_f64(z)
        e.set_weights(w)
        gw, _ = e.greeks_f64(z)
    np.testing.assert_array_equal(g0, g1)      # weight 1 is exactly the unweighted portfolio
    m, _ = O.greeks(cfg, z, weights=w)
    np.testing.assert_allclose(gw[0], m, rtol=RTOL_F64, atol=1e-13 * np.abs(m).max())


def test_weighted_forward_backward_pair_and_bump():
    import torch
    P = pkg()
    cfg = cfgs().workload(4, 4096)
    w = _weights(len(cfg.swaprates), 3)
    z = O.normals_f32(5, cfg.paths, cfg.nmat)
    dz = torch.from_numpy(z).cuda()
    with P.Engine(cfg) as e:
        e.set_weights(w)
        fused, _ = e.greeks_f32(z)
        t = e.tape(cfg.paths)
        val = torch.zeros(1, dtype=torch.float64, device="cuda")
        grad = torch.zeros(2 * cfg.nn, dtype=torch.float64, device="cuda")
        e.forward_f32_device(dz.data_ptr(), cfg.paths, t, val.data_ptr())
        e.backward_f32_device(dz.data_ptr(), t, [1.0], grad.data_ptr())
        e.synchronize()
        t.close()
        b, _ = e.bump_greeks_f64(z.astype(np.float64), 1e-6)
    assert val.item() == pytest.approx(fused[0][0], rel=1e-12)
    np.testing.assert_allclose(grad.cpu().numpy(), fused[0][1:], rtol=1e-6,
                               atol=1e-6 * np.abs(fused[0][1:]).max())
    m, _ = O.greeks(cfg, z.astype(np.float64), weights=w)
    # one-sided differences at h = 1e-6 against the weighted adjoint
    np.testing.assert_allclose(b[0][0], m[0], rtol=1e-12)
    np.testing.assert_allclose(b[0][1:], m[1:], rtol=0, atol=2e-4 * np.abs(m[1:]).max())


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_breakdown_per_swaption(precision):
    import torch
    P = pkg()
    cfg = cfgs().workload(1, 2048)
    nopt, nout = len(cfg.swaprates), 1 + 2 * cfg.nn
    z = O.normals_f32(77, cfg.paths, cfg.nmat)
    z64 = z.astype(np.float64)
    dt = torch.float32 if precision == "f32" else torch.float64
    dz = torch.from_numpy(z).to(dt).cuda()
    out = torch.zeros(nopt * nout, dtype=torch.float64, device="cuda")
    se = torch.zeros(nopt * nout, dtype=torch.float64, device="cuda")
    port = torch.zeros(nout, dtype=torch.float64, device="cuda")
    with P.Engine(cfg) as e:
        e.set_weights(_weights(nopt, 9))       # the breakdown ignores the caller's weights
        if precision == "f32":
            e.breakdown_f32_device(dz.data_ptr(), cfg.paths, out.data_ptr(), se.data_ptr())
            assert e.last_launches == 2 * nopt
            e.set_weights(None)
            e.greeks_f32_device(dz.data_ptr(), cfg.paths, port.data_ptr())
        else:
            e.breakdown_f64_device(dz.data_ptr(), cfg.paths, out.data_ptr(), se.data_ptr())
            e.set_weights(None)
            e.greeks_f64_device(dz.data_ptr(), cfg.paths, port.data_ptr())
        e.synchronize()
    bd = out.cpu().numpy().reshape(nopt, nout)
    for o in range(nopt):
        unit = np.zeros(nopt)
        unit[o] = 1.0
        m, _ = O.greeks(cfg, z64, weights=unit)
        if precision == "f32":
            # a swaption out of the money on every path has all-zero Greeks
            if np.abs(m).max() > 0:
                assert_f32_close(bd[o], m, cfg.nn, f"swaption {o}")
            else:
                assert np.abs(bd[o]).max() == 0.0
        else:
            np.testing.assert_allclose(bd[o], m, rtol=RTOL_F64, atol=1e-13 * max(np.abs(m).max(), 1e-300))
    total = bd.sum(axis=0)
    p = port.cpu().numpy()
    tol = 1e-5 if precision == "f32" else 1e-12
    np.testing.assert_allclose(total, p, rtol=tol, atol=tol * np.abs(p).max())


def test_weights_validation():
    P = pkg()
    cfg = cfgs().workload(1, 64)
    with P.Engine(cfg) as e:
        bad = np.ones(len(cfg.swaprates))
        bad[3] = np.nan
        with pytest.raises(P.LmmError):
            e.set_weights(bad)
        with pytest.raises(P.LmmError):
            e.set_weights(np.ones(len(cfg.swaprates) + 1))
    empty = cfgs().LmmConfig("no-swaptions", 20, 10, 0.25, np.full(20, 0.05), np.full(20, 0.2),
                             np.zeros(0, dtype=np.int32), np.zeros(0), 64)
    with P.Engine(empty) as e:
        assert P.lib().lmm_swaption_breakdown_f64_device(e.h, 16, 64, 16, None) == -1

"""GPU parity: the CUDA kernels, called through the C-ABI, against the oracle
on identical normals.

Tolerances:
  FP64 kernels: relative 1e-12 per output (value, every delta, every vega).
  FP32 adjoint: per Greek |gpu - oracle| <= 1e-4 * max(|oracle|, 1e-2 * max|group|),
                groups = {value}, {deltas}, {vegas}; i.e. relative 1e-4, with
                Greeks below 1% of their group's largest measured against
                that 1% (their absolute FP32 rounding does not shrink with them).
"""
import numpy as np
import pytest

from conftest import cfgs, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL_F32 = 1e-4
RTOL_F64 = 1e-12


def scaled_err(gpu, ref, nn):
    gpu, ref = np.asarray(gpu, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    out = np.zeros_like(ref)
    for sl in (slice(0, 1), slice(1, 1 + nn), slice(1 + nn, 1 + 2 * nn)):
        g, r = gpu[sl], ref[sl]
        floor = 1e-2 * np.max(np.abs(r)) if r.size > 1 else 0.0
        den = np.maximum(np.abs(r), floor)
        den = np.where(den > 0, den, 1.0)
        out[sl] = np.abs(g - r) / den
    return out


def assert_f32_close(gpu, ref, nn, label=""):
    e = scaled_err(gpu, ref, nn)
    worst = int(np.argmax(e))
    print(f"{label} FP32 vs FP64 oracle: max scaled err {e.max():.3e} at output {worst} "
          f"(value {e[0]:.2e}, deltas {e[1:1 + nn].max():.2e}, vegas {e[1 + nn:].max():.2e})")
    assert e.max() <= RTOL_F32, (worst, gpu[worst], ref[worst])


@pytest.fixture(scope="module")
def P():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return pkg()


def test_fp64_kernel_matches_oracle_1e12(P):
    cfg = cfgs().workload(1, 2048)
    z = O.normals_f64(101, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, gse = e.greeks_f64(z)
        assert e.last_launches == 2
    m, se = O.greeks(cfg, z)
    np.testing.assert_allclose(g[0], m, rtol=RTOL_F64, atol=1e-13 * np.abs(m).max())
    np.testing.assert_allclose(gse[0], se, rtol=1e-6)


def test_fp64_kernel_long_tenor_and_vol_vector(P):
    for cfg in (cfgs().workload(3, 64), cfgs().workload(4, 256)):
        z = O.normals_f64(7, cfg.paths, cfg.nmat)
        with P.Engine(cfg) as e:
            g, _ = e.greeks_f64(z)
        m, _ = O.greeks(cfg, z)
        np.testing.assert_allclose(g[0], m, rtol=1e-11, atol=1e-12 * np.abs(m).max())


def test_reference_signature_fp64_drop_in(P):
    """lmm_swaption_greeks: normals written back into z, value and dV/dL0[79]
    equal the reference's (NLOOPS-divided) outputs on that z."""
    num_paths = 512
    z, d_v, d_lb = P.swaption_greeks(num_paths, 0.0, 1.0, seed=1234)
    z_ref = O.normals_f64(12345, num_paths, 40)
    np.testing.assert_allclose(z, z_ref, rtol=1e-13, atol=1e-13)
    cfg = cfgs().reference_params(num_paths)
    m, _ = O.greeks(cfg, z)
    assert d_v == pytest.approx(m[0], rel=RTOL_F64)
    assert d_lb == pytest.approx(m[cfg.nn], rel=RTOL_F64)
    # seed is ignored, as in the reference
    z2, d_v2, _ = P.swaption_greeks(num_paths, 0.0, 1.0, seed=99)
    assert d_v2 == d_v and np.array_equal(z2, z)


def test_reference_signature_fp32_drop_in(P):
    num_paths = 1024
    z, d_v, d_lb = P.swaption_greeks_f32(num_paths)
    cfg = cfgs().reference_params(num_paths)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert d_v == pytest.approx(m[0], rel=RTOL_F32)
    assert d_lb == pytest.approx(m[cfg.nn], rel=RTOL_F32)


@pytest.mark.parametrize("wl", [1, 4])
def test_fp32_adjoint_matches_oracle(P, wl):
    cfg = cfgs().workload(wl, 8192)
    z = O.normals_f32(2024 + wl, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, gse = e.greeks_f32(z)
    m, se = O.greeks(cfg, z.astype(np.float64))
    assert_f32_close(g[0], m, cfg.nn, f"workload {wl}")
    np.testing.assert_allclose(gse[0], se, rtol=2e-3, atol=1e-6 * np.abs(se).max())
    assert g[0][-1] == 0.0                      # vega[NN-1]: lambda[NN-1] is never read


def test_fp32_philox_mode_matches_oracle_on_same_counters(P):
    cfg = cfgs().workload(4, 4096)
    seed, path0 = 0x1234_5678_9ABC, 1_000_003
    z = O.normals_f32(seed, cfg.paths, cfg.nmat, path0=path0)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_philox(seed, cfg.paths, path0=path0)
        g2, _ = e.greeks_f32(z)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert_f32_close(g[0], m, cfg.nn, "philox")
    # in-kernel normals vs the same normals read from memory: same kernels
    np.testing.assert_allclose(g[0], g2[0], rtol=2e-6, atol=1e-7 * np.abs(g2).max())


def test_device_normals_match_oracle_spec(P):
    import torch
    n, nmat, seed = 3000, 40, 77
    d32 = torch.empty(n * nmat, dtype=torch.float32, device="cuda")
    d64 = torch.empty(n * nmat, dtype=torch.float64, device="cuda")
    P.normals_f32_device(seed, n, nmat, d32.data_ptr(), path0=5)
    P.normals_f64_device(seed, n, nmat, d64.data_ptr(), path0=5)
    torch.cuda.synchronize()
    np.testing.assert_allclose(d32.cpu().numpy(), O.normals_f32(seed, n, nmat, path0=5), rtol=0, atol=4e-6)
    np.testing.assert_allclose(d64.cpu().numpy(), O.normals_f64(seed, n, nmat, path0=5), rtol=0, atol=1e-13)


def test_forward_backward_pair_equals_fused(P):
    import torch
    cfg = cfgs().workload(4, 3000)
    z = O.normals_f32(5, cfg.paths, cfg.nmat)
    dz = torch.from_numpy(z).cuda()
    with P.Engine(cfg) as e:
        fused, _ = e.greeks_f32(z)
        t = e.tape(cfg.paths)
        val = torch.zeros(1, dtype=torch.float64, device="cuda")
        grad = torch.zeros(2 * cfg.nn, dtype=torch.float64, device="cuda")
        e.forward_f32_device(dz.data_ptr(), cfg.paths, t, val.data_ptr())
        e.backward_f32_device(dz.data_ptr(), t, [2.5], grad.data_ptr())
        e.synchronize()
        t.close()
    f = fused[0]
    assert val.item() == pytest.approx(f[0], rel=1e-12)
    np.testing.assert_allclose(grad.cpu().numpy(), 2.5 * f[1:], rtol=2e-6, atol=1e-6 * np.abs(f[1:]).max())


def test_bump_comparator_matches_oracle_bumped_values(P):
    cfg = cfgs().workload(1, 512)
    z = O.normals_f64(9, cfg.paths, cfg.nmat)
    h = 1e-6
    with P.Engine(cfg) as e:
        g, _ = e.bump_greeks_f64(z, h)
        assert e.last_launches == 3
    base, _ = O.value(cfg, z)
    assert g[0][0] == pytest.approx(base, rel=RTOL_F64)
    for i in (0, 17, 45, 79):
        L0 = cfg.L0.copy(); L0[i] += h
        up, _ = O.value(cfg, z, L0=L0)
        lam = cfg.lam.copy(); lam[i] += h
        upl, _ = O.value(cfg, z, lam=lam)
        assert g[0][1 + i] == pytest.approx((up - base) / h, rel=1e-6, abs=1e-6)
        assert g[0][1 + cfg.nn + i] == pytest.approx((upl - base) / h, rel=1e-6, abs=1e-6)


def test_scenarios_equal_separate_runs(P):
    base = cfgs().workload(5, 1500)
    cfg = base.with_paths(1500)
    cfg.L0 = base.L0[:3].copy()
    z = O.normals_f32(11, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
    assert g.shape == (3, cfg.nout)
    for s in range(3):
        one = cfg.scenario(s)
        with P.Engine(one) as e1:
            g1, _ = e1.greeks_f32(z)
        np.testing.assert_allclose(g[s], g1[0], rtol=1e-6, atol=1e-7 * np.abs(g1).max())
        m, _ = O.greeks(one, z.astype(np.float64))
        assert_f32_close(g[s], m, one.nn, f"scenario {s}")


def test_deterministic_bitwise(P):
    cfg = cfgs().workload(1, 5000)
    z = O.normals_f32(3, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        a, _ = e.greeks_f32(z)
        b, _ = e.greeks_f32(z)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("paths", [1, 31, 33, 129, 1000])
def test_ragged_path_counts(P, paths):
    cfg = cfgs().workload(4, paths)
    z = O.normals_f32(8, paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
        g64, _ = e.greeks_f64(z.astype(np.float64))
    m, _ = O.greeks(cfg, z.astype(np.float64))
    np.testing.assert_allclose(g64[0], m, rtol=1e-11, atol=1e-12 * np.abs(m).max())
    assert_f32_close(g[0], m, cfg.nn, f"{paths} paths")


def test_error_statuses(P):
    cfg = cfgs().workload(1, 64)
    z = O.normals_f32(1, 64, 40)
    with P.Engine(cfg) as e:
        with pytest.raises(P.LmmError) as ei:
            e.greeks_f32(z, paths=0)
        assert ei.value.code == -1
        bad = z.copy(); bad[100] = np.nan
        with pytest.raises(P.LmmError) as ei:
            e.greeks_f32(bad)
        assert ei.value.code == -4
        ok, _ = e.greeks_f32(z)                  # the engine stays usable
        assert np.all(np.isfinite(ok))
    bad_cfg = cfgs().workload(1, 64)
    bad_cfg.maturities = bad_cfg.maturities.copy(); bad_cfg.maturities[0] = 77
    with pytest.raises(P.LmmError) as ei:
        P.Engine(bad_cfg)
    assert ei.value.code == -1


def test_full_size_fp32_vs_fp64_on_gpu(P):
    """Headline size (4,194,304 paths): FP32 adjoint against the GPU FP64
    kernel (itself pinned to the oracle above) on the identical normals."""
    import torch
    cfg = cfgs().workload(2)
    n = cfg.paths
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(42, n, cfg.nmat, dz.data_ptr())
    dz64 = dz.double()
    out32 = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    se32 = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    out64 = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with P.Engine(cfg) as e:
        e.greeks_f32_device(dz.data_ptr(), n, out32.data_ptr(), se32.data_ptr())
        e.greeks_f64_device(dz64.data_ptr(), n, out64.data_ptr())
        e.synchronize()
    g, r, se = out32.cpu().numpy(), out64.cpu().numpy(), se32.cpu().numpy()
    assert_f32_close(g, r, cfg.nn, "4,194,304 paths")
    # rounding error far below the Monte Carlo error
    assert np.all(np.abs(g - r) <= 0.05 * se + 1e-12)


def _random_cfg(nn, nmat, nopt, seed, paths, vol=(0.1, 0.2)):
    """Random curve, vols and portfolio. Vols up to 0.2 keep every Euler path
    tame over the horizons used here: with higher vols over long horizons a few
    paths explode, their Greeks become astronomically large and chaotic in the
    last bits of exp(), and no two implementations agree on their mean."""
    rng = np.random.default_rng(seed)
    c = cfgs().LmmConfig(f"random{nn}x{nmat}", nn, nmat, 0.25, rng.uniform(0.02, 0.07, nn),
                         rng.uniform(*vol, nn), rng.integers(1, nn - nmat + 1, nopt).astype(np.int32),
                         rng.uniform(0.03, 0.06, nopt), paths)
    return c


@pytest.mark.parametrize("philox", [False, True])
def test_long_tenor_checkpointed_fp32_matches_oracle(P, philox):
    """Workload 3 (NN=160, NMAT=120, 30 swaptions): the fused call runs one
    thread per path, the forward in two passes of 80 rates and the reverse in
    passes over blocks of 40 rates, each step rebuilt from the forward's drift
    sum at the block's top rate, with the rates saved every 8 steps."""
    cfg = cfgs().workload(3, 512)
    seed = 303
    z = O.normals_f32(seed, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_philox(seed, cfg.paths) if philox else e.greeks_f32(z)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert_f32_close(g[0], m, cfg.nn, f"160x120 philox={philox}")


@pytest.mark.parametrize("nn,nmat,nopt", [(20, 10, 4), (33, 7, 3), (64, 32, 15), (96, 60, 8), (160, 80, 9),
                                         (200, 100, 12), (256, 40, 5)])
def test_other_shapes_fp32_match_oracle(P, nn, nmat, nopt):
    cfg = _random_cfg(nn, nmat, nopt, nn * 1000 + nmat, 700)
    z = O.normals_f32(nn, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
        g64, _ = e.greeks_f64(z.astype(np.float64))
    m, _ = O.greeks(cfg, z.astype(np.float64))
    np.testing.assert_allclose(g64[0], m, rtol=1e-11, atol=1e-12 * np.abs(m).max())
    assert_f32_close(g[0], m, cfg.nn, f"{nn}x{nmat}")


@pytest.mark.parametrize("shape", [(160, 120, 3), (33, 7, 2), (200, 100, 4)])
def test_pair_api_on_other_shapes(P, shape):
    """160x120 (the pair runs two threads per path with a tape of terminal
    rates and drift sums; the fused call one thread per path) and the
    warp-per-path shapes (the backward recomputes the forward from the
    same normals): value and vbar-scaled Greeks equal the fused call's."""
    import torch
    nn, nmat, seed = shape
    cfg = cfgs().workload(3, 256) if nn == 160 else _random_cfg(nn, nmat, 6, seed, 256)
    z = O.normals_f32(40 + nn, cfg.paths, cfg.nmat)
    dz = torch.from_numpy(z).cuda()
    with P.Engine(cfg) as e:
        fused, _ = e.greeks_f32(z)
        t = e.tape(cfg.paths)
        val = torch.zeros(1, dtype=torch.float64, device="cuda")
        grad = torch.zeros(2 * cfg.nn, dtype=torch.float64, device="cuda")
        e.forward_f32_device(dz.data_ptr(), cfg.paths, t, val.data_ptr())
        e.backward_f32_device(dz.data_ptr(), t, [-1.5], grad.data_ptr())
        e.synchronize()
        t.close()
    f = fused[0]
    assert val.item() == pytest.approx(f[0], rel=1e-12)
    np.testing.assert_allclose(grad.cpu().numpy(), -1.5 * f[1:], rtol=2e-6, atol=1e-6 * np.abs(f[1:]).max())


def test_pair_api_needs_normals(P):
    """The pair reads its normals from memory: a NULL normals pointer is an
    argument error, for every shape."""
    import torch
    cfg = cfgs().workload(3, 64)
    val = torch.zeros(1, dtype=torch.float64, device="cuda")
    with P.Engine(cfg) as e:
        t = e.tape(64)
        with pytest.raises(P.LmmError) as ei:
            e.forward_f32_device(0, 64, t, val.data_ptr())
        assert ei.value.code == -1
        t.close()


def test_fp32_range_is_never_silently_wrong(P):
    """Long Euler horizons with high vol let some paths' rates approach the
    FP32 range (the FP64 oracle stays finite). The FP32 call must then either
    fail with LMM_ERR_NONFINITE or return results within the FP32 tolerance,
    never garbage; the FP64 call still works."""
    cfg = _random_cfg(200, 150, 6, 350, 64)
    cfg.lam = np.full(200, 0.35)
    z = O.normals_f32(5, cfg.paths, cfg.nmat)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert np.all(np.isfinite(m))
    with P.Engine(cfg) as e:
        try:
            g, _ = e.greeks_f32(z)
        except P.LmmError as ex:
            assert ex.code == -4
        else:
            assert_f32_close(g[0], m, cfg.nn, "200x150 lambda=0.35")
        g64, _ = e.greeks_f64(z.astype(np.float64))
    np.testing.assert_allclose(g64[0], m, rtol=1e-9, atol=1e-10 * np.abs(m).max())


def _host_pieces(paths, sms, blocks_per_sm=1, per_block=384, split=(1, 2, 6, 18, 45)):
    """The pieces the pipelined host call cuts `paths` into: boundaries at the
    cumulative shares of `split` (LMM_HOST_SPLIT), rounded to whole waves of
    the device (sms x blocks per SM x paths per block: one 384-path block per
    SM for the fused 80/40 kernel), empty pieces dropped."""
    wave = sms * blocks_per_sm * per_block
    tot, cum, bnd = sum(split), 0, [0]
    for c in range(1, len(split)):
        cum += split[c - 1]
        x = paths * cum // tot
        bnd.append(min(max((x + wave // 2) // wave * wave, bnd[-1]), paths))
    bnd.append(paths)
    return [(a, b) for a, b in zip(bnd, bnd[1:]) if b > a]


def test_pipelined_host_call_on_an_odd_path_count(P):
    """300,001 paths: the host call copies the normals up in pieces whose
    boundaries fall on whole waves of the device (the last piece takes the odd
    remainder) and launches one kernel per piece plus the finalize; the result
    equals one device call on the same normals, to FP64 summation order."""
    import torch
    cfg = cfgs().workload(2, 300_001)
    z = O.normals_f32(17, cfg.paths, cfg.nmat)
    dz = torch.from_numpy(z).cuda()
    out = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    pieces = _host_pieces(cfg.paths, torch.cuda.get_device_properties(0).multi_processor_count)
    assert len(pieces) >= 2 and pieces[-1][1] == cfg.paths
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
        assert e.last_launches == len(pieces) + 1
        e.greeks_f32_device(dz.data_ptr(), cfg.paths, out.data_ptr())
        e.synchronize()
    d = out.cpu().numpy()
    np.testing.assert_allclose(g[0], d, rtol=1e-11, atol=1e-13 * np.abs(d).max())


def test_full_size_long_tenor_fp32_vs_fp64(P):
    """Workload 3 at its named size (1,048,576 paths, NN=160, NMAT=120, rates
    saved every 8 steps) against the FP64 kernel on identical normals."""
    import torch
    cfg = cfgs().workload(3)
    n = cfg.paths
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(3, n, cfg.nmat, dz.data_ptr())
    dz64 = dz.double()
    o32 = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    o64 = torch.zeros_like(o32)
    with P.Engine(cfg) as e:
        e.greeks_f32_device(dz.data_ptr(), n, o32.data_ptr())
        e.greeks_f64_device(dz64.data_ptr(), n, o64.data_ptr())
        e.synchronize()
    assert_f32_close(o32.cpu().numpy(), o64.cpu().numpy(), cfg.nn, "workload 3 full size")


def test_full_size_scenario_sweep_consistent(P):
    """Workload 5 at its named size (256 curves x 262,144 paths, one launch):
    every scenario finite, and three of them equal to single-curve runs."""
    import torch
    cfg = cfgs().workload(5)
    n = cfg.paths
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(5, n, cfg.nmat, dz.data_ptr())
    out = torch.zeros(cfg.nscen * cfg.nout, dtype=torch.float64, device="cuda")
    with P.Engine(cfg) as e:
        e.greeks_f32_device(dz.data_ptr(), n, out.data_ptr())
        e.synchronize()
    g = out.cpu().numpy().reshape(cfg.nscen, cfg.nout)
    assert np.all(np.isfinite(g))
    for s in (0, 101, 255):
        one = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
        with P.Engine(cfg.scenario(s)) as e1:
            e1.greeks_f32_device(dz.data_ptr(), n, one.data_ptr())
            e1.synchronize()
        r = one.cpu().numpy()
        np.testing.assert_allclose(g[s], r, rtol=1e-9, atol=1e-12 * np.abs(r).max())


@pytest.mark.parametrize("nn,nmat,nopt", [(80, 40, 64), (96, 60, 64), (2, 1, 1), (3, 2, 2)])
def test_portfolio_and_shape_limits(P, nn, nmat, nopt):
    """The largest portfolio (64 swaptions: every bit of the payoff mask) on both
    FP32 kernel families, and the smallest shapes (NN=2, NMAT=1)."""
    cfg = _random_cfg(nn, nmat, nopt, 7000 + nn + nopt, 600)
    z = O.normals_f32(nn + nopt, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
        g64, _ = e.greeks_f64(z.astype(np.float64))
    m, _ = O.greeks(cfg, z.astype(np.float64))
    np.testing.assert_allclose(g64[0], m, rtol=1e-11, atol=1e-12 * np.abs(m).max())
    if np.abs(m).max() > 0:
        assert_f32_close(g[0], m, cfg.nn, f"{nn}x{nmat}, {nopt} swaptions")
    else:                                   # out of the money on every path
        assert np.all(g[0] == 0.0)


@pytest.mark.parametrize("nn,nmat", [(80, 40), (160, 120)])
def test_empty_portfolio_prices_zero(P, nn, nmat):
    """No swaptions: value and every Greek are exactly 0 (FP32 and FP64)."""
    cfg = cfgs().LmmConfig("empty", nn, nmat, 0.25, np.full(nn, 0.05), np.full(nn, 0.2),
                           np.zeros(0, dtype=np.int32), np.zeros(0), 300)
    z = O.normals_f32(5, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, gse = e.greeks_f32(z)
        g64, _ = e.greeks_f64(z.astype(np.float64))
    assert np.all(g == 0.0) and np.all(gse == 0.0) and np.all(g64 == 0.0)


@pytest.mark.parametrize("paths", [300_000, 4_194_304 + 77])
def test_pipelined_host_call_equals_device_call(P, paths):
    """The host call above 2^18 paths copies the normals up in pieces on
    whole waves of the device and launches one kernel per piece: the result
    equals one device call on the same normals, to FP64 summation order."""
    import torch
    cfg = cfgs().workload(2, paths)
    dz = torch.empty(paths * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(61, paths, cfg.nmat, dz.data_ptr())
    z = dz.cpu().numpy()
    out = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    with P.Engine(cfg) as e:
        e.greeks_f32_device(dz.data_ptr(), paths, out.data_ptr())
        e.synchronize()
        g, _ = e.greeks_f32(z, paths)
        assert e.last_launches >= 3
    d = out.cpu().numpy()
    np.testing.assert_allclose(g[0], d, rtol=1e-11, atol=1e-13 * np.abs(d).max())


@pytest.mark.parametrize("paths,nscen", [(1, 1), (77, 1), (300, 2)])
def test_long_tenor_ragged_and_scenarios(P, paths, nscen):
    """160x120: the fused call runs one thread per path in batches of 256
    paths, the forward/backward pair two threads per path in batches of 128;
    a ragged last batch leaves lanes idle, and scenarios loop over units of
    the one-block-per-SM grid. Every scenario matches the FP64 oracle, and the
    pair equals the fused call to FP32 rounding."""
    import torch
    base = cfgs().workload(3, paths)
    cfg = base.with_paths(paths)
    if nscen > 1:
        cfg.L0 = np.stack([base.L0, base.L0 * 1.1])
    nn = cfg.nn
    z = O.normals_f32(500 + paths, paths, cfg.nmat)
    dz = torch.from_numpy(z).cuda()
    val = torch.zeros(nscen, dtype=torch.float64, device="cuda")
    grad = torch.zeros(nscen * 2 * nn, dtype=torch.float64, device="cuda")
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
        t = e.tape(paths)
        e.forward_f32_device(dz.data_ptr(), paths, t, val.data_ptr())
        e.backward_f32_device(dz.data_ptr(), t, [1.0] * nscen, grad.data_ptr())
        e.synchronize()
        t.close()
    v = val.cpu().numpy()
    gr = grad.cpu().numpy().reshape(nscen, 2 * nn)
    for s in range(nscen):
        one = cfg.scenario(s) if nscen > 1 else cfg
        m, _ = O.greeks(one, z.astype(np.float64))
        assert_f32_close(g[s], m, nn, f"160x120 {paths} paths scenario {s}")
        assert v[s] == pytest.approx(g[s][0], rel=1e-12)
        np.testing.assert_allclose(gr[s], g[s][1:], rtol=2e-6, atol=1e-6 * np.abs(g[s][1:]).max())

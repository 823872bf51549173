"""GPU parity of the MRG32k3a stream (csrc/lmm_mrg.cu) through the C ABI,
against the oracle's restatement: uniforms bit-exact, normals bit-exact in
the central branch of AS241 (|u - 1/2| <= 0.425, no log; values within 1e-6
of the branch boundary are left to the tolerance check, since the FP32 path
branches on its FP32 q) and within a few units in the last place in the tails;
the reference-signature calls that draw z from this stream."""
import numpy as np
import pytest

from conftest import cfgs, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _dev(n, dtype):
    import torch
    return torch.full((max(n, 1),), float("nan"), dtype=dtype, device="cuda")


@pytest.mark.parametrize("seed,first,count", [
    (12345, 0, 100_000),            # the reference's stream from its start
    (7, 123_457, 65_537),           # ragged start and length
    (12345, 2**40 + 3, 5_000),      # far skip-ahead
    (1, 16_383, 16_385),            # across the per-warp chunk boundary (32 x 512)
    (12345, 0, 1),
])
def test_uniforms_bit_exact(seed, first, count):
    import torch
    P = pkg()
    d = _dev(count, torch.float64)
    P.mrg32k3a_uniforms_device(seed, first, count, d.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d[:count].cpu().numpy(), O.mrg32k3a_uniforms(seed, first, count))


def test_zero_count_writes_nothing():
    import torch
    P = pkg()
    d = _dev(4, torch.float64)
    P.mrg32k3a_uniforms_device(12345, 10, 0, d.data_ptr())
    P.mrg32k3a_normals_f32_device(12345, 10, 0, 0)
    torch.cuda.synchronize()
    assert torch.isnan(d).all()


@pytest.mark.parametrize("first,count,mean,sd", [(0, 200_000, 0.0, 1.0), (999_999, 70_001, 0.5, 2.0)])
def test_normals_f64(first, count, mean, sd):
    import torch
    P = pkg()
    d = _dev(count, torch.float64)
    P.mrg32k3a_normals_f64_device(12345, first, count, d.data_ptr(), mean=mean, sd=sd)
    torch.cuda.synchronize()
    g = d.cpu().numpy()
    r = O.mrg32k3a_normals_f64(12345, first, count, mean, sd)
    u = O.mrg32k3a_uniforms(12345, first, count)
    central = np.abs(u - 0.5) <= 0.425
    np.testing.assert_array_equal(g[central], r[central])
    np.testing.assert_allclose(g[~central], r[~central], rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("first,count,mean,sd", [(0, 200_000, 0.0, 1.0), (40 * 7, 40 * 1001, -1.0, 0.5)])
def test_normals_f32(first, count, mean, sd):
    import torch
    P = pkg()
    d = _dev(count, torch.float32)
    P.mrg32k3a_normals_f32_device(12345, first, count, d.data_ptr(), mean=mean, sd=sd)
    torch.cuda.synchronize()
    g = d.cpu().numpy()
    r = O.mrg32k3a_normals_f32(12345, first, count, mean, sd)
    u = O.mrg32k3a_uniforms(12345, first, count)
    central = np.abs(u - 0.5) <= 0.425 - 1e-6
    np.testing.assert_array_equal(g[central], r[central])
    # the tails go through logf: CUDA's and the host's may differ by an ulp
    np.testing.assert_allclose(g[~central], r[~central], rtol=1e-6, atol=1e-6)


def test_invalid_arguments():
    P = pkg()
    lib = P.lib()
    assert lib.lmm_mrg32k3a_uniforms_device(1, -1, 5, 16, None) == -1
    assert lib.lmm_mrg32k3a_uniforms_device(1, 0, -5, 16, None) == -1
    assert lib.lmm_mrg32k3a_uniforms_device(1, 2**62, 2**62, 16, None) == -1
    assert lib.lmm_mrg32k3a_normals_f64_device(1, 0, 5, 0.0, 1.0, None, None) == -1
    assert lib.lmm_mrg32k3a_normals_f64_device(1, 0, 5, 0.0, float("inf"), 16, None) == -1


def test_reference_signature_with_mrg_stream_fp64():
    P = pkg()
    n = 4096
    z, v, lb = P.swaption_greeks(n, rng="mrg32k3a")
    zr = O.mrg32k3a_normals_f64(12345, 0, 40 * n)
    u = O.mrg32k3a_uniforms(12345, 0, 40 * n)
    central = np.abs(u - 0.5) <= 0.425
    np.testing.assert_array_equal(z[central], zr[central])
    np.testing.assert_allclose(z, zr, rtol=1e-14, atol=1e-14)
    cfg = cfgs().reference_params(n)
    m, _ = O.greeks(cfg, z)
    assert v == pytest.approx(m[0], rel=1e-12)
    assert lb == pytest.approx(m[cfg.nn], rel=1e-11)
    # a different stream from the default (Philox) call
    z2, v2, _ = P.swaption_greeks(n)
    assert not np.allclose(z2[:100], z[:100])


def test_reference_signature_with_mrg_stream_fp32():
    P = pkg()
    n = 8192
    z, v, lb = P.swaption_greeks_f32(n, rng="mrg32k3a")
    zr = O.mrg32k3a_normals_f32(12345, 0, 40 * n)
    np.testing.assert_allclose(z, zr, rtol=1e-6, atol=1e-6)
    cfg = cfgs().reference_params(n)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert v == pytest.approx(m[0], rel=1e-4)
    assert lb == pytest.approx(m[cfg.nn], rel=1e-4, abs=1e-4 * np.abs(m[1:1 + cfg.nn]).max())

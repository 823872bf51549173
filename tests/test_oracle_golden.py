"""The oracle against the reference's golden vectors (CPU only).

The oracle is what every GPU parity test compares against, so it is pinned
here first: Philox known answers, bit-level agreement with the unmodified
reference in bug-compatible mode, and the reference's own finite differences
for every delta and vega of the fixed adjoint.
"""
import numpy as np
import pytest

from conftest import cfg_from_record, cfgs, normals_from_record
from oracle import oracle as O


def test_philox_known_answers(golden):
    for kat in golden["philox_kat"]:
        assert O.philox4x32_10(kat["ctr"], kat["key"]) == kat["out"]
    # The published Random123 vector for ctr=key=0 (independent of the fixture file).
    assert O.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]


def test_normals_are_standard_and_reproducible():
    z = O.normals_f64(5, 20000, 40)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    z2 = O.normals_f64(5, 100, 40, path0=19900)
    np.testing.assert_array_equal(z[19900 * 40:], z2)       # counter-based: any path range
    z32 = O.normals_f32(5, 1000, 40)
    assert abs(z32.astype(np.float64).mean()) < 0.02


@pytest.mark.parametrize("case", ["entry_f64_256", "entry_f64_4096"])
def test_oracle_matches_reference_entry_fp64(golden, case):
    g = golden["cases"][case]
    z = normals_from_record(g["normals"])
    cfg = cfg_from_record(g["cfg"], g["normals"]["paths"])
    m, _ = O.greeks(cfg, z)
    # The reference repeats the whole MC NLOOPS times and divides by numPaths
    # only (liborSwaptionGreeks.cpp:278,355-356): its outputs are NLOOPS x mean.
    assert m[0] == pytest.approx(g["d_v"] / g["nloops"], rel=1e-12)
    assert m[cfg.nn] == pytest.approx(g["d_Lb"] / g["nloops"], rel=1e-12)


def test_oracle_matches_reference_entry_fp32_build(golden):
    g = golden["cases"]["entry_f32_4096"]
    z = normals_from_record(g["normals"])
    cfg = cfg_from_record(g["cfg"], g["normals"]["paths"])
    m, _ = O.greeks(cfg, z.astype(np.float64))
    # FP32 reference vs FP64 oracle on the same (float) normals.
    assert m[0] == pytest.approx(g["d_v"] / g["nloops"], rel=2e-5)
    assert m[cfg.nn] == pytest.approx(g["d_Lb"] / g["nloops"], rel=2e-5)


@pytest.mark.parametrize("case", ["paths_f64_w1", "paths_f64_w4"])
def test_bug_compatible_mode_reproduces_reference_bit_for_bit(golden, case):
    g = golden["cases"][case]
    z = normals_from_record(g["normals"])
    cfg = cfg_from_record(g["cfg"], 32)
    pp = O.per_path(cfg, z, 32, aliased=True)
    np.testing.assert_allclose(pp[:, 0], g["value"], rtol=1e-14, atol=0)
    lb = np.array(g["Lb_aliased"])
    np.testing.assert_allclose(pp[:, 1:cfg.nn + 1], lb, rtol=1e-12, atol=1e-12 * np.abs(lb).max())
    # The fixed adjoint agrees with the aliased one only on the last rate.
    fixed = O.per_path(cfg, z, 32, aliased=False)
    np.testing.assert_allclose(fixed[:, cfg.nn], lb[:, -1], rtol=1e-13)
    assert np.max(np.abs(fixed[:, 1:cfg.nn] - lb[:, :-1])) > 1.0


@pytest.mark.parametrize("case", ["fd_f64_w1", "fd_f64_w4"])
def test_fixed_adjoint_matches_reference_finite_differences(golden, case):
    g = golden["cases"][case]
    z = normals_from_record(g["normals"])
    cfg = cfg_from_record(g["cfg"], g["normals"]["paths"])
    m, _ = O.greeks(cfg, z)
    assert m[0] == pytest.approx(g["value"], rel=1e-13)
    d_fd, v_fd = np.array(g["delta_fd"]), np.array(g["vega_fd"])
    # Central FD at h=1e-6 in FP64: truncation + rounding ~1e-8 of the scale.
    assert np.max(np.abs(m[1:cfg.nn + 1] - d_fd)) <= 1e-7 * np.abs(d_fd).max()
    assert np.max(np.abs(m[cfg.nn + 1:] - v_fd)) <= 1e-7 * np.abs(v_fd).max()
    assert m[-1] == 0.0 and abs(v_fd[-1]) < 1e-9   # lambda[NN-1] is never read


def test_long_tenor_oracle_vs_reference(golden):
    g = golden["cases"].get("w3_f64_160x120")
    if g is None:
        pytest.skip("long-tenor reference case not generated")
    z = normals_from_record(g["normals"])
    cfg = cfg_from_record(g["cfg"], 16)
    pp = O.per_path(cfg, z, 16, aliased=True)
    np.testing.assert_allclose(pp[:, 0], g["value"], rtol=1e-13)
    lb = np.array(g["Lb_aliased"])
    np.testing.assert_allclose(pp[:, 1:cfg.nn + 1], lb, rtol=1e-11, atol=1e-11 * np.abs(lb).max())
    m, _ = O.greeks(cfg, z, 16)
    d_fd, v_fd = np.array(g["delta_fd"]), np.array(g["vega_fd"])
    assert np.max(np.abs(m[1:cfg.nn + 1] - d_fd)) <= 1e-6 * np.abs(d_fd).max()
    assert np.max(np.abs(m[cfg.nn + 1:] - v_fd)) <= 1e-6 * np.abs(v_fd).max()


def test_oracle_self_consistency_fd_and_ragged_paths():
    cfg = cfgs().workload(4, 37)                 # 37: not a multiple of the 16-lane block
    z = O.normals_f64(99, 37, 40)
    m, se = O.greeks(cfg, z)
    fd = O.fd_greeks(cfg, z, h=1e-6)
    assert np.max(np.abs(m[1:] - fd[1:])) <= 1e-6 * np.abs(fd[1:]).max()
    pp = O.per_path(cfg, z, 37)
    np.testing.assert_allclose(pp.mean(axis=0), m, rtol=1e-12, atol=1e-14)
    assert np.all(se >= 0)


def test_reference_work_port_matches_oracle():
    cfg = cfgs().workload(1, 256)
    z = O.normals_f64(3, 256, 40)
    v, d = O.reference_work(cfg, z, 256)
    m, _ = O.greeks(cfg, z)
    assert v == pytest.approx(m[0], rel=1e-13) and d == pytest.approx(m[cfg.nn], rel=1e-13)


def test_tuned_cpu_baseline_build_computes_the_same_work():
    """The timed CPU baseline (the oracle's source under the reference-like
    fast-math flags) returns the checker's value and last delta to rounding:
    it times the same work, not a different one."""
    cfg = cfgs().workload(2, 4096)
    z = O.normals_f64(5, 4096, 40)
    v, d = O.reference_work(cfg, z, 4096, build="checker")
    vt, dt = O.reference_work(cfg, z, 4096, build="tuned")
    assert vt == pytest.approx(v, rel=1e-10) and dt == pytest.approx(d, rel=1e-9)

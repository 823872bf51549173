"""The MRG32k3a + AS241 restatement in the oracle (oracle/lmm_mrg_oracle.c)
against published values: the skip-ahead matrix powers A^(2^76) and A^(2^127)
listed by L'Ecuyer, Simard, Chen and Kelton (Operations Research 50(6), 2002,
the RngStreams package), the inverse normal CDF against scipy, and stream
consistency (skip-ahead equals sequential generation)."""
import numpy as np
import pytest

from oracle import oracle as O

# Published matrix powers of the two MRG32k3a components (mod m1, mod m2).
A1P76 = [[82758667, 1871391091, 4127413238], [3672831523, 69195019, 1871391091],
         [3672091415, 3528743235, 69195019]]
A2P76 = [[1511326704, 3759209742, 1610795712], [4292754251, 1511326704, 3889917532],
         [3859662829, 4292754251, 3708466080]]
A1P127 = [[2427906178, 3580155704, 949770784], [226153695, 1230515664, 3580155704],
          [1988835001, 986791581, 1230515664]]
A2P127 = [[1464411153, 277697599, 1610723613], [32183930, 1464411153, 1022607788],
          [2824425944, 32183930, 2093834863]]


def test_skip_ahead_matrices_match_published_powers():
    a1, a2 = O.mrg32k3a_pow2(76)
    assert a1 == A1P76 and a2 == A2P76
    a1, a2 = O.mrg32k3a_pow2(127)
    assert a1 == A1P127 and a2 == A2P127


def test_skip_ahead_equals_sequential():
    u = O.mrg32k3a_uniforms(12345, 0, 300_000)
    for first in (1, 2, 3, 39, 40, 1023, 65_536, 299_990):
        np.testing.assert_array_equal(O.mrg32k3a_uniforms(12345, first, 10)[: 300_000 - first],
                                      u[first:first + 10])
    # far jumps compose: [F, F+10) then [F+5, F+10)
    for F in (2**40 + 3, 2**62 - 17):
        a = O.mrg32k3a_uniforms(99, F, 10)
        b = O.mrg32k3a_uniforms(99, F + 5, 5)
        np.testing.assert_array_equal(a[5:], b)


def test_uniforms_are_open_unit_interval_and_uniform():
    u = O.mrg32k3a_uniforms(12345, 0, 1_000_000)
    assert u.min() > 0.0 and u.max() < 1.0
    # Kolmogorov-Smirnov distance of 1e6 uniforms: 1.63/sqrt(n) is the 1% level
    s = np.sort(u)
    d = np.max(np.abs(s - (np.arange(1, s.size + 1) / s.size)))
    assert d < 1.63 / np.sqrt(s.size)
    # seeds give different streams
    assert not np.array_equal(u[:100], O.mrg32k3a_uniforms(12346, 0, 100))


def test_ppnd16_against_scipy():
    sp = pytest.importorskip("scipy.special")
    p = np.concatenate([np.linspace(1e-6, 1 - 1e-6, 100_001), np.logspace(-300, -1, 2000),
                        1 - np.logspace(-16, -1, 300), [0.075, 0.925, 0.5 - 1e-12]])
    x = O.ppnd16(p)
    r = sp.ndtri(p)
    big = np.abs(r) > 1e-12
    assert np.max(np.abs(x - r)[big] / np.abs(r)[big]) < 4e-15
    assert np.max(np.abs(x - r)[~big]) < 1e-16


def test_normals_follow_the_stream():
    sp = pytest.importorskip("scipy.special")
    u = O.mrg32k3a_uniforms(12345, 1000, 50_000)
    z = O.mrg32k3a_normals_f64(12345, 1000, 50_000, mean=0.25, sd=2.0)
    np.testing.assert_allclose(z, 0.25 + 2.0 * sp.ndtri(u), rtol=4e-15, atol=4e-15)
    zf = O.mrg32k3a_normals_f32(12345, 1000, 50_000)
    # PPND7 is accurate to about 1e-7 relative; FP32 rounding adds an ulp or two
    np.testing.assert_allclose(zf, sp.ndtri(u), rtol=5e-7, atol=1e-7)


def test_normal_moments():
    z = O.mrg32k3a_normals_f64(12345, 0, 1_000_000)
    n = z.size
    assert abs(z.mean()) < 5 / np.sqrt(n)
    assert abs(z.var() - 1.0) < 5 * np.sqrt(2.0 / n)
    assert abs(np.mean(z**3)) < 5 * np.sqrt(15.0 / n)

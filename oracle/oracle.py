"""ctypes bindings of the oracle (oracle/lmm_oracle.c) and of the reference
harness (oracle/ref_harness.cpp). TEST INFRASTRUCTURE ONLY: the checker, never
the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_ref

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_refs: dict = {}


class OracleParams(C.Structure):
    _fields_ = [("nn", C.c_int32), ("nmat", C.c_int32), ("nopt", C.c_int32),
                ("reserved", C.c_int32), ("delta", C.c_double),
                ("L0", C.POINTER(C.c_double)), ("lam", C.POINTER(C.c_double)),
                ("maturities", C.POINTER(C.c_int32)), ("swaprates", C.POINTER(C.c_double)),
                ("weights", C.POINTER(C.c_double))]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build_oracle()
        L = C.CDLL(path)
        P = C.POINTER(OracleParams)
        dp, fp = C.POINTER(C.c_double), C.POINTER(C.c_float)
        L.lmmo_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                         C.POINTER(C.c_uint32)]
        L.lmmo_normals_f64.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int32,
                                       C.c_double, C.c_double, dp]
        L.lmmo_normals_f32.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int32, fp]
        L.lmmo_paths.argtypes = [P, dp, C.c_int64, C.c_int32, C.c_int32, dp]
        L.lmmo_greeks.argtypes = [P, dp, C.c_int64, C.c_int32, C.c_int32, dp, dp]
        L.lmmo_value.argtypes = [P, dp, C.c_int64, C.c_int32, dp, dp]
        L.lmmo_fd_greeks.argtypes = [P, dp, C.c_int64, C.c_double, C.c_int32, dp]
        L.lmmo_reference_work.argtypes = [P, dp, C.c_int64, C.c_int32, dp, dp]
        u64p = C.POINTER(C.c_uint64)
        L.lmmo_mrg32k3a_pow2.argtypes = [C.c_int32, u64p, u64p]
        L.lmmo_mrg32k3a_uniforms.argtypes = [C.c_uint32, C.c_int64, C.c_int64, dp]
        L.lmmo_mrg32k3a_normals_f64.argtypes = [C.c_uint32, C.c_int64, C.c_int64, C.c_double,
                                                C.c_double, dp]
        L.lmmo_mrg32k3a_normals_f32.argtypes = [C.c_uint32, C.c_int64, C.c_int64, C.c_float,
                                                C.c_float, fp]
        L.lmmo_ppnd16_array.argtypes = [dp, C.c_int64, dp]
        for f in ("lmmo_paths", "lmmo_greeks", "lmmo_value", "lmmo_fd_greeks",
                  "lmmo_reference_work", "lmmo_max_threads"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


class _Bound:
    """Keeps the numpy arrays a params struct points into alive."""

    def __init__(self, cfg, L0=None, lam=None, weights=None):
        self.L0 = np.ascontiguousarray(cfg.L0 if L0 is None else L0, dtype=np.float64)
        self.lam = np.ascontiguousarray(cfg.lam if lam is None else lam, dtype=np.float64)
        assert self.L0.ndim == 1, "the oracle takes one curve; loop over scenarios"
        self.mat = np.ascontiguousarray(cfg.maturities, dtype=np.int32)
        self.rates = np.ascontiguousarray(cfg.swaprates, dtype=np.float64)
        self.w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        assert self.w is None or self.w.shape == self.rates.shape
        self.p = OracleParams(cfg.nn, cfg.nmat, int(self.mat.shape[0]), 0, float(cfg.delta),
                              _dp(self.L0), _dp(self.lam),
                              self.mat.ctypes.data_as(C.POINTER(C.c_int32)), _dp(self.rates),
                              _dp(self.w) if self.w is not None else None)


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().lmmo_philox4x32_10(c, k, o)
    return [int(x) for x in o]


def normals_f64(seed, paths, nmat, path0=0, mean=0.0, sd=1.0):
    z = np.empty(paths * nmat, dtype=np.float64)
    lib().lmmo_normals_f64(seed, path0, paths, nmat, mean, sd, _dp(z))
    return z


def normals_f32(seed, paths, nmat, path0=0):
    z = np.empty(paths * nmat, dtype=np.float32)
    lib().lmmo_normals_f32(seed, path0, paths, nmat, z.ctypes.data_as(C.POINTER(C.c_float)))
    return z


def mrg32k3a_pow2(k):
    """(A1^(2^k) mod m1, A2^(2^k) mod m2) as 3x3 integer lists."""
    a1 = (C.c_uint64 * 9)()
    a2 = (C.c_uint64 * 9)()
    lib().lmmo_mrg32k3a_pow2(k, a1, a2)
    return [list(a1[3 * i:3 * i + 3]) for i in range(3)], [list(a2[3 * i:3 * i + 3]) for i in range(3)]


def mrg32k3a_uniforms(seed, first, count):
    u = np.empty(count, dtype=np.float64)
    lib().lmmo_mrg32k3a_uniforms(seed, first, count, _dp(u))
    return u


def mrg32k3a_normals_f64(seed, first, count, mean=0.0, sd=1.0):
    z = np.empty(count, dtype=np.float64)
    lib().lmmo_mrg32k3a_normals_f64(seed, first, count, mean, sd, _dp(z))
    return z


def mrg32k3a_normals_f32(seed, first, count, mean=0.0, sd=1.0):
    z = np.empty(count, dtype=np.float32)
    lib().lmmo_mrg32k3a_normals_f32(seed, first, count, mean, sd, z.ctypes.data_as(C.POINTER(C.c_float)))
    return z


def ppnd16(p):
    p = np.ascontiguousarray(p, dtype=np.float64)
    x = np.empty_like(p)
    lib().lmmo_ppnd16_array(_dp(p), p.size, _dp(x))
    return x


def _z64(z):
    return np.ascontiguousarray(z, dtype=np.float64)


def greeks(cfg, z, paths=None, aliased=False, threads=0, L0=None, lam=None, weights=None):
    """(mean[1+2nn], se[1+2nn]): value, dV/dL0[i], dV/dlambda[k]; `weights`
    scales each swaption's payoff (default all 1, the reference's portfolio)."""
    b = _Bound(cfg, L0, lam, weights)
    z = _z64(z)
    paths = cfg.paths if paths is None else paths
    m = np.zeros(cfg.nout)
    s = np.zeros(cfg.nout)
    rc = lib().lmmo_greeks(C.byref(b.p), _dp(z), paths, int(aliased), threads, _dp(m), _dp(s))
    if rc:
        raise RuntimeError(f"lmmo_greeks failed ({rc})")
    return m, s


def per_path(cfg, z, paths, aliased=False, want_vega=True):
    b = _Bound(cfg)
    z = _z64(z)
    r = np.zeros((paths, cfg.nout))
    rc = lib().lmmo_paths(C.byref(b.p), _dp(z), paths, int(want_vega), int(aliased), _dp(r))
    if rc:
        raise RuntimeError(f"lmmo_paths failed ({rc})")
    return r


def value(cfg, z, paths=None, threads=0, L0=None, lam=None):
    b = _Bound(cfg, L0, lam)
    z = _z64(z)
    m, s = C.c_double(), C.c_double()
    rc = lib().lmmo_value(C.byref(b.p), _dp(z), cfg.paths if paths is None else paths, threads,
                          C.byref(m), C.byref(s))
    if rc:
        raise RuntimeError(f"lmmo_value failed ({rc})")
    return m.value, s.value


def fd_greeks(cfg, z, paths=None, h=1e-6, threads=0):
    b = _Bound(cfg)
    z = _z64(z)
    out = np.zeros(cfg.nout)
    rc = lib().lmmo_fd_greeks(C.byref(b.p), _dp(z), cfg.paths if paths is None else paths, h,
                              threads, _dp(out))
    if rc:
        raise RuntimeError(f"lmmo_fd_greeks failed ({rc})")
    return out


_cpubase = None


def cpubase_lib():
    """liblmm_cpubase.so: the oracle's source built like the reference's own
    CPU build (build_ref.CPUBASE_FLAGS); timed, never used as the checker."""
    global _cpubase
    if _cpubase is None:
        L = C.CDLL(build_ref.build_cpu_baseline())
        L.lmmo_reference_work.argtypes = [C.POINTER(OracleParams), C.POINTER(C.c_double), C.c_int64,
                                          C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.lmmo_reference_work.restype = C.c_int
        _cpubase = L
    return _cpubase


def reference_work(cfg, z, paths, threads=0, build="checker"):
    """The CPU-baseline port: the reference's per-path work (value + delta
    adjoint). build="checker": the oracle library (portable flags);
    build="tuned": liblmm_cpubase.so (reference-like flags)."""
    b = _Bound(cfg)
    z = _z64(z)
    v, d = C.c_double(), C.c_double()
    L = cpubase_lib() if build == "tuned" else lib()
    rc = L.lmmo_reference_work(C.byref(b.p), _dp(z), paths, threads, C.byref(v), C.byref(d))
    if rc:
        raise RuntimeError(f"lmmo_reference_work failed ({rc})")
    return v.value, d.value


def max_threads():
    return int(lib().lmmo_max_threads())


# ---------------------------------------------------------------------------
# the unmodified reference, compiled from its own sources (only where present)
# ---------------------------------------------------------------------------

class RefLib:
    def __init__(self, path):
        L = C.CDLL(path)
        self.L = L
        for f in ("ref_nn", "ref_nmat", "ref_nopt", "ref_simdvlen", "ref_nloops",
                  "ref_real_bytes"):
            getattr(L, f).restype = C.c_int
        self.nn, self.nmat = L.ref_nn(), L.ref_nmat()
        self.nopt, self.simd = L.ref_nopt(), L.ref_simdvlen()
        self.nloops = L.ref_nloops()
        self.dtype = np.float64 if L.ref_real_bytes() == 8 else np.float32
        self.ct = C.c_double if self.dtype == np.float64 else C.c_float

    def _p(self, a):
        return a.ctypes.data_as(C.POINTER(self.ct))

    def entry(self, z, num_paths):
        """liborSwaptionGreeks on z (NMAT*num_paths normals). Returns (d_v, d_Lb)
        exactly as the reference reports them (NLOOPS x the MC mean)."""
        z = np.ascontiguousarray(z, dtype=self.dtype).copy()
        v, lb = self.ct(), self.ct()
        self.L.ref_entry(self._p(z), num_paths, C.byref(v), C.byref(lb))
        return float(v.value), float(lb.value)

    def block(self, z, L0, lam, value_only=False):
        """One SIMDVLEN block: (value[simd], Lb[nn, simd]) from the static kernels."""
        z = np.ascontiguousarray(z, dtype=self.dtype)
        L0 = np.ascontiguousarray(L0, dtype=self.dtype)
        lam = np.ascontiguousarray(lam, dtype=self.dtype)
        v = np.zeros(self.simd, dtype=self.dtype)
        if value_only:
            self.L.ref_block_value(self._p(z), self._p(L0), self._p(lam), self._p(v))
            return v
        lb = np.zeros((self.nn, self.simd), dtype=self.dtype)
        self.L.ref_block(self._p(z), self._p(L0), self._p(lam), self._p(v), self._p(lb))
        return v, lb

    def paths(self, z, paths, L0, lam):
        """Per-path value and aliased rate adjoint for paths % SIMDVLEN == 0."""
        assert paths % self.simd == 0
        vals, lbs = [], []
        for b in range(paths // self.simd):
            v, lb = self.block(z[b * self.simd * self.nmat:(b + 1) * self.simd * self.nmat], L0, lam)
            vals.append(v)
            lbs.append(lb.T)
        return np.concatenate(vals).astype(np.float64), np.concatenate(lbs).astype(np.float64)

    def values(self, z, paths, L0, lam):
        assert paths % self.simd == 0
        out = []
        for b in range(paths // self.simd):
            out.append(self.block(z[b * self.simd * self.nmat:(b + 1) * self.simd * self.nmat],
                                  L0, lam, value_only=True))
        return np.concatenate(out).astype(np.float64)

    def portfolio(self):
        mat = (C.c_int * self.nopt)()
        rates = (C.c_double * self.nopt)()
        self.L.ref_portfolio(mat, rates)
        return np.array(mat[:], dtype=np.int32), np.array(rates[:])


def reference(tag="f64"):
    """The reference build `tag`, or None where the reference tree is absent."""
    if tag not in _refs:
        built = build_ref.build_reference()
        _refs[tag] = RefLib(built[tag]) if tag in built else None
    return _refs[tag]

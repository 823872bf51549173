"""GB300-native LIBOR Market Model swaption-portfolio Monte Carlo with pathwise Greeks.

Python binding (ctypes) of the C ABI declared in include/lmm_gb300.h. The
compute lives in liblmm_gb300.so (CUDA for sm_103a, built in-tree by
build_lib.py); there is no CPU fallback: without the library every call raises.

Device pointers are plain integers (e.g. ``torch.Tensor.data_ptr()``); host
arrays are numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import configs  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "liblmm_gb300.so")

LMM_OK = 0
STATUS = {0: "ok", -1: "invalid argument", -2: "unsupported", -3: "CUDA error",
          -4: "non-finite result", -5: "no CUDA device", -6: "too large", -7: "out of device memory"}

# Every symbol include/lmm_gb300.h declares.
EXPORTS = (
    "lmm_validate_params", "lmm_num_outputs", "lmm_status_string", "lmm_last_error", "lmm_version",
    "lmm_engine_create", "lmm_engine_destroy", "lmm_engine_set_stream", "lmm_engine_synchronize",
    "lmm_engine_last_launches", "lmm_engine_set_timing", "lmm_engine_kernel_time", "lmm_fp32_peak_tflops",
    "lmm_greeks_f32_host", "lmm_greeks_f32_device", "lmm_greeks_philox_host", "lmm_greeks_philox_device",
    "lmm_tape_create", "lmm_tape_destroy", "lmm_forward_f32_device", "lmm_backward_f32_device",
    "lmm_greeks_f64_host", "lmm_greeks_f64_device", "lmm_bump_greeks_f64_device",
    "lmm_bump_greeks_f64_host", "lmm_bump_greeks_central_f64_device", "lmm_bump_greeks_central_f64_host",
    "lmm_greeks_f32_rounding_device", "lmm_normals_f32_device", "lmm_normals_f64_device",
    "lmm_swaption_greeks", "lmm_swaption_greeks_f32", "lmm_greeks_f32_device_noalloc",
    "lmm_mrg32k3a_uniforms_device", "lmm_mrg32k3a_normals_f64_device", "lmm_mrg32k3a_normals_f32_device",
    "lmm_swaption_greeks_mrg32k3a", "lmm_swaption_greeks_mrg32k3a_f32",
    "lmm_engine_set_weights", "lmm_swaption_breakdown_f32_device", "lmm_swaption_breakdown_f64_device",
    "lmm_mufu_peak_gops", "lmm_fp64_peak_tflops", "lmm_engine_set_checkpoint_interval",
    "lmm_engine_checkpoint_interval",
)


class LmmError(RuntimeError):
    def __init__(self, code, what, detail=""):
        super().__init__(f"{what}: {STATUS.get(code, code)} ({code}){': ' + detail if detail else ''}")
        self.code = code


class LmmParams(C.Structure):
    _fields_ = [("nn", C.c_int32), ("nmat", C.c_int32), ("nopt", C.c_int32), ("nscen", C.c_int32),
                ("delta", C.c_double), ("L0", C.POINTER(C.c_double)), ("lam", C.POINTER(C.c_double)),
                ("maturities", C.POINTER(C.c_int32)), ("swaprates", C.POINTER(C.c_double))]


_lib = None


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile liblmm_gb300.so for sm_103a (needs nvcc, not a GPU)."""
    from . import build_lib
    return build_lib.build(force=force, verbose=verbose)


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LmmError(-2, "load", f"{LIB_PATH} is missing: run build() first")
    L = C.CDLL(LIB_PATH)
    vp, i64, i32, u64 = C.c_void_p, C.c_int64, C.c_int32, C.c_uint64
    dp, fp = C.POINTER(C.c_double), C.POINTER(C.c_float)
    P = C.POINTER(LmmParams)
    sig = {
        "lmm_validate_params": ([P], C.c_int),
        "lmm_num_outputs": ([P], i64),
        "lmm_status_string": ([C.c_int], C.c_char_p),
        "lmm_last_error": ([], C.c_char_p),
        "lmm_version": ([], C.c_char_p),
        "lmm_engine_create": ([P, i32, C.POINTER(vp)], C.c_int),
        "lmm_engine_destroy": ([vp], C.c_int),
        "lmm_engine_set_stream": ([vp, vp], C.c_int),
        "lmm_engine_synchronize": ([vp], C.c_int),
        "lmm_engine_last_launches": ([vp], i32),
        "lmm_engine_set_timing": ([vp, i32], C.c_int),
        "lmm_engine_kernel_time": ([vp, dp, dp], C.c_int),
        "lmm_fp32_peak_tflops": ([i32, C.c_double, dp], C.c_int),
        "lmm_mufu_peak_gops": ([i32, C.c_double, dp, dp, dp], C.c_int),
        "lmm_fp64_peak_tflops": ([i32, C.c_double, dp], C.c_int),
        "lmm_greeks_f32_host": ([vp, fp, i64, dp, dp], C.c_int),
        "lmm_greeks_f32_device": ([vp, vp, i64, vp, vp], C.c_int),
        "lmm_greeks_philox_host": ([vp, u64, i64, i64, dp, dp], C.c_int),
        "lmm_greeks_philox_device": ([vp, u64, i64, i64, vp, vp], C.c_int),
        "lmm_tape_create": ([vp, i64, C.POINTER(vp)], C.c_int),
        "lmm_tape_destroy": ([vp], C.c_int),
        "lmm_forward_f32_device": ([vp, vp, i64, vp, vp, vp], C.c_int),
        "lmm_backward_f32_device": ([vp, vp, vp, dp, vp, vp], C.c_int),
        "lmm_greeks_f64_host": ([vp, dp, i64, dp, dp], C.c_int),
        "lmm_greeks_f64_device": ([vp, vp, i64, vp, vp], C.c_int),
        "lmm_bump_greeks_f64_device": ([vp, vp, i64, C.c_double, vp, vp], C.c_int),
        "lmm_bump_greeks_f64_host": ([vp, dp, i64, C.c_double, dp, dp], C.c_int),
        "lmm_bump_greeks_central_f64_device": ([vp, vp, i64, C.c_double, vp, vp], C.c_int),
        "lmm_bump_greeks_central_f64_host": ([vp, dp, i64, C.c_double, dp, dp], C.c_int),
        "lmm_greeks_f32_rounding_device": ([vp, vp, i64, vp, vp, vp], C.c_int),
        "lmm_normals_f32_device": ([u64, i64, i64, i32, vp, vp], C.c_int),
        "lmm_normals_f64_device": ([u64, i64, i64, i32, C.c_double, C.c_double, vp, vp], C.c_int),
        "lmm_swaption_greeks": ([dp, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp, C.c_int], C.c_int),
        "lmm_swaption_greeks_f32": ([fp, C.c_int, C.c_float, C.c_float, C.c_int, fp, fp, C.c_int], C.c_int),
        "lmm_greeks_f32_device_noalloc": ([P, vp, i64, vp, vp, vp], C.c_int),
        "lmm_engine_set_weights": ([vp, dp], C.c_int),
        "lmm_engine_set_checkpoint_interval": ([vp, i32], C.c_int),
        "lmm_engine_checkpoint_interval": ([vp], i32),
        "lmm_swaption_breakdown_f32_device": ([vp, vp, i64, vp, vp], C.c_int),
        "lmm_swaption_breakdown_f64_device": ([vp, vp, i64, vp, vp], C.c_int),
        "lmm_mrg32k3a_uniforms_device": ([C.c_uint32, i64, i64, vp, vp], C.c_int),
        "lmm_mrg32k3a_normals_f64_device": ([C.c_uint32, i64, i64, C.c_double, C.c_double, vp, vp], C.c_int),
        "lmm_mrg32k3a_normals_f32_device": ([C.c_uint32, i64, i64, C.c_float, C.c_float, vp, vp], C.c_int),
        "lmm_swaption_greeks_mrg32k3a": ([dp, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp, C.c_int],
                                         C.c_int),
        "lmm_swaption_greeks_mrg32k3a_f32": ([fp, C.c_int, C.c_float, C.c_float, C.c_int, fp, fp, C.c_int],
                                             C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def engine_lib():
    return lib()


def last_error() -> str:
    return lib().lmm_last_error().decode()


def _check(rc, what):
    if rc != LMM_OK:
        raise LmmError(rc, what, last_error())


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class _ParamsRef:
    """A LmmParams struct plus the numpy arrays it points into."""

    def __init__(self, cfg):
        self.L0 = np.ascontiguousarray(np.atleast_2d(cfg.L0), dtype=np.float64)
        self.lam = np.ascontiguousarray(cfg.lam, dtype=np.float64)
        self.mat = np.ascontiguousarray(cfg.maturities, dtype=np.int32)
        self.rates = np.ascontiguousarray(cfg.swaprates, dtype=np.float64)
        self.p = LmmParams(int(cfg.nn), int(cfg.nmat), int(self.mat.shape[0]), int(self.L0.shape[0]),
                           float(cfg.delta), _dp(self.L0), _dp(self.lam),
                           self.mat.ctypes.data_as(C.POINTER(C.c_int32)), _dp(self.rates))


def validate(cfg) -> int:
    r = _ParamsRef(cfg)
    return int(lib().lmm_validate_params(C.byref(r.p)))


class Engine:
    """One lmm_engine: a model/portfolio (and its scenario curves) on one GPU."""

    def __init__(self, cfg, device: int = 0):
        self.cfg = cfg
        self._ref = _ParamsRef(cfg)
        self.nn, self.nmat, self.nscen = int(cfg.nn), int(cfg.nmat), int(self._ref.L0.shape[0])
        self.nopt = int(len(cfg.swaprates))
        self.nout = 1 + 2 * self.nn
        h = C.c_void_p()
        _check(lib().lmm_engine_create(C.byref(self._ref.p), device, C.byref(h)), "lmm_engine_create")
        self.h = h
        if getattr(cfg, "ckpt_every", None) is not None:
            self.set_checkpoint_interval(cfg.ckpt_every)

    def close(self):
        if getattr(self, "h", None):
            lib().lmm_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr: int):
        _check(lib().lmm_engine_set_stream(self.h, C.c_void_p(stream_ptr)), "lmm_engine_set_stream")

    def synchronize(self):
        _check(lib().lmm_engine_synchronize(self.h), "lmm_engine_synchronize")

    def set_checkpoint_interval(self, steps: int):
        """Steps between the rate checkpoints of the FP32 reverse sweep (0: none)."""
        _check(lib().lmm_engine_set_checkpoint_interval(self.h, int(steps)), "lmm_engine_set_checkpoint_interval")

    @property
    def checkpoint_interval(self) -> int:
        return int(lib().lmm_engine_checkpoint_interval(self.h))

    @property
    def last_launches(self) -> int:
        return int(lib().lmm_engine_last_launches(self.h))

    def set_timing(self, on: bool = True):
        _check(lib().lmm_engine_set_timing(self.h, int(on)), "lmm_engine_set_timing")

    def kernel_time(self):
        """(main kernel ms, whole call ms) of the last compute call (waits for it)."""
        a, b = C.c_double(), C.c_double()
        _check(lib().lmm_engine_kernel_time(self.h, C.byref(a), C.byref(b)), "lmm_engine_kernel_time")
        return a.value, b.value

    def _outs(self, n):
        return np.zeros(self.nscen * n), np.zeros(self.nscen * n)

    def greeks_f32(self, z: np.ndarray, paths: int | None = None):
        """Value + all Greeks, FP32 adjoint, host normals z[paths*nmat] (float32)."""
        z = np.ascontiguousarray(z, dtype=np.float32)
        paths = z.size // self.nmat if paths is None else paths
        out, se = self._outs(self.nout)
        _check(lib().lmm_greeks_f32_host(self.h, _fp(z), paths, _dp(out), _dp(se)), "lmm_greeks_f32_host")
        return out.reshape(self.nscen, self.nout), se.reshape(self.nscen, self.nout)

    def greeks_f32_device(self, d_z: int, paths: int, d_out: int, d_se: int = 0):
        _check(lib().lmm_greeks_f32_device(self.h, d_z, paths, d_out, d_se or None), "lmm_greeks_f32_device")

    def greeks_f32_rounding_device(self, d_z: int, paths: int, d_out: int, d_se: int, d_err: int):
        """FP32 results plus |FP32 - FP64| per output on the identical normals."""
        _check(lib().lmm_greeks_f32_rounding_device(self.h, d_z, paths, d_out, d_se or None, d_err),
               "lmm_greeks_f32_rounding_device")

    def greeks_philox(self, seed: int, paths: int, path0: int = 0):
        out, se = self._outs(self.nout)
        _check(lib().lmm_greeks_philox_host(self.h, seed, path0, paths, _dp(out), _dp(se)),
               "lmm_greeks_philox_host")
        return out.reshape(self.nscen, self.nout), se.reshape(self.nscen, self.nout)

    def greeks_philox_device(self, seed: int, paths: int, d_out: int, d_se: int = 0, path0: int = 0):
        _check(lib().lmm_greeks_philox_device(self.h, seed, path0, paths, d_out, d_se or None),
               "lmm_greeks_philox_device")

    def greeks_f64(self, z: np.ndarray, paths: int | None = None):
        z = np.ascontiguousarray(z, dtype=np.float64)
        paths = z.size // self.nmat if paths is None else paths
        out, se = self._outs(self.nout)
        _check(lib().lmm_greeks_f64_host(self.h, _dp(z), paths, _dp(out), _dp(se)), "lmm_greeks_f64_host")
        return out.reshape(self.nscen, self.nout), se.reshape(self.nscen, self.nout)

    def greeks_f64_device(self, d_z: int, paths: int, d_out: int, d_se: int = 0):
        _check(lib().lmm_greeks_f64_device(self.h, d_z, paths, d_out, d_se or None), "lmm_greeks_f64_device")

    def bump_greeks_f64(self, z: np.ndarray, h: float, paths: int | None = None, central: bool = False):
        """FP64 bump-and-revalue Greeks: one-sided, or central (+h and -h) differences."""
        z = np.ascontiguousarray(z, dtype=np.float64)
        paths = z.size // self.nmat if paths is None else paths
        out, se = self._outs(self.nout)
        fn = "lmm_bump_greeks_central_f64_host" if central else "lmm_bump_greeks_f64_host"
        _check(getattr(lib(), fn)(self.h, _dp(z), paths, h, _dp(out), _dp(se)), fn)
        return out.reshape(self.nscen, self.nout), se.reshape(self.nscen, self.nout)

    def bump_greeks_f64_device(self, d_z: int, paths: int, h: float, d_out: int, d_se: int = 0,
                               central: bool = False):
        fn = "lmm_bump_greeks_central_f64_device" if central else "lmm_bump_greeks_f64_device"
        _check(getattr(lib(), fn)(self.h, d_z, paths, h, d_out, d_se or None), fn)

    # portfolio weights and per-swaption breakdown
    def set_weights(self, weights=None):
        """Notional weight per swaption (order of the config's swaprates); None = all 1."""
        if weights is None:
            _check(lib().lmm_engine_set_weights(self.h, None), "lmm_engine_set_weights")
            return
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.shape != (self.nopt,):
            raise LmmError(-1, "set_weights", f"need {self.nopt} weights")
        _check(lib().lmm_engine_set_weights(self.h, _dp(w)), "lmm_engine_set_weights")

    def breakdown_f32_device(self, d_z: int, paths: int, d_out: int, d_se: int = 0):
        """[nopt][nscen][1+2nn]: each swaption's value and Greeks at unit weight."""
        _check(lib().lmm_swaption_breakdown_f32_device(self.h, d_z, paths, d_out, d_se or None),
               "lmm_swaption_breakdown_f32_device")

    def breakdown_f64_device(self, d_z: int, paths: int, d_out: int, d_se: int = 0):
        _check(lib().lmm_swaption_breakdown_f64_device(self.h, d_z, paths, d_out, d_se or None),
               "lmm_swaption_breakdown_f64_device")

    # forward/backward pair
    def tape(self, paths: int) -> "Tape":
        return Tape(self, paths)

    def forward_f32_device(self, d_z: int, paths: int, tape: "Tape", d_value: int, d_value_se: int = 0):
        _check(lib().lmm_forward_f32_device(self.h, d_z, paths, tape.h, d_value, d_value_se or None),
               "lmm_forward_f32_device")

    def backward_f32_device(self, d_z: int, tape: "Tape", value_bar, d_grad: int, d_grad_se: int = 0):
        vb = np.ascontiguousarray(np.atleast_1d(value_bar), dtype=np.float64)
        _check(lib().lmm_backward_f32_device(self.h, d_z, tape.h, _dp(vb), d_grad, d_grad_se or None),
               "lmm_backward_f32_device")


class Tape:
    def __init__(self, eng: Engine, paths: int):
        self.eng, self.paths = eng, paths
        h = C.c_void_p()
        _check(lib().lmm_tape_create(eng.h, paths, C.byref(h)), "lmm_tape_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().lmm_tape_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fp32_peak_tflops(device: int = 0, ms: float = 200.0) -> float:
    """Measured FP32 FMA throughput of the device (roofline denominator)."""
    t = C.c_double()
    _check(lib().lmm_fp32_peak_tflops(device, ms, C.byref(t)), "lmm_fp32_peak_tflops")
    return t.value


def fp64_peak_tflops(device: int = 0, ms: float = 200.0) -> float:
    """Measured FP64 FMA throughput of the device (FP64 kernels' roofline)."""
    t = C.c_double()
    _check(lib().lmm_fp64_peak_tflops(device, ms, C.byref(t)), "lmm_fp64_peak_tflops")
    return t.value


def mufu_peak_gops(device: int = 0, ms: float = 100.0) -> dict:
    """Measured MUFU throughput (10^9 ops/s): ex2, rcp and the two alternating."""
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    _check(lib().lmm_mufu_peak_gops(device, ms, C.byref(a), C.byref(b), C.byref(c)), "lmm_mufu_peak_gops")
    return {"ex2": a.value, "rcp": b.value, "mixed": c.value}


def normals_f32_device(seed: int, paths: int, nmat: int, d_z: int, stream: int = 0, path0: int = 0):
    _check(lib().lmm_normals_f32_device(seed, path0, paths, nmat, d_z, stream or None),
           "lmm_normals_f32_device")


def normals_f64_device(seed: int, paths: int, nmat: int, d_z: int, stream: int = 0, path0: int = 0,
                       mean: float = 0.0, sd: float = 1.0):
    _check(lib().lmm_normals_f64_device(seed, path0, paths, nmat, mean, sd, d_z, stream or None),
           "lmm_normals_f64_device")


def mrg32k3a_uniforms_device(seed: int, first: int, count: int, d_u: int, stream: int = 0):
    """Stream elements [first, first+count) of MRG32k3a as FP64 uniforms in (0,1)."""
    _check(lib().lmm_mrg32k3a_uniforms_device(seed, first, count, d_u, stream or None),
           "lmm_mrg32k3a_uniforms_device")


def mrg32k3a_normals_f64_device(seed: int, first: int, count: int, d_z: int, stream: int = 0,
                                mean: float = 0.0, sd: float = 1.0):
    _check(lib().lmm_mrg32k3a_normals_f64_device(seed, first, count, mean, sd, d_z, stream or None),
           "lmm_mrg32k3a_normals_f64_device")


def mrg32k3a_normals_f32_device(seed: int, first: int, count: int, d_z: int, stream: int = 0,
                                mean: float = 0.0, sd: float = 1.0):
    _check(lib().lmm_mrg32k3a_normals_f32_device(seed, first, count, mean, sd, d_z, stream or None),
           "lmm_mrg32k3a_normals_f32_device")


def swaption_greeks(num_paths: int, mean: float = 0.0, std_dev: float = 1.0, seed: int = 1234,
                    rng: str = "philox"):
    """The reference's liborSwaptionGreeks call (FP64). Returns (z, d_v, d_Lb).
    rng = "mrg32k3a" draws z from the MRG32k3a/AS241 stream instead."""
    z = np.zeros(40 * num_paths)
    v, lb = C.c_double(), C.c_double()
    name = {"philox": "lmm_swaption_greeks", "mrg32k3a": "lmm_swaption_greeks_mrg32k3a"}[rng]
    _check(getattr(lib(), name)(_dp(z), 40 * num_paths, mean, std_dev, seed, C.byref(v), C.byref(lb),
                                num_paths), name)
    return z, v.value, lb.value


def swaption_greeks_f32(num_paths: int, mean: float = 0.0, std_dev: float = 1.0, seed: int = 1234,
                        rng: str = "philox"):
    z = np.zeros(40 * num_paths, dtype=np.float32)
    v, lb = C.c_float(), C.c_float()
    name = {"philox": "lmm_swaption_greeks_f32", "mrg32k3a": "lmm_swaption_greeks_mrg32k3a_f32"}[rng]
    _check(getattr(lib(), name)(_fp(z), 40 * num_paths, mean, std_dev, seed, C.byref(v),
                                C.byref(lb), num_paths), name)
    return z, v.value, lb.value

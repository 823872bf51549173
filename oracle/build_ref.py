"""Build recipe for the oracle libraries (test infrastructure only).

  oracle/_build/liblmm_oracle.so   the FP64 C restatement (oracle/lmm_oracle.c) and
                                   the MRG32k3a/AS241 stream (oracle/lmm_mrg_oracle.c)
  oracle/_build/liblmm_cpubase.so  the same sources under reference-like flags
                                   (fast math, explicit vector target): the
                                   timed CPU baseline, not the checker
  oracle/_ref/libref_<tag>.so      the UNMODIFIED reference
                                   LiborMarketModel/liborSwaptionGreeks.cpp,
                                   compiled where it lies together with
                                   oracle/ref_harness.cpp and oracle/shim/

The reference builds need the reference tree: set LMM_REFERENCE_ROOT to the
directory that holds LiborMarketModel/. Without it they are skipped.
Reference shapes other than the default NN=80/NMAT=40 are built against a
configuration header generated here (same macro names as params.h, other
values); GCC's -I- makes the reference's quoted #include "params.h" resolve
to it instead of the file beside liborSwaptionGreeks.cpp.

Usage: python oracle/build_ref.py [--oracle-only]
"""
from __future__ import annotations

import importlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("LMM_REFERENCE_ROOT", "")
LMM_DIR = os.path.join(REF_ROOT, "LiborMarketModel") if REF_ROOT else ""


def _cfg_module():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    return importlib.import_module("financial-services-workload-samples_gb300.configs")


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _cpu_target_flags():
    """An explicit target CPU for the timed baseline build (never -march=native,
    so that what is built is the same wherever the recipe runs): Neoverse V2
    (the Grace cores) on aarch64, AVX2 on x86-64, as the reference's build
    targets core-avx2 (LiborMarketModel/compile.sh)."""
    import platform
    m = platform.machine().lower()
    if m in ("aarch64", "arm64"):
        return ["-mcpu=neoverse-v2"]
    if m in ("x86_64", "amd64"):
        return ["-march=x86-64-v3"]
    return []


# The timed CPU baseline: the same source built the way the reference builds
# its own (LiborMarketModel/compile.sh: -O3, OpenMP, a vector ISA target, the
# compiler's fast floating-point model with vector math, which icpc applies by
# default and GCC under -ffast-math). It is timed, never used as the checker:
# fast math may contract and reorder, so its results are not bitwise the
# checker's.
CPUBASE_FLAGS = ["-O3", "-std=c99", "-fopenmp", "-ffast-math", "-fPIC", "-shared", "-w"]


def build_oracle(force=False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "lmm_oracle.c"), os.path.join(HERE, "lmm_mrg_oracle.c")]
    out = os.path.join(BUILD, "liblmm_oracle.so")
    if force or _stale(out, srcs):
        tmp = out + f".tmp{os.getpid()}"
        _run(["gcc", "-O3", "-std=c99", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wextra",
              "-Wno-unused-parameter", *srcs, "-o", tmp, "-lm"])
        os.replace(tmp, out)
    return out


def build_cpu_baseline(force=False) -> str:
    """liblmm_cpubase.so: the oracle's source under the reference-like flags
    (CPUBASE_FLAGS plus an explicit target CPU), for bench.py's timed CPU legs."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "lmm_oracle.c"), os.path.join(HERE, "lmm_mrg_oracle.c")]
    out = os.path.join(BUILD, "liblmm_cpubase.so")
    if force or _stale(out, srcs):
        tmp = out + f".tmp{os.getpid()}"
        _run(["gcc", *CPUBASE_FLAGS, *_cpu_target_flags(), *srcs, "-o", tmp, "-lm"])
        os.replace(tmp, out)
    return out


PARAMS_TEMPLATE = """/* Generated by oracle/build_ref.py: configuration header for the reference
 * harness, shape {tag}. Same macro names as LiborMarketModel/params.h, other values. */
#ifndef LMM_REF_GENERATED_PARAMS_H
#define LMM_REF_GENERATED_PARAMS_H
#ifdef USE_DOUBLE
typedef double REAL;
#define ONE 1.0
#define ZERO 0.0
#define HALF 0.5
#define HUNDRED 100.0
const int SIMDVLEN = 16;
#else
typedef float REAL;
#define ONE 1.0f
#define ZERO 0.0f
#define HALF 0.5f
#define HUNDRED 100.0f
const int SIMDVLEN = 32;
#endif
#define NN {nn}
#define NMAT {nmat}
#define L2_SIZE ({nn} * ({nmat} + 1))
#define NOPT {nopt}
#define SEED 1
#define DELTA ((REAL){delta!r})
#define SQRT_DELTA ((REAL){sqrt_delta!r})
#define BLOCK 16
const int maturities[] = {{{mats}}};
const REAL swaprates[] = {{{rates}}};
#endif
"""


def ref_shapes():
    """Reference builds: tag -> (USE_DOUBLE, config or None for params.h as shipped)."""
    cfgm = _cfg_module()
    return {
        "f64": (True, None),
        "f32": (False, None),
        "f64_160x120": (True, cfgm.workload(3)),
    }


def build_reference(force=False) -> dict:
    """Returns {tag: path} for the reference builds; {} without the reference tree."""
    if not LMM_DIR or not os.path.isfile(os.path.join(LMM_DIR, "liborSwaptionGreeks.cpp")):
        return {}
    os.makedirs(REF_OUT, exist_ok=True)
    harness = os.path.join(HERE, "ref_harness.cpp")
    deps = [harness, os.path.join(HERE, "shim", "mkl_vsl.h"),
            os.path.join(LMM_DIR, "liborSwaptionGreeks.cpp"), os.path.join(LMM_DIR, "params.h")]
    out = {}
    for tag, (dbl, cfg) in ref_shapes().items():
        so = os.path.join(REF_OUT, f"libref_{tag}.so")
        cmd = ["g++", "-std=c++11", "-O3", "-fopenmp", "-fPIC", "-shared", "-w"]
        if dbl:
            cmd.append("-DUSE_DOUBLE")
        if cfg is not None:
            pdir = os.path.join(REF_OUT, f"params_{tag}")
            os.makedirs(pdir, exist_ok=True)
            mats = ", ".join(str(int(m)) for m in cfg.maturities)
            rates = ", ".join(repr(float(r)) for r in cfg.swaprates)
            text = PARAMS_TEMPLATE.format(tag=tag, nn=cfg.nn, nmat=cfg.nmat, nopt=cfg.nopt,
                                          delta=float(cfg.delta),
                                          sqrt_delta=float(cfg.delta) ** 0.5,
                                          mats=mats, rates=rates)
            ph = os.path.join(pdir, "params.h")
            if not os.path.exists(ph) or open(ph).read() != text:
                with open(ph, "w") as f:
                    f.write(text)
            deps_t = deps + [ph]
            cmd += ["-I" + pdir, "-I-"]
        else:
            deps_t = deps
        cmd += ["-I" + os.path.join(HERE, "shim"), "-I" + LMM_DIR, harness]
        if force or _stale(so, deps_t):
            tmp = so + f".tmp{os.getpid()}"
            _run(cmd + ["-o", tmp])
            os.replace(tmp, so)
        out[tag] = so
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_cpu_baseline(force="--force" in sys.argv))
    if "--oracle-only" not in sys.argv:
        for k, v in build_reference(force="--force" in sys.argv).items():
            print(k, v)

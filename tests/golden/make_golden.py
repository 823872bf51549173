"""Generate tests/golden/reference_golden.json from the UNMODIFIED reference.

Run where the reference tree exists (it builds oracle/_ref/ through
oracle/build_ref.py):  python tests/golden/make_golden.py

Every case feeds the reference normals generated by the Philox4x32-10 +
Box-Muller spec of oracle/lmm_oracle.c (seed, first path and count are stored,
together with checksums, so the tests regenerate the identical array without
the reference). What is recorded, all computed by the reference's own code:

  entry_*     liborSwaptionGreeks (liborSwaptionGreeks.cpp:241) as it reports:
              d_v = NLOOPS x mean value, d_Lb = NLOOPS x mean dV/dL0[NN-1]
              (FP64 build and FP32 build, params.h:10-24).
  paths_*     per-path value and per-path rate adjoint left by path_calc_b2,
              from the static kernels (:34, :86, :120). The adjoint is the
              reference's ALIASED one (:178/:181), so only its last index is a
              true delta; the oracle's bug-compatible mode must match all of it.
  fd_*        central finite differences of the reference's own value
              (path_calc_b1 + portfolio_b) with respect to every L0[i] and
              every lambda[k]: the reference-side pin for all deltas and vegas.
"""
from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

cfgm = importlib.import_module("financial-services-workload-samples_gb300.configs")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")


def zsig(z):
    a = np.ascontiguousarray(z)
    return {"sha256": hashlib.sha256(a.tobytes()).hexdigest(), "sum": float(a.astype(np.float64).sum())}


def normals_case(seed, paths, nmat, dtype="f64"):
    z = O.normals_f64(seed, paths, nmat) if dtype == "f64" else O.normals_f32(seed, paths, nmat)
    return z, {"seed": seed, "path0": 0, "paths": paths, "nmat": nmat, "dtype": dtype, **zsig(z)}


def ref_fd(ref, z, paths, L0, lam, h):
    nn = ref.nn
    out = np.zeros(2 * nn)
    for i in range(nn):
        for off, base in ((0, L0), (nn, lam)):
            up_arr = base.copy(); up_arr[i] += h
            dn_arr = base.copy(); dn_arr[i] -= h
            if off == 0:
                up = ref.values(z, paths, up_arr, lam).mean()
                dn = ref.values(z, paths, dn_arr, lam).mean()
            else:
                up = ref.values(z, paths, L0, up_arr).mean()
                dn = ref.values(z, paths, L0, dn_arr).mean()
            out[off + i] = (up - dn) / (2 * h)
    return out


def cfg_record(cfg):
    return {"nn": cfg.nn, "nmat": cfg.nmat, "delta": cfg.delta, "L0": cfg.L0.tolist(),
            "lam": cfg.lam.tolist(), "maturities": cfg.maturities.tolist(),
            "swaprates": cfg.swaprates.tolist()}


def main():
    ref64 = O.reference("f64")
    ref32 = O.reference("f32")
    ref160 = O.reference("f64_160x120")
    if ref64 is None:
        raise SystemExit("reference tree not found: set LMM_REFERENCE_ROOT")
    g = {"generator": "tests/golden/make_golden.py",
         "philox_kat": [
             # Known-answer vectors of Philox4x32-10 published with Random123
             # (Salmon et al., SC'11): ctr, key, output.
             {"ctr": [0, 0, 0, 0], "key": [0, 0], "out": O.philox4x32_10([0, 0, 0, 0], [0, 0])},
             {"ctr": [0xffffffff] * 4, "key": [0xffffffff] * 2,
              "out": O.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2)},
             {"ctr": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], "key": [0xa4093822, 0x299f31d0],
              "out": O.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                     [0xa4093822, 0x299f31d0])}],
         "cases": {}}
    C = g["cases"]

    # 1) the reference entry point, its own hard-coded curve (L0=0.051, lambda=0.2)
    for paths, seed in ((256, 12345), (4096, 777)):
        z, zrec = normals_case(seed, paths, 40, "f64")
        d_v, d_lb = ref64.entry(z, paths)
        C[f"entry_f64_{paths}"] = {"normals": zrec, "cfg": cfg_record(cfgm.reference_params(paths)),
                                   "nloops": ref64.nloops, "d_v": d_v, "d_Lb": d_lb}
        z32, zrec32 = normals_case(seed, paths, 40, "f32")
        d_v32, d_lb32 = ref32.entry(z32, paths)
        C[f"entry_f32_{paths}"] = {"normals": zrec32, "cfg": cfg_record(cfgm.reference_params(paths)),
                                   "nloops": ref32.nloops, "d_v": d_v32, "d_Lb": d_lb32}

    # 2) per-path value + aliased rate adjoint, workload-1 curve and workload-4 curve
    for tag, cfg, seed in (("w1", cfgm.workload(1, 32), 11), ("w4", cfgm.workload(4, 32), 44)):
        z, zrec = normals_case(seed, 32, 40, "f64")
        v, lb = ref64.paths(z, 32, cfg.L0, cfg.lam)
        C[f"paths_f64_{tag}"] = {"normals": zrec, "cfg": cfg_record(cfg), "value": v.tolist(),
                                 "Lb_aliased": lb.tolist()}

    # 3) reference finite differences: all deltas and vegas
    for tag, cfg, seed, paths in (("w1", cfgm.workload(1, 64), 21, 64),
                                  ("w4", cfgm.workload(4, 64), 24, 64)):
        z, zrec = normals_case(seed, paths, 40, "f64")
        h = 1e-6
        fd = ref_fd(ref64, z, paths, cfg.L0.copy(), cfg.lam.copy(), h)
        v = ref64.values(z, paths, cfg.L0, cfg.lam).mean()
        C[f"fd_f64_{tag}"] = {"normals": zrec, "cfg": cfg_record(cfg), "h": h, "value": v,
                              "delta_fd": fd[:cfg.nn].tolist(), "vega_fd": fd[cfg.nn:].tolist()}

    # 4) long tenor NN=160/NMAT=120 (workload 3 portfolio and curve)
    if ref160 is not None:
        cfg = cfgm.workload(3, 16)
        z, zrec = normals_case(33, 16, 120, "f64")
        v, lb = ref160.paths(z, 16, cfg.L0, cfg.lam)
        h = 1e-6
        fd = ref_fd(ref160, z, 16, cfg.L0.copy(), cfg.lam.copy(), h)
        C["w3_f64_160x120"] = {"normals": zrec, "cfg": cfg_record(cfg), "value": v.tolist(),
                               "Lb_aliased": lb.tolist(), "h": h,
                               "delta_fd": fd[:cfg.nn].tolist(), "vega_fd": fd[cfg.nn:].tolist()}

    with open(OUT, "w") as f:
        json.dump(g, f, indent=0)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()

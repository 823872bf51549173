"""The drop-in shim (shim/liborSwaptionGreeks_gb300.cpp) run on the GPU.

A caller that calls liborSwaptionGreeks as the reference's driver does
(LiborMarketModel/main.cpp:65-86) is compiled against the shim and the
library, with test stand-ins for the reference's params.h and
liborSwaptionGreeks.hpp (tests/dropin_caller/), and run as its own process.
The shim must refill z with the MRG32k3a/AS241 stream (seed 12345, elements
0..num-1), and return NLOOPS = 10 times the Monte Carlo mean value and
dV/dL0[NN-1] of lmm_swaption_greeks_mrg32k3a, as the reference's outputs are
10x the means (liborSwaptionGreeks.cpp:27,355-356), in the FP64 and FP32
builds.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, pkg

pytestmark = pytest.mark.gpu

PKG_DIR = os.path.join(ROOT, "financial-services-workload-samples_gb300")
CALLER = os.path.join(ROOT, "tests", "dropin_caller")
NLOOPS = 10          # liborSwaptionGreeks.cpp:27


def _build(tmp_path, double):
    P = pkg()
    if not os.path.exists(P.LIB_PATH):
        P.build()
    exe = str(tmp_path / ("caller_f64" if double else "caller_f32"))
    cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++11", "-I" + CALLER, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(PKG_DIR, "shim", "include"), os.path.join(CALLER, "caller.cpp"),
           os.path.join(PKG_DIR, "shim", "liborSwaptionGreeks_gb300.cpp"), "-L" + PKG_DIR, "-llmm_gb300",
           "-Wl,-rpath," + PKG_DIR, "-o", exe]
    if double:
        cmd.insert(1, "-DUSE_DOUBLE")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("double", [True, False])
def test_shim_refills_z_and_scales_by_nloops(tmp_path, double):
    import torch
    P = pkg()
    paths = 4096
    exe = _build(tmp_path, double)
    r = subprocess.run([exe, str(paths)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout)
    ftype = np.float64 if double else np.float32
    z_shim = np.array(got["z"], dtype=ftype)

    # z: the MRG32k3a/AS241 stream from element 0, seed 12345, N(0, 1)
    dz = torch.empty(40 * paths, dtype=torch.float64 if double else torch.float32, device="cuda")
    fn = P.mrg32k3a_normals_f64_device if double else P.mrg32k3a_normals_f32_device
    fn(12345, 0, 40 * paths, dz.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(z_shim, dz.cpu().numpy())

    # value and last delta: NLOOPS x the library call's means
    if double:
        _, v, lb = P.swaption_greeks(paths, rng="mrg32k3a")
        assert got["value"] == NLOOPS * v
        assert got["delta"] == NLOOPS * lb
    else:
        _, v, lb = P.swaption_greeks_f32(paths, rng="mrg32k3a")
        assert np.float32(got["value"]) == np.float32(v) * np.float32(NLOOPS)
        assert np.float32(got["delta"]) == np.float32(lb) * np.float32(NLOOPS)
    assert 40 < v < 60 and lb > 0        # the reference portfolio's value per path and its last delta

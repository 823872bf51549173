"""The no-allocation entry point, lmm_greeks_f32_device_noalloc.

It serves callers that cannot allocate device memory (a host application that
owns every allocation through its own pool, a process whose allocator is
locked): it runs the same fused FP32 kernel as lmm_greeks_f32_device, with its
scratch in a static device array instead of an engine's buffers. This file is
named to be collected last; it passes alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import cfgs, pkg

pytestmark = pytest.mark.gpu


def _scaled_err(g, r, nn):
    out = []
    for sl in (slice(0, 1), slice(1, 1 + nn), slice(1 + nn, 1 + 2 * nn)):
        floor = 1e-2 * np.abs(r[sl]).max() if r[sl].size > 1 else 0.0
        den = np.maximum(np.abs(r[sl]), max(floor, 1e-300))
        out.append(np.max(np.abs(g[sl] - r[sl]) / den))
    return max(out)


def _call(P, cfg, dz, paths, out, se, stream):
    ref = P._ParamsRef(cfg)
    return P.lib().lmm_greeks_f32_device_noalloc(C.byref(ref.p), dz.data_ptr(), paths, out.data_ptr(),
                                                 se.data_ptr(), C.c_void_p(stream))


@pytest.mark.parametrize("nscen", [1, 3])
def test_noalloc_matches_engine_on_two_calls_in_a_row(nscen):
    import torch
    P = pkg()
    base = cfgs().workload(5 if nscen > 1 else 4, 100_003)
    cfg = base.with_paths(base.paths)
    if nscen > 1:
        cfg.L0 = base.L0[:nscen].copy()
    n = cfg.paths
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(77, n, cfg.nmat, dz.data_ptr())
    ref = torch.zeros(nscen * cfg.nout, dtype=torch.float64, device="cuda")
    ref_se = torch.zeros_like(ref)
    with P.Engine(cfg) as e:
        e.greeks_f32_device(dz.data_ptr(), n, ref.data_ptr(), ref_se.data_ptr())
        e.synchronize()
    r = ref.cpu().numpy().reshape(nscen, cfg.nout)
    r_se = ref_se.cpu().numpy().reshape(nscen, cfg.nout)
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.full((nscen * cfg.nout,), np.nan, dtype=torch.float64, device="cuda") for _ in range(4)]
    for call in range(2):
        out, se = outs[2 * call], outs[2 * call + 1]
        torch.cuda.synchronize()
        free0, allocated0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
        assert _call(P, cfg, dz, n, out, se, stream) == 0
        torch.cuda.synchronize()
        if call == 1:
            # the first call may load the library's kernels; the second
            # allocates no device memory at all
            assert torch.cuda.mem_get_info()[0] == free0
            assert torch.cuda.memory_allocated() == allocated0
        g = out.cpu().numpy().reshape(nscen, cfg.nout)
        g_se = se.cpu().numpy().reshape(nscen, cfg.nout)
        for s in range(nscen):
            # the engine's fused call runs the split-reverse kernel, this call
            # the one-pass kernel: the same cells, rounded in another order,
            # so they agree within the FP32 rule of the parity tests
            assert _scaled_err(g[s], r[s], cfg.nn) <= 1e-4
            np.testing.assert_allclose(g_se[s], r_se[s], rtol=1e-4)
        if call == 1:
            # the second call sees the first call's leftovers in the shared
            # array and still returns the same bits
            np.testing.assert_array_equal(outs[2].cpu().numpy(), outs[0].cpu().numpy())
            np.testing.assert_array_equal(outs[3].cpu().numpy(), outs[1].cpu().numpy())


def test_noalloc_limits_are_errors():
    import torch
    P = pkg()
    dz = torch.zeros(64 * 120, dtype=torch.float32, device="cuda")
    out = torch.zeros(321, dtype=torch.float64, device="cuda")
    se = torch.zeros_like(out)
    assert _call(P, cfgs().workload(3, 64), dz, 64, out, se, 0) == -2          # nn=160: unsupported
    many = cfgs().workload(5, 64)                                              # 256 curves > 8
    assert _call(P, many, dz, 64, out, se, 0) == -6
    one = cfgs().workload(1, 64)
    assert _call(P, one, dz, 0, out, se, 0) == -1
    assert "paths" in P.last_error()


def test_noalloc_replays_from_a_cuda_graph():
    """After a first call outside any capture (which looks up the static
    scratch and the occupancy), the call enqueues only kernels on the given
    stream -- the model constants travel as a kernel's parameters, not as a
    copy from host memory -- so a stream capture records it, and replays,
    with the host's parameter struct gone, return the direct call's bits."""
    import torch
    P = pkg()
    cfg = cfgs().workload(2, 40_000)
    n = cfg.paths
    dz = torch.empty(n * cfg.nmat, dtype=torch.float32, device="cuda")
    P.normals_f32_device(31, n, cfg.nmat, dz.data_ptr())
    out_d = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    se_d = torch.zeros_like(out_d)
    out_g = torch.zeros_like(out_d)
    se_g = torch.zeros_like(out_d)
    s = torch.cuda.Stream()
    assert _call(P, cfg, dz, n, out_d, se_d, s.cuda_stream) == 0
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        assert _call(P, cfg, dz, n, out_g, se_g, s.cuda_stream) == 0
    for _ in range(3):
        out_g.zero_()
        se_g.zero_()
        g.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out_g.cpu().numpy(), out_d.cpu().numpy())
    np.testing.assert_array_equal(se_g.cpu().numpy(), se_d.cpu().numpy())

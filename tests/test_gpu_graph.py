"""Device calls inside CUDA graphs: after one call of a given size has sized
the engine's buffers, lmm_greeks_f32_device and the MRG32k3a generator enqueue
only kernels and async memsets on the engine's stream, so a stream capture
records them and replays give bit-identical results."""
import numpy as np
import pytest

from conftest import cfgs, pkg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("wl,paths", [(2, 65536), (3, 2048)])
def test_fused_call_replays_from_a_cuda_graph(wl, paths):
    import torch
    P = pkg()
    cfg = cfgs().workload(wl, paths)
    dz = torch.empty(paths * cfg.nmat, dtype=torch.float32, device="cuda")
    out_direct = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    out_graph = torch.zeros(cfg.nout, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    with P.Engine(cfg) as e:
        e.set_stream(s.cuda_stream)
        with torch.cuda.stream(s):
            P.mrg32k3a_normals_f32_device(12345, 0, paths * cfg.nmat, dz.data_ptr(), stream=s.cuda_stream)
            e.greeks_f32_device(dz.data_ptr(), paths, out_direct.data_ptr())   # sizes the buffers
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            P.mrg32k3a_normals_f32_device(12345, 0, paths * cfg.nmat, dz.data_ptr(), stream=s.cuda_stream)
            e.greeks_f32_device(dz.data_ptr(), paths, out_graph.data_ptr())
        for _ in range(3):
            out_graph.zero_()
            g.replay()
        torch.cuda.synchronize()
        e.set_stream(0)
    np.testing.assert_array_equal(out_graph.cpu().numpy(), out_direct.cpu().numpy())

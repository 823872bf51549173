"""The forward/backward C-ABI pair as a torch.autograd.Function (test harness
only): d(value)/dL0 and d(value)/dlambda through autograd must equal the fused
call's deltas and vegas, and scale with the upstream gradient."""
import numpy as np
import pytest

from conftest import cfgs, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_fn(P, eng, dz, paths):
    import torch

    class LmmValue(torch.autograd.Function):
        """value = E[discounted payoff](L0, lambda) for fixed normals."""

        @staticmethod
        def forward(ctx, L0, lam):
            tape = eng.tape(paths)
            val = torch.zeros(1, dtype=torch.float64, device="cuda")
            eng.forward_f32_device(dz.data_ptr(), paths, tape, val.data_ptr())
            eng.synchronize()
            ctx.tape = tape
            return val

        @staticmethod
        def backward(ctx, gval):
            grad = torch.zeros(2 * eng.nn, dtype=torch.float64, device="cuda")
            eng.backward_f32_device(dz.data_ptr(), ctx.tape, [float(gval.item())], grad.data_ptr())
            eng.synchronize()
            ctx.tape.close()
            return grad[:eng.nn].clone(), grad[eng.nn:].clone()

    return LmmValue.apply


def test_autograd_function_gives_adjoint_greeks():
    import torch
    P = pkg()
    cfg = cfgs().workload(4, 20000)
    z = O.normals_f32(31, cfg.paths, cfg.nmat)
    dz = torch.from_numpy(z).cuda()
    with P.Engine(cfg) as eng:
        fused, _ = eng.greeks_f32(z)
        f = make_fn(P, eng, dz, cfg.paths)
        L0 = torch.tensor(cfg.L0, device="cuda", requires_grad=True)
        lam = torch.tensor(cfg.lam, device="cuda", requires_grad=True)
        v = f(L0, lam)
        (3.0 * v).sum().backward()
    g = fused[0]
    assert v.item() == pytest.approx(g[0], rel=1e-12)
    np.testing.assert_allclose(L0.grad.cpu().numpy(), 3.0 * g[1:1 + cfg.nn], rtol=2e-6,
                               atol=1e-6 * np.abs(g[1:1 + cfg.nn]).max())
    np.testing.assert_allclose(lam.grad.cpu().numpy(), 3.0 * g[1 + cfg.nn:], rtol=2e-6,
                               atol=1e-6 * np.abs(g[1 + cfg.nn:]).max())
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert np.max(np.abs(L0.grad.cpu().numpy() / 3.0 - m[1:1 + cfg.nn])) <= 1e-4 * np.abs(m[1:1 + cfg.nn]).max()

"""The checkpoint interval of the FP32 reverse sweep (lmm_engine_set_checkpoint_interval).

The reference stores the whole rate trajectory of a path block for its reverse
sweep (params.h:29 L2_SIZE, liborSwaptionGreeks.cpp:76). The long-tenor
kernels here rebuild each step backwards from saved drift sums and restore
saved rates every k steps; k is an engine setting. Every k must give the
oracle's Greeks within the FP32 rule, and the setter must refuse what a
kernel cannot take.
"""
import numpy as np
import pytest

from conftest import cfgs
from oracle import oracle as O
from test_gpu_parity import _random_cfg, assert_f32_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from conftest import pkg
    return pkg()


@pytest.mark.parametrize("k", [0, 4, 8, 12, 16, 116])
def test_long_tenor_interval_matches_oracle(P, k):
    """160x120 (the fused call: one thread per path in 40-rate block passes),
    30 swaptions, random curve and vols:
    rates restored every k steps (0: never), on the same normals for every k
    (those of test_long_tenor_checkpointed_fp32_matches_oracle)."""
    cfg = cfgs().workload(3, 512)
    cfg.ckpt_every = k
    z = O.normals_f32(303, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        assert e.checkpoint_interval == k
        g, _ = e.greeks_f32(z)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert_f32_close(g[0], m, cfg.nn, f"160x120 k={k}")


@pytest.mark.parametrize("k", [0, 4, 8, 16])
def test_warp_per_path_interval_matches_oracle(P, k):
    """A warp-per-path shape (200x100): rates restored every k steps."""
    cfg = _random_cfg(200, 100, 12, 200 * 1000 + 100, 384)
    cfg.ckpt_every = k
    z = O.normals_f32(9200, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        g, _ = e.greeks_f32(z)
    m, _ = O.greeks(cfg, z.astype(np.float64))
    assert_f32_close(g[0], m, cfg.nn, f"200x100 k={k}")


def test_interval_changes_only_rounding(P):
    """Within one engine, moving k between calls changes the Greeks by FP32
    rounding only, and the value not at all (the forward is the same)."""
    cfg = cfgs().workload(3, 256)
    z = O.normals_f32(77, cfg.paths, cfg.nmat)
    with P.Engine(cfg) as e:
        assert e.checkpoint_interval == 8
        g8, _ = e.greeks_f32(z)
        e.set_checkpoint_interval(4)
        g2, _ = e.greeks_f32(z)
        e.set_checkpoint_interval(8)
        g8b, _ = e.greeks_f32(z)
    np.testing.assert_array_equal(g8, g8b)
    assert g2[0, 0] == g8[0, 0]
    np.testing.assert_allclose(g2[0], g8[0], rtol=1e-4, atol=1e-4 * np.abs(g8[0, 1:]).max())


def test_interval_errors(P):
    """80/40 keeps every drift sum on chip and takes no rate checkpoints; the
    160/120 fused kernel restores checkpoints between groups of four reverse
    steps (k not a multiple of 4 is refused); k must lie in [0, nmat]. A
    refused setting leaves the interval as it was."""
    with P.Engine(cfgs().workload(2, 64)) as e:
        assert e.checkpoint_interval == 0
        e.set_checkpoint_interval(0)
        with pytest.raises(P.LmmError) as ei:
            e.set_checkpoint_interval(8)
        assert ei.value.code == -2
        assert e.checkpoint_interval == 0
    with P.Engine(cfgs().workload(3, 64)) as e:
        for bad, code in ((3, -2), (6, -2), (-1, -1), (121, -1)):
            with pytest.raises(P.LmmError) as ei:
                e.set_checkpoint_interval(bad)
            assert ei.value.code == code
        assert e.checkpoint_interval == 8
        e.set_checkpoint_interval(120)
        assert e.checkpoint_interval == 120
    with P.Engine(_random_cfg(33, 7, 2, 5, 64)) as e:
        assert e.checkpoint_interval == 8
        e.set_checkpoint_interval(3)
        assert e.checkpoint_interval == 3

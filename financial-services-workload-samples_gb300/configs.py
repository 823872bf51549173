"""Model and portfolio configurations of the LMM swaption-portfolio Monte Carlo.

The reference fixes its parameters at compile time (LiborMarketModel/params.h:27-40)
and hard-codes the curve inside its entry point (liborSwaptionGreeks.cpp:269-271).
Here they are runtime values; ``reference_params`` reproduces the reference's
own set bit for bit, and ``workload`` builds the five named workloads:

  1. NN=80/NMAT=40, flat L0=0.05, flat lambda=0.2, 15 swaptions, 65,536 paths (FP64)
  2. same model, 4,194,304 paths, FP32 normals read from HBM (the headline)
  3. NN=160/NMAT=120, random L0/lambda, 30 swaptions, 1,048,576 paths, rates saved
     every 8 steps for the reverse sweep
  4. NN=80/NMAT=40, lambda[i]=0.15+0.1exp(-0.05i), L0[i]=0.03+0.0005i, 16,777,216 paths, in-kernel Philox
  5. 256 curves x 262,144 paths in one launch
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# params.h:38 -- swap lengths (in accrual periods) of the 15 payer swaptions.
REF_MATURITIES = np.array([4, 4, 4, 8, 8, 8, 20, 20, 20, 28, 28, 28, 40, 40, 40], dtype=np.int32)
# params.h:39-40 writes the strikes as float literals (.045f, ...), so the FP64
# build of the reference prices with their float-rounded values. Keep that.
REF_SWAPRATES = np.array([0.045, 0.05, 0.055] * 5, dtype=np.float32).astype(np.float64)
REF_NN, REF_NMAT, REF_DELTA = 80, 40, 0.25          # params.h:27-28,33
REF_L0, REF_LAMBDA = 0.051, 0.2                      # liborSwaptionGreeks.cpp:270-271
REF_NLOOPS = 10                                      # liborSwaptionGreeks.cpp:27
REF_NUMPATHS = 131072                                # main.cpp:31


@dataclass
class LmmConfig:
    """One workload: model shape, curve, vols, portfolio and path count.

    ``L0`` is [nn] for a single curve or [nscen, nn] for a scenario sweep.
    ``lam`` is indexed by time to maturity, lam[i-n-1] for rate i at step n,
    exactly as the reference reads it (liborSwaptionGreeks.cpp:65,102).
    """
    name: str
    nn: int
    nmat: int
    delta: float
    L0: np.ndarray
    lam: np.ndarray
    maturities: np.ndarray
    swaprates: np.ndarray
    paths: int
    normals: str = "hbm"          # "hbm": pre-generated array; "philox": in-kernel
    seed: int = 1
    ckpt_every: int | None = None  # steps between the rate checkpoints the FP32 reverse
                                   # sweep restores (Engine applies it through
                                   # lmm_engine_set_checkpoint_interval); 0: none; None:
                                   # the engine's default (8, and none at 80/40)
    extra: dict = field(default_factory=dict)

    @property
    def nopt(self) -> int:
        return int(self.maturities.shape[0])

    @property
    def nscen(self) -> int:
        return 1 if self.L0.ndim == 1 else int(self.L0.shape[0])

    @property
    def nout(self) -> int:
        return 1 + 2 * self.nn

    def with_paths(self, paths: int) -> "LmmConfig":
        c = LmmConfig(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        c.paths = int(paths)
        return c

    def scenario(self, s: int) -> "LmmConfig":
        c = self.with_paths(self.paths)
        c.L0 = np.ascontiguousarray(self.L0[s] if self.L0.ndim == 2 else self.L0)
        return c


def _portfolio_ref():
    return REF_MATURITIES.copy(), REF_SWAPRATES.copy()


def reference_params(paths: int = REF_NUMPATHS) -> LmmConfig:
    """The parameter set the reference binary runs (params.h + :269-271)."""
    mat, rates = _portfolio_ref()
    return LmmConfig("reference-default", REF_NN, REF_NMAT, REF_DELTA,
                     np.full(REF_NN, REF_L0), np.full(REF_NN, REF_LAMBDA), mat, rates, paths)


def par_swap_rate(L0: np.ndarray, nmat: int, delta: float, m: int) -> float:
    """Forward par rate of the swap a maturity-m swaption exercises into, on the
    initial curve: (1 - B_m)/S_m with B, S built as in portfolio_b (:133-143)."""
    b, s = 1.0, 0.0
    for k in range(m):
        b = b / (1.0 + delta * L0[nmat + k])
        s = s + delta * b
    return (1.0 - b) / s


def workload(n: int, paths: int | None = None) -> LmmConfig:
    """Workload n (1..5) at its named size, or at ``paths`` paths."""
    mat, rates = _portfolio_ref()
    if n == 1:
        c = LmmConfig("lmm80x40-flat-65536-fp64", 80, 40, 0.25, np.full(80, 0.05),
                      np.full(80, 0.2), mat, rates, 65536)
    elif n == 2:
        c = LmmConfig("lmm80x40-flat-4194304-fp32adj", 80, 40, 0.25, np.full(80, 0.05),
                      np.full(80, 0.2), mat, rates, 4194304)
    elif n == 3:
        rng = np.random.default_rng(20260603)
        L0 = rng.uniform(0.02, 0.07, 160)
        lam = rng.uniform(0.1, 0.3, 160)
        # Swap lengths must not exceed NN-NMAT=40 (the payoff reads rates
        # NMAT..NMAT+m-1, liborSwaptionGreeks.cpp:133,161), so the six
        # maturities are spread evenly over 8..40 instead of 8..120.
        mats = np.rint(np.linspace(8, 40, 6)).astype(np.int32)
        m_list, k_list = [], []
        for m in mats:
            par = par_swap_rate(L0, 120, 0.25, int(m))
            for bp in (-100, -50, 0, 50, 100):
                m_list.append(int(m))
                k_list.append(par + bp * 1e-4)
        c = LmmConfig("lmm160x120-random-1048576-ckpt8", 160, 120, 0.25, L0, lam,
                      np.array(m_list, dtype=np.int32), np.array(k_list), 1048576,
                      ckpt_every=8)
    elif n == 4:
        i = np.arange(80)
        c = LmmConfig("lmm80x40-volvec-16777216-philox", 80, 40, 0.25, 0.03 + 0.0005 * i,
                      0.15 + 0.1 * np.exp(-0.05 * i), mat, rates, 16777216, normals="philox")
    elif n == 5:
        rng = np.random.default_rng(20260605)
        shift = rng.uniform(-0.02, 0.02, 256)
        slope = rng.uniform(-1e-4, 1e-4, 256)
        i = np.arange(80)
        L0 = 0.05 + shift[:, None] + slope[:, None] * i[None, :]
        c = LmmConfig("lmm80x40-256curves-262144-scenarios", 80, 40, 0.25, L0,
                      np.full(80, 0.2), mat, rates, 262144)
    else:
        raise ValueError(f"unknown workload {n}")
    if paths is not None:
        c.paths = int(paths)
    return c

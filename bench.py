"""Benchmark: LMM swaption-portfolio value + all 2*NN Greeks per second on GB300.

Workload (the headline configuration): NN=80 forward rates, NMAT=40 steps,
delta=0.25, flat L0=0.05, flat lambda=0.2, the 15-swaption portfolio of
LiborMarketModel/params.h:38-40, 4,194,304 paths per step, FP32 N(0,1) normals
[paths x 40] resident in HBM (generated once by the library's Philox4x32-10
generator; synthetic, seeded). A step is one call of the FP32 adjoint:
forward + payoff adjoint + reverse sweep for every path, value + 80 deltas +
80 vegas, reduced in FP64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0). `value` is device-resident throughput (normals
already in HBM, CUDA events on the launching stream); `e2e` is the same metric
through the host C-ABI call lmm_greeks_f32_host with the normals in pinned host
memory (host->device copy and result read-back inside the timed region).
--impl reference times the reference's CPU algorithm for the same workload on
the host cores (the C restatement under oracle/, built like the reference's
own CPU build, since the reference tree is not available where this runs).
"""
from __future__ import annotations

import argparse
import csv
import importlib
import io
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "paths/s value+all Greeks: FP32 adjoint vs FP64 bump, 1 GB300, rel err<=1e-4"
WORKLOAD = 2
# The timed fused kernel and its ncu DRAM-traffic summary, per workload that
# --workload accepts (normals in HBM).
KERNELS = {2: ("k_tps<80,40,hbm>", os.path.join(ROOT, "profiles", "lmm_fused_f32_80x40.json")),
           3: ("k_tpq<160,120,hbm>", os.path.join(ROOT, "profiles", "lmm_fused_f32_160x120.json"))}

# Algorithmic operations per path (reference formulas, liborSwaptionGreeks.cpp),
# counting a divide and an exp as one operation each, C = cells of the
# triangle = sum_{n<NMAT} (NN-1-n):
#   forward  :68-73   9 flops + 1 div + 1 exp   = 11 per cell
#   deltas   :105-111 10 flops + 2 div          = 12 per cell
#   vegas    (derived adjoint) 9 flops          =  9 per cell
#   portfolio_b :120-211                        ~900 per path
OPS_PER_CELL = 32
OPS_PORTFOLIO = 900
# One FP64 forward revaluation (the bump comparator's unit of work): the
# forward cell of :68-73 (11 operations) over the triangle plus the portfolio.
OPS_FWD_CELL = 11
# Special-function (MUFU) operations per path: each cell issues one ex2 and one
# reciprocal in the forward and again in the reverse reconstruction; the
# payoff and its adjoint take 2*NN reciprocals.
MUFU_PER_CELL = 4


# Paths of the FP64 central-difference check in the accuracy section.
CENTRAL_FD_PATHS = 16384
# Wall-clock budget of the reference arm's warm-up and timed steps together.
REF_BUDGET_S = 150.0


def cells(nn, nmat):
    return sum(nn - 1 - n for n in range(nmat))


def pkg():
    return importlib.import_module("financial-services-workload-samples_gb300")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_path0(rank: int, paths_per_rank: int) -> int:
    """First global path index of a rank: replicas take disjoint path ranges
    (Philox counters are keyed by the global path index)."""
    return rank * paths_per_rank


def max_over_ranks(x: float, device=None) -> float:
    """The slowest rank's time (any torch.distributed backend; identity when
    not distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, steps: int, world_size: int, t_max: float) -> float:
    """Units processed by all ranks per second of the slowest rank."""
    return world_size * units_per_rank * steps / t_max


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r for r in csv.reader(io.StringIO(self.out)) if len(r) >= 9]
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons)}


CPUBASE_NOTE = ("the oracle's C restatement of liborSwaptionGreeks.cpp:34-211 built like the reference's own "
                "CPU build (LiborMarketModel/compile.sh: -O3, OpenMP over 16-path blocks, omp simd lanes, "
                "fast floating-point model with vector math, explicit vector target)")


def _time_work(O, cfg, z, n, threads, build):
    t0 = time.perf_counter()
    O.reference_work(cfg, z, n, threads, build=build)
    return max(time.perf_counter() - t0, 1e-6)


def cpu_baseline_port(cfg, target_s=10.0, threads=0):
    """The reference's per-path work (value + delta adjoint) on the host cores,
    through the oracle's C restatement built like the reference's own build,
    on a bounded sample of the workload (about target_s seconds); beside it
    the same on one core and the portable (checker) build on all cores."""
    from oracle import oracle as O
    threads = threads or O.max_threads()
    calib = 4096
    z = O.normals_f64(7, calib, cfg.nmat)
    dt = _time_work(O, cfg, z, calib, threads, "tuned")
    n = int(min(cfg.paths, max(calib, calib * target_s / dt)))
    n = max(16, n - n % 16)
    z = O.normals_f64(7, n, cfg.nmat)
    dt = _time_work(O, cfg, z, n, threads, "tuned")
    n1 = max(16, int(n / max(threads, 1) / 10) // 16 * 16)
    dt1 = _time_work(O, cfg, z, n1, 1, "tuned")
    nc = max(16, n // 4 // 16 * 16)
    dtc = _time_work(O, cfg, z, nc, threads, "checker")
    return {"value": n / dt, "unit": "paths/s", "cores": threads, "kind": "port",
            "value_1core": n1 / dt1, "value_portable_build": nc / dtc,
            "build": "oracle/_build/liblmm_cpubase.so (" + " ".join(O.build_ref.CPUBASE_FLAGS[:5]) + " "
                     + " ".join(O.build_ref._cpu_target_flags()) + ")",
            "sample": f"{n} paths of the same workload (FP64, value + {cfg.nn} deltas by the reference's "
                      f"adjoint; the reference computes no vegas), {dt:.2f} s wall on {threads} threads; "
                      f"value_portable_build: {nc} paths through the checker build (-O3, no fast math)",
            "seconds": dt}


def run_reference_arm(args):
    """The reference's CPU algorithm for the workload, on all host cores: per
    step the workload's full path count when the whole run fits in about
    REF_BUDGET_S seconds, else the largest multiple of 16 paths that does."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cfgm = pkg().configs
    cfg = cfgm.workload(args.workload)
    from oracle import oracle as O
    threads = O.max_threads()
    calib = 65536
    zc = O.normals_f64(11, calib, cfg.nmat)
    _time_work(O, cfg, zc, calib, threads, "tuned")
    per_path = _time_work(O, cfg, zc, calib, threads, "tuned") / calib
    del zc
    fit = int(REF_BUDGET_S / max(per_path, 1e-12) / (args.steps + args.warmup))
    sample = max(16, min(cfg.paths, fit) // 16 * 16)
    z = O.normals_f64(11, sample, cfg.nmat)
    for _ in range(args.warmup):
        O.reference_work(cfg, z, sample, threads, build="tuned")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.reference_work(cfg, z, sample, threads, build="tuned")
    dt = time.perf_counter() - t0
    v = args.steps * sample / dt
    why = ("the workload's full path count" if sample == cfg.paths else
           f"{sample} of the workload's {cfg.paths} paths per step, so that {args.warmup}+{args.steps} "
           f"steps fit in about {REF_BUDGET_S:.0f} s")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "paths/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: Philox4x32-10 + Box-Muller FP64 normals",
            "config": {"workload": cfg.name, "nn": cfg.nn, "nmat": cfg.nmat, "paths_per_step": sample,
                       "paths_per_step_why": why,
                       "work": f"value + {cfg.nn} deltas per path (the reference's adjoint; no vegas)"},
            "cpu_baseline": {"value": v, "unit": "paths/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} paths per step, FP64, " + CPUBASE_NOTE},
            "e2e": {"value": v, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    P = pkg()
    if not os.path.exists(P.LIB_PATH):
        P.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    cfg = P.configs.workload(args.workload, args.paths)
    kernel_name, profile_json = KERNELS[args.workload]
    n, nmat, nout = cfg.paths, cfg.nmat, cfg.nout
    stream = torch.cuda.current_stream(dev)

    dz = torch.empty(n * nmat, dtype=torch.float32, device=dev)
    P.normals_f32_device(20260603, n, nmat, dz.data_ptr(), stream=stream.cuda_stream,
                         path0=rank_path0(rank, n))
    out = torch.zeros(nout, dtype=torch.float64, device=dev)
    se = torch.zeros(nout, dtype=torch.float64, device=dev)
    eng = P.Engine(cfg, device=local)
    eng.set_stream(stream.cuda_stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    # ---- device-resident throughput -------------------------------------
    for _ in range(args.warmup):
        eng.greeks_f32_device(dz.data_ptr(), n, out.data_ptr(), se.data_ptr())
    eng.set_timing(True)
    kern_ms = []
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            eng.greeks_f32_device(dz.data_ptr(), n, out.data_ptr(), se.data_ptr())
            kern_ms.append(eng.kernel_time()[0]) if args.kernel_times else None
        ev1.record(stream)
        barrier()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    launches = args.steps * eng.last_launches
    # main-kernel duration: time it on separate, event-bracketed calls
    if not kern_ms:
        for _ in range(min(args.steps, 20)):
            eng.greeks_f32_device(dz.data_ptr(), n, out.data_ptr(), se.data_ptr())
            kern_ms.append(eng.kernel_time()[0])
    eng.set_timing(False)
    res32 = out.cpu().numpy().copy()
    se32 = se.cpu().numpy().copy()

    t_max = max_over_ranks(elapsed, dev)
    value = whole_job_rate(n, args.steps, ws, t_max)

    # ---- end to end through the host C-ABI call, pinned host normals -----
    hz = torch.empty(n * nmat, dtype=torch.float32, pin_memory=True)
    hz.copy_(dz)
    hz_np = hz.numpy()
    for _ in range(max(1, args.warmup)):
        eng.greeks_f32(hz_np, n)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.greeks_f32(hz_np, n)
    e2e_dt = max_over_ranks(time.perf_counter() - t0, dev)
    e2e = whole_job_rate(n, args.steps, ws, e2e_dt)
    e2e_launches = eng.last_launches

    # ---- accuracy: FP64 GPU kernel on the identical normals --------------
    acc = None
    if rank == 0 and not args.skip_accuracy:
        dz64 = dz.double()
        o64 = torch.zeros(nout, dtype=torch.float64, device=dev)
        eng.greeks_f64_device(dz64.data_ptr(), n, o64.data_ptr())
        eng.synchronize()
        r64 = o64.cpu().numpy()
        del dz64
        err = []
        for sl in (slice(0, 1), slice(1, 1 + cfg.nn), slice(1 + cfg.nn, nout)):
            floor = 1e-2 * np.abs(r64[sl]).max() if r64[sl].size > 1 else 0.0
            den = np.maximum(np.abs(r64[sl]), floor)
            den = np.where(den > 0, den, 1.0)
            err.append(float(np.max(np.abs(res32[sl] - r64[sl]) / den)))
        acc = {"reference": "FP64 GPU kernel (pinned to the FP64 CPU oracle at 1e-12) on the identical normals",
               "max_rel_err_value": err[0], "max_rel_err_deltas": err[1], "max_rel_err_vegas": err[2],
               "tolerance": 1e-4, "rule": "|f32-f64| / max(|f64|, 1% of the largest of its group)",
               "max_abs_err_over_mc_se": float(np.max(np.abs(res32 - r64) / np.maximum(se32, 1e-300))),
               # per output, in output order (value, dV/dL0[0..NN-1], dV/dlambda[0..NN-1]): the
               # FP32 result's rounding error |FP32 - FP64| beside its Monte Carlo standard error
               "rounding_error": [float(f"{x:.3g}") for x in np.abs(res32 - r64)],
               "se": [float(f"{x:.3g}") for x in se32]}
        # FP64 central differences (h = 1e-6, common random numbers) on the
        # first CENTRAL_FD_PATHS paths, against the FP32 adjoint on those paths
        nf = min(n, CENTRAL_FD_PATHS)
        dzf = dz[: nf * nmat]
        dzf64 = dzf.double()
        fd = torch.zeros(nout, dtype=torch.float64, device=dev)
        a32 = torch.zeros(nout, dtype=torch.float64, device=dev)
        eng.bump_greeks_f64_device(dzf64.data_ptr(), nf, 1e-6, fd.data_ptr(), central=True)
        eng.greeks_f32_device(dzf.data_ptr(), nf, a32.data_ptr())
        eng.synchronize()
        fd, a32 = fd.cpu().numpy(), a32.cpu().numpy()
        del dzf64
        errf = []
        for sl in (slice(1, 1 + cfg.nn), slice(1 + cfg.nn, nout)):
            den = np.maximum(np.abs(fd[sl]), 1e-2 * np.abs(fd[sl]).max())
            errf.append(float(np.max(np.abs(a32[sl] - fd[sl]) / np.where(den > 0, den, 1.0))))
        acc["central_fd"] = {"paths": nf, "h": 1e-6, "max_rel_err_deltas": errf[0], "max_rel_err_vegas": errf[1],
                             "method": "FP64 (V(+h) - V(-h)) / 2h, 1+4NN forward runs on the identical normals"}

    # ---- phase split: forward (+payoff, tape write) and backward (tape read,
    # payoff adjoint, reverse sweep) as separate calls of the C-ABI pair --------
    phases = None
    if rank == 0 and not args.skip_phases:
        tape = eng.tape(n)
        val = torch.zeros(1, dtype=torch.float64, device=dev)
        grad = torch.zeros(2 * cfg.nn, dtype=torch.float64, device=dev)

        def med_ms(f, k=5):
            for _ in range(2):
                f()
            eng.set_timing(True)
            ts = []
            for _ in range(k):
                f()
                ts.append(eng.kernel_time()[0])
            eng.set_timing(False)
            return statistics.median(ts)

        fw = med_ms(lambda: eng.forward_f32_device(dz.data_ptr(), n, tape, val.data_ptr()))
        bw = med_ms(lambda: eng.backward_f32_device(dz.data_ptr(), tape, [1.0], grad.data_ptr()))
        tape.close()
        long_tenor = cfg.nn == 160
        phases = {"forward_ms": fw, "backward_ms": bw, "fused_ms": statistics.median(kern_ms),
                  "tape_bytes": 4 * (cfg.nn + (2 if long_tenor else 1) * nmat) * n,
                  "note": "forward = Euler steps + payoff + tape write (terminal rates, per-step drift "
                          "sums" + (", and the drift sums at rate 79" if long_tenor else "") +
                          "); backward = tape read + payoff adjoint + reverse sweep (the pair runs " +
                          ("the two-thread k_tp2 kernels; the fused call runs k_tpq, one thread per path "
                           "in 40-rate blocks with a per-block scratch" if long_tenor else
                           "the one-pass k_tpp kernels; the fused call keeps its state on chip, the "
                           "idle rate half in an L2 scratch") + ")"}

    # ---- the MRG32k3a/AS241 normal stream (the reference's generator family):
    # the workload's normals generated on the device vs the oracle on one core
    rng = None
    if rank == 0 and not args.skip_rng:
        from oracle import oracle as O
        cnt = n * nmat
        zr = torch.empty(cnt, dtype=torch.float64, device=dev)
        rates = {}
        for kind, buf in (("f32", dz), ("f64", zr)):
            fn = P.mrg32k3a_normals_f32_device if kind == "f32" else P.mrg32k3a_normals_f64_device
            fn(12345, 0, cnt, buf.data_ptr(), stream=stream.cuda_stream)
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            for _ in range(3):
                fn(12345, 0, cnt, buf.data_ptr(), stream=stream.cuda_stream)
            g1.record(stream)
            torch.cuda.synchronize(dev)
            ms = g0.elapsed_time(g1) / 3
            rates[kind] = {"normals_per_s": cnt / (ms * 1e-3), "ms": ms,
                           "output_gbs": cnt * buf.element_size() / (ms * 1e-3) / 1e9}
        del zr
        ns = 2_000_000
        t0 = time.perf_counter()
        O.mrg32k3a_normals_f64(12345, 0, ns)
        cpu_rate = ns / (time.perf_counter() - t0)
        rng = {"count": cnt, "device": rates, "cpu_oracle_normals_per_s_1core": cpu_rate,
               "note": "MRG32k3a (L'Ecuyer 1999) with skip-ahead, AS241 inversion (PPND16 FP64, PPND7 FP32); "
                       "FP64 output computed in FP64 (GB300 FP64 rate), FP32 output by PPND7 in FP32"}
        # restore the bench's Philox normals in dz (overwritten above)
        P.normals_f32_device(20260603, n, nmat, dz.data_ptr(), stream=stream.cuda_stream,
                             path0=rank_path0(rank, n))
        torch.cuda.synchronize(dev)

    # ---- per-swaption breakdown (value + all Greeks of each swaption alone) --
    breakdown = None
    if rank == 0 and not args.skip_breakdown:
        nopt = len(cfg.swaprates)
        bo = torch.zeros(nopt * nout, dtype=torch.float64, device=dev)
        eng.breakdown_f32_device(dz.data_ptr(), n, bo.data_ptr())
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        eng.breakdown_f32_device(dz.data_ptr(), n, bo.data_ptr())
        b1.record(stream)
        torch.cuda.synchronize(dev)
        bms = b0.elapsed_time(b1)
        bsum = bo.view(nopt, nout).sum(0).cpu().numpy()
        scale = np.abs(res32).max()
        breakdown = {"swaptions": nopt, "ms": bms, "launches": eng.last_launches,
                     "paths_per_s_per_swaption": nopt * n / (bms * 1e-3),
                     "max_abs_diff_sum_vs_portfolio_over_scale": float(np.max(np.abs(bsum - res32)) / scale)}
        del bo

    # ---- FP64 bump-and-revalue comparator on a bounded sample -------------
    bump = None
    if rank == 0 and not args.skip_bump:
        nb = args.bump_paths
        dzb = dz[: nb * nmat].double()
        ob = torch.zeros(nout, dtype=torch.float64, device=dev)
        eng.bump_greeks_f64_device(dzb.data_ptr(), nb, 1e-6, ob.data_ptr())
        eng.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        eng.bump_greeks_f64_device(dzb.data_ptr(), nb, 1e-6, ob.data_ptr())
        s1.record(stream)
        torch.cuda.synchronize(dev)
        bt = s0.elapsed_time(s1) / 1e3
        f64_peak = P.fp64_peak_tflops(local, 200.0)
        bump_ops = (OPS_FWD_CELL * cells(cfg.nn, nmat) + OPS_PORTFOLIO) * (1 + 2 * cfg.nn) * nb
        bump = {"paths_per_s": nb / bt, "sample_paths": nb, "forward_runs": 1 + 2 * cfg.nn,
                "roofline": {"bound": "fp64", "achieved": bump_ops / bt / 1e12, "peak": f64_peak,
                             "unit": "TFLOP/s", "frac": bump_ops / bt / 1e12 / f64_peak,
                             "ops_per_forward_run": OPS_FWD_CELL * cells(cfg.nn, nmat) + OPS_PORTFOLIO,
                             "peak_source": "measured live: DFMA-chain kernel lmm_fp64_peak_tflops"},
                "seconds": bt, "method": "FP64 forward re-run per bumped input (one-sided, h=1e-6)",
                "fp32_adjoint_speedup": value / ws / (nb / bt)}

    # ---- the other named workloads (median of three timed calls each, after warm-up) ----
    others = None
    if rank == 0 and not args.skip_others:
        others = {}
        for wl, mode in ((3, "hbm"), (4, "philox"), (5, "hbm")):
            if wl == args.workload:
                continue
            c = P.configs.workload(wl)
            with P.Engine(c, device=local) as ew:
                ew.set_stream(stream.cuda_stream)
                o = torch.zeros(c.nscen * c.nout, dtype=torch.float64, device=dev)
                zw = None
                if mode == "hbm":
                    zw = torch.empty(c.paths * c.nmat, dtype=torch.float32, device=dev)
                    P.normals_f32_device(wl, c.paths, c.nmat, zw.data_ptr(), stream=stream.cuda_stream)
                run = (lambda: ew.greeks_f32_device(zw.data_ptr(), c.paths, o.data_ptr())) if mode == "hbm" \
                    else (lambda: ew.greeks_philox_device(wl, c.paths, o.data_ptr()))
                run()
                ew.set_timing(True)
                kt = []
                for _ in range(3):
                    run()
                    kt.append(ew.kernel_time()[1])
                kms = sorted(kt)[1]
                others[c.name] = {"paths_per_s": c.nscen * c.paths / (kms * 1e-3), "ms": kms,
                                  "nn": c.nn, "nmat": c.nmat, "scenarios": c.nscen, "normals": mode,
                                  "kernel": "k_tps (thread per path, reverse split over the rate halves)" if c.nn == 80 else
                                  "k_tpq (thread per path; reverse in passes over blocks of 40 rates, rebuilt "
                                  "from each block's top drift sums, rates saved every 8 steps)"}
                del zw

    # ---- roofline -----------------------------------------------------------
    roof = None
    if rank == 0:
        kms = statistics.median(kern_ms)
        ops = (OPS_PER_CELL * cells(cfg.nn, nmat) + OPS_PORTFOLIO) * n
        peak = P.fp32_peak_tflops(local, 300.0)
        traffic = None
        if os.path.exists(profile_json):
            with open(profile_json) as f:
                prof = json.load(f)
            if prof.get("scaled_to_paths") == n:
                traffic = prof.get("dram_bytes_per_launch")
        achieved = ops / (kms * 1e-3) / 1e12
        roof = {"bound": "fp32", "kernel": kernel_name, "achieved": achieved,
                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                "peak_source": "measured live: FFMA-chain kernel lmm_fp32_peak_tflops (MEASURED_PEAKS.json "
                               "has no FP32 SIMT figure)",
                "ops_per_path": OPS_PER_CELL * cells(cfg.nn, nmat) + OPS_PORTFOLIO,
                "kernel_ms": kms, "algorithmic_bytes_per_launch": 4 * nmat * n,
                "hbm_gbs_algorithmic": 4 * nmat * n / (kms * 1e-3) / 1e9}
        mufu = P.mufu_peak_gops(local, 100.0)
        mufu_ops = (MUFU_PER_CELL * cells(cfg.nn, nmat) + 2 * cfg.nn) * n
        mach = mufu_ops / (kms * 1e-3) / 1e9
        hbm_peak, hbm_src = 6800.0, "fallback (MEASURED_PEAKS.json absent)"
        mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(mp):
            with open(mp) as f:
                hbm_peak, hbm_src = float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
        hbm_ach = (traffic if traffic else 4 * nmat * n) / (kms * 1e-3) / 1e9
        roof["hbm"] = {"achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_ach / hbm_peak,
                       "bytes": "ncu DRAM traffic per launch" if traffic else "algorithmic (normals read once)",
                       "peak_source": hbm_src,
                       "note": f"the kernel is not memory-bound: {nmat} FP32 normals per path against about "
                               f"{roof['ops_per_path'] / 1e3:.0f}k operations"}
        roof["mufu"] = {"achieved": mach, "peak": mufu["mixed"], "unit": "Gop/s", "frac": mach / mufu["mixed"],
                        "ops_per_path": MUFU_PER_CELL * cells(cfg.nn, nmat) + 2 * cfg.nn,
                        "peak_source": "measured live: lmm_mufu_peak_gops, ex2 and rcp chains alternating",
                        "peaks_gops": mufu}

    line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic: Philox4x32-10 + Box-Muller N(0,1), FP32 [{n} x {nmat}] path-major in HBM",
            "config": {"workload": cfg.name, "nn": cfg.nn, "nmat": nmat, "paths_per_step": n,
                       "greeks": 2 * cfg.nn, "normals": "HBM, read once per step",
                       "l2": f"inputs larger than L2: {4 * n * nmat / 1e6:.0f} MB of normals per step vs 129 MB L2",
                       "parallelism": f"replicas x{ws} (independent path ranges, no collective)"},
            "gpu_launches": launches,
            "e2e": {"value": e2e, "unit": "paths/s", "h2d_bytes_per_step": 4 * n * nmat,
                    "d2h_bytes_per_step": 2 * 8 * nout + 4, "launches_per_step": e2e_launches,
                    "api": "lmm_greeks_f32_host (pinned host normals)"},
            "roofline": roof, "clocks": clk.summary(), "accuracy": acc, "phase_split": phases,
            "rng_mrg32k3a": rng, "swaption_breakdown": breakdown,
            "fp64_bump_comparator": bump,
            "other_workloads": others}
    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline_port(cfg, target_s=args.cpu_seconds)
        line["cpu_baseline"].pop("seconds", None)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", type=int, default=WORKLOAD, choices=sorted(KERNELS),
                    help="the workload timed as the bench line: 2 = 80/40 at 4,194,304 paths (default), "
                         "3 = 160/120 at 1,048,576 paths with rates saved every 8 steps")
    ap.add_argument("--paths", type=int, default=None,
                    help="paths per step (default: the workload's own count); smaller only for profiling")
    ap.add_argument("--bump-paths", type=int, default=16384)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--kernel-times", action="store_true",
                    help="read the main-kernel time after every timed step (adds a host sync per step)")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--skip-bump", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-others", action="store_true")
    ap.add_argument("--skip-phases", action="store_true")
    ap.add_argument("--skip-rng", action="store_true")
    ap.add_argument("--skip-breakdown", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

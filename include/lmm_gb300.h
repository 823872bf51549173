/*
 * lmm_gb300.h -- C ABI of the GB300 (sm_103a) LIBOR Market Model
 * swaption-portfolio Monte Carlo with pathwise adjoint Greeks.
 *
 * Drop-in boundary for intel/Financial-Services-Workload-Samples,
 * LiborMarketModel: the reference exposes exactly one entry point,
 *
 *   void liborSwaptionGreeks(REAL *z, int num, REAL mean, REAL std_dev,
 *                            int seed, REAL *d_v, REAL *d_Lb, int numPaths);
 *   (LiborMarketModel/liborSwaptionGreeks.hpp:12-13, defined at
 *    liborSwaptionGreeks.cpp:241-368)
 *
 * whose compute is path_calc_b1 (:34-82), portfolio_b (:120-211) and
 * path_calc_b2 (:86-117), with the model fixed at compile time by
 * LiborMarketModel/params.h:10-40 and the curve hard-coded at :269-271.
 * lmm_swaption_greeks / lmm_swaption_greeks_f32 below keep that signature.
 * The engine API generalises it: runtime model/portfolio (params.h as a
 * struct), all NN deltas AND all NN vegas (the reference returns one delta
 * and no vega), scenario batches, device-resident inputs, and a
 * forward/backward pair.
 *
 * Conventions
 *   - Every call returns an int status (LMM_OK = 0, negative on error); no
 *     exception or abort crosses the ABI. lmm_last_error() gives detail.
 *   - Results: for each scenario s, out[s*(1+2nn) + j] with j = 0 the
 *     discounted portfolio value, j = 1+i the delta dV/dL0[i], j = 1+nn+k
 *     the vega dV/dlambda[k] (lambda indexed by time to maturity, as the
 *     reference reads lambda[i-n-1], liborSwaptionGreeks.cpp:65,102).
 *     Values are Monte Carlo means over the paths; se (may be NULL) holds
 *     their standard errors in the same layout.
 *   - Normals are path-major, z[p*nmat + n], as in the reference
 *     (liborSwaptionGreeks.cpp:56). All scenarios of an engine use the same
 *     normals (common random numbers).
 *   - *_host calls take host pointers and block until results are back.
 *     *_device calls take device pointers, are enqueued on the engine's
 *     stream and return without waiting.
 *   - One engine is not thread-safe; distinct engines are independent and may
 *     be driven from different host threads at once. The reference-signature
 *     calls share one internal engine behind a lock and may be called from
 *     any thread.
 */
#ifndef LMM_GB300_H
#define LMM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    LMM_OK = 0,
    LMM_ERR_INVALID_ARG = -1,   /* bad pointer, size or parameter value       */
    LMM_ERR_UNSUPPORTED = -2,   /* shape or option the kernels do not cover   */
    LMM_ERR_CUDA = -3,          /* a CUDA runtime call failed                 */
    LMM_ERR_NONFINITE = -4,     /* a result came out NaN or Inf               */
    LMM_ERR_NO_DEVICE = -5,     /* no usable CUDA device                      */
    LMM_ERR_TOO_LARGE = -6,     /* size beyond a documented limit             */
    LMM_ERR_OUT_OF_MEMORY = -7  /* device allocation failed                   */
};

/* Limits. */
#define LMM_MAX_NN 256          /* forward rates                               */
#define LMM_MAX_NOPT 64         /* swaptions per portfolio                     */
#define LMM_MAX_SCEN 65536      /* initial curves per engine                   */

/* The model and portfolio: LiborMarketModel/params.h:27-40 as runtime data,
 * plus the curve and vols that liborSwaptionGreeks.cpp:269-271 hard-codes. */
typedef struct lmm_params {
    int32_t nn;                 /* NN, number of forward rates (params.h:27)      */
    int32_t nmat;               /* NMAT, time steps = normals per path (:28)      */
    int32_t nopt;               /* NOPT, swaptions (:30)                          */
    int32_t nscen;              /* initial curves; 1 for a single valuation       */
    double delta;               /* DELTA, accrual fraction (:33); sqrt(delta)
                                   replaces SQRT_DELTA (:34)                      */
    const double *L0;           /* [nscen][nn] initial forward curves (:271)      */
    const double *lambda;       /* [nn] vol by time to maturity (:270)            */
    const int32_t *maturities;  /* [nopt] swap length in periods, 1..nn-nmat (:38) */
    const double *swaprates;    /* [nopt] strikes (:39-40)                        */
} lmm_params;

typedef struct lmm_engine lmm_engine;
typedef struct lmm_tape lmm_tape;

/* ---- housekeeping ---------------------------------------------------- */

/* Checks a parameter set on the host only (no GPU needed). */
int lmm_validate_params(const lmm_params *p);
/* Number of doubles per scenario in a result: 1 + 2*nn. */
int64_t lmm_num_outputs(const lmm_params *p);
const char *lmm_status_string(int status);
/* Detail of the last failure on the calling thread ("" if none). */
const char *lmm_last_error(void);
/* Library version as "major.minor.patch". */
const char *lmm_version(void);

/* Uploads the parameters to `device` and creates the engine's own stream. */
int lmm_engine_create(const lmm_params *p, int32_t device, lmm_engine **out);
int lmm_engine_destroy(lmm_engine *e);
/* Use `stream` (a cudaStream_t, NULL = legacy default stream) from now on.
 * CUDA graphs: once a device call (lmm_greeks_f32_device, lmm_greeks_philox_device,
 * lmm_greeks_f64_device, the mrg32k3a/normals generators) has run for a
 * given engine and path count, repeating it enqueues only kernels and async
 * memsets on the stream and allocates nothing, so it can be recorded by a
 * stream capture and replayed. */
int lmm_engine_set_stream(lmm_engine *e, void *stream);
/* Checkpoint interval of the FP32 reverse sweep (fused calls). Storing the
 * whole NN x NMAT trajectory per path, as the reference does (params.h:29
 * L2_SIZE, liborSwaptionGreeks.cpp:76), would not fit on chip, so the
 * reverse sweep runs each Euler step backwards from the drift sums the
 * forward saved; the long-tenor kernels also save the rates every `steps`
 * steps and restore them in the reverse, so that FP32 rounding of the
 * backward steps accumulates over at most `steps` steps. 0: no rate
 * checkpoints. The default is 8 for every shape but nn = 80, nmat = 40,
 * whose kernel keeps all its drift sums on chip and takes no rate
 * checkpoints (only 0 is accepted there: LMM_ERR_UNSUPPORTED otherwise).
 * nn = 160, nmat = 120 restores the checkpoints between groups of four
 * reverse steps and needs a multiple of 4 (LMM_ERR_UNSUPPORTED otherwise;
 * its forward/backward pair runs steps in pairs, which any such interval
 * suits); steps outside [0, nmat] is
 * LMM_ERR_INVALID_ARG. Applies to later calls; a smaller interval may grow
 * the engine's device scratch on the next call. */
int lmm_engine_set_checkpoint_interval(lmm_engine *e, int32_t steps);
/* The current interval (-1 for a NULL engine). */
int32_t lmm_engine_checkpoint_interval(const lmm_engine *e);
/* Blocks until all work enqueued on the engine's stream is done. */
int lmm_engine_synchronize(lmm_engine *e);
/* Launches enqueued by the last compute call (kernels only). */
int32_t lmm_engine_last_launches(const lmm_engine *e);
/* Tracing: with timing on, every compute call brackets its main kernel and
 * its whole launch sequence with CUDA events on the engine's stream;
 * lmm_engine_kernel_time waits for the last call and returns both, in ms
 * (the reference's phase timers, liborSwaptionGreeks.cpp:250-366). */
int lmm_engine_set_timing(lmm_engine *e, int32_t enable);
int lmm_engine_kernel_time(lmm_engine *e, double *main_kernel_ms, double *total_ms);

/* Roofline calibration: sustained FP32 FMA throughput (TFLOP/s, 2 flops per
 * FMA) of `device`, from a register-resident FMA-chain kernel timed with CUDA
 * events over about `ms` milliseconds. */
int lmm_fp32_peak_tflops(int32_t device, double ms, double *tflops);
/* The same for FP64 FMA (DFMA chains): the roofline of the FP64 kernels. */
int lmm_fp64_peak_tflops(int32_t device, double ms, double *tflops);
/* Measured special-function (MUFU) throughput on `device`, in 10^9 operations
 * per second, for ex2.approx, rcp.approx and the two alternating (the mix the
 * LMM cells issue: one exp and one reciprocal per cell), each from an
 * independent-chain kernel run for about `ms` milliseconds. Any output may
 * be NULL. The roofline of the FP32 kernels against the MUFU pipe. */
int lmm_mufu_peak_gops(int32_t device, double ms, double *ex2_gops, double *rcp_gops,
                       double *mixed_gops);

/* ---- value + all Greeks, FP32 adjoint (the fast path) ----------------- */
/* Replaces the per-path work of liborSwaptionGreeks.cpp:281-344 (forward,
 * payoff adjoint, reverse sweep) plus the vega adjoint, for every path, with
 * FP64 cross-path sums. Oracle mode: normals read from memory. The host call
 * overlaps the host->device copy of z with the computation (z in pinned
 * memory gets the full copy bandwidth). */
int lmm_greeks_f32_host(lmm_engine *e, const float *z, int64_t paths, double *out, double *se);
int lmm_greeks_f32_device(lmm_engine *e, const float *d_z, int64_t paths, double *d_out,
                          double *d_se);
/* Throughput mode: normals generated in-kernel by Philox4x32-10, counter
 * {n/4, 0, lo32(path0+p), hi32(path0+p)}, key {lo32(seed), hi32(seed)}. */
int lmm_greeks_philox_host(lmm_engine *e, uint64_t seed, int64_t path0, int64_t paths,
                           double *out, double *se);
int lmm_greeks_philox_device(lmm_engine *e, uint64_t seed, int64_t path0, int64_t paths,
                             double *d_out, double *d_se);

/* ---- forward/backward pair (same arithmetic as the fused call) ------- */
/* The forward/backward split of the fused FP32 call at the payoff, for use as
 * an autograd node. For nn = 80, nmat = 40 the tape holds, per path, the
 * inverse terminal rates 1/L and the per-step drift sums the reverse sweep
 * restarts from: (nn + nmat) floats. For nn = 160, nmat = 120 (two threads
 * per path) it also holds the per-step drift sums at rate nn/2 - 1:
 * (nn + 2 nmat) floats. For the other shapes (warp-per-path kernels) the
 * backward recomputes the forward from the same normals d_z, and the tape
 * holds no device memory. */
int lmm_tape_create(lmm_engine *e, int64_t paths, lmm_tape **out);
int lmm_tape_destroy(lmm_tape *t);
/* Forward: value per scenario (d_value[nscen], d_value_se[nscen] or NULL). */
int lmm_forward_f32_device(lmm_engine *e, const float *d_z, int64_t paths, lmm_tape *t,
                           double *d_value, double *d_value_se);
/* Backward: value_bar[nscen] (host) is the upstream gradient of each value;
 * d_grad[s*2nn + i] = value_bar[s] * dV_s/dL0[i], d_grad[s*2nn + nn + k] =
 * value_bar[s] * dV_s/dlambda[k]. d_grad_se (or NULL): their standard errors. */
int lmm_backward_f32_device(lmm_engine *e, const float *d_z, const lmm_tape *t,
                            const double *value_bar, double *d_grad, double *d_grad_se);

/* ---- FP64 paths (oracle mode and the bump-and-revalue comparator) ---- */
/* Same outputs as lmm_greeks_f32_*, computed in FP64 end to end. */
int lmm_greeks_f64_host(lmm_engine *e, const double *z, int64_t paths, double *out, double *se);
int lmm_greeks_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double *d_out,
                          double *d_se);
/* The FP32 results of lmm_greeks_f32_device (d_out, d_se) and, per output,
 * their rounding error d_err = |FP32 result - FP64 result| on the identical
 * normals (the FP64 kernel run on d_z widened to FP64), so that each
 * result's arithmetic error is reported apart from its Monte Carlo standard
 * error d_se. d_err has the layout of d_out. Costs one FP64 run and
 * paths * nmat * 8 bytes of engine scratch. The reference reports its value
 * and one delta (main.cpp:91-92) with neither. */
int lmm_greeks_f32_rounding_device(lmm_engine *e, const float *d_z, int64_t paths, double *d_out,
                                   double *d_se, double *d_err);
/* FP64 forward only, re-run with bumped inputs: one-sided differences
 * (V(theta + h e_j) - V(theta)) / h for the nn L0[i] and the nn lambda[k];
 * out/se layout as above (se is the standard error of the value only; the
 * Greek entries of se are 0). This is the plain bump-and-revalue method. */
int lmm_bump_greeks_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double h,
                               double *d_out, double *d_se);
int lmm_bump_greeks_f64_host(lmm_engine *e, const double *z, int64_t paths, double h,
                             double *out, double *se);
/* FP64 central differences under common random numbers:
 * (V(theta + h e_j) - V(theta - h e_j)) / 2h for the nn L0[i] and the nn
 * lambda[k], all 1 + 4nn forward runs on the same normals; out/se layout and
 * se convention as lmm_bump_greeks_f64_*. This is the finite-difference
 * check of the FP32 adjoint (bump 1e-6 in the headline workload); the
 * reference's own sensitivities come from its adjoint
 * (liborSwaptionGreeks.cpp:86-117), which this cross-checks. */
int lmm_bump_greeks_central_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double h,
                                       double *d_out, double *d_se);
int lmm_bump_greeks_central_f64_host(lmm_engine *e, const double *z, int64_t paths, double h,
                                     double *out, double *se);

/* ---- portfolio weights and per-swaption breakdown ----------------------- */
/* The reference prices a fixed portfolio: every swaption with notional 100
 * (portfolio_b, liborSwaptionGreeks.cpp:159-171). weights[o] (one per
 * swaption, in the order of lmm_params.swaprates) scales swaption o's payoff
 * in every later call of the engine -- value and all Greeks, FP32 and FP64,
 * the forward/backward pair and the bump comparator; NULL restores all 1.
 * Weights must be finite (0 and negative values are allowed: a short
 * position). Waits for the engine's earlier work. */
int lmm_engine_set_weights(lmm_engine *e, const double *weights);
/* Per-swaption breakdown: for each swaption o, the value and all 2*nn Greeks
 * of that swaption alone at unit weight (times the reference's 100), as one
 * fused call each. d_out/d_se: [nopt][nscen][1+2*nn] (swaption-major; d_se
 * may be NULL). Summing over o gives the unit-weight portfolio. */
int lmm_swaption_breakdown_f32_device(lmm_engine *e, const float *d_z, int64_t paths,
                                      double *d_out, double *d_se);
int lmm_swaption_breakdown_f64_device(lmm_engine *e, const double *d_z, int64_t paths,
                                      double *d_out, double *d_se);

/* ---- normals ---------------------------------------------------------- */
/* z[p*nmat+n] for paths path0..path0+paths-1, the same numbers the Philox
 * mode consumes in-kernel (FP32 spec). Enqueued on `stream`. */
int lmm_normals_f32_device(uint64_t seed, int64_t path0, int64_t paths, int32_t nmat,
                           float *d_z, void *stream);
/* FP64 spec: 32-bit uniforms, FP64 Box-Muller; mean + std_dev * N(0,1). */
int lmm_normals_f64_device(uint64_t seed, int64_t path0, int64_t paths, int32_t nmat,
                           double mean, double std_dev, double *d_z, void *stream);

/* ---- MRG32k3a stream (the reference's generator family) ----------------- */
/* Replaces generateRand (LiborMarketModel/mklRng.cpp:44-110), which draws
 * ONE MRG32k3a stream (vslNewStream(..., VSL_BRNG_MRG32K3A, seed), :91),
 * read sequentially into z with a skip-ahead per thread (:97) and Gaussians
 * by inversion (VSL_RNG_METHOD_GAUSSIAN_ICDF, :25/:31). These calls write
 * elements [first, first+count) of that kind of stream: MRG32k3a
 * (L'Ecuyer 1999) seeded from one 32-bit seed as x = (seed mod m1, 1, 1),
 * y = (1, 1, 1); u = z/(m1+1) with z in [1, m1]; normals by AS241 (Wichura
 * 1988): PPND16 in FP64, PPND7 in FP32; out = mean + std_dev * x. MKL's own
 * seeding, scaling and inversion are not reproduced (closed), so the numbers
 * are not MKL's. Skip-ahead is exact for any first < 2^63. Enqueued on
 * `stream` (the current device); count = 0 is a no-op. */
int lmm_mrg32k3a_uniforms_device(uint32_t seed, int64_t first, int64_t count, double *d_u,
                                 void *stream);
int lmm_mrg32k3a_normals_f64_device(uint32_t seed, int64_t first, int64_t count, double mean,
                                    double std_dev, double *d_z, void *stream);
int lmm_mrg32k3a_normals_f32_device(uint32_t seed, int64_t first, int64_t count, float mean,
                                    float std_dev, float *d_z, void *stream);

/* ---- no-allocation variant ---------------------------------------------- */
/* No counterpart in the reference. Some callers cannot call cudaMalloc: a
 * library embedded in a host application that owns every device allocation
 * through its own pool, a plug-in whose process has locked or exhausted its
 * allocator, a loop that must never touch the allocator. This is a fused
 * FP32 value + Greeks launch like lmm_greeks_f32_device, without an engine
 * and without any allocation (no cudaMalloc, no cudaFree, no allocating
 * library call). It runs the one-pass kernel, which needs no per-path
 * scratch; the engine's fused call runs the split-reverse kernel, and the
 * two agree within the FP32 tolerance (same cells, rounded in another
 * order). The caller passes the parameters, the device normals d_z and the
 * device outputs d_out/d_se (layout as above); everything else -- model
 * constants, per-block partial sums, the non-finite flag -- lives in one
 * static device array of LMM_NOALLOC_SCRATCH_BYTES that every GPU loading
 * the library holds until the process exits.
 *   - Limits: nn = 80, nmat = 40 (LMM_ERR_UNSUPPORTED otherwise),
 *     nscen <= LMM_NOALLOC_MAX_SCEN and paths <= 2^40 (LMM_ERR_TOO_LARGE).
 *   - Works on the current device and enqueues on `stream` without waiting:
 *     the model constants travel as a kernel parameter, so nothing of the
 *     caller's host memory is read after the call returns.
 *   - The first call on a device looks up the array's device address and the
 *     kernel's occupancy and caches them: make it before any stream capture.
 *     Later calls enqueue only kernels, so a stream capture records them and
 *     graph replays repeat the call (tested). After cudaDeviceReset the next
 *     call on that device looks them up again.
 *   - Every call shares the one array, which keeps the last call's
 *     contents: calls that overlap on the GPU (other streams, other host
 *     threads) race on it and must be serialised by the caller.
 *   - Non-finite results are not reported (there is no engine to hold the
 *     flag); check d_out. Failures set lmm_last_error() as every call does. */
#define LMM_NOALLOC_SCRATCH_BYTES (4u << 20)
#define LMM_NOALLOC_MAX_SCEN 8
int lmm_greeks_f32_device_noalloc(const lmm_params *p, const float *d_z, int64_t paths,
                                  double *d_out, double *d_se, void *stream);

/* ---- the reference's signature ---------------------------------------- */
/* Drop-in for liborSwaptionGreeks (liborSwaptionGreeks.hpp:12-13) in the
 * reference's FP64 build (REAL = double, params.h:10-16): fills z[0..num)
 * with mean + std_dev * N(0,1) from the library's generator (as the
 * reference refills z through generateRand, :261; like the reference, the
 * stream is fixed -- key 12345, the reference's default seed, mklRng.h:9 --
 * and `seed` is accepted and ignored), prices the params.h portfolio on the
 * :269-271 curve (L0 = 0.051, lambda = 0.2) in FP64 on the GPU, and writes
 * the MC mean value to *d_v and the MC mean dV/dL0[NN-1] to *d_Lb.
 * Difference: the reference repeats its whole Monte Carlo NLOOPS = 10 times
 * and divides by numPaths only (:27,:278,:355-356), so its outputs are
 * 10x these means. num must equal 40*numPaths. Uses device 0. */
int lmm_swaption_greeks(double *z, int num, double mean, double std_dev, int seed,
                        double *d_v, double *d_Lb, int numPaths);
/* The same for the reference's FP32 build (REAL = float, params.h:17-24),
 * computed with the FP32 adjoint kernels. */
int lmm_swaption_greeks_f32(float *z, int num, float mean, float std_dev, int seed,
                            float *d_v, float *d_Lb, int numPaths);
/* The same two calls with z drawn from the MRG32k3a stream above (seed
 * 12345, elements 0..num-1), the reference's generator family and stream
 * order, instead of the library's Philox stream. */
int lmm_swaption_greeks_mrg32k3a(double *z, int num, double mean, double std_dev, int seed,
                                 double *d_v, double *d_Lb, int numPaths);
int lmm_swaption_greeks_mrg32k3a_f32(float *z, int num, float mean, float std_dev, int seed,
                                     float *d_v, float *d_Lb, int numPaths);

#ifdef __cplusplus
}
#endif

#endif /* LMM_GB300_H */

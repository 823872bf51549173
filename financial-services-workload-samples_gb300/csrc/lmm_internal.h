// Internal interface between the C-ABI host layer (lmm_capi.cpp) and the
// CUDA translation units. Plain C++ types only; no device code.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lmm {

constexpr int kMaxNN = 256;
constexpr int kMaxNopt = 64;

// Per-engine model data resident in HBM, passed to kernels by value.
// Per time-to-maturity k (the reference's lambda[i-n-1] index):
//   kc[k] = { lambda_k*log2(e), -delta*lambda_k^2*log2(e)/2, delta^2*lambda_k, lambda_k }
// so that one Euler cell (liborSwaptionGreeks.cpp:68-73) is
//   t = L/(1+delta L); V += kc.z*t; L *= 2^(kc.x*(V + sqrt(delta) z) + kc.y)
// with V = delta * (the reference's running sum v).
struct DevModel {
    int nn, nmat, nopt, nscen;
    float delta, sqd, d2;                 // delta, sqrt(delta), delta^2
    double deltad, sqdd;
    const float4 *kc;                     // [nn]
    const float4 *kc_host;                // [nn] the same constants in host memory, for
                                          // launches that pass them as kernel parameters
    const float *L0f;                     // [nscen][nn]
    const float *invL0f;                  // [nscen][nn]
    const double *L0d;                    // [nscen][nn]
    const double *lamd;                   // [nn]
    const int *opt_start;                 // [nn-nmat+1] options grouped by maturity-1 (CSR)
    const float *optKf;                   // [nopt] strikes in that grouped order
    const double *optKd;                  // [nopt]
    const float *optWf;                   // [nopt] notional weights in that grouped order
    const double *optWd;                  // [nopt] (the reference's portfolio: all 1)
    int ckpt;                             // steps between the rate checkpoints the
                                          // FP32 reverse sweeps restore (0: none)
};

// Path partition of one launch: grid = nscen * items blocks; block b takes
// scenario b / items and the path range [item*ipaths, (item+1)*ipaths) of it.
struct Work {
    int64_t paths;        // per scenario
    int items;            // items per scenario
    int ppt;              // paths per thread per item
    double *partial;      // [nscen*items][2*nout]: per-item sums and sums of squares
    int nout;             // outputs per scenario reduced by this launch
    int grid = 0;         // FP32 kernels: blocks launched (0: one per unit); block b
                          // runs units b, b+grid, ... of the nscen*items units
};

enum class Mode : int { Fused = 0, Forward = 1, Backward = 2 };

// The calling thread's lmm_last_error() detail (lmm_capi.cpp): sets it and
// returns `status`; the CUDA form maps the error to its LMM status.
int record_error(int status, const char *what);
int record_cuda_error(cudaError_t e, const char *what);

// FP32 thread-per-path kernels (lmm_f32_tpp.cu, NN=80, NMAT=40).
bool f32_tpp_supports(int nn, int nmat);
int tpp_block_threads(Mode mode);     // threads per block = paths per batch
cudaError_t tpp_blocks_per_sm(Mode mode, bool philox, int *blocks);
cudaError_t launch_tpp_any(const DevModel &m, Mode mode, const float *z, uint64_t seed,
                           int64_t path0, bool philox, const Work &w, float *tape,
                           const double *vbar, cudaStream_t s);
// The fused 80/40 kernel with the reverse sweep split over the rate halves
// (lmm_f32_tpp.cu, k_tps): 12 warps per SM, a per-block scratch of
// tps_scratch_floats_per_block floats.
int tps_block_threads();
size_t tps_scratch_floats_per_block(int nn, int nmat);
cudaError_t tps_blocks_per_sm(bool philox, int *blocks);
cudaError_t launch_tps_any(const DevModel &m, const float *z, uint64_t seed, int64_t path0, bool philox,
                           const Work &w, float *scratch, cudaStream_t s);
// The fused 160/120 kernel with one thread per path and the reverse in passes
// over blocks of 40 rates (lmm_f32_tpp.cu, k_tpq): a per-block scratch of
// tpq_scratch_floats_per_block floats; checkpoint intervals multiples of 4.
bool f32_tpq_supports(int nn, int nmat);
int tpq_block_threads();
size_t tpq_scratch_floats_per_block(int nn, int nmat, int ckpt);
cudaError_t tpq_blocks_per_sm(bool philox, int *blocks);
cudaError_t launch_tpq_any(const DevModel &m, const float *z, uint64_t seed, int64_t path0, bool philox,
                           const Work &w, float *scratch, cudaStream_t s);
// FP32 kernels with two threads per path (lmm_f32_tp2.cu): nn=160, nmat=120.
// The forward/backward pair's tape: [nn][total] terminal inverse rates,
// [nmat][total] full drift sums, [nmat][total] drift sums at rate nn/2 - 1.
bool f32_tp2_supports(int nn, int nmat);
int tp2_paths_per_block(int nn);
// Scratch of the fused kernel per block (floats): the drift sums at the top
// rate of every rate block but the last, per step, and the rate checkpoints,
// one every ckpt steps (ckpt even; 0: none).
size_t tp2_scratch_floats_per_block(int nn, int nmat, int ckpt);
cudaError_t tp2_blocks_per_sm(int nn, int nmat, Mode mode, bool philox, int *blocks);
cudaError_t launch_tp2_any(const DevModel &m, Mode mode, const float *z, uint64_t seed, int64_t path0,
                           bool philox, const Work &w, float *tape, const double *vbar, cudaStream_t s);
// FP32 warp-per-path kernels (lmm_f32_wpp.cu, any NN <= kMaxNN; the reverse
// sweep rebuilds each step from the forward's per-lane drift sums and takes
// the saved rates every DevModel::ckpt steps).
bool f32_wpp_supports(int nn, int nmat);
int wpp_block_threads();
cudaError_t wpp_blocks_per_sm(int nn, int nmat, Mode mode, bool philox, int *blocks);
// Device scratch the warp-per-path kernels take per warp (floats): the
// forward's per-step drift sums at each lane's top rate, and rate checkpoints
// every ckpt steps (0: none).
size_t wpp_scratch_floats_per_warp(int nn, int nmat, int ckpt);
int wpp_slots(int nn);
cudaError_t launch_wpp_any(const DevModel &m, Mode mode, const float *z, uint64_t seed,
                           int64_t path0, bool philox, const Work &w, float *tape,
                           const double *vbar, cudaStream_t s);

// FP64 kernels: thread per path, runtime shape.
int f64_block_threads();
cudaError_t f64_blocks_per_sm(bool bump, int *blocks);
cudaError_t launch_f64_greeks(const DevModel &m, const double *z, const Work &w, cudaStream_t s);
// Bumped forward re-runs: 1 + 2nn variants per scenario (1 + 4nn with
// `central`: each input bumped by +h and by -h); the launch's virtual
// scenarios are (scenario, variant) and each reduces one output, the
// variant's value (w.nout = 1).
cudaError_t launch_f64_bump(const DevModel &m, const double *z, double h, bool central, const Work &w,
                            cudaStream_t s);

// Sums the per-item partials of each scenario in a fixed order and writes
// mean and standard error; sets *flag if a result is not finite.
cudaError_t launch_finalize(const double *partial, int nscen, int items, int nout, int64_t paths,
                            double *mean, double *se, int *flag, cudaStream_t s);
// Turns bumped means into one-sided differences in place: out[j] =
// (out[j]-out[0])/h for j >= 1, per scenario.
cudaError_t launch_bump_diff(double *mean, double *se, int nscen, int nout, double h,
                             cudaStream_t s);
// Central differences (V(+h) - V(-h)) / 2h from the 1+4nn variant means per
// scenario [nscen][1+4nn] into out/se [nscen][1+2nn].
cudaError_t launch_bump_central(const double *mean, const double *se_in, double *out, double *se, int nscen,
                                int nn, double h, cudaStream_t s);
// z64 = (double)z32, element by element (n elements).
cudaError_t launch_widen(const float *z32, double *z64, int64_t n, cudaStream_t s);
// err = |a - b|, element by element (n elements).
cudaError_t launch_abs_diff(const double *a, const double *b, double *err, int n, cudaStream_t s);

// FFMA throughput probe: `blocks` x 256 threads, `iters` iterations of 16
// independent FMA chains each; one float per thread to `sink`.
cudaError_t launch_ffma_peak(int blocks, int iters, float a, float b, float *sink, cudaStream_t s);
cudaError_t launch_dfma_peak(int blocks, int iters, double a, double b, float *sink, cudaStream_t s);
// kind 0: ex2.approx, 1: rcp.approx, 2: both alternately; 16 per thread per iteration
cudaError_t launch_mufu_peak(int kind, int blocks, int iters, float *sink, cudaStream_t s);

// MRG32k3a jump tables (lmm_mrg.cu): A1^(2^k), A2^(2^k) for k < 64 and the
// per-lane offsets A1^(l*span), A2^(l*span) for l < 32, entries mod m1/m2.
struct MrgTables {
    uint32_t p1[64][9], p2[64][9], l1[32][9], l2[32][9];
};
// kind 0: uniforms (double), 1: normals (double, PPND16), 2: normals (float, PPND7)
cudaError_t launch_mrg32k3a(int kind, uint32_t seed, int64_t first, int64_t count, double mean, double sd,
                            void *out, cudaStream_t s);
cudaError_t launch_normals_f32(uint64_t seed, int64_t path0, int64_t paths, int nmat, float mean,
                               float sd, float *z, cudaStream_t s);
cudaError_t launch_normals_f64(uint64_t seed, int64_t path0, int64_t paths, int nmat, double mean,
                               double sd, double *z, cudaStream_t s);

}  // namespace lmm

// C-ABI host layer of the GB300 LMM engine (declared in include/lmm_gb300.h).
//
// Owns parameter validation, the device-resident model (params.h as data),
// the engine stream, scratch buffers, the path partition of each launch, and
// the two entry points with the reference's signature
// (LiborMarketModel/liborSwaptionGreeks.hpp:12-13). No CPU fallback exists:
// every compute call runs the CUDA kernels or returns an error.
#include "lmm_gb300.h"
#include "lmm_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

using lmm::DevModel;
using lmm::Mode;
using lmm::Work;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return LMM_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return LMM_ERR_NO_DEVICE;
    return LMM_ERR_CUDA;
}

}  // namespace

namespace lmm {
int record_error(int status, const char *what) { return fail(status, what); }
int record_cuda_error(cudaError_t e, const char *what) { return cuda_fail(e, what); }
}  // namespace lmm

namespace {

#define LMM_CK(call)                                         \
    do {                                                     \
        cudaError_t lmm_e_ = (call);                         \
        if (lmm_e_ != cudaSuccess) return cuda_fail(lmm_e_, #call); \
    } while (0)

#define LMM_TRY(call)                    \
    do {                                 \
        int lmm_rc_ = (call);            \
        if (lmm_rc_ != LMM_OK) return lmm_rc_; \
    } while (0)

// Growable device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    int ensure(size_t n)
    {
        if (n <= bytes) return LMM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return cuda_fail(e, "cudaMalloc");
        }
        bytes = n;
        return LMM_OK;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const { return static_cast<T *>(p); }
};

constexpr int64_t kMaxPaths = int64_t(1) << 40;
// Steps between the rate checkpoints of the long-tenor FP32 reverse sweeps
// when the caller sets none (the 160/120 workload's interval).
constexpr int kDefaultCkpt = 8;

}  // namespace

struct lmm_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int nn = 0, nmat = 0, nopt = 0, nscen = 0;
    double delta = 0.0;
    int sms = 0;
    DevModel dm{};
    DevBuf model;                  // all model arrays
    std::vector<int> opt_slot;     // opt_slot[o]: grouped position of swaption o
    float *wf_rows = nullptr;      // [1+nopt][nopt] weights: row 0 the caller's, row 1+g unit at g
    double *wd_rows = nullptr;
    DevBuf partial, z32, z64, out, se, flag, vbar;
    DevBuf wscratch;               // warp-per-path kernels: Y_top per warp, step and lane
    DevBuf bumpvar;                // central bumps: the variants' means and standard errors
    std::vector<float4> kc_host;   // the per-maturity constants, host copy
    std::map<int, int> bps;        // cached blocks per SM per kernel variant
    int32_t last_launches = 0;
    bool timing = false;
    bool timed = false;            // the last call recorded its events
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};   // begin, main kernel done, all done
    // host-call pipelining: chunked host->device copies on their own stream
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[8] = {};
    cudaEvent_t ready_ev = nullptr;
};

struct lmm_tape {
    lmm_engine *e = nullptr;
    int64_t paths = 0;
    DevBuf buf;
};

namespace {

int validate(const lmm_params *p)
{
    if (!p) return fail(LMM_ERR_INVALID_ARG, "params is NULL");
    if (p->nn < 2 || p->nn > LMM_MAX_NN)
        return fail(LMM_ERR_INVALID_ARG, "nn must be in [2, " + std::to_string(LMM_MAX_NN) + "]");
    if (p->nmat < 1 || p->nmat >= p->nn) return fail(LMM_ERR_INVALID_ARG, "nmat must be in [1, nn-1]");
    if (p->nopt < 0 || p->nopt > LMM_MAX_NOPT)
        return fail(LMM_ERR_INVALID_ARG, "nopt must be in [0, " + std::to_string(LMM_MAX_NOPT) + "]");
    if (p->nscen < 1 || p->nscen > LMM_MAX_SCEN)
        return fail(LMM_ERR_INVALID_ARG, "nscen must be in [1, " + std::to_string(LMM_MAX_SCEN) + "]");
    if (!(p->delta > 0.0) || !std::isfinite(p->delta)) return fail(LMM_ERR_INVALID_ARG, "delta must be finite and > 0");
    if (!p->L0 || !p->lambda) return fail(LMM_ERR_INVALID_ARG, "L0 and lambda are required");
    if (p->nopt > 0 && (!p->maturities || !p->swaprates))
        return fail(LMM_ERR_INVALID_ARG, "maturities and swaprates are required when nopt > 0");
    for (int64_t i = 0; i < (int64_t)p->nscen * p->nn; ++i)
        if (!(p->L0[i] > 0.0) || !std::isfinite(p->L0[i]))
            return fail(LMM_ERR_INVALID_ARG, "L0[" + std::to_string(i) + "] must be finite and > 0");
    for (int i = 0; i < p->nn; ++i)
        if (!(p->lambda[i] >= 0.0) || !std::isfinite(p->lambda[i]))
            return fail(LMM_ERR_INVALID_ARG, "lambda[" + std::to_string(i) + "] must be finite and >= 0");
    for (int o = 0; o < p->nopt; ++o) {
        if (p->maturities[o] < 1 || p->maturities[o] > p->nn - p->nmat)
            return fail(LMM_ERR_INVALID_ARG, "maturities[" + std::to_string(o) +
                                                 "] must be in [1, nn-nmat]: the swap reads rates nmat.."
                                                 "nmat+m-1 (liborSwaptionGreeks.cpp:133,161)");
        if (!std::isfinite(p->swaprates[o]))
            return fail(LMM_ERR_INVALID_ARG, "swaprates[" + std::to_string(o) + "] must be finite");
    }
    return LMM_OK;
}

int set_device(const lmm_engine *e)
{
    LMM_CK(cudaSetDevice(e->device));
    return LMM_OK;
}

void mark(lmm_engine *e, int i)
{
    if (e->timing) cudaEventRecord(e->ev[i], e->stream);
    if (i == 2) e->timed = e->timing;
}

// Kernel variant keys for the blocks-per-SM cache.
int variant_key(int family, Mode mode, bool philox) { return family * 16 + (int)mode * 2 + (philox ? 1 : 0); }

int f32_family(const lmm_engine *e)
{
    if (lmm::f32_tpp_supports(e->nn, e->nmat)) return 1;
    if (lmm::f32_wpp_supports(e->nn, e->nmat)) return 2;
    return 0;
}

// Kernel family of an FP32 call: 7 (one thread per path, the forward in two
// passes of 80 rates and the reverse in passes over blocks of 40 rates,
// k_tpq) for fused nn=160, nmat=120 calls (LMM_USE_TPQ; GB300, 1,048,576
// paths: 14.15 ms against 18.29 for the thread pair); 5 (two threads per
// path, lmm_f32_tp2.cu) for that shape's forward/backward pair (and its fused
// calls without LMM_USE_TPQ; 2.1x the warp-per-path rate); 6 (one thread per
// path with the reverse split over the rate halves, k_tps) for fused 80/40
// calls (LMM_USE_TPS); otherwise f32_family. At 80/40 the thread pair ran
// 13.4-15.5 ms against 11.7 ms for the thread-per-path kernel (4,194,304
// paths), so it does not take that shape.
#ifndef LMM_USE_TPS
#define LMM_USE_TPS 1
#endif
#ifndef LMM_USE_TPQ
#define LMM_USE_TPQ 1
#endif
int family_for(const lmm_engine *e, Mode mode)
{
    if (lmm::f32_tp2_supports(e->nn, e->nmat))
        return LMM_USE_TPQ && mode == Mode::Fused && lmm::f32_tpq_supports(e->nn, e->nmat) ? 7 : 5;
    const int f = f32_family(e);
    if (LMM_USE_TPS && f == 1 && mode == Mode::Fused) return 6;
    return f;
}

// Paths one block takes per batch.
int batch_paths(const lmm_engine *e, int fam, Mode mode)
{
    if (fam == 1) return lmm::tpp_block_threads(mode);
    if (fam == 5) return lmm::tp2_paths_per_block(e->nn);
    if (fam == 6) return lmm::tps_block_threads();
    if (fam == 7) return lmm::tpq_block_threads();
    return lmm::wpp_block_threads() / 32;
}

cudaError_t launch_f32_family(int fam, const lmm::DevModel &m, Mode mode, const float *z, uint64_t seed,
                              int64_t path0, bool philox, const Work &w, float *tape, const double *vbar,
                              cudaStream_t s)
{
    if (fam == 1) return lmm::launch_tpp_any(m, mode, z, seed, path0, philox, w, tape, vbar, s);
    if (fam == 5) return lmm::launch_tp2_any(m, mode, z, seed, path0, philox, w, tape, vbar, s);
    if (fam == 6) return lmm::launch_tps_any(m, z, seed, path0, philox, w, tape, s);
    if (fam == 7) return lmm::launch_tpq_any(m, z, seed, path0, philox, w, tape, s);
    return lmm::launch_wpp_any(m, mode, z, seed, path0, philox, w, tape, vbar, s);
}

int blocks_per_sm(lmm_engine *e, int family, Mode mode, bool philox, int *out)
{
    const int key = variant_key(family, mode, philox);
    auto it = e->bps.find(key);
    if (it != e->bps.end()) {
        *out = it->second;
        return LMM_OK;
    }
    int b = 0;
    cudaError_t err;
    if (family == 1) err = lmm::tpp_blocks_per_sm(mode, philox, &b);
    else if (family == 2) err = lmm::wpp_blocks_per_sm(e->nn, e->nmat, mode, philox, &b);
    else if (family == 5) err = lmm::tp2_blocks_per_sm(e->nn, e->nmat, mode, philox, &b);
    else if (family == 6) err = lmm::tps_blocks_per_sm(philox, &b);
    else if (family == 7) err = lmm::tpq_blocks_per_sm(philox, &b);
    else if (family == 3) err = lmm::f64_blocks_per_sm(false, &b);
    else err = lmm::f64_blocks_per_sm(true, &b);
    if (err != cudaSuccess) return cuda_fail(err, "occupancy query");
    if (b < 1) return fail(LMM_ERR_UNSUPPORTED, "kernel does not fit on this device");
    e->bps[key] = b;
    *out = b;
    return LMM_OK;
}

// Items per virtual scenario (and paths per thread) of a launch. Each block
// runs ppt batches of paths, all blocks equally long, so a launch costs
// ceil(blocks / slots) block-times, slots = SMs x resident blocks per SM.
// The plan takes the fewest waves (1..8) whose blocks fill at least 97% of
// the slots they occupy: one wave for one scenario (every block starts at
// once, no staggered tail), three waves for 256 scenarios (256 x 7 blocks
// of 608 slots) where one wave would leave a quarter-full second wave.
void plan_items(const lmm_engine *e, int64_t nvs, int64_t paths, int block, int bps, int64_t *items,
                int64_t *ppt)
{
    const int64_t cap = std::max<int64_t>(1, (int64_t)e->sms * bps);
    double best = -1.0;
    for (int w = 1; w <= 8; ++w) {
        int64_t it = std::max<int64_t>(1, w * cap / nvs);
        const int64_t p = std::max<int64_t>(1, (paths + block * it - 1) / (block * it));
        it = (paths + block * p - 1) / (block * p);
        const int64_t blocks = nvs * it;
        const double fill = (double)blocks / (double)(((blocks + cap - 1) / cap) * cap);
        if (fill > best + 1e-12) {
            best = fill;
            *items = it;
            *ppt = p;
        }
        if (fill >= 0.97) break;
    }
}

// plan_items, and sizes the partial-sum scratch.
int plan(lmm_engine *e, int64_t nvs, int64_t paths, int block, int bps, int nout, Work *w)
{
    int64_t items = 1, ppt = 1;
    plan_items(e, nvs, paths, block, bps, &items, &ppt);
    if (ppt > INT32_MAX || items > INT32_MAX || nvs * items > INT32_MAX)
        return fail(LMM_ERR_TOO_LARGE, "launch too large");
    w->paths = paths;
    w->items = (int)items;
    w->ppt = (int)ppt;
    w->nout = nout;
    // FP32 kernels: one wave of blocks, each looping over its units
    w->grid = (int)std::min<int64_t>(nvs * items, std::max<int64_t>(1, (int64_t)e->sms * bps));
    LMM_TRY(e->partial.ensure(sizeof(double) * (size_t)(nvs * items) * 2 * nout));
    w->partial = e->partial.as<double>();
    return LMM_OK;
}

int check_paths(int64_t paths)
{
    if (paths < 1) return fail(LMM_ERR_INVALID_ARG, "paths must be >= 1");
    if (paths > kMaxPaths) return fail(LMM_ERR_TOO_LARGE, "paths must be <= 2^40");
    return LMM_OK;
}

// Scratch of the warp-per-path kernels for a grid of `blocks` blocks (the
// forward's per-step drift sums at each lane's top rate, and rate checkpoints).
int wpp_scratch(lmm_engine *e, int64_t blocks, float **out)
{
    const size_t warps = (size_t)blocks * (lmm::wpp_block_threads() / 32);
    LMM_TRY(e->wscratch.ensure(sizeof(float) * warps * lmm::wpp_scratch_floats_per_warp(e->nn, e->nmat, e->dm.ckpt)));
    *out = e->wscratch.as<float>();
    return LMM_OK;
}

// Scratch of the fused split-reverse kernel (k_tps) for a grid of `blocks`
// blocks: per block the drift sums at the half boundary, the suffix sums
// handed from the upper to the lower half, the lower half's parked rates and
// the upper half's deltas.
int tps_scratch(lmm_engine *e, int64_t blocks, float **out)
{
    LMM_TRY(e->wscratch.ensure(sizeof(float) * (size_t)blocks * lmm::tps_scratch_floats_per_block(e->nn, e->nmat)));
    *out = e->wscratch.as<float>();
    return LMM_OK;
}

// Scratch of the fused long-tenor block-pass kernel (k_tpq) for a grid of
// `blocks` blocks: block-top drift sums, block-bottom suffix sums, parked
// rates and deltas, and the rate checkpoints of the engine's interval.
int tpq_scratch(lmm_engine *e, int64_t blocks, float **out)
{
    LMM_TRY(e->wscratch.ensure(sizeof(float) * (size_t)blocks *
                               lmm::tpq_scratch_floats_per_block(e->nn, e->nmat, e->dm.ckpt)));
    *out = e->wscratch.as<float>();
    return LMM_OK;
}

// Scratch of the fused thread-pair kernel for a grid of `blocks` blocks: the
// forward's drift sums at the half boundary and its rate checkpoints.
int tp2_scratch(lmm_engine *e, int64_t blocks, float **out)
{
    LMM_TRY(e->wscratch.ensure(sizeof(float) * (size_t)blocks *
                               lmm::tp2_scratch_floats_per_block(e->nn, e->nmat, e->dm.ckpt)));
    *out = e->wscratch.as<float>();
    return LMM_OK;
}

int run_f32(lmm_engine *e, Mode mode, const float *d_z, uint64_t seed, int64_t path0, bool philox,
            int64_t paths, float *tape, const double *d_vbar, double *d_mean, double *d_se)
{
    LMM_TRY(check_paths(paths));
    if (!philox && !d_z) return fail(LMM_ERR_INVALID_ARG, "normals pointer is NULL");
    if (!d_mean) return fail(LMM_ERR_INVALID_ARG, "output pointer is NULL");
    if (philox && (path0 < 0 || path0 > kMaxPaths)) return fail(LMM_ERR_INVALID_ARG, "path0 out of range");
    const int fam = family_for(e, mode);
    if (fam == 0)
        return fail(LMM_ERR_UNSUPPORTED, "no FP32 kernel for nn=" + std::to_string(e->nn) +
                                             ", nmat=" + std::to_string(e->nmat));
    if (philox && mode != Mode::Fused)
        return fail(LMM_ERR_UNSUPPORTED, "the forward/backward pair reads its normals from memory");
    LMM_TRY(set_device(e));
    int bps = 0;
    LMM_TRY(blocks_per_sm(e, fam, mode, philox, &bps));
    const int nout = mode == Mode::Fused ? 1 + 2 * e->nn : (mode == Mode::Forward ? 1 : 2 * e->nn);
    const int per_batch = batch_paths(e, fam, mode);
    Work w{};
    LMM_TRY(plan(e, e->nscen, paths, per_batch, bps, nout, &w));
    if (fam == 2) LMM_TRY(wpp_scratch(e, w.grid, &tape));
    if (fam == 5 && mode == Mode::Fused) LMM_TRY(tp2_scratch(e, w.grid, &tape));
    if (fam == 6) LMM_TRY(tps_scratch(e, w.grid, &tape));
    if (fam == 7) LMM_TRY(tpq_scratch(e, w.grid, &tape));
    LMM_TRY(e->flag.ensure(sizeof(int)));
    LMM_CK(cudaMemsetAsync(e->flag.p, 0, sizeof(int), e->stream));
    mark(e, 0);
    cudaError_t err = launch_f32_family(fam, e->dm, mode, d_z, seed, path0, philox, w, tape, d_vbar, e->stream);
    if (err != cudaSuccess) return cuda_fail(err, "FP32 LMM kernel launch");
    mark(e, 1);
    LMM_CK(lmm::launch_finalize(w.partial, e->nscen, w.items, nout, paths, d_mean, d_se,
                                e->flag.as<int>(), e->stream));
    mark(e, 2);
    e->last_launches = 2;
    return LMM_OK;
}

// Copies nscen*nout results (and the non-finite flag) back and waits.
int fetch(lmm_engine *e, int nout, double *out, double *se)
{
    const size_t n = (size_t)e->nscen * nout;
    int flag = 0;
    LMM_CK(cudaMemcpyAsync(out, e->out.p, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    if (se) LMM_CK(cudaMemcpyAsync(se, e->se.p, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    LMM_CK(cudaMemcpyAsync(&flag, e->flag.p, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    LMM_CK(cudaStreamSynchronize(e->stream));
    if (flag) return fail(LMM_ERR_NONFINITE, "a result is NaN or Inf");
    return LMM_OK;
}

int ensure_outputs(lmm_engine *e, int nout)
{
    const size_t n = sizeof(double) * (size_t)e->nscen * nout;
    LMM_TRY(e->out.ensure(n));
    LMM_TRY(e->se.ensure(n));
    return LMM_OK;
}

int run_f64(lmm_engine *e, const double *d_z, int64_t paths, double *d_mean, double *d_se)
{
    LMM_TRY(check_paths(paths));
    if (!d_z || !d_mean) return fail(LMM_ERR_INVALID_ARG, "NULL device pointer");
    LMM_TRY(set_device(e));
    int bps = 0;
    LMM_TRY(blocks_per_sm(e, 3, Mode::Fused, false, &bps));
    const int nout = 1 + 2 * e->nn;
    Work w{};
    LMM_TRY(plan(e, e->nscen, paths, lmm::f64_block_threads(), bps, nout, &w));
    LMM_TRY(e->flag.ensure(sizeof(int)));
    LMM_CK(cudaMemsetAsync(e->flag.p, 0, sizeof(int), e->stream));
    mark(e, 0);
    LMM_CK(lmm::launch_f64_greeks(e->dm, d_z, w, e->stream));
    mark(e, 1);
    LMM_CK(lmm::launch_finalize(w.partial, e->nscen, w.items, nout, paths, d_mean, d_se,
                                e->flag.as<int>(), e->stream));
    mark(e, 2);
    e->last_launches = 2;
    return LMM_OK;
}

int run_bump(lmm_engine *e, const double *d_z, int64_t paths, double h, bool central, double *d_mean,
             double *d_se)
{
    LMM_TRY(check_paths(paths));
    if (!d_z || !d_mean) return fail(LMM_ERR_INVALID_ARG, "NULL device pointer");
    if (!(h > 0.0) || !std::isfinite(h)) return fail(LMM_ERR_INVALID_ARG, "bump h must be finite and > 0");
    LMM_TRY(set_device(e));
    int bps = 0;
    LMM_TRY(blocks_per_sm(e, 4, Mode::Fused, false, &bps));
    const int nb = central ? 1 + 4 * e->nn : 1 + 2 * e->nn;
    Work w{};
    LMM_TRY(plan(e, (int64_t)e->nscen * nb, paths, lmm::f64_block_threads(), bps, 1, &w));
    LMM_TRY(e->flag.ensure(sizeof(int)));
    // central: the 1+4nn variant means (and their standard errors) go to the
    // engine's scratch and are differenced into the caller's 1+2nn outputs
    double *vmean = d_mean, *vse = d_se;
    if (central) {
        LMM_TRY(e->bumpvar.ensure(2 * sizeof(double) * (size_t)e->nscen * nb));
        vmean = e->bumpvar.as<double>();
        vse = vmean + (size_t)e->nscen * nb;
    }
    LMM_CK(cudaMemsetAsync(e->flag.p, 0, sizeof(int), e->stream));
    mark(e, 0);
    LMM_CK(lmm::launch_f64_bump(e->dm, d_z, h, central, w, e->stream));
    mark(e, 1);
    LMM_CK(lmm::launch_finalize(w.partial, e->nscen * nb, w.items, 1, paths, vmean, vse,
                                e->flag.as<int>(), e->stream));
    if (central)
        LMM_CK(lmm::launch_bump_central(vmean, vse, d_mean, d_se, e->nscen, e->nn, h, e->stream));
    else
        LMM_CK(lmm::launch_bump_diff(d_mean, d_se, e->nscen, nb, h, e->stream));
    mark(e, 2);
    e->last_launches = 3;
    return LMM_OK;
}

// Process-wide engine with the reference's own parameter set, for the
// reference-signature entry points.
std::mutex g_ref_mu;
lmm_engine *g_ref_engine = nullptr;

const int kRefMat[15] = {4, 4, 4, 8, 8, 8, 20, 20, 20, 28, 28, 28, 40, 40, 40};  // params.h:38

int ref_engine(lmm_engine **out)
{
    if (g_ref_engine) {
        *out = g_ref_engine;
        return LMM_OK;
    }
    // params.h:39-40 spells the strikes as float literals; the FP64 build
    // therefore prices with their float-rounded values.
    const float kRateF[3] = {0.045f, 0.05f, 0.055f};
    double rates[15];
    for (int o = 0; o < 15; ++o) rates[o] = (double)kRateF[o % 3];
    std::vector<double> L0(80, 0.051), lam(80, 0.2);  // liborSwaptionGreeks.cpp:270-271
    lmm_params p{80, 40, 15, 1, 0.25, L0.data(), lam.data(), kRefMat, rates};
    LMM_TRY(lmm_engine_create(&p, 0, &g_ref_engine));
    *out = g_ref_engine;
    return LMM_OK;
}

}  // namespace

extern "C" {

int lmm_validate_params(const lmm_params *p) { return validate(p); }

int64_t lmm_num_outputs(const lmm_params *p) { return p ? 1 + 2 * (int64_t)p->nn : 0; }

const char *lmm_status_string(int s)
{
    switch (s) {
        case LMM_OK: return "ok";
        case LMM_ERR_INVALID_ARG: return "invalid argument";
        case LMM_ERR_UNSUPPORTED: return "unsupported";
        case LMM_ERR_CUDA: return "CUDA error";
        case LMM_ERR_NONFINITE: return "non-finite result";
        case LMM_ERR_NO_DEVICE: return "no CUDA device";
        case LMM_ERR_TOO_LARGE: return "too large";
        case LMM_ERR_OUT_OF_MEMORY: return "out of device memory";
        default: return "unknown status";
    }
}

const char *lmm_last_error(void) { return g_last_error.c_str(); }

const char *lmm_version(void) { return "0.1.0"; }

int lmm_engine_create(const lmm_params *p, int32_t device, lmm_engine **out)
{
    if (!out) return fail(LMM_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    LMM_TRY(validate(p));
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0) return fail(LMM_ERR_NO_DEVICE, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(LMM_ERR_INVALID_ARG, "device index out of range");
    std::unique_ptr<lmm_engine> e(new lmm_engine());
    e->device = device;
    e->nn = p->nn;
    e->nmat = p->nmat;
    e->nopt = p->nopt;
    e->nscen = p->nscen;
    e->delta = p->delta;
    LMM_CK(cudaSetDevice(device));
    LMM_CK(cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, device));

    const int nn = p->nn, nmat = p->nmat, nopt = p->nopt, ns = p->nscen, M = nn - nmat;
    const double d = p->delta;
    const double log2e = 1.4426950408889634073599246810019;
    std::vector<float4> kc(nn);
    std::vector<float> L0f((size_t)ns * nn), iL0f((size_t)ns * nn);
    for (int k = 0; k < nn; ++k) {
        const double l = p->lambda[k];
        kc[k] = make_float4((float)(l * log2e), (float)(-0.5 * d * l * l * log2e), (float)(d * d * l), (float)l);
    }
    for (size_t i = 0; i < (size_t)ns * nn; ++i) {
        L0f[i] = (float)p->L0[i];
        iL0f[i] = 1.0f / L0f[i];
    }
    // options grouped by swap length (CSR over m = maturity-1), stable order
    std::vector<int> order(nopt);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return p->maturities[a] < p->maturities[b]; });
    std::vector<int> ost(M + 1, 0);
    std::vector<float> okf(nopt);
    std::vector<double> okd(nopt);
    for (int o = 0; o < nopt; ++o) {
        ost[p->maturities[order[o]]] += 1;  // count at m+1 = maturity
        okf[o] = (float)p->swaprates[order[o]];
        okd[o] = p->swaprates[order[o]];
    }
    for (int m = 0; m < M; ++m) ost[m + 1] += ost[m];

    // one allocation, 256-byte aligned sections
    size_t off = 0;
    auto sect = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~size_t(255);
        return o;
    };
    const size_t o_kc = sect(sizeof(float4) * nn);
    const size_t o_l0f = sect(sizeof(float) * L0f.size()), o_il0f = sect(sizeof(float) * iL0f.size());
    const size_t o_l0d = sect(sizeof(double) * L0f.size()), o_lamd = sect(sizeof(double) * nn);
    const size_t o_ost = sect(sizeof(int) * (M + 1)), o_okf = sect(sizeof(float) * std::max(1, nopt));
    const size_t o_okd = sect(sizeof(double) * std::max(1, nopt));
    const size_t wrow = (size_t)std::max(1, nopt);
    const size_t o_wf = sect(sizeof(float) * wrow * (nopt + 1)), o_wd = sect(sizeof(double) * wrow * (nopt + 1));
    std::vector<float> wf(wrow * (nopt + 1), 0.0f);
    std::vector<double> wd(wrow * (nopt + 1), 0.0);
    for (int g = 0; g < nopt; ++g) {
        wf[g] = 1.0f;
        wd[g] = 1.0;
        wf[wrow * (1 + g) + g] = 1.0f;
        wd[wrow * (1 + g) + g] = 1.0;
    }
    e->opt_slot.assign(nopt, 0);
    for (int g = 0; g < nopt; ++g) e->opt_slot[order[g]] = g;
    LMM_TRY(e->model.ensure(off));
    char *base = e->model.as<char>();
    auto up = [&](size_t o, const void *src, size_t bytes) {
        return bytes ? cudaMemcpy(base + o, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    LMM_CK(up(o_kc, kc.data(), sizeof(float4) * nn));
    LMM_CK(up(o_l0f, L0f.data(), sizeof(float) * L0f.size()));
    LMM_CK(up(o_il0f, iL0f.data(), sizeof(float) * iL0f.size()));
    LMM_CK(up(o_l0d, p->L0, sizeof(double) * L0f.size()));
    LMM_CK(up(o_lamd, p->lambda, sizeof(double) * nn));
    LMM_CK(up(o_ost, ost.data(), sizeof(int) * (M + 1)));
    LMM_CK(up(o_okf, okf.data(), sizeof(float) * nopt));
    LMM_CK(up(o_okd, okd.data(), sizeof(double) * nopt));
    LMM_CK(up(o_wf, wf.data(), sizeof(float) * wf.size()));
    LMM_CK(up(o_wd, wd.data(), sizeof(double) * wd.size()));
    e->wf_rows = reinterpret_cast<float *>(base + o_wf);
    e->wd_rows = reinterpret_cast<double *>(base + o_wd);

    DevModel &m = e->dm;
    m.nn = nn;
    m.nmat = nmat;
    m.nopt = nopt;
    m.nscen = ns;
    m.delta = (float)d;
    m.sqd = (float)std::sqrt(d);
    m.d2 = (float)(d * d);
    m.deltad = d;
    m.sqdd = std::sqrt(d);
    m.kc = reinterpret_cast<const float4 *>(base + o_kc);
    e->kc_host = kc;
    m.kc_host = e->kc_host.data();
    m.L0f = reinterpret_cast<const float *>(base + o_l0f);
    m.invL0f = reinterpret_cast<const float *>(base + o_il0f);
    m.L0d = reinterpret_cast<const double *>(base + o_l0d);
    m.lamd = reinterpret_cast<const double *>(base + o_lamd);
    m.opt_start = reinterpret_cast<const int *>(base + o_ost);
    m.optKf = reinterpret_cast<const float *>(base + o_okf);
    m.optKd = reinterpret_cast<const double *>(base + o_okd);
    m.optWf = e->wf_rows;
    m.optWd = e->wd_rows;
    // The long-tenor kernels restore saved rates every kDefaultCkpt steps;
    // the thread-per-path kernel (80/40) takes no rate checkpoints.
    m.ckpt = lmm::f32_tpp_supports(nn, nmat) ? 0 : kDefaultCkpt;

    LMM_CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    e->own_stream = true;
    *out = e.release();
    return LMM_OK;
}

int lmm_engine_destroy(lmm_engine *e)
{
    if (!e) return LMM_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->model.release();
    e->wscratch.release();
    e->partial.release();
    e->z32.release();
    e->z64.release();
    e->out.release();
    e->se.release();
    e->flag.release();
    e->vbar.release();
    if (e->copy_stream) {
        cudaStreamSynchronize(e->copy_stream);
        cudaStreamDestroy(e->copy_stream);
    }
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    for (auto &ev : e->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : e->copy_ev)
        if (ev) cudaEventDestroy(ev);
    if (e->ready_ev) cudaEventDestroy(e->ready_ev);
    delete e;
    return LMM_OK;
}

int lmm_engine_set_checkpoint_interval(lmm_engine *e, int32_t steps)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    if (steps < 0 || steps > e->nmat) return fail(LMM_ERR_INVALID_ARG, "steps must be in [0, nmat]");
    const int fam = family_for(e, Mode::Fused);
    if (fam == 0)
        return fail(LMM_ERR_UNSUPPORTED, "no FP32 kernel for nn=" + std::to_string(e->nn) +
                                             ", nmat=" + std::to_string(e->nmat));
    if ((fam == 1 || fam == 6) && steps != 0)
        return fail(LMM_ERR_UNSUPPORTED, "the nn=80, nmat=40 kernel keeps every step's drift sums on chip and "
                                         "takes no rate checkpoints: only 0 is accepted");
    if (fam == 5 && steps % 2 != 0)
        return fail(LMM_ERR_UNSUPPORTED, "the nn=160, nmat=120 kernel runs its steps in pairs: the interval "
                                         "must be even");
    if (fam == 7 && steps % 4 != 0)
        return fail(LMM_ERR_UNSUPPORTED, "the nn=160, nmat=120 kernel restores checkpoints between groups of "
                                         "four reverse steps: the interval must be a multiple of 4");
    e->dm.ckpt = steps;
    return LMM_OK;
}

int32_t lmm_engine_checkpoint_interval(const lmm_engine *e) { return e ? e->dm.ckpt : -1; }

int lmm_engine_set_stream(lmm_engine *e, void *stream)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    LMM_TRY(set_device(e));
    if (e->own_stream && e->stream) {
        LMM_CK(cudaStreamSynchronize(e->stream));
        LMM_CK(cudaStreamDestroy(e->stream));
    }
    e->stream = static_cast<cudaStream_t>(stream);
    e->own_stream = false;
    return LMM_OK;
}

int lmm_engine_synchronize(lmm_engine *e)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    LMM_TRY(set_device(e));
    LMM_CK(cudaStreamSynchronize(e->stream));
    return LMM_OK;
}

int32_t lmm_engine_last_launches(const lmm_engine *e) { return e ? e->last_launches : 0; }

int lmm_engine_set_timing(lmm_engine *e, int32_t enable)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    LMM_TRY(set_device(e));
    if (enable && !e->ev[0])
        for (auto &ev : e->ev) LMM_CK(cudaEventCreate(&ev));
    e->timing = enable != 0;
    e->timed = false;
    return LMM_OK;
}

int lmm_engine_kernel_time(lmm_engine *e, double *main_kernel_ms, double *total_ms)
{
    if (!e || !main_kernel_ms) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    if (!e->timed) return fail(LMM_ERR_INVALID_ARG, "no timed call: enable timing first");
    LMM_TRY(set_device(e));
    LMM_CK(cudaEventSynchronize(e->ev[2]));
    float a = 0.0f, b = 0.0f;
    LMM_CK(cudaEventElapsedTime(&a, e->ev[0], e->ev[1]));
    LMM_CK(cudaEventElapsedTime(&b, e->ev[0], e->ev[2]));
    *main_kernel_ms = a;
    if (total_ms) *total_ms = b;
    return LMM_OK;
}

// Times a calibration kernel (16 operations per thread per iteration, 8 x 256
// threads per SM) for about `ms` milliseconds; returns operations per second.
static int peak_probe(int32_t device, double ms, const char *what,
                      const std::function<cudaError_t(int, int, float *, cudaStream_t)> &launch, double *ops_s)
{
    if (!ops_s || !(ms > 0.0)) return fail(LMM_ERR_INVALID_ARG, "need an output and ms > 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(LMM_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(LMM_ERR_INVALID_ARG, "device index out of range");
    LMM_CK(cudaSetDevice(device));
    int sms = 0;
    LMM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int blocks = sms * 8;                  // 8 x 256 threads per SM
    DevBuf sink;
    LMM_TRY(sink.ensure(sizeof(float) * (size_t)blocks * 256));
    cudaStream_t st;
    LMM_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    auto run = [&](int iters, float *out_ms) -> cudaError_t {
        cudaEventRecord(a, st);
        cudaError_t err = launch(blocks, iters, sink.as<float>(), st);
        cudaEventRecord(b, st);
        if (err != cudaSuccess) return err;
        err = cudaEventSynchronize(b);
        if (err != cudaSuccess) return err;
        return cudaEventElapsedTime(out_ms, a, b);
    };
    float t = 0.0f;
    int iters = 4096;
    cudaError_t err = run(iters, &t);           // warm-up and calibration
    if (err == cudaSuccess && t > 0.0f) {
        iters = (int)std::min(1e8, std::max(4096.0, iters * ms / t));
        err = run(iters, &t);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    sink.release();
    if (err != cudaSuccess) return cuda_fail(err, what);
    *ops_s = 16.0 * (double)iters * blocks * 256.0 / (t * 1e-3);
    return LMM_OK;
}

int lmm_fp32_peak_tflops(int32_t device, double ms, double *tflops)
{
    if (!tflops) return fail(LMM_ERR_INVALID_ARG, "tflops is NULL");
    double fma_s = 0.0;
    LMM_TRY(peak_probe(device, ms, "FFMA peak probe",
                       [](int blocks, int iters, float *sink, cudaStream_t st) {
                           return lmm::launch_ffma_peak(blocks, iters, 0.9999f, 1e-4f, sink, st);
                       },
                       &fma_s));
    *tflops = 2.0 * fma_s / 1e12;
    return LMM_OK;
}

int lmm_fp64_peak_tflops(int32_t device, double ms, double *tflops)
{
    if (!tflops) return fail(LMM_ERR_INVALID_ARG, "tflops is NULL");
    double fma_s = 0.0;
    LMM_TRY(peak_probe(device, ms, "DFMA peak probe",
                       [](int blocks, int iters, float *sink, cudaStream_t st) {
                           return lmm::launch_dfma_peak(blocks, iters, 0.9999, 1e-4, sink, st);
                       },
                       &fma_s));
    *tflops = 2.0 * fma_s / 1e12;
    return LMM_OK;
}

int lmm_mufu_peak_gops(int32_t device, double ms, double *ex2_gops, double *rcp_gops, double *mixed_gops)
{
    double *outs[3] = {ex2_gops, rcp_gops, mixed_gops};
    for (int kind = 0; kind < 3; ++kind) {
        if (!outs[kind]) continue;
        double r = 0.0;
        LMM_TRY(peak_probe(device, ms, "MUFU peak probe",
                           [kind](int blocks, int iters, float *sink, cudaStream_t st) {
                               return lmm::launch_mufu_peak(kind, blocks, iters, sink, st);
                           },
                           &r));
        *outs[kind] = r / 1e9;
    }
    return LMM_OK;
}

// ---- FP32 adjoint ----------------------------------------------------------

int lmm_greeks_f32_device(lmm_engine *e, const float *d_z, int64_t paths, double *d_out, double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    return run_f32(e, Mode::Fused, d_z, 0, 0, false, paths, nullptr, nullptr, d_out, d_se);
}

// ---- portfolio weights and per-swaption breakdown ---------------------------

int lmm_engine_set_weights(lmm_engine *e, const double *weights)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    const int nopt = e->nopt;
    std::vector<double> wd(std::max(1, nopt), 1.0);
    std::vector<float> wf(std::max(1, nopt), 1.0f);
    for (int o = 0; o < nopt && weights; ++o) {
        if (!std::isfinite(weights[o])) return fail(LMM_ERR_INVALID_ARG, "weights must be finite");
        wd[e->opt_slot[o]] = weights[o];
        wf[e->opt_slot[o]] = (float)weights[o];
    }
    LMM_TRY(set_device(e));
    // ordered after earlier work on the engine's stream; the host vectors
    // stay alive until the copies have run
    LMM_CK(cudaMemcpyAsync(e->wd_rows, wd.data(), sizeof(double) * nopt, cudaMemcpyHostToDevice, e->stream));
    LMM_CK(cudaMemcpyAsync(e->wf_rows, wf.data(), sizeof(float) * nopt, cudaMemcpyHostToDevice, e->stream));
    LMM_CK(cudaStreamSynchronize(e->stream));
    return LMM_OK;
}

// One fused call per swaption with that swaption alone at unit weight: the
// model is passed to each launch by value, so only the weight pointers change.
static int per_swaption(lmm_engine *e, const std::function<int(int)> &call)
{
    const DevModel saved = e->dm;
    const size_t row = (size_t)std::max(1, e->nopt);
    int rc = LMM_OK;
    int32_t launches = 0;
    for (int o = 0; o < e->nopt && rc == LMM_OK; ++o) {
        e->dm.optWf = e->wf_rows + row * (1 + e->opt_slot[o]);
        e->dm.optWd = e->wd_rows + row * (1 + e->opt_slot[o]);
        rc = call(o);
        launches += e->last_launches;
    }
    e->dm = saved;
    e->last_launches = launches;
    return rc;
}

int lmm_swaption_breakdown_f32_device(lmm_engine *e, const float *d_z, int64_t paths, double *d_out,
                                      double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    if (e->nopt < 1) return fail(LMM_ERR_INVALID_ARG, "the portfolio has no swaptions");
    const size_t per = (size_t)e->nscen * (1 + 2 * e->nn);
    return per_swaption(e, [&](int o) {
        return run_f32(e, Mode::Fused, d_z, 0, 0, false, paths, nullptr, nullptr, d_out + per * o,
                       d_se ? d_se + per * o : nullptr);
    });
}

int lmm_swaption_breakdown_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double *d_out,
                                      double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    if (e->nopt < 1) return fail(LMM_ERR_INVALID_ARG, "the portfolio has no swaptions");
    const size_t per = (size_t)e->nscen * (1 + 2 * e->nn);
    return per_swaption(e, [&](int o) {
        return run_f64(e, d_z, paths, d_out + per * o, d_se ? d_se + per * o : nullptr);
    });
}

// Host call with the copy overlapped: the normals go up in kHostChunks
// pieces on the engine's copy stream; the fused kernel of piece c starts as
// soon as piece c has landed, while the later pieces are still in flight.
// Relative piece sizes kHostSplit: the first piece's copy is the only one
// nothing overlaps, so it is small (1/72: one wave of the split-reverse
// kernel, 9 MB of 671 MB at 4M paths, 0.04 ms at the measured 211 GB/s), and
// each later piece, about three times the one before, lands before the
// compute of the pieces ahead of it ends (a wave computes in about 0.14 ms
// and copies in 0.04 ms). Measured on GB300 at 4,194,304 paths: four equal
// pieces cost 0.6 ms per call more than {1,3,6,6}/16 (an earlier kernel);
// piece boundaries on whole device waves: 363 -> 369 M paths/s;
// {1,3,10,22}/36: 369 -> 373 M paths/s; with the 9.8 ms kernel,
// {1,3,10,22}, {1,2,5,10,18}, {1,2,4,8,21}, {1,3,8,24}, {1,4,31}: 10.07,
// 10.05, 10.06, 10.03, 11.70 ms per call, and {1,3,8,24}, {1,3,9,27,32},
// {1,2,6,18,45}, {1,4,16,51}, {1,3,9,59}: 10.04, 10.02, 10.02, 10.23, 11.32.
// Each piece writes its own range of partial sums and one ordered k_finalize
// covers them all. Single-scenario engines only.
#ifndef LMM_HOST_SPLIT
#define LMM_HOST_SPLIT 1, 2, 6, 18, 45
#endif
constexpr int kHostSplit[] = {LMM_HOST_SPLIT};
constexpr int kHostChunks = sizeof(kHostSplit) / sizeof(kHostSplit[0]);
static_assert(kHostChunks <= 8, "one copy event per piece");
constexpr int64_t kPipelineMinPaths = int64_t(1) << 18;

int run_f32_host_pipelined(lmm_engine *e, const float *z, int64_t paths)
{
    const int fam = family_for(e, Mode::Fused);
    if (fam == 0) return fail(LMM_ERR_UNSUPPORTED, "no FP32 kernel for this shape");
    int bps = 0;
    LMM_TRY(blocks_per_sm(e, fam, Mode::Fused, false, &bps));
    const int per_batch = batch_paths(e, fam, Mode::Fused);
    const int nout = 1 + 2 * e->nn;
    int64_t cpaths[kHostChunks], cfirst[kHostChunks], citems[kHostChunks], cppt[kHostChunks];
    int64_t total_items = 0, wsum = 0, wcum = 0;
    for (int c = 0; c < kHostChunks; ++c) wsum += kHostSplit[c];
    // Piece boundaries on whole waves of the device (SMs x resident blocks x
    // paths per block): every piece but the last runs full waves, so the
    // pieces together take as many waves as one launch would. Pieces that
    // round to nothing are dropped.
    const int64_t wave = (int64_t)e->sms * bps * per_batch;
    int64_t bnd[kHostChunks + 1];
    bnd[0] = 0;
    for (int c = 1; c < kHostChunks; ++c) {
        wcum += kHostSplit[c - 1];
        const int64_t x = paths * wcum / wsum;
        bnd[c] = std::min(std::max((x + wave / 2) / wave * wave, bnd[c - 1]), paths);
    }
    bnd[kHostChunks] = paths;
    int C = 0;
    for (int c = 0; c < kHostChunks; ++c) {
        if (bnd[c + 1] <= bnd[c]) continue;
        cfirst[C] = bnd[c];
        cpaths[C] = bnd[c + 1] - bnd[c];
        ++C;
    }
    for (int c = 0; c < C; ++c) {
        plan_items(e, 1, cpaths[c], per_batch, bps, &citems[c], &cppt[c]);
        if (cppt[c] > INT32_MAX || citems[c] > INT32_MAX) return fail(LMM_ERR_TOO_LARGE, "launch too large");
        total_items += citems[c];
    }
    LMM_TRY(e->partial.ensure(sizeof(double) * (size_t)total_items * 2 * nout));
    float *wscr = nullptr;
    if (fam == 2 || fam == 5 || fam == 6 || fam == 7) {
        int64_t most = 0;
        for (int c = 0; c < C; ++c) most = std::max(most, std::min<int64_t>(citems[c], (int64_t)e->sms * bps));
        // the pieces run one after another
        LMM_TRY(fam == 2 ? wpp_scratch(e, most, &wscr)
                         : fam == 5 ? tp2_scratch(e, most, &wscr)
                                    : fam == 6 ? tps_scratch(e, most, &wscr) : tpq_scratch(e, most, &wscr));
    }
    LMM_TRY(e->flag.ensure(sizeof(int)));
    if (!e->copy_stream) LMM_CK(cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking));
    if (!e->ready_ev) LMM_CK(cudaEventCreateWithFlags(&e->ready_ev, cudaEventDisableTiming));
    for (int c = 0; c < C; ++c)
        if (!e->copy_ev[c]) LMM_CK(cudaEventCreateWithFlags(&e->copy_ev[c], cudaEventDisableTiming));
    // the copies must not overtake earlier work on the engine's stream
    LMM_CK(cudaEventRecord(e->ready_ev, e->stream));
    LMM_CK(cudaStreamWaitEvent(e->copy_stream, e->ready_ev, 0));
    float *dz = e->z32.as<float>();
    for (int c = 0; c < C; ++c) {
        const size_t off = (size_t)cfirst[c] * e->nmat, n = (size_t)cpaths[c] * e->nmat;
        LMM_CK(cudaMemcpyAsync(dz + off, z + off, sizeof(float) * n, cudaMemcpyHostToDevice, e->copy_stream));
        LMM_CK(cudaEventRecord(e->copy_ev[c], e->copy_stream));
    }
    LMM_CK(cudaMemsetAsync(e->flag.p, 0, sizeof(int), e->stream));
    mark(e, 0);
    double *part = e->partial.as<double>();
    for (int c = 0; c < C; ++c) {
        LMM_CK(cudaStreamWaitEvent(e->stream, e->copy_ev[c], 0));
        Work w{};
        w.paths = cpaths[c];
        w.items = (int)citems[c];
        w.ppt = (int)cppt[c];
        w.nout = nout;
        w.grid = (int)std::min<int64_t>(citems[c], (int64_t)e->sms * bps);
        w.partial = part;
        const float *zc = dz + (size_t)cfirst[c] * e->nmat;
        cudaError_t err = launch_f32_family(fam, e->dm, Mode::Fused, zc, 0, 0, false, w, wscr, nullptr, e->stream);
        if (err != cudaSuccess) return cuda_fail(err, "FP32 LMM kernel launch");
        part += (size_t)citems[c] * 2 * nout;
    }
    mark(e, 1);
    LMM_CK(lmm::launch_finalize(e->partial.as<double>(), 1, (int)total_items, nout, paths,
                                e->out.as<double>(), e->se.as<double>(), e->flag.as<int>(), e->stream));
    mark(e, 2);
    e->last_launches = C + 1;
    return LMM_OK;
}

int lmm_greeks_f32_host(lmm_engine *e, const float *z, int64_t paths, double *out, double *se)
{
    if (!e || !z || !out) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    LMM_TRY(check_paths(paths));
    LMM_TRY(set_device(e));
    const size_t zb = sizeof(float) * (size_t)paths * e->nmat;
    LMM_TRY(e->z32.ensure(zb));
    LMM_TRY(ensure_outputs(e, 1 + 2 * e->nn));
    if (e->nscen == 1 && paths >= kPipelineMinPaths) {
        LMM_TRY(run_f32_host_pipelined(e, z, paths));
    } else {
        LMM_CK(cudaMemcpyAsync(e->z32.p, z, zb, cudaMemcpyHostToDevice, e->stream));
        LMM_TRY(run_f32(e, Mode::Fused, e->z32.as<float>(), 0, 0, false, paths, nullptr, nullptr,
                        e->out.as<double>(), e->se.as<double>()));
    }
    return fetch(e, 1 + 2 * e->nn, out, se);
}

int lmm_greeks_philox_device(lmm_engine *e, uint64_t seed, int64_t path0, int64_t paths,
                             double *d_out, double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    return run_f32(e, Mode::Fused, nullptr, seed, path0, true, paths, nullptr, nullptr, d_out, d_se);
}

int lmm_greeks_philox_host(lmm_engine *e, uint64_t seed, int64_t path0, int64_t paths, double *out,
                           double *se)
{
    if (!e || !out) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    LMM_TRY(check_paths(paths));
    LMM_TRY(set_device(e));
    LMM_TRY(ensure_outputs(e, 1 + 2 * e->nn));
    LMM_TRY(run_f32(e, Mode::Fused, nullptr, seed, path0, true, paths, nullptr, nullptr,
                    e->out.as<double>(), e->se.as<double>()));
    return fetch(e, 1 + 2 * e->nn, out, se);
}

// ---- forward/backward pair ---------------------------------------------------

int lmm_tape_create(lmm_engine *e, int64_t paths, lmm_tape **out)
{
    if (!e || !out) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    LMM_TRY(check_paths(paths));
    LMM_TRY(set_device(e));
    std::unique_ptr<lmm_tape> t(new lmm_tape());
    t->e = e;
    t->paths = paths;
    // The thread-per-path (nn=80, nmat=40) and thread-pair (nn=160, nmat=120)
    // kernels keep the terminal rates and the per-step drift sums; the
    // warp-per-path backward recomputes its forward from the same normals and
    // needs no tape.
    const int fam = family_for(e, Mode::Forward);
    if (fam == 1 || fam == 5) {
        // thread pair: also the drift sums at the half boundary
        const size_t rows = (size_t)e->nn + (size_t)e->nmat * (fam == 5 ? 2 : 1);
        LMM_TRY(t->buf.ensure(sizeof(float) * rows * e->nscen * (size_t)paths));
    }
    *out = t.release();
    return LMM_OK;
}

int lmm_tape_destroy(lmm_tape *t)
{
    if (!t) return LMM_OK;
    cudaSetDevice(t->e->device);
    t->buf.release();
    delete t;
    return LMM_OK;
}

int lmm_forward_f32_device(lmm_engine *e, const float *d_z, int64_t paths, lmm_tape *t,
                           double *d_value, double *d_value_se)
{
    if (!e || !t) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    if (t->e != e || t->paths != paths) return fail(LMM_ERR_INVALID_ARG, "tape belongs to another engine or size");
    return run_f32(e, Mode::Forward, d_z, 0, 0, false, paths, t->buf.as<float>(), nullptr, d_value,
                   d_value_se);
}

int lmm_backward_f32_device(lmm_engine *e, const float *d_z, const lmm_tape *t,
                            const double *value_bar, double *d_grad, double *d_grad_se)
{
    if (!e || !t || !value_bar) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    if (t->e != e) return fail(LMM_ERR_INVALID_ARG, "tape belongs to another engine");
    for (int s = 0; s < e->nscen; ++s)
        if (!std::isfinite(value_bar[s])) return fail(LMM_ERR_INVALID_ARG, "value_bar must be finite");
    LMM_TRY(set_device(e));
    LMM_TRY(e->vbar.ensure(sizeof(double) * e->nscen));
    LMM_CK(cudaMemcpyAsync(e->vbar.p, value_bar, sizeof(double) * e->nscen, cudaMemcpyHostToDevice,
                           e->stream));
    return run_f32(e, Mode::Backward, d_z, 0, 0, false, t->paths, const_cast<float *>(t->buf.as<float>()),
                   e->vbar.as<double>(), d_grad, d_grad_se);
}

// ---- FP64 -------------------------------------------------------------------

int lmm_greeks_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double *d_out, double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    return run_f64(e, d_z, paths, d_out, d_se);
}

int lmm_greeks_f32_rounding_device(lmm_engine *e, const float *d_z, int64_t paths, double *d_out, double *d_se,
                                   double *d_err)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    if (!d_err) return fail(LMM_ERR_INVALID_ARG, "rounding-error pointer is NULL");
    LMM_TRY(run_f32(e, Mode::Fused, d_z, 0, 0, false, paths, nullptr, nullptr, d_out, d_se));
    const int32_t l32 = e->last_launches;
    const size_t nz = (size_t)paths * e->nmat;
    const int nout = 1 + 2 * e->nn;
    LMM_TRY(e->z64.ensure(sizeof(double) * nz));
    LMM_TRY(ensure_outputs(e, nout));
    LMM_CK(lmm::launch_widen(d_z, e->z64.as<double>(), (int64_t)nz, e->stream));
    LMM_TRY(run_f64(e, e->z64.as<double>(), paths, e->out.as<double>(), e->se.as<double>()));
    LMM_CK(lmm::launch_abs_diff(d_out, e->out.as<double>(), d_err, e->nscen * nout, e->stream));
    e->last_launches = l32 + e->last_launches + 2;
    return LMM_OK;
}

int lmm_greeks_f64_host(lmm_engine *e, const double *z, int64_t paths, double *out, double *se)
{
    if (!e || !z || !out) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    LMM_TRY(check_paths(paths));
    LMM_TRY(set_device(e));
    const size_t zb = sizeof(double) * (size_t)paths * e->nmat;
    LMM_TRY(e->z64.ensure(zb));
    LMM_TRY(ensure_outputs(e, 1 + 2 * e->nn));
    LMM_CK(cudaMemcpyAsync(e->z64.p, z, zb, cudaMemcpyHostToDevice, e->stream));
    LMM_TRY(run_f64(e, e->z64.as<double>(), paths, e->out.as<double>(), e->se.as<double>()));
    return fetch(e, 1 + 2 * e->nn, out, se);
}

int lmm_bump_greeks_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double h,
                               double *d_out, double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    return run_bump(e, d_z, paths, h, false, d_out, d_se);
}

int lmm_bump_greeks_central_f64_device(lmm_engine *e, const double *d_z, int64_t paths, double h,
                                       double *d_out, double *d_se)
{
    if (!e) return fail(LMM_ERR_INVALID_ARG, "engine is NULL");
    return run_bump(e, d_z, paths, h, true, d_out, d_se);
}

namespace {
int bump_host(lmm_engine *e, const double *z, int64_t paths, double h, bool central, double *out, double *se)
{
    if (!e || !z || !out) return fail(LMM_ERR_INVALID_ARG, "NULL argument");
    LMM_TRY(check_paths(paths));
    LMM_TRY(set_device(e));
    const size_t zb = sizeof(double) * (size_t)paths * e->nmat;
    LMM_TRY(e->z64.ensure(zb));
    LMM_TRY(ensure_outputs(e, 1 + 2 * e->nn));
    LMM_CK(cudaMemcpyAsync(e->z64.p, z, zb, cudaMemcpyHostToDevice, e->stream));
    LMM_TRY(run_bump(e, e->z64.as<double>(), paths, h, central, e->out.as<double>(), e->se.as<double>()));
    return fetch(e, 1 + 2 * e->nn, out, se);
}
}  // namespace

int lmm_bump_greeks_f64_host(lmm_engine *e, const double *z, int64_t paths, double h, double *out,
                             double *se)
{
    return bump_host(e, z, paths, h, false, out, se);
}

int lmm_bump_greeks_central_f64_host(lmm_engine *e, const double *z, int64_t paths, double h, double *out,
                                     double *se)
{
    return bump_host(e, z, paths, h, true, out, se);
}

// ---- normals -------------------------------------------------------------------

int lmm_normals_f32_device(uint64_t seed, int64_t path0, int64_t paths, int32_t nmat, float *d_z,
                           void *stream)
{
    if (!d_z || paths < 1 || nmat < 1 || path0 < 0) return fail(LMM_ERR_INVALID_ARG, "bad normals request");
    LMM_CK(lmm::launch_normals_f32(seed, path0, paths, nmat, 0.0f, 1.0f, d_z,
                                   static_cast<cudaStream_t>(stream)));
    return LMM_OK;
}

int lmm_normals_f64_device(uint64_t seed, int64_t path0, int64_t paths, int32_t nmat, double mean,
                           double std_dev, double *d_z, void *stream)
{
    if (!d_z || paths < 1 || nmat < 1 || path0 < 0 || !std::isfinite(mean) || !std::isfinite(std_dev))
        return fail(LMM_ERR_INVALID_ARG, "bad normals request");
    LMM_CK(lmm::launch_normals_f64(seed, path0, paths, nmat, mean, std_dev, d_z,
                                   static_cast<cudaStream_t>(stream)));
    return LMM_OK;
}

static int check_stream_range(int64_t first, int64_t count, const void *out)
{
    if (first < 0 || count < 0 || count > INT64_MAX - first)
        return fail(LMM_ERR_INVALID_ARG, "need first >= 0, count >= 0, first + count < 2^63");
    if (count > 0 && !out) return fail(LMM_ERR_INVALID_ARG, "output pointer is NULL");
    return LMM_OK;
}

int lmm_mrg32k3a_uniforms_device(uint32_t seed, int64_t first, int64_t count, double *d_u, void *stream)
{
    LMM_TRY(check_stream_range(first, count, d_u));
    LMM_CK(lmm::launch_mrg32k3a(0, seed, first, count, 0.0, 1.0, d_u, static_cast<cudaStream_t>(stream)));
    return LMM_OK;
}

int lmm_mrg32k3a_normals_f64_device(uint32_t seed, int64_t first, int64_t count, double mean,
                                    double std_dev, double *d_z, void *stream)
{
    LMM_TRY(check_stream_range(first, count, d_z));
    if (!std::isfinite(mean) || !std::isfinite(std_dev)) return fail(LMM_ERR_INVALID_ARG, "mean/std_dev must be finite");
    LMM_CK(lmm::launch_mrg32k3a(1, seed, first, count, mean, std_dev, d_z, static_cast<cudaStream_t>(stream)));
    return LMM_OK;
}

int lmm_mrg32k3a_normals_f32_device(uint32_t seed, int64_t first, int64_t count, float mean,
                                    float std_dev, float *d_z, void *stream)
{
    LMM_TRY(check_stream_range(first, count, d_z));
    if (!std::isfinite(mean) || !std::isfinite(std_dev)) return fail(LMM_ERR_INVALID_ARG, "mean/std_dev must be finite");
    LMM_CK(lmm::launch_mrg32k3a(2, seed, first, count, mean, std_dev, d_z, static_cast<cudaStream_t>(stream)));
    return LMM_OK;
}

// ---- the reference's signature ----------------------------------------------------

static int swaption_greeks_f64(bool mrg, double *z, int num, double mean, double std_dev, double *d_v,
                               double *d_Lb, int numPaths)
{
    if (!z || !d_v || !d_Lb || numPaths < 1 || (int64_t)num != 40 * (int64_t)numPaths)
        return fail(LMM_ERR_INVALID_ARG, "need z[40*numPaths], d_v, d_Lb and numPaths >= 1");
    if (!std::isfinite(mean) || !std::isfinite(std_dev)) return fail(LMM_ERR_INVALID_ARG, "mean/std_dev must be finite");
    std::lock_guard<std::mutex> lk(g_ref_mu);
    lmm_engine *e = nullptr;
    LMM_TRY(ref_engine(&e));
    LMM_TRY(set_device(e));
    LMM_TRY(e->z64.ensure(sizeof(double) * (size_t)num));
    LMM_TRY(ensure_outputs(e, 1 + 2 * e->nn));
    if (mrg)
        LMM_CK(lmm::launch_mrg32k3a(1, 12345u, 0, num, mean, std_dev, e->z64.p, e->stream));
    else
        LMM_CK(lmm::launch_normals_f64(12345u, 0, numPaths, 40, mean, std_dev, e->z64.as<double>(), e->stream));
    LMM_CK(cudaMemcpyAsync(z, e->z64.p, sizeof(double) * (size_t)num, cudaMemcpyDeviceToHost, e->stream));
    LMM_TRY(run_f64(e, e->z64.as<double>(), numPaths, e->out.as<double>(), e->se.as<double>()));
    std::vector<double> out(1 + 2 * e->nn);
    LMM_TRY(fetch(e, 1 + 2 * e->nn, out.data(), nullptr));
    *d_v = out[0];
    *d_Lb = out[e->nn];
    return LMM_OK;
}

static int swaption_greeks_f32(bool mrg, float *z, int num, float mean, float std_dev, float *d_v,
                               float *d_Lb, int numPaths)
{
    if (!z || !d_v || !d_Lb || numPaths < 1 || (int64_t)num != 40 * (int64_t)numPaths)
        return fail(LMM_ERR_INVALID_ARG, "need z[40*numPaths], d_v, d_Lb and numPaths >= 1");
    if (!std::isfinite(mean) || !std::isfinite(std_dev)) return fail(LMM_ERR_INVALID_ARG, "mean/std_dev must be finite");
    std::lock_guard<std::mutex> lk(g_ref_mu);
    lmm_engine *e = nullptr;
    LMM_TRY(ref_engine(&e));
    LMM_TRY(set_device(e));
    LMM_TRY(e->z32.ensure(sizeof(float) * (size_t)num));
    LMM_TRY(ensure_outputs(e, 1 + 2 * e->nn));
    if (mrg)
        LMM_CK(lmm::launch_mrg32k3a(2, 12345u, 0, num, mean, std_dev, e->z32.p, e->stream));
    else
        LMM_CK(lmm::launch_normals_f32(12345u, 0, numPaths, 40, mean, std_dev, e->z32.as<float>(), e->stream));
    LMM_CK(cudaMemcpyAsync(z, e->z32.p, sizeof(float) * (size_t)num, cudaMemcpyDeviceToHost, e->stream));
    LMM_TRY(run_f32(e, Mode::Fused, e->z32.as<float>(), 0, 0, false, numPaths, nullptr, nullptr,
                    e->out.as<double>(), e->se.as<double>()));
    std::vector<double> out(1 + 2 * e->nn);
    LMM_TRY(fetch(e, 1 + 2 * e->nn, out.data(), nullptr));
    *d_v = (float)out[0];
    *d_Lb = (float)out[e->nn];
    return LMM_OK;
}

// `seed` is accepted and ignored, as in the reference (generateRand uses its
// default seed 12345).
int lmm_swaption_greeks(double *z, int num, double mean, double std_dev, int seed, double *d_v,
                        double *d_Lb, int numPaths)
{
    (void)seed;
    return swaption_greeks_f64(false, z, num, mean, std_dev, d_v, d_Lb, numPaths);
}

int lmm_swaption_greeks_f32(float *z, int num, float mean, float std_dev, int seed, float *d_v,
                            float *d_Lb, int numPaths)
{
    (void)seed;
    return swaption_greeks_f32(false, z, num, mean, std_dev, d_v, d_Lb, numPaths);
}

int lmm_swaption_greeks_mrg32k3a(double *z, int num, double mean, double std_dev, int seed, double *d_v,
                                 double *d_Lb, int numPaths)
{
    (void)seed;
    return swaption_greeks_f64(true, z, num, mean, std_dev, d_v, d_Lb, numPaths);
}

int lmm_swaption_greeks_mrg32k3a_f32(float *z, int num, float mean, float std_dev, int seed, float *d_v,
                                     float *d_Lb, int numPaths)
{
    (void)seed;
    return swaption_greeks_f32(true, z, num, mean, std_dev, d_v, d_Lb, numPaths);
}

}  // extern "C"

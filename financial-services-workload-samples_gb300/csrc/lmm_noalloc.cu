// lmm_greeks_f32_device_noalloc: a fused FP32 value + Greeks launch for
// callers that cannot allocate device memory. It runs the one-pass fused
// kernel (k_tpp), which needs no per-path scratch.
//
// Some callers cannot call cudaMalloc: code embedded in a host application
// that owns every device allocation through its own pool, a plug-in whose
// process has exhausted or locked its allocator, or a latency-critical loop
// that must not touch the allocator at all. This entry point needs no engine
// and allocates nothing. Its scratch -- the model constants, the per-block
// FP64 partial sums and the non-finite flag -- lives in one file-scope static
// device array of kScratchBytes, which every GPU that loads the library holds
// until the process exits.
//
// Host code must not pass g_noalloc_scratch itself to a kernel: in host code
// that name is a host-side stand-in, not a device address. The first call on
// each device (with that device current) looks the address up with
// cudaGetSymbolAddress, queries the kernel's occupancy and caches both; make
// that first call before any stream capture. The cache is keyed by the
// device's context: after cudaDeviceReset the next call looks the address up
// again in the new context (the array moves with the reloaded module).
//
// The model constants reach the scratch through a copy kernel that takes them
// by value as its parameter: the launch carries its own copy of them, so no
// host buffer has to outlive the call and the call never waits for the GPU.
#include "lmm_gb300.h"
#include "lmm_internal.h"

#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>

namespace {

constexpr int kNN = 80, kNMAT = 40, kM = kNN - kNMAT, kNout = 1 + 2 * kNN;
constexpr size_t kScratchBytes = LMM_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// Model section of the scratch, uploaded by every call (device layout).
struct NoallocModel {
    float4 kc[kNN];
    float L0f[LMM_NOALLOC_MAX_SCEN * kNN];
    float iL0f[LMM_NOALLOC_MAX_SCEN * kNN];
    double L0d[LMM_NOALLOC_MAX_SCEN * kNN];
    double lamd[kNN];
    int ost[kM + 1];
    float okf[LMM_MAX_NOPT];
    double okd[LMM_MAX_NOPT];
    float owf[LMM_MAX_NOPT];     // notional weights: the reference's portfolio, all 1
    double owd[LMM_MAX_NOPT];
};

constexpr size_t kModelBytes = (sizeof(NoallocModel) + 255) & ~size_t(255);
constexpr size_t kFlagBytes = 256;
constexpr size_t kPartialBytes = kScratchBytes - kModelBytes - kFlagBytes;
constexpr int kMaxItems = (int)(kPartialBytes / (sizeof(double) * 2 * kNout));
static_assert(kMaxItems >= 64 * LMM_NOALLOC_MAX_SCEN, "scratch too small");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

static_assert(sizeof(NoallocModel) % 4 == 0, "the model is copied in 32-bit words");
static_assert(sizeof(NoallocModel) + 2 * sizeof(void *) <= 32000, "the model travels as a kernel parameter");

// Copies the model (a kernel parameter, so the launch owns its own copy of
// it) into the scratch and clears the non-finite flag.
__global__ void k_noalloc_upload(const __grid_constant__ NoallocModel hm, NoallocModel *dst, int *flag)
{
    const unsigned *src = reinterpret_cast<const unsigned *>(&hm);
    unsigned *d = reinterpret_cast<unsigned *>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(NoallocModel) / 4); i += blockDim.x) d[i] = src[i];
    if (threadIdx.x == 0) *flag = 0;
}

struct DeviceSetup {
    bool ready = false;
    unsigned long long ctx_id = 0;      // context the address belongs to
    unsigned char *scratch = nullptr;   // device address of g_noalloc_scratch
    int sms = 0, bps = 0;
};

std::mutex g_mu;
DeviceSetup g_setup[kMaxDevices];

// The current context's unique id (cuCtxGetId through the runtime's driver
// entry points, so the library needs no link against libcuda). *found is
// false while the calling thread has no current context yet.
int current_context_id(unsigned long long *id, bool *found)
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess)
            return lmm::record_error(LMM_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId unavailable");
        get_current = reinterpret_cast<GetCurrent>(f1);
        get_id = reinterpret_cast<GetId>(f2);
    }
    CUcontext ctx = nullptr;
    *found = false;
    if (get_current(&ctx) != CUDA_SUCCESS) return lmm::record_error(LMM_ERR_CUDA, "cuCtxGetCurrent failed");
    if (!ctx) return LMM_OK;
    if (get_id(ctx, id) != CUDA_SUCCESS) return lmm::record_error(LMM_ERR_CUDA, "cuCtxGetId failed");
    *found = true;
    return LMM_OK;
}

int setup_device(int dev, DeviceSetup *out)
{
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceSetup &s = g_setup[dev];
    unsigned long long ctx = 0;
    bool found = false;
    int rc = current_context_id(&ctx, &found);
    if (rc != LMM_OK) return rc;
    if (!s.ready || !found || s.ctx_id != ctx) {
        s.ready = false;
        void *ptr = nullptr;
        // The lookup also makes the device's primary context current.
        cudaError_t ce = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (ce != cudaSuccess) return lmm::record_cuda_error(ce, "cudaGetSymbolAddress(g_noalloc_scratch)");
        if (!ptr) return lmm::record_error(LMM_ERR_CUDA, "cudaGetSymbolAddress returned NULL");
        if ((rc = current_context_id(&ctx, &found)) != LMM_OK) return rc;
        if (!found) return lmm::record_error(LMM_ERR_CUDA, "no current CUDA context after the lookup");
        int sms = 0, bps = 0;
        ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (ce != cudaSuccess) return lmm::record_cuda_error(ce, "cudaDeviceGetAttribute");
        ce = lmm::tpp_blocks_per_sm(lmm::Mode::Fused, false, &bps);
        if (ce != cudaSuccess) return lmm::record_cuda_error(ce, "occupancy query");
        if (bps < 1) return lmm::record_error(LMM_ERR_UNSUPPORTED, "the fused kernel does not fit on this device");
        s.scratch = static_cast<unsigned char *>(ptr);
        s.ctx_id = ctx;
        s.sms = sms;
        s.bps = bps;
        s.ready = true;
    }
    *out = s;
    return LMM_OK;
}

}  // namespace

extern "C" int lmm_greeks_f32_device_noalloc(const lmm_params *p, const float *d_z, int64_t paths,
                                             double *d_out, double *d_se, void *stream)
{
    int rc = lmm_validate_params(p);
    if (rc != LMM_OK) return rc;
    if (p->nn != kNN || p->nmat != kNMAT)
        return lmm::record_error(LMM_ERR_UNSUPPORTED, "the no-allocation call covers nn=80, nmat=40 only");
    if (p->nscen > LMM_NOALLOC_MAX_SCEN)
        return lmm::record_error(LMM_ERR_TOO_LARGE, "nscen above LMM_NOALLOC_MAX_SCEN");
    if (!d_z || !d_out) return lmm::record_error(LMM_ERR_INVALID_ARG, "NULL device pointer");
    if (paths < 1) return lmm::record_error(LMM_ERR_INVALID_ARG, "paths must be >= 1");
    if (paths > (int64_t(1) << 40)) return lmm::record_error(LMM_ERR_TOO_LARGE, "paths must be <= 2^40");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return lmm::record_error(LMM_ERR_NO_DEVICE, "no CUDA device");
    if (dev < 0 || dev >= kMaxDevices) return lmm::record_error(LMM_ERR_UNSUPPORTED, "device ordinal above 63");
    DeviceSetup ds;
    if ((rc = setup_device(dev, &ds)) != LMM_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // Model constants, built on the host stack in the device layout.
    NoallocModel hm;
    std::memset(&hm, 0, sizeof(hm));
    const double d = p->delta, log2e = 1.4426950408889634073599246810019;
    for (int k = 0; k < kNN; ++k) {
        const double l = p->lambda[k];
        hm.kc[k] = make_float4((float)(l * log2e), (float)(-0.5 * d * l * l * log2e), (float)(d * d * l), (float)l);
        hm.lamd[k] = l;
    }
    for (int i = 0; i < p->nscen * kNN; ++i) {
        hm.L0f[i] = (float)p->L0[i];
        hm.iL0f[i] = 1.0f / hm.L0f[i];
        hm.L0d[i] = p->L0[i];
    }
    // options grouped by swap length (a counting sort keeps the input order)
    int cnt[kM + 2] = {0};
    for (int o = 0; o < p->nopt; ++o) cnt[p->maturities[o]] += 1;
    for (int m = 0; m <= kM; ++m) hm.ost[m] = (m == 0 ? 0 : hm.ost[m - 1] + cnt[m]);
    int fill[kM + 1];
    for (int m = 0; m <= kM; ++m) fill[m] = hm.ost[m];
    for (int o = 0; o < p->nopt; ++o) {
        const int slot = fill[p->maturities[o] - 1]++;
        hm.okf[slot] = (float)p->swaprates[o];
        hm.okd[slot] = p->swaprates[o];
        hm.owf[slot] = 1.0f;
        hm.owd[slot] = 1.0;
    }

    // About two waves of the device, capped by the partial-sum space.
    const int64_t block = lmm::tpp_block_threads(lmm::Mode::Fused);
    const int64_t nscen = p->nscen;
    int64_t items = (2 * (int64_t)ds.sms * ds.bps + nscen - 1) / nscen;
    if (items * nscen > kMaxItems) items = kMaxItems / nscen;
    if (items < 1) items = 1;
    int64_t ppt = (paths + block * items - 1) / (block * items);
    items = (paths + block * ppt - 1) / (block * ppt);
    if (ppt > 0x7fffffff) return lmm::record_error(LMM_ERR_TOO_LARGE, "too many paths per thread");
    unsigned char *base = ds.scratch;
    NoallocModel *dmod = reinterpret_cast<NoallocModel *>(base);
    int *flag = reinterpret_cast<int *>(base + kModelBytes);
    double *partial = reinterpret_cast<double *>(base + kModelBytes + kFlagBytes);
    k_noalloc_upload<<<1, 256, 0, st>>>(hm, dmod, flag);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return lmm::record_cuda_error(ce, "model upload launch");

    lmm::DevModel m{};
    m.nn = kNN;
    m.nmat = kNMAT;
    m.nopt = p->nopt;
    m.nscen = p->nscen;
    m.delta = (float)d;
    m.sqd = (float)std::sqrt(d);
    m.d2 = (float)(d * d);
    m.deltad = d;
    m.sqdd = std::sqrt(d);
    m.kc = dmod->kc;
    m.kc_host = hm.kc;
    m.L0f = dmod->L0f;
    m.invL0f = dmod->iL0f;
    m.L0d = dmod->L0d;
    m.lamd = dmod->lamd;
    m.opt_start = dmod->ost;
    m.optKf = dmod->okf;
    m.optKd = dmod->okd;
    m.optWf = dmod->owf;
    m.optWd = dmod->owd;

    lmm::Work w{};
    w.paths = paths;
    w.items = (int)items;
    w.ppt = (int)ppt;
    w.partial = partial;
    w.nout = kNout;

    ce = lmm::launch_tpp_any(m, lmm::Mode::Fused, d_z, 0, 0, false, w, nullptr, nullptr, st);
    if (ce != cudaSuccess) return lmm::record_cuda_error(ce, "FP32 LMM kernel launch");
    ce = lmm::launch_finalize(partial, p->nscen, w.items, kNout, paths, d_out, d_se, flag, st);
    if (ce != cudaSuccess) return lmm::record_cuda_error(ce, "finalize launch");
    return LMM_OK;
}

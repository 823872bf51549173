// Auxiliary kernels: deterministic final reduction, bump differences, and
// the Philox4x32-10 + Box-Muller normal generators (FP32 and FP64 specs).
#include "lmm_device.cuh"

namespace lmm {
namespace {

constexpr int kFinX = 32, kFinY = 8;

// Block b covers scenario b / nchunk and outputs (b % nchunk)*32 .. +31;
// thread (x = output, y = item group): group y adds items y, y+8, ... in
// order, then group 0 adds the 8 group sums in order.
__global__ void __launch_bounds__(kFinX *kFinY)
k_finalize(const double *__restrict__ partial, int items, int nout, int64_t paths,
           double *__restrict__ mean, double *__restrict__ se, int *__restrict__ flag)
{
    __shared__ double s1[kFinY][kFinX], s2[kFinY][kFinX];
    const int nchunk = (nout + kFinX - 1) / kFinX;
    const int scen = blockIdx.x / nchunk;
    const int o = (blockIdx.x % nchunk) * kFinX + threadIdx.x;
    double a = 0.0, b = 0.0;
    if (o < nout) {
        for (int it = threadIdx.y; it < items; it += kFinY) {
            const double *p = partial + ((size_t)scen * items + it) * 2 * nout;
            a += p[o];
            b += p[nout + o];
        }
    }
    s1[threadIdx.y][threadIdx.x] = a;
    s2[threadIdx.y][threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.y == 0 && o < nout) {
        double sa = 0.0, sb = 0.0;
#pragma unroll
        for (int g = 0; g < kFinY; ++g) {
            sa += s1[g][threadIdx.x];
            sb += s2[g][threadIdx.x];
        }
        const double n = (double)paths;
        const double mu = sa / n;
        double var = paths > 1 ? (sb - sa * mu) / (n - 1.0) : 0.0;
        var = var > 0.0 ? var : 0.0;
        const double e = sqrt(var / n);
        mean[(size_t)scen * nout + o] = mu;
        if (se) se[(size_t)scen * nout + o] = e;
        if (!isfinite(mu) || !isfinite(e)) atomicOr(flag, 1);
    }
}

__global__ void k_bump_diff(double *mean, double *se, int nscen, int nout, double h)
{
    const int s = blockIdx.x;
    const double base = mean[(size_t)s * nout];
    __syncthreads();
    for (int j = 1 + threadIdx.x; j < nout; j += blockDim.x) {
        mean[(size_t)s * nout + j] = (mean[(size_t)s * nout + j] - base) / h;
        if (se) se[(size_t)s * nout + j] = 0.0;
    }
}

// Central differences from the 1+4nn variant means of one scenario
// (base, +h on each of the 2nn inputs, -h on each): out[0] = base,
// out[j] = (V(+h) - V(-h)) / 2h; se: the base's, 0 for the differences.
__global__ void k_bump_central(const double *mean, const double *se_in, double *out, double *se,
                               int nscen, int nn, double h)
{
    const int s = blockIdx.x;
    const int nb = 1 + 4 * nn, nout = 1 + 2 * nn;
    const double *m = mean + (size_t)s * nb;
    for (int j = threadIdx.x; j < nout; j += blockDim.x) {
        out[(size_t)s * nout + j] = j == 0 ? m[0] : (m[j] - m[2 * nn + j]) / (2.0 * h);
        if (se) se[(size_t)s * nout + j] = j == 0 ? se_in[(size_t)s * nb] : 0.0;
    }
}

// z64[i] = z32[i] (exact): the FP32 normals as FP64, for the FP64 kernel on
// the identical inputs.
__global__ void k_widen(const float *__restrict__ z32, double *__restrict__ z64, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z64[i] = (double)z32[i];
}

// err[i] = |a[i] - b[i]|
__global__ void k_abs_diff(const double *a, const double *b, double *err, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) err[i] = fabs(a[i] - b[i]);
}

__global__ void k_normals_f32(uint64_t seed, int64_t path0, int64_t paths, int nmat, float mean,
                              float sd, float *z)
{
    const int nq = (nmat + 3) >> 2;
    const int64_t tot = paths * nq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / nq;
        const int q = (int)(t - p * nq);
        float g[4];
        normals_quad_f32(seed, (uint64_t)(path0 + p), (uint32_t)q, g);
        float *zp = z + p * nmat;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int n = 4 * q + e;
            if (n < nmat) zp[n] = fmaf(sd, g[e], mean);
        }
    }
}

__global__ void k_normals_f64(uint64_t seed, int64_t path0, int64_t paths, int nmat, double mean,
                              double sd, double *z)
{
    const int nq = (nmat + 3) >> 2;
    const int64_t tot = paths * nq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / nq;
        const int q = (int)(t - p * nq);
        const U4 x = philox_quad(seed, (uint64_t)(path0 + p), (uint32_t)q);
        double g[4];
        box_muller_f64(x.x, x.y, g[0], g[1]);
        box_muller_f64(x.z, x.w, g[2], g[3]);
        double *zp = z + p * nmat;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int n = 4 * q + e;
            if (n < nmat) zp[n] = mean + sd * g[e];
        }
    }
}

// 16 independent dependency chains per thread keep the FMA pipe busy
// without depending on latency; the result goes to `sink` so nothing is
// eliminated.
__global__ void __launch_bounds__(256) k_ffma_peak(int iters, float a, float b, float *sink)
{
    float x[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = (float)(threadIdx.x + j) * 1e-3f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = fmaf(x[j], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 16; ++j) s += x[j];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 FMA throughput probe: 16 independent DFMA chains per thread.
__global__ void __launch_bounds__(256) k_dfma_peak(int iters, double a, double b, float *sink)
{
    double x[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = (double)(threadIdx.x + j) * 1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = fma(x[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 16; ++j) s += x[j];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = (float)s;
}

// MUFU throughput probe: 16 independent chains per thread of ex2 (KIND 0:
// x = 2^-x, which stays in (1/2, 1)), rcp (KIND 1: x = 1/(1+x), which tends
// to 0.618; x = 1/x would be folded away) or both alternately (KIND 2), so
// the special-function pipe, not latency, limits.
template <int KIND>
__global__ void __launch_bounds__(256) k_mufu_peak(int iters, float *sink)
{
    float x[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = 0.5f + (float)(threadIdx.x + j) * 1e-6f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            if (KIND == 0 || (KIND == 2 && (j & 1) == 0))
                x[j] = ex2_approx(-x[j]);
            else
                x[j] = rcp_approx(x[j] + 1.0f);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 16; ++j) s += x[j];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

unsigned grid_for(int64_t work, int block)
{
    int64_t g = (work + block - 1) / block;
    if (g > 152 * 64) g = 152 * 64;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t launch_finalize(const double *partial, int nscen, int items, int nout, int64_t paths,
                            double *mean, double *se, int *flag, cudaStream_t s)
{
    const int64_t blocks = (int64_t)nscen * ((nout + kFinX - 1) / kFinX);
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    dim3 block(kFinX, kFinY);
    k_finalize<<<(unsigned)blocks, block, 0, s>>>(partial, items, nout, paths, mean, se, flag);
    return cudaGetLastError();
}

cudaError_t launch_bump_central(const double *mean, const double *se_in, double *out, double *se, int nscen,
                                int nn, double h, cudaStream_t s)
{
    k_bump_central<<<nscen, 256, 0, s>>>(mean, se_in, out, se, nscen, nn, h);
    return cudaGetLastError();
}

cudaError_t launch_widen(const float *z32, double *z64, int64_t n, cudaStream_t s)
{
    k_widen<<<grid_for(n, 256), 256, 0, s>>>(z32, z64, n);
    return cudaGetLastError();
}

cudaError_t launch_abs_diff(const double *a, const double *b, double *err, int n, cudaStream_t s)
{
    k_abs_diff<<<(n + 255) / 256, 256, 0, s>>>(a, b, err, n);
    return cudaGetLastError();
}

cudaError_t launch_bump_diff(double *mean, double *se, int nscen, int nout, double h,
                             cudaStream_t s)
{
    k_bump_diff<<<nscen, 256, 0, s>>>(mean, se, nscen, nout, h);
    return cudaGetLastError();
}

cudaError_t launch_ffma_peak(int blocks, int iters, float a, float b, float *sink, cudaStream_t s)
{
    k_ffma_peak<<<blocks, 256, 0, s>>>(iters, a, b, sink);
    return cudaGetLastError();
}

cudaError_t launch_dfma_peak(int blocks, int iters, double a, double b, float *sink, cudaStream_t s)
{
    k_dfma_peak<<<blocks, 256, 0, s>>>(iters, a, b, sink);
    return cudaGetLastError();
}

cudaError_t launch_mufu_peak(int kind, int blocks, int iters, float *sink, cudaStream_t s)
{
    switch (kind) {
        case 0: k_mufu_peak<0><<<blocks, 256, 0, s>>>(iters, sink); break;
        case 1: k_mufu_peak<1><<<blocks, 256, 0, s>>>(iters, sink); break;
        case 2: k_mufu_peak<2><<<blocks, 256, 0, s>>>(iters, sink); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_normals_f32(uint64_t seed, int64_t path0, int64_t paths, int nmat, float mean,
                               float sd, float *z, cudaStream_t s)
{
    const int64_t work = paths * ((nmat + 3) / 4);
    k_normals_f32<<<grid_for(work, 256), 256, 0, s>>>(seed, path0, paths, nmat, mean, sd, z);
    return cudaGetLastError();
}

cudaError_t launch_normals_f64(uint64_t seed, int64_t path0, int64_t paths, int nmat, double mean,
                               double sd, double *z, cudaStream_t s)
{
    const int64_t work = paths * ((nmat + 3) / 4);
    k_normals_f64<<<grid_for(work, 256), 256, 0, s>>>(seed, path0, paths, nmat, mean, sd, z);
    return cudaGetLastError();
}

}  // namespace lmm

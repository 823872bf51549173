// MRG32k3a normal stream on the device: the generator family, stream order and
// inversion method of the reference's generateRand
// (LiborMarketModel/mklRng.cpp:44-110: one MRG32k3a stream, seed 12345,
// skip-ahead per thread, Gaussians by inverse CDF), restated from the
// published algorithms:
//   P. L'Ecuyer, Operations Research 47(1), 1999 (MRG32k3a: two order-3
//   recurrences mod m1 = 2^32-209 and m2 = 2^32-22853, combined
//   z = (x - y) mod m1 in [1, m1], u = z / (m1+1));
//   skip-ahead by powers of the 3x3 companion matrices;
//   M. J. Wichura, Applied Statistics 37(3), 1988, AS241: PPND16 (FP64
//   output) and PPND7 in FP32 arithmetic (FP32 output; its arguments
//   q = u - 1/2 and min(u, 1-u) are formed from the integer z, so the FP32
//   path has no FP64 operation).
// Seeding from one 32-bit seed s: x state (s mod m1, 1, 1), y state (1,1,1).
//
// Work layout. Each warp owns a chunk of 32*kSpan consecutive stream
// elements; lane l generates elements [l*kSpan, (l+1)*kSpan) of the chunk
// with the plain recurrence after two jumps: the warp's chunk start
// (A^(2^k) table, the same entries for every lane) and the lane's offset
// (A^(l*kSpan) table). Generated values go through a 32x33 shared-memory tile
// per warp so that each store instruction writes 32 consecutive elements.
//
// Arithmetic order: the central branch of the inversion and mean + sd*x use
// explicitly rounded multiplies and adds (no contraction), as the C
// restatement evaluates them, so those values are bit-identical to it; the
// tails go through log and may differ in the last bits.
#include <type_traits>

#include "lmm_internal.h"

namespace lmm {
namespace {

constexpr uint64_t kM1 = 4294967087ULL;
constexpr uint64_t kM2 = 4294944443ULL;
constexpr int kSpan = 512;        // elements per lane per chunk (multiple of 32)
constexpr int64_t kHalfM1p1 = 2147483544;            // (m1 + 1) / 2
constexpr float kNormF = (float)(1.0 / 4294967088.0); // 1 / (m1 + 1), rounded to FP32
constexpr int kWarps = 4;         // warps per block

__device__ __forceinline__ void jump(const uint32_t *m, uint64_t v[3], uint64_t mod)
{
    uint64_t r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        uint64_t s = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) s = (s + ((uint64_t)m[3 * i + k] * v[k]) % mod) % mod;
        r[i] = s;
    }
    v[0] = r[0];
    v[1] = r[1];
    v[2] = r[2];
}

// One step of both recurrences; returns z in [1, m1].
__device__ __forceinline__ uint32_t mrg_step(uint64_t x[3], uint64_t y[3])
{
    int64_t p1 = ((int64_t)(1403580ULL * x[1]) - (int64_t)(810728ULL * x[0])) % (int64_t)kM1;
    int64_t p2 = ((int64_t)(527612ULL * y[2]) - (int64_t)(1370589ULL * y[0])) % (int64_t)kM2;
    if (p1 < 0) p1 += (int64_t)kM1;
    if (p2 < 0) p2 += (int64_t)kM2;
    x[0] = x[1];
    x[1] = x[2];
    x[2] = (uint64_t)p1;
    y[0] = y[1];
    y[1] = y[2];
    y[2] = (uint64_t)p2;
    return (uint32_t)(p1 > p2 ? p1 - p2 : p1 - p2 + (int64_t)kM1);
}

__device__ __forceinline__ double horner_rn(const double (&c)[8], double x)
{
    double r = c[7];
#pragma unroll
    for (int i = 6; i >= 0; --i) r = __dadd_rn(__dmul_rn(r, x), c[i]);
    return r;
}

// AS241 PPND16.
__device__ double ppnd16(double p)
{
    const double a[8] = {3.3871328727963666080e0, 1.3314166789178437745e+2, 1.9715909503065514427e+3,
                         1.3731693765509461125e+4, 4.5921953931549871457e+4, 6.7265770927008700853e+4,
                         3.3430575583588128105e+4, 2.5090809287301226727e+3};
    const double b[8] = {1.0, 4.2313330701600911252e+1, 6.8718700749205790830e+2, 5.3941960214247511077e+3,
                         2.1213794301586595867e+4, 3.9307895800092710610e+4, 2.8729085735721942674e+4,
                         5.2264952788528545610e+3};
    const double c[8] = {1.42343711074968357734e0, 4.63033784615654529590e0, 5.76949722146069140550e0,
                         3.64784832476320460504e0, 1.27045825245236838258e0, 2.41780725177450611770e-1,
                         2.27238449892691845833e-2, 7.74545014278341407640e-4};
    const double d[8] = {1.0, 2.05319162663775882187e0, 1.67638483018380384940e0, 6.89767334985100004550e-1,
                         1.48103976427480074590e-1, 1.51986665636164571966e-2, 5.47593808499534494600e-4,
                         1.05075007164441684324e-9};
    const double e[8] = {6.65790464350110377720e0, 5.46378491116411436990e0, 1.78482653991729133580e0,
                         2.96560571828504891230e-1, 2.65321895265761230930e-2, 1.24266094738807843860e-3,
                         2.71155556874348757815e-5, 2.01033439929228813265e-7};
    const double f[8] = {1.0, 5.99832206555887937690e-1, 1.36929880922735805310e-1, 1.48753612908506148525e-2,
                         7.86869131145613259100e-4, 1.84631831751005468180e-5, 1.42151175831644588870e-7,
                         2.04426310338993978564e-15};
    const double q = __dadd_rn(p, -0.5);
    if (fabs(q) <= 0.425) {
        const double r = __dadd_rn(0.180625, -__dmul_rn(q, q));
        return __dmul_rn(q, horner_rn(a, r)) / horner_rn(b, r);
    }
    double r = q < 0.0 ? p : __dadd_rn(1.0, -p);
    r = sqrt(-log(r));
    double v;
    if (r <= 5.0) {
        r = __dadd_rn(r, -1.6);
        v = horner_rn(c, r) / horner_rn(d, r);
    } else {
        r = __dadd_rn(r, -5.0);
        v = horner_rn(e, r) / horner_rn(f, r);
    }
    return q < 0.0 ? -v : v;
}

__device__ __forceinline__ float mad_rn(float r, float x, float c) { return __fadd_rn(__fmul_rn(r, x), c); }

// AS241 PPND7 in FP32 from q = p - 1/2 and pt = min(p, 1-p).
__device__ float ppnd7(float q, float pt)
{
    if (fabsf(q) <= 0.425f) {
        const float r = __fadd_rn(0.180625f, -__fmul_rn(q, q));
        const float num = mad_rn(mad_rn(mad_rn(59.109374720f, r, 159.29113202f), r, 50.434271938f), r, 3.3871327179f);
        const float den = mad_rn(mad_rn(mad_rn(67.187563600f, r, 78.757757664f), r, 17.895169469f), r, 1.0f);
        return __fmul_rn(q, num) / den;
    }
    float r = sqrtf(-logf(pt));
    float v;
    if (r <= 5.0f) {
        r = __fadd_rn(r, -1.6f);
        v = mad_rn(mad_rn(mad_rn(0.17023821103f, r, 1.3067284816f), r, 2.7568153900f), r, 1.4234372777f) /
            mad_rn(mad_rn(0.12021132975f, r, 0.73700164250f), r, 1.0f);
    } else {
        r = __fadd_rn(r, -5.0f);
        v = mad_rn(mad_rn(mad_rn(0.017337203997f, r, 0.42868294337f), r, 3.0812263860f), r, 6.6579051150f) /
            mad_rn(mad_rn(0.012258202635f, r, 0.24197894225f), r, 1.0f);
    }
    return q < 0.0f ? -v : v;
}

template <int KIND>  // 0: uniforms (double), 1: normals (double), 2: normals (float)
__global__ void __launch_bounds__(32 * kWarps)
k_mrg32k3a(const MrgTables J, uint32_t seed, int64_t first, int64_t count, double mean, double sd, void *out)
{
    using T = typename std::conditional<KIND == 2, float, double>::type;
    __shared__ T tile[kWarps][32][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t chunk = ((int64_t)blockIdx.x * kWarps + w) * (32 * (int64_t)kSpan);
    if (chunk >= count) return;  // warp-uniform

    uint64_t x[3] = {seed % kM1, 1, 1}, y[3] = {1, 1, 1};
    const uint64_t e0 = (uint64_t)(first + chunk);
    for (int k = 0; k < 64; ++k) {
        if ((e0 >> k) & 1ULL) {  // the same k for every lane: broadcast reads
            jump(J.p1[k], x, kM1);
            jump(J.p2[k], y, kM2);
        }
    }
    jump(J.l1[lane], x, kM1);
    jump(J.l2[lane], y, kM2);

    T *o = static_cast<T *>(out);
    const float fmean = (float)mean, fsd = (float)sd;
    for (int t = 0; t < kSpan / 32; ++t) {
#pragma unroll 4
        for (int i = 0; i < 32; ++i) {
            const uint32_t z = mrg_step(x, y);
            if constexpr (KIND == 2) {
                // q = u - 1/2 and min(u, 1-u) from the integer z, in FP32 (no FP64)
                const float q = __fmul_rn(__int2float_rn((int32_t)((int64_t)z - kHalfM1p1)), kNormF);
                const uint32_t zt = min(z, (uint32_t)(2 * kHalfM1p1) - z);
                const float pt = __fmul_rn(__uint2float_rn(zt), kNormF);
                tile[w][lane][i] = __fadd_rn(fmean, __fmul_rn(fsd, ppnd7(q, pt)));
            } else {
                const double u = (double)z * (1.0 / 4294967088.0);
                if constexpr (KIND == 0)
                    tile[w][lane][i] = (T)u;
                else
                    tile[w][lane][i] = (T)__dadd_rn(mean, __dmul_rn(sd, ppnd16(u)));
            }
        }
        __syncwarp();
#pragma unroll 4
        for (int r = 0; r < 32; ++r) {
            const int64_t e = chunk + (int64_t)r * kSpan + t * 32 + lane;
            if (e < count) o[e] = tile[w][r][lane];
        }
        __syncwarp();
    }
}

// Host-side powers of the companion matrices.
struct Mat {
    uint64_t a[9];
};

Mat mat_mul(const Mat &x, const Mat &y, uint64_t m)
{
    Mat r{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            uint64_t s = 0;
            for (int k = 0; k < 3; ++k) s = (s + (x.a[3 * i + k] * y.a[3 * k + j]) % m) % m;
            r.a[3 * i + j] = s;
        }
    return r;
}

Mat mat_pow(Mat a, uint64_t e, uint64_t m)
{
    Mat r{{1, 0, 0, 0, 1, 0, 0, 0, 1}};
    while (e) {
        if (e & 1) r = mat_mul(r, a, m);
        a = mat_mul(a, a, m);
        e >>= 1;
    }
    return r;
}

void store(uint32_t dst[9], const Mat &m)
{
    for (int i = 0; i < 9; ++i) dst[i] = (uint32_t)m.a[i];
}

MrgTables make_tables()
{
    MrgTables t{};
    const Mat A1{{0, 1, 0, 0, 0, 1, kM1 - 810728ULL, 1403580ULL, 0}};
    const Mat A2{{0, 1, 0, 0, 0, 1, kM2 - 1370589ULL, 0, 527612ULL}};
    Mat p1 = A1, p2 = A2;
    for (int k = 0; k < 64; ++k) {
        store(t.p1[k], p1);
        store(t.p2[k], p2);
        p1 = mat_mul(p1, p1, kM1);
        p2 = mat_mul(p2, p2, kM2);
    }
    const Mat s1 = mat_pow(A1, kSpan, kM1), s2 = mat_pow(A2, kSpan, kM2);
    Mat l1{{1, 0, 0, 0, 1, 0, 0, 0, 1}}, l2 = l1;
    for (int l = 0; l < 32; ++l) {
        store(t.l1[l], l1);
        store(t.l2[l], l2);
        l1 = mat_mul(l1, s1, kM1);
        l2 = mat_mul(l2, s2, kM2);
    }
    return t;
}

}  // namespace

const MrgTables &mrg_tables()
{
    static const MrgTables t = make_tables();
    return t;
}

cudaError_t launch_mrg32k3a(int kind, uint32_t seed, int64_t first, int64_t count, double mean, double sd,
                            void *out, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    const int64_t per_block = (int64_t)kWarps * 32 * kSpan;
    const int64_t blocks = (count + per_block - 1) / per_block;
    if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
    const MrgTables &t = mrg_tables();
    const dim3 grid((unsigned)blocks), block(32 * kWarps);
    switch (kind) {
        case 0: k_mrg32k3a<0><<<grid, block, 0, s>>>(t, seed, first, count, mean, sd, out); break;
        case 1: k_mrg32k3a<1><<<grid, block, 0, s>>>(t, seed, first, count, mean, sd, out); break;
        case 2: k_mrg32k3a<2><<<grid, block, 0, s>>>(t, seed, first, count, mean, sd, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace lmm

// FP32 thread-per-path LMM kernels for the reference shape NN=80, NMAT=40.
//
// One CUDA thread carries one Monte Carlo path through
//   forward   path_calc_b1   (LiborMarketModel/liborSwaptionGreeks.cpp:34-82)
//   payoff    portfolio_b    (:120-211), adjoint aliasing of :178/:181 fixed
//   reverse   path_calc_b2   (:86-117) plus the vega adjoint (not in the reference)
// with the NN forward rates L[] and their log-adjoints Pb[] = L*dV/dL held in
// registers (the rate index is a compile-time register index; the step index
// is a runtime loop).
//
// The reverse sweep needs, at step n, the pre-step rates L_{n,i}. Instead of
// storing the NN x NMAT trajectory (9.5 KB per path) it runs the Euler step
// backwards: with V_i the inclusive drift sum of step n (saved per step in
// shared memory by the forward), L_{n,i} = L_{n+1,i} * 2^-(a_k (V_i + sqez) + c_k)
// and V_{i-1} = V_i - delta^2 lambda_k L_{n,i}/(1+delta L_{n,i}), descending in
// i, which is the order the adjoint needs. In terms of Pb the reference's
// update (:108-111) becomes
//   S  += lambda_k Pb_i                         (S is the reference's v1)
//   Pb_i += delta^2 lambda_k t r S,  t = L/(1+delta L), r = 1/(1+delta L)
// and the vega of cell (n,i), k = i-n-1, is
//   dV/dlambda_k += Pb_i (V_i + sqez - delta lambda_k) + delta^2 t S.
//
// Cross-path reduction: per warp, each lane sums one output column over the
// warp's 32 paths (shared-memory transpose), then adds into per-warp FP64
// accumulators; each block writes its FP64 partial sums, and lmm_aux.cu adds
// the partials in a fixed order, so results are bit-reproducible.
#include "lmm_device.cuh"

namespace lmm {
namespace {

constexpr int kTppBlock = 128;
constexpr int kTppMinBlocks = 3;

__host__ __device__ constexpr int align16(int x) { return (x + 15) & ~15; }

template <int NN, int NMAT, Mode MODE>
struct TppLayout {
    static constexpr int B = kTppBlock;
    static constexpr int NW = B / 32;
    static constexpr int M = NN - NMAT;
    static constexpr int NOUT = MODE == Mode::Fused ? 1 + 2 * NN : (MODE == Mode::Forward ? 1 : 2 * NN);
    static constexpr int kc = 0;                                    // float4[NN]
    static constexpr int kd = kc + 16 * NN;                         // float[NN]
    static constexpr int l0 = kd + 4 * NN;                          // float[NN]
    static constexpr int il0 = l0 + 4 * NN;                         // float[NN]
    static constexpr int ost = il0 + 4 * NN;                        // int[M+1]
    static constexpr int okf = align16(ost + 4 * (M + 1));          // float[kMaxNopt]
    static constexpr int okd = align16(okf + 4 * kMaxNopt);         // double[kMaxNopt]
    static constexpr int vg = align16(okd + 8 * kMaxNopt);          // float[NN][B]
    static constexpr int vg_bytes = MODE == Mode::Forward ? 0 : 4 * NN * B;
    static constexpr int vt = vg + vg_bytes;                        // float[NMAT][B]
    static constexpr int vt_bytes = MODE == Mode::Fused ? 4 * NMAT * B : 0;
    static constexpr int acc = align16(vt + vt_bytes);              // double[NW][2*NOUT]
    static constexpr int bytes = acc + 8 * NW * 2 * NOUT;
};

__device__ __forceinline__ float pick4(const float (&q)[4], int j)
{
    float r = q[0];
    r = j == 1 ? q[1] : r;
    r = j == 2 ? q[2] : r;
    r = j == 3 ? q[3] : r;
    return r;
}

// Portfolio value, portfolio_b :133-171 and :186-197. Reciprocals are the
// correctly rounded FP32 1/(1+delta L); the discount and annuity products,
// the annuity sum and the payoffs are FP64. Returns the discounted value;
// *disc_out, *b_out receive the discount factor and the last annuity factor,
// *mask_out which swaptions (in grouped order) paid.
template <int NN, int NMAT>
__device__ __forceinline__ double payoff_forward(const float (&L)[NN], float delta, const int *ost,
                                                 const double *oKd, double *disc_out,
                                                 double *b_out, unsigned long long *mask_out)
{
    constexpr int M = NN - NMAT;
    double disc = 1.0;
#pragma unroll
    for (int n = 0; n < NMAT; ++n) disc *= (double)__frcp_rn(fmaf(delta, L[n], 1.0f));
    double b = 1.0, s = 0.0, vs = 0.0;
    unsigned long long mask = 0ull;
    const double dd = (double)delta;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        b *= (double)__frcp_rn(fmaf(delta, L[NMAT + m], 1.0f));
        s = fma(dd, b, s);
        const int o1 = ost[m + 1];
        for (int o = ost[m]; o < o1; ++o) {
            const double sw = fma(oKd[o], s, b) - 1.0;
            if (sw < 0.0) {
                vs -= 100.0 * sw;
                mask |= 1ull << o;
            }
        }
    }
    *disc_out = disc;
    *b_out = b;
    *mask_out = mask;
    return disc * vs;
}

// Payoff adjoint, portfolio_b :173-184 (with the rate and its adjoint kept
// apart) and :199-209, seeded with vbar = dOut/dV. Writes the log-adjoints
// Pb[i] = L_i dOut/dL_i of the terminal rates.
template <int NN, int NMAT>
__device__ __forceinline__ void payoff_adjoint(const float (&L)[NN], float (&Pb)[NN], float vbar,
                                               double V, double disc, double bM,
                                               unsigned long long mask, float delta,
                                               const int *ost, const float *oKf)
{
    constexpr int M = NN - NMAT;
    const float scale = -vbar * (float)disc * delta;
    float Bm = (float)bM;      // B[m] of :139, rebuilt backwards: B[m-1] = B[m] (1 + delta L)
    float Sb = 0.0f, Bb = 0.0f;
#pragma unroll
    for (int m = M - 1; m >= 0; --m) {
        const float Ln = L[NMAT + m];
        const float den = fmaf(delta, Ln, 1.0f);
        const float r = __frcp_rn(den);
        const int o1 = ost[m + 1];
        for (int o = ost[m]; o < o1; ++o) {
            if ((mask >> o) & 1ull) {
                Sb -= 100.0f * oKf[o];
                Bb -= 100.0f;
            }
        }
        Bb = fmaf(delta, Sb, Bb);
        Pb[NMAT + m] = scale * Bb * Bm * (Ln * r);
        Bb *= r;
        Bm *= den;
    }
    const float vs = -vbar * (float)V * delta;
#pragma unroll
    for (int n = 0; n < NMAT; ++n) {
        const float Ln = L[n];
        Pb[n] = vs * (Ln * __frcp_rn(fmaf(delta, Ln, 1.0f)));
    }
}

// Column sums of a warp's 32 shared-memory columns: lane handles outputs
// k = lane, lane+32, ...; the (t+lane)&31 rotation keeps the 32 lanes on 32
// different banks. Adds sums and sums of squares into FP64 accumulators.
template <int NN, int B>
__device__ __forceinline__ void column_reduce(const float *vg, int warp, int lane, double *acc,
                                              int nout, int off)
{
    for (int k = lane; k < NN; k += 32) {
        const float *col = vg + k * B + warp * 32;
        float a = 0.0f, a2 = 0.0f;
#pragma unroll 8
        for (int t = 0; t < 32; ++t) {
            const float x = col[(t + lane) & 31];
            a += x;
            a2 = fmaf(x, x, a2);
        }
        acc[off + k] += (double)a;
        acc[nout + off + k] += (double)a2;
    }
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
__global__ void __launch_bounds__(kTppBlock, kTppMinBlocks)
k_tpp(const DevModel m, const float *__restrict__ z, uint64_t seed, int64_t path0, const Work w,
      float *__restrict__ tape, const double *__restrict__ vbar)
{
    using Lay = TppLayout<NN, NMAT, MODE>;
    constexpr int B = Lay::B, M = Lay::M, NOUT = Lay::NOUT;
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *kc_s = reinterpret_cast<float4 *>(smem + Lay::kc);
    float *kd_s = reinterpret_cast<float *>(smem + Lay::kd);
    float *l0_s = reinterpret_cast<float *>(smem + Lay::l0);
    float *il0_s = reinterpret_cast<float *>(smem + Lay::il0);
    int *ost_s = reinterpret_cast<int *>(smem + Lay::ost);
    float *okf_s = reinterpret_cast<float *>(smem + Lay::okf);
    double *okd_s = reinterpret_cast<double *>(smem + Lay::okd);
    float *vg_s = reinterpret_cast<float *>(smem + Lay::vg);
    float *vt_s = reinterpret_cast<float *>(smem + Lay::vt);
    double *acc_s = reinterpret_cast<double *>(smem + Lay::acc);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int scen = blockIdx.x / w.items, item = blockIdx.x % w.items;
    for (int i = tid; i < NN; i += B) {
        kc_s[i] = m.kc[i];
        kd_s[i] = m.kd[i];
        l0_s[i] = m.L0f[scen * NN + i];
        il0_s[i] = m.invL0f[scen * NN + i];
    }
    for (int i = tid; i <= M; i += B) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += B) {
        okf_s[i] = m.optKf[i];
        okd_s[i] = m.optKd[i];
    }
    double *acc = acc_s + warp * 2 * NOUT;
    for (int i = tid; i < Lay::NW * 2 * NOUT; i += B) acc_s[i] = 0.0;
    __syncthreads();

    const float delta = m.delta, sqd = m.sqd, d2 = m.d2;
    const int64_t total = (int64_t)m.nscen * w.paths;
    const int64_t ibase = (int64_t)item * w.ppt * B;
    const float vb = MODE == Mode::Backward ? (float)vbar[scen] : 1.0f;

    for (int j = 0; j < w.ppt; ++j) {
        const int64_t pl = ibase + (int64_t)j * B + tid;
        if (ibase + (int64_t)j * B >= w.paths) break;          // warp-uniform: whole batch past the end
        const bool active = pl < w.paths;
        const int64_t pc = active ? pl : w.paths - 1;
        const int64_t tp = (int64_t)scen * w.paths + pc;
        const float *zp = PHILOX ? nullptr : z + pc * NMAT;
        const uint64_t gpath = (uint64_t)(path0 + pc);

        float L[NN];
        float Pb[NN];
        float zq[4];
        double V = 0.0, disc = 1.0, bM = 1.0;
        unsigned long long mask = 0ull;

        if (MODE != Mode::Backward) {
#pragma unroll
            for (int i = 0; i < NN; ++i) L[i] = l0_s[i];
            for (int n = 0; n < NMAT; ++n) {
                float zn;
                if (PHILOX) {
                    if ((n & 3) == 0) normals_quad_f32(seed, gpath, (uint32_t)(n >> 2), zq);
                    zn = pick4(zq, n & 3);
                } else {
                    zn = __ldg(zp + n);
                }
                const float sqez = sqd * zn;
                float Vs = 0.0f;
#pragma unroll
                for (int i = 1; i < NN; ++i) {
                    if (i > n) {
                        const float4 k = kc_s[i - n - 1];
                        const float r = rcp_approx(fmaf(delta, L[i], 1.0f));
                        Vs = fmaf(k.z, L[i] * r, Vs);
                        L[i] *= ex2_approx(fmaf(k.x, Vs + sqez, k.y));
                    }
                }
                if (MODE == Mode::Fused)
                    vt_s[n * B + tid] = Vs;
                else if (active)
                    tape[(int64_t)(NN + n) * total + tp] = Vs;
            }
            if (MODE == Mode::Forward && active) {
#pragma unroll
                for (int i = 0; i < NN; ++i) tape[(int64_t)i * total + tp] = L[i];
            }
        } else {
#pragma unroll
            for (int i = 0; i < NN; ++i) L[i] = tape[(int64_t)i * total + tp];
        }

        V = payoff_forward<NN, NMAT>(L, delta, ost_s, okd_s, &disc, &bM, &mask);

        if (MODE != Mode::Forward) {
            payoff_adjoint<NN, NMAT>(L, Pb, vb, V, disc, bM, mask, delta, ost_s, okf_s);
#pragma unroll
            for (int k = 0; k < NN; ++k) vg_s[k * B + tid] = 0.0f;
            for (int n = NMAT - 1; n >= 0; --n) {
                float zn;
                if (PHILOX) {
                    if ((n & 3) == 3 || n == NMAT - 1) normals_quad_f32(seed, gpath, (uint32_t)(n >> 2), zq);
                    zn = pick4(zq, n & 3);
                } else {
                    zn = __ldg(zp + n);
                }
                const float sqez = sqd * zn;
                float Vs = MODE == Mode::Fused ? vt_s[n * B + tid] : tape[(int64_t)(NN + n) * total + tp];
                float S = 0.0f;
#pragma unroll
                for (int i = NN - 1; i >= 1; --i) {
                    if (i > n) {
                        const int kk = i - n - 1;
                        const float4 k = kc_s[kk];
                        const float y = Vs + sqez;
                        const float Ln = L[i] * ex2_approx(-fmaf(k.x, y, k.y));
                        const float r = rcp_approx(fmaf(delta, Ln, 1.0f));
                        const float t = Ln * r;
                        Vs = fmaf(-k.z, t, Vs);
                        const float pb = Pb[i];
                        S = fmaf(k.w, pb, S);
                        const float tS = t * S;
                        vg_s[kk * B + tid] += fmaf(pb, y - kd_s[kk], d2 * tS);
                        Pb[i] = fmaf(k.z * r, tS, pb);
                        L[i] = Ln;
                    }
                }
            }
        }

        // ---- cross-path reduction of this batch of B paths ----
        if (MODE != Mode::Backward) {
            const float v = active ? (float)V : 0.0f;
            const float s1 = warp_sum(v), s2 = warp_sum(v * v);
            if (lane == 0) {
                acc[0] += (double)s1;
                acc[NOUT] += (double)s2;
            }
        }
        if (MODE != Mode::Forward) {
            constexpr int voff = MODE == Mode::Fused ? 1 + NN : NN;
            constexpr int doff = MODE == Mode::Fused ? 1 : 0;
            if (!active) {
#pragma unroll
                for (int k = 0; k < NN; ++k) vg_s[k * B + tid] = 0.0f;
            }
            __syncwarp();
            column_reduce<NN, B>(vg_s, warp, lane, acc, NOUT, voff);
            __syncwarp();
#pragma unroll
            for (int i = 0; i < NN; ++i) vg_s[i * B + tid] = active ? Pb[i] * il0_s[i] : 0.0f;
            __syncwarp();
            column_reduce<NN, B>(vg_s, warp, lane, acc, NOUT, doff);
            __syncwarp();
        }
    }

    __syncthreads();
    for (int o = tid; o < 2 * NOUT; o += B) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < Lay::NW; ++q) s += acc_s[q * 2 * NOUT + o];
        w.partial[(size_t)blockIdx.x * 2 * NOUT + o] = s;
    }
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
cudaError_t launch_tpp(const DevModel &m, const float *z, uint64_t seed, int64_t path0,
                       const Work &w, float *tape, const double *vbar, cudaStream_t s)
{
    using Lay = TppLayout<NN, NMAT, MODE>;
    auto kern = k_tpp<NN, NMAT, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((int64_t)m.nscen * w.items);
    kern<<<grid, kTppBlock, Lay::bytes, s>>>(m, z, seed, path0, w, tape, vbar);
    return cudaGetLastError();
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
cudaError_t occ_tpp(int *blocks)
{
    using Lay = TppLayout<NN, NMAT, MODE>;
    auto kern = k_tpp<NN, NMAT, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, kTppBlock, Lay::bytes);
}

}  // namespace

bool f32_tpp_supports(int nn, int nmat) { return nn == 80 && nmat == 40; }

int tpp_block_threads() { return kTppBlock; }

#define LMM_TPP_DISPATCH(FN, ...)                                                            \
    do {                                                                                     \
        if (philox) {                                                                        \
            switch (mode) {                                                                  \
                case Mode::Fused: return FN<80, 40, true, Mode::Fused>(__VA_ARGS__);         \
                case Mode::Forward: return FN<80, 40, true, Mode::Forward>(__VA_ARGS__);     \
                case Mode::Backward: return FN<80, 40, true, Mode::Backward>(__VA_ARGS__);   \
            }                                                                                \
        } else {                                                                             \
            switch (mode) {                                                                  \
                case Mode::Fused: return FN<80, 40, false, Mode::Fused>(__VA_ARGS__);        \
                case Mode::Forward: return FN<80, 40, false, Mode::Forward>(__VA_ARGS__);    \
                case Mode::Backward: return FN<80, 40, false, Mode::Backward>(__VA_ARGS__);  \
            }                                                                                \
        }                                                                                    \
        return cudaErrorInvalidValue;                                                        \
    } while (0)

cudaError_t tpp_blocks_per_sm(Mode mode, bool philox, int *blocks)
{
    LMM_TPP_DISPATCH(occ_tpp, blocks);
}

cudaError_t launch_tpp_any(const DevModel &m, Mode mode, const float *z, uint64_t seed,
                           int64_t path0, bool philox, const Work &w, float *tape,
                           const double *vbar, cudaStream_t s)
{
    LMM_TPP_DISPATCH(launch_tpp, m, z, seed, path0, w, tape, vbar, s);
}

}  // namespace lmm

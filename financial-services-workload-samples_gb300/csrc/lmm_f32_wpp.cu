// FP32 warp-per-path LMM kernels: any NN <= 256 (long tenor, e.g. NN=160,
// NMAT=120).
//
// One warp carries one Monte Carlo path. Lane l holds the S consecutive rates
// i = S*l + s (s < S) in registers, so
//   - the drift sum of path_calc_b1 (LiborMarketModel/liborSwaptionGreeks.cpp:70),
//     an inclusive prefix sum over i, is a local prefix over the lane's slots
//     plus an exclusive warp scan of the lane totals (shuffles);
//   - the reverse running sum v1 of path_calc_b2 (:108), a suffix sum over i,
//     is the mirror image (local suffix + exclusive warp suffix scan).
// Reverse sweep without a stored trajectory: the forward saves, per step and
// lane, Y_top = V + sqrt(delta) z at the lane's top rate (one float per lane
// and step, in a per-warp device scratch that stays in L2), and the rates
// every ck steps (DevModel::ckpt, the engine's checkpoint interval; 0: none).
// The reverse restarts each step from Y_top and runs
// the Euler step backwards down the lane's own slots,
//   L_{n,i} = L_{n+1,i} 2^-(a_k Y_i + c_k),  Y_{i-1} = Y_i - delta^2 lambda_k t_i,
// so the serial chain is S cells long, not NN; at every ck-th step it
// replaces the rebuilt rates by the saved ones, so FP32 rounding of the
// reconstruction accumulates over at most ck steps. The adjoint in log form
// (Pb = L dV/dL) is
//   S'_i = delta^2 sum_{j>=i} lambda_k Pb_j,  Pb_i += lambda_k t r S'_i
//   dV/dlambda_k += Pb_i (Y_i - delta lambda_k) + t S'_i.
// The payoff (portfolio_b :120-211, aliasing fixed) runs with double-FP32
// products and sums (F2, lmm_device.cuh): the discount product is a warp
// product reduction, the annuity recursion runs on lane 0.
#include "lmm_device.cuh"

namespace lmm {
namespace {

constexpr int kWppBlock = 128;
constexpr int kWppWarps = kWppBlock / 32;
// 1: the constant and vega tables carry nmat zero/discard rows in front, so a
// cell's row is base - n without a clamp (3.8 KB more shared memory per
// block at 160/120, still 6 blocks per SM; 1.4% faster on GB300). 0: one
// head row and row max(base - n, 0).
#ifndef LMM_WPP_PAD
#define LMM_WPP_PAD 1
#endif

// Resident blocks the register budget is sized for: 6 (shared memory allows
// no more at NN=160); 5 for S=8, which spills at 6.
#ifdef LMM_WPP_MINB
__host__ __device__ constexpr int wpp_min_blocks(int) { return LMM_WPP_MINB; }
#else
__host__ __device__ constexpr int wpp_min_blocks(int S) { return S >= 8 ? 5 : 6; }
#endif

// Scratch per warp, in floats: Y_top per step and lane, then the rates at
// every ck-th step (ck = DevModel::ckpt; 0: none), [checkpoint][slot][lane].
__host__ __device__ constexpr size_t wpp_scratch_floats(int nmat, int S, int ck)
{
    return (size_t)32 * nmat + (ck > 0 ? (size_t)32 * S * ((nmat + ck - 1) / ck) : 0);
}

__host__ __device__ constexpr size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

// Shared-memory layout (bytes), shared by host and device.
struct WppLay {
    int nn, nmat, S, nout, M;
    size_t kc, l0, il0, ost, okf, owf, okk, warp0, per_warp, vg, lw, bw, acc, bytes;
};

// Rows in front of the tables: row k + head holds k; rows below head are zero
// (constants) or discarded (vegas).
__host__ __device__ constexpr int wpp_head(int nmat) { return LMM_WPP_PAD ? nmat : 1; }

__host__ __device__ inline WppLay wpp_layout(int nn, int nmat, int S, Mode mode = Mode::Fused)
{
    WppLay L{};
    L.nn = nn;
    L.nmat = nmat;
    L.S = S;
    L.M = nn - nmat;
    L.nout = mode == Mode::Fused ? 1 + 2 * nn : (mode == Mode::Forward ? 1 : 2 * nn);
    size_t o = 0;
    L.kc = o; o = al16(o + 16 * (size_t)(nn + wpp_head(nmat)));   // head zero rows, then constants of k
    L.l0 = o; o = al16(o + 4 * (size_t)nn);
    L.il0 = o; o = al16(o + 4 * (size_t)nn);
    L.ost = o; o = al16(o + 4 * (size_t)(L.M + 1));
    L.okf = o; o = al16(o + 4 * (size_t)kMaxNopt);
    L.owf = o; o = al16(o + 4 * (size_t)kMaxNopt);    // notional weights
    L.okk = o; o = al16(o + 8 * (size_t)kMaxNopt);    // F2 K delta
    L.warp0 = o;
    size_t w = 0;
    L.vg = w; w = al16(w + 4 * (size_t)(32 * S + wpp_head(nmat)));   // head rows discard, then vegas
    L.lw = w; w = al16(w + 4 * (size_t)32 * S);           // payoff staging [32*S]
    L.bw = w; w = al16(w + 4 * (size_t)32 * S);           // annuity factors B[m] [32*S]
    L.acc = w; w = al16(w + 8 * (size_t)2 * L.nout);      // FP64 sums [2*nout]
    L.per_warp = w;
    L.bytes = o + kWppWarps * w;
    return L;
}

// Exclusive warp scans. The exclusive value is the neighbour's inclusive
// value (one more shuffle), not inclusive - x: that subtraction cancels
// catastrophically when the lane's own term dominates the sum.
__device__ __forceinline__ float warp_excl_prefix(float x, int lane)
{
    float inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += y;
    }
    const float ex = __shfl_up_sync(0xffffffffu, inc, 1);
    return lane == 0 ? 0.0f : ex;
}

__device__ __forceinline__ float warp_excl_suffix(float x, int lane)
{
    float inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float y = __shfl_down_sync(0xffffffffu, inc, d);
        if (lane + d < 32) inc += y;
    }
    const float ex = __shfl_down_sync(0xffffffffu, inc, 1);
    return lane == 31 ? 0.0f : ex;
}

// Constants and vega row of slot s at step n. The tables hold k at row
// k + head; the rows below head are zero (constants) or discarded (vegas).
// base[s] = i + head - 1 for a real rate i < nn, so row base - n belongs to
// k = i-n-1 (a rate not yet moving, k < 0, lands below head), and head - 1
// for a padding slot (i >= nn), which stays below head for every step. With
// head = nmat no clamp is needed; with head = 1 the row is clamped at 0. A
// zero row makes the cell an exact no-op: L *= 2^0, the sums gain 0 and Pb
// keeps its value, so the steps need no per-slot branches.
template <int S>
__device__ __forceinline__ int wpp_row(const int (&base)[S], int s, int n)
{
    return LMM_WPP_PAD ? base[s] - n : max(base[s] - n, 0);
}

// One forward step n over the lane's slots; returns Y at the lane's top slot
// (its drift sum plus sqrt(delta) z), from which the reverse restarts.
template <int S>
__device__ __forceinline__ float wpp_fwd_step(float (&L)[S], const int (&base)[S], int n, float sqez,
                                              int lane, const float4 *kc, float delta)
{
    float a[S];
    float4 kk[S];
    float P = 0.0f;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        kk[s] = kc[wpp_row(base, s, n)];
        const float r = rcp_approx(fmaf(delta, L[s], 1.0f));
        P = fmaf(kk[s].z, L[s] * r, P);
        a[s] = P;                                   // local inclusive prefix
    }
    const float X = warp_excl_prefix(P, lane) + sqez;
#pragma unroll
    for (int s = 0; s < S; ++s) L[s] *= ex2_approx(fmaf(kk[s].x, X + a[s], kk[s].y));
    return X + a[S - 1];
}

// Reverse step n (path_calc_b2 :100-112 in log-adjoint form) + vega: L holds
// L_{n+1} on entry and L_n on exit; ytop is the forward's Y at the lane's top
// slot. The suffix sum, taken over the log-adjoints before the step's update,
// is carried as S' = delta^2 S (sums of delta^2 lambda_k Pb), so that
// Pb += lambda_k r t S' and the vega term t S' need no further factor.
template <int S>
__device__ __forceinline__ void wpp_rev_step(float (&L)[S], float (&Pb)[S], const int (&base)[S], int n,
                                             int lane, float ytop, const float4 *kc, float *vg, float delta)
{
    float b[S];
    float4 kk[S];
    float Q = 0.0f;
#pragma unroll
    for (int s = S - 1; s >= 0; --s) {
        kk[s] = kc[wpp_row(base, s, n)];
        Q = fmaf(kk[s].z, Pb[s], Q);
        b[s] = Q;                                   // local inclusive suffix
    }
    const float Yx = warp_excl_suffix(Q, lane);
    float Y = ytop;
#pragma unroll
    for (int s = S - 1; s >= 0; --s) {
        const float Ln = L[s] * ex2_approx(-fmaf(kk[s].x, Y, kk[s].y));
        const float r = rcp_approx(fmaf(delta, Ln, 1.0f));
        const float t = Ln * r;
        const float tS = t * (Yx + b[s]);
        vg[wpp_row(base, s, n)] += fmaf(Pb[s], fmaf(-delta, kk[s].w, Y), tS);
        Pb[s] = fmaf(kk[s].w * r, tS, Pb[s]);
        L[s] = Ln;
        Y = fmaf(-kk[s].z, t, Y);
    }
    // The next step's vega rows overlap neighbouring lanes' rows of this
    // step: order the shared-memory read-modify-writes across the warp.
    __syncwarp();
}

template <bool PHILOX>
struct ZChunk {
    // Normals of steps 32q..32q+31 of one path spread over the warp: lane l
    // holds step 32q+l (memory) or steps 32q+4l..+3 (Philox, lanes < 8).
    float v[4];
    int q = -1;
    __device__ __forceinline__ void load(int qq, const float *zp, int nmat, uint64_t seed,
                                         uint64_t gpath, int lane)
    {
        q = qq;
        if (PHILOX) {
            const int quad = 8 * qq + lane;
            if (lane < 8 && 4 * quad < nmat) normals_quad_f32(seed, gpath, (uint32_t)quad, v);
        } else {
            const int n = 32 * qq + lane;
            v[0] = n < nmat ? __ldg(zp + n) : 0.0f;
        }
    }
    __device__ __forceinline__ float get(int n, const float *zp, int nmat, uint64_t seed,
                                         uint64_t gpath, int lane)
    {
        if ((n >> 5) != q) load(n >> 5, zp, nmat, seed, gpath, lane);
        if (PHILOX) {
            const int j = n & 3;
            float x = v[0];
            x = j == 1 ? v[1] : x;
            x = j == 2 ? v[2] : x;
            x = j == 3 ? v[3] : x;
            return __shfl_sync(0xffffffffu, x, (n & 31) >> 2);
        }
        return __shfl_sync(0xffffffffu, v[0], n & 31);
    }
};

// MODE: Fused (value + all Greeks), Forward (value only) or Backward (Greeks
// of vbar[scen] x value; the forward is recomputed from the same normals, so
// no tape is needed). ytop: gridDim.x * kWppWarps blocks of
// wpp_scratch_floats(nmat, S, m.ckpt) floats of scratch, one per resident warp
// (unused in Forward mode).
template <int S, bool PHILOX, Mode MODE>
__global__ void __launch_bounds__(kWppBlock, wpp_min_blocks(S))
k_wpp(const DevModel m, const float *__restrict__ z, uint64_t seed, int64_t path0, const Work w,
      const double *__restrict__ vbar, float *__restrict__ ytop)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int nn = m.nn, nmat = m.nmat;
    const WppLay Ly = wpp_layout(nn, nmat, S, MODE);
    const int M = Ly.M, nout = Ly.nout;
    float4 *kc_s = reinterpret_cast<float4 *>(smem + Ly.kc);
    float *l0_s = reinterpret_cast<float *>(smem + Ly.l0);
    float *il0_s = reinterpret_cast<float *>(smem + Ly.il0);
    int *ost_s = reinterpret_cast<int *>(smem + Ly.ost);
    float *okf_s = reinterpret_cast<float *>(smem + Ly.okf);
    float *owf_s = reinterpret_cast<float *>(smem + Ly.owf);
    F2 *okk_s = reinterpret_cast<F2 *>(smem + Ly.okk);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned char *wbase = smem + Ly.warp0 + warp * Ly.per_warp;
    const int ckn = m.ckpt;                 // the reverse restores the exact rates every ckn steps (0: never)
    float *yt = ytop + ((size_t)blockIdx.x * kWppWarps + warp) * wpp_scratch_floats(nmat, S, ckn) + lane;
    float *ck = yt + (size_t)32 * nmat;     // ck[(c*S + s)*32]: rate of slot s at step c*ckn
    float *vg_s = reinterpret_cast<float *>(wbase + Ly.vg);
    float *lw_s = reinterpret_cast<float *>(wbase + Ly.lw);
    float *bw_s = reinterpret_cast<float *>(wbase + Ly.bw);
    double *acc = reinterpret_cast<double *>(wbase + Ly.acc);

    const int head = wpp_head(nmat);
    for (int i = tid; i < nn + head; i += kWppBlock)
        kc_s[i] = i < head ? make_float4(0.f, 0.f, 0.f, 0.f) : m.kc[i - head];
    for (int i = tid; i <= M; i += kWppBlock) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += kWppBlock) {
        okf_s[i] = m.optKf[i];
        owf_s[i] = m.optWf[i];
        okk_s[i] = f2_from(m.optKd[i] * m.deltad);
    }
    for (int i = lane; i < 32 * S + head; i += 32) vg_s[i] = 0.0f;

    int base[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int i = S * lane + s;
        base[s] = i < nn ? i + head - 1 : head - 1;   // row of k = i-n-1 is base - n
    }
    const float delta = m.delta, sqd = m.sqd;

    // Units (scenario, item) in a block-stride loop over a grid of one wave
    // (blocks start together and stay on the same code).
    const int units = m.nscen * w.items;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int scen = unit / w.items, item = unit % w.items;
        __syncthreads();          // the previous unit's reads of l0/il0 are done
        for (int i = tid; i < nn; i += kWppBlock) {
            l0_s[i] = m.L0f[scen * nn + i];
            il0_s[i] = m.invL0f[scen * nn + i];
        }
        for (int i = lane; i < 2 * nout; i += 32) acc[i] = 0.0;
        __syncthreads();

        const float vb = MODE == Mode::Backward ? (float)vbar[scen] : 1.0f;
        const int64_t ibase = (int64_t)item * w.ppt * kWppWarps;
        for (int j = 0; j < w.ppt; ++j) {
            const int64_t p = ibase + (int64_t)j * kWppWarps + warp;
            if (p >= w.paths) break;                                  // warp-uniform
            const float *zp = PHILOX ? nullptr : z + p * nmat;
            const uint64_t gpath = (uint64_t)(path0 + p);
            ZChunk<PHILOX> zc;

            float L[S], Pb[S];
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const int i = S * lane + s;
                L[s] = i < nn ? l0_s[i] : 1.0f;
            }
            // ---- forward ----
            for (int n = 0; n < nmat; ++n) {
                if (MODE != Mode::Forward && ckn > 0 && n % ckn == 0) {
#pragma unroll
                    for (int s = 0; s < S; ++s) ck[((n / ckn) * S + s) * 32] = L[s];
                }
                const float sqez = sqd * zc.get(n, zp, nmat, seed, gpath, lane);
                const float y = wpp_fwd_step<S>(L, base, n, sqez, lane, kc_s, delta);
                if (MODE != Mode::Forward) yt[n * 32] = y;
            }
            // ---- payoff (double-FP32 products) and its adjoint ----
            F2 dprod{1.0f, 0.0f};
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const int i = S * lane + s;
                if (i < nmat) dprod = f2_mul(dprod, __frcp_rn(fmaf(delta, L[s], 1.0f)));
                if (i < nn) lw_s[i] = L[s];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const F2 other{__shfl_xor_sync(0xffffffffu, dprod.hi, o), __shfl_xor_sync(0xffffffffu, dprod.lo, o)};
                dprod = f2_mul(dprod, other);
            }
            const float disc = dprod.hi;
            __syncwarp();
            float V = 0.0f;
            if (lane == 0) {
                F2 bb{1.0f, 0.0f}, sb{0.0f, 0.0f}, vs{0.0f, 0.0f};
                unsigned long long mask = 0ull;
                for (int mm = 0; mm < M; ++mm) {
                    bb = f2_mul(bb, __frcp_rn(fmaf(delta, lw_s[nmat + mm], 1.0f)));
                    sb = f2_add(sb, bb);                      // annuity / delta
                    bw_s[mm] = bb.hi;
                    for (int o = ost_s[mm]; o < ost_s[mm + 1]; ++o) {
                        const float sw = f2_swap_value(okk_s[o], sb, bb);
                        if (sw < 0.0f) {
                            vs = f2_add(vs, (-100.0f * sw) * owf_s[o]);
                            mask |= 1ull << o;
                        }
                    }
                }
                const F2 v = f2_mul(vs, dprod);
                V = __fadd_rn(v.hi, v.lo);
                if (MODE == Mode::Forward) mask = 0ull;     // no adjoint
                // :173-184 with the rate kept apart from its adjoint; lw_s[i] becomes
                // the log-adjoint of rate i >= nmat. B[m] comes from the forward
                // (bw_s): rebuilding it backwards from the last, smallest factor
                // would underflow FP32 on paths whose rates grow large.
                const float scale = -vb * disc * delta;
                float Sb = 0.0f, Bb = 0.0f;
                for (int mm = M - 1; mm >= 0; --mm) {
                    const float Ln = lw_s[nmat + mm];
                    const float r = __frcp_rn(fmaf(delta, Ln, 1.0f));
                    const float Bm = bw_s[mm];
                    for (int o = ost_s[mm]; o < ost_s[mm + 1]; ++o) {
                        if ((mask >> o) & 1ull) {
                            Sb -= (100.0f * okf_s[o]) * owf_s[o];
                            Bb -= 100.0f * owf_s[o];
                        }
                    }
                    Bb = fmaf(delta, Sb, Bb);
                    lw_s[nmat + mm] = scale * Bb * Bm * (Ln * r);
                    Bb *= r;
                }
            }
            V = __shfl_sync(0xffffffffu, V, 0);
            __syncwarp();
            if (MODE == Mode::Forward) {
                if (lane == 0) {
                    acc[0] += (double)V;
                    acc[nout] += (double)V * V;
                }
                continue;
            }
            const float vsd = -vb * V * delta;
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const int i = S * lane + s;
                if (i < nmat) Pb[s] = vsd * (L[s] * __frcp_rn(fmaf(delta, L[s], 1.0f)));
                else Pb[s] = i < nn ? lw_s[i] : 0.0f;
            }
            // ---- reverse: each step rebuilt from the forward's Y_top ----
            float ynext = yt[(nmat - 1) * 32];
            for (int n = nmat - 1; n >= 0; --n) {
                const float y = ynext;
                if (n > 0) ynext = yt[(n - 1) * 32];
                wpp_rev_step<S>(L, Pb, base, n, lane, y, kc_s, vg_s, delta);
                if (ckn > 0 && n % ckn == 0) {
#pragma unroll
                    for (int s = 0; s < S; ++s) L[s] = ck[((n / ckn) * S + s) * 32];
                }
            }
            // ---- accumulate this path: value, deltas, vegas ----
            __syncwarp();
            constexpr int doff = MODE == Mode::Fused ? 1 : 0;   // deltas at doff, vegas at doff + nn
            if (MODE == Mode::Fused && lane == 0) {
                acc[0] += (double)V;
                acc[nout] += (double)V * V;
            }
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const int i = S * lane + s;
                if (i < nn) {
                    const double dl = (double)(Pb[s] * il0_s[i]);
                    acc[doff + i] += dl;
                    acc[nout + doff + i] += dl * dl;
                }
            }
            for (int k = lane; k < nn; k += 32) {
                const double vgk = (double)vg_s[k + head];
                acc[doff + nn + k] += vgk;
                acc[nout + doff + nn + k] += vgk * vgk;
                vg_s[k + head] = 0.0f;
            }
            __syncwarp();
        }
        __syncthreads();
        for (int o = tid; o < 2 * nout; o += kWppBlock) {
            double s = 0.0;
            for (int q = 0; q < kWppWarps; ++q)
                s += reinterpret_cast<const double *>(smem + Ly.warp0 + q * Ly.per_warp + Ly.acc)[o];
            w.partial[(size_t)unit * 2 * nout + o] = s;
        }
    }  // units
}

template <int S, bool PHILOX, Mode MODE>
cudaError_t wpp_launch_s(const DevModel &m, const float *z, uint64_t seed, int64_t path0, const Work &w,
                         const double *vbar, float *ytop, cudaStream_t st)
{
    const int bytes = (int)wpp_layout(m.nn, m.nmat, S, MODE).bytes;
    auto kern = k_wpp<S, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)(w.grid > 0 ? w.grid : (int64_t)m.nscen * w.items);
    kern<<<grid, kWppBlock, bytes, st>>>(m, z, seed, path0, w, vbar, ytop);
    return cudaGetLastError();
}

template <int S, bool PHILOX, Mode MODE>
cudaError_t wpp_occ_s(int nn, int nmat, int *blocks)
{
    const int bytes = (int)wpp_layout(nn, nmat, S, MODE).bytes;
    auto kern = k_wpp<S, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, kWppBlock, bytes);
}

// The instantiated variants: Fused with normals from memory or Philox;
// Forward and Backward (the ABI pair) with normals from memory.
template <int S>
cudaError_t wpp_dispatch_launch(const DevModel &m, Mode mode, bool philox, const float *z, uint64_t seed,
                                int64_t path0, const Work &w, const double *vbar, float *ytop,
                                cudaStream_t st)
{
    if (mode == Mode::Fused)
        return philox ? wpp_launch_s<S, true, Mode::Fused>(m, z, seed, path0, w, vbar, ytop, st)
                      : wpp_launch_s<S, false, Mode::Fused>(m, z, seed, path0, w, vbar, ytop, st);
    if (philox) return cudaErrorNotSupported;
    return mode == Mode::Forward ? wpp_launch_s<S, false, Mode::Forward>(m, z, seed, path0, w, vbar, ytop, st)
                                 : wpp_launch_s<S, false, Mode::Backward>(m, z, seed, path0, w, vbar, ytop, st);
}

template <int S>
cudaError_t wpp_dispatch_occ(int nn, int nmat, Mode mode, bool philox, int *blocks)
{
    if (mode == Mode::Fused)
        return philox ? wpp_occ_s<S, true, Mode::Fused>(nn, nmat, blocks)
                      : wpp_occ_s<S, false, Mode::Fused>(nn, nmat, blocks);
    if (philox) return cudaErrorNotSupported;
    return mode == Mode::Forward ? wpp_occ_s<S, false, Mode::Forward>(nn, nmat, blocks)
                                 : wpp_occ_s<S, false, Mode::Backward>(nn, nmat, blocks);
}

}  // namespace

// Slots per lane for a shape: the smallest instantiated S with 32*S >= nn.
int wpp_slots(int nn)
{
    if (nn <= 64) return 2;
    if (nn <= 96) return 3;
    if (nn <= 160) return 5;
    if (nn <= 256) return 8;
    return 0;
}

size_t wpp_scratch_floats_per_warp(int nn, int nmat, int ckpt)
{
    return wpp_scratch_floats(nmat, wpp_slots(nn), ckpt);
}

bool f32_wpp_supports(int nn, int nmat)
{
    return nn >= 2 && nn <= kMaxNN && nmat >= 1 && nmat < nn && wpp_slots(nn) > 0 &&
           wpp_layout(nn, nmat, wpp_slots(nn)).bytes <= 227 * 1024;
}

int wpp_block_threads() { return kWppBlock; }

cudaError_t wpp_blocks_per_sm(int nn, int nmat, Mode mode, bool philox, int *blocks)
{
    *blocks = 0;
    if (!f32_wpp_supports(nn, nmat)) return cudaErrorNotSupported;
    switch (wpp_slots(nn)) {
        case 2: return wpp_dispatch_occ<2>(nn, nmat, mode, philox, blocks);
        case 3: return wpp_dispatch_occ<3>(nn, nmat, mode, philox, blocks);
        case 5: return wpp_dispatch_occ<5>(nn, nmat, mode, philox, blocks);
        case 8: return wpp_dispatch_occ<8>(nn, nmat, mode, philox, blocks);
    }
    return cudaErrorNotSupported;
}

cudaError_t launch_wpp_any(const DevModel &m, Mode mode, const float *z, uint64_t seed,
                           int64_t path0, bool philox, const Work &w, float *ytop, const double *vbar,
                           cudaStream_t s)
{
    if (!f32_wpp_supports(m.nn, m.nmat)) return cudaErrorNotSupported;
    if (mode != Mode::Forward && !ytop) return cudaErrorInvalidValue;
    switch (wpp_slots(m.nn)) {
        case 2: return wpp_dispatch_launch<2>(m, mode, philox, z, seed, path0, w, vbar, ytop, s);
        case 3: return wpp_dispatch_launch<3>(m, mode, philox, z, seed, path0, w, vbar, ytop, s);
        case 5: return wpp_dispatch_launch<5>(m, mode, philox, z, seed, path0, w, vbar, ytop, s);
        case 8: return wpp_dispatch_launch<8>(m, mode, philox, z, seed, path0, w, vbar, ytop, s);
    }
    return cudaErrorNotSupported;
}

}  // namespace lmm

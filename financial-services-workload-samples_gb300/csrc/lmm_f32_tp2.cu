// FP32 LMM value + Greeks with two threads per path (a thread pair), for
// NN=160, NMAT=120 (H = 80 rates per thread; the code takes any NN = 2H with
// NMAT >= H).
//
// The same Euler cells, payoff and adjoint as the thread-per-path kernel
// (lmm_f32_tpp.cu; reference LiborMarketModel/liborSwaptionGreeks.cpp
// path_calc_b1 :34-82, portfolio_b :120-211 with the :178/:181 aliasing
// fixed, path_calc_b2 :86-117, plus the vega adjoint), with the rates of a
// path split between the two warps 2q, 2q+1 of a block: one holds rates
// 0..H-1 of 32 paths ("lower"), the other rates H..NN-1 of the same 32 paths
// ("upper"). A thread keeps H inverse rates and H log-adjoints in registers,
// so NN=160 runs with the per-thread footprint that NN=80 has in the
// thread-per-path kernel.
//
// The drift sum of a step runs upwards over i, the adjoint's suffix sum and
// the drift reconstruction downwards, so the halves work in rounds, one
// barrier per round, each round one pair of steps:
//   forward   round r: lower takes steps 2r, 2r+1 and leaves the drift sums
//             at rate H-1; upper takes steps 2r-2, 2r-1 from those sums;
//   reverse   round r: upper takes steps NMAT-1-2r, NMAT-2-2r from the
//             saved full drift sums and leaves the adjoint's suffix sums at
//             rate H; lower takes the previous round's steps from those and
//             from the drift sums at rate H-1 that its forward saved, so each
//             half rebuilds the drift over its own H rates only.
// In a reverse round the upper half adds vega rows k >= H-n-1 and the lower
// half rows k <= H-n-3 (n the upper half's first step), so the two never
// touch the same row in one round. The payoff splits too: the lower half
// forms its discount factors, the upper half the rest of the discount, the
// annuities, the swaptions and their adjoint, and passes the value back for
// the lower half's discount adjoints.
//
// Within a thread the cells are those of the thread-per-path kernel: the
// forward pairs steps n, n+1 (cell (n,p) beside cell (n+1,p-1)); the reverse
// pairs steps n, n-1 as a skewed wavefront with constants and vega partial
// sums in register rings; branch-free triangles through NMAT zero constant
// rows; drift sums carry the normal term (Y = V + sqrt(delta) z).
#include "lmm_device.cuh"

namespace lmm {
namespace {

constexpr int kTp2Chunk = 8;       // rates per chunk of the step bodies
constexpr int kTp2Pref = 2;        // constants loaded this many positions ahead
// The fused kernel saves each half's rates every ck = DevModel::ckpt steps
// (0: never; ck even, so that checkpoints fall between step pairs) and the
// reverse sweep takes them in place of its rebuilt rates there, so FP32
// rounding of the backward Euler steps accumulates over at most ck steps.
// Rate checkpoints of a fused launch: at times ck, 2 ck, ... < nmat.
__host__ __device__ constexpr int tp2_nckpt(int nmat, int ck) { return ck > 0 ? (nmat - 1) / ck : 0; }

// Warps per block (8: one block per SM; 4: two blocks per SM), and whether
// warps w and w+4, which share a scheduler, take opposite halves (1) or the
// same half (0). GB300, 160/120, 1,048,576 paths: 8 warps alternating 19.4 ms,
// 8 warps not alternating 21.0 ms, two blocks of 4 warps 21.1-22.0 ms.
#ifndef LMM_TP2_WARPS160
#define LMM_TP2_WARPS160 8
#endif
#ifndef LMM_TP2_SWIZZLE
#define LMM_TP2_SWIZZLE 1
#endif

template <int NN>
struct Tp2Shape {
    // Threads per block and resident blocks the registers are sized for:
    // 80+80 floats per thread, one block of 8 warps (4 thread pairs) per SM.
    static constexpr int kBlock = 32 * LMM_TP2_WARPS160;
    static constexpr int kMinBlocks = 8 / LMM_TP2_WARPS160;
};

__host__ __device__ constexpr int al16(int x) { return (x + 15) & ~15; }

template <int NN, int NMAT, Mode MODE>
struct Tp2Layout {
    static constexpr int H = NN / 2;
    static constexpr int B = Tp2Shape<NN>::kBlock;
    static constexpr int NP = B / 64;                  // thread pairs per block
    static constexpr int PB = 32 * NP;                 // paths per batch
    static constexpr int M = NN - NMAT;
    static constexpr int PADK = NMAT;                  // zero constant rows in front
    static constexpr int VPAD = 16;                    // spare vega rows in front (k >= -9 is used)
    static constexpr int NOUT = MODE == Mode::Fused ? 1 + 2 * NN : (MODE == Mode::Forward ? 1 : 2 * NN);
    static constexpr int kc = 0;                                     // float4[PADK+NN]
    static constexpr int il0 = al16(kc + 16 * (PADK + NN));          // float[NN]
    static constexpr int ost = al16(il0 + 4 * NN);                   // int[M+1]
    static constexpr int okf = al16(ost + 4 * (M + 1));              // float[kMaxNopt]
    static constexpr int owf = al16(okf + 4 * kMaxNopt);             // float[kMaxNopt]
    static constexpr int okk = al16(owf + 4 * kMaxNopt);             // F2[kMaxNopt]: K delta
    static constexpr int vt = al16(okk + 8 * kMaxNopt);              // float[NMAT][PB] full drift sums
    static constexpr int vg = vt + 4 * NMAT * PB;                    // float[VPAD+NN][PB] vega rows
    static constexpr int hf = vg + 4 * (VPAD + NN) * PB;             // float[2][2][PB] forward hand-over
    static constexpr int hr = hf + 4 * 4 * PB;                       // float[2][4][PB] reverse hand-over (suffix sums)
    static constexpr int pd = hr + 4 * 8 * PB;                       // float[3][PB] payoff exchange
    static constexpr int acc = al16(pd + 4 * 3 * PB);                // double[NP][2*NOUT]
    static constexpr int bytes = acc + 8 * NP * 2 * NOUT;
};

// Forward cell on the inverse rate X = 1/L (path_calc_b1 :66-72), with the
// drift sum Y carrying the normal term: t = 1/(X + delta); Y += delta^2
// lambda_k t; X *= 2^-(lambda_k log2(e) Y - delta lambda_k^2 log2(e)/2).
__device__ __forceinline__ void tp2_fwd_cell(float &X, float &Y, const float4 &k, float delta)
{
    Y = fmaf(k.z, rcp_approx(X + delta), Y);
    X *= ex2_approx(-fmaf(k.x, Y, k.y));
}

// Steps n and n+1 over a thread's H rates (local p, global rate base + p):
// cell (n, p) and cell (n+1, p-1) at position p; kcn[j] holds the constants
// of step n at local rate j, which are those of step n+1 at local rate j+1.
// Entered at chunk c0 (c0 * CH < H), which holds step n's first active rate
// (or 0); the cells of either step below its first active rate see zero
// constants and are exact no-ops.
template <int H, int CH, int P>
__device__ __forceinline__ void tp2_fwd_pair(float (&X)[H], const float4 *kcn, int c0, float delta,
                                             float &Y0, float &Y1)
{
    constexpr int R = 3 + P;
    float4 C[R];
#pragma unroll
    for (int c = 0; c * CH < H; ++c) {
        if (c >= c0) {
            if (c == c0) {
#pragma unroll
                for (int j = c * CH - 2; j < c * CH + P; ++j)
                    if (j < H) C[(j + R) % R] = kcn[j];
            }
#pragma unroll
            for (int p = c * CH; p < (c + 1) * CH && p < H; ++p) {
                if (p + P < H) C[(p + P) % R] = kcn[p + P];
                tp2_fwd_cell(X[p], Y0, C[p % R], delta);
                if (p >= 1) tp2_fwd_cell(X[p - 1], Y1, C[(p + R - 2) % R], delta);
            }
        }
    }
    tp2_fwd_cell(X[H - 1], Y1, C[(H - 2) % R], delta);
}

// Reverse cell (path_calc_b2 :105-111 in log-adjoint form) + vega, on local
// rate i; s = {Y, S'}: the drift sum at rate i (rebuilt downwards) and
// delta^2 times the reference's suffix sum v1.
template <int H>
__device__ __forceinline__ void tp2_rev_cell(float (&X)[H], float (&Pb)[H], float2 &s, int i,
                                             const float4 &k, float &acc, float delta)
{
    const float y = s.x;
    const float xn = X[i] * ex2_approx(fmaf(k.x, y, k.y));
    const float t = rcp_approx(xn + delta);
    s.x = fmaf(-k.z, t, s.x);
    const float pb = Pb[i];
    s.y = fmaf(k.z, pb, s.y);
    const float tS = t * s.y;
    acc += fmaf(pb, fmaf(-delta, k.w, y), tS);
    Pb[i] = fmaf(k.w * fmaf(-delta, t, 1.0f), tS, pb);
    X[i] = xn;
}

// Reverse steps n and n-1 over a thread's H rates, positions descending:
// cell (n-g, i+g) at position i, its constants kcn[i+2g] and vega row
// vgn[(i+2g)*PB] (rows of step n's k), in register rings of 3+P slots so that
// each constant is loaded once and each vega row gets one read-modify-write
// per two cells. Left at the first chunk below position imin, the lowest
// position with an active cell; rows still open there are spare rows.
// Position -1 takes step n-1's cell at local rate 0, and the slot of local
// rate 0 is flushed after the last position.
template <int H, int PB, int CH, int P>
__device__ __forceinline__ void tp2_rev_pair(float (&X)[H], float (&Pb)[H], float2 (&st)[2],
                                             const float4 *kcn, float *vgn, float delta, int imin)
{
    constexpr int G = 2;
    constexpr int JMAX = H + G - 2;
    constexpr int W = 2 * G - 1 + P;
    float4 C[W];
    float A[W];
#pragma unroll
    for (int j = H - P; j <= JMAX; ++j) {
        C[j % W] = kcn[j];
        if (j >= H) A[j % W] = 0.0f;
    }
#pragma unroll
    for (int q = 0; q * CH < H + G - 1; ++q) {
        const int top = H - 1 - q * CH;
        if (top < imin) return;
#pragma unroll
        for (int i = top; i > top - CH && i >= -(G - 1); --i) {
            if (i - P >= 0) C[(i - P) % W] = kcn[i - P];
            if (i >= 0) A[i % W] = 0.0f;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (i + g >= 0 && i + g <= H - 1) {
                    const int j = i + 2 * g;
                    tp2_rev_cell<H>(X, Pb, st[g], i + g, C[j % W], A[j % W], delta);
                }
            }
            const int jf = i + 2 * (G - 1);
            if (jf >= 0 && jf <= JMAX) vgn[jf * PB] += A[jf % W];
        }
    }
    vgn[0] += A[0];
}

// Column sums over a pair's 32 paths of H rows (stride PB): lane handles rows
// lane, lane+32, ...; the (t+lane)&31 rotation keeps the lanes on distinct
// banks. Adds sums (TwoSum-compensated, LMM_COMP_SUMS) and sums of squares
// into FP64 accumulators.
template <int H, int PB>
__device__ __forceinline__ void tp2_rows_reduce(const float *rows, int lane, double *acc, int nout, int off)
{
    for (int k = lane; k < H; k += 32) {
        const float *col = rows + k * PB;
        float a = 0.0f, c = 0.0f, a2 = 0.0f;
#pragma unroll 8
        for (int t = 0; t < 32; ++t) {
            const float x = col[(t + lane) & 31];
            if (LMM_COMP_SUMS)
                two_sum_acc(a, c, x);
            else
                a += x;
            a2 = fmaf(x, x, a2);
        }
        acc[off + k] += (double)a + (double)c;
        acc[nout + off + k] += (double)a2;
    }
}

// MODE Fused: value + Greeks; `tape` is the launch's scratch: [grid][NMAT][PB]
// drift sums at rate H-1, then [grid][tp2_nckpt][NN][PB] rate checkpoints, one every m.ckpt steps. Forward: value, and the tape: terminal inverse rates
// [NN][total], the full drift sum of every step [NMAT][total], the drift sum
// at rate H-1 of every step [NMAT][total]. Backward: the Greeks of
// vbar[scen] * value from the tape (payoff rebuilt from the terminal rates).
template <int NN, int NMAT, bool PHILOX, Mode MODE>
__global__ void __launch_bounds__(Tp2Shape<NN>::kBlock, Tp2Shape<NN>::kMinBlocks)
k_tp2(const DevModel m, const float *__restrict__ z, uint64_t seed, int64_t path0, const Work w,
      float *__restrict__ tape, const double *__restrict__ vbar)
{
    using Lay = Tp2Layout<NN, NMAT, MODE>;
    constexpr int H = Lay::H, PB = Lay::PB, M = Lay::M, NOUT = Lay::NOUT, PADK = Lay::PADK;
    constexpr int CH = kTp2Chunk, P = kTp2Pref;
    static_assert(NN % 2 == 0 && NMAT >= H && NMAT < NN, "upper half holds every annuity rate");
    static_assert(NMAT % 4 == 0, "normals are read in aligned quads, steps in pairs");
    static_assert(H % CH == 0, "whole chunks per half");
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *kc_s = reinterpret_cast<float4 *>(smem + Lay::kc);
    float *il0_s = reinterpret_cast<float *>(smem + Lay::il0);
    int *ost_s = reinterpret_cast<int *>(smem + Lay::ost);
    float *okf_s = reinterpret_cast<float *>(smem + Lay::okf);
    float *owf_s = reinterpret_cast<float *>(smem + Lay::owf);
    F2 *okk_s = reinterpret_cast<F2 *>(smem + Lay::okk);
    float *vt_s = reinterpret_cast<float *>(smem + Lay::vt);
    float *vg_s = reinterpret_cast<float *>(smem + Lay::vg);
    float *hf_s = reinterpret_cast<float *>(smem + Lay::hf);
    float *hr_s = reinterpret_cast<float *>(smem + Lay::hr);
    float *pd_s = reinterpret_cast<float *>(smem + Lay::pd);
    double *acc_s = reinterpret_cast<double *>(smem + Lay::acc);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Warp w runs on scheduler w % 4. The upper half has the larger share of
    // the cells (every rate of it is active in steps below H), so warps w
    // and w + 4 take opposite halves: each scheduler gets one warp of each.
    const int upper = (warp & 1) ^ (LMM_TP2_SWIZZLE ? (warp >> 2) & 1 : 0), pair = warp >> 1;
    const int ps = pair * 32 + lane;                 // path slot in the batch
    const int base = upper * H;                      // first global rate of this thread
    for (int i = tid; i < PADK + NN; i += Lay::B) {
        const int k = i - PADK;
        kc_s[i] = k < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : m.kc[k];
    }
    for (int i = tid; i <= M; i += Lay::B) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += Lay::B) {
        okf_s[i] = m.optKf[i];
        owf_s[i] = m.optWf[i];
        okk_s[i] = f2_from(m.optKd[i] * m.deltad);
    }
    double *acc = acc_s + pair * 2 * NOUT;
    const float delta = m.delta, sqd = m.sqd;
    const float4 *kc0 = kc_s + PADK + base;          // kc0[j - n - 1]: step n, local rate j
    float *vg0 = vg_s + Lay::VPAD * PB + ps;         // vega row k of this path: vg0[k*PB]
    float *vt0 = vt_s + ps;
    const int64_t total = (int64_t)m.nscen * w.paths;
    // drift sums at rate H-1, saved by the lower half's forward for its reverse
    const int64_t hs = MODE == Mode::Fused ? PB : total;

    const int units = m.nscen * w.items;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int scen = unit / w.items, item = unit % w.items;
        __syncthreads();          // the previous unit's reads of il0/acc are done
        for (int i = tid; i < NN; i += Lay::B) il0_s[i] = m.invL0f[scen * NN + i];
        for (int i = tid; i < Lay::NP * 2 * NOUT; i += Lay::B) acc_s[i] = 0.0;
        __syncthreads();

        const int64_t ibase = (int64_t)item * w.ppt * PB;
        const float vb = MODE == Mode::Backward ? (float)vbar[scen] : 1.0f;
        for (int jb = 0; jb < w.ppt; ++jb) {
            if (ibase + (int64_t)jb * PB >= w.paths) break;          // block-uniform
            const int64_t pl = ibase + (int64_t)jb * PB + ps;
            const bool active = pl < w.paths;
            const int64_t pc = active ? pl : w.paths - 1;
            const int64_t tp = (int64_t)scen * w.paths + pc;
            const float *zp = PHILOX ? nullptr : z + pc * NMAT;
            const uint64_t gpath = (uint64_t)(path0 + pc);
            float *tape_v = MODE == Mode::Fused ? nullptr : tape + (int64_t)NN * total + tp;
            float *hsum = MODE == Mode::Fused ? tape + (int64_t)blockIdx.x * NMAT * PB + ps
                                              : tape + (int64_t)(NN + NMAT) * total + tp;
            const int ck = MODE == Mode::Fused ? m.ckpt : 0;
            const int NCK = tp2_nckpt(NMAT, ck);
            // checkpoint c (the rates after step (c+1) ck - 1), local rate i: ckp[(c*NN + i)*PB]
            float *ckp = tape + (int64_t)gridDim.x * NMAT * PB + (int64_t)blockIdx.x * NCK * NN * PB + base * PB + ps;

            float X[H];
            float Pb[H];
#pragma unroll
            for (int i = 0; i < H; ++i)
                X[i] = MODE == Mode::Backward ? tape[(int64_t)(base + i) * total + tp] : il0_s[base + i];

            // ---- forward: the lower half leads by one round ----
            float4 zq = make_float4(0.f, 0.f, 0.f, 0.f), zq_next = zq;
            if (!upper) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, 0);
            for (int r = 0; r <= (MODE == Mode::Backward ? -1 : NMAT / 2); ++r) {
                const bool run = upper ? r >= 1 : r < NMAT / 2;
                if (run) {
                    const int n = upper ? 2 * r - 2 : 2 * r;
                    float Y0, Y1;
                    if (!upper) {
                        if ((n & 3) == 0) {
                            zq = zq_next;
                            if ((n >> 2) + 1 < NMAT / 4) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) + 1);
                        }
                        Y0 = sqd * ((n & 2) ? zq.z : zq.x);
                        Y1 = sqd * ((n & 2) ? zq.w : zq.y);
                    } else {
                        const float *h = hf_s + ((r - 1) & 1) * 2 * PB + ps;
                        Y0 = h[0];
                        Y1 = h[PB];
                    }
                    const int first = n + 1 - base;          // step n's first active local rate
                    if (first < H) {
                        const int c0 = first > 0 ? first / CH : 0;
                        tp2_fwd_pair<H, CH, P>(X, kc0 - (n + 1), c0, delta, Y0, Y1);
                    }
                    if (!upper) {
                        float *h = hf_s + (r & 1) * 2 * PB + ps;
                        h[0] = Y0;
                        h[PB] = Y1;
                        if (MODE == Mode::Fused || active) {
                            hsum[n * hs] = Y0;
                            hsum[(n + 1) * hs] = Y1;
                        }
                    } else if (MODE == Mode::Fused) {
                        vt0[n * PB] = Y0;
                        vt0[(n + 1) * PB] = Y1;
                    } else if (active) {
                        tape_v[(int64_t)n * total] = Y0;
                        tape_v[(int64_t)(n + 1) * total] = Y1;
                    }
                    if (NCK > 0 && (n + 2) % ck == 0 && n + 2 < NMAT) {
                        // rates i <= n+2 are final from here on: only the others are saved
                        const int c = (n + 2) / ck - 1;
#pragma unroll
                        for (int i = 0; i < H; ++i)
                            if (base + i > n + 2) ckp[(c * NN + i) * PB] = X[i];
                    }
                }
                __syncthreads();
            }
            if (MODE == Mode::Forward && active) {
#pragma unroll
                for (int i = 0; i < H; ++i) tape[(int64_t)(base + i) * total + tp] = X[i];
            }

            // ---- payoff (portfolio_b :133-171, :186-197) and its adjoint ----
            if (!upper) {
                F2 d{1.0f, 0.0f};
#pragma unroll
                for (int i = 0; i < H; ++i) d = f2_mul(d, bond_ratio(X[i], delta));
                pd_s[ps] = d.hi;
                pd_s[PB + ps] = d.lo;
            }
            __syncthreads();
            float V = 0.0f;
            if (upper) {
                F2 disc{pd_s[ps], pd_s[PB + ps]};
#pragma unroll
                for (int i = 0; i < NMAT - H; ++i) disc = f2_mul(disc, bond_ratio(X[i], delta));
                // annuity rates NMAT..NN-1 staged in vega rows 0..M-1, the
                // annuity factors B[m] in rows M..2M-1 (free until the reverse)
                float *ILst = vg0;
                float *Bst = vg0 + M * PB;
#pragma unroll
                for (int mm = 0; mm < M; ++mm) ILst[mm * PB] = X[NMAT - H + mm];
                F2 b{1.0f, 0.0f}, sb{0.0f, 0.0f}, vs{0.0f, 0.0f};
                unsigned long long mask = 0ull;
#pragma unroll 1
                for (int mm = 0; mm < M; ++mm) {
                    b = f2_mul(b, bond_ratio(ILst[mm * PB], delta));
                    sb = f2_add(sb, b);                                   // annuity / delta
                    Bst[mm * PB] = b.hi;
                    const int o1 = ost_s[mm + 1];
#pragma unroll 1
                    for (int o = ost_s[mm]; o < o1; ++o) {
                        const float sw = f2_swap_value(okk_s[o], sb, b);
                        if (sw < 0.0f) {
                            vs = f2_add(vs, (-100.0f * sw) * owf_s[o]);
                            mask |= 1ull << o;
                        }
                    }
                }
                const F2 v = f2_mul(vs, disc);
                V = __fadd_rn(v.hi, v.lo);
              if (MODE != Mode::Forward) {
                // adjoint (:173-184 with rate and adjoint kept apart, :199-209),
                // seeded with vb = dOut/dV
                const float scale = -vb * disc.hi * delta;
                float Sb = 0.0f, Bb = 0.0f;
#pragma unroll 1
                for (int mm = M - 1; mm >= 0; --mm) {
                    const float il = ILst[mm * PB];
                    const float t = rcp_approx(il + delta);
                    const float rr = bond_ratio_t(il, delta, t);
                    const float Bm = Bst[mm * PB];
                    const int o1 = ost_s[mm + 1];
#pragma unroll 1
                    for (int o = ost_s[mm]; o < o1; ++o) {
                        if ((mask >> o) & 1ull) {
                            Sb -= (100.0f * okf_s[o]) * owf_s[o];
                            Bb -= 100.0f * owf_s[o];
                        }
                    }
                    Bb = fmaf(delta, Sb, Bb);
                    ILst[mm * PB] = scale * Bb * Bm * t;
                    Bb *= rr;
                }
#pragma unroll
                for (int mm = 0; mm < M; ++mm) Pb[NMAT - H + mm] = ILst[mm * PB];
                const float vsd = -vb * V * delta;
#pragma unroll
                for (int i = 0; i < NMAT - H; ++i) Pb[i] = vsd * rcp_approx(X[i] + delta);
#pragma unroll
                for (int k = 0; k < NN; ++k) vg0[k * PB] = 0.0f;
                pd_s[2 * PB + ps] = V;
              }
            }
            if (MODE != Mode::Forward) {
                __syncthreads();
                if (!upper) {
                    const float vsd = -vb * pd_s[2 * PB + ps] * delta;
#pragma unroll
                    for (int i = 0; i < H; ++i) Pb[i] = vsd * rcp_approx(X[i] + delta);
                }
            }

            // ---- reverse: the upper half leads by one round; the lower half
            // starts each step from the forward's drift sum at rate H-1 (so
            // each half rebuilds the drift over its own H rates only), loaded
            // one round ahead ----
            float hn0 = 0.0f, hn1 = 0.0f;
            if (MODE != Mode::Forward && !upper) {
                hn0 = hsum[(NMAT - 1) * hs];
                hn1 = hsum[(NMAT - 2) * hs];
            }
            for (int r = 0; r <= (MODE == Mode::Forward ? -1 : NMAT / 2); ++r) {
                const bool run = upper ? r < NMAT / 2 : r >= 1;
                if (run) {
                    const int n = NMAT - 1 - 2 * (upper ? r : r - 1);
                    float2 st[2];
                    if (upper) {
                        if (MODE == Mode::Fused) {
                            st[0] = make_float2(vt0[n * PB], 0.0f);
                            st[1] = make_float2(vt0[(n - 1) * PB], 0.0f);
                        } else {
                            st[0] = make_float2(tape_v[(int64_t)n * total], 0.0f);
                            st[1] = make_float2(tape_v[(int64_t)(n - 1) * total], 0.0f);
                        }
                    } else {
                        const float *h = hr_s + ((r - 1) & 1) * 4 * PB + ps;
                        st[0] = make_float2(hn0, h[PB]);
                        st[1] = make_float2(hn1, h[3 * PB]);
                        if (n - 2 > 0) {
                            hn0 = hsum[(n - 2) * hs];
                            hn1 = hsum[(n - 3) * hs];
                        }
                    }
                    const int imin = n - 1 - base;           // lowest position with an active cell
                    if (imin < H)
                        tp2_rev_pair<H, PB, CH, P>(X, Pb, st, kc0 - (n + 1), vg0 + (base - n - 1) * PB, delta, imin);
                    if (NCK > 0 && (n - 1) % ck == 0 && n - 1 >= ck) {
                        // the reverse of steps >= n-1 leaves rates i <= n-1 untouched
                        const int c = (n - 1) / ck - 1;
#pragma unroll
                        for (int i = 0; i < H; ++i)
                            if (base + i > n - 1) X[i] = ckp[(c * NN + i) * PB];
                    }
                    if (upper) {
                        float *h = hr_s + (r & 1) * 4 * PB + ps;
                        h[PB] = st[0].y;
                        h[3 * PB] = st[1].y;
                    }
                }
                __syncthreads();
            }

            // ---- cross-path reduction of the batch: each half reduces the
            // vega and delta columns of its own rates; the upper half the value
            if (MODE != Mode::Forward) {
                constexpr int doff = MODE == Mode::Fused ? 1 : 0;
                float *rows = vg_s + (Lay::VPAD + base) * PB + pair * 32;
                float *mine = vg0 + base * PB;
                if (!active) {
#pragma unroll
                    for (int i = 0; i < H; ++i) mine[i * PB] = 0.0f;
                }
                __syncwarp();
                tp2_rows_reduce<H, PB>(rows, lane, acc, NOUT, doff + NN + base);
                __syncwarp();
#pragma unroll
                for (int i = 0; i < H; ++i) mine[i * PB] = active ? Pb[i] * il0_s[base + i] : 0.0f;
                __syncwarp();
                tp2_rows_reduce<H, PB>(rows, lane, acc, NOUT, doff + base);
            }
            if (MODE != Mode::Backward && upper) {
                const float v = active ? V : 0.0f;
                const float s1 = warp_sum(v), s2 = warp_sum(v * v);
                if (lane == 0) {
                    acc[0] += (double)s1;
                    acc[NOUT] += (double)s2;
                }
            }
            __syncthreads();      // vega rows are zeroed by the next batch's payoff
        }

        for (int o = tid; o < 2 * NOUT; o += Lay::B) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < Lay::NP; ++q) s += acc_s[q * 2 * NOUT + o];
            w.partial[(size_t)unit * 2 * NOUT + o] = s;
        }
    }  // units
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
cudaError_t launch_tp2(const DevModel &m, const float *z, uint64_t seed, int64_t path0, const Work &w,
                       float *tape, const double *vbar, cudaStream_t s)
{
    using Lay = Tp2Layout<NN, NMAT, MODE>;
    auto kern = k_tp2<NN, NMAT, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)(w.grid > 0 ? w.grid : (int64_t)m.nscen * w.items);
    kern<<<grid, Lay::B, Lay::bytes, s>>>(m, z, seed, path0, w, tape, vbar);
    return cudaGetLastError();
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
cudaError_t occ_tp2(int *blocks)
{
    using Lay = Tp2Layout<NN, NMAT, MODE>;
    auto kern = k_tp2<NN, NMAT, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, Lay::B, Lay::bytes);
}

}  // namespace

bool f32_tp2_supports(int nn, int nmat) { return nn == 160 && nmat == 120; }

int tp2_paths_per_block(int) { return Tp2Shape<160>::kBlock / 2; }

size_t tp2_scratch_floats_per_block(int nn, int nmat, int ckpt)
{
    return (size_t)(nmat + tp2_nckpt(nmat, ckpt) * nn) * tp2_paths_per_block(nn);
}

// Philox normals only in the fused kernel; the pair reads its normals from memory.
#define LMM_TP2_SHAPE(FN, NN, NMAT, ...)                                                   \
    do {                                                                                   \
        switch (mode) {                                                                    \
            case Mode::Fused:                                                              \
                return philox ? FN<NN, NMAT, true, Mode::Fused>(__VA_ARGS__)               \
                              : FN<NN, NMAT, false, Mode::Fused>(__VA_ARGS__);             \
            case Mode::Forward: return FN<NN, NMAT, false, Mode::Forward>(__VA_ARGS__);    \
            case Mode::Backward: return FN<NN, NMAT, false, Mode::Backward>(__VA_ARGS__);  \
        }                                                                                  \
        return cudaErrorInvalidValue;                                                      \
    } while (0)

#define LMM_TP2_DISPATCH(FN, ...)                                                          \
    do {                                                                                   \
        if (philox && mode != Mode::Fused) return cudaErrorInvalidValue;                   \
        if (nn == 160 && nmat == 120) LMM_TP2_SHAPE(FN, 160, 120, __VA_ARGS__);             \
        return cudaErrorInvalidValue;                                                      \
    } while (0)

cudaError_t tp2_blocks_per_sm(int nn, int nmat, Mode mode, bool philox, int *blocks)
{
    LMM_TP2_DISPATCH(occ_tp2, blocks);
}

cudaError_t launch_tp2_any(const DevModel &m, Mode mode, const float *z, uint64_t seed, int64_t path0,
                           bool philox, const Work &w, float *tape, const double *vbar, cudaStream_t s)
{
    const int nn = m.nn, nmat = m.nmat;
    LMM_TP2_DISPATCH(launch_tp2, m, z, seed, path0, w, tape, vbar, s);
}

}  // namespace lmm

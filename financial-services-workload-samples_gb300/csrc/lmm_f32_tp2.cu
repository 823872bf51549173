// FP32 LMM value + Greeks with two threads per path (a thread pair), for
// NN=160, NMAT=120 (H = 80 rates per thread; the code takes any NN = 2H with
// NMAT >= H).
//
// The same Euler cells, payoff and adjoint as the thread-per-path kernel
// (lmm_f32_tpp.cu; reference LiborMarketModel/liborSwaptionGreeks.cpp
// path_calc_b1 :34-82, portfolio_b :120-211 with the :178/:181 aliasing
// fixed, path_calc_b2 :86-117, plus the vega adjoint), with the rates of a
// path split between the two warps 2q, 2q+1 of a block ("role" 0 and 1).
// A thread keeps H inverse rates and H log-adjoints in registers, so NN=160
// runs with the per-thread footprint that NN=80 has in the thread-per-path
// kernel.
//
// Rate blocks. The rates are cut into S = NN/L blocks of L consecutive rates
// (block s holds rates sL .. sL+L-1) and the two roles own alternate blocks:
// role 0 blocks 0, 2, 4, ..., role 1 blocks 1, 3, 5, ...; a thread's local
// register j holds rate (2(j/L) + role) L + j%L. Step n moves only the rates
// above n, so with two halves (L = H) the lower half runs out of work after
// step H-1 while the upper half stays busy: at 160/120 the halves own 3,160
// and 8,780 cells. Alternating blocks share the cells of every step between
// the roles (a round-cost model of the skewed schedule below, the sum over
// rounds of the busier role's cells: two halves 8,937; blocks of 40 7,326;
// of 20 6,670; ideal 5,970).
//
// The drift sum of a step runs upwards over i, the adjoint's suffix sum and
// the drift reconstruction downwards, so the blocks form a pipeline worked in
// rounds, one barrier per round, each round one pair of steps per block:
//   forward   round r: block s takes steps 2(r-s), 2(r-s)+1, starting from
//             the drift sums block s-1 left at its top rate in round r-1
//             (block 0: sqrt(delta) z), and leaves its own top drift sums
//             for block s+1 (and, for the reverse, in device scratch);
//   reverse   round r: block s takes steps n, n-1 with n = NMAT-1 -
//             2(r-(S-1-s)), starting from the forward's drift sums at its top
//             rate (the top block: the full sums) and from the adjoint's
//             suffix sums block s+1 left at its bottom in round r-1 (the top
//             block: 0), so each block rebuilds the drift over its own L
//             rates only.
// In a reverse round block s (steps n_s, n_s-1) adds vega rows
// k in [sL - n_s - 2, sL + L - n_s - 1] and block s+1 runs two steps earlier
// (n_{s+1} = n_s - 2), so adjacent blocks never touch the same row in one
// round (checked on the CPU by tests/test_kernel_schedules.py).
// The payoff: each role forms the discount factors of its rates below NMAT
// and stages its annuity rates in shared memory; role 1 (which owns the top
// block) combines the discount, runs the annuities, the swaptions and their
// adjoint, and passes the value and the annuity rates' log-adjoints back.
//
// The fused kernel (value + Greeks in one launch) runs L = LMM_TP2_SEG; the
// forward/backward pair runs L = H (two halves), the layout its tape holds.
//
// Within a thread the cells are those of the thread-per-path kernel: the
// forward pairs steps n, n+1 (cell (n,p) beside cell (n+1,p-1)); the reverse
// pairs steps n, n-1 as a skewed wavefront with constants and vega partial
// sums in register rings; branch-free triangles through NMAT zero constant
// rows; drift sums carry the normal term (Y = V + sqrt(delta) z).
#include "lmm_device.cuh"

// Rates per block of the fused kernel (40: two blocks per thread at NN=160;
// 80: the two halves). GB300, 160/120, 1,048,576 paths: blocks of 20 / 40 /
// 80 rates 25.6 / 18.3 / 20.4 ms: blocks of 20 lose more to the per-block
// window set-up and hand-overs than the better balance gains.
#ifndef LMM_TP2_SEG
#define LMM_TP2_SEG 40
#endif

namespace lmm {
namespace {

constexpr int kTp2Pref = 2;        // constants loaded this many positions ahead
// Rates per chunk of the step bodies inside a block of L rates.
__host__ __device__ constexpr int tp2_chunk(int L) { return L % 8 == 0 ? 8 : 4; }
// The fused kernel saves the rates every ck = DevModel::ckpt steps (0: never;
// ck even, so that checkpoints fall between step pairs) and the reverse sweep
// takes them in place of its rebuilt rates there, so FP32 rounding of the
// backward Euler steps accumulates over at most ck steps.
// Rate checkpoints of a fused launch: at times ck, 2 ck, ... < nmat.
__host__ __device__ constexpr int tp2_nckpt(int nmat, int ck) { return ck > 0 ? (nmat - 1) / ck : 0; }

// Warps per block (8: one block per SM; 4: two blocks per SM), and whether
// warps w and w+4, which share a scheduler, take opposite roles (1) or the
// same role (0). GB300, 160/120, 1,048,576 paths, two halves: 8 warps
// alternating 19.4 ms, 8 warps not alternating 21.0 ms, two blocks of 4 warps
// 21.1-22.0 ms.
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

template <int NN, Mode MODE>
__host__ __device__ constexpr int tp2_seg() { return MODE == Mode::Fused ? LMM_TP2_SEG : NN / 2; }

template <int NN, int NMAT, Mode MODE>
struct Tp2Layout {
    static constexpr int H = NN / 2;
    static constexpr int L = tp2_seg<NN, MODE>();      // rates per block
    static constexpr int S = NN / L;                   // blocks
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
    static constexpr int hf = vg + 4 * (VPAD + NN) * PB;             // float[S-1][2][2][PB] forward hand-over
    static constexpr int hr = hf + 4 * (S - 1) * 4 * PB;             // float[S-1][2][2][PB] reverse hand-over
    static constexpr int pd = hr + 4 * (S - 1) * 4 * PB;             // float[5][PB] payoff exchange
    static constexpr int hp = pd + 4 * 5 * PB;                       // float[S/2][2][B] restart sums in flight
    static constexpr int acc = al16(hp + 4 * (S / 2) * 2 * B);       // double[NP][2*NOUT]
    static constexpr int bytes = acc + 8 * NP * 2 * NOUT;
    static_assert(NN % L == 0 && S % 2 == 0, "whole blocks, alternating between the two roles");
    static_assert(L % tp2_chunk(L) == 0, "whole chunks per block");
};

// Forward cell on the inverse rate X = 1/L (path_calc_b1 :66-72), with the
// drift sum Y carrying the normal term: t = 1/(X + delta); Y += delta^2
// lambda_k t; X *= 2^-(lambda_k log2(e) Y - delta lambda_k^2 log2(e)/2).
__device__ __forceinline__ void tp2_fwd_cell(float &X, float &Y, const float4 &k, float delta)
{
    Y = fmaf(k.z, rcp_approx(X + delta), Y);
    X *= ex2_approx(-fmaf(k.x, Y, k.y));
}

// tp2_fwd_cell with t = 1/(X + delta) given.
__device__ __forceinline__ void tp2_fwd_cell_t(float &X, float &Y, const float4 &k, float t)
{
    Y = fmaf(k.z, t, Y);
    X *= ex2_approx(-fmaf(k.x, Y, k.y));
}

// Steps n and n+1 over one block of L rates held in X[OFF .. OFF+L) (local
// position p, the block's rate p): cell (n, p) and cell (n+1, p-1) at
// position p; kcn[j] holds the constants of step n at the block's rate j,
// which are those of step n+1 at rate j+1. Entered at chunk c0 (c0 * CH < L),
// which holds step n's first active rate (or 0); the cells of either step
// below its first active rate see zero constants and are exact no-ops.
template <int NX, int OFF, int L, int CH, int P>
__device__ __forceinline__ void tp2_fwd_pair(float (&X)[NX], const float4 *kcn, int c0, float delta,
                                             float &Y0, float &Y1)
{
    constexpr int R = 3 + P;
    float4 C[R];
    // LMM_FWD_RCP2_LONG: the cells of one step at rates 2m, 2m+1 share one
    // reciprocal, paired and ordered as in the fused kernel (the block's first
    // rate is even), so the two round alike
    static_assert(!LMM_FWD_RCP2_LONG || (CH % 2 == 0 && L % 2 == 0), "reciprocal pairs (2m, 2m+1) inside chunks");
    float t0n = 0.0f, t1n = 0.0f;
#pragma unroll
    for (int c = 0; c * CH < L; ++c) {
        if (c >= c0) {
            if (c == c0) {
#pragma unroll
                for (int j = c * CH - 2; j < c * CH + P; ++j)
                    if (j < L) C[(j + R) % R] = kcn[j];
                if (LMM_FWD_RCP2_LONG && c * CH >= 2) {       // step n+1's pair below the chunk
                    float ta;
                    rcp_pair(X[OFF + c * CH - 2] + delta, X[OFF + c * CH - 1] + delta, ta, t1n);
                }
            }
#pragma unroll
            for (int p = c * CH; p < (c + 1) * CH && p < L; ++p) {
                if (p + P < L) C[(p + P) % R] = kcn[p + P];
                if (LMM_FWD_RCP2_LONG) {
                    float t;
                    if (p % 2 == 0)
                        rcp_pair(X[OFF + p] + delta, X[OFF + p + 1] + delta, t, t0n);
                    else
                        t = t0n;
                    tp2_fwd_cell_t(X[OFF + p], Y0, C[p % R], t);
                    if (p % 2 == 1) {
                        float ta;
                        rcp_pair(X[OFF + p - 1] + delta, X[OFF + p] + delta, ta, t1n);
                        tp2_fwd_cell_t(X[OFF + p - 1], Y1, C[(p + R - 2) % R], ta);
                    } else if (p >= 1) {
                        tp2_fwd_cell_t(X[OFF + p - 1], Y1, C[(p + R - 2) % R], t1n);
                    }
                } else {
                    tp2_fwd_cell(X[OFF + p], Y0, C[p % R], delta);
                    if (p >= 1) tp2_fwd_cell(X[OFF + p - 1], Y1, C[(p + R - 2) % R], delta);
                }
            }
        }
    }
    if (LMM_FWD_RCP2_LONG)
        tp2_fwd_cell_t(X[OFF + L - 1], Y1, C[(L - 2) % R], t1n);
    else
        tp2_fwd_cell(X[OFF + L - 1], Y1, C[(L - 2) % R], delta);
}

// Reverse cell (path_calc_b2 :105-111 in log-adjoint form) + vega on one
// rate (x its inverse rate, pb its log-adjoint); s = {Y, S'}: the drift sum
// at the rate (rebuilt downwards) and delta^2 times the reference's suffix
// sum v1.
__device__ __forceinline__ void tp2_rev_cell(float &x, float &pbr, float2 &s, const float4 &k, float &acc,
                                             float delta)
{
    const float y = s.x;
    const float xn = x * ex2_approx(fmaf(k.x, y, k.y));
    const float t = rcp_approx(xn + delta);
    s.x = fmaf(-k.z, t, s.x);
    const float pb = pbr;
    s.y = fmaf(k.z, pb, s.y);
    const float tS = t * s.y;
    acc += fmaf(pb, fmaf(-delta, k.w, y), tS);
    pbr = fmaf(k.w * fmaf(-delta, t, 1.0f), tS, pb);
    x = xn;
}

// Reverse steps n and n-1 over one block of L rates (X, Pb at OFF ..
// OFF+L), positions descending: cell (n-g, i+g) at position i, its constants
// kcn[i+2g] and vega row vgn[(i+2g)*PB] (rows of step n's k), in register
// rings of 3+P slots so that each constant is loaded once and each vega row
// gets one read-modify-write per two cells. Left at the first chunk below
// position imin, the lowest position with an active cell; rows still open
// there are spare rows. Position -1 takes step n-1's cell at the block's rate
// 0, and the slot of rate 0 is flushed after the last position.
template <int NX, int OFF, int L, int PB, int CH, int P>
__device__ __forceinline__ void tp2_rev_pair(float (&X)[NX], float (&Pb)[NX], float2 (&st)[2],
                                             const float4 *kcn, float *vgn, float delta, int imin)
{
    constexpr int G = 2;
    constexpr int JMAX = L + G - 2;
    constexpr int W = 2 * G - 1 + P;
    float4 C[W];
    float A[W];
#pragma unroll
    for (int j = L - P; j <= JMAX; ++j) {
        C[j % W] = kcn[j];
        if (j >= L) A[j % W] = 0.0f;
    }
#pragma unroll
    for (int q = 0; q * CH < L + G - 1; ++q) {
        const int top = L - 1 - q * CH;
        if (top < imin) return;
#pragma unroll
        for (int i = top; i > top - CH && i >= -(G - 1); --i) {
            if (i - P >= 0) C[(i - P) % W] = kcn[i - P];
            if (i >= 0) A[i % W] = 0.0f;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (i + g >= 0 && i + g <= L - 1) {
                    const int j = i + 2 * g;
                    tp2_rev_cell(X[OFF + i + g], Pb[OFF + i + g], st[g], C[j % W], A[j % W], delta);
                }
            }
            const int jf = i + 2 * (G - 1);
            if (jf >= 0 && jf <= JMAX) vgn[jf * PB] += A[jf % W];
        }
    }
    vgn[0] += A[0];
}

// 4-byte asynchronous copy global -> shared (cp.async, completes at
// cp_async_wait_all of the issuing thread): no register holds the value in
// flight.
__device__ __forceinline__ void cp_async4(float *sdst, const float *gsrc)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// The block windows for the thread's block q (a loop index that unrolling
// makes a constant, which these chains fold to one call).
template <int NX, int L, int CH, int P, int QI = 0>
__device__ __forceinline__ void tp2_fwd_block(int q, float (&X)[NX], const float4 *kcn, int c0, float delta,
                                              float &Y0, float &Y1)
{
    if (q == QI)
        tp2_fwd_pair<NX, QI * L, L, CH, P>(X, kcn, c0, delta, Y0, Y1);
    else if constexpr ((QI + 1) * L < NX)
        tp2_fwd_block<NX, L, CH, P, QI + 1>(q, X, kcn, c0, delta, Y0, Y1);
}

template <int NX, int L, int PB, int CH, int P, int QI = 0>
__device__ __forceinline__ void tp2_rev_block(int q, float (&X)[NX], float (&Pb)[NX], float2 (&st)[2],
                                              const float4 *kcn, float *vgn, float delta, int imin)
{
    if (q == QI)
        tp2_rev_pair<NX, QI * L, L, PB, CH, P>(X, Pb, st, kcn, vgn, delta, imin);
    else if constexpr ((QI + 1) * L < NX)
        tp2_rev_block<NX, L, PB, CH, P, QI + 1>(q, X, Pb, st, kcn, vgn, delta, imin);
}

// Column sums over a pair's 32 paths of the rows of one role's rates (row of
// local j: rate (2(j/L) + role) L + j%L, stride PB): lane handles local
// rates lane, lane+32, ...; the (t+lane)&31 rotation keeps the lanes on
// distinct banks. Adds sums (TwoSum-compensated, LMM_COMP_SUMS) and sums of
// squares into FP64 accumulators at off + rate.
template <int H, int L, int PB>
__device__ __forceinline__ void tp2_rows_reduce(const float *rows0, int lane, int role, double *acc, int nout,
                                                int off)
{
    for (int j = lane; j < H; j += 32) {
        const int k = (2 * (j / L) + role) * L + j % L;
        const float *col = rows0 + k * PB;
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

// MODE Fused: value + Greeks; `tape` is the launch's scratch: [grid][S-1][NMAT][PB]
// drift sums at the top rate of every block but the last, then
// [grid][tp2_nckpt][NN][PB] rate checkpoints, one every m.ckpt steps.
// Forward (two halves): value, and the tape: terminal inverse rates
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
    constexpr int L = Lay::L, S = Lay::S, Q = S / 2;   // Q blocks per thread
    constexpr int CH = tp2_chunk(L), P = kTp2Pref;
    constexpr int ROUNDS = NMAT / 2 + S - 1;
    static_assert(NN % 2 == 0 && NMAT >= H && NMAT < NN, "role 1 holds the top block");
    static_assert(NMAT % 4 == 0, "normals are read in aligned quads, steps in pairs");
    static_assert(MODE == Mode::Fused || S == 2, "the pair's tape holds two halves");
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
    float *hp_s = reinterpret_cast<float *>(smem + Lay::hp);
    double *acc_s = reinterpret_cast<double *>(smem + Lay::acc);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Warp w runs on scheduler w % 4: warps w and w + 4 take opposite roles,
    // so each scheduler gets one warp of each.
    const int role = (warp & 1) ^ (LMM_TP2_SWIZZLE ? (warp >> 2) & 1 : 0), pair = warp >> 1;
    const int ps = pair * 32 + lane;                 // path slot in the batch
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
    float *vg0 = vg_s + Lay::VPAD * PB + ps;         // vega row k of this path: vg0[k*PB]
    float *vt0 = vt_s + ps;
    const int64_t total = (int64_t)m.nscen * w.paths;
    // Drift sums at the top rate of block s < S-1 for the reverse restart:
    // fused, per block of the launch in its scratch; the pair, in the tape.
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
            // hsum0 + s * NMAT * hs: block s's top drift sums (fused; the pair has s = 0 only)
            float *hsum0 = MODE == Mode::Fused ? tape + (int64_t)blockIdx.x * (S - 1) * NMAT * PB + ps
                                               : tape + (int64_t)(NN + NMAT) * total + tp;
            const int ck = MODE == Mode::Fused ? m.ckpt : 0;
            const int NCK = tp2_nckpt(NMAT, ck);
            const int ckd = ck > 0 ? ck : 1;             // divisor of the checkpoint tests (used when NCK > 0)
            // checkpoint c (the rates after step (c+1) ck - 1), rate i: ckp[(c*NN + i)*PB]
            float *ckp = tape + (int64_t)gridDim.x * (S - 1) * NMAT * PB + (int64_t)blockIdx.x * NCK * NN * PB + ps;

            float X[H];
            float Pb[H];
#pragma unroll
            for (int j = 0; j < H; ++j) {
                const int g = (2 * (j / L) + role) * L + j % L;
                X[j] = MODE == Mode::Backward ? tape[(int64_t)g * total + tp] : il0_s[g];
            }

            // ---- forward: block s runs round r - s's steps ----
            float4 zq = make_float4(0.f, 0.f, 0.f, 0.f), zq_next = zq;
            if (role == 0) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, 0);
            for (int r = 0; r < (MODE == Mode::Backward ? 0 : ROUNDS); ++r) {
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const int s = 2 * q + role, lo = s * L;
                    const int n = 2 * (r - s);
                    if (n < 0 || n >= NMAT) continue;
                    float Y0, Y1;
                    if (s == 0) {
                        if ((n & 3) == 0) {
                            zq = zq_next;
                            if ((n >> 2) + 1 < NMAT / 4) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) + 1);
                        }
                        Y0 = sqd * ((n & 2) ? zq.z : zq.x);
                        Y1 = sqd * ((n & 2) ? zq.w : zq.y);
                    } else {
                        const float *h = hf_s + ((s - 1) * 2 + ((r - 1) & 1)) * 2 * PB + ps;
                        Y0 = h[0];
                        Y1 = h[PB];
                    }
                    const int first = n + 1 - lo;            // step n's first active rate in the block
                    if (first < L) {
                        const int c0 = first > 0 ? first / CH : 0;
                        tp2_fwd_block<H, L, CH, P>(q, X, kc_s + PADK + lo - (n + 1), c0, delta, Y0, Y1);
                    }
                    if (s < S - 1) {
                        float *h = hf_s + (s * 2 + (r & 1)) * 2 * PB + ps;
                        h[0] = Y0;
                        h[PB] = Y1;
                        if (MODE == Mode::Fused || active) {
                            float *hsum = hsum0 + (int64_t)s * NMAT * hs;
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
                    if (NCK > 0 && (n + 2) % ckd == 0 && n + 2 < NMAT) {
                        // rates i <= n+2 are final from here on: only the others are saved
                        const int c = (n + 2) / ckd - 1;
#pragma unroll
                        for (int p = 0; p < L; ++p)
                            if (lo + p > n + 2) ckp[(c * NN + lo + p) * PB] = X[q * L + p];
                    }
                }
                __syncthreads();
            }
            if (MODE == Mode::Forward && active) {
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int g = (2 * (j / L) + role) * L + j % L;
                    tape[(int64_t)g * total + tp] = X[j];
                }
            }

            // ---- payoff (portfolio_b :133-171, :186-197) and its adjoint ----
            // annuity rates NMAT..NN-1 staged in vega rows 0..M-1, the annuity
            // factors B[m] in rows M..2M-1 (free until the reverse)
            float *ILst = vg0;
            float *Bst = vg0 + M * PB;
            {
                F2 d{1.0f, 0.0f};
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int g = (2 * (j / L) + role) * L + j % L;
                    if (g < NMAT)
                        d = f2_mul(d, bond_ratio(X[j], delta));
                    else
                        ILst[(g - NMAT) * PB] = X[j];
                }
                pd_s[2 * role * PB + ps] = d.hi;
                pd_s[(2 * role + 1) * PB + ps] = d.lo;
            }
            __syncthreads();
            float V = 0.0f;
            if (role == 1) {
                const F2 disc = f2_mul(F2{pd_s[ps], pd_s[PB + ps]}, F2{pd_s[2 * PB + ps], pd_s[3 * PB + ps]});
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
                    // seeded with vb = dOut/dV; each staged rate is replaced by its
                    // log-adjoint
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
                    pd_s[4 * PB + ps] = V;
                }
            }
            if (MODE != Mode::Forward) {
                __syncthreads();
                const float vsd = -vb * pd_s[4 * PB + ps] * delta;
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int g = (2 * (j / L) + role) * L + j % L;
                    if (g >= NMAT)
                        Pb[j] = ILst[(g - NMAT) * PB];
                    else
                        Pb[j] = vsd * rcp_approx(X[j] + delta);
                }
                __syncthreads();      // every staged log-adjoint is read
                for (int k = role; k < NN; k += 2) vg0[k * PB] = 0.0f;
                __syncthreads();
            }

            // ---- reverse: block s runs steps n, n-1 with n = NMAT-1-2(r-(S-1-s)),
            // restarting the drift reconstruction at its top rate from the
            // forward's sums there, copied to shared memory one round ahead
            // (hp[(q*2 + e)*B + tid]: block q's sums of steps n, n-1) ----
            float *hp0 = hp_s + tid;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int s = 2 * q + role;
                if (MODE != Mode::Forward && s < S - 1) {
                    const float *hsum = hsum0 + (int64_t)s * NMAT * hs;
                    cp_async4(hp0 + (q * 2) * Lay::B, hsum + (NMAT - 1) * hs);
                    cp_async4(hp0 + (q * 2 + 1) * Lay::B, hsum + (NMAT - 2) * hs);
                }
            }
            for (int r = 0; r < (MODE == Mode::Forward ? 0 : ROUNDS); ++r) {
                cp_async_wait_all();
#pragma unroll
                for (int qq = 0; qq < Q; ++qq) {
                    const int q = Q - 1 - qq;                // the thread's top block first
                    const int s = 2 * q + role, lo = s * L;
                    const int jr = r - (S - 1 - s);
                    if (jr < 0 || jr >= NMAT / 2) continue;
                    const int n = NMAT - 1 - 2 * jr;
                    float2 st[2];
                    if (s == S - 1) {
                        if (MODE == Mode::Fused) {
                            st[0] = make_float2(vt0[n * PB], 0.0f);
                            st[1] = make_float2(vt0[(n - 1) * PB], 0.0f);
                        } else {
                            st[0] = make_float2(tape_v[(int64_t)n * total], 0.0f);
                            st[1] = make_float2(tape_v[(int64_t)(n - 1) * total], 0.0f);
                        }
                    } else {
                        const float *h = hr_s + (s * 2 + ((r - 1) & 1)) * 2 * PB + ps;
                        st[0] = make_float2(hp0[(q * 2) * Lay::B], h[0]);
                        st[1] = make_float2(hp0[(q * 2 + 1) * Lay::B], h[PB]);
                        if (n - 2 > 0) {
                            const float *hsum = hsum0 + (int64_t)s * NMAT * hs;
                            cp_async4(hp0 + (q * 2) * Lay::B, hsum + (n - 2) * hs);
                            cp_async4(hp0 + (q * 2 + 1) * Lay::B, hsum + (n - 3) * hs);
                        }
                    }
                    const int imin = n - 1 - lo;             // lowest position with an active cell
                    if (imin < L)
                        tp2_rev_block<H, L, PB, CH, P>(q, X, Pb, st, kc_s + PADK + lo - (n + 1),
                                                       vg0 + (lo - n - 1) * PB, delta, imin);
                    if (NCK > 0 && (n - 1) % ckd == 0 && n - 1 >= ck) {
                        // the reverse of steps >= n-1 leaves rates i <= n-1 untouched
                        const int c = (n - 1) / ckd - 1;
#pragma unroll
                        for (int p = 0; p < L; ++p)
                            if (lo + p > n - 1) X[q * L + p] = ckp[(c * NN + lo + p) * PB];
                    }
                    if (s > 0) {
                        float *h = hr_s + ((s - 1) * 2 + (r & 1)) * 2 * PB + ps;
                        h[0] = st[0].y;
                        h[PB] = st[1].y;
                    }
                }
                __syncthreads();
            }

            // ---- cross-path reduction of the batch: each role reduces the
            // vega and delta rows of its own rates; role 1 the value ----
            if (MODE != Mode::Forward) {
                constexpr int doff = MODE == Mode::Fused ? 1 : 0;
                float *rows = vg_s + Lay::VPAD * PB + pair * 32;
                if (!active) {
#pragma unroll
                    for (int j = 0; j < H; ++j) vg0[((2 * (j / L) + role) * L + j % L) * PB] = 0.0f;
                }
                __syncwarp();
                tp2_rows_reduce<H, L, PB>(rows, lane, role, acc, NOUT, doff + NN);
                __syncwarp();
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int g = (2 * (j / L) + role) * L + j % L;
                    vg0[g * PB] = active ? Pb[j] * il0_s[g] : 0.0f;
                }
                __syncwarp();
                tp2_rows_reduce<H, L, PB>(rows, lane, role, acc, NOUT, doff);
            }
            if (MODE != Mode::Backward && role == 1) {
                const float v = active ? V : 0.0f;
                const float s1 = warp_sum(v), s2 = warp_sum(v * v);
                if (lane == 0) {
                    acc[0] += (double)s1;
                    acc[NOUT] += (double)s2;
                }
            }
            __syncthreads();      // vega rows are restaged by the next batch's payoff
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
    const int S = nn / LMM_TP2_SEG;
    return (size_t)((S - 1) * nmat + tp2_nckpt(nmat, ckpt) * nn) * tp2_paths_per_block(nn);
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

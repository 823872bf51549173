// FP32 thread-per-path LMM kernels for the reference shape NN=80, NMAT=40.
//
// One CUDA thread carries one Monte Carlo path through
//   forward   path_calc_b1   (LiborMarketModel/liborSwaptionGreeks.cpp:34-82)
//   payoff    portfolio_b    (:120-211), adjoint aliasing of :178/:181 fixed
//   reverse   path_calc_b2   (:86-117) plus the vega adjoint (not in the reference)
// with the NN inverse forward rates IL[] = 1/L and the log-adjoints
// Pb[] = L*dV/dL held in registers (the rate index is a compile-time register
// index; the step index is a runtime loop). Carrying 1/L gives
// t = L/(1+delta L) = 1/(IL + delta) from one add and one reciprocal, and
// r = 1/(1+delta L) = 1 - delta t.
//
// Branch-free steps. Step n moves rates i > n only. The per-maturity
// constants are stored with NMAT zero entries in front (k = i-n-1 < 0), so a
// cell with i <= n multiplies IL by 2^0 = 1 and adds 0 to every running sum:
// it is an exact no-op. The forward and the reverse each have ONE unrolled
// body over the rates, cut into chunks (LMM_TPP_CHUNK rates in the forward,
// LMM_TPP_RCHUNK in the reverse): a step enters (forward) or leaves (reverse)
// the body at the chunk holding its first active rate, so at most a chunk
// minus one no-op cells run per step and the code stays small enough for the
// instruction cache.
//
// Reverse sweep without a stored trajectory. With V_i the inclusive drift sum
// of step n (saved per step by the forward), the Euler step runs backwards,
// descending in i as the adjoint needs:
//   IL_{n,i} = IL_{n+1,i} * 2^(a_k (V_i + sqez) + c_k),  V_{i-1} = V_i - delta^2 lambda_k t
// with t = L/(1+delta L), r = 1/(1+delta L). In terms of Pb the reference's
// update (:108-111) becomes
//   S += lambda_k Pb_i,   Pb_i += delta^2 lambda_k t r S     (S is the reference's v1)
// and the vega of cell (n,i), k = i-n-1, is
//   dV/dlambda_k += Pb_i (V_i + sqez - delta lambda_k) + delta^2 t S.
// The kernel carries S' = delta^2 S (S' += delta^2 lambda_k Pb_i, Pb_i +=
// lambda_k r t S'), which saves a multiply per cell. Vega slots of no-op cells
// (k < 0) are spare rows in front of row 0 that are never read; a reverse
// window touches rows k >= 1 - (its chunk of positions), so four suffice.
// The reconstruction is a serial chain (exp -> rcp -> drift sum) per step, so
// steps are processed as a skewed wavefront: cell (n,i) next to cell
// (n-1,i+1), next to (n-2,i+2), ..., G independent chains in one instruction
// stream (G = LMM_TPP_SKEW = 4 in the fused kernel, LMM_TPP_SKEW_BWD = 2 in
// the backward-only kernel). Cell (n-g, i+g) uses the constants and vega row
// that cell (n, i+2g) used 2g positions earlier; they are kept in register
// rings (rev_group_window), so each constant is read from shared memory once
// and each vega row gets one read-modify-write per G cells. The fused forward
// pairs steps the same way (fwd_pair_window).
//
// Cross-path reduction: per warp, each lane sums one output column over the
// warp's 32 paths (shared-memory transpose), then adds into per-warp FP64
// accumulators; each block writes FP64 partial sums that lmm_aux.cu adds in a
// fixed order, so results are bit-reproducible.
#include "lmm_device.cuh"

#include <cuda_bf16.h>

// Threads per block of the fused kernel: 254 registers per thread leave room
// for 8 warps per SM, run as one block of 256 threads so that the block
// barrier keeps all 8 warps on the same stretch of code (GB300, 4,194,304
// paths: 11.73 ms with two 128-thread blocks per SM, 11.54 ms with one of
// 256). The forward-only kernel (168 registers, 12 warps per SM) runs one
// block of 384 threads (4.02 -> 3.76 ms against three of 128), the
// backward-only kernel two blocks of 128 (8.94 ms; one of 256: 9.03 ms).
#ifndef LMM_TPP_BLOCK
#define LMM_TPP_BLOCK 256
#endif
#ifndef LMM_TPP_BLOCK_FWD
#define LMM_TPP_BLOCK_FWD 384
#endif
#ifndef LMM_TPP_BLOCK_BWD
#define LMM_TPP_BLOCK_BWD 128
#endif
// Reverse steps processed together as a skewed wavefront (independent
// reconstruction chains per instruction stream): 2 or 4, in the fused and in
// the backward-only kernel. GB300, 4,194,304 paths: fused 11.29 ms with 2,
// 11.08 ms with 4 (254 registers, no spills); backward-only 8.7 ms with 2,
// 9.2 ms with 4.
#ifndef LMM_TPP_SKEW
#define LMM_TPP_SKEW 4
#endif
#ifndef LMM_TPP_SKEW_BWD
#define LMM_TPP_SKEW_BWD 2
#endif
// Rates per chunk of the single forward body, and of the reverse body (a
// step group leaves it at the first chunk below its lowest active cell).
// GB300, 4,194,304 paths, fused: reverse chunks of 4 / 8 / 16 rates: 10.98 /
// 11.09 / 11.41 ms, and of 2 see LMM_TPP_FSYNC; forward chunks of 4 were
// slower than 8.
#ifndef LMM_TPP_CHUNK
#define LMM_TPP_CHUNK 8
#endif
#ifndef LMM_TPP_RCHUNK
#define LMM_TPP_RCHUNK 2
#endif
#ifndef LMM_TPP_RCHUNK_PHILOX
#define LMM_TPP_RCHUNK_PHILOX 4
#endif
// Forward step pairs between block barriers in the fused kernel, with normals
// from memory and with Philox normals. GB300, 4,194,304 paths: reverse
// chunks 2 and a barrier every second pair 10.90 -> 10.80 ms; with Philox
// normals (16.8M paths) the same settings cost 44.22 -> 44.83 ms, so that
// variant keeps chunks of 4 and a barrier every pair.
#ifndef LMM_TPP_FSYNC
#define LMM_TPP_FSYNC 2
#endif
#ifndef LMM_TPP_FSYNC_PHILOX
#define LMM_TPP_FSYNC_PHILOX 1
#endif
// 1: carry Y = V + sqrt(delta) z as the running drift sum: one add fewer per
// cell in each phase (4.6% faster on GB300), at the price of accumulating the
// drift on top of the normal term (FP32 vs FP64 Greek errors about 15% larger,
// still 1e-6 of the 1e-4 bound).
// 1: a block barrier per forward step pair and reverse step group, so that
// the warps of a block stay on the same stretch of the unrolled bodies
// (instruction cache). Without it, blocks that run long drift apart: on 256
// curve scenarios x 262,144 paths (GB300) 310 ms without, 243 ms with; equal
// on one scenario.
#ifndef LMM_TPP_SYNC
#define LMM_TPP_SYNC 1
#endif
#ifndef LMM_TPP_YRUN
#define LMM_TPP_YRUN 1
#endif
// 1: Kahan-compensated per-thread vega rows (the compensations held as BF16
// rows beside the FP32 rows); 0: plain FP32 read-modify-writes. GB300,
// 4,194,304 paths: 11.04 -> 12.20 ms, and the largest value/delta/vega errors
// against FP64 on the same normals unchanged to three digits (6.95e-7,
// 1.14e-6, 3.32e-6): the rows' rounding is not where the FP32 error comes from.
#ifndef LMM_TPP_VCOMP
#define LMM_TPP_VCOMP 0
#endif
// 1: in the fused kernel the per-maturity constants travel as a kernel
// parameter and the step windows read them from the parameter (constant)
// bank; 0: from shared memory. GB300, 4,194,304 paths: 11.04 -> 10.85 ms
// (232 instead of 252 registers); the forward-only and backward-only kernels
// ran slower that way (3.75 -> 4.82 and 9.07 -> 9.41 ms) and keep shared memory.
#ifndef LMM_TPP_KCPARAM
#define LMM_TPP_KCPARAM 1
#endif
// Positions ahead at which the step windows load the constants of a rate
// from shared memory (0: at the position that first uses them), with the
// normals read from memory and with Philox normals (more live registers).
// GB300, one 256-thread block per SM, 4,194,304 paths: 0 / 1 / 2 / 3 ahead:
// 11.65 / 11.30 / 11.52 / 11.57 ms (HBM normals); 16,777,216 Philox paths
// with reverse groups of four: 0 / 1 / 2 ahead: 46.02 / 46.13 / 46.79 ms.
#ifndef LMM_TPP_PREF
#define LMM_TPP_PREF 1
#endif
#ifndef LMM_TPP_PREF_PHILOX
#define LMM_TPP_PREF_PHILOX 0
#endif


namespace lmm {
namespace {

template <Mode MODE>
__host__ __device__ constexpr int tpp_block()
{
    return MODE == Mode::Fused ? LMM_TPP_BLOCK : (MODE == Mode::Forward ? LMM_TPP_BLOCK_FWD : LMM_TPP_BLOCK_BWD);
}
// Resident blocks the registers are sized for: 8 warps per SM; the
// forward-only kernel holds no adjoints, and 168 registers give it 12.
template <Mode MODE>
__host__ __device__ constexpr int tpp_min_blocks() { return (MODE == Mode::Forward ? 12 : 8) * 32 / tpp_block<MODE>(); }
constexpr bool kYrun = LMM_TPP_YRUN != 0;
template <bool PHILOX>
constexpr int kPref = PHILOX ? LMM_TPP_PREF_PHILOX : LMM_TPP_PREF;

__host__ __device__ constexpr int align16(int x) { return (x + 15) & ~15; }

template <int NN, int NMAT, Mode MODE>
struct TppLayout {
    static constexpr int B = tpp_block<MODE>();
    static constexpr int NW = B / 32;
    static constexpr int M = NN - NMAT;
    static constexpr int PAD = NMAT;                 // k = i-n-1 >= -NMAT
    // Spare vega rows in front of row 0: a reverse window flushes rows
    // k >= 1 - (its chunk of positions) >= -3.
    static constexpr int VPAD = 4;
    static constexpr int NOUT = MODE == Mode::Fused ? 1 + 2 * NN : (MODE == Mode::Forward ? 1 : 2 * NN);
    static constexpr int kc = 0;                                     // float4[PAD+NN]
    static constexpr int il0 = align16(kc + 16 * (PAD + NN));        // float[NN]
    static constexpr int ost = il0 + 4 * NN;                         // int[M+1]
    static constexpr int okf = align16(ost + 4 * (M + 1));           // float[kMaxNopt]
    static constexpr int owf = align16(okf + 4 * kMaxNopt);          // float[kMaxNopt] weights
    static constexpr int okk = align16(owf + 4 * kMaxNopt);          // F2[kMaxNopt]: K delta
    static constexpr int vt = align16(okk + 8 * kMaxNopt);           // float[NMAT][B]
    static constexpr int vt_bytes = MODE == Mode::Fused ? 4 * NMAT * B : 0;
    static constexpr int vg = vt + vt_bytes;                         // float[VPAD+NN][B]
    // Backward/Fused: per-thread vega rows k = -VPAD..NN-1; the payoff also
    // stages the annuity rates there. Forward: only the M staging rows.
    static constexpr int vg_bytes = MODE == Mode::Forward ? 4 * M * B : 4 * (VPAD + NN) * B;
    // LMM_TPP_VCOMP: the vega rows' Kahan compensations, BF16 [VPAD+NN][B].
    static constexpr int vc = vg + vg_bytes;
    static constexpr int vc_bytes = (LMM_TPP_VCOMP && MODE != Mode::Forward) ? 2 * (VPAD + NN) * B : 0;
    static constexpr int acc = align16(vc + vc_bytes);               // double[NW][2*NOUT]
    static constexpr int bytes = acc + 8 * NW * 2 * NOUT;
};

__device__ __forceinline__ float pick4(const float4 &q, int j)
{
    float r = q.x;
    r = j == 1 ? q.y : r;
    r = j == 2 ? q.z : r;
    r = j == 3 ? q.w : r;
    return r;
}

// Running drift sum at the start of a step: V = 0, or Y = sqrt(delta) z.
__device__ __forceinline__ float drift0(float sqez) { return kYrun ? sqez : 0.0f; }

// One forward cell (path_calc_b1 :66-72): drift sum and rate update on the
// inverse rate IL = 1/L. k holds the constants of k = i-n-1 (zero for k < 0:
// an exact no-op).
__device__ __forceinline__ void fwd_cell(float &IL, float &V, const float4 &k, float sqez, float delta)
{
    V = fmaf(k.z, rcp_approx(IL + delta), V);
    IL *= ex2_approx(-fmaf(k.x, kYrun ? V : V + sqez, k.y));
}

// fwd_cell with its reciprocal t = 1/(IL + delta) given.
__device__ __forceinline__ void fwd_cell_t(float &IL, float &V, const float4 &k, float sqez, float t)
{
    V = fmaf(k.z, t, V);
    IL *= ex2_approx(-fmaf(k.x, kYrun ? V : V + sqez, k.y));
}

// 1: the forward cells of one step at positions 2m and 2m+1 share one MUFU
// reciprocal (rcp_pair), in the 80/40 forwards (the fused kernels' skewed
// pairs and the forward-only kernel's single steps). The forward runs two
// MUFU instructions per cell and is bound by the special-function pipe (a
// reciprocal takes it twice as long as an ex2); GB300, split-reverse fused
// kernel: 4,194,304 paths 10.45 -> 10.03 ms, 16.8M Philox paths 43.73 ->
// 42.38 ms.
#ifndef LMM_FWD_RCP2
#define LMM_FWD_RCP2 1
#endif

// One forward step with a single body: rates are grouped in chunks of CH,
// and the step starts at the chunk holding its first active rate n+1 (cells
// of that chunk with i <= n are no-ops). Returns the step's drift sum.
template <int NN, int CH>
__device__ __forceinline__ float fwd_step_chunked(float (&IL)[NN], const float4 *kcn, float sqez,
                                                  float delta, int n)
{
    float V = drift0(sqez);
    const int c0 = (n + 1) / CH;
    static_assert(!LMM_FWD_RCP2 || (CH % 2 == 0 && NN % 2 == 0), "reciprocal pairs (2m, 2m+1) inside chunks");
    float tn = 0.0f;
#pragma unroll
    for (int c = 0; c * CH < NN; ++c) {
        if (c >= c0) {
#pragma unroll
            for (int i = c * CH; i < (c + 1) * CH && i < NN; ++i) {
                if (LMM_FWD_RCP2) {
                    float t;
                    if (i % 2 == 0)
                        rcp_pair(IL[i] + delta, IL[i + 1] + delta, t, tn);
                    else
                        t = tn;
                    if (i >= 1) fwd_cell_t(IL[i], V, kcn[i], sqez, t);
                } else if (i >= 1) {
                    fwd_cell(IL[i], V, kcn[i], sqez, delta);
                }
            }
        }
    }
    return V;
}

// Forward steps n and n+1 with one body over positions p (ascending): cell
// (n, p) and cell (n+1, p-1). The second finds IL_{n+1,p-1} written by cell
// (n, p-1) one position earlier, so the two drift chains are independent
// within a position. Cell (n+1, p-1) has k = p-n-3, the constants loaded for
// cell (n, p-2), so each constant is loaded once per two cells (ring C of
// 3+P slots, loaded P positions ahead of its first use).
// Entered at the chunk holding rate n+1; step n+1's cells below its first
// active rate n+2 see zero constants and are exact no-ops.
// With LMM_FWD_RCP2 the cells of one step at positions 2m and 2m+1 share one
// reciprocal: step n's pair is formed at position 2m (both rates still at
// time n), step n+1's at position 2m+1, right after cell (n, 2m+1) (both
// rates then at time n+1), so every step pairs the same positions as the
// single-step forward (fwd_step_chunked) and rounds the same way; neither
// reciprocal of a pair depends on the drift sums.
// fwd_pair_window_cap also returns the drift sums at rate CAP of both steps
// (the running sum after cell (n, CAP) and after cell (n+1, CAP)); steps whose
// active rates all lie above CAP return their starting value there.
template <int NN, int CH, int P, int CAP>
__device__ __forceinline__ void fwd_pair_window_cap(float (&IL)[NN], const float4 *kcn, float sqez0,
                                                    float sqez1, float delta, int n, float &V0, float &V1,
                                                    float &V0c, float &V1c)
{
    constexpr int R = 3 + P;
    float4 C[R];
    V0 = drift0(sqez0);
    V1 = drift0(sqez1);
    V0c = V0;
    V1c = V1;
    const int c0 = (n + 1) / CH;
    static_assert(!LMM_FWD_RCP2 || (CH % 2 == 0 && NN % 2 == 0), "reciprocal pairs (2m, 2m+1) inside chunks");
    float t0n = 0.0f, t1n = 0.0f;   // LMM_FWD_RCP2: the second reciprocals of the steps' pairs in flight
#pragma unroll
    for (int c = 0; c * CH < NN; ++c) {
        if (c >= c0) {
            if (c == c0) {
#pragma unroll
                for (int j = c * CH - 2; j < c * CH + P; ++j)
                    if (j >= 0 && j < NN) C[j % R] = kcn[j];
                // step n+1's pair below the chunk: rates inactive in step n, unchanged
                if (LMM_FWD_RCP2 && c * CH >= 2) {
                    float ta;
                    rcp_pair(IL[c * CH - 2] + delta, IL[c * CH - 1] + delta, ta, t1n);
                }
            }
#pragma unroll
            for (int p = c * CH; p < (c + 1) * CH && p < NN; ++p) {
                if (p + P < NN) C[(p + P) % R] = kcn[p + P];
                if (LMM_FWD_RCP2) {
                    float t;
                    if (p % 2 == 0) {
                        rcp_pair(IL[p] + delta, IL[p + 1] + delta, t, t0n);
                    } else {
                        t = t0n;
                    }
                    if (p >= 1) fwd_cell_t(IL[p], V0, C[p % R], sqez0, t);
                    if (p % 2 == 1) {          // step n+1's pair (p-1, p), both now at time n+1
                        float ta;
                        rcp_pair(IL[p - 1] + delta, IL[p] + delta, ta, t1n);
                        if (p - 1 >= 1) fwd_cell_t(IL[p - 1], V1, C[(p + R - 2) % R], sqez1, ta);
                    } else if (p - 1 >= 1) {
                        fwd_cell_t(IL[p - 1], V1, C[(p + R - 2) % R], sqez1, t1n);
                    }
                } else {
                    if (p >= 1) fwd_cell(IL[p], V0, C[p % R], sqez0, delta);
                    if (p - 1 >= 1) fwd_cell(IL[p - 1], V1, C[(p + R - 2) % R], sqez1, delta);
                }
                if (p == CAP) V0c = V0;
                if (p == CAP + 1) V1c = V1;
            }
        }
    }
    if (LMM_FWD_RCP2)
        fwd_cell_t(IL[NN - 1], V1, C[(NN - 2) % R], sqez1, t1n);
    else
        fwd_cell(IL[NN - 1], V1, C[(NN - 2) % R], sqez1, delta);
}

template <int NN, int CH, int P>
__device__ __forceinline__ void fwd_pair_window(float (&IL)[NN], const float4 *kcn, float sqez0,
                                                float sqez1, float delta, int n, float &V0, float &V1)
{
    float V0c, V1c;
    fwd_pair_window_cap<NN, CH, P, -2>(IL, kcn, sqez0, sqez1, delta, n, V0, V1, V0c, V1c);
}

struct RevStep {
    float V, S, sqez;   // drift sum, delta^2 times the reference's v1, sqrt(delta) z
    const float4 *kc;   // kc[i]: constants of k = i-n-1
    float *vg;          // vg[i*B]: this thread's vega slot of k = i-n-1
    unsigned short *vc; // vc[i*B]: its BF16 compensation (LMM_TPP_VCOMP)
};

__device__ __forceinline__ float bf16_bits_to_float(unsigned short b) { return __uint_as_float((unsigned)b << 16); }

// Kahan step s += x with the compensation c held as BF16 bits: c is the
// negated rounding error of the previous additions, so s - c is the sum.
__device__ __forceinline__ void kahan_add_bf16c(float &s, unsigned short &cb, float x)
{
    const float y = __fsub_rn(x, bf16_bits_to_float(cb));
    const float t = __fadd_rn(s, y);
    cb = __bfloat16_as_ushort(__float2bfloat16_rn(__fsub_rn(__fsub_rn(t, s), y)));
    s = t;
}

// 1: the reverse windows keep d = -delta*lambda_k beside each constant of
// their ring (one multiply per position, shared by the G cells of the
// position), and the cell forms lambda(1 - delta t) as one FMA,
// fma(d, t, lambda), instead of an FMA and a multiply. Per kernel: k_tpp,
// k_tps, k_tpq.
#ifndef LMM_TPP_DCONST
#define LMM_TPP_DCONST 1
#endif
#ifndef LMM_TPS_DCONST
#define LMM_TPS_DCONST 1
#endif
#ifndef LMM_TPQ_DCONST
#define LMM_TPQ_DCONST 0
#endif

// One reverse cell (path_calc_b2 :105-111 in log-adjoint form) + vega, with
// its constants (k, and d = -delta*k.w with DC) and vega partial sum
// passed in from the window.
template <int NN, bool DC>
__device__ __forceinline__ void rev_cell(float (&IL)[NN], float (&Pb)[NN], RevStep &s, int i,
                                         const float4 &k, float d, float &acc, float delta)
{
    const float y = kYrun ? s.V : s.V + s.sqez;
    const float iln = IL[i] * ex2_approx(fmaf(k.x, y, k.y));
    const float t = rcp_approx(iln + delta);
    s.V = fmaf(-k.z, t, s.V);
    const float pb = Pb[i];
    s.S = fmaf(k.z, pb, s.S);
    const float tS = t * s.S;
    if (DC) {
        acc += fmaf(pb, y + d, tS);
        Pb[i] = fmaf(fmaf(d, t, k.w), tS, pb);
    } else {
        acc += fmaf(pb, fmaf(-delta, k.w, y), tS);
        Pb[i] = fmaf(k.w * fmaf(-delta, t, 1.0f), tS, pb);
    }
    IL[i] = iln;
}

// Reverse steps n, n-1, ..., n-G+1 with a single body over positions
// NN-1 .. -(G-1): cell (n-g, i+g) at position i, which finds
// IL_{n-g+1, i+g} written by cell (n-g+1, i+g) one position earlier. With
// j = i+2g, the constants of cell (n-g, i+g) are st[0].kc[j] and its vega row
// is st[0].vg[j*B] (k = j-n-1 of step n): C holds the constants from
// position j+P (load, P positions ahead of the first use) and A the vega
// partial sum from position j, both to position j-2(G-1) (last use, vega
// flush), in rings of 2G-1+P slots indexed j mod (2G-1+P), so that each
// constant is loaded once and each vega row gets one read-modify-write per
// G cells. The body is left at the first
// chunk of CH positions lying wholly below the lowest active position
// n-2G+3. A vega row is valid (k >= 0) for all or none of its G
// contributors, and all contributors of a valid row sit at or above that
// position, so leaving there is exact: the rows still open are spare rows
// (k < 0), which are never read.
template <int NN, int B, int G, int CH, int P>
__device__ __forceinline__ void rev_group_window(float (&IL)[NN], float (&Pb)[NN], RevStep (&st)[G],
                                                 float delta, int n)
{
    constexpr int JMAX = NN + G - 2;
    constexpr int W = 2 * G - 1 + P;
    const float4 *kc = st[0].kc;
    float *vg = st[0].vg;
    unsigned short *vc = st[0].vc;
    float4 C[W];
    float D[W];
    float A[W];
#pragma unroll
    for (int j = NN - P; j <= JMAX; ++j) {
        C[j % W] = kc[j];
        D[j % W] = -delta * C[j % W].w;
        if (j >= NN) A[j % W] = 0.0f;
    }
    const int imin = n - 2 * G + 3;
#pragma unroll
    for (int q = 0; q * CH < NN + G - 1; ++q) {
        const int top = NN - 1 - q * CH;
        if (top < imin) return;
#pragma unroll
        for (int i = top; i > top - CH && i >= -(G - 1); --i) {
            if (i - P >= 1) {
                C[(i - P) % W] = kc[i - P];
                D[(i - P) % W] = -delta * C[(i - P) % W].w;
            }
            if (i >= 1) A[i % W] = 0.0f;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (i + g >= 1 && i + g <= NN - 1) {
                    const int j = i + 2 * g;
                    rev_cell<NN, LMM_TPP_DCONST != 0>(IL, Pb, st[g], i + g, C[j % W], D[j % W], A[j % W], delta);
                }
            }
            const int jf = i + 2 * (G - 1);
            if (jf >= 1 && jf <= JMAX) {
                if (LMM_TPP_VCOMP)
                    kahan_add_bf16c(vg[jf * B], vc[jf * B], A[jf % W]);
                else
                    vg[jf * B] += A[jf % W];
            }
        }
    }
}

// Portfolio value, portfolio_b :133-171 and :186-197, from the inverse rates.
// The factors 1/(1+delta L) come from t = 1/(IL + delta) (MUFU reciprocal,
// within 1 ulp) as 1 - delta t while delta L < 1 (within 0.5 + delta L ulp:
// about 0.5 ulp for ordinary rates) and as IL t above (within 2.5 ulp). The
// discount and annuity products, the annuity sum, the swap values and the
// payoff sum are double-FP32 (F2, lmm_device.cuh): FP64-like products on
// the FP32 pipe (FP64 products cost 10% of the fused kernel's time on
// GB300). Returns the discounted value; *disc_out receives the discount
// factor, *mask_out which swaptions (in grouped order) paid, and Bst[m*B] (if
// given) the annuity factors B[m] of :139 rounded to FP32, for the adjoint.
// payoff_forward_staged is its annuity part, from the discount product
// `disc` and the M annuity rates staged in ILst[m*B].
template <int M, int B>
__device__ __forceinline__ float payoff_forward_staged(F2 disc, float delta, const int *ost, const F2 *oKd,
                                                       const float *oWf, float *disc_out, float *Bst,
                                                       const float *ILst, unsigned long long *mask_out)
{
    F2 b{1.0f, 0.0f}, sb{0.0f, 0.0f}, vs{0.0f, 0.0f};
    unsigned long long mask = 0ull;
#pragma unroll 1
    for (int m = 0; m < M; ++m) {
        b = f2_mul(b, bond_ratio(ILst[m * B], delta));
        sb = f2_add(sb, b);                                   // annuity / delta
        if (Bst) Bst[m * B] = b.hi;
        const int o1 = ost[m + 1];
#pragma unroll 1
        for (int o = ost[m]; o < o1; ++o) {
            const float sw = f2_swap_value(oKd[o], sb, b);
            if (sw < 0.0f) {
                vs = f2_add(vs, (-100.0f * sw) * oWf[o]);
                mask |= 1ull << o;
            }
        }
    }
    *disc_out = disc.hi;
    *mask_out = mask;
    const F2 v = f2_mul(vs, disc);
    return __fadd_rn(v.hi, v.lo);
}

template <int NN, int NMAT, int B>
__device__ __forceinline__ float payoff_forward(const float (&IL)[NN], float delta, const int *ost,
                                                const F2 *oKd, const float *oWf, float *disc_out,
                                                float *Bst, float *ILst, unsigned long long *mask_out)
{
    constexpr int M = NN - NMAT;
    F2 disc{1.0f, 0.0f};
#pragma unroll
    for (int n = 0; n < NMAT; ++n) disc = f2_mul(disc, bond_ratio(IL[n], delta));
    // The annuity recursion runs as a rolled loop over the rates staged in
    // shared memory: one copy of its code instead of one per maturity
    // (instruction cache).
#pragma unroll
    for (int m = 0; m < M; ++m) ILst[m * B] = IL[NMAT + m];
    return payoff_forward_staged<M, B>(disc, delta, ost, oKd, oWf, disc_out, Bst, ILst, mask_out);
}

// Payoff adjoint, portfolio_b :173-184 (with the rate and its adjoint kept
// apart) and :199-209, seeded with vbar = dOut/dV. Writes the log-adjoints
// Pb[i] = L_i dOut/dL_i of the terminal rates. Bst[m*B] holds B[m] from the
// forward: rebuilding B[m-1] = B[m](1 + delta L) backwards from the last,
// smallest factor would underflow FP32 on paths whose rates grow large.
template <int NN, int NMAT, int B>
__device__ __forceinline__ void payoff_adjoint_stage(float vbar, float disc, const float *Bst, float *ILst,
                                                     unsigned long long mask, float delta, const int *ost,
                                                     const float *oKf, const float *oWf)
{
    constexpr int M = NN - NMAT;
    const float scale = -vbar * disc * delta;
    float Sb = 0.0f, Bb = 0.0f;
    // Rolled over the rates staged by payoff_forward; each staged rate is
    // replaced by its log-adjoint, copied into Pb[] afterwards.
#pragma unroll 1
    for (int m = M - 1; m >= 0; --m) {
        const float il = ILst[m * B];
        const float t = rcp_approx(il + delta);               // L/(1+delta L)
        const float r = bond_ratio_t(il, delta, t);
        const float Bm = Bst[m * B];
        const int o1 = ost[m + 1];
#pragma unroll 1
        for (int o = ost[m]; o < o1; ++o) {
            if ((mask >> o) & 1ull) {
                Sb -= (100.0f * oKf[o]) * oWf[o];
                Bb -= 100.0f * oWf[o];
            }
        }
        Bb = fmaf(delta, Sb, Bb);
        ILst[m * B] = scale * Bb * Bm * t;
        Bb *= r;
    }
}

template <int NN, int NMAT, int B>
__device__ __forceinline__ void payoff_adjoint(const float (&IL)[NN], float (&Pb)[NN], float vbar,
                                               float V, float disc, const float *Bst, float *ILst,
                                               unsigned long long mask, float delta,
                                               const int *ost, const float *oKf, const float *oWf)
{
    constexpr int M = NN - NMAT;
    payoff_adjoint_stage<NN, NMAT, B>(vbar, disc, Bst, ILst, mask, delta, ost, oKf, oWf);
#pragma unroll
    for (int m = 0; m < M; ++m) Pb[NMAT + m] = ILst[m * B];
    const float vs = -vbar * V * delta;
#pragma unroll
    for (int n = 0; n < NMAT; ++n) {
        Pb[n] = vs * rcp_approx(IL[n] + delta);
    }
}

// Column sums of a warp's 32 shared-memory columns: lane handles outputs
// k = lane, lane+32, ...; the (t+lane)&31 rotation keeps the 32 lanes on 32
// different banks. Adds sums (TwoSum-compensated, LMM_COMP_SUMS) and sums of
// squares into FP64 accumulators; vc: the rows' BF16 Kahan compensations.
template <int NN, int B>
__device__ __forceinline__ void column_reduce(const float *vg, int warp, int lane, double *acc,
                                              int nout, int off, const unsigned short *vc = nullptr)
{
    for (int k = lane; k < NN; k += 32) {
        const float *col = vg + k * B + warp * 32;
        const unsigned short *ccol = vc ? vc + k * B + warp * 32 : nullptr;
        float a = 0.0f, c = 0.0f, a2 = 0.0f;
#pragma unroll 8
        for (int t = 0; t < 32; ++t) {
            const float x = ccol ? __fsub_rn(col[(t + lane) & 31], bf16_bits_to_float(ccol[(t + lane) & 31]))
                                 : col[(t + lane) & 31];
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

// Forward over all steps. The fused kernel runs steps in skewed pairs; the
// forward-only kernel runs single steps (the pair's extra live constants
// cost it more occupancy than they save) and writes the tape.
template <int NN, int NMAT, bool PHILOX, Mode MODE>
__device__ __forceinline__ void forward_all(float (&IL)[NN], const float4 *kc0, float4 &zq,
                                            float4 &zq_next, const float *zp, uint64_t seed,
                                            uint64_t gpath, float sqd, float delta, float *vt_s,
                                            float *tape_v, int64_t total, bool active)
{
    constexpr int B = tpp_block<MODE>();
    if constexpr (MODE == Mode::Fused) {
        static_assert(NMAT % 2 == 0, "paired forward steps");
        for (int n = 0; n < NMAT; n += 2) {
            if (LMM_TPP_SYNC && (n % (2 * (PHILOX ? LMM_TPP_FSYNC_PHILOX : LMM_TPP_FSYNC))) == 0) __syncthreads();
            if ((n & 3) == 0) {
                zq = zq_next;
                if ((n >> 2) + 1 < NMAT / 4) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) + 1);
            }
            const float sqez0 = sqd * ((n & 2) ? zq.z : zq.x);
            const float sqez1 = sqd * ((n & 2) ? zq.w : zq.y);
            float V0, V1;
            fwd_pair_window<NN, LMM_TPP_CHUNK, kPref<PHILOX>>(IL, kc0 - (n + 1), sqez0, sqez1, delta, n, V0, V1);
            vt_s[n * B] = V0;
            vt_s[(n + 1) * B] = V1;
        }
    } else {
        for (int n = 0; n < NMAT; ++n) {
            if ((n & 3) == 0) {
                zq = zq_next;
                if ((n >> 2) + 1 < NMAT / 4) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) + 1);
            }
            const float sqez = sqd * pick4(zq, n & 3);
            const float V = fwd_step_chunked<NN, LMM_TPP_CHUNK>(IL, kc0 - (n + 1), sqez, delta, n);
            if (active) tape_v[(int64_t)n * total] = V;
        }
    }
}

// Reverse over all steps, in groups of G steps from the last.
template <int NN, int NMAT, bool PHILOX, Mode MODE>
__device__ __forceinline__ void reverse_all(float (&IL)[NN], float (&Pb)[NN], const float4 *kc0,
                                            float *vg0, unsigned short *vc0, float4 &zq, float4 &zq_next, const float *zp,
                                            uint64_t seed, uint64_t gpath, float sqd, float delta,
                                            const float *vt_s, const float *tape_v, int64_t total)
{
    constexpr int G = MODE == Mode::Fused ? LMM_TPP_SKEW : LMM_TPP_SKEW_BWD;
    static_assert(NMAT % G == 0 && (G == 2 || G == 4), "whole step groups");
    constexpr int RCH = PHILOX ? LMM_TPP_RCHUNK_PHILOX : LMM_TPP_RCHUNK;
    static_assert(RCH - 1 <= TppLayout<NN, NMAT, MODE>::VPAD, "the windows' spare vega rows lie inside the table");
    constexpr int B = tpp_block<MODE>();
    for (int n = NMAT - 1; n > 0; n -= G) {
        if (LMM_TPP_SYNC) __syncthreads();
        // The drift sums carry the normal term (kYrun): the reverse needs no
        // normals. Skipped explicitly: left to the compiler, the unused
        // loads and Philox evaluations stayed in (GB300, 4,194,304 paths:
        // 11.00 -> 10.92 ms; 16.8M Philox paths: 46.11 -> 44.29 ms).
        if (!kYrun && (n & 3) == 3) {
            zq = zq_next;
            if ((n >> 2) > 0) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) - 1);
        }
        RevStep st[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int m = n - g;
            st[g].sqez = kYrun ? 0.0f : sqd * pick4(zq, m & 3);
            st[g].V = MODE == Mode::Fused ? vt_s[m * B] : tape_v[(int64_t)m * total];
            st[g].S = 0.0f;
            st[g].kc = kc0 - (m + 1);
            st[g].vg = vg0 - (m + 1) * B;
            st[g].vc = vc0 - (m + 1) * B;
        }
        rev_group_window<NN, B, G, RCH, kPref<PHILOX>>(IL, Pb, st, delta, n);
    }
}

// The per-maturity constants with NMAT zero rows in front (k = i-n-1 < 0),
// passed by value as a kernel parameter.
template <int NN, int NMAT>
struct TppConst {
    float4 v[NMAT + NN];
};

template <int NN, int NMAT, bool PHILOX, Mode MODE>
__global__ void __launch_bounds__(tpp_block<MODE>(), tpp_min_blocks<MODE>())
k_tpp(const DevModel m, const float *__restrict__ z, uint64_t seed, int64_t path0, const Work w,
      float *__restrict__ tape, const double *__restrict__ vbar, const __grid_constant__ TppConst<NN, NMAT> kp)
{
    using Lay = TppLayout<NN, NMAT, MODE>;
    constexpr int B = Lay::B, M = Lay::M, NOUT = Lay::NOUT, PAD = Lay::PAD;
    static_assert(NMAT % 4 == 0, "normals are read in aligned quads");
    static_assert(2 * M <= NN, "annuity staging rows inside the vega rows");
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *kc_s = reinterpret_cast<float4 *>(smem + Lay::kc);
    float *il0_s = reinterpret_cast<float *>(smem + Lay::il0);
    int *ost_s = reinterpret_cast<int *>(smem + Lay::ost);
    float *okf_s = reinterpret_cast<float *>(smem + Lay::okf);
    float *owf_s = reinterpret_cast<float *>(smem + Lay::owf);
    F2 *okk_s = reinterpret_cast<F2 *>(smem + Lay::okk);
    float *vt_s = reinterpret_cast<float *>(smem + Lay::vt);
    float *vg_s = reinterpret_cast<float *>(smem + Lay::vg);
    double *acc_s = reinterpret_cast<double *>(smem + Lay::acc);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr bool kKcParam = LMM_TPP_KCPARAM && MODE == Mode::Fused;
    if (!kKcParam) {
        for (int i = tid; i < PAD + NN; i += B) {
            const int k = i - PAD;
            kc_s[i] = k < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : m.kc[k];
        }
    }
    for (int i = tid; i <= M; i += B) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += B) {
        okf_s[i] = m.optKf[i];
        owf_s[i] = m.optWf[i];
        okk_s[i] = f2_from(m.optKd[i] * m.deltad);
    }
    double *acc = acc_s + warp * 2 * NOUT;
    const float delta = m.delta, sqd = m.sqd;
    const int64_t total = (int64_t)m.nscen * w.paths;
    const float4 *kc0 = (kKcParam ? kp.v : kc_s) + PAD;
    float *vg0 = vg_s + Lay::VPAD * B + tid;
    unsigned short *vc_s = reinterpret_cast<unsigned short *>(smem + Lay::vc);
    unsigned short *vc0 = vc_s + Lay::VPAD * B + tid;
    float *vt0 = vt_s + tid;

    // Units (scenario, item) in a block-stride loop: with a grid of one wave,
    // every block starts together and runs equal units, so the blocks of an
    // SM stay on the same stretch of code (instruction cache).
    const int units = m.nscen * w.items;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int scen = unit / w.items, item = unit % w.items;
        __syncthreads();          // the previous unit's reads of l0/il0/acc are done
        for (int i = tid; i < NN; i += B) {
            il0_s[i] = m.invL0f[scen * NN + i];
        }
        for (int i = tid; i < Lay::NW * 2 * NOUT; i += B) acc_s[i] = 0.0;
        __syncthreads();

        const int64_t ibase = (int64_t)item * w.ppt * B;
        const float vb = MODE == Mode::Backward ? (float)vbar[scen] : 1.0f;
        for (int j = 0; j < w.ppt; ++j) {
            if (ibase + (int64_t)j * B >= w.paths) break;          // block-uniform
            const int64_t pl = ibase + (int64_t)j * B + tid;
            const bool active = pl < w.paths;
            const int64_t pc = active ? pl : w.paths - 1;
            const int64_t tp = (int64_t)scen * w.paths + pc;
            const float *zp = PHILOX ? nullptr : z + pc * NMAT;
            const uint64_t gpath = (uint64_t)(path0 + pc);
            float *tape_v = tape ? tape + (int64_t)NN * total + tp : nullptr;

            float IL[NN];
            float Pb[NN];
            float4 zq, zq_next;

            if (MODE != Mode::Backward) {
#pragma unroll
                for (int i = 0; i < NN; ++i) IL[i] = il0_s[i];
                zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, 0);
                forward_all<NN, NMAT, PHILOX, MODE>(IL, kc0, zq, zq_next, zp, seed, gpath, sqd, delta, vt0,
                                                    tape_v, total, active);
                if (MODE == Mode::Forward && active) {
#pragma unroll
                    for (int i = 0; i < NN; ++i) tape[(int64_t)i * total + tp] = IL[i];
                }
            } else {
#pragma unroll
                for (int i = 0; i < NN; ++i) IL[i] = tape[(int64_t)i * total + tp];
            }

            float disc = 1.0f;
            unsigned long long mask = 0ull;
            // B[m] goes to this thread's vega column, unused until the reverse sweep.
            float *Bst = MODE == Mode::Forward ? nullptr : vg0;
            // Staging rows for the annuity rates: vega rows k = M..2M-1 (free
            // until the reverse sweep), or the forward kernel's own M rows.
            float *ILst = MODE == Mode::Forward ? vg_s + tid : vg0 + M * B;
            const float V = payoff_forward<NN, NMAT, B>(IL, delta, ost_s, okk_s, owf_s, &disc, Bst, ILst, &mask);

            if (MODE != Mode::Forward) {
                payoff_adjoint<NN, NMAT, B>(IL, Pb, vb, V, disc, Bst, ILst, mask, delta, ost_s, okf_s, owf_s);
#pragma unroll
                for (int k = 0; k < NN; ++k) vg0[k * B] = 0.0f;
                if (LMM_TPP_VCOMP) {
#pragma unroll
                    for (int k = 0; k < NN; ++k) vc0[k * B] = 0;
                }
                if (!kYrun) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, NMAT / 4 - 1);
                reverse_all<NN, NMAT, PHILOX, MODE>(IL, Pb, kc0, vg0, vc0, zq, zq_next, zp, seed, gpath, sqd, delta,
                                                    vt0, tape_v, total);
            }

            // ---- cross-path reduction of this batch of B paths ----
            if (MODE != Mode::Backward) {
                const float v = active ? V : 0.0f;
                const float s1 = warp_sum(v), s2 = warp_sum(v * v);
                if (lane == 0) {
                    acc[0] += (double)s1;
                    acc[NOUT] += (double)s2;
                }
            }
            if (MODE != Mode::Forward) {
                constexpr int voff = MODE == Mode::Fused ? 1 + NN : NN;
                constexpr int doff = MODE == Mode::Fused ? 1 : 0;
                float *vgw = vg_s + Lay::VPAD * B;
                if (!active) {
#pragma unroll
                    for (int k = 0; k < NN; ++k) vg0[k * B] = 0.0f;
                    if (LMM_TPP_VCOMP) {
#pragma unroll
                        for (int k = 0; k < NN; ++k) vc0[k * B] = 0;
                    }
                }
                __syncwarp();
                column_reduce<NN, B>(vgw, warp, lane, acc, NOUT, voff, LMM_TPP_VCOMP ? vc_s + Lay::VPAD * B : nullptr);
                __syncwarp();
#pragma unroll
                for (int i = 0; i < NN; ++i) vg0[i * B] = active ? Pb[i] * il0_s[i] : 0.0f;
                __syncwarp();
                column_reduce<NN, B>(vgw, warp, lane, acc, NOUT, doff);
                __syncwarp();
            }
        }

        __syncthreads();
        for (int o = tid; o < 2 * NOUT; o += B) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < Lay::NW; ++q) s += acc_s[q * 2 * NOUT + o];
            w.partial[(size_t)unit * 2 * NOUT + o] = s;
        }
    }  // units
}

// ---------------------------------------------------------------------------
// k_tps: the fused kernel with the reverse sweep split over the two rate
// halves, for more warps per SM.
//
// In k_tpp the reverse sweep holds all NN inverse rates and NN log-adjoints
// in registers (232 per thread), which allows 8 warps per SM: two per
// scheduler, too few to cover the cells' ex2 -> rcp dependency chains. The
// forward needs only the NN rates. Here the reverse runs as two passes over
// the halves of the rates, one after the other in the same thread:
//   R1: rates H..NN-1 for every step, starting each step from the full drift
//       sum (saved by the forward, shared memory) and an empty suffix sum;
//       it leaves, per step, the suffix sum at rate H in the scratch;
//   R2: rates 0..H-1 for every step, starting each step from the forward's
//       drift sum at rate H-1 (scratch) and R1's suffix sum.
// The lower half's terminal rates wait in the scratch during R1, the upper
// half's deltas during R2, so at most H rates and H log-adjoints are live:
// about 150 registers, 12 warps per SM (three per scheduler). The cells, the
// step windows (G = 4 reverse steps per body, constants and vega partial sums
// in rings), the payoff and the reductions are those of k_tpp; a vega row
// takes read-modify-writes from both passes.
// The scratch (per block of the wave, FP32, [row][B] so that a warp's 32
// paths are contiguous): the drift sums at rate H-1 [NMAT], R1's suffix sums
// at rate H [NMAT], the lower half's terminal inverse rates [H] and the upper
// half's deltas [NN-H]. It is written and read back by the same thread within
// one batch of B paths, and stays in L2 (about 37 MB per wave at NN = 80).
// ---------------------------------------------------------------------------
#ifndef LMM_TPS_BLOCK
#define LMM_TPS_BLOCK 384
#endif
// Barriers in k_tps's step loops (0: none; they keep the warps of a block on
// the same stretch of code; every array the loops touch is per thread).
#ifndef LMM_TPS_SYNC
#define LMM_TPS_SYNC LMM_TPP_SYNC
#endif
// 1: k_tps reads the per-maturity constants from the kernel-parameter bank;
// 0: from shared memory.
#ifndef LMM_TPS_KCPARAM
#define LMM_TPS_KCPARAM 1
#endif
// Forward step pairs between block barriers, reverse chunk lengths and the
// constant prefetch distance of k_tps, with normals from memory and with
// Philox normals (the k_tpp kernels keep LMM_TPP_*). GB300, with the shared
// forward reciprocals: 4,194,304 paths, a forward barrier every 2, 4, 8 pairs
// or once per batch (20 pairs) 10.01, 9.88, 9.86, 9.83 ms; constants at the
// position of use 9.98 against 9.88 (one ahead); 16.8M Philox paths, 42.35 ms
// as LMM_TPP_*, 41.54 with 2-position reverse chunks and constants one ahead,
// 41.33 / 41.24 / 41.15 / 40.81 with a forward barrier every 2 / 4 / 8 pairs /
// once per batch. 256 curves x 262,144 paths with these settings: 163.5 ms
// (166.2 before). Reverse chunks of one position (the body left right below
// the lowest active position): 9.80 -> 9.78 ms, Philox 40.62 -> 40.58 ms.
#ifndef LMM_TPS_FSYNC
#define LMM_TPS_FSYNC 20
#endif
// Reverse step groups between block barriers. GB300: every group, every
// second, fourth, tenth: 4,194,304 paths 9.84, 9.81, 9.83, 9.92 ms; 16.8M
// Philox paths 40.84 / 40.62 ms (every group / every second).
#ifndef LMM_TPS_RSYNC
#define LMM_TPS_RSYNC 2
#endif
#ifndef LMM_TPS_FSYNC_PHILOX
#define LMM_TPS_FSYNC_PHILOX 20
#endif
#ifndef LMM_TPS_RCHUNK
#define LMM_TPS_RCHUNK 1
#endif
#ifndef LMM_TPS_RCHUNK_PHILOX
#define LMM_TPS_RCHUNK_PHILOX 1
#endif
#ifndef LMM_TPS_PREF
#define LMM_TPS_PREF LMM_TPP_PREF
#endif
#ifndef LMM_TPS_PREF_PHILOX
#define LMM_TPS_PREF_PHILOX 1
#endif

template <int NN, int NMAT>
struct TpsLayout {
    static constexpr int B = LMM_TPS_BLOCK;
    static constexpr int NW = B / 32;
    static constexpr int H = NN / 2;
    static constexpr int M = NN - NMAT;
    static constexpr int VPAD = 4;
    static constexpr int NOUT = 1 + 2 * NN;
    static constexpr int il0 = 0;                                    // float[NN]
    static constexpr int ost = align16(il0 + 4 * NN);                // int[M+1]
    static constexpr int okf = align16(ost + 4 * (M + 1));           // float[kMaxNopt]
    static constexpr int owf = align16(okf + 4 * kMaxNopt);          // float[kMaxNopt]
    static constexpr int okk = align16(owf + 4 * kMaxNopt);          // F2[kMaxNopt]
    static constexpr int vt = align16(okk + 8 * kMaxNopt);           // float[NMAT][B] full drift sums
    static constexpr int vg = vt + 4 * NMAT * B;                     // float[VPAD+NN][B] vega rows
    static constexpr int kc = align16(vg + 4 * (VPAD + NN) * B);     // float4[NMAT+NN] (!LMM_TPS_KCPARAM)
    static constexpr int acc = align16(kc + (LMM_TPS_KCPARAM ? 0 : 16 * (NMAT + NN)));   // double[NW][2*NOUT]
    static constexpr int bytes = acc + 8 * NW * 2 * NOUT;
    // scratch rows per block
    static constexpr int s_v = 0, s_s = NMAT, s_il = 2 * NMAT, s_d = 2 * NMAT + H, rows = 2 * NMAT + NN;
    static_assert(NN % 2 == 0 && NMAT == H, "the upper half is the annuity rates");
};


// Reverse steps n .. n-G+1 over one half of the rates, rates LO .. LO+H-1 held
// in X[], Pb[] at local positions 0 .. H-1: rev_group_window on a block of
// rates. st[0].kc and st[0].vg point at step n's constants and vega rows of
// the block's local position 0. The upper half (LO > 0) is active in every
// step (n < NMAT <= LO), so its body runs to the last position and flushes
// the vega slots of positions 0 .. G-2, which hold its cells' sums; the lower
// half (LO = 0) leaves the body as rev_group_window does.
template <int H, int LO, int B, int G, int CH, int P>
__device__ __forceinline__ void rev_half_window(float (&X)[H], float (&Pb)[H], RevStep (&st)[G], float delta,
                                                int n)
{
    constexpr int JMAX = H + G - 2;
    constexpr int W = 2 * G - 1 + P;
    const float4 *kc = st[0].kc;
    float *vg = st[0].vg;
    float4 C[W];
    float D[W];
    float A[W];
#pragma unroll
    for (int j = H - P; j <= JMAX; ++j) {
        C[j % W] = kc[j];
        D[j % W] = -delta * C[j % W].w;
        if (j >= H) A[j % W] = 0.0f;
    }
    const int imin = n - 2 * G + 3 - LO;     // lowest local position with an active cell
#pragma unroll
    for (int q = 0; q * CH < H + G - 1; ++q) {
        const int top = H - 1 - q * CH;
        if (LO == 0 && top < imin) return;
#pragma unroll
        for (int i = top; i > top - CH && i >= -(G - 1); --i) {
            if (i - P >= (LO > 0 ? 0 : 1)) {
                C[(i - P) % W] = kc[i - P];
                D[(i - P) % W] = -delta * C[(i - P) % W].w;
            }
            if (i >= (LO > 0 ? 0 : 1)) A[i % W] = 0.0f;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (i + g >= (LO > 0 ? 0 : 1) && i + g <= H - 1) {
                    const int j = i + 2 * g;
                    rev_cell<H, LMM_TPS_DCONST != 0>(X, Pb, st[g], i + g, C[j % W], D[j % W], A[j % W], delta);
                }
            }
            const int jf = i + 2 * (G - 1);
            if (jf >= (LO > 0 ? 0 : 1) && jf <= JMAX) vg[jf * B] += A[jf % W];
        }
    }
    if (LO > 0) {
#pragma unroll
        for (int j = 0; j < G - 1; ++j) vg[j * B] += A[j % W];
    }
}

template <int NN, int NMAT, bool PHILOX>
__global__ void __launch_bounds__(LMM_TPS_BLOCK, 384 / LMM_TPS_BLOCK)
k_tps(const DevModel m, const float *__restrict__ z, uint64_t seed, int64_t path0, const Work w,
      float *__restrict__ scr, const __grid_constant__ TppConst<NN, NMAT> kp)
{
    using Lay = TpsLayout<NN, NMAT>;
    constexpr int B = Lay::B, H = Lay::H, M = Lay::M, NOUT = Lay::NOUT, PAD = NMAT;
    constexpr int G = LMM_TPP_SKEW, RCH = PHILOX ? LMM_TPS_RCHUNK_PHILOX : LMM_TPS_RCHUNK;
    constexpr int PF = PHILOX ? LMM_TPS_PREF_PHILOX : LMM_TPS_PREF;
    static_assert(NMAT % 4 == 0 && NMAT % G == 0, "normals in quads, reverse steps in groups");
    static_assert(RCH - 1 <= Lay::VPAD, "the windows' spare vega rows lie inside the table");
    extern __shared__ __align__(16) unsigned char smem[];
    float *il0_s = reinterpret_cast<float *>(smem + Lay::il0);
    int *ost_s = reinterpret_cast<int *>(smem + Lay::ost);
    float *okf_s = reinterpret_cast<float *>(smem + Lay::okf);
    float *owf_s = reinterpret_cast<float *>(smem + Lay::owf);
    F2 *okk_s = reinterpret_cast<F2 *>(smem + Lay::okk);
    float *vt_s = reinterpret_cast<float *>(smem + Lay::vt);
    float *vg_s = reinterpret_cast<float *>(smem + Lay::vg);
    double *acc_s = reinterpret_cast<double *>(smem + Lay::acc);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i <= M; i += B) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += B) {
        okf_s[i] = m.optKf[i];
        owf_s[i] = m.optWf[i];
        okk_s[i] = f2_from(m.optKd[i] * m.deltad);
    }
    double *acc = acc_s + warp * 2 * NOUT;
    const float delta = m.delta, sqd = m.sqd;
    float4 *kc_s = reinterpret_cast<float4 *>(smem + Lay::kc);
    if (!LMM_TPS_KCPARAM) {
        for (int i = tid; i < PAD + NN; i += B) kc_s[i] = kp.v[i];
    }
    const float4 *kc0 = (LMM_TPS_KCPARAM ? kp.v : kc_s) + PAD;
    float *vg0 = vg_s + Lay::VPAD * B + tid;
    float *vt0 = vt_s + tid;
    float *sc = scr + (size_t)blockIdx.x * Lay::rows * B + tid;    // sc[row * B]

    const int units = m.nscen * w.items;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int scen = unit / w.items, item = unit % w.items;
        __syncthreads();          // the previous unit's reads of il0/acc are done
        for (int i = tid; i < NN; i += B) il0_s[i] = m.invL0f[scen * NN + i];
        for (int i = tid; i < Lay::NW * 2 * NOUT; i += B) acc_s[i] = 0.0;
        __syncthreads();

        const int64_t ibase = (int64_t)item * w.ppt * B;
        for (int jb = 0; jb < w.ppt; ++jb) {
            if (ibase + (int64_t)jb * B >= w.paths) break;          // block-uniform
            const int64_t pl = ibase + (int64_t)jb * B + tid;
            const bool active = pl < w.paths;
            const int64_t pc = active ? pl : w.paths - 1;
            const float *zp = PHILOX ? nullptr : z + pc * NMAT;
            const uint64_t gpath = (uint64_t)(path0 + pc);

            float disc = 1.0f, V, vs;
            float Xu[H], Pu[H];       // upper half: inverse rates and log-adjoints
            unsigned long long mask = 0ull;
            {
                // ---- forward over all NN rates (path_calc_b1 :34-82) ----
                float IL[NN];
#pragma unroll
                for (int i = 0; i < NN; ++i) IL[i] = il0_s[i];
                float4 zq, zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, 0);
                for (int n = 0; n < NMAT; n += 2) {
                    if (LMM_TPS_SYNC && (n % (2 * (PHILOX ? LMM_TPS_FSYNC_PHILOX : LMM_TPS_FSYNC))) == 0)
                        __syncthreads();
                    if ((n & 3) == 0) {
                        zq = zq_next;
                        if ((n >> 2) + 1 < NMAT / 4) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) + 1);
                    }
                    const float sqez0 = sqd * ((n & 2) ? zq.z : zq.x);
                    const float sqez1 = sqd * ((n & 2) ? zq.w : zq.y);
                    float V0, V1, V0c, V1c;
                    fwd_pair_window_cap<NN, LMM_TPP_CHUNK, PF, H - 1>(IL, kc0 - (n + 1), sqez0, sqez1,
                                                                                delta, n, V0, V1, V0c, V1c);
                    vt0[n * B] = V0;
                    vt0[(n + 1) * B] = V1;
                    sc[(Lay::s_v + n) * B] = V0c;
                    sc[(Lay::s_v + n + 1) * B] = V1c;
                }
                // ---- payoff (portfolio_b :133-171, :186-197) and the annuity adjoint ----
                float *Bst = vg0;
                float *ILst = vg0 + M * B;
                V = payoff_forward<NN, NMAT, B>(IL, delta, ost_s, okk_s, owf_s, &disc, Bst, ILst, &mask);
                payoff_adjoint_stage<NN, NMAT, B>(1.0f, disc, Bst, ILst, mask, delta, ost_s, okf_s, owf_s);
#pragma unroll
                for (int i = 0; i < H; ++i) {
                    Xu[i] = IL[H + i];
                    Pu[i] = ILst[i * B];
                    sc[(Lay::s_il + i) * B] = IL[i];     // the lower half waits in the scratch
                }
                vs = -V * delta;
            }
#pragma unroll
            for (int k = 0; k < NN; ++k) vg0[k * B] = 0.0f;

            // ---- R1: the upper half's reverse, every step ----
            for (int n = NMAT - 1; n > 0; n -= G) {
                if (LMM_TPS_SYNC && ((NMAT - 1 - n) / G) % LMM_TPS_RSYNC == 0) __syncthreads();
                RevStep st[G];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const int mm = n - g;
                    st[g].sqez = 0.0f;
                    st[g].V = vt0[mm * B];
                    st[g].S = 0.0f;
                    st[g].kc = kc0 - (mm + 1) + H;
                    st[g].vg = vg0 + (H - mm - 1) * B;
                }
                rev_half_window<H, H, B, G, RCH, PF>(Xu, Pu, st, delta, n);
#pragma unroll
                for (int g = 0; g < G; ++g) sc[(Lay::s_s + n - g) * B] = st[g].S;
            }
#pragma unroll
            for (int i = 0; i < H; ++i) sc[(Lay::s_d + i) * B] = active ? Pu[i] * il0_s[H + i] : 0.0f;

            // ---- R2: the lower half's reverse ----
            float Xl[H], Pl[H];
#pragma unroll
            for (int i = 0; i < H; ++i) {
                Xl[i] = sc[(Lay::s_il + i) * B];
                Pl[i] = vs * rcp_approx(Xl[i] + delta);
            }
            float nv[G], ns[G];       // the next group's restart sums, loaded a group ahead
#pragma unroll
            for (int g = 0; g < G; ++g) {
                nv[g] = sc[(Lay::s_v + NMAT - 1 - g) * B];
                ns[g] = sc[(Lay::s_s + NMAT - 1 - g) * B];
            }
            for (int n = NMAT - 1; n > 0; n -= G) {
                if (LMM_TPS_SYNC && ((NMAT - 1 - n) / G) % LMM_TPS_RSYNC == 0) __syncthreads();
                RevStep st[G];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const int mm = n - g;
                    st[g].sqez = 0.0f;
                    st[g].V = nv[g];
                    st[g].S = ns[g];
                    st[g].kc = kc0 - (mm + 1);
                    st[g].vg = vg0 - (mm + 1) * B;
                }
                if (n - G > 0) {
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        nv[g] = sc[(Lay::s_v + n - G - g) * B];
                        ns[g] = sc[(Lay::s_s + n - G - g) * B];
                    }
                }
                rev_half_window<H, 0, B, G, RCH, PF>(Xl, Pl, st, delta, n);
            }

            // ---- cross-path reduction of this batch of B paths ----
            {
                const float v = active ? V : 0.0f;
                const float s1 = warp_sum(v), s2 = warp_sum(v * v);
                if (lane == 0) {
                    acc[0] += (double)s1;
                    acc[NOUT] += (double)s2;
                }
            }
            float *vgw = vg_s + Lay::VPAD * B;
            if (!active) {
#pragma unroll
                for (int k = 0; k < NN; ++k) vg0[k * B] = 0.0f;
            }
            __syncwarp();
            column_reduce<NN, B>(vgw, warp, lane, acc, NOUT, 1 + NN);
            __syncwarp();
#pragma unroll
            for (int i = 0; i < H; ++i) {
                vg0[i * B] = active ? Pl[i] * il0_s[i] : 0.0f;
                vg0[(H + i) * B] = sc[(Lay::s_d + i) * B];
            }
            __syncwarp();
            column_reduce<NN, B>(vgw, warp, lane, acc, NOUT, 1);
            __syncwarp();
        }

        __syncthreads();
        for (int o = tid; o < 2 * NOUT; o += B) {
            double s2 = 0.0;
#pragma unroll
            for (int q = 0; q < Lay::NW; ++q) s2 += acc_s[q * 2 * NOUT + o];
            w.partial[(size_t)unit * 2 * NOUT + o] = s2;
        }
    }  // units
}

template <int NN, int NMAT, bool PHILOX>
cudaError_t launch_tps(const DevModel &m, const float *z, uint64_t seed, int64_t path0, const Work &w,
                       float *scr, cudaStream_t s)
{
    using Lay = TpsLayout<NN, NMAT>;
    auto kern = k_tps<NN, NMAT, PHILOX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    TppConst<NN, NMAT> kp;
    for (int i = 0; i < NMAT + NN; ++i)
        kp.v[i] = i < NMAT ? make_float4(0.f, 0.f, 0.f, 0.f) : m.kc_host[i - NMAT];
    const unsigned grid = (unsigned)(w.grid > 0 ? w.grid : (int64_t)m.nscen * w.items);
    kern<<<grid, Lay::B, Lay::bytes, s>>>(m, z, seed, path0, w, scr, kp);
    return cudaGetLastError();
}

template <int NN, int NMAT, bool PHILOX>
cudaError_t occ_tps(int *blocks)
{
    using Lay = TpsLayout<NN, NMAT>;
    auto kern = k_tps<NN, NMAT, PHILOX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, Lay::B, Lay::bytes);
}

// ---------------------------------------------------------------------------
// k_tpq: the fused long-tenor call (NN = 160, NMAT = 120) with one thread per
// path, the reverse sweep in passes over blocks of 40 rates.
//
// The forward runs in two passes of 80 rates through one copy of the pass
// body (rates 0..79 for the steps that move them, then rates 80..159 for
// every step from the first pass's drift sums at rate 79), so at most 80
// inverse rates are live (255 registers in all: 8 warps, 256 paths per SM,
// the vega rows of 256 paths fill shared memory), and saves, per step, the
// drift sum at the top rate of every block and the rates every ck steps
// (ck = DevModel::ckpt, a multiple of 4); the per-maturity constants are read
// from shared memory. The reverse then runs the blocks one after another from the
// top, in one thread: block b (rates 40b .. 40b+39) for every group of four
// steps with an active cell in it, each step starting from the forward's
// drift sum at the block's top rate and from the suffix sum the block above
// left at its bottom; the rates above a checkpoint time are taken back from
// the checkpoint at group boundaries. At most 40 rates and 40 log-adjoints
// are live in the reverse, the other blocks wait in a per-block scratch, and
// one copy of the 40-position reverse body serves every block (the block's
// offset is a runtime value). The loads of the rates a group hands on (a
// checkpoint, or the block below's parked rates) are issued inside the
// group's body, each right after the group's last cell on its rate, so their
// latency overlaps the rest of the body and the next group's top positions.
// Against two threads per path (k_tp2) there is no pair to balance and no
// barrier per round; the warps of a block run without barriers.
// Scratch per block of the wave, rows of B floats (one per thread):
// [Q][NMAT] block-top drift sums, [Q-1][NMAT] block-bottom suffix sums,
// [NN-H] parked inverse rates of the lower blocks, [NN-H] deltas of the upper
// blocks, [NCK][NN] rate checkpoints.
// ---------------------------------------------------------------------------
#ifndef LMM_TPQ_BLOCK
#define LMM_TPQ_BLOCK 256
#endif
// Block barriers of the long-tenor fused kernel: one every LMM_TPQ_FSYNC
// forward step pairs and every LMM_TPQ_RSYNC reverse step groups (0: none).
// GB300, 160/120, 1,048,576 paths, rates saved every 8 steps: none 15.76 ms;
// every second pair 16.17; every second or fourth group 16.01, 15.99; every
// second pair and every group 17.20.
#ifndef LMM_TPQ_FSYNC
#define LMM_TPQ_FSYNC 0
#endif
// 1: the per-maturity constants copied to shared memory (one 16-byte load per
// ring entry) instead of read from the kernel-parameter bank. GB300,
// 1,048,576 paths: 14.88 -> 14.15 ms.
#ifndef LMM_TPQ_KCSMEM
#define LMM_TPQ_KCSMEM 1
#endif
// Steps per reverse group, reverse and forward chunk lengths and the constant
// prefetch distance of the long-tenor fused kernel (as LMM_TPP_*). GB300,
// 1,048,576 paths, the forward in one pass body: forward chunks of 8, 16, 20
// or 40 rates 15.20, 14.91, 14.97, 15.42 ms; constants one position ahead or
// at the position of use (16-rate chunks) 14.91, 14.89 ms; two positions
// ahead 14.99. Groups of 8 steps 18.5 ms (against 15.77 with 4, in an earlier
// build); reverse chunks of 1, 2, 4 within 1%.
#ifndef LMM_TPQ_SKEW
#define LMM_TPQ_SKEW LMM_TPP_SKEW
#endif
#ifndef LMM_TPQ_RCHUNK
#define LMM_TPQ_RCHUNK LMM_TPP_RCHUNK
#endif
#ifndef LMM_TPQ_RCHUNK_PHILOX
#define LMM_TPQ_RCHUNK_PHILOX LMM_TPP_RCHUNK_PHILOX
#endif
#ifndef LMM_TPQ_CHUNK
#define LMM_TPQ_CHUNK 16
#endif
#ifndef LMM_TPQ_PREF
#define LMM_TPQ_PREF 0
#endif
#ifndef LMM_TPQ_PREF_PHILOX
#define LMM_TPQ_PREF_PHILOX LMM_TPP_PREF_PHILOX
#endif
#ifndef LMM_TPQ_RSYNC
#define LMM_TPQ_RSYNC 0
#endif

template <int NN, int NMAT>
struct TpqLayout {
    static constexpr int B = LMM_TPQ_BLOCK;
    static constexpr int NW = B / 32;
    static constexpr int H = 40;
    static constexpr int Q = NN / H;
    static constexpr int M = NN - NMAT;
    static constexpr int VPAD = 4;
    static constexpr int NOUT = 1 + 2 * NN;
    static constexpr int il0 = 0;                                    // float[NN]
    static constexpr int ost = align16(il0 + 4 * NN);                // int[M+1]
    static constexpr int okf = align16(ost + 4 * (M + 1));           // float[kMaxNopt]
    static constexpr int owf = align16(okf + 4 * kMaxNopt);          // float[kMaxNopt]
    static constexpr int okk = align16(owf + 4 * kMaxNopt);          // F2[kMaxNopt]
    static constexpr int vg = align16(okk + 8 * kMaxNopt);           // float[VPAD+NN][B] vega rows
    static constexpr int acc = align16(vg + 4 * (VPAD + NN) * B);    // double[NW][2*NOUT]
    static constexpr int kcs = align16(acc + 8 * NW * 2 * NOUT);     // float4[NMAT+NN] (LMM_TPQ_KCSMEM)
    static constexpr int bytes = kcs + (LMM_TPQ_KCSMEM ? 16 * (NMAT + NN) : 0);
    static_assert(bytes <= 227 * 1024, "one block's shared memory");
    static constexpr int s_vt = 0, s_sb = Q * NMAT, s_il = s_sb + (Q - 1) * NMAT, s_d = s_il + NN - H,
                         s_ck = s_d + NN - H;
    static_assert(NN % H == 0 && M == H && H % 4 == 0, "the top block is the annuity rates");
};

// Forward steps n and n+1 over the NP rates LO .. LO+NP-1 held in IL[] at
// local positions 0 .. NP-1, paired as fwd_pair_window: cell (n, p) with
// cell (n+1, p-1). V0, V1 enter as the steps' drift sums below the pass (at
// rate LO-1; the normal term alone for LO = 0) and leave as the sums at its
// top rate; V0c[q], V1c[q] return the sums at local position qH + H-1, the
// top rate of each H-rate block of the pass. kcn points at step n's
// constants for local position 0 (k = LO - n - 1; the NMAT zero rows below
// k = 0 make the inactive cells exact no-ops); nrel = n - LO < NP - 1.
template <int NP, int H, int CH, int P>
__device__ __forceinline__ void fwd_pair_pass(float (&IL)[NP], const float4 *kcn, float delta, int nrel,
                                              float &V0, float &V1, float (&V0c)[NP / H], float (&V1c)[NP / H])
{
    constexpr int R = 3 + P;
    float4 C[R];
#pragma unroll
    for (int q = 0; q < NP / H; ++q) {
        V0c[q] = V0;
        V1c[q] = V1;
    }
    const int c0 = nrel + 1 > 0 ? (nrel + 1) / CH : 0;
    static_assert(!LMM_FWD_RCP2_LONG || (CH % 2 == 0 && NP % 2 == 0), "reciprocal pairs (2m, 2m+1) inside chunks");
    float t0n = 0.0f, t1n = 0.0f;   // LMM_FWD_RCP2_LONG: the second reciprocals of the steps' pairs in flight
#pragma unroll
    for (int c = 0; c * CH < NP; ++c) {
        if (c >= c0) {
            if (c == c0) {
#pragma unroll
                for (int j = c * CH - 2; j < c * CH + P; ++j)
                    if (j < NP) C[(j % R + R) % R] = kcn[j];
                // step n+1's pair below the chunk: rates inactive in step n, unchanged
                if (LMM_FWD_RCP2_LONG && c * CH >= 2) {
                    float ta;
                    rcp_pair(IL[c * CH - 2] + delta, IL[c * CH - 1] + delta, ta, t1n);
                }
            }
#pragma unroll
            for (int p = c * CH; p < (c + 1) * CH && p < NP; ++p) {
                if (p + P < NP) C[(p + P) % R] = kcn[p + P];
                if (LMM_FWD_RCP2_LONG) {     // pairs as fwd_pair_window_cap (LO even)
                    float t;
                    if (p % 2 == 0)
                        rcp_pair(IL[p] + delta, IL[p + 1] + delta, t, t0n);
                    else
                        t = t0n;
                    fwd_cell_t(IL[p], V0, C[p % R], 0.0f, t);
                    if (p % 2 == 1) {
                        float ta;
                        rcp_pair(IL[p - 1] + delta, IL[p] + delta, ta, t1n);
                        fwd_cell_t(IL[p - 1], V1, C[((p - 2) % R + R) % R], 0.0f, ta);
                    } else if (p >= 1) {
                        fwd_cell_t(IL[p - 1], V1, C[((p - 2) % R + R) % R], 0.0f, t1n);
                    }
                } else {
                    fwd_cell(IL[p], V0, C[p % R], 0.0f, delta);
                    if (p >= 1) fwd_cell(IL[p - 1], V1, C[((p - 2) % R + R) % R], 0.0f, delta);
                }
                if (p % H == H - 1) V0c[p / H] = V0;
                if (p >= 1 && (p - 1) % H == H - 1) V1c[(p - 1) / H] = V1;
            }
        }
    }
    if (LMM_FWD_RCP2_LONG)
        fwd_cell_t(IL[NP - 1], V1, C[(NP - 2) % R], 0.0f, t1n);
    else
        fwd_cell(IL[NP - 1], V1, C[(NP - 2) % R], 0.0f, delta);
    V1c[NP / H - 1] = V1;
}

// Reverse steps n .. n-G+1 over the block of H rates LO .. LO+H-1 (X[], Pb[]
// at local positions 0 .. H-1; LO a runtime multiple of G): rev_group_window
// on a block. st[0].kc and st[0].vg point at step n's constants and vega rows
// of the block's local position 0. When every step of the group is active at
// the block's bottom rate (LO > n) the body runs to its last position and
// flushes the vega slots of positions 0 .. G-2 (they hold active cells);
// otherwise it is left at the first chunk wholly below the lowest active
// position, as rev_group_window, and the slots still open hold no-op cells
// of spare rows. Rates that the caller replaces after the group (positions
// j > tl, from rs[j*B]) are loaded as soon as the group's last cell on them
// is done, position j - G + 1, so that the loads overlap the rest of the
// body; every such position lies at or above the lowest active one.
template <int H, int B, int G, int CH, int P>
__device__ __forceinline__ void rev_block_window(float (&X)[H], float (&Pb)[H], RevStep (&st)[G], float delta,
                                                 int n, int LO, const float *rs, int tl)
{
    constexpr int JMAX = H + G - 2;
    constexpr int W = 2 * G - 1 + P;
    const float4 *kc = st[0].kc;
    float *vg = st[0].vg;
    float4 C[W];
    float D[W];
    float A[W];
#pragma unroll
    for (int j = H - P; j <= JMAX; ++j) {
        C[j % W] = kc[j];
        D[j % W] = -delta * C[j % W].w;
        if (j >= H) A[j % W] = 0.0f;
    }
    const bool full = LO > n;
    const int imin = n - 2 * G + 3 - LO;     // lowest local position with an active cell
#pragma unroll
    for (int q = 0; q * CH < H + G - 1; ++q) {
        const int top = H - 1 - q * CH;
        if (!full && top < imin) return;
#pragma unroll
        for (int i = top; i > top - CH && i >= -(G - 1); --i) {
            if (i - P >= 0) {
                C[(i - P) % W] = kc[i - P];
                D[(i - P) % W] = -delta * C[(i - P) % W].w;
            }
            if (i >= 0) A[i % W] = 0.0f;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (i + g >= 0 && i + g <= H - 1) {
                    const int j = i + 2 * g;
                    rev_cell<H, LMM_TPQ_DCONST != 0>(X, Pb, st[g], i + g, C[j % W], D[j % W], A[j % W], delta);
                }
            }
            const int jf = i + 2 * (G - 1);
            if (jf >= 0 && jf <= JMAX) vg[jf * B] += A[jf % W];
            const int jr = i + G - 1;
            if (jr >= 0 && jr <= H - 1 && jr > tl) X[jr] = rs[jr * B];
        }
    }
    if (full) {
#pragma unroll
        for (int j = 0; j < G - 1; ++j) vg[j * B] += A[j % W];
    }
}

template <int NN, int NMAT, bool PHILOX>
__global__ void __launch_bounds__(LMM_TPQ_BLOCK, 1)
k_tpq(const DevModel m, const float *__restrict__ z, uint64_t seed, int64_t path0, const Work w,
      float *__restrict__ scr, const __grid_constant__ TppConst<NN, NMAT> kp)
{
    using Lay = TpqLayout<NN, NMAT>;
    constexpr int B = Lay::B, H = Lay::H, Q = Lay::Q, M = Lay::M, NOUT = Lay::NOUT, PAD = NMAT;
    constexpr int G = LMM_TPQ_SKEW, RCH = PHILOX ? LMM_TPQ_RCHUNK_PHILOX : LMM_TPQ_RCHUNK;
    constexpr int PF = PHILOX ? LMM_TPQ_PREF_PHILOX : LMM_TPQ_PREF;
    static_assert(NMAT % 4 == 0 && NMAT % G == 0 && H % G == 0, "normals in quads, reverse steps in groups");
    static_assert(RCH - 1 <= Lay::VPAD, "the windows' spare vega rows lie inside the table");
    constexpr int kFsync = LMM_TPQ_FSYNC > 0 ? LMM_TPQ_FSYNC : 1, kRsync = LMM_TPQ_RSYNC > 0 ? LMM_TPQ_RSYNC : 1;
    constexpr int HF = 2 * H;      // rates per forward pass
    static_assert(kYrun, "the drift sums carry the normal term");
    static_assert(NN == 2 * HF && NMAT > HF && NMAT - HF + M == HF, "two forward passes");
    extern __shared__ __align__(16) unsigned char smem[];
    float *il0_s = reinterpret_cast<float *>(smem + Lay::il0);
    int *ost_s = reinterpret_cast<int *>(smem + Lay::ost);
    float *okf_s = reinterpret_cast<float *>(smem + Lay::okf);
    float *owf_s = reinterpret_cast<float *>(smem + Lay::owf);
    F2 *okk_s = reinterpret_cast<F2 *>(smem + Lay::okk);
    float *vg_s = reinterpret_cast<float *>(smem + Lay::vg);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i <= M; i += B) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += B) {
        okf_s[i] = m.optKf[i];
        owf_s[i] = m.optWf[i];
        okk_s[i] = f2_from(m.optKd[i] * m.deltad);
    }
    const float delta = m.delta, sqd = m.sqd;
    const float4 *kc0 = kp.v + PAD;
    if (LMM_TPQ_KCSMEM) {          // read by the cells after the unit loop's first barrier
        float4 *kcs = reinterpret_cast<float4 *>(smem + Lay::kcs);
        for (int i = tid; i < NMAT + NN; i += B) kcs[i] = kp.v[i];
        kc0 = kcs + PAD;
    }
    float *vg0 = vg_s + Lay::VPAD * B + tid;
    const int ck = m.ckpt;
    const int nck = ck > 0 ? (NMAT - 1) / ck : 0;
    const int ckd = ck > 0 ? ck : 1;
    const int64_t rows = Lay::s_ck + (int64_t)nck * NN;
    float *sc = scr + (size_t)blockIdx.x * rows * B + tid;          // sc[row * B]
    double *acc_s = reinterpret_cast<double *>(smem + Lay::acc);     // [NW][2*NOUT]
    double *acc = acc_s + warp * 2 * NOUT;
    float *ckp = sc + (size_t)Lay::s_ck * B;                         // checkpoint c, rate i: ckp[(c*NN + i)*B]

    const int units = m.nscen * w.items;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int scen = unit / w.items, item = unit % w.items;
        __syncthreads();          // the previous unit's reads of il0/acc are done
        for (int i = tid; i < NN; i += B) il0_s[i] = m.invL0f[scen * NN + i];
        for (int i = tid; i < Lay::NW * 2 * NOUT; i += B) acc_s[i] = 0.0;
        __syncthreads();

        const int64_t ibase = (int64_t)item * w.ppt * B;
        for (int jb = 0; jb < w.ppt; ++jb) {
            if (ibase + (int64_t)jb * B >= w.paths) break;          // block-uniform
            const int64_t pl = ibase + (int64_t)jb * B + tid;
            const bool active = pl < w.paths;
            const int64_t pc = active ? pl : w.paths - 1;
            const float *zp = PHILOX ? nullptr : z + pc * NMAT;
            const uint64_t gpath = (uint64_t)(path0 + pc);

            float disc = 1.0f, V, vs;
            float X[H], Pb[H];        // the block in the reverse: inverse rates, log-adjoints
            unsigned long long mask = 0ull;
            {
                // ---- forward (path_calc_b1 :34-82) in two passes of HF rates through one copy of
                // the body: pass 0 rates 0 .. HF-1 from the normals, pass 1 rates HF .. NN-1 from
                // pass 0's drift sums at rate HF-1 ----
                F2 dprod{1.0f, 0.0f};          // the discount product, rates 0 .. NMAT-1 in order
                float IL[HF];
                const float *vin = sc + (size_t)(Lay::s_vt + (HF / H - 1) * NMAT) * B;
#pragma unroll 1
                for (int ps = 0; ps < 2; ++ps) {
                    const int LOp = ps * HF;
#pragma unroll
                    for (int i = 0; i < HF; ++i) IL[i] = il0_s[LOp + i];
                    float4 zq = make_float4(0.f, 0.f, 0.f, 0.f), zq_next = zq;
                    float nv0 = 0.0f, nv1 = 0.0f;
                    if (ps == 0) {
                        zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, 0);
                    } else {
                        nv0 = vin[0];
                        nv1 = vin[B];
                    }
                    for (int n = 0; n < NMAT; n += 2) {
                        if (LMM_TPQ_FSYNC && (n % (2 * kFsync)) == 0) __syncthreads();
                        float V0, V1;
                        if (ps == 0) {
                            if ((n & 3) == 0) {
                                zq = zq_next;
                                if ((n >> 2) + 1 < NMAT / 4) zq_next = zquad<PHILOX, NMAT>(zp, seed, gpath, (n >> 2) + 1);
                            }
                            V0 = sqd * ((n & 2) ? zq.z : zq.x);     // drift sums from the normal term (kYrun)
                            V1 = sqd * ((n & 2) ? zq.w : zq.y);
                        } else {
                            V0 = nv0;
                            V1 = nv1;
                            if (n + 2 < NMAT) {
                                nv0 = vin[(n + 2) * B];
                                nv1 = vin[(n + 3) * B];
                            }
                        }
                        float V0c[HF / H], V1c[HF / H];
                        if (n - LOp < HF - 1) {
                            fwd_pair_pass<HF, H, LMM_TPQ_CHUNK, PF>(IL, kc0 - (n + 1) + LOp, delta, n - LOp, V0, V1,
                                                                     V0c, V1c);
                        } else {                 // no rate of the pass moves
#pragma unroll
                            for (int q = 0; q < HF / H; ++q) {
                                V0c[q] = V0;
                                V1c[q] = V1;
                            }
                        }
#pragma unroll
                        for (int q = 0; q < HF / H; ++q) {
                            sc[(Lay::s_vt + (ps * (HF / H) + q) * NMAT + n) * B] = V0c[q];
                            sc[(Lay::s_vt + (ps * (HF / H) + q) * NMAT + n + 1) * B] = V1c[q];
                        }
                        if (nck > 0 && (n + 2) % ckd == 0 && n + 2 < NMAT) {
                            // rates i <= n+2 are final from here on: only the others are saved
                            const int c = (n + 2) / ckd - 1;
#pragma unroll
                            for (int i = 0; i < HF; ++i)
                                if (LOp + i > n + 2) ckp[(c * NN + LOp + i) * B] = IL[i];
                        }
                    }
#pragma unroll
                    for (int i = 0; i < HF; ++i) {
                        if (LOp + i < NMAT) {
                            dprod = f2_mul(dprod, bond_ratio(IL[i], delta));
                            sc[(Lay::s_il + LOp + i) * B] = IL[i];
                        }
                    }
                }
                // ---- payoff (portfolio_b :133-171, :186-197) and the annuity adjoint ----
                float *Bst = vg0;
                float *ILst = vg0 + M * B;
#pragma unroll
                for (int m2 = 0; m2 < M; ++m2) ILst[m2 * B] = IL[NMAT - HF + m2];
                V = payoff_forward_staged<M, B>(dprod, delta, ost_s, okk_s, owf_s, &disc, Bst, ILst, &mask);
                payoff_adjoint_stage<NN, NMAT, B>(1.0f, disc, Bst, ILst, mask, delta, ost_s, okf_s, owf_s);
#pragma unroll
                for (int i = 0; i < H; ++i) {
                    X[i] = IL[NN - HF - H + i];
                    Pb[i] = ILst[i * B];
                }
                vs = -V * delta;
            }
#pragma unroll
            for (int k = 0; k < NN; ++k) vg0[k * B] = 0.0f;

            // ---- reverse: the blocks from the top, each over its groups of steps ----
            for (int b = Q - 1; b >= 0; --b) {
                const int LO = b * H;
                if (b < Q - 1) {          // X holds the block's parked rates (the last group above loaded them)
#pragma unroll
                    for (int i = 0; i < H; ++i) Pb[i] = vs * rcp_approx(X[i] + delta);
                }
                // the block's first group with an active cell (its top rate above the group's lowest step)
                int n0 = NMAT - 1;
                while (LO + H - 1 <= n0 - G + 1) n0 -= G;
                float nv[G], ns[G];   // the next group's restart sums, loaded a group ahead
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    nv[g] = sc[(Lay::s_vt + b * NMAT + n0 - g) * B];
                    ns[g] = b < Q - 1 ? sc[(Lay::s_sb + b * NMAT + n0 - g) * B] : 0.0f;
                }
                for (int n = n0; n > 0; n -= G) {
                    if (LMM_TPQ_RSYNC && ((n0 - n) / G) % kRsync == 0) __syncthreads();
                    RevStep st[G];
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        const int mm = n - g;
                        st[g].sqez = 0.0f;
                        st[g].V = nv[g];
                        st[g].S = ns[g];
                        st[g].kc = kc0 - (mm + 1) + LO;
                        st[g].vg = vg0 + (LO - mm - 1) * B;
                    }
                    if (n - G > 0) {
#pragma unroll
                        for (int g = 0; g < G; ++g) {
                            nv[g] = sc[(Lay::s_vt + b * NMAT + n - G - g) * B];
                            ns[g] = b < Q - 1 ? sc[(Lay::s_sb + b * NMAT + n - G - g) * B] : 0.0f;
                        }
                    }
                    // the rates the group hands on that come from memory: a checkpoint at
                    // its end time t (the reverse of steps >= t leaves rates i <= t
                    // untouched), or in a block's last group the block below's parked rates
                    const int t = n - G + 1;
                    const float *rs = sc;
                    int tl = H;
                    if (nck > 0 && t % ckd == 0 && t >= ck) {
                        rs = ckp + (size_t)((t / ckd - 1) * NN + LO) * B;
                        tl = t - LO;
                    } else if (b > 0 && n - G <= 0) {
                        rs = sc + (size_t)(Lay::s_il + LO - H) * B;
                        tl = -1;
                    }
                    rev_block_window<H, B, G, RCH, PF>(X, Pb, st, delta, n, LO, rs, tl);
                    if (b > 0) {
#pragma unroll
                        for (int g = 0; g < G; ++g) sc[(Lay::s_sb + (b - 1) * NMAT + n - g) * B] = st[g].S;
                    }
                }
                if (b > 0) {
#pragma unroll
                    for (int i = 0; i < H; ++i)
                        sc[(Lay::s_d + LO - H + i) * B] = active ? Pb[i] * il0_s[LO + i] : 0.0f;
                }
            }

            // ---- cross-path reduction of this batch of B paths ----
            {
                const float v = active ? V : 0.0f;
                const float s1 = warp_sum(v), s2 = warp_sum(v * v);
                if (lane == 0) {
                    acc[0] += (double)s1;
                    acc[NOUT] += (double)s2;
                }
            }
            float *vgw = vg_s + Lay::VPAD * B;
            if (!active) {
#pragma unroll
                for (int k = 0; k < NN; ++k) vg0[k * B] = 0.0f;
            }
            __syncwarp();
            column_reduce<NN, B>(vgw, warp, lane, acc, NOUT, 1 + NN);
            __syncwarp();
#pragma unroll
            for (int i = 0; i < H; ++i) vg0[i * B] = active ? Pb[i] * il0_s[i] : 0.0f;
#pragma unroll
            for (int i = 0; i < NN - H; ++i) vg0[(H + i) * B] = sc[(Lay::s_d + i) * B];
            __syncwarp();
            column_reduce<NN, B>(vgw, warp, lane, acc, NOUT, 1);
            __syncwarp();
        }

        __syncthreads();
        for (int o = tid; o < 2 * NOUT; o += B) {
            double s2 = 0.0;
#pragma unroll
            for (int q = 0; q < Lay::NW; ++q) s2 += acc_s[q * 2 * NOUT + o];
            w.partial[(size_t)unit * 2 * NOUT + o] = s2;
        }
    }  // units
}

template <int NN, int NMAT, bool PHILOX>
cudaError_t launch_tpq(const DevModel &m, const float *z, uint64_t seed, int64_t path0, const Work &w,
                       float *scr, cudaStream_t s)
{
    using Lay = TpqLayout<NN, NMAT>;
    auto kern = k_tpq<NN, NMAT, PHILOX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    TppConst<NN, NMAT> kp;
    for (int i = 0; i < NMAT + NN; ++i)
        kp.v[i] = i < NMAT ? make_float4(0.f, 0.f, 0.f, 0.f) : m.kc_host[i - NMAT];
    const unsigned grid = (unsigned)(w.grid > 0 ? w.grid : (int64_t)m.nscen * w.items);
    kern<<<grid, Lay::B, Lay::bytes, s>>>(m, z, seed, path0, w, scr, kp);
    return cudaGetLastError();
}

template <int NN, int NMAT, bool PHILOX>
cudaError_t occ_tpq(int *blocks)
{
    using Lay = TpqLayout<NN, NMAT>;
    auto kern = k_tpq<NN, NMAT, PHILOX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, Lay::B, Lay::bytes);
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
cudaError_t launch_tpp(const DevModel &m, const float *z, uint64_t seed, int64_t path0,
                       const Work &w, float *tape, const double *vbar, cudaStream_t s)
{
    using Lay = TppLayout<NN, NMAT, MODE>;
    auto kern = k_tpp<NN, NMAT, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    TppConst<NN, NMAT> kp;
    for (int i = 0; i < NMAT + NN; ++i)
        kp.v[i] = i < NMAT ? make_float4(0.f, 0.f, 0.f, 0.f) : m.kc_host[i - NMAT];
    const unsigned grid = (unsigned)(w.grid > 0 ? w.grid : (int64_t)m.nscen * w.items);
    kern<<<grid, Lay::B, Lay::bytes, s>>>(m, z, seed, path0, w, tape, vbar, kp);
    return cudaGetLastError();
}

template <int NN, int NMAT, bool PHILOX, Mode MODE>
cudaError_t occ_tpp(int *blocks)
{
    using Lay = TppLayout<NN, NMAT, MODE>;
    auto kern = k_tpp<NN, NMAT, PHILOX, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, Lay::B, Lay::bytes);
}

}  // namespace

bool f32_tpp_supports(int nn, int nmat) { return nn == 80 && nmat == 40; }

int tps_block_threads() { return LMM_TPS_BLOCK; }

bool f32_tpq_supports(int nn, int nmat) { return nn == 160 && nmat == 120; }

int tpq_block_threads() { return LMM_TPQ_BLOCK; }

size_t tpq_scratch_floats_per_block(int nn, int nmat, int ckpt)
{
    const int H = 40, Q = nn / H;
    const int nck = ckpt > 0 ? (nmat - 1) / ckpt : 0;
    return (size_t)(Q * nmat + (Q - 1) * nmat + 2 * (nn - H) + (size_t)nck * nn) * LMM_TPQ_BLOCK;
}

cudaError_t tpq_blocks_per_sm(bool philox, int *blocks)
{
    return philox ? occ_tpq<160, 120, true>(blocks) : occ_tpq<160, 120, false>(blocks);
}

cudaError_t launch_tpq_any(const DevModel &m, const float *z, uint64_t seed, int64_t path0, bool philox,
                           const Work &w, float *scratch, cudaStream_t s)
{
    return philox ? launch_tpq<160, 120, true>(m, z, seed, path0, w, scratch, s)
                  : launch_tpq<160, 120, false>(m, z, seed, path0, w, scratch, s);
}

size_t tps_scratch_floats_per_block(int nn, int nmat) { return (size_t)(2 * nmat + nn) * LMM_TPS_BLOCK; }

cudaError_t tps_blocks_per_sm(bool philox, int *blocks)
{
    return philox ? occ_tps<80, 40, true>(blocks) : occ_tps<80, 40, false>(blocks);
}

cudaError_t launch_tps_any(const DevModel &m, const float *z, uint64_t seed, int64_t path0, bool philox,
                           const Work &w, float *scratch, cudaStream_t s)
{
    return philox ? launch_tps<80, 40, true>(m, z, seed, path0, w, scratch, s)
                  : launch_tps<80, 40, false>(m, z, seed, path0, w, scratch, s);
}

int tpp_block_threads(Mode mode)
{
    return mode == Mode::Fused ? tpp_block<Mode::Fused>()
                               : (mode == Mode::Forward ? tpp_block<Mode::Forward>() : tpp_block<Mode::Backward>());
}

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

// FP64 LMM kernels: the GPU oracle mode (value + all Greeks in FP64, matched
// against the reference to 1e-12) and the plain FP64 bump-and-revalue
// comparator (forward only, re-run with each input bumped).
//
// One thread per path, runtime NN/NMAT (<= kMaxNN), per-thread state in local
// memory. The arithmetic follows the reference formula by formula:
//   forward  path_calc_b1 (LiborMarketModel/liborSwaptionGreeks.cpp:50-81)
//   payoff   portfolio_b  (:133-209, with the :178/:181 aliasing fixed)
//   reverse  path_calc_b2 (:94-116) in log-adjoint form, running the Euler
//            step backwards from the saved per-step drift sums (no stored
//            trajectory), plus the vega adjoint.
#include "lmm_device.cuh"

namespace lmm {
namespace {

constexpr int kF64Block = 128;

struct F64Smem {
    double *lam;     // [nn]
    int *ost;        // [nn-nmat+1]
    double *okd;     // [nopt]
    double *acc;     // [NW][2*nout]
};

// portfolio_b :133-171 and :186-197 in FP64; returns the discounted value.
// Bst (if given) receives the annuity factors B[m] of :139 for the adjoint.
__device__ double payoff_value_f64(const double *L, int nn, int nmat, double d, const int *ost,
                                   const double *okd, const double *okw, double *disc_out, double *Bst,
                                   unsigned long long *mask_out)
{
    double b = 1.0, s = 0.0, vs = 0.0;
    unsigned long long mask = 0ull;
    for (int m = 0; m < nn - nmat; ++m) {
        b = b / (1.0 + d * L[nmat + m]);
        s = s + d * b;
        if (Bst) Bst[m] = b;
        for (int o = ost[m]; o < ost[m + 1]; ++o) {
            const double sw = b + okd[o] * s - 1.0;
            if (sw < 0.0) {
                vs += (-100.0 * sw) * okw[o];
                mask |= 1ull << o;
            }
        }
    }
    double disc = 1.0;
    for (int n = 0; n < nmat; ++n) disc = disc / (1.0 + d * L[n]);
    *disc_out = disc;
    *mask_out = mask;
    return disc * vs;
}

__device__ void forward_f64(double *L, double *Vt, const double *z, const double *lam, int nn,
                            int nmat, double d, double sqd)
{
    for (int n = 0; n < nmat; ++n) {
        const double sqez = sqd * z[n];
        double v = 0.0;
        for (int i = n + 1; i < nn; ++i) {
            const double l = lam[i - n - 1];
            const double con1 = d * l;
            v += con1 * L[i] / (1.0 + d * L[i]);
            L[i] = L[i] * exp(con1 * v + l * (sqez - 0.5 * con1));
        }
        if (Vt) Vt[n] = v;
    }
}

__global__ void __launch_bounds__(kF64Block)
k_f64_greeks(const DevModel m, const double *__restrict__ z, const Work w)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int nn = m.nn, nmat = m.nmat, M = nn - nmat, nout = w.nout;
    const int NW = kF64Block / 32;
    double *lam_s = reinterpret_cast<double *>(smem);
    double *okd_s = lam_s + kMaxNN;
    double *okw_s = okd_s + kMaxNopt;
    double *acc_s = okw_s + kMaxNopt;
    int *ost_s = reinterpret_cast<int *>(acc_s + NW * 2 * nout);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int scen = blockIdx.x / w.items, item = blockIdx.x % w.items;
    for (int i = tid; i < nn; i += kF64Block) lam_s[i] = m.lamd[i];
    for (int i = tid; i <= M; i += kF64Block) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += kF64Block) {
        okd_s[i] = m.optKd[i];
        okw_s[i] = m.optWd[i];
    }
    for (int i = tid; i < NW * 2 * nout; i += kF64Block) acc_s[i] = 0.0;
    __syncthreads();
    double *acc = acc_s + warp * 2 * nout;
    const double d = m.deltad, sqd = m.sqdd;
    const double *L0 = m.L0d + (size_t)scen * nn;

    double L[kMaxNN], Pb[kMaxNN], vg[kMaxNN], Vt[kMaxNN], Bs[kMaxNN];
    const int64_t ibase = (int64_t)item * w.ppt * kF64Block;
    for (int j = 0; j < w.ppt; ++j) {
        if (ibase + (int64_t)j * kF64Block >= w.paths) break;
        const int64_t pl = ibase + (int64_t)j * kF64Block + tid;
        const bool active = pl < w.paths;
        const double *zp = z + (active ? pl : w.paths - 1) * nmat;
        for (int i = 0; i < nn; ++i) {
            L[i] = L0[i];
            vg[i] = 0.0;
        }
        forward_f64(L, Vt, zp, lam_s, nn, nmat, d, sqd);
        double disc;
        unsigned long long mask;
        const double V = payoff_value_f64(L, nn, nmat, d, ost_s, okd_s, okw_s, &disc, Bs, &mask);
        // payoff adjoint (:173-184 with the rate kept apart from its adjoint,
        // then :199-209), written as log-adjoints Pb = L * dV/dL. B[m] comes
        // from the forward as in the reference: rebuilding it backwards from
        // the last factor underflows on paths whose rates explode.
        {
            double Sb = 0.0, Bb = 0.0;
            for (int mm = M - 1; mm >= 0; --mm) {
                const double Bm = Bs[mm];
                const double Ln = L[nmat + mm];
                for (int o = ost_s[mm]; o < ost_s[mm + 1]; ++o) {
                    if ((mask >> o) & 1ull) {
                        Sb += (-100.0 * okd_s[o]) * okw_s[o];
                        Bb += -100.0 * okw_s[o];
                    }
                }
                Bb += d * Sb;
                const double den = 1.0 + d * Ln;
                Pb[nmat + mm] = disc * (-Bb * Bm * d / den) * Ln;
                Bb = Bb / den;
            }
            for (int n = 0; n < nmat; ++n) Pb[n] = (-V * d / (1.0 + d * L[n])) * L[n];
        }
        for (int n = nmat - 1; n >= 0; --n) {
            const double sqez = sqd * zp[n];
            double v = Vt[n], v1 = 0.0;
            for (int i = nn - 1; i > n; --i) {
                const double l = lam_s[i - n - 1];
                const double con1 = d * l;
                const double wexp = con1 * v + l * (sqez - 0.5 * con1);
                const double Ln = L[i] * exp(-wexp);         // L_{n,i} from L_{n+1,i}
                const double r = 1.0 / (1.0 + d * Ln);
                const double t = Ln * r;
                const double pb = Pb[i];
                v1 += l * pb;                                 // :108
                vg[i - n - 1] += pb * (d * v + sqez - d * l) + d * d * t * v1;
                Pb[i] = pb + d * con1 * t * r * v1;           // :110-111 in log form
                v -= con1 * t;
                L[i] = Ln;
            }
        }
        // reduce this batch: value, deltas Pb/L0, vegas
        for (int o = 0; o < nout; ++o) {
            double x;
            if (o == 0) x = V;
            else if (o <= nn) x = Pb[o - 1] / L0[o - 1];
            else x = vg[o - 1 - nn];
            x = active ? x : 0.0;
            const double s1 = warp_sum(x), s2 = warp_sum(x * x);
            if (lane == 0) {
                acc[o] += s1;
                acc[nout + o] += s2;
            }
        }
    }
    __syncthreads();
    for (int o = tid; o < 2 * nout; o += kF64Block) {
        double s = 0.0;
        for (int q = 0; q < NW; ++q) s += acc_s[q * 2 * nout + o];
        w.partial[(size_t)blockIdx.x * 2 * nout + o] = s;
    }
}

// Plain FP64 bump-and-revalue: block b covers virtual scenario vs = b/items
// = (scenario, variant j); j = 0 is the base, j = 1..nn bumps L0[j-1] by h,
// j = nn+1..2nn bumps lambda[j-nn-1] by h; with `central`, j = 2nn+1..4nn
// repeat those 2nn inputs bumped by -h. Output per variant: mean value.
__global__ void __launch_bounds__(kF64Block)
k_f64_bump(const DevModel m, const double *__restrict__ z, double h, int central, const Work w)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int nn = m.nn, nmat = m.nmat, M = nn - nmat;
    const int NW = kF64Block / 32;
    double *lam_s = reinterpret_cast<double *>(smem);
    double *okd_s = lam_s + kMaxNN;
    double *okw_s = okd_s + kMaxNopt;
    double *acc_s = okw_s + kMaxNopt;
    int *ost_s = reinterpret_cast<int *>(acc_s + NW * 2);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = central ? 1 + 4 * nn : 1 + 2 * nn;
    const int vs = blockIdx.x / w.items, item = blockIdx.x % w.items;
    const int scen = vs / nb, vb = vs % nb;
    // input bumped: 1..nn the rate L0[var-1], nn+1..2nn lambda[var-nn-1]; by hb
    const int var = vb > 2 * nn ? vb - 2 * nn : vb;
    const double hb = vb > 2 * nn ? -h : h;
    for (int i = tid; i < nn; i += kF64Block)
        lam_s[i] = m.lamd[i] + ((var > nn && i == var - nn - 1) ? hb : 0.0);
    for (int i = tid; i <= M; i += kF64Block) ost_s[i] = m.opt_start[i];
    for (int i = tid; i < m.nopt; i += kF64Block) {
        okd_s[i] = m.optKd[i];
        okw_s[i] = m.optWd[i];
    }
    if (tid < NW * 2) acc_s[tid] = 0.0;
    __syncthreads();
    const double d = m.deltad, sqd = m.sqdd;
    const double *L0 = m.L0d + (size_t)scen * nn;
    double L[kMaxNN];
    const int64_t ibase = (int64_t)item * w.ppt * kF64Block;
    for (int j = 0; j < w.ppt; ++j) {
        if (ibase + (int64_t)j * kF64Block >= w.paths) break;
        const int64_t pl = ibase + (int64_t)j * kF64Block + tid;
        const bool active = pl < w.paths;
        const double *zp = z + (active ? pl : w.paths - 1) * nmat;
        for (int i = 0; i < nn; ++i) L[i] = L0[i] + ((var >= 1 && var <= nn && i == var - 1) ? hb : 0.0);
        forward_f64(L, nullptr, zp, lam_s, nn, nmat, d, sqd);
        double disc;
        unsigned long long mask;
        double V = payoff_value_f64(L, nn, nmat, d, ost_s, okd_s, okw_s, &disc, nullptr, &mask);
        V = active ? V : 0.0;
        const double s1 = warp_sum(V), s2 = warp_sum(V * V);
        if (lane == 0) {
            acc_s[warp * 2] += s1;
            acc_s[warp * 2 + 1] += s2;
        }
    }
    __syncthreads();
    if (tid < 2) {
        double s = 0.0;
        for (int q = 0; q < NW; ++q) s += acc_s[q * 2 + tid];
        w.partial[(size_t)blockIdx.x * 2 + tid] = s;
    }
}

size_t f64_smem_bytes(int nout)
{
    return sizeof(double) * (kMaxNN + 2 * kMaxNopt + (kF64Block / 32) * 2 * (size_t)nout) +
           sizeof(int) * (kMaxNN + 1);
}

}  // namespace

int f64_block_threads() { return kF64Block; }

cudaError_t f64_blocks_per_sm(bool bump, int *blocks)
{
    if (bump) {
        const size_t sm = f64_smem_bytes(1);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_f64_bump, kF64Block, sm);
    }
    const size_t sm = f64_smem_bytes(1 + 2 * kMaxNN);
    cudaError_t e = cudaFuncSetAttribute(k_f64_greeks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_f64_greeks, kF64Block, sm);
}

cudaError_t launch_f64_greeks(const DevModel &m, const double *z, const Work &w, cudaStream_t s)
{
    const size_t sm = f64_smem_bytes(w.nout);
    cudaError_t e = cudaFuncSetAttribute(k_f64_greeks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f64_smem_bytes(1 + 2 * kMaxNN));
    if (e != cudaSuccess) return e;
    k_f64_greeks<<<(unsigned)((int64_t)m.nscen * w.items), kF64Block, sm, s>>>(m, z, w);
    return cudaGetLastError();
}

cudaError_t launch_f64_bump(const DevModel &m, const double *z, double h, bool central, const Work &w,
                            cudaStream_t s)
{
    const int nb = central ? 1 + 4 * m.nn : 1 + 2 * m.nn;
    const size_t sm = f64_smem_bytes(1);
    k_f64_bump<<<(unsigned)((int64_t)m.nscen * nb * w.items), kF64Block, sm, s>>>(m, z, h, central ? 1 : 0, w);
    return cudaGetLastError();
}

}  // namespace lmm

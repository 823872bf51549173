/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY. Wraps the UNMODIFIED reference
 * LiborMarketModel/liborSwaptionGreeks.cpp (included from the reference tree
 * at build time, never copied) so that the tests can drive it through ctypes:
 *
 *   ref_entry        the reference entry point liborSwaptionGreeks
 *                    (liborSwaptionGreeks.cpp:241-368) on caller-supplied
 *                    normals; returns NLOOPS x the MC mean, as the reference
 *                    does (:278,:355-356).
 *   ref_block        one SIMDVLEN-path block through the static kernels
 *                    path_calc_b1 (:34), portfolio_b (:120), path_calc_b2
 *                    (:86) with caller-chosen L0/lambda, as :303-344 does;
 *                    returns the per-path value and the per-path rate
 *                    adjoint left in L (aliased as in the reference, :178).
 *   ref_block_value  path_calc_b1 + portfolio_b only (the value), so that
 *                    finite differences can be taken with the reference's own
 *                    arithmetic.
 *
 * generateRand (LiborMarketModel/mklRng.cpp:44) is replaced by a no-op: the
 * caller fills z, so the reference and every other implementation consume the
 * same normals. mkl_vsl.h comes from oracle/shim (one typedef).
 * Build recipe: oracle/build_ref.py -> oracle/_ref/.
 */
#include "liborSwaptionGreeks.cpp"

#include <cstring>

void generateRand(REAL *z, int num, REAL mean, REAL stddev, int seed)
{
    (void)z; (void)num; (void)mean; (void)stddev; (void)seed;
}

extern "C" {

int ref_nn(void) { return NN; }
int ref_nmat(void) { return NMAT; }
int ref_nopt(void) { return NOPT; }
int ref_simdvlen(void) { return SIMDVLEN; }
int ref_nloops(void) { return NLOOPS; }
int ref_real_bytes(void) { return (int)sizeof(REAL); }

void ref_entry(REAL *z, int numPaths, REAL *d_v, REAL *d_Lb)
{
    liborSwaptionGreeks(z, NMAT * numPaths, (REAL)0, (REAL)1, 1234, d_v, d_Lb, numPaths);
}

static void load_block(REAL L[][SIMDVLEN], REAL (*L2)[SIMDVLEN], const REAL *L0)
{
    for (int i = 0; i < NN; ++i)
        for (int j = 0; j < SIMDVLEN; ++j) L[i][j] = L0[i];
    for (int i = 0; i < L2_SIZE; ++i)
        for (int j = 0; j < SIMDVLEN; ++j) L2[i][j] = (REAL)0;
}

/* z: [SIMDVLEN][NMAT] path-major; value: [SIMDVLEN]; Lb: [NN][SIMDVLEN]. */
void ref_block(const REAL *z, const REAL *L0, const REAL *lambda, REAL *value, REAL *Lb)
{
    REAL (*L)[SIMDVLEN] = new REAL[NN][SIMDVLEN];
    REAL (*L2)[SIMDVLEN] = new REAL[L2_SIZE][SIMDVLEN];
    load_block(L, L2, L0);
    path_calc_b1(const_cast<REAL *>(z), L, L2, lambda);
    portfolio_b(L, value);
    path_calc_b2(L, L2, lambda);
    std::memcpy(Lb, L, sizeof(REAL) * NN * SIMDVLEN);
    delete[] L;
    delete[] L2;
}

void ref_block_value(const REAL *z, const REAL *L0, const REAL *lambda, REAL *value)
{
    REAL (*L)[SIMDVLEN] = new REAL[NN][SIMDVLEN];
    REAL (*L2)[SIMDVLEN] = new REAL[L2_SIZE][SIMDVLEN];
    load_block(L, L2, L0);
    path_calc_b1(const_cast<REAL *>(z), L, L2, lambda);
    portfolio_b(L, value);
    delete[] L;
    delete[] L2;
}

/* The portfolio as compiled into the reference (params.h:38-40). */
void ref_portfolio(int *mat, double *rates)
{
    for (int o = 0; o < NOPT; ++o) {
        mat[o] = maturities[o];
        rates[o] = (double)swaprates[o];
    }
}

} /* extern "C" */

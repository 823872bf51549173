// Drop-in replacement of the reference's compute and RNG translation units.
//
// Build the reference's driver with this file instead of
// LiborMarketModel/liborSwaptionGreeks.cpp and LiborMarketModel/mklRng.cpp,
// keeping main.cpp, params.h, Timer.hpp, mklRng.h and liborSwaptionGreeks.hpp
// unchanged, and link liblmm_gb300.so:
//
//   g++ -O2 -DUSE_DOUBLE -fopenmp -I <reference>/LiborMarketModel -I <repo>/include \
//       -I <dir with an mkl_vsl.h that declares VSLStreamStatePtr, if MKL is absent> \
//       <reference>/LiborMarketModel/main.cpp liborSwaptionGreeks_gb300.cpp \
//       -L <lib dir> -llmm_gb300 -Wl,-rpath,<lib dir>
//
// liborSwaptionGreeks (liborSwaptionGreeks.hpp:12-13) keeps its signature
// and its meaning: z is refilled with N(mean, std_dev) normals from an
// MRG32k3a stream seeded with 12345, read from element 0 and inverted by
// AS241 (the reference's generator family and stream order; define
// LMM_SHIM_PHILOX for the library's Philox stream instead), and the
// params.h portfolio is priced on the GPU. The reference repeats its
// Monte Carlo NLOOPS = 10 times and divides by numPaths only
// (liborSwaptionGreeks.cpp:27,278,355-356), so its outputs are 10x the
// means; the shim multiplies by NLOOPS to print the same figures.
#include "params.h"
#include "liborSwaptionGreeks.hpp"
#include "lmm_gb300.h"

#include <cstdio>
#include <cstdlib>

namespace {
constexpr int kReferenceLoops = 10;   // NLOOPS, liborSwaptionGreeks.cpp:27

void check(int rc)
{
    if (rc != LMM_OK) {
        std::fprintf(stderr, "liborSwaptionGreeks: %s (%s)\n", lmm_status_string(rc), lmm_last_error());
        std::exit(EXIT_FAILURE);
    }
}
}  // namespace

// mklRng.cpp's generateRand: main.cpp fills z once before the timed call;
// liborSwaptionGreeks refills it from the library's stream, so nothing is
// drawn here.
void generateRand(REAL *, int, REAL, REAL, int) {}

void liborSwaptionGreeks(REAL *z, int num, REAL mean, REAL std_dev, int seed, REAL *d_v, REAL *d_Lb,
                         int numPaths)
{
#ifdef USE_DOUBLE
#ifdef LMM_SHIM_PHILOX
    check(lmm_swaption_greeks(z, num, mean, std_dev, seed, d_v, d_Lb, numPaths));
#else
    check(lmm_swaption_greeks_mrg32k3a(z, num, mean, std_dev, seed, d_v, d_Lb, numPaths));
#endif
#else
#ifdef LMM_SHIM_PHILOX
    check(lmm_swaption_greeks_f32(z, num, mean, std_dev, seed, d_v, d_Lb, numPaths));
#else
    check(lmm_swaption_greeks_mrg32k3a_f32(z, num, mean, std_dev, seed, d_v, d_Lb, numPaths));
#endif
#endif
    *d_v *= kReferenceLoops;
    *d_Lb *= kReferenceLoops;
}

/* Test stand-in for the reference's LiborMarketModel/liborSwaptionGreeks.hpp:
 * the one entry point it declares (liborSwaptionGreeks.hpp:12-13), which the
 * drop-in shim defines. */
#ifndef LMM_TEST_LIBORSWAPTIONGREEKS_HPP
#define LMM_TEST_LIBORSWAPTIONGREEKS_HPP
#include "params.h"
void liborSwaptionGreeks(REAL *z, int num, REAL mean, REAL std_dev, int seed, REAL *d_v, REAL *d_Lb,
                         int numPaths);
#endif

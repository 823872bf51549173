/* Test stand-in for the reference's LiborMarketModel/params.h (params.h:10-24):
 * only the REAL type the drop-in shim needs, double with USE_DOUBLE as in the
 * reference's FP64 build, float otherwise. */
#ifndef LMM_TEST_PARAMS_H
#define LMM_TEST_PARAMS_H
#ifdef USE_DOUBLE
typedef double REAL;
#else
typedef float REAL;
#endif
#endif

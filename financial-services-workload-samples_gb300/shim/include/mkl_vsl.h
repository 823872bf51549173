/* Stand-in for MKL's mkl_vsl.h where MKL is absent: the reference's driver
 * (LiborMarketModel/main.cpp, mklRng.h) only needs the stream handle type to
 * compile; with the drop-in shim no MKL function is called. */
#ifndef LMM_DROPIN_MKL_VSL_H
#define LMM_DROPIN_MKL_VSL_H
typedef void *VSLStreamStatePtr;
#endif

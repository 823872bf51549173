/* Stand-in for MKL's mkl_vsl.h, which is closed and absent here. The
 * reference only needs the stream handle type to compile
 * (LiborMarketModel/mklRng.h:10-13, main.cpp:59); its generateRand is
 * replaced by oracle/ref_harness.cpp, so no MKL function is ever called. */
#ifndef LMM_SHIM_MKL_VSL_H
#define LMM_SHIM_MKL_VSL_H
typedef void *VSLStreamStatePtr;
#endif

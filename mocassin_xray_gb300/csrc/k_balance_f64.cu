// k_balance_f64.cu - the balance kernels in FP64 throughout, compiled with
// --fmad=false: the plain path checked against the oracle.
#define MCX_BAL_REAL double
#define MCX_BAL_NS bal_f64
#define MCX_BAL_EXACT 1
#include "k_balance_impl.cuh"

// k_balance_mixed.cu - the balance kernels with FP32 rates, collision
// strengths and exponentials; the level-population LU, the ionisation ladder
// and the Te bracketing stay FP64.
#define MCX_BAL_REAL float
#define MCX_BAL_NS bal_mixed
#define MCX_BAL_EXACT 0
#include "k_balance_impl.cuh"

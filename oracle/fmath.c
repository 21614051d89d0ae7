/*
 * fmath.c - array entry points of the portable FP64 exp / log / log10 / pow
 * (mcx_fmath.h), so that the CPU tests can check them against the host's libm.
 *
 * TEST INFRASTRUCTURE ONLY.
 */
#include "oracle.h"
#include "mcx_fmath.h"

void orc_fm_eval(int32_t fn, const double* x, const double* y, int64_t n, double* out) {
    for (int64_t i = 0; i < n; ++i) {
        switch (fn) {
        case 0: out[i] = mcx_fm_exp(x[i]); break;
        case 1: out[i] = mcx_fm_log(x[i]); break;
        case 2: out[i] = mcx_fm_log10(x[i]); break;
        case 4: out[i] = mcx_fm_sin(x[i]); break;
        case 5: out[i] = mcx_fm_cos(x[i]); break;
        default: out[i] = mcx_fm_pow(x[i], y[i]); break;
        }
    }
}

// k_gaunt.cuh - Hummer (1988) free-free Gaunt factor fit of getGauntFF
// (source/ionization_mod.f90:196-334), FP32 device functions shared by the
// opacity and emission kernels.
#pragma once
#include <cuda_runtime.h>

namespace mcx {

namespace {

__constant__ double kGauntD[88] = {
    8.986940175e+00, -4.009515855e+00, 8.808871266e-01, 2.640245111e-02, -4.580645915e-02, -3.568055702e-03,
    2.827798067e-03, 3.365860195e-04, -8.006936989e-01, 9.466021705e-01, 9.043402532e-02, -9.608451450e-02,
    -1.885629865e-02, 1.050313890e-02, 2.800889961e-03, -1.078209202e-03, -3.781305103e-01, 1.102726332e-01,
    -1.543619180e-02, 8.310561114e-03, 2.179620525e-02, 4.259726289e-03, -4.181588794e-03, -1.770208330e-03,
    1.877213132e-02, -1.004885705e-01, -5.483366378e-02, -4.520154409e-03, 8.366530426e-03, 3.700273930e-03,
    6.889320423e-04, 9.460313195e-05, 7.300158392e-02, 3.576785497e-03, -4.545307025e-03, -1.017965604e-02,
    -9.530211924e-03, -3.450186162e-03, 1.040482914e-03, 1.407073544e-03, -1.744671550e-03, 2.864013856e-02,
    1.903394837e-02, 7.091074494e-03, -9.668371391e-04, -2.999107465e-03, -1.820642230e-03, -3.874082085e-04,
    -1.707268366e-02, -4.694254776e-03, 1.311691517e-03, 5.316703136e-03, 5.178193095e-03, 2.451228935e-03,
    -2.277321615e-05, -8.182359057e-04, 2.567331664e-04, -9.155339970e-03, -6.997479192e-03, -3.571518641e-03,
    -2.096101038e-04, 1.553822487e-03, 1.509584686e-03, 6.212627837e-04, 4.098322531e-03, 1.635218463e-03,
    -5.918883504e-04, -2.333091048e-03, -2.484138313e-03, -1.359996060e-03, -5.371426147e-05, 5.553549563e-04,
    3.837562402e-05, 2.938325230e-03, 2.393747064e-03, 1.328839809e-03, 9.135013312e-05, -7.137252303e-04,
    -7.656848158e-04, -3.504683798e-04, -8.491991820e-04, -3.615327726e-04, 3.148015257e-04, 8.909207650e-04,
    9.869737522e-04, 6.134671184e-04, 1.068883394e-04, -2.046080100e-04};

}  // namespace

// Hummer (1988) Chebyshev fit: per-temperature coefficients c(1..8) and
// gamma^2 (getGauntFF, source/ionization_mod.f90:262-276).
__device__ inline void gauntCoeffs(float z, float log10Te, float c[9], float& con, float& gamma2) {
  float xlrkt;
  if (log10Te < 2.5f) xlrkt = 5.1983649f - 2.5f;
  else if (log10Te > 8.f) xlrkt = 5.1983649f - 8.f;
  else xlrkt = 5.1983649f - log10Te;
  float txg = 0.66666667f * (2.0f * z + xlrkt);
  gamma2 = exp10f(txg * 1.5f);
  con = 0.72727273f * xlrkt + 0.90909091f;
  float b[12];
  for (int j = 1; j <= 8; ++j) {
    int ir = 9;
    b[11] = (float)kGauntD[(j - 1) + 8 * 10];
    b[10] = txg * b[11] + (float)kGauntD[(j - 1) + 8 * 9];
    for (int i = 1; i <= 9; ++i) {
      b[ir] = txg * b[ir + 1] - b[ir + 2] + (float)kGauntD[(j - 1) + 8 * (ir - 1)];
      ir = ir - 1;
    }
    c[j] = 0.25f * (b[1] - b[3]);
  }
}

// getGauntFF frequency part (source/ionization_mod.f90:278-331)
__device__ inline float gauntAt(const float c[9], float con, float gamma2, float log10nu) {
  float txu = 0.72727273f * log10nu + con;
  float u = exp10f((txu - .90909091f) / .72727273f);
  if (fabsf(txu) <= 2.0f) {
    float b[9];
    int ir = 6;
    b[8] = c[8];
    b[7] = txu * b[8] + c[7];
    for (int j = 1; j <= 6; ++j) { b[ir] = txu * b[ir + 1] - b[ir + 2] + c[ir]; ir = ir - 1; }
    return b[1] - b[3];
  }
  float lu = log10f(u);
  if (lu < -4.0f && gamma2 < 0.3f) return 0.551329f * logf(2.24593f / u);
  if (lu < -4.0f && gamma2 >= 0.3f) return 0.551329f * logf(0.944931f / u / sqrtf(gamma2));
  if (txu > 2.0f) {
    float lg = log10f(gamma2);
    if (lg < -3.f) return sqrtf(0.9549297f / u);
    if (lg < 0.0f) {
      float slope = (sqrtf(12.f * gamma2 / u) - sqrtf(0.9549297f / u)) / 3.0f;
      return sqrtf(12.f * gamma2 / u) + slope * lg;
    }
    return fminf(1.05f, sqrtf(12.f * gamma2 / u));
  }
  return 0.f;
}

}  // namespace mcx

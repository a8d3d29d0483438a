// pair_math.cuh -- FP32 pair-term helpers shared by the real-space kernels.
#pragma once

namespace tcp {

// t Q(t) with the coefficients printed by fit_erfc.py (P = 0.5, degree 8):
// erfc(x) = exp(-x^2) t Q(t), t = 1/(1 + x/2).
__device__ __forceinline__ float erfc_poly(float t) {
    float q = -5.783473762e-02f;
    q = fmaf(q, t, 2.784859768e-01f);
    q = fmaf(q, t, -4.744286455e-01f);
    q = fmaf(q, t, 2.632348585e-01f);
    q = fmaf(q, t, -1.622527577e-02f);
    q = fmaf(q, t, 1.981928108e-01f);
    q = fmaf(q, t, 2.442685012e-01f);
    q = fmaf(q, t, 2.822102988e-01f);
    q = fmaf(q, t, 2.820961743e-01f);
    return q * t;
}

}  // namespace tcp

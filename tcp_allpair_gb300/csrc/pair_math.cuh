// pair_math.cuh -- FP32 pair-term helpers shared by the real-space kernels.
#pragma once

namespace tcp {

// erfc(x) = exp(-x^2) t Q(t), t = 1/(1 + kErfcP x): the factor of the
// reciprocal argument (host constants p_alpha = kErfcP alpha, p_lam = kErfcP/lambda).
constexpr double kErfcP = 0.4;

// t Q(t) with the coefficients printed by fit_erfc.py (P = 0.4, degree 7).
__device__ __forceinline__ float erfc_poly(float t) {
    float q = 6.807732388e-02f;
    q = fmaf(q, t, -3.663086635e-01f);
    q = fmaf(q, t, 6.308091155e-01f);
    q = fmaf(q, t, -3.190751584e-01f);
    q = fmaf(q, t, 3.760577549e-01f);
    q = fmaf(q, t, 1.510029235e-01f);
    q = fmaf(q, t, 2.343213173e-01f);
    q = fmaf(q, t, 2.251152860e-01f);
    return q * t;
}

}  // namespace tcp

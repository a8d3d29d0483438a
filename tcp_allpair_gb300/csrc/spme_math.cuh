// spme_math.cuh -- B-spline charge-assignment weights shared by the SPME
// kernels of the single-system and the batched paths.
#pragma once

#include <cuda_runtime.h>

namespace tcp {

// B-spline weights W[j] = M_P(w + P-1-j) and dW[j] = dM_P/du on the grid
// points INT(u) + j - (P-3).  Order 4 uses the reference's explicit cubics
// (force.f90:703-738); other orders the Cox-de Boor recursion run upward on
// the P nonzero values.
template <int P, typename T>
__device__ __forceinline__ void spline_w(double u, T *W, T *dW) {
    if (P == 4) {
        T z = (T)(trunc(u) - u + 1.0);
        W[0] = z * z * z / (T)6;
        dW[0] = (T)-3. * z * z / (T)6;
        z += (T)1;
        W[1] = ((T)-3. * z * z * z + (T)12. * z * z - (T)12. * z + (T)4.) / (T)6;
        dW[1] = ((T)9. * z * z - (T)24. * z + (T)12.) / (T)6;
        z += (T)1;
        W[2] = ((T)3. * z * z * z - (T)24. * z * z + (T)60. * z - (T)44.) / (T)6;
        dW[2] = ((T)-9. * z * z + (T)48. * z - (T)60.) / (T)6;
        z += (T)1;
        W[3] = (-z * z * z + (T)12. * z * z - (T)48. * z + (T)64.) / (T)6;
        dW[3] = ((T)3. * z * z - (T)24. * z + (T)48.) / (T)6;
        return;
    }
    const T w = (T)(u - trunc(u));
    T a[P];
    a[0] = (T)1;
#pragma unroll
    for (int j = 1; j < P; ++j) a[j] = (T)0;
    // a_n[j] = ((w+n-1-j) a_{n-1}[j-1] + (1-w+j) a_{n-1}[j]) / (n-1)
#pragma unroll
    for (int nn = 2; nn <= P; ++nn) {
        if (nn == P) {
#pragma unroll
            for (int j = 0; j < P; ++j) dW[j] = (j > 0 ? a[j - 1] : (T)0) - (j < P - 1 ? a[j] : (T)0);
        }
        const T inv = (T)1 / (T)(nn - 1);
#pragma unroll
        for (int j = nn - 1; j >= 0; --j) {
            const T left = j > 0 ? a[j - 1] : (T)0;
            const T right = j < nn - 1 ? a[j] : (T)0;
            a[j] = ((w + (T)(nn - 1 - j)) * left + ((T)1 - w + (T)j) * right) * inv;
        }
    }
#pragma unroll
    for (int j = 0; j < P; ++j) W[j] = a[j];
}

// Weights with first and second derivatives (d/du, d^2/du^2) for every order
// P >= 4 by the same recursion: the order P-2 values give
// M_P''(y) = M_{P-2}(y) - 2 M_{P-2}(y-1) + M_{P-2}(y-2), the order P-1 values
// M_P'(y) = M_{P-1}(y) - M_{P-1}(y-1).
template <int P>
__device__ __forceinline__ void spline_w2(double u, double *W, double *dW, double *d2W) {
    const double w = u - trunc(u);
    double a[P];
    a[0] = 1.0;
#pragma unroll
    for (int j = 1; j < P; ++j) a[j] = 0.0;
#pragma unroll
    for (int nn = 2; nn <= P; ++nn) {
        if (nn == P - 1) {
#pragma unroll
            for (int j = 0; j < P; ++j)
                d2W[j] = (j >= 2 ? a[j - 2] : 0.0) - 2.0 * (j >= 1 && j - 1 < P - 2 ? a[j - 1] : 0.0) +
                         (j < P - 2 ? a[j] : 0.0);
        }
        if (nn == P) {
#pragma unroll
            for (int j = 0; j < P; ++j) dW[j] = (j > 0 ? a[j - 1] : 0.0) - (j < P - 1 ? a[j] : 0.0);
        }
        const double inv = 1.0 / (double)(nn - 1);
#pragma unroll
        for (int j = nn - 1; j >= 0; --j) {
            const double left = j > 0 ? a[j - 1] : 0.0;
            const double right = j < nn - 1 ? a[j] : 0.0;
            a[j] = ((w + (double)(nn - 1 - j)) * left + (1.0 - w + (double)j) * right) * inv;
        }
    }
#pragma unroll
    for (int j = 0; j < P; ++j) W[j] = a[j];
}

__device__ __forceinline__ int wrapi(int i, int K) {
    i %= K;
    return i < 0 ? i + K : i;
}

}  // namespace tcp

// pair_math.cuh -- FP32 pair-term helpers shared by the real-space kernels.
#pragma once

#include "device_util.cuh"
#include "tcp_internal.h"

namespace tcp {

// Exact RDF bin of one pair from its fixed-point separations (RdfEdges):
// `bin` is the FP32 estimate on entry and the exact bin on return; *ok is
// set to whether r < rc holds exactly.  The estimate is within one bin, so
// each loop runs at most once in practice.
template <bool CUBIC>
__device__ __forceinline__ int rdf_exact_bin(int d0, int d1, int d2, const RdfEdges *__restrict__ E, int t,
                                             const double *box, int bin, bool &ok) {
    bin = min(max(bin, 0), kNbin);
    if (CUBIC) {
        const long long a = d0, b = d1, c = d2;
        const unsigned long long q =
            (unsigned long long)(a * a) + (unsigned long long)(b * b) + (unsigned long long)(c * c);
        ok = q < E->rc2;
        while (bin > 0 && q < __ldg(&E->e[t][bin])) --bin;
        while (bin < kNbin && q >= __ldg(&E->e[t][bin + 1])) ++bin;
    } else {
        constexpr double k2m32 = 1.0 / 4294967296.0;
        const double a = (double)d0 * (box[0] * k2m32), b = (double)d1 * (box[1] * k2m32),
                     c = (double)d2 * (box[2] * k2m32);
        const double q = a * a + b * b + c * c;
        ok = q < E->rc2d;
        while (bin > 0 && q < __ldg(&E->d[t][bin])) --bin;
        while (bin < kNbin && q >= __ldg(&E->d[t][bin + 1])) ++bin;
    }
    return bin;
}

// true when the FP32 bin estimate tb = r/dx or r^2 (against rc^2) is too
// close to an edge to be trusted
__device__ __forceinline__ bool rdf_near_edge(float tb, int bin, float r2, float rc2) {
    const float fr = tb - (float)bin;
    return fr < kRdfEdge || fr > 1.0f - kRdfEdge || fabsf(r2 - rc2) < kRdfEdge * rc2;
}

// erfc(x) = exp(-x^2) t Q(t), t = 1/(1 + kErfcP x): the factor of the
// reciprocal argument (host constants p_alpha = kErfcP alpha, p_lam = kErfcP/lambda).
constexpr double kErfcP = 0.36;

// Q(t) of degree kErfcDeg, coefficients printed by fit_erfc.py (highest power
// first), listed once here for the scalar and the packed evaluations.
constexpr int kErfcDeg = 6;
#define TCP_ERFC_Q                                                                                  \
    {-1.717338572e-01f, 5.984714114e-01f, -4.147594920e-01f, 4.816444120e-01f, 8.168755304e-02f,    \
     2.231449970e-01f, 2.015448752e-01f}

// The Ewald term alone needs erfc(x) only for x = alpha r <= alpha rc, which
// is 3.1 for the reference's alpha = 3.1/rc and 3.46 for a 1e-6 Ewald error.
// On [0, kErfc5Xmax] a degree-5 Q with P = kErfc5P (fit_erfc.py --short)
// reaches 8.5e-7 max / 3.7e-7 rms relative error in FP32 Horner form, one
// FMA less per pair than the degree-6 fit; the host selects it when
// alpha rc <= kErfc5Xmax.
constexpr double kErfc5P = 0.41;
constexpr double kErfc5Xmax = 3.6;
constexpr int kErfc5Deg = 5;
#define TCP_ERFC5_Q                                                                                 \
    {-1.858996734e-01f, 6.017686447e-01f, -2.337225564e-01f, 3.931379106e-01f, 1.894349663e-01f,    \
     2.352810149e-01f}

// t Q(t)
__device__ __forceinline__ float erfc_poly(float t) {
    constexpr float q_[kErfcDeg + 1] = TCP_ERFC_Q;
    float q = q_[0];
#pragma unroll
    for (int k = 1; k <= kErfcDeg; ++k) q = fmaf(q, t, q_[k]);
    return q * t;
}

// Kelbg e-i pairs at r < lambda/2 with alpha r < 1/2: erfc(alpha r) and
// g = exp(-r^2/lambda^2) both tend to 1 as r -> 0, and the force numerator
// erfc(x) + 2x/sqrt(pi) e^{-x^2} - g (x = alpha r) is left with the FP32
// rounding of its terms divided by its own size (~ r^2/lambda^2).  Rewritten as
//   (1 - g) + h(x),  h(x) = 2x/sqrt(pi) e^{-x^2} - erf(x) = x^3 H(x^2),
// and the energy numerator erfc(x) - g as (1 - g) - erf(x), erf(x) = x E(x^2),
// with Taylor series for 1 - e^{-y} (y = r^2/lambda^2 <= 1/4, six terms,
// 5e-8 relative), h (eight terms, 1e-8 for x <= 1/2) and erf (eight terms,
// 2e-11), every part keeps its relative accuracy.  Arguments y = r^2/lambda^2,
// x = alpha r; returns r * (force numerator) and r * (energy numerator
// without the sqrt(pi)/lambda erfc(r/lambda) term).
__device__ __forceinline__ void kelbg_close(float y, float x, float &num_f, float &num_e) {
    const float z = x * x;
    const float one_m_g =
        y * fmaf(fmaf(fmaf(fmaf(fmaf(-1.0f / 720.0f, y, 1.0f / 120.0f), y, -1.0f / 24.0f), y, 1.0f / 6.0f), y, -0.5f),
                 y, 1.0f);
    // coefficients of x^(2n+1), n = 1..8: (-1)^n (2/sqrt(pi)) 2n / ((2n+1) n!)
    float hz = 2.63393830e-05f;
    hz = fmaf(hz, z, -2.08959105e-04f);
    hz = fmaf(hz, z, 1.44663996e-03f);
    hz = fmaf(hz, z, -8.54832702e-03f);
    hz = fmaf(hz, z, 4.17918210e-02f);
    hz = fmaf(hz, z, -1.61197024e-01f);
    hz = fmaf(hz, z, 4.51351667e-01f);
    hz = fmaf(hz, z, -7.52252778e-01f);
    num_f = fmaf(x * z, hz, one_m_g);
    // erf(x) = 2/sqrt(pi) x sum_n (-1)^n z^n / (n! (2n+1)), n = 0..7
    float ez = -1.32275132e-05f;
    ez = fmaf(ez, z, 1.06837607e-04f);
    ez = fmaf(ez, z, -7.57575758e-04f);
    ez = fmaf(ez, z, 4.62962963e-03f);
    ez = fmaf(ez, z, -2.38095238e-02f);
    ez = fmaf(ez, z, 1.00000000e-01f);
    ez = fmaf(ez, z, -3.33333333e-01f);
    ez = fmaf(ez, z, 1.0f);
    num_e = fmaf(-1.1283791671f * x, ez, one_m_g);
}

// ---- FP64, table-driven (the FP64 pair and adjoint kernels) ----------------------
// The tables of fit_erfcx64.py, copied once per CTA into shared memory, where
// each lane indexes them by its own argument.
#include "erfcx64_table.inc"

struct F64Tab {
    double ewq[kEwqDeg + 1][kEwqSeg];   // [k][j]: lanes on different segments use different banks
    double exp2[kExpTab];
};

// all threads of the CTA; the caller synchronises before first use
__device__ __forceinline__ void load_f64_tab(F64Tab &t) {
    for (int i = threadIdx.x; i < (kEwqDeg + 1) * kEwqSeg; i += blockDim.x) (&t.ewq[0][0])[i] = (&kEwqTab[0][0])[i];
    for (int i = threadIdx.x; i < kExpTab; i += blockDim.x) t.exp2[i] = kExp2Tab[i];
}

constexpr double kRound52 = 6755399441055744.0;   // 1.5 * 2^52: x + kRound52 holds rint(x) in its low word
constexpr double kTwoOverSqrtPi = 1.1283791670955126;

// exp(-z) for 0 <= z < 700 (0 beyond): -z = k ln2/256 + f with
// k = rint(-256 z/ln2) and |f| <= ln2/512, exp(-z) = 2^(k >> 8) 2^((k & 255)/256)
// (1 + p(f)), p the degree-4 Taylor polynomial of exp(f) - 1 (truncation
// 4e-17).  The first reduction step is exact (one FMA of a 16-bit k), ln2/256
// is split in two doubles; relative error 2e-16.  9 FP64 operations.
__device__ __forceinline__ double exp_neg_tab(double z, const F64Tab &t) {
    constexpr double kInvLn2x256 = 369.3299304675746;
    constexpr double kLn2d256Hi = 0.0027076061740622863, kLn2d256Lo = 9.058776616587108e-20;
    const double kd = fma(z, -kInvLn2x256, kRound52);
    const int k = __double2loint(kd);
    const double kf = kd - kRound52;
    double f = fma(-kf, kLn2d256Hi, -z);
    f = fma(-kf, kLn2d256Lo, f);
    double q = fma(f, 1.0 / 24.0, 1.0 / 6.0);
    q = fma(q, f, 0.5);
    q = fma(q, f, 1.0);
    const double tk = t.exp2[k & (kExpTab - 1)];
    const double v = fma(tk, q * f, tk);
    // times 2^(k >> 8) by the exponent field; the result stays normal for z < 700
    const double sc = __hiloint2double((int)((unsigned)__double2hiint(v) + ((unsigned)(k >> 8) << 20)),
                                       __double2loint(v));
    return __double2hiint(z) < 0x4085E000 ? sc : 0.0;   // z < 700 (z >= 0: the high words order as z)
}

// Q(x) = erfcx(x) + 2x/sqrt(pi) for x >= 0, so that the Ewald real-space force
// term erfc(x) + 2x/sqrt(pi) exp(-x^2) is exp(-x^2) Q(x): for x <= 9,
// x = j/8 + h with |h| <= 1/16 and Q by the degree-9 segment polynomial j in h
// (relative error 2e-16); beyond 9 (where exp(-x^2) < 7e-36) and for NaN, 0.
// No branch: the segment index of an argument out of range is replaced by 0
// and its value discarded.  13 FP64 operations.
__device__ __forceinline__ double ewald_q(double x, const F64Tab &t) {
    const bool in = (unsigned)__double2hiint(x) <= 0x40220000u;   // x <= 9 on the high word (x >= 0)
    const double kd = fma(x, 8.0, kRound52);
    const int j = in ? __double2loint(kd) : 0;
    const double h = fma(kd - kRound52, -0.125, x);
    double q = t.ewq[kEwqDeg][j];
#pragma unroll
    for (int k = kEwqDeg - 1; k >= 0; --k) q = fma(q, h, t.ewq[k][j]);
    return in ? q : 0.0;
}

// erfc(x) = g (Q(x) - 2x/sqrt(pi)) for x >= 0 with g = exp(-x^2) from the
// caller (relative error 1e-14 at x = 6 from the cancellation, absolute below
// 2e-16 g Q(x)); 0 beyond 9 (erfc < 5e-37).
__device__ __forceinline__ double erfc_tab(double x, double g, const F64Tab &t) {
    const double v = g * fma(-kTwoOverSqrtPi, x, ewald_q(x, t));
    return (unsigned)__double2hiint(x) <= 0x40220000u ? v : 0.0;
}

// 1/sqrt(x) for positive normal x: the hardware approximation
// (rsqrt.approx.ftz.f64) and two Newton steps y += y (1 - x y^2)/2 written as
// y = fma(y, 0.5 - (x/2) y^2, y).  7 FP64 operations.
__device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double hx = 0.5 * x;
    y = fma(y, fma(-hx, y * y, 0.5), y);
    return fma(y, fma(-hx, y * y, 0.5), y);
}
}  // namespace tcp

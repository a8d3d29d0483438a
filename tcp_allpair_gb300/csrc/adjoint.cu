// adjoint.cu -- derivatives of the force-and-integrate path: dE/dlambda_ei,
// dE/d(charge scale), Hessian-vector products of the potential energy, and
// reverse mode of the mean kinetic temperature through K velocity-Verlet
// steps with checkpoints every M steps and recomputation in between.
//
// The reference computes no derivatives.  These are the analytic derivatives
// of the energy it defines (force.f90 pair terms :99-175, SPME :652-929,
// EWALD_SELF :44-45) and of its discrete NOTEMP step (vverlet.f90:132-223 with
// REMOVE_RIGIDMTN, force.f90:986-1004), for the same parameters.
//
// Pair terms.  For a pair term phi(r) (u = x_i - x_j, qq = eps q_i q_j):
//   G1 = -phi'(r)/r            force on i: qq G1 u
//   G2 = -G1'(r)/r             pair Hessian: qq (-G1 I + G2 u u^T)
//   dl = d phi / d lambda,  gl = d G1 / d lambda
// with lambda = lambda_ei (Kelbg) or rs (Deutsch); only the e-i term depends
// on it.  For erfc(ar)/r, w0 = (erfc(ar)/r + c e)/r^2, c = 2a/sqrt(pi),
// e = exp(-a^2 r^2): G1 = w0, G2 = (3 w0 + 2 a^2 c e)/r^2.  Kelbg adds
// G1 -= g/r^3, G2 -= g (3/r^3 + 2/(l^2 r))/r^2, dl = -sqrt(pi) erfc(r/l)/l^2,
// gl = -2 g/(l^3 r), g = exp(-r^2/l^2).  Deutsch adds G1 -= y (1/(rs r^2) +
// 1/r^3), G2 -= y (3/(rs r^2) + 3/r^3 + 1/(rs^2 r))/r^2, dl = -y/rs^2,
// gl = -y/(rs^3 r), y = exp(-r/rs).
//
// The default real-space kernel (adj_n3_kernel) visits every unique pair once
// on the Newton-3 item schedule of the force kernels and adds +t to row i and
// -t to row j.  With TCP_FLAG_DETERMINISTIC the ordered-pair kernel visits
// every ordered pair (i, j) once: thread i sums
// (H w)_i = sum_j qq (-G1 dw + G2 (u.dw) u), dw = w_i - w_j, and the scalars
// dE/dlambda = 1/2 sum qq dl and dF/dlambda . w = sum qq gl (u.w_i).  The
// j-range is split over gridDim.y; rows are added to hw with FP64 atomics.
// FP64 precision uses CUDA's erfc/exp; FP32C uses the fixed-point separations
// and the SFU forms of the force kernel, per-tile FP32 partials and FP64 sums.
// The reciprocal part (spme.cu) is always FP64.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "device_util.cuh"
#include "pair_math.cuh"
#include "pair_n3.cuh"
#include "tcp_internal.h"

namespace tcp {

constexpr int kAdjThreads = 128;
enum { kAdjDEdl = 0, kAdjDFdl = 1, kAdjJ = 2, kAdjCount = 8 };

struct AdjArgs {
    const int4 *xq;
    const double4_32a *xd;
    const longlong4_32a *xl;   // 64-bit fixed-point positions (FP64 Newton-3 form)
    const double *w;      // [3][n] (HVP) or nullptr
    double *hw;           // [3][n], atomic adds
    double *scal;         // kAdj*
    int nel, n, jchunk;
    PairConsts c;
    double c2a, k_l2, k_dl, k_gl, inv_rs2, inv_rs3;        // see radial_f64
    float c2a_f, k_l2_f, k_dl_f, k_gl_f, inv_rs2_f, inv_rs3_f;
};

template <int KIND>
__device__ __forceinline__ void radial_f64(const AdjArgs &a, const F64Tab &tb, double r2, double &G1, double &G2,
                                           double &dl, double &gl) {
    // no divisions (GB300's FP64 rate): 1/r from rsqrt_nr, the table-driven
    // exponentials, erfc from the Gaussians (pair_math.cuh)
    const double rinv = rsqrt_nr(r2), r = r2 * rinv, rinv2 = rinv * rinv;
    const double al = a.c.alpha;
    const double e = exp_neg_tab(a.c.alpha2 * r2, tb);
    const double w0 = e * ewald_q(al * r, tb) * rinv * rinv2;   // (erfc(ar)/r + 2a/sqrt(pi) e)/r^2
    G1 = w0;
    G2 = (3.0 * w0 + a.c2a * e) * rinv2;
    dl = 0.0;
    gl = 0.0;
    if (KIND == 1) {
        const double irs = a.c.inv_rs_d, y = exp_neg_tab(r * irs, tb);
        G1 -= y * (irs + rinv) * rinv2;
        G2 -= y * (3.0 * irs * rinv2 + 3.0 * rinv2 * rinv + a.inv_rs2 * rinv) * rinv2;
        dl = -y * a.inv_rs2;
        gl = -y * a.inv_rs3 * rinv;
    } else if (KIND == 2) {
        const double g = exp_neg_tab(r2 * a.c.inv_lam2, tb);
        G1 -= g * rinv2 * rinv;
        G2 -= g * (3.0 * rinv2 * rinv + a.k_l2 * rinv) * rinv2;
        dl = -a.k_dl * erfc_tab(r * a.c.inv_lam, g, tb);   // erfc(r/l), exp(-(r/l)^2) = g
        gl = -a.k_gl * g * rinv;
    }
}

template <int KIND>
__device__ __forceinline__ void radial_f32(const AdjArgs &a, float r2, float &G1, float &G2, float &dl, float &gl) {
    const PairConsts &c = a.c;
    const float rinv = rsqrt_approx(r2), r = r2 * rinv, rinv2 = rinv * rinv;
    const float t = rcp_approx(fmaf(c.p_alpha, r, 1.0f));
    const float e = ex2_approx(c.c_exp * r2);
    const float w0 = fmaf(c.c_gauss, e, e * erfc_poly(t) * rinv) * rinv2;
    G1 = w0;
    G2 = fmaf(3.0f, w0, a.c2a_f * e) * rinv2;
    dl = 0.0f;
    gl = 0.0f;
    if (KIND == 1) {
        const float y = ex2_approx(c.c_rs * r);
        G1 -= y * (c.inv_rs + rinv) * rinv2;
        G2 -= y * (3.0f * c.inv_rs * rinv2 + 3.0f * rinv2 * rinv + a.inv_rs2_f * rinv) * rinv2;
        dl = -y * a.inv_rs2_f;
        gl = -y * a.inv_rs3_f * rinv;
    } else if (KIND == 2) {
        const float g = ex2_approx(c.c_lam * r2);
        G1 -= g * rinv2 * rinv;
        G2 -= g * (3.0f * rinv2 * rinv + a.k_l2_f * rinv) * rinv2;
        const float t2 = rcp_approx(fmaf(c.p_lam, r, 1.0f));
        dl = -a.k_dl_f * (g * erfc_poly(t2));
        gl = -a.k_gl_f * g * rinv;
    }
}

template <bool F32, int EIK, bool HVP>
__global__ void __launch_bounds__(kAdjThreads) adj_pair_kernel(const AdjArgs a) {
    using T = typename std::conditional<F32, float, double>::type;
    __shared__ double sw[3][HVP ? kAdjThreads : 1];
    __shared__ int4 sxq[F32 ? kAdjThreads : 1];
    __shared__ double4_32a sxd[F32 ? 1 : kAdjThreads];
    __shared__ double red[32];
    __shared__ F64Tab tab;
    load_f64_tab(tab);     // ordered before first use by the tile loop's barrier
    const int tid = threadIdx.x;
    const int i = blockIdx.x * kAdjThreads + tid;
    const bool vi = i < a.n;
    const int ii = vi ? i : 0;
    const int si = ii < a.nel ? 0 : 1;
    int4 xqi = make_int4(0, 0, 0, 0);
    double4_32a xdi = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    if (F32) xqi = a.xq[ii];
    else xdi = a.xd[ii];
    double wi0 = 0.0, wi1 = 0.0, wi2 = 0.0;
    if (HVP) {
        wi0 = a.w[ii];
        wi1 = a.w[(size_t)a.n + ii];
        wi2 = a.w[2 * (size_t)a.n + ii];
    }
    const int j0 = blockIdx.y * a.jchunk, j1 = min(a.n, j0 + a.jchunk);
    double h0 = 0.0, h1 = 0.0, h2 = 0.0, el = 0.0, fl = 0.0;
    for (int jt = j0; jt < j1; jt += kAdjThreads) {
        __syncthreads();
        const int jj = jt + tid;
        if (jj < j1) {
            if (F32) sxq[tid] = a.xq[jj];
            else sxd[tid] = a.xd[jj];
            if (HVP) {
                sw[0][tid] = a.w[jj];
                sw[1][tid] = a.w[(size_t)a.n + jj];
                sw[2][tid] = a.w[2 * (size_t)a.n + jj];
            }
        }
        __syncthreads();
        if (!vi) continue;
        const int cnt = min(kAdjThreads, j1 - jt);
        T t0 = 0, t1 = 0, t2 = 0, te = 0, tf = 0;
        for (int k = 0; k < cnt; ++k) {
            const int j = jt + k;
            if (j == i) continue;
            const int type = si + (j < a.nel ? 0 : 1);
            T u0, u1, u2;
            if (F32) {
                const int4 xj = sxq[k];
                // wrapping int32 difference = minimum image in 2^-32 box units
                u0 = (T)(float)(int)((unsigned)xqi.x - (unsigned)xj.x) * (T)a.c.sx;
                u1 = (T)(float)(int)((unsigned)xqi.y - (unsigned)xj.y) * (T)a.c.sy;
                u2 = (T)(float)(int)((unsigned)xqi.z - (unsigned)xj.z) * (T)a.c.sz;
            } else {
                const double4_32a xj = sxd[k];
                double d0 = xdi.x - xj.x, d1 = xdi.y - xj.y, d2 = xdi.z - xj.z;
                d0 -= a.c.box[0] * round(d0 / a.c.box[0]);
                d1 -= a.c.box[1] * round(d1 / a.c.box[1]);
                d2 -= a.c.box[2] * round(d2 / a.c.box[2]);
                u0 = (T)d0;
                u1 = (T)d1;
                u2 = (T)d2;
            }
            const T r2 = u0 * u0 + u1 * u1 + u2 * u2;
            if (!(r2 < (F32 ? (T)a.c.rc2f : (T)a.c.rc2))) continue;
            T G1, G2, dl, gl;
            if (F32) {
                float g1, g2, d, g;
                if (type == 1 && EIK == 2 && (float)r2 < a.c.close2) {
                    // close Kelbg pairs: the FP32 terms of G1, G2 cancel to order
                    // r^2/lambda^2 (the force kernels use the series of kelbg_close);
                    // these rare pairs take the FP64 radial functions
                    double h1, h2, hd, hg;
                    radial_f64<2>(a, tab, (double)r2, h1, h2, hd, hg);
                    g1 = (float)h1; g2 = (float)h2; d = (float)hd; g = (float)hg;
                } else if (type == 1 && EIK == 1) radial_f32<1>(a, (float)r2, g1, g2, d, g);
                else if (type == 1 && EIK == 2) radial_f32<2>(a, (float)r2, g1, g2, d, g);
                else radial_f32<0>(a, (float)r2, g1, g2, d, g);
                G1 = g1; G2 = g2; dl = d; gl = g;
            } else {
                double g1, g2, d, g;
                if (type == 1 && EIK == 1) radial_f64<1>(a, tab, (double)r2, g1, g2, d, g);
                else if (type == 1 && EIK == 2) radial_f64<2>(a, tab, (double)r2, g1, g2, d, g);
                else radial_f64<0>(a, tab, (double)r2, g1, g2, d, g);
                G1 = g1; G2 = g2; dl = d; gl = g;
            }
            const T qq = F32 ? (T)(a.c.qqf[type] * (float)kEps) : (T)(a.c.qq[type] * kEps);
            te += qq * dl;
            if (HVP) {
                const T dw0 = (T)(wi0 - sw[0][k]), dw1 = (T)(wi1 - sw[1][k]), dw2 = (T)(wi2 - sw[2][k]);
                const T ud = u0 * dw0 + u1 * dw1 + u2 * dw2;
                const T a1 = -qq * G1, a2 = qq * G2 * ud;
                t0 += a1 * dw0 + a2 * u0;
                t1 += a1 * dw1 + a2 * u1;
                t2 += a1 * dw2 + a2 * u2;
                tf += qq * gl * (u0 * (T)wi0 + u1 * (T)wi1 + u2 * (T)wi2);
            }
        }
        h0 += (double)t0;
        h1 += (double)t1;
        h2 += (double)t2;
        el += (double)te;
        fl += (double)tf;
    }
    if (HVP && vi) {
        atomicAdd(a.hw + i, h0);
        atomicAdd(a.hw + (size_t)a.n + i, h1);
        atomicAdd(a.hw + 2 * (size_t)a.n + i, h2);
    }
    el = block_sum(el, red);
    fl = block_sum(fl, red);
    if (tid == 0) {
        atomicAdd(a.scal + kAdjDEdl, 0.5 * el);
        if (HVP) atomicAdd(a.scal + kAdjDFdl, fl);
    }
}

// ---- Newton-3 form -------------------------------------------------------------
// The same sums over unique pairs (i < j), on the item schedule of the Newton-3
// force kernels (pair_n3.cuh: i-tiles of kAdjN3Tile particles x j-subtiles of
// kN3Sub, every item taken from an atomic counter).  A lane holds one
// i-particle; the j position, w_j and the reaction (H w)_j rotate through the
// warp with shuffles.  Per unique pair with t = qq (-G1 dw + G2 (u.dw) u):
// (H w)_i += t, (H w)_j -= t; dE/dlambda += qq dl; dF/dlambda . w += qq gl (u.dw)
// (the ordered-pair sums counted each of these twice or split them over i, j).
constexpr int kAdjN3Warps = 8;
constexpr int kAdjN3Threads = 32 * kAdjN3Warps;
constexpr int kAdjN3Tile = kAdjN3Threads;     // one i-particle per lane

__device__ __forceinline__ void adj_radial_t(const AdjArgs &a, const F64Tab &tb, int type, int eik, float r2,
                                             float &G1, float &G2, float &dl, float &gl) {
    if (type == 1 && eik == 2 && r2 < a.c.close2) {   // close Kelbg pairs, as in adj_pair_kernel
        double h1, h2, hd, hg;
        radial_f64<2>(a, tb, (double)r2, h1, h2, hd, hg);
        G1 = (float)h1;
        G2 = (float)h2;
        dl = (float)hd;
        gl = (float)hg;
        return;
    }
    if (type == 1 && eik == 1) radial_f32<1>(a, r2, G1, G2, dl, gl);
    else if (type == 1 && eik == 2) radial_f32<2>(a, r2, G1, G2, dl, gl);
    else radial_f32<0>(a, r2, G1, G2, dl, gl);
}

__device__ __forceinline__ void adj_radial_t(const AdjArgs &a, const F64Tab &tb, int type, int eik, double r2,
                                             double &G1, double &G2, double &dl, double &gl) {
    if (type == 1 && eik == 1) radial_f64<1>(a, tb, r2, G1, G2, dl, gl);
    else if (type == 1 && eik == 2) radial_f64<2>(a, tb, r2, G1, G2, dl, gl);
    else radial_f64<0>(a, tb, r2, G1, G2, dl, gl);
}

template <bool F32, int EIK, bool HVP>
__global__ void __launch_bounds__(kAdjN3Threads) adj_n3_kernel(const AdjArgs a, const N3Geom g, long long total,
                                                                 unsigned *counter) {
    using T = typename std::conditional<F32, float, double>::type;
    __shared__ int4 sxq[F32 ? kN3Sub : 1];
    __shared__ longlong4_32a sxl[F32 ? 1 : kN3Sub];
    __shared__ double sw[3][HVP ? kN3Sub : 1];
    __shared__ double sh[HVP ? kN3Sub : 1][3];
    __shared__ double red[32];
    __shared__ long long s_next;
    __shared__ F64Tab tab;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int src = (lane + 1) & 31;
    for (int k = tid; k < (HVP ? kN3Sub : 1) * 3; k += kAdjN3Threads) (&sh[0][0])[k] = 0.0;
    load_f64_tab(tab);     // ordered before first use by the item loop's barrier

    int curI = -1, istart = 0, iend = 0, isp = 0, ifirst = 0, ibase = 0;
    int4 xqi = make_int4(0, 0, 0, 0);
    longlong3 xli = make_longlong3(0, 0, 0);
    T wi[3] = {0, 0, 0};
    double hi[3] = {0.0, 0.0, 0.0};
    double el = 0.0, fl = 0.0;

    auto flush_i = [&]() {
        if (HVP && curI >= 0 && ibase < iend)
            for (int d = 0; d < 3; ++d) atomicAdd(a.hw + (size_t)d * a.n + ibase, hi[d]);
        hi[0] = hi[1] = hi[2] = 0.0;
    };

    while (true) {
        if (tid == 0) s_next = (long long)atomicAdd(counter, 1u);
        __syncthreads();
        const long long it = s_next;
        if (it >= total) break;
        int I, S;
        n3_decode<kAdjN3Tile>(g, it, I, S);
        if (I != curI) {
            flush_i();
            curI = I;
            n3_itile<kAdjN3Tile>(g, I, istart, iend, isp, ifirst);
            ibase = istart + warp * 32 + lane;
            const int ir = ibase < iend ? ibase : istart;
            if (F32) {
                xqi = a.xq[ir];
            } else {
                const longlong4_32a t = a.xl[ir];
                xli = make_longlong3(t.x, t.y, t.z);
            }
            if (HVP)
                for (int d = 0; d < 3; ++d) wi[d] = (T)a.w[(size_t)d * a.n + ir];
        }
        int jstart, cnt, jsp;
        n3_sub(g, S, jstart, cnt, jsp);
        for (int k = tid; k < cnt; k += kAdjN3Threads) {
            if (F32) sxq[k] = a.xq[jstart + k];
            else sxl[k] = a.xl[jstart + k];
            if (HVP)
                for (int d = 0; d < 3; ++d) sw[d][k] = a.w[(size_t)d * a.n + jstart + k];
        }
        __syncthreads();
        const bool masked = (S < ifirst + kAdjN3Tile / kN3Sub && jsp == isp) || cnt < kN3Sub || (iend - istart) < kAdjN3Tile;
        const int type = isp + jsp;
        const T qq = F32 ? (T)(a.c.qqf[type] * (float)kEps) : (T)(a.c.qq[type] * kEps);
        T ti0 = 0, ti1 = 0, ti2 = 0, te = 0, tf = 0;   // per-item partials (FP32 in FP32C mode)
        for (int ch = 0; ch * 32 < cnt; ++ch) {
            const int jl = ch * 32 + lane;
            const bool jv = jl < cnt;
            int4 xqj = make_int4(0, 0, 0, 0);
            long long xj0 = 0, xj1 = 0, xj2 = 0;
            if (jv) {
                if (F32) {
                    xqj = sxq[jl];
                } else {
                    xj0 = sxl[jl].x;
                    xj1 = sxl[jl].y;
                    xj2 = sxl[jl].z;
                }
            }
            T wj0 = HVP && jv ? (T)sw[0][jl] : (T)0, wj1 = HVP && jv ? (T)sw[1][jl] : (T)0,
              wj2 = HVP && jv ? (T)sw[2][jl] : (T)0;
            T hj0 = 0, hj1 = 0, hj2 = 0;
#pragma unroll 1
            for (int s = 0; s < 32; ++s) {
                const int jo = ch * 32 + ((lane + s) & 31);
                T u0, u1, u2;
                if (F32) {
                    u0 = (T)(float)(int)((unsigned)xqi.x - (unsigned)xqj.x) * (T)a.c.sx;
                    u1 = (T)(float)(int)((unsigned)xqi.y - (unsigned)xqj.y) * (T)a.c.sy;
                    u2 = (T)(float)(int)((unsigned)xqi.z - (unsigned)xqj.z) * (T)a.c.sz;
                } else {   // wrapped 64-bit fixed-point difference = minimum image
                    u0 = (T)((double)(long long)((unsigned long long)xli.x - (unsigned long long)xj0) * a.c.sl[0]);
                    u1 = (T)((double)(long long)((unsigned long long)xli.y - (unsigned long long)xj1) * a.c.sl[1]);
                    u2 = (T)((double)(long long)((unsigned long long)xli.z - (unsigned long long)xj2) * a.c.sl[2]);
                }
                const T r2 = u0 * u0 + u1 * u1 + u2 * u2;
                bool ok = r2 < (F32 ? (T)a.c.rc2f : (T)a.c.rc2) && r2 > (T)0;
                if (masked) ok = ok && ibase < iend && jo < cnt && ibase < jstart + jo;
                if (ok) {
                    T G1, G2, dl, gl;
                    adj_radial_t(a, tab, type, EIK, r2, G1, G2, dl, gl);
                    te += qq * dl;
                    if (HVP) {
                        const T dw0 = wi[0] - wj0, dw1 = wi[1] - wj1, dw2 = wi[2] - wj2;
                        const T ud = u0 * dw0 + u1 * dw1 + u2 * dw2;
                        const T a1 = -qq * G1, a2 = qq * G2 * ud;
                        const T t0 = a1 * dw0 + a2 * u0, t1 = a1 * dw1 + a2 * u1, t2 = a1 * dw2 + a2 * u2;
                        ti0 += t0;
                        ti1 += t1;
                        ti2 += t2;
                        hj0 -= t0;
                        hj1 -= t1;
                        hj2 -= t2;
                        tf += qq * gl * ud;
                    }
                }
                // rotate j (position, w and reaction) to the next lane
                if (F32) {
                    xqj.x = __shfl_sync(0xffffffffu, xqj.x, src);
                    xqj.y = __shfl_sync(0xffffffffu, xqj.y, src);
                    xqj.z = __shfl_sync(0xffffffffu, xqj.z, src);
                } else {
                    xj0 = __shfl_sync(0xffffffffu, xj0, src);
                    xj1 = __shfl_sync(0xffffffffu, xj1, src);
                    xj2 = __shfl_sync(0xffffffffu, xj2, src);
                }
                if (HVP) {
                    wj0 = __shfl_sync(0xffffffffu, wj0, src);
                    wj1 = __shfl_sync(0xffffffffu, wj1, src);
                    wj2 = __shfl_sync(0xffffffffu, wj2, src);
                    hj0 = __shfl_sync(0xffffffffu, hj0, src);
                    hj1 = __shfl_sync(0xffffffffu, hj1, src);
                    hj2 = __shfl_sync(0xffffffffu, hj2, src);
                }
            }
            if (HVP && jv) {
                atomicAdd(&sh[jl][0], (double)hj0);
                atomicAdd(&sh[jl][1], (double)hj1);
                atomicAdd(&sh[jl][2], (double)hj2);
            }
        }
        hi[0] += (double)ti0;
        hi[1] += (double)ti1;
        hi[2] += (double)ti2;
        el += (double)te;
        fl += (double)tf;
        __syncthreads();                   // reactions of this subtile complete; tiles free
        if (HVP && tid < cnt)
            for (int d = 0; d < 3; ++d) {
                atomicAdd(a.hw + (size_t)d * a.n + jstart + tid, sh[tid][d]);
                sh[tid][d] = 0.0;
            }
    }
    flush_i();
    el = block_sum(el, red);
    fl = block_sum(fl, red);
    if (tid == 0) {
        atomicAdd(a.scal + kAdjDEdl, el);
        if (HVP) atomicAdd(a.scal + kAdjDFdl, fl);
    }
}

// ---- host-layout transposes ---------------------------------------------------
__global__ void aos_to_soa_kernel(const double *__restrict__ in, double *__restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int d = 0; d < 3; ++d) out[(size_t)d * n + i] = in[3 * (size_t)i + d];
}

__global__ void soa_to_aos_kernel(const double *__restrict__ in, double *__restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int d = 0; d < 3; ++d) out[3 * (size_t)i + d] = in[(size_t)d * n + i];
}

// ---- reverse-mode step kernels ------------------------------------------------
struct RevArgs {
    const double *v;      // v_k [3][n]
    double *xb, *vb, *fb, *g, *part;
    const double *hw;
    int nel, n;
    double a0, a1;        // dt/(2 m) per species
    double cj0, cj1;      // 2 m/(3 N K) per species
    double dt;
};

// step k >= 1: vb += 2 m v_k/(3NK), g = fb + a vb (the two uses of F_k);
// k = 0 (initial_only): g = fb.  Per-block sums of g for the mean.
__global__ void rev_seed_kernel(const RevArgs r, bool initial_only) {
    __shared__ double red[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s[3] = {0.0, 0.0, 0.0};
    if (i < r.n) {
        const bool el = i < r.nel;
        const double a = el ? r.a0 : r.a1, cj = el ? r.cj0 : r.cj1;
        for (int d = 0; d < 3; ++d) {
            const size_t k = (size_t)d * r.n + i;
            if (initial_only) {
                s[d] = r.fb[k];
            } else {
                const double vb = r.vb[k] + cj * r.v[k];
                r.vb[k] = vb;
                s[d] = r.fb[k] + a * vb;
            }
            r.g[k] = s[d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        const double t = block_sum(s[d], red);
        if (threadIdx.x == 0) r.part[3 * blockIdx.x + d] = t;
    }
}

// g -= mean(g) (REMOVE_RIGIDMTN applied to the adjoint, force.f90:986-1004);
// every block sums the per-block partials in the same order.
__global__ void rev_center_kernel(const RevArgs r, int nparts) {
    __shared__ double mean[3];
    __shared__ double red[32];
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nparts; b += blockDim.x) s += r.part[3 * b + d];
        s = block_sum(s, red);
        if (threadIdx.x == 0) mean[d] = s / (double)r.n;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r.n) return;
    for (int d = 0; d < 3; ++d) r.g[(size_t)d * r.n + i] -= mean[d];
}

// xb -= H P g;  vb += dt xb;  fb = a vb
__global__ void rev_update_kernel(const RevArgs r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r.n) return;
    const double a = i < r.nel ? r.a0 : r.a1;
    for (int d = 0; d < 3; ++d) {
        const size_t k = (size_t)d * r.n + i;
        const double xb = r.xb[k] - r.hw[k];
        const double vb = r.vb[k] + r.dt * xb;
        r.xb[k] = xb;
        r.vb[k] = vb;
        r.fb[k] = a * vb;
    }
}

// J accumulator: scal[kAdjJ] += mv2el + mv2ion of the step just taken
__global__ void rev_accum_kernel(const double *__restrict__ scal, double *__restrict__ adj) {
    if (threadIdx.x == 0 && blockIdx.x == 0) adj[kAdjJ] += scal[kScalMv2e] + scal[kScalMv2i];
}

// ---- host side -------------------------------------------------------------------
constexpr int kRevThreads = 256;
static int rev_blocks(int n) { return (n + kRevThreads - 1) / kRevThreads; }

void adjoint_free(tcp_ctx *c) {
    double **bufs[] = {&c->adj_w, &c->adj_hw, &c->adj_xb, &c->adj_vb, &c->adj_fb, &c->adj_save,
                       &c->adj_io, &c->adj_scal, &c->adj_part, &c->adj_ck, &c->adj_seg};
    for (double **b : bufs) {
        cudaFree(*b);
        *b = nullptr;
    }
    c->adj_ck_cap = 0;
    c->adj_seg_cap = 0;
}

static int adj_alloc(tcp_ctx *c) {
    if (c->adj_w) return TCP_OK;
    const size_t v3 = sizeof(double) * 3 * (size_t)c->n;
    if (cudaMalloc(&c->adj_w, v3) != cudaSuccess || cudaMalloc(&c->adj_hw, v3) != cudaSuccess ||
        cudaMalloc(&c->adj_xb, v3) != cudaSuccess || cudaMalloc(&c->adj_vb, v3) != cudaSuccess ||
        cudaMalloc(&c->adj_fb, v3) != cudaSuccess || cudaMalloc(&c->adj_save, 3 * v3) != cudaSuccess ||
        cudaMalloc(&c->adj_io, v3) != cudaSuccess ||
        cudaMalloc(&c->adj_scal, sizeof(double) * kAdjCount) != cudaSuccess ||
        cudaMalloc(&c->adj_part, sizeof(double) * 3 * (size_t)rev_blocks(c->n)) != cudaSuccess) {
        adjoint_free(c);
        return set_error(TCP_ERR_NOMEM, "derivative buffers: device allocation failed");
    }
    return TCP_OK;
}

static AdjArgs adj_args(tcp_ctx *c, const double *w, double *hw) {
    AdjArgs a;
    a.xq = c->xq;
    a.xd = c->xd;
    a.xl = c->xl;
    a.w = w;
    a.hw = hw;
    a.scal = c->adj_scal;
    a.nel = c->nel;
    a.n = c->n;
    a.c = c->pc;
    const double al = c->alpha, l = c->pc.lambda, rs = c->pc.rs;
    a.c2a = 2.0 * al * al * (2.0 * al / kSqrtPi);
    a.k_l2 = 2.0 / (l * l);
    a.k_dl = kSqrtPi / (l * l);
    a.k_gl = 2.0 / (l * l * l);
    a.inv_rs2 = 1.0 / (rs * rs);
    a.inv_rs3 = 1.0 / (rs * rs * rs);
    a.c2a_f = (float)a.c2a;
    a.k_l2_f = (float)a.k_l2;
    a.k_dl_f = (float)a.k_dl;
    a.k_gl_f = (float)a.k_gl;
    a.inv_rs2_f = (float)a.inv_rs2;
    a.inv_rs3_f = (float)a.inv_rs3;
    // j-split so that the grid covers about four CTAs per SM
    const int bx = (c->n + kAdjThreads - 1) / kAdjThreads;
    int ny = std::max(1, std::min(bx, (4 * c->num_sms + bx - 1) / bx));
    const int chunk = ((c->n + ny - 1) / ny + kAdjThreads - 1) / kAdjThreads * kAdjThreads;
    a.jchunk = chunk;
    return a;
}

template <bool F32, int EIK, bool HVP>
static int launch_adj_n3_t(tcp_ctx *c, const AdjArgs &a) {
    long long total = 0;
    const N3Geom g = n3_geometry(0, c->nel, c->nion, kAdjN3Tile, 0, &total);
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, adj_n3_kernel<F32, EIK, HVP>, kAdjN3Threads, 0);
    const int grid = (int)std::max<long long>(1, std::min<long long>((long long)c->num_sms * std::max(bps, 1), total));
    TCP_CUDA(cudaMemsetAsync(c->counter, 0, sizeof(unsigned), c->stream));
    adj_n3_kernel<F32, EIK, HVP><<<grid, kAdjN3Threads, 0, c->stream>>>(a, g, total, c->counter);
    return TCP_OK;
}

// Real-space part: hw += H_real w (when w), scalars into adj_scal.  The
// Newton-3 form unless TCP_FLAG_DETERMINISTIC asks for the ordered-pair sums
// (which add their rows in a fixed pattern).
static int launch_adj_pair(tcp_ctx *c, const double *w, double *hw) {
    AdjArgs a = adj_args(c, w, hw);
    if (!(c->flags & TCP_FLAG_DETERMINISTIC)) {
        const bool f32 = c->p.precision == TCP_PREC_FP32C;
        const int eik = c->p.ei_model == TCP_EI_DEUTSCH ? 1 : (c->p.ei_model == TCP_EI_KELBG ? 2 : 0);
        int rc;
#define ADJ_N3(F, E, H) rc = launch_adj_n3_t<F, E, H>(c, a)
        if (w) {
            if (f32) {
                if (eik == 1) ADJ_N3(true, 1, true);
                else if (eik == 2) ADJ_N3(true, 2, true);
                else ADJ_N3(true, 0, true);
            } else {
                if (eik == 1) ADJ_N3(false, 1, true);
                else if (eik == 2) ADJ_N3(false, 2, true);
                else ADJ_N3(false, 0, true);
            }
        } else {
            if (f32) {
                if (eik == 1) ADJ_N3(true, 1, false);
                else if (eik == 2) ADJ_N3(true, 2, false);
                else ADJ_N3(true, 0, false);
            } else {
                if (eik == 1) ADJ_N3(false, 1, false);
                else if (eik == 2) ADJ_N3(false, 2, false);
                else ADJ_N3(false, 0, false);
            }
        }
#undef ADJ_N3
        if (rc) return rc;
        c->launches++;
        TCP_CUDA(cudaGetLastError());
        return TCP_OK;
    }
    const int bx = (c->n + kAdjThreads - 1) / kAdjThreads;
    const int by = (c->n + a.jchunk - 1) / a.jchunk;
    const dim3 grid(bx, by);
    const bool f32 = c->p.precision == TCP_PREC_FP32C;
    const int eik = c->p.ei_model == TCP_EI_DEUTSCH ? 1 : (c->p.ei_model == TCP_EI_KELBG ? 2 : 0);
#define ADJ_LAUNCH(F, E, H) adj_pair_kernel<F, E, H><<<grid, kAdjThreads, 0, c->stream>>>(a)
    if (w) {
        if (f32) {
            if (eik == 1) ADJ_LAUNCH(true, 1, true);
            else if (eik == 2) ADJ_LAUNCH(true, 2, true);
            else ADJ_LAUNCH(true, 0, true);
        } else {
            if (eik == 1) ADJ_LAUNCH(false, 1, true);
            else if (eik == 2) ADJ_LAUNCH(false, 2, true);
            else ADJ_LAUNCH(false, 0, true);
        }
    } else {
        if (f32) {
            if (eik == 1) ADJ_LAUNCH(true, 1, false);
            else if (eik == 2) ADJ_LAUNCH(true, 2, false);
            else ADJ_LAUNCH(true, 0, false);
        } else {
            if (eik == 1) ADJ_LAUNCH(false, 1, false);
            else if (eik == 2) ADJ_LAUNCH(false, 2, false);
            else ADJ_LAUNCH(false, 0, false);
        }
    }
#undef ADJ_LAUNCH
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

// hw = H w at the current positions (device SoA), scal[kAdjDFdl] += dF/dl . w
static int hvp_device(tcp_ctx *c, const double *w, double *hw) {
    int rc;
    TCP_CUDA(cudaMemsetAsync(hw, 0, sizeof(double) * 3 * (size_t)c->n, c->stream));
    if ((rc = launch_adj_pair(c, w, hw))) return rc;
    if (c->p.reciprocal == TCP_RECIP_SPME) return launch_spme_hvp(c, w, hw);
    if (c->p.reciprocal == TCP_RECIP_EWALD) return launch_ewald_hvp(c, w, hw);
    return TCP_OK;
}

static int read_adj(tcp_ctx *c, double *out, int count) {
    TCP_CUDA(cudaMemcpyAsync(out, c->adj_scal, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

static RevArgs rev_args(tcp_ctx *c, const double *v, double dt, int K) {
    RevArgs r;
    r.v = v;
    r.xb = c->adj_xb;
    r.vb = c->adj_vb;
    r.fb = c->adj_fb;
    r.g = c->adj_w;
    r.part = c->adj_part;
    r.hw = c->adj_hw;
    r.nel = c->nel;
    r.n = c->n;
    r.a0 = 0.5 * dt / c->p.xm[0];
    r.a1 = 0.5 * dt / c->p.xm[1];
    r.cj0 = 2.0 * c->p.xm[0] / (3.0 * c->n * (double)K);
    r.cj1 = 2.0 * c->p.xm[1] / (3.0 * c->n * (double)K);
    r.dt = dt;
    return r;
}

// g (adj_w) = P (fb + a vb) for a step k >= 1, P fb for k = 0
static int rev_seed(tcp_ctx *c, const RevArgs &r, bool initial_only) {
    const int nb = rev_blocks(c->n);
    rev_seed_kernel<<<nb, kRevThreads, 0, c->stream>>>(r, initial_only);
    rev_center_kernel<<<nb, kRevThreads, 0, c->stream>>>(r, nb);
    c->launches += 2;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

static int copy_state(tcp_ctx *c, double *dst_x, double *dst_v, const double *src_x, const double *src_v) {
    const size_t b = sizeof(double) * 3 * (size_t)c->n;
    if (dst_x) TCP_CUDA(cudaMemcpyAsync(dst_x, src_x, b, cudaMemcpyDeviceToDevice, c->stream));
    if (dst_v) TCP_CUDA(cudaMemcpyAsync(dst_v, src_v, b, cudaMemcpyDeviceToDevice, c->stream));
    return TCP_OK;
}

}  // namespace tcp

using namespace tcp;

#define TCP_ADJ_READY(c)                                                                           \
    do {                                                                                           \
        if (!(c)) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");                             \
        if (!(c)->ewald_ready) return set_error(TCP_ERR_STATE, "tcp_ewald_self must be called first"); \
        cudaSetDevice((c)->device);                                                                \
        int _rc = adj_alloc(c);                                                                    \
        if (_rc) return _rc;                                                                       \
    } while (0)

extern "C" {

int tcp_adjoint_energy(tcp_ctx *c, double *E, double *dE_dlambda, double *dE_dscale) {
    TCP_TRACE("tcp_adjoint_energy");
    TCP_ADJ_READY(c);
    int rc;
    const size_t b = sizeof(double) * 3 * (size_t)c->n;
    // the stored forces are state (Finit's f belongs to x - dt v): keep them
    TCP_CUDA(cudaMemcpyAsync(c->adj_save, c->f, b, cudaMemcpyDeviceToDevice, c->stream));
    TCP_CUDA(cudaMemcpyAsync(c->adj_save + 3 * (size_t)c->n, c->frec, b, cudaMemcpyDeviceToDevice, c->stream));
    const unsigned flags = c->flags;
    c->flags = (flags | TCP_FLAG_ENERGY) & ~(unsigned)TCP_FLAG_RDF;
    if ((rc = autotune_pair(c))) {
        c->flags = flags;
        return rc;
    }
    rc = force_eval(c, true);
    c->flags = flags;
    if (rc) return rc;
    TCP_CUDA(cudaMemcpyAsync(c->f, c->adj_save, b, cudaMemcpyDeviceToDevice, c->stream));
    TCP_CUDA(cudaMemcpyAsync(c->frec, c->adj_save + 3 * (size_t)c->n, b, cudaMemcpyDeviceToDevice, c->stream));
    TCP_CUDA(cudaMemsetAsync(c->adj_scal, 0, sizeof(double) * kAdjCount, c->stream));
    if ((rc = launch_adj_pair(c, nullptr, nullptr))) return rc;
    if ((rc = md_finish(c))) return rc;
    double s[kAdjCount];
    if ((rc = read_adj(c, s, kAdjCount))) return rc;
    const double e = c->last.Epot + c->last.Um;
    if (E) *E = e;
    if (dE_dlambda) *dE_dlambda = c->p.ei_model == TCP_EI_COULOMB ? 0.0 : s[kAdjDEdl];
    // every term (pair, mesh, self) is quadratic in the charge scale s
    if (dE_dscale) *dE_dscale = 2.0 * e / c->p.charge_scale;
    return TCP_OK;
}

int tcp_hvp(tcp_ctx *c, const double *w, double *hw, double *dF_dlambda_w) {
    TCP_TRACE("tcp_hvp");
    TCP_ADJ_READY(c);
    if (!w || !hw) return set_error(TCP_ERR_BAD_PARAM, "w and hw must not be NULL");
    int rc;
    const size_t b = sizeof(double) * 3 * (size_t)c->n;
    const int nb = rev_blocks(c->n);
    TCP_CUDA(cudaMemcpyAsync(c->adj_io, w, b, cudaMemcpyHostToDevice, c->stream));
    aos_to_soa_kernel<<<nb, kRevThreads, 0, c->stream>>>(c->adj_io, c->adj_w, c->n);
    TCP_CUDA(cudaMemsetAsync(c->adj_scal, 0, sizeof(double) * kAdjCount, c->stream));
    if ((rc = hvp_device(c, c->adj_w, c->adj_hw))) return rc;
    soa_to_aos_kernel<<<nb, kRevThreads, 0, c->stream>>>(c->adj_hw, c->adj_io, c->n);
    c->launches += 2;
    TCP_CUDA(cudaGetLastError());
    TCP_CUDA(cudaMemcpyAsync(hw, c->adj_io, b, cudaMemcpyDeviceToHost, c->stream));
    double s[kAdjCount];
    if ((rc = read_adj(c, s, kAdjCount))) return rc;
    if (dF_dlambda_w) *dF_dlambda_w = c->p.ei_model == TCP_EI_COULOMB ? 0.0 : s[kAdjDFdl];
    return TCP_OK;
}

int tcp_reverse_md(tcp_ctx *c, double dt, int nsteps, int every, double *J, double *dJ_dlambda) {
    TCP_TRACE("tcp_reverse_md");
    TCP_ADJ_READY(c);
    if (nsteps <= 0 || every <= 0) return set_error(TCP_ERR_BAD_PARAM, "nsteps and every must be positive");
    if (c->p.thermo != TCP_THERMO_NOTEMP)
        return set_error(TCP_ERR_BAD_PARAM, "reverse mode covers the NOTEMP step only");
    int rc;
    const int K = nsteps, M = std::min(every, nsteps);
    const int nck = (K + M - 1) / M;
    const size_t n3 = 3 * (size_t)c->n, b = sizeof(double) * n3;
    if (c->adj_ck_cap < nck) {
        cudaFree(c->adj_ck);
        c->adj_ck = nullptr;
        c->adj_ck_cap = 0;
        TCP_CUDA(cudaMalloc(&c->adj_ck, 2 * b * (size_t)nck));
        c->adj_ck_cap = nck;
    }
    if (c->adj_seg_cap < M + 1) {
        cudaFree(c->adj_seg);
        c->adj_seg = nullptr;
        c->adj_seg_cap = 0;
        TCP_CUDA(cudaMalloc(&c->adj_seg, 2 * b * (size_t)(M + 1)));
        c->adj_seg_cap = M + 1;
    }
    if ((rc = autotune_pair(c))) return rc;
    const long long step0 = c->step_index;
    TCP_CUDA(cudaMemsetAsync(c->adj_scal, 0, sizeof(double) * kAdjCount, c->stream));
    // forward: f_0 = F(x_0; lambda), then K steps with checkpoints
    if ((rc = force_eval(c, true))) return rc;
    for (int k = 0; k < K; ++k) {
        if (k % M == 0 && (rc = copy_state(c, c->adj_ck + 2 * n3 * (k / M), c->adj_ck + 2 * n3 * (k / M) + n3, c->x, c->v)))
            return rc;
        if ((rc = md_advance(c, dt, 1))) return rc;
        rev_accum_kernel<<<1, 32, 0, c->stream>>>(c->scal, c->adj_scal);
        c->launches++;
    }
    if ((rc = md_finish(c))) return rc;           // energies of step K, as tcp_md_steps
    const tcp_energies last = c->last;
    // final state, restored after the sweep
    if ((rc = copy_state(c, c->adj_save, c->adj_save + n3, c->x, c->v))) return rc;
    TCP_CUDA(cudaMemcpyAsync(c->adj_save + 2 * n3, c->f, b, cudaMemcpyDeviceToDevice, c->stream));
    // scalars and histograms as after step K (the recomputation steps repeat them)
    double scal_save[kScalCount];
    std::vector<unsigned long long> hist(5 * kNbin);
    TCP_CUDA(cudaMemcpyAsync(scal_save, c->scal, sizeof(scal_save), cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaMemcpyAsync(hist.data(), c->rdf, sizeof(unsigned long long) * 3 * kNbin, cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaMemcpyAsync(hist.data() + 3 * kNbin, c->vdf, sizeof(unsigned long long) * 2 * kNbin,
                             cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    // reverse sweep
    TCP_CUDA(cudaMemsetAsync(c->adj_xb, 0, b, c->stream));
    TCP_CUDA(cudaMemsetAsync(c->adj_vb, 0, b, c->stream));
    TCP_CUDA(cudaMemsetAsync(c->adj_fb, 0, b, c->stream));
    for (int s = nck - 1; s >= 0; --s) {
        const int k0 = s * M, k1 = std::min(k0 + M, K);
        if ((rc = copy_state(c, c->x, c->v, c->adj_ck + 2 * n3 * s, c->adj_ck + 2 * n3 * s + n3))) return rc;
        if ((rc = launch_refresh_positions(c))) return rc;
        if ((rc = force_eval(c, true))) return rc;
        for (int k = k0 + 1; k <= k1; ++k) {
            if ((rc = md_advance(c, dt, 1))) return rc;
            if ((rc = copy_state(c, c->adj_seg + 2 * n3 * (k - k0), c->adj_seg + 2 * n3 * (k - k0) + n3, c->x, c->v)))
                return rc;
        }
        for (int k = k1; k > k0; --k) {
            const double *xk = c->adj_seg + 2 * n3 * (k - k0), *vk = xk + n3;
            if ((rc = copy_state(c, c->x, nullptr, xk, nullptr))) return rc;
            if ((rc = launch_refresh_positions(c))) return rc;
            const RevArgs r = rev_args(c, vk, dt, K);
            if ((rc = rev_seed(c, r, false))) return rc;
            if ((rc = hvp_device(c, c->adj_w, c->adj_hw))) return rc;   // scal[kAdjDFdl] accumulates dJ/dlambda
            rev_update_kernel<<<rev_blocks(c->n), kRevThreads, 0, c->stream>>>(r);
            c->launches++;
            TCP_CUDA(cudaGetLastError());
        }
    }
    // f_0 = F(x_0; lambda): the lambda term only
    if ((rc = copy_state(c, c->x, nullptr, c->adj_ck, nullptr))) return rc;
    if ((rc = launch_refresh_positions(c))) return rc;
    {
        const RevArgs r = rev_args(c, c->v, dt, K);
        if ((rc = rev_seed(c, r, true))) return rc;
        if ((rc = launch_adj_pair(c, c->adj_w, c->adj_hw))) return rc;
    }
    double sres[kAdjCount];
    if ((rc = read_adj(c, sres, kAdjCount))) return rc;
    // restore the state after step K
    if ((rc = copy_state(c, c->x, c->v, c->adj_save, c->adj_save + n3))) return rc;
    TCP_CUDA(cudaMemcpyAsync(c->f, c->adj_save + 2 * n3, b, cudaMemcpyDeviceToDevice, c->stream));
    TCP_CUDA(cudaMemcpyAsync(c->scal, scal_save, sizeof(scal_save), cudaMemcpyHostToDevice, c->stream));
    TCP_CUDA(cudaMemcpyAsync(c->rdf, hist.data(), sizeof(unsigned long long) * 3 * kNbin, cudaMemcpyHostToDevice, c->stream));
    TCP_CUDA(cudaMemcpyAsync(c->vdf, hist.data() + 3 * kNbin, sizeof(unsigned long long) * 2 * kNbin,
                             cudaMemcpyHostToDevice, c->stream));
    if ((rc = launch_refresh_positions(c))) return rc;
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    c->step_index = step0 + K;
    c->last = last;
    if (J) *J = sres[kAdjJ] / (3.0 * c->n * (double)K);
    if (dJ_dlambda) *dJ_dlambda = c->p.ei_model == TCP_EI_COULOMB ? 0.0 : sres[kAdjDFdl];
    return TCP_OK;
}

}  // extern "C"

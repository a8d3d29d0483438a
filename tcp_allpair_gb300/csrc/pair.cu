// pair.cu -- the all-pair Ewald real-space sum (Force_direct_self /
// Force_direct_ext / Force_direct_sum of force.f90:52-372 for the whole
// system on one GPU).
//
// Layout.  Particles are species-ordered (electrons, then ions).  A CTA owns
// a block of i-particles of one species and walks a range of j-tiles; each
// j-tile holds particles of one species, so the pair type (e-e, e-i, i-i)
// and the charge product are uniform per (CTA, tile).  j-tiles are copied
// into shared memory by the bulk-copy engine (cp.async.bulk + mbarrier,
// kStages-deep ring), released by a CTA barrier per tile.  Every ordered
// pair (i, j) is evaluated (no Newton-3 reactions, so no atomics); TPP
// threads share one i-particle and split the tile, and are reduced with
// warp shuffles at the end.  The j-range of the system is split over
// gridDim.y CTAs; their per-particle partial forces go to fpart[split][3][n]
// and are summed in a fixed order by force_finalize (deterministic).
//
// FP32C kernel: positions are 32-bit fixed point (2^32 units per box
// length), so the int32 difference is the minimum image (the DNINT of
// force.f90:92) exactly and converts to FP32 with relative error 6e-8.
// rsqrt / reciprocal / exp2 run on the SFU; erfc(x) = exp(-x^2) t Q(t)
// shares its exponential with the Gaussian force term (fit_erfc.py).  Each
// thread sums a tile's pair forces in FP32 (<= kTjF/kTppF terms) and folds the
// tile partial into a (hi, lo) TwoSum accumulator; the final value is
// hi + lo in FP64.
//
// FP64 kernel: the reference's expressions (force.f90:99-110, 130-144,
// 163-175) in double precision with CUDA's erf/erfc/exp/sqrt.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>

#include "device_util.cuh"
#include "pair_math.cuh"
#include "tcp_internal.h"

namespace tcp {

constexpr int kPairThreads = 256;
constexpr int kTppF = 4;      // threads per i-particle (FP32)
constexpr int kTjF = 512;     // particles per j-tile (16 B each)
constexpr int kStagesF = 3;
constexpr int kTppD = 2;      // FP64
constexpr int kTjD = 256;     // 32 B each
constexpr int kStagesD = 3;

struct PairArgs {
    const int4 *xq;
    const double4_32a *xd;
    int nel, n;
    int bi;                 // i-particles per CTA
    int nblk_e, nblk;       // i-blocks (electron blocks first)
    int tj;                 // particles per j-tile
    int ntile_e, ntile;     // j-tiles (electron tiles first)
    int tiles_per_split;
    double *fpart;          // [gridDim.y][3][n]
    double *upart;          // [gridDim.y * gridDim.x]
    unsigned long long *rdf;
    const RdfEdges *rdf_edges;   // exact bin edges of the FP32C RDF
    unsigned *status;
    PairConsts c;
};

__device__ __forceinline__ void tile_range(const PairArgs &a, int t, int &j0, int &cnt, int &sj) {
    if (t < a.ntile_e) {
        sj = 0;
        j0 = t * a.tj;
        cnt = min(a.tj, a.nel - j0);
    } else {
        sj = 1;
        j0 = a.nel + (t - a.ntile_e) * a.tj;
        cnt = min(a.tj, a.n - j0);
    }
}

// One j-tile for one i-particle (FP32).  KIND: 0 Coulomb erfc (e-e, i-i and
// TCP_EI_COULOMB), 1 Deutsch e-i, 2 Kelbg e-i.  Accumulates sum_j w dx (the
// force divided by eps q_i q_j) and sum_j u/r (energy / q_i q_j).
// FULL: the tile holds kTjF particles (no tail test).  DIAG: the tile may
// contain the i-particle itself (r^2 > 0 test).  CUBIC: all box lengths are
// equal, so the fixed-point difference is used unscaled (lengths in units of
// L/2^32) and the scale is folded into the constants and the per-tile factor
// applied when the tile partial is folded.
// RDF (+1 per ordered pair inside rc): the FP32 bin, or the exact one of the
// fixed-point separation near a bin edge or rc (rdf_exact_bin); vi is false
// for the padding lanes of a partial i-block, which count nothing.
template <int KIND, bool ENERGY, bool RDF, int TPP, bool FULL, bool DIAG, bool CUBIC>
__device__ __forceinline__ void tile_f32(const int4 *__restrict__ tj, int cnt, int sub, int4 xi,
                                         const PairConsts &c, float &px, float &py, float &pz,
                                         float &pe, unsigned *hist, float inv_dx, bool vi = true,
                                         const RdfEdges *E = nullptr, int pt = 0) {
    const int cnt_up = FULL ? kTjF : (cnt + TPP - 1) / TPP * TPP;   // uniform trip count per warp
    // constants in the units of this path
    const float rc2 = CUBIC ? c.u_rc2 : c.rc2f;
    const float p_alpha = CUBIC ? c.u_p_alpha : c.p_alpha;
    const float c_exp = CUBIC ? c.u_c_exp : c.c_exp;
    const float c_gauss = CUBIC ? c.u_c_gauss : c.c_gauss;
    const float c_rs = CUBIC ? c.u_c_rs : c.c_rs;
    const float inv_rs = CUBIC ? c.u_inv_rs : c.inv_rs;
    const float c_lam = CUBIC ? c.u_c_lam : c.c_lam;
    const float p_lam = CUBIC ? c.u_p_lam : c.p_lam;
    const float sqrtpi_lam = CUBIC ? c.u_sqrtpi_lam : c.sqrtpi_lam;
    const float rshort2 = CUBIC ? c.u_rshort2 : c.rshort2;
    const float close2 = CUBIC ? c.u_close2 : c.close2;
    const float inv_lam2 = CUBIC ? c.u_inv_lam2 : c.inv_lam2f;
    const float alpha_ = CUBIC ? c.u_alpha : c.alphaf;
#pragma unroll 8
    for (int jj = sub; jj < cnt_up; jj += TPP) {
        const int4 xj = tj[jj];
        float dx = (float)(xi.x - xj.x);
        float dy = (float)(xi.y - xj.y);
        float dz = (float)(xi.z - xj.z);
        if (!CUBIC) {
            dx *= c.sx;
            dy *= c.sy;
            dz *= c.sz;
        }
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        bool ok = r2 < rc2;
        if (DIAG) ok = ok && (r2 > 0.0f);
        if (!FULL) ok = ok && (jj < cnt);
        // the mask is applied once, to 1/r (er, energy and weight carry it);
        // DIAG / partial tiles may hold the i-particle or padding (r2 = 0)
        const float r2s = (DIAG || !FULL) ? (ok ? r2 : 1.0f) : r2;
        const float rinv = rsqrt_approx(r2s);
        const float rinv_m = ok ? rinv : 0.0f;
        const float r = r2s * rinv;
        const float t = rcp_approx(fmaf(p_alpha, r, 1.0f));
        const float e = ex2_approx(c_exp * r2s);
        const float er = (e * erfc_poly(t)) * rinv_m;   // erfc(ar)/r, shared by energy and force
        float s = fmaf(c_gauss, e, er);                  // (erfc(ar) + 2ar/sqrt(pi) exp(-a^2r^2)) / r
        float u = er;
        if (KIND == 1) {                                 // Deutsch, force.f90:136-139
            const float y = ex2_approx(c_rs * r);        // exp(-r/rs)
            s = fmaf(-y, rinv + inv_rs, s);
            if (ENERGY) u = fmaf(-y, rinv_m, u);
        }
        if (KIND == 2) {                                 // Kelbg
            const bool near = ok && (r2s < rshort2);
            if (__any_sync(0xffffffffu, near)) {
                const float g = near ? ex2_approx(c_lam * r2s) : 0.0f;   // exp(-r^2/lambda^2)
                s = fmaf(-g, rinv, s);
                float erfc_rl = 0.0f;
                if (ENERGY) {
                    const float t2 = rcp_approx(fmaf(p_lam, r, 1.0f));
                    erfc_rl = g * erfc_poly(t2);                 // erfc(r/lambda)
                    u += fmaf(sqrtpi_lam, erfc_rl, -g * rinv);
                }
                const bool close = near && (r2s < close2);
                if (__any_sync(0xffffffffu, close) && close) {
                    float nf, ne;
                    kelbg_close(r2s * inv_lam2, r * alpha_, nf, ne);
                    s = nf * rinv;
                    if (ENERGY) u = fmaf(sqrtpi_lam, erfc_rl, ne * rinv);
                }
            }
        }
        const float w = s * (rinv_m * rinv_m);
        px = fmaf(w, dx, px);
        py = fmaf(w, dy, py);
        pz = fmaf(w, dz, pz);
        if (ENERGY) pe += u;
        if (RDF) {
            const bool valid = vi && (!DIAG || r2 > 0.0f) && (FULL || jj < cnt);
            const float tb = r * inv_dx;
            int bin = (int)tb;
            bool okr = ok && vi;
            if (valid && rdf_near_edge(tb, bin, r2, rc2)) {
                if (!ok) bin = (int)(sqrtf(r2) * inv_dx);
                bin = rdf_exact_bin<CUBIC>((int)((unsigned)xi.x - (unsigned)xj.x),
                                           (int)((unsigned)xi.y - (unsigned)xj.y),
                                           (int)((unsigned)xi.z - (unsigned)xj.z), E, pt, c.box, bin, okr);
            }
            if (okr && bin <= kNdist) atomicAdd(&hist[bin], 1u);
        }
    }
}

// Dispatch one tile to the specialised loop (uniform per CTA and tile).
template <int KIND, bool ENERGY, bool RDF, bool CUBIC>
__device__ __forceinline__ void tile_f32_any(const int4 *__restrict__ tj, int cnt, bool diag, int sub, int4 xi,
                                             const PairConsts &c, float &px, float &py, float &pz, float &pe,
                                             unsigned *hist, float inv_dx, bool vi, const RdfEdges *E, int pt) {
    constexpr int TPP = kTppF;
    if (RDF) {
        tile_f32<KIND, ENERGY, RDF, TPP, false, true, CUBIC>(tj, cnt, sub, xi, c, px, py, pz, pe, hist, inv_dx, vi,
                                                              E, pt);
    } else if (cnt == kTjF) {
        if (diag) tile_f32<KIND, ENERGY, false, TPP, true, true, CUBIC>(tj, cnt, sub, xi, c, px, py, pz, pe, hist, inv_dx);
        else tile_f32<KIND, ENERGY, false, TPP, true, false, CUBIC>(tj, cnt, sub, xi, c, px, py, pz, pe, hist, inv_dx);
    } else {
        tile_f32<KIND, ENERGY, false, TPP, false, true, CUBIC>(tj, cnt, sub, xi, c, px, py, pz, pe, hist, inv_dx);
    }
}

template <int EIKIND, bool ENERGY, bool RDF, bool CUBIC>
__global__ void __launch_bounds__(kPairThreads) pair_fp32c_kernel(const PairArgs a) {
    constexpr int TPP = kTppF;
    __shared__ __align__(128) int4 tiles[kStagesF][kTjF];
    __shared__ __align__(8) uint64_t bars[kStagesF];
    __shared__ unsigned hist[RDF ? 3 * kNbin : 1];
    __shared__ double red[32];

    const int tid = threadIdx.x;
    const int b = blockIdx.x;
    int si, i0, iend;
    if (b < a.nblk_e) {
        si = 0;
        i0 = b * a.bi;
        iend = a.nel;
    } else {
        si = 1;
        i0 = a.nel + (b - a.nblk_e) * a.bi;
        iend = a.n;
    }
    const int i = i0 + tid / TPP;
    const int sub = tid % TPP;
    const bool vi = i < iend;
    const int4 xi = a.xq[vi ? i : i0];

    const int t0 = blockIdx.y * a.tiles_per_split;
    const int nt = max(0, min(a.tiles_per_split, a.ntile - t0));

    if (tid == 0) {
        for (int s = 0; s < kStagesF; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    if (RDF)
        for (int k = tid; k < 3 * kNbin; k += blockDim.x) hist[k] = 0u;
    __syncthreads();
    if (tid == 0) {
        for (int k = 0; k < min(kStagesF, nt); ++k) {
            int j0, cnt, sj;
            tile_range(a, t0 + k, j0, cnt, sj);
            const uint32_t bytes = (uint32_t)cnt * sizeof(int4);
            mbar_arrive_expect_tx(&bars[k], bytes);
            bulk_g2s(tiles[k], a.xq + j0, bytes, &bars[k]);
        }
    }

    float fxh = 0.f, fxl = 0.f, fyh = 0.f, fyl = 0.f, fzh = 0.f, fzl = 0.f, eh = 0.f, el = 0.f;
    int k = 0;
    for (; k < nt; ++k) {
        const int stage = k % kStagesF;
        const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / kStagesF) & 1), kWaitLimitCycles);
        int j0, cnt, sj;
        tile_range(a, t0 + k, j0, cnt, sj);
        const int pt = si + sj;   // 0 e-e, 1 e-i, 2 i-i
        float px = 0.f, py = 0.f, pz = 0.f, pe = 0.f;
        unsigned *h = RDF ? hist + pt * kNbin : nullptr;
        const float inv_dx = RDF ? (CUBIC ? a.c.u_inv_dx[pt] : a.c.inv_dx[pt]) : 0.f;
        // the tile can hold the i-particles of this CTA only on the diagonal
        const bool diag = (j0 < i0 + a.bi) && (i0 < j0 + cnt);
        if (pt == 1 && EIKIND == 1)
            tile_f32_any<1, ENERGY, RDF, CUBIC>(tiles[stage], cnt, diag, sub, xi, a.c, px, py, pz, pe, h, inv_dx,
                                                 vi, a.rdf_edges, pt);
        else if (pt == 1 && EIKIND == 2)
            tile_f32_any<2, ENERGY, RDF, CUBIC>(tiles[stage], cnt, diag, sub, xi, a.c, px, py, pz, pe, h, inv_dx,
                                                 vi, a.rdf_edges, pt);
        else
            tile_f32_any<0, ENERGY, RDF, CUBIC>(tiles[stage], cnt, diag, sub, xi, a.c, px, py, pz, pe, h, inv_dx,
                                                 vi, a.rdf_edges, pt);
        const float qf = CUBIC ? a.c.u_qq_force[pt] : a.c.qqf[pt];
        const float qe = CUBIC ? a.c.u_qq_energy[pt] : a.c.qqf[pt];
        acc2(fxh, fxl, px * qf);
        acc2(fyh, fyl, py * qf);
        acc2(fzh, fzl, pz * qf);
        if (ENERGY) acc2(eh, el, pe * qe);
        // every thread has finished reading this stage: refill it
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(a.status, kStatusTmaTimeout);
            break;
        }
        if (tid == 0 && k + kStagesF < nt) {
            int j1, c1, s1;
            tile_range(a, t0 + k + kStagesF, j1, c1, s1);
            const uint32_t bytes = (uint32_t)c1 * sizeof(int4);
            mbar_arrive_expect_tx(&bars[stage], bytes);
            bulk_g2s(tiles[stage], a.xq + j1, bytes, &bars[stage]);
        }
    }
    if (k < nt) {
        // timed out: wait (bounded) for the copies still in flight, then leave
        if (tid == 0)
            for (int kk = k; kk < min(nt, k + kStagesF); ++kk)
                mbar_wait_bounded(&bars[kk % kStagesF], (uint32_t)((kk / kStagesF) & 1), kWaitLimitCycles);
        __syncthreads();
        return;
    }

    // reduce the TPP threads of one i-particle
#pragma unroll
    for (int o = TPP / 2; o > 0; o >>= 1) {
        float s, e, h2, l2;
        h2 = __shfl_xor_sync(0xffffffffu, fxh, o);
        l2 = __shfl_xor_sync(0xffffffffu, fxl, o);
        two_sum(fxh, h2, s, e);
        fxh = s;
        fxl = fxl + l2 + e;
        h2 = __shfl_xor_sync(0xffffffffu, fyh, o);
        l2 = __shfl_xor_sync(0xffffffffu, fyl, o);
        two_sum(fyh, h2, s, e);
        fyh = s;
        fyl = fyl + l2 + e;
        h2 = __shfl_xor_sync(0xffffffffu, fzh, o);
        l2 = __shfl_xor_sync(0xffffffffu, fzl, o);
        two_sum(fzh, h2, s, e);
        fzh = s;
        fzl = fzl + l2 + e;
    }
    if (vi && sub == 0) {
        double *fp = a.fpart + (size_t)blockIdx.y * 3 * a.n;
        fp[i] = kEps * ((double)fxh + (double)fxl);
        fp[a.n + i] = kEps * ((double)fyh + (double)fyl);
        fp[2 * a.n + i] = kEps * ((double)fzh + (double)fzl);
    }
    if (ENERGY) {
        const double ed = vi ? (double)eh + (double)el : 0.0;
        const double tot = block_sum(ed, red);
        if (tid == 0) a.upart[blockIdx.y * gridDim.x + blockIdx.x] = 0.5 * tot;
    }
    if (RDF) {
        __syncthreads();
        for (int q = tid; q < 3 * kNbin; q += blockDim.x)
            if (hist[q]) atomicAdd(&a.rdf[q], (unsigned long long)hist[q]);
    }
}

// ---------------------------------------------------------------------------
// FP64 kernel
template <int KIND, bool ENERGY, bool RDF, int TPP>
__device__ __forceinline__ void tile_f64(const double4_32a *__restrict__ tj, int cnt, int sub, double4_32a xi,
                                         const PairConsts &c, double qq, double &fx, double &fy,
                                         double &fz, double &ue, unsigned *hist, double inv_dx,
                                         const F64Tab &tb, bool vi = true) {
    // The expressions of force.f90 without divisions (GB300 issues FP64 at 1/64
    // of the FP32 rate): DNINT of d/box by multiplication with 1/box, 1/r from
    // rsqrt_nr, the exponentials from the table-driven exp_neg_tab, the Ewald
    // force term erfc(ar) + 2ar/sqrt(pi) exp(-a^2 r^2) (the reference's
    // 1 - erf(ar)) as exp(-a^2 r^2) ewald_q(ar), and erfc(r/lambda) from the
    // Kelbg Gaussian exp(-r^2/lambda^2) (erfc_tab; pair_math.cuh).
    const double a = c.alpha;
    for (int jj = sub; jj < cnt; jj += TPP) {
        const double4_32a xj = tj[jj];
        double xr0 = xi.x - xj.x, xr1 = xi.y - xj.y, xr2 = xi.z - xj.z;
        xr0 = fma(-c.box[0], round(xr0 * c.inv_box[0]), xr0);   // force.f90:92 (DNINT)
        xr1 = fma(-c.box[1], round(xr1 * c.inv_box[1]), xr1);
        xr2 = fma(-c.box[2], round(xr2 * c.inv_box[2]), xr2);
        const double r2 = xr0 * xr0 + xr1 * xr1 + xr2 * xr2;
        if (r2 < c.rc2 && r2 > 0.0) {
            const double rinv = rsqrt_nr(r2), r = r2 * rinv, rinv3 = rinv * rinv * rinv;
            const double e = exp_neg_tab(c.alpha2 * r2, tb);
            const double sq = e * ewald_q(a * r, tb);          // erfc(ar) + 2ar/sqrt(pi) exp(-a^2 r^2)
            const double er = fma(sq, rinv, -c.c_gauss_d * e);  // erfc(ar)/r
            double df, u;
            if (KIND == 0) {                                   // force.f90:104-106
                df = kEps * qq * sq * rinv3;
                u = qq * er;
            } else if (KIND == 1) {                            // force.f90:135-139
                const double y = exp_neg_tab(r * c.inv_rs_d, tb);
                df = kEps * qq * (sq - y - y * r * c.inv_rs_d) * rinv3;
                u = qq * (er - y * rinv);
            } else {                                           // Kelbg
                const double g = exp_neg_tab(r2 * c.inv_lam2, tb);
                df = kEps * qq * (sq - g) * rinv3;
                u = qq * ((er - g * rinv) + c.sqrtpi_lam_d * erfc_tab(r * c.inv_lam, g, tb));
            }
            fx += df * xr0;
            fy += df * xr1;
            fz += df * xr2;
            if (ENERGY) ue += u;
            if (RDF && vi) {                                   // (padding lanes count nothing)
                const double tb = sqrt(r2) * inv_dx;             // INT(r/dx) from the rounded sqrt
                if (tb < (double)kNbin) atomicAdd(&hist[(int)tb], 1u);
            }
        }
    }
}

template <int EIKIND, bool ENERGY, bool RDF>
__global__ void __launch_bounds__(kPairThreads) pair_fp64_kernel(const PairArgs a) {
    constexpr int TPP = kTppD;
    __shared__ __align__(128) double4_32a tiles[kStagesD][kTjD];
    __shared__ __align__(8) uint64_t bars[kStagesD];
    __shared__ unsigned hist[RDF ? 3 * kNbin : 1];
    __shared__ double red[32];
    __shared__ F64Tab tab;

    const int tid = threadIdx.x;
    const int b = blockIdx.x;
    int si, i0, iend;
    if (b < a.nblk_e) {
        si = 0;
        i0 = b * a.bi;
        iend = a.nel;
    } else {
        si = 1;
        i0 = a.nel + (b - a.nblk_e) * a.bi;
        iend = a.n;
    }
    const int i = i0 + tid / TPP;
    const int sub = tid % TPP;
    const bool vi = i < iend;
    const double4_32a xi = a.xd[vi ? i : i0];
    const int t0 = blockIdx.y * a.tiles_per_split;
    const int nt = max(0, min(a.tiles_per_split, a.ntile - t0));

    if (tid == 0) {
        for (int s = 0; s < kStagesD; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    if (RDF)
        for (int k = tid; k < 3 * kNbin; k += blockDim.x) hist[k] = 0u;
    load_f64_tab(tab);
    __syncthreads();
    if (tid == 0) {
        for (int k = 0; k < min(kStagesD, nt); ++k) {
            int j0, cnt, sj;
            tile_range(a, t0 + k, j0, cnt, sj);
            const uint32_t bytes = (uint32_t)cnt * sizeof(double4_32a);
            mbar_arrive_expect_tx(&bars[k], bytes);
            bulk_g2s(tiles[k], a.xd + j0, bytes, &bars[k]);
        }
    }
    double fx = 0.0, fy = 0.0, fz = 0.0, ue = 0.0;
    int k = 0;
    for (; k < nt; ++k) {
        const int stage = k % kStagesD;
        const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / kStagesD) & 1), kWaitLimitCycles);
        int j0, cnt, sj;
        tile_range(a, t0 + k, j0, cnt, sj);
        const int pt = si + sj;
        unsigned *h = RDF ? hist + pt * kNbin : nullptr;
        const double inv_dx = RDF ? a.c.inv_dxd[pt] : 0.0;
        const double qq = a.c.qq[pt];
        if (pt == 1 && EIKIND == 1)
            tile_f64<1, ENERGY, RDF, TPP>(tiles[stage], cnt, sub, xi, a.c, qq, fx, fy, fz, ue, h, inv_dx, tab, vi);
        else if (pt == 1 && EIKIND == 2)
            tile_f64<2, ENERGY, RDF, TPP>(tiles[stage], cnt, sub, xi, a.c, qq, fx, fy, fz, ue, h, inv_dx, tab, vi);
        else
            tile_f64<0, ENERGY, RDF, TPP>(tiles[stage], cnt, sub, xi, a.c, qq, fx, fy, fz, ue, h, inv_dx, tab, vi);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(a.status, kStatusTmaTimeout);
            break;
        }
        if (tid == 0 && k + kStagesD < nt) {
            int j1, c1, s1;
            tile_range(a, t0 + k + kStagesD, j1, c1, s1);
            const uint32_t bytes = (uint32_t)c1 * sizeof(double4_32a);
            mbar_arrive_expect_tx(&bars[stage], bytes);
            bulk_g2s(tiles[stage], a.xd + j1, bytes, &bars[stage]);
        }
    }
    if (k < nt) {
        if (tid == 0)
            for (int kk = k; kk < min(nt, k + kStagesD); ++kk)
                mbar_wait_bounded(&bars[kk % kStagesD], (uint32_t)((kk / kStagesD) & 1), kWaitLimitCycles);
        __syncthreads();
        return;
    }
#pragma unroll
    for (int o = TPP / 2; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
    if (vi && sub == 0) {
        double *fp = a.fpart + (size_t)blockIdx.y * 3 * a.n;
        fp[i] = fx;
        fp[a.n + i] = fy;
        fp[2 * a.n + i] = fz;
    }
    if (ENERGY) {
        const double tot = block_sum(vi ? ue : 0.0, red);
        if (tid == 0) a.upart[blockIdx.y * gridDim.x + blockIdx.x] = 0.5 * tot;
    }
    if (RDF) {
        __syncthreads();
        for (int q = tid; q < 3 * kNbin; q += blockDim.x)
            if (hist[q]) atomicAdd(&a.rdf[q], (unsigned long long)hist[q]);
    }
}

// ---------------------------------------------------------------------------
// f = sum over splits of fpart (+ frec: the SPME_SUM add of force.f90:953-964
// fused); per-block partial sums of f for REMOVE_RIGIDMTN (force.f90:986-993).
// When a tile wait of the pair kernel ran out (status), some partials were
// never written: f is then left as it was and the caller reports the error.
__global__ void force_finalize_kernel(const double *__restrict__ fpart, int nsplit,
                                      const double *__restrict__ frec, double *__restrict__ f, int n,
                                      double *__restrict__ fsum_part, const unsigned *__restrict__ status) {
    __shared__ double red[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool write = !(status && (*status & kStatusTmaTimeout));
    double s[3] = {0.0, 0.0, 0.0};
    if (i < n) {
        for (int k = 0; k < 3; ++k) {
            double acc = 0.0;
            for (int sp = 0; sp < nsplit; ++sp) acc += fpart[((size_t)sp * 3 + k) * n + i];
            if (frec) acc += frec[(size_t)k * n + i];
            if (write) f[(size_t)k * n + i] = acc;
            s[k] = acc;
        }
    }
    for (int k = 0; k < 3; ++k) {
        const double t = block_sum(s[k], red);
        if (threadIdx.x == 0) fsum_part[k * gridDim.x + blockIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// host side
void make_pair_consts(tcp_ctx *c) {
    PairConsts &k = c->pc;
    const tcp_params &p = c->p;
    const double two32 = 4294967296.0;
    k.sx = (float)(p.box[0] / two32);
    k.sy = (float)(p.box[1] / two32);
    k.sz = (float)(p.box[2] / two32);
    k.rc2f = (float)c->rc2;
    const double log2e = 1.4426950408889634;
    k.c_exp = (float)(-c->alpha * c->alpha * log2e);
    k.p_alpha = (float)(kErfcP * c->alpha);
    k.c_gauss = (float)(2.0 * c->alpha / kSqrtPi);
    const double rs = p.rs > 0 ? p.rs : 1.0;
    k.c_rs = (float)(-log2e / rs);
    k.inv_rs = (float)(1.0 / rs);
    const double lam = p.lambda_ei > 0 ? p.lambda_ei : 1.0;
    k.c_lam = (float)(-log2e / (lam * lam));
    k.p_lam = (float)(kErfcP / lam);
    k.sqrtpi_lam = (float)(kSqrtPi / lam);
    k.rshort2 = (float)(36.0 * lam * lam);
    const double close2 = std::min(0.25 * lam * lam, 0.25 / (c->alpha * c->alpha));
    k.close2 = (float)close2;
    k.inv_lam2f = (float)(1.0 / (lam * lam));
    k.alphaf = (float)c->alpha;
    const double dxs[3] = {p.dx_ee, p.dx_ei, p.dx_ii};
    const double s = p.charge_scale;
    const double qq[3] = {s * p.q[0] * s * p.q[0], s * p.q[0] * s * p.q[1], s * p.q[1] * s * p.q[1]};
    for (int t = 0; t < 3; ++t) {
        k.inv_dx[t] = dxs[t] > 0 ? (float)(1.0 / dxs[t]) : 0.f;
        k.inv_dxd[t] = dxs[t] > 0 ? 1.0 / dxs[t] : 0.0;
        k.qqf[t] = (float)qq[t];
        k.qq[t] = qq[t];
    }
    // cubic-box constants in units of u = L/2^32
    k.cubic = (p.box[0] == p.box[1] && p.box[1] == p.box[2]) ? 1 : 0;
    const double u = p.box[0] / two32;
    k.u_rc2 = (float)(c->rc2 / (u * u));
    k.u_p_alpha = (float)(kErfcP * c->alpha * u);
    k.u_p_alpha5 = (float)(kErfc5P * c->alpha * u);
    k.erfc5_ok = c->alpha * std::sqrt(c->rc2) <= kErfc5Xmax ? 1 : 0;
    k.u_c_exp = (float)(-c->alpha * c->alpha * log2e * u * u);
    k.u_c_gauss = (float)(2.0 * c->alpha / kSqrtPi * u);
    k.u_c_rs = (float)(-log2e / rs * u);
    k.u_inv_rs = (float)(u / rs);
    k.u_c_lam = (float)(-log2e / (lam * lam) * u * u);
    k.u_p_lam = (float)(kErfcP / lam * u);
    k.u_sqrtpi_lam = (float)(kSqrtPi / lam * u);
    k.u_rshort2 = (float)(36.0 * lam * lam / (u * u));
    k.u_close2 = (float)(close2 / (u * u));
    k.u_inv_lam2 = (float)(u * u / (lam * lam));
    k.u_alpha = (float)(c->alpha * u);
    for (int t = 0; t < 3; ++t) {
        k.u_inv_dx[t] = dxs[t] > 0 ? (float)(u / dxs[t]) : 0.f;
        k.u_qq_force[t] = (float)(qq[t] / (u * u));
        k.u_qq_energy[t] = (float)(qq[t] / u);
    }
    for (int d = 0; d < 3; ++d) {
        k.box[d] = p.box[d];
        k.inv_box[d] = 1.0 / p.box[d];
        k.sl[d] = p.box[d] / 18446744073709551616.0;
    }
    k.sl2 = k.sl[0] * k.sl[0];
    k.rc2 = c->rc2;
    k.alpha = c->alpha;
    k.rs = rs;
    k.lambda = lam;
    k.alpha2 = c->alpha * c->alpha;
    k.c_gauss_d = 2.0 * c->alpha / kSqrtPi;
    k.inv_rs_d = 1.0 / rs;
    k.inv_lam2 = 1.0 / (lam * lam);
    k.inv_lam = 1.0 / lam;
    k.sqrtpi_lam_d = kSqrtPi / lam;
    k.kelbg_far2 = (8.5 * lam) * (8.5 * lam);
    k.ei_model = p.ei_model;
}

static int ceil_div(int a, int b) { return (a + b - 1) / b; }

struct Geometry {
    int bi, tj, nblk_e, nblk, ntile_e, ntile;
};

static Geometry geometry(const tcp_ctx *c, bool fp64) {
    Geometry g;
    g.bi = kPairThreads / (fp64 ? kTppD : kTppF);
    g.tj = fp64 ? kTjD : kTjF;
    g.nblk_e = ceil_div(c->nel, g.bi);
    g.nblk = g.nblk_e + ceil_div(c->nion, g.bi);
    g.ntile_e = ceil_div(c->nel, g.tj);
    g.ntile = g.ntile_e + ceil_div(c->nion, g.tj);
    return g;
}

// Number of j-splits: fill the GPU with whole waves of CTAs.
static int choose_jsplit(const tcp_ctx *c, const Geometry &g, int blocks_per_sm) {
    const int slots = std::max(1, c->num_sms * std::max(1, blocks_per_sm));
    int best = 1;
    double best_eff = -1.0;
    for (int s = 1; s <= std::min(g.ntile, 64); ++s) {
        const int tps = ceil_div(g.ntile, s);
        const int s_eff = ceil_div(g.ntile, tps);
        const double waves = (double)g.nblk * s_eff / slots;
        // efficiency: wave quantisation times tile-split balance
        const double eff = waves / std::ceil(waves) * ((double)g.ntile / (double)(tps * s_eff));
        if (eff > best_eff + 0.02) {
            best_eff = eff;
            best = s_eff;
        }
    }
    return best;
}

// Bin edges of the exact RDF test (RdfEdges): in units of u^2 for cubic
// boxes, rounded up to integers, and in A^2 for the others.  Long double
// keeps (k dx/u)^2 < 2^64 to within a unit wherever it differs from double.
static void fill_rdf_edges(const tcp_ctx *c, RdfEdges &E) {
    const double dxs[3] = {c->p.dx_ee, c->p.dx_ei, c->p.dx_ii};
    const long double u = (long double)c->p.box[0] / 4294967296.0L;
    auto ceil_u64 = [](long double v) -> unsigned long long {
        if (!(v > 0.0L)) return 0ull;
        if (v >= 18446744073709551615.0L) return ~0ull;
        return (unsigned long long)ceill(v);
    };
    for (int t = 0; t < 3; ++t)
        for (int k = 0; k <= kNbin; ++k) {
            const long double x = (long double)k * (long double)dxs[t] / u;
            E.e[t][k] = dxs[t] > 0.0 ? ceil_u64(x * x) : ~0ull;
            const double d = (double)k * dxs[t];
            E.d[t][k] = dxs[t] > 0.0 ? d * d : 1e308;
        }
    E.rc2 = ceil_u64((long double)c->rc2 / (u * u));
    E.rc2d = c->rc2;
}

int pair_setup(tcp_ctx *c) {
    make_pair_consts(c);
    if (c->rdf_edges) {
        RdfEdges E;
        fill_rdf_edges(c, E);
        TCP_CUDA(cudaMemcpyAsync(c->rdf_edges, &E, sizeof E, cudaMemcpyHostToDevice, c->stream));
        TCP_CUDA(cudaStreamSynchronize(c->stream));   // E is a stack copy
    }
    const bool fp64 = c->p.precision == TCP_PREC_FP64;
    Geometry g = geometry(c, fp64);
    int bps = 1;
    if (fp64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pair_fp64_kernel<0, true, false>, kPairThreads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pair_fp32c_kernel<2, true, false, true>, kPairThreads, 0);
    const char *env = getenv("TCP_JSPLIT");
    int js = env ? atoi(env) : choose_jsplit(c, g, bps);
    js = std::max(1, std::min(js, g.ntile));
    const int tps = ceil_div(g.ntile, js);
    js = ceil_div(g.ntile, tps);
    if (c->fpart) cudaFree(c->fpart);
    if (c->upart) cudaFree(c->upart);
    c->fpart = nullptr;
    c->upart = nullptr;
    c->jsplit = js;
    c->n_upart = std::max(g.nblk * js, fp64 ? n3_f64_grid(c) : n3_grid(c));
    if (!fp64 && c->pc.cubic)
        if (int rc = n3_prepare_chunks(c)) return rc;
    TCP_CUDA(cudaMalloc(&c->fpart, sizeof(double) * 3 * (size_t)c->n * js));
    TCP_CUDA(cudaMalloc(&c->upart, sizeof(double) * (size_t)c->n_upart));
    TCP_CUDA(cudaMemsetAsync(c->upart, 0, sizeof(double) * (size_t)c->n_upart, c->stream));
    return TCP_OK;
}

int launch_pair(tcp_ctx *c, bool energy, bool rdf) {
    const bool fp64 = c->p.precision == TCP_PREC_FP64;
    if (n3_applicable(c)) {
        c->fpart_splits = 1;
        return launch_pair_n3(c, energy, rdf);
    }
    if (n3_f64_applicable(c)) {
        c->fpart_splits = 1;
        return launch_pair_n3_f64(c, energy, rdf);
    }
    c->fpart_splits = c->jsplit;
    Geometry g = geometry(c, fp64);
    PairArgs a;
    a.xq = c->xq;
    a.xd = c->xd;
    a.nel = c->nel;
    a.n = c->n;
    a.bi = g.bi;
    a.nblk_e = g.nblk_e;
    a.nblk = g.nblk;
    a.tj = g.tj;
    a.ntile_e = g.ntile_e;
    a.ntile = g.ntile;
    a.tiles_per_split = ceil_div(g.ntile, c->jsplit);
    a.fpart = c->fpart;
    a.upart = c->upart;
    a.rdf = c->rdf;
    a.rdf_edges = c->rdf_edges;
    a.status = c->status;
    a.c = c->pc;
    dim3 grid(g.nblk, c->jsplit);
    // the energy reduction sums all n_upart partials: clear the ones this grid
    // does not write (an earlier Newton-3 launch may have used more CTAs)
    if (energy && (size_t)g.nblk * c->jsplit < (size_t)c->n_upart)
        TCP_CUDA(cudaMemsetAsync(c->upart + (size_t)g.nblk * c->jsplit, 0,
                                 sizeof(double) * ((size_t)c->n_upart - (size_t)g.nblk * c->jsplit), c->stream));
    const int ei = c->p.ei_model == TCP_EI_DEUTSCH ? 1 : (c->p.ei_model == TCP_EI_KELBG ? 2 : 0);
#define TCP_PAIR_DISPATCH(KERNEL, ...)                                                                   \
    do {                                                                                                 \
        if (ei == 0) {                                                                                   \
            if (energy && rdf) KERNEL<0, true, true __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);   \
            else if (energy) KERNEL<0, true, false __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);    \
            else if (rdf) KERNEL<0, false, true __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);       \
            else KERNEL<0, false, false __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);               \
        } else if (ei == 1) {                                                                            \
            if (energy && rdf) KERNEL<1, true, true __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);   \
            else if (energy) KERNEL<1, true, false __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);    \
            else if (rdf) KERNEL<1, false, true __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);       \
            else KERNEL<1, false, false __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);               \
        } else {                                                                                         \
            if (energy && rdf) KERNEL<2, true, true __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);   \
            else if (energy) KERNEL<2, true, false __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);    \
            else if (rdf) KERNEL<2, false, true __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);       \
            else KERNEL<2, false, false __VA_ARGS__><<<grid, kPairThreads, 0, c->stream>>>(a);               \
        }                                                                                                \
    } while (0)
    if (fp64)
        TCP_PAIR_DISPATCH(pair_fp64_kernel);
    else if (c->pc.cubic)
        TCP_PAIR_DISPATCH(pair_fp32c_kernel, , true);
    else
        TCP_PAIR_DISPATCH(pair_fp32c_kernel, , false);
#undef TCP_PAIR_DISPATCH
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

int launch_force_finalize(tcp_ctx *c, bool add_rec) {
    const int threads = 256;
    const int blocks = ceil_div(c->n, threads);
    force_finalize_kernel<<<blocks, threads, 0, c->stream>>>(c->fpart, c->fpart_splits, add_rec ? c->frec : nullptr,
                                                             c->f, c->n, c->red, c->status);
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

}  // namespace tcp

// ---------------------------------------------------------------------------
// tcp_force_direct_noalloc: the real-space sum of tcp_force_direct for callers
// that cannot allocate device memory.
//
// Some programs that call this library may not allocate at the point where
// they need forces: a host code whose device memory is owned by another
// allocator (for example a framework pool that reserved the free HBM at
// start-up, so a cudaMalloc here would fail or fragment it), or a time-step
// loop that forbids allocation after set-up because cudaMalloc and cudaFree
// can synchronise the whole device and stall the other streams of the
// process.  This variant allocates nothing: every temporary (fixed-point or
// FP64 positions, per-split partial forces, energy and force-sum partials, the
// status word) lives in one file-scope device array of kNoAllocBytes, which
// every GPU that loads the library holds until the process exits.  The caller
// passes the positions and the force array (device memory, SoA [3][n]) and a
// host double for Ur.
//
// After a non-zero return the contents of f are undefined (a timed-out tile
// wait leaves them as they were).  The array's device address is looked up
// on every call with the caller's device current.
//
// The array is shared by all calls and keeps the last call's contents; this
// function clears what must start at zero (the status word) and overwrites
// everything else before reading it.  Calls that overlap on the GPU (from two
// host threads, or on two streams) race on the array: serialise them.
namespace tcp {

constexpr size_t kNoAllocBytes = 8u << 20;   // 8 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

__global__ void noalloc_positions_kernel(const double *__restrict__ x, int n, double iL0, double iL1, double iL2,
                                         int4 *xq, double4_32a *xd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double y0 = x[i], y1 = x[(size_t)n + i], y2 = x[2 * (size_t)n + i];
    if (xq) xq[i] = make_int4(fixed_coord(y0, iL0), fixed_coord(y1, iL1), fixed_coord(y2, iL2), 0);
    if (xd) xd[i] = make_double4_32a(y0, y1, y2, 0.0);
}

__global__ void noalloc_sum_kernel(const double *__restrict__ part, int np, double *out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int k = threadIdx.x; k < np; k += blockDim.x) s += part[k];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = s;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace tcp

extern "C" int tcp_force_direct_noalloc(const tcp_params *p, int nel, int nion, const double *x, double *f,
                                        double *Ur, void *stream) {
    using namespace tcp;
    if (!p || !x || !f) return set_error(TCP_ERR_BAD_PARAM, "NULL argument");
    if (nel < 0 || nion < 0 || nel + nion < 2) return set_error(TCP_ERR_BAD_PARAM, "need nel, nion >= 0 and nel+nion >= 2");
    for (int d = 0; d < 3; ++d)
        if (!(p->box[d] > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "box lengths must be positive");
    if (!(p->rc > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "rc must be positive");
    if (p->rc > std::min(std::min(p->box[0], p->box[1]), p->box[2]) / 2.0)
        return set_error(TCP_ERR_CUTOFF, " *** error at cut-off radius *** (rc > min(box)/2)");
    if (p->precision != TCP_PREC_FP64 && p->precision != TCP_PREC_FP32C && p->precision != TCP_PREC_FP32C_R64)
        return set_error(TCP_ERR_BAD_PARAM, "unknown precision");
    if (p->ei_model < TCP_EI_DEUTSCH || p->ei_model > TCP_EI_COULOMB) return set_error(TCP_ERR_BAD_PARAM, "unknown ei_model");
    if (p->ei_model == TCP_EI_DEUTSCH && !(p->rs > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "Deutsch model needs rs > 0");
    if (p->ei_model == TCP_EI_KELBG && !(p->lambda_ei > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "Kelbg model needs lambda_ei > 0");

    // The device address of the array, looked up on every call with the
    // caller's device current.  The lookup allocates nothing and costs far
    // less than the launch; a cached address could outlive the module (after
    // cudaDeviceReset the module is loaded again and the array may move).
    int dev = 0;
    TCP_CUDA(cudaGetDevice(&dev));
    void *base = nullptr;
    {
        const cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    }

    // the same constants and geometry as tcp_force_direct (host-side copy only)
    tcp_ctx tmp;
    tmp.p = *p;
    if (tmp.p.charge_scale == 0.0) tmp.p.charge_scale = 1.0;
    tmp.nel = nel;
    tmp.nion = nion;
    tmp.n = nel + nion;
    tmp.alpha = p->a > 0.0 ? p->a : 3.1 / p->rc;
    tmp.rc2 = p->rc * p->rc;
    TCP_CUDA(cudaDeviceGetAttribute(&tmp.num_sms, cudaDevAttrMultiProcessorCount, dev));
    make_pair_consts(&tmp);
    const bool fp64 = p->precision == TCP_PREC_FP64;
    const Geometry g = geometry(&tmp, fp64);
    int bps = 1;
    if (fp64)
        TCP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pair_fp64_kernel<0, true, false>, kPairThreads, 0));
    else
        TCP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pair_fp32c_kernel<2, true, false, true>, kPairThreads, 0));
    const size_t n = (size_t)tmp.n;
    const int nbf = ceil_div(tmp.n, 256);
    auto need = [&](int js) {
        return align256(16) + align256(n * (fp64 ? sizeof(double4_32a) : sizeof(int4))) +
               align256(sizeof(double) * 3 * (size_t)nbf) + align256(sizeof(double) * (size_t)g.nblk * js) +
               align256(sizeof(double) * 3 * n * js);
    };
    int js = choose_jsplit(&tmp, g, bps);
    js = ceil_div(g.ntile, ceil_div(g.ntile, std::max(1, std::min(js, g.ntile))));
    while (js > 1 && need(js) > kNoAllocBytes) js = ceil_div(g.ntile, ceil_div(g.ntile, js - 1));
    if (need(js) > kNoAllocBytes)
        return set_error(TCP_ERR_BAD_PARAM, "n = " + std::to_string(n) + " needs " + std::to_string(need(1)) +
                                                " bytes of scratch; the static array holds " +
                                                std::to_string(kNoAllocBytes) + " (8 MiB): use tcp_force_direct");
    unsigned char *b = static_cast<unsigned char *>(base);
    unsigned *status = reinterpret_cast<unsigned *>(b);
    b += align256(16);
    void *pos = b;
    b += align256(n * (fp64 ? sizeof(double4_32a) : sizeof(int4)));
    double *fsum = reinterpret_cast<double *>(b);
    b += align256(sizeof(double) * 3 * (size_t)nbf);
    double *upart = reinterpret_cast<double *>(b);
    b += align256(sizeof(double) * (size_t)g.nblk * js);
    double *fpart = reinterpret_cast<double *>(b);

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    TCP_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
    noalloc_positions_kernel<<<ceil_div(tmp.n, 256), 256, 0, st>>>(
        x, tmp.n, 1.0 / p->box[0], 1.0 / p->box[1], 1.0 / p->box[2], fp64 ? nullptr : static_cast<int4 *>(pos),
        fp64 ? static_cast<double4_32a *>(pos) : nullptr);
    PairArgs a;
    a.xq = fp64 ? nullptr : static_cast<const int4 *>(pos);
    a.xd = fp64 ? static_cast<const double4_32a *>(pos) : nullptr;
    a.nel = nel;
    a.n = tmp.n;
    a.bi = g.bi;
    a.nblk_e = g.nblk_e;
    a.nblk = g.nblk;
    a.tj = g.tj;
    a.ntile_e = g.ntile_e;
    a.ntile = g.ntile;
    a.tiles_per_split = ceil_div(g.ntile, js);
    a.fpart = fpart;
    a.upart = upart;
    a.rdf = nullptr;
    a.rdf_edges = nullptr;
    a.status = status;
    a.c = tmp.pc;
    dim3 grid(g.nblk, js);
    const int ei = p->ei_model == TCP_EI_DEUTSCH ? 1 : (p->ei_model == TCP_EI_KELBG ? 2 : 0);
    if (fp64) {
        if (ei == 0) pair_fp64_kernel<0, true, false><<<grid, kPairThreads, 0, st>>>(a);
        else if (ei == 1) pair_fp64_kernel<1, true, false><<<grid, kPairThreads, 0, st>>>(a);
        else pair_fp64_kernel<2, true, false><<<grid, kPairThreads, 0, st>>>(a);
    } else {
        if (tmp.pc.cubic) {
            if (ei == 0) pair_fp32c_kernel<0, true, false, true><<<grid, kPairThreads, 0, st>>>(a);
            else if (ei == 1) pair_fp32c_kernel<1, true, false, true><<<grid, kPairThreads, 0, st>>>(a);
            else pair_fp32c_kernel<2, true, false, true><<<grid, kPairThreads, 0, st>>>(a);
        } else {
            if (ei == 0) pair_fp32c_kernel<0, true, false, false><<<grid, kPairThreads, 0, st>>>(a);
            else if (ei == 1) pair_fp32c_kernel<1, true, false, false><<<grid, kPairThreads, 0, st>>>(a);
            else pair_fp32c_kernel<2, true, false, false><<<grid, kPairThreads, 0, st>>>(a);
        }
    }
    force_finalize_kernel<<<nbf, 256, 0, st>>>(fpart, js, nullptr, f, tmp.n, fsum, status);
    noalloc_sum_kernel<<<1, 1024, 0, st>>>(upart, g.nblk * js, fsum);   // Ur into fsum[0]
    TCP_CUDA(cudaGetLastError());
    double ur = 0.0;
    unsigned h_status = 0;
    TCP_CUDA(cudaMemcpyAsync(&ur, fsum, sizeof(double), cudaMemcpyDeviceToHost, st));
    TCP_CUDA(cudaMemcpyAsync(&h_status, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    TCP_CUDA(cudaStreamSynchronize(st));
    if (h_status & kStatusTmaTimeout) return set_error(TCP_ERR_TIMEOUT, "a pair-kernel tile wait exceeded its bound");
    if (Ur) *Ur = ur;
    return TCP_OK;
}

// ---------------------------------------------------------------------------
// Autotuner of the FP32C real-space kernel.  Candidates: the ordered-pair
// kernel (variant 0, any box) and the Newton-3 kernels (variants 1..V, cubic
// boxes: unroll depth of the rotation loop x CTAs per SM).  Each candidate is
// launched once to warm up and timed over two launches with CUDA events on the
// context's stream, on the positions currently on the device; the fastest is
// kept.  TCP_PAIR_VARIANT=k forces variant k; TCP_AUTOTUNE=0 keeps the default
// (Newton-3 variant 1 for cubic boxes); TCP_AUTOTUNE_CACHE=<file> stores the
// choice per (device, n, nel, e-i model), and the grid reserve per the same
// and the reciprocal setting (sum, mesh, order, FP64 chain), and reuses them
// without timing.
namespace tcp {

static std::string tune_key(const tcp_ctx *c) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, c->device);
    return std::string(prop.name) + "|" + std::to_string(c->n) + "|" + std::to_string(c->nel) + "|" +
           std::to_string(c->p.ei_model);
}

static int cache_lookup(const char *path, const std::string &key) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char line[512];
    int v = -1;
    while (fgets(line, sizeof line, f)) {
        std::string s(line);
        const size_t sp = s.rfind(' ');
        if (sp != std::string::npos && s.substr(0, sp) == key) v = atoi(s.c_str() + sp + 1);
    }
    fclose(f);
    return v;
}

// Real-space kernel of an FP32C context: the variant with the shortest
// pair-kernel time (TCP_PAIR_VARIANT forces one).
static int choose_variant(tcp_ctx *c, const char *cache, const std::string &key) {
    const int nv = c->pc.cubic ? std::min(n3_variant_count(), 31) : 0;
    c->pair_variant = c->pc.cubic ? 1 : 0;
    if (const char *forced = getenv("TCP_PAIR_VARIANT")) {
        const int v = std::min(std::max(atoi(forced), 0), nv);
        c->pair_variant = v == 0 || n3_variant_usable(c, v) ? v : c->pair_variant;
        return TCP_OK;
    }
    if (const char *off = getenv("TCP_AUTOTUNE"))
        if (atoi(off) == 0) return TCP_OK;
    if (cache) {
        const int v = cache_lookup(cache, key);
        if (v == 0 || (v >= 1 && v <= nv && n3_variant_usable(c, v))) {
            c->pair_variant = v;
            return TCP_OK;
        }
    }
    cudaEvent_t e0, e1;
    TCP_CUDA(cudaEventCreate(&e0));
    TCP_CUDA(cudaEventCreate(&e1));
    double best = 1e300;
    int best_v = c->pair_variant;
    int rc = TCP_OK;
    for (int v = 0; v <= nv && !rc; ++v) {
        if (v >= 1 && !n3_variant_usable(c, v)) continue;   // ms stays 0: not timed
        c->pair_variant = v;
        const long long before = c->launches;
        rc = launch_pair(c, true, false);
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 2 && !rc; ++r) rc = launch_pair(c, true, false);
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        c->launches = before;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        c->pair_variant_ms[v] = ms / 2;
        if (ms / 2 < best) {
            best = ms / 2;
            best_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    c->pair_variant = best_v;
    if (cache) {
        if (FILE *f = fopen(cache, "a")) {
            fprintf(f, "%s %d\n", key.c_str(), best_v);
            fclose(f);
        }
    }
    return TCP_OK;
}

// CTAs left out of the persistent Newton-3 grid.  In a step the reciprocal
// chain runs on a second stream beside the pair kernel; with every SM holding
// its full share of pair CTAs, the chain's kernels (cuFFT's among them) find no
// registers free and wait for the pair kernel's tail.  The reserved CTAs
// rejoin the pair launch once the chain is done (launch_pair_n3_rejoin), so a
// large reserve costs the pair kernel only while the chain runs: where the
// chain is long against the pair kernel (small N, or the FP64 chain) it lets
// the chain finish first.  Each candidate is timed as the pair kernel with the
// chain beside it, up to the join of both, captured as one graph and replayed
// (time_pair_with_recip; TCP_PAIR_RESERVE forces one).
static constexpr int kReserveCandidates[] = {0, 16, 32, 64, 128, 256, 512};
static int choose_reserve(tcp_ctx *c, const char *cache, const std::string &key) {
    c->pair_reserve = 0;
    if (const char *forced = getenv("TCP_PAIR_RESERVE")) {
        c->pair_reserve = std::max(atoi(forced), 0);
        return TCP_OK;
    }
    if (c->p.reciprocal == TCP_RECIP_NONE || !n3_applicable(c)) return TCP_OK;
    if (const char *off = getenv("TCP_AUTOTUNE"))
        if (atoi(off) == 0) return TCP_OK;
    const std::string rkey = key + "|" + std::to_string(c->p.reciprocal) + "|" + std::to_string(c->K1) + "x" +
                             std::to_string(c->K2) + "x" + std::to_string(c->K3) + "|" +
                             std::to_string(c->p.order) + "|" + (c->recip_fp64 ? "r64" : "r32") + " reserve";
    if (cache) {
        const int r = cache_lookup(cache, rkey);
        if (r >= 0) {
            c->pair_reserve = r;
            return TCP_OK;
        }
    }
    double best = 1e300;
    int k = 0;
    for (const int r : kReserveCandidates) {
        c->pair_reserve = r;
        double ms = 0.0;
        const long long before = c->launches;
        const int rc = time_pair_with_recip(c, 4, &ms);
        c->launches = before;
        if (rc) return rc;
        c->pair_reserve_ms[k++] = ms;
        best = std::min(best, ms);
    }
    // the smallest reserve within 0.3 % of the fastest: the candidates near the
    // optimum differ by less than the run-to-run spread, and inside a step (L2
    // flushed, graph-launched) the smaller ones have timed faster
    int best_r = kReserveCandidates[0];
    for (int j = k - 1; j >= 0; --j)
        if (c->pair_reserve_ms[j] <= best * 1.003) best_r = kReserveCandidates[j];
    c->pair_reserve = best_r;
    if (cache) {
        if (FILE *f = fopen(cache, "a")) {
            fprintf(f, "%s %d\n", rkey.c_str(), best_r);
            fclose(f);
        }
    }
    return TCP_OK;
}

int autotune_pair(tcp_ctx *c) {
    if (c->p.precision != TCP_PREC_FP32C || c->tuned) return TCP_OK;
    c->tuned = true;
    const char *cache = getenv("TCP_AUTOTUNE_CACHE");
    const std::string key = tune_key(c);
    int rc = choose_variant(c, cache, key);
    if (!rc) rc = choose_reserve(c, cache, key);
    if (rc) return rc;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

}  // namespace tcp

extern "C" const char *tcp_pair_variant_name(int variant) {
    using namespace tcp;
    if (variant < 0 || variant > n3_variant_count()) return nullptr;
    return n3_variant_name(variant);
}

extern "C" const char *tcp_batch_variant_name(int variant) {
    using namespace tcp;
    if (variant < 0 || variant >= n3_batch_variant_count()) return nullptr;
    return n3_batch_variant_name(variant);
}

extern "C" int tcp_autotune_report(tcp_ctx *c, int *variant, double *ms, int nmax) {
    using namespace tcp;
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    if (variant) *variant = c->pair_variant;
    for (int k = 0; ms && k < nmax && k < 32; ++k) ms[k] = c->pair_variant_ms[k];
    return TCP_OK;
}

extern "C" int tcp_overlap_report(tcp_ctx *c, int *reserve, int *candidates, double *ms, int nmax) {
    using namespace tcp;
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    if (reserve) *reserve = c->pair_reserve;
    constexpr int nc = (int)(sizeof kReserveCandidates / sizeof kReserveCandidates[0]);
    for (int k = 0; k < nmax && k < nc; ++k) {
        if (candidates) candidates[k] = kReserveCandidates[k];
        if (ms) ms[k] = c->pair_reserve_ms[k];
    }
    return TCP_OK;
}

// pair_n3.cu -- the compensated-FP32 real-space sum with Newton's third law:
// every unique pair (i < j) is evaluated once and its force is added to both
// particles (Force_direct_self / _ext / _sum of force.f90:52-372, whose
// triangular loops also evaluate each pair once).
//
// Work: particles are split per species into i-tiles of TILE = 32 R W
// particles (W warps, R i-particles per lane) and j-subtiles of kN3Sub = 128
// (tiles never straddle the e/i boundary).  An item is (i-tile I, j-subtile
// S) with S at or after I's first subtile; items are enumerated row by row.
// A persistent grid claims chunks of consecutive items from an atomic
// counter, the chunks shorter towards the end of the list (guided
// self-scheduling): the i-tile stays in registers along the long early
// chunks, and the single items at the end absorb the cost differences
// between items (pair types, masked items).
//
// A lane holds R i-particles (R i-chunks of 32 per warp).  A j-subtile is
// copied into shared memory by the bulk-copy engine (cp.async.bulk +
// mbarrier, kN3Stages-deep ring, issued three items ahead).  Each
// warp takes the subtile in chunks of 32: lane l loads j = l, and for 32
// steps computes the R pairs (i_r, j) and rotates j's position and reaction
// accumulator to the next lane with shuffles, so after 32 steps every lane
// holds the reaction of its own j again (the LDSJ variants read j's position
// from a warp-private doubled copy of the chunk instead of rotating it).
// The autotuner picks the variant; with a reciprocal sum running beside the
// launch, c->pair_reserve CTAs may be left out of the persistent grid.
// Reactions are summed over the
// warps in shared memory and added to the global FP64 force with one atomic
// per j and component per item; i-forces are folded per item into TwoSum
// (hi, lo) accumulators and added with atomics when the CTA leaves the row.
// Subtiles inside the i-tile (the diagonal) and partial tiles use an index
// mask i < j; all others run unmasked except for the cut-off.
//
// Pair arithmetic is that of pair_fp32c_kernel (fixed-point differences in
// units of L/2^32, SFU rsqrt/rcp/ex2, erfc = exp(-x^2) t Q(t), the series
// form of kelbg_close for close Kelbg pairs).  Cubic boxes only; other boxes
// use the ordered-pair kernel.
#include <algorithm>
#include <cstring>

#include "device_util.cuh"
#include "pair_n3.cuh"

namespace tcp {

// One pair in units of u = L/2^32.  Returns the force weight w (force on i is
// eps qq/u^2 * w * d) and, with ENERGY, adds the energy term / r to pe.
//   er = erfc(ar)/r is shared by the energy and by
//   w  = [erfc(ar)/r + 2a/sqrt(pi) exp(-a^2r^2) (- e-i terms)] / r^2.
// KIND 2 (Kelbg) adds its Gaussian terms only when `near_any` (a warp vote
// taken by the caller for all i-particles of the lane) is set.
template <int KIND, bool ENERGY, bool MASKED>
__device__ __forceinline__ float n3_pair(const PairConsts &c, float r2, bool ok, bool near_any, float &pe) {
    // The cut-off / index mask is applied once, to 1/r: er, the energy and
    // the weight all carry a factor rinv_m, so a masked pair adds exact zeros.
    // Unmasked items only hold distinct particles (r2 > 0); masked items may
    // pair a particle with itself or with padding, so r2 is replaced first.
    const float r2s = MASKED ? (ok ? r2 : 1.0f) : r2;
    const float rinv = rsqrt_approx(r2s);
    const float rinv_m = ok ? rinv : 0.0f;
    const float r = r2s * rinv;
    const float t = rcp_approx(fmaf(c.u_p_alpha, r, 1.0f));
    const float e = ex2_approx(c.u_c_exp * r2s);
    const float er = (e * erfc_poly(t)) * rinv_m;        // erfc(ar)/r
    float s = fmaf(c.u_c_gauss, e, er);                   // (erfc(ar) + 2ar/sqrt(pi) e^{-a^2r^2}) / r
    float u = er;
    if (KIND == 1) {                                      // Deutsch, force.f90:136-139
        const float y = ex2_approx(c.u_c_rs * r);         // exp(-r/rs)
        s = fmaf(-y, rinv + c.u_inv_rs, s);
        if (ENERGY) u = fmaf(-y, rinv_m, u);
    }
    if (KIND == 2 && near_any) {                          // Kelbg
        const bool near = ok && (r2s < c.u_rshort2);
        const float g = near ? ex2_approx(c.u_c_lam * r2s) : 0.0f;   // exp(-r^2/lambda^2)
        s = fmaf(-g, rinv, s);
        float erfc_rl = 0.0f;
        if (ENERGY) {
            const float t2 = rcp_approx(fmaf(c.u_p_lam, r, 1.0f));
            erfc_rl = g * erfc_poly(t2);                  // erfc(r/lambda)
            u += fmaf(c.u_sqrtpi_lam, erfc_rl, -g * rinv);
        }
        const bool close = near && (r2s < c.u_close2);
        if (__any_sync(0xffffffffu, close) && close) {    // series form, kelbg_close
            float nf, ne;
            kelbg_close(r2s * c.u_inv_lam2, r * c.u_alpha, nf, ne);
            s = nf * rinv;
            if (ENERGY) u = fmaf(c.u_sqrtpi_lam, erfc_rl, ne * rinv);
        }
    }
    if (ENERGY) pe += u;
    return s * (rinv_m * rinv_m);
}

// One item: the R i-particles of this lane against a j-subtile in shared
// memory.  MASKED: apply validity and i < j index masks.
template <int KIND, bool ENERGY, bool MASKED, int UNROLL, int R>
__device__ __forceinline__ void n3_item(const PairConsts &c, const int4 *__restrict__ tj, int cnt, int jstart,
                                        const int4 (&xi)[R], int ibase, int iend,
                                        float (*sjacc)[3], float (&p)[R][3], float &pe) {
    const int lane = threadIdx.x & 31;
    const int src = (lane + 1) & 31;
    for (int ch = 0; ch * 32 < cnt; ++ch) {
        int4 xj = tj[ch * 32 + lane];
        float jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll UNROLL
        for (int s = 0; s < 32; ++s) {
            float d[R][3], r2[R];
            bool ok[R];
            float r2min = 3.0e38f;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                d[r][0] = (float)(xi[r].x - xj.x);
                d[r][1] = (float)(xi[r].y - xj.y);
                d[r][2] = (float)(xi[r].z - xj.z);
                r2[r] = fmaf(d[r][0], d[r][0], fmaf(d[r][1], d[r][1], d[r][2] * d[r][2]));
                ok[r] = r2[r] < c.u_rc2;
                if (MASKED) {
                    const int jo = ch * 32 + ((lane + s) & 31);
                    const int ir = ibase + 32 * r;     // i-particle r of this lane
                    ok[r] = ok[r] && (ir < iend) && (jo < cnt) && (ir < jstart + jo);
                }
                if (KIND == 2) r2min = fminf(r2min, r2[r]);
            }
            // a vote without the masks: a false positive only runs the branch
            bool near_any = false;
            if (KIND == 2) near_any = __any_sync(0xffffffffu, r2min < c.u_rshort2);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float w = n3_pair<KIND, ENERGY, MASKED>(c, r2[r], ok[r], near_any, pe);
                p[r][0] = fmaf(w, d[r][0], p[r][0]);
                p[r][1] = fmaf(w, d[r][1], p[r][1]);
                p[r][2] = fmaf(w, d[r][2], p[r][2]);
                jx = fmaf(w, d[r][0], jx);
                jy = fmaf(w, d[r][1], jy);
                jz = fmaf(w, d[r][2], jz);
            }
            // rotate j (position and reaction) to the next lane
            xj.x = __shfl_sync(0xffffffffu, xj.x, src);
            xj.y = __shfl_sync(0xffffffffu, xj.y, src);
            xj.z = __shfl_sync(0xffffffffu, xj.z, src);
            jx = __shfl_sync(0xffffffffu, jx, src);
            jy = __shfl_sync(0xffffffffu, jy, src);
            jz = __shfl_sync(0xffffffffu, jz, src);
        }
        // back home: lane l holds the reaction sum of j = ch*32 + l
        float *q = sjacc[ch * 32 + lane];
        atomicAdd(q + 0, jx);
        atomicAdd(q + 1, jy);
        atomicAdd(q + 2, jz);
    }
}

// ---- paired FP32 (f32x2) form -------------------------------------------------
// The same pair arithmetic on two pairs per instruction with Blackwell's
// packed FP32 operations (__ffma2_rn / __fmul2_rn / __fadd2_rn, one issue slot
// for two lanes of work): the R i-particles of a lane form R/2 pairs (i_2g,
// i_2g+1) that share every FP32 step; the SFU operations, the int -> float
// conversions, compares and selects stay scalar.  Results equal the scalar
// form up to FMA contraction order (both are IEEE round-to-nearest per op).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

// The coefficients as (c, c) pairs in constant memory, so the packed FMAs can
// take them as 64-bit constant operands instead of register pairs.
struct ErfcQ2Table {
    float2 q[kErfcDeg + 1];
};
static constexpr ErfcQ2Table make_erfc_q2() {
    constexpr float q_[kErfcDeg + 1] = TCP_ERFC_Q;
    ErfcQ2Table t{};
    for (int k = 0; k <= kErfcDeg; ++k) t.q[k] = float2{q_[k], q_[k]};
    return t;
}
__constant__ ErfcQ2Table kErfcQ2 = make_erfc_q2();

struct Erfc5Q2Table {
    float2 q[kErfc5Deg + 1];
};
static constexpr Erfc5Q2Table make_erfc5_q2() {
    constexpr float q_[kErfc5Deg + 1] = TCP_ERFC5_Q;
    Erfc5Q2Table t{};
    for (int k = 0; k <= kErfc5Deg; ++k) t.q[k] = float2{q_[k], q_[k]};
    return t;
}
__constant__ Erfc5Q2Table kErfc5Q2 = make_erfc5_q2();

// Forms of the Ewald erfc polynomial of the packed kernels (Horner): degree 6
// (any argument up to 4.5), or degree 5 with kErfc5P for arguments up to
// kErfc5Xmax.  (An Estrin form of degree 5, a dependency chain of 3 instead
// of 5 for one operation more, was slower.)
constexpr int kErfcH6 = 6, kErfcH5 = 5;

template <int PD = kErfcH6>
__device__ __forceinline__ float2 erfc_poly2(float2 t) {
    static_assert(PD == kErfcH6 || PD == kErfcH5, "erfc polynomial forms");
    float2 q = PD == kErfcH6 ? kErfcQ2.q[0] : kErfc5Q2.q[0];
#pragma unroll
    for (int k = 1; k <= PD; ++k) q = __ffma2_rn(q, t, PD == kErfcH6 ? kErfcQ2.q[k] : kErfc5Q2.q[k]);
    return __fmul2_rn(q, t);
}

// RDF: +2 per unique pair inside rc in bin INT(r/dx) <= kNdist of this pair
// type (the ordered-pair kernels add 1 from each side), in a CTA histogram.
// Branch-free on the common path: a pair that does not count adds to its
// lane's spare slot (kRdfSpare + lane, never flushed), so every lane issues
// the same atomic (a predicated atomic, skipping the ~half of the pairs past
// rc = L/2, made the RDF step 10 % slower).  Measured at N = 65,536: the
// binning with its atomics costs 0.5 ms of a 2.6 ms step, the exact test of
// the pairs near a bin edge (taken in ~2 % of the steps) 2.6 ms when inlined
// behind a per-lane branch, 1.7 ms behind a warp vote, 1.1 ms out of line.  Pairs whose FP32 r/dx or r^2 lies
// near a bin edge or rc take the exact test of the fixed-point separation
// (rdf_exact_bin), so the counts equal those of exact arithmetic on the
// fixed-point positions.
constexpr int kRdfSpare = 3 * kNbin;
struct N3Rdf {
    unsigned *hist;
    int hoff;                  // pair type * kNbin
    int pt;                    // pair type
    float inv_dx;              // u / dx of this pair type
    float rc2;                 // cut-off^2 in u^2
    const RdfEdges *E;
};

__device__ __forceinline__ int idiff_i(int a, int b) { return (int)((unsigned)a - (unsigned)b); }

// The exact bin test of one pair, out of line: inlined, its 64-bit integer
// arithmetic and table loops weighed on the register allocation and
// scheduling of every rotation step although a step takes it rarely.  bin:
// the FP32 estimate, or -1 when the pair lies past rc in FP32 (the estimate is
// then taken from r2).  Returns bin << 1 | (r < rc exactly).
__device__ __noinline__ int rdf_exact_call(int d0, int d1, int d2, const RdfEdges *E, int t, int bin, float r2,
                                           float inv_dx) {
    if (bin < 0) bin = (int)(sqrtf(r2) * inv_dx);
    bool ok;
    bin = rdf_exact_bin<true>(d0, d1, d2, E, t, nullptr, bin, ok);
    return (bin << 1) | (ok ? 1 : 0);
}

// The bins of the two pairs of a packed step.  r: FP32 distances (meaningless
// where the caller replaced r^2 by 1); r2: the pairs' FP32 r^2; ok: the FP32
// cut-off and index masks; v: the index masks.  floor(r/dx) comes from packed
// FP32 arithmetic without a float->int conversion: (tb - 1/2) + 1.5 2^23
// rounds tb - 1/2 to an integer held in the low mantissa bits, which is
// floor(tb) unless tb lies within rounding of an integer; there, and within
// 2^-12 of any bin edge or of rc, the exact test of the fixed-point separation
// decides (two conversions per pair on the slow pipe had cost more than the
// pair's own arithmetic).
constexpr float kRdfRound = 12582912.0f;   // 1.5 * 2^23
constexpr int kRdfRoundBits = 0x4B400000;  // the bit pattern of kRdfRound
template <bool RDF>
__device__ __forceinline__ void rdf_add2(const N3Rdf &h, float2 r, float2 r2, bool ok0, bool ok1, bool v0, bool v1,
                                         const int4 &xa, const int4 &xb, const int4 &xj) {
    if (RDF) {
        const float2 tb = __fmul2_rn(r, make_float2(h.inv_dx, h.inv_dx));
        const float2 m = __fadd2_rn(__fadd2_rn(tb, make_float2(-0.5f, -0.5f)), make_float2(kRdfRound, kRdfRound));
        const float2 binf = __fadd2_rn(m, make_float2(-kRdfRound, -kRdfRound));
        const float2 fr = __ffma2_rn(binf, make_float2(-1.0f, -1.0f), tb);   // tb - floor estimate, exact
        int bin0 = __float_as_int(m.x) - kRdfRoundBits, bin1 = __float_as_int(m.y) - kRdfRoundBits;
        // the exact test where the estimate may be wrong: a bin edge within
        // 2^-12 of a pair inside rc, or rc itself within 2^-12; a pair clearly
        // past rc counts nothing whatever its bin
        // (one warp vote per step: a per-lane branch in every rotation step,
        // rarely taken, had cost as much as the pair arithmetic by breaking
        // the step's straight-line code)
        const float nrc = kRdfEdge * h.rc2;
        const bool x0 = v0 && (fabsf(r2.x - h.rc2) < nrc || (ok0 && fabsf(fr.x - 0.5f) > 0.5f - kRdfEdge));
        const bool x1 = v1 && (fabsf(r2.y - h.rc2) < nrc || (ok1 && fabsf(fr.y - 0.5f) > 0.5f - kRdfEdge));
        if (__any_sync(0xffffffffu, x0 || x1)) {
            if (x0) {
                const int pk = rdf_exact_call(idiff_i(xa.x, xj.x), idiff_i(xa.y, xj.y), idiff_i(xa.z, xj.z), h.E,
                                              h.pt, ok0 ? bin0 : -1, r2.x, h.inv_dx);
                bin0 = pk >> 1;
                ok0 = (pk & 1) != 0;
            }
            if (x1) {
                const int pk = rdf_exact_call(idiff_i(xb.x, xj.x), idiff_i(xb.y, xj.y), idiff_i(xb.z, xj.z), h.E,
                                              h.pt, ok1 ? bin1 : -1, r2.y, h.inv_dx);
                bin1 = pk >> 1;
                ok1 = (pk & 1) != 0;
            }
        }
        const int spare = kRdfSpare + (int)(threadIdx.x & 31);
        atomicAdd(&h.hist[(ok0 && bin0 <= kNdist) ? h.hoff + bin0 : spare], 2u);
        atomicAdd(&h.hist[(ok1 && bin1 <= kNdist) ? h.hoff + bin1 : spare], 2u);
    }
}

// PD: degree of the Ewald erfc polynomial (kErfcH6, or kErfcH5 when
// alpha rc <= kErfc5Xmax); the Kelbg erfc(r/lambda) always uses kErfcH6.
// RDF: h, the index masks v0, v1 and the positions xa, xb (i-particles) and
// xj of the two pairs.
template <int KIND, bool ENERGY, bool MASKED, bool RDF = false, int PD = kErfcH6>
__device__ __forceinline__ float2 n3_pair_x2(const PairConsts &c, float2 r2, bool ok0, bool ok1, bool near_any,
                                             float2 &pe, const N3Rdf *h = nullptr, bool v0 = true, bool v1 = true,
                                             const int4 *xa = nullptr, const int4 *xb = nullptr,
                                             const int4 *xj = nullptr) {
    const float2 r2s = MASKED ? make_float2(ok0 ? r2.x : 1.0f, ok1 ? r2.y : 1.0f) : r2;
    const float2 rinv = make_float2(rsqrt_approx(r2s.x), rsqrt_approx(r2s.y));
    const float2 rinv_m = make_float2(ok0 ? rinv.x : 0.0f, ok1 ? rinv.y : 0.0f);
    const float2 r = __fmul2_rn(r2s, rinv);
    if (RDF) rdf_add2<RDF>(*h, r, r2, ok0, ok1, v0, v1, *xa, *xb, *xj);
    const float2 ta = __ffma2_rn(f2(PD == kErfcH6 ? c.u_p_alpha : c.u_p_alpha5), r, f2(1.0f));
    const float2 t = make_float2(rcp_approx(ta.x), rcp_approx(ta.y));
    const float2 ea = __fmul2_rn(f2(c.u_c_exp), r2s);
    const float2 e = make_float2(ex2_approx(ea.x), ex2_approx(ea.y));
    const float2 er = __fmul2_rn(__fmul2_rn(e, erfc_poly2<PD>(t)), rinv_m);   // erfc(ar)/r
    float2 s = __ffma2_rn(f2(c.u_c_gauss), e, er);
    float2 u = er;
    if (KIND == 1) {                                      // Deutsch, force.f90:136-139
        const float2 ya = __fmul2_rn(f2(c.u_c_rs), r);
        const float2 y = make_float2(ex2_approx(ya.x), ex2_approx(ya.y));   // exp(-r/rs)
        s = __ffma2_rn(y, __ffma2_rn(rinv, f2(-1.0f), f2(-c.u_inv_rs)), s);
        if (ENERGY) u = __ffma2_rn(y, __fmul2_rn(rinv_m, f2(-1.0f)), u);
    }
    if (KIND == 2 && near_any) {                          // Kelbg
        const bool n0 = ok0 && (r2s.x < c.u_rshort2), n1 = ok1 && (r2s.y < c.u_rshort2);
        const float2 ga = __fmul2_rn(f2(c.u_c_lam), r2s);
        const float2 g = make_float2(n0 ? ex2_approx(ga.x) : 0.0f, n1 ? ex2_approx(ga.y) : 0.0f);
        const float2 nrinv = __fmul2_rn(rinv, f2(-1.0f));
        s = __ffma2_rn(g, nrinv, s);
        float2 erfc_rl = f2(0.0f);
        if (ENERGY) {
            const float2 t2a = __ffma2_rn(f2(c.u_p_lam), r, f2(1.0f));
            const float2 t2 = make_float2(rcp_approx(t2a.x), rcp_approx(t2a.y));
            erfc_rl = __fmul2_rn(g, erfc_poly2<kErfcH6>(t2));   // erfc(r/lambda)
            u = __fadd2_rn(u, __ffma2_rn(f2(c.u_sqrtpi_lam), erfc_rl, __fmul2_rn(g, nrinv)));
        }
        const bool c0 = n0 && (r2s.x < c.u_close2), c1 = n1 && (r2s.y < c.u_close2);
        if (__any_sync(0xffffffffu, c0 || c1)) {          // series form, kelbg_close
            float nf, ne;
            if (c0) {
                kelbg_close(r2s.x * c.u_inv_lam2, r.x * c.u_alpha, nf, ne);
                s.x = nf * rinv.x;
                if (ENERGY) u.x = fmaf(c.u_sqrtpi_lam, erfc_rl.x, ne * rinv.x);
            }
            if (c1) {
                kelbg_close(r2s.y * c.u_inv_lam2, r.y * c.u_alpha, nf, ne);
                s.y = nf * rinv.y;
                if (ENERGY) u.y = fmaf(c.u_sqrtpi_lam, erfc_rl.y, ne * rinv.y);
            }
        }
    }
    if (ENERGY) pe = __fadd2_rn(pe, u);
    return __fmul2_rn(s, __fmul2_rn(rinv_m, rinv_m));
}

__device__ __forceinline__ float idiff(int a, int b) { return (float)(int)((unsigned)a - (unsigned)b); }

// LDSJ: j positions read from a warp-private copy of the chunk written twice
// in a row (jb[64]), so that step s reads jb[lane + s] with one shared load
// instead of rotating them with three shuffles; the reactions still rotate.
template <int KIND, bool ENERGY, bool MASKED, int UNROLL, int R, bool LDSJ = false, bool RDF = false,
          int PD = kErfcH6>
__device__ __forceinline__ void n3_item_x2(const PairConsts &c, const int4 *__restrict__ tj, int cnt, int jstart,
                                           const int4 (&xi)[R], int ibase, int iend,
                                           float (*sjacc)[3], float (&p)[R][3], float &pe, int4 *jb = nullptr,
                                           const N3Rdf *rh = nullptr) {
    static_assert(R % 2 == 0, "paired form needs an even number of i-particles per lane");
    constexpr int G = R / 2;
    const int lane = threadIdx.x & 31;
    const int src = (lane + 1) & 31;
    float2 pg[G][3];
    float2 pe2 = f2(0.0f);
#pragma unroll
    for (int g = 0; g < G; ++g) pg[g][0] = pg[g][1] = pg[g][2] = f2(0.0f);
    for (int ch = 0; ch * 32 < cnt; ++ch) {
        int4 xj = tj[ch * 32 + lane];
        if (LDSJ) {
            __syncwarp();                // the previous chunk's reads of jb are done
            jb[lane] = xj;
            jb[lane + 32] = xj;
            __syncwarp();
        }
        float2 jx = f2(0.0f), jy = f2(0.0f), jz = f2(0.0f);
#pragma unroll UNROLL
        for (int s = 0; s < 32; ++s) {
            if (LDSJ) xj = jb[lane + s];
            float2 d[G][3], r2[G];
            bool ok[R], valid[R];
            float r2min = 3.0e38f;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                d[g][0] = make_float2(idiff(xi[2 * g].x, xj.x), idiff(xi[2 * g + 1].x, xj.x));
                d[g][1] = make_float2(idiff(xi[2 * g].y, xj.y), idiff(xi[2 * g + 1].y, xj.y));
                d[g][2] = make_float2(idiff(xi[2 * g].z, xj.z), idiff(xi[2 * g + 1].z, xj.z));
                r2[g] = __ffma2_rn(d[g][0], d[g][0], __ffma2_rn(d[g][1], d[g][1], __fmul2_rn(d[g][2], d[g][2])));
                valid[2 * g] = valid[2 * g + 1] = true;
                if (MASKED) {
                    const int jo = ch * 32 + ((lane + s) & 31);
                    const int i0 = ibase + 64 * g, i1 = i0 + 32;   // i-particles 2g, 2g+1 of this lane
                    valid[2 * g] = (i0 < iend) && (jo < cnt) && (i0 < jstart + jo);
                    valid[2 * g + 1] = (i1 < iend) && (jo < cnt) && (i1 < jstart + jo);
                }
                ok[2 * g] = (r2[g].x < c.u_rc2) && valid[2 * g];
                ok[2 * g + 1] = (r2[g].y < c.u_rc2) && valid[2 * g + 1];
                if (KIND == 2) r2min = fminf(r2min, fminf(r2[g].x, r2[g].y));
            }
            bool near_any = false;
            if (KIND == 2) near_any = __any_sync(0xffffffffu, r2min < c.u_rshort2);
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const float2 w = n3_pair_x2<KIND, ENERGY, MASKED, RDF, PD>(
                    c, r2[g], ok[2 * g], ok[2 * g + 1], near_any, pe2, rh, valid[2 * g], valid[2 * g + 1], &xi[2 * g],
                    &xi[2 * g + 1], &xj);
                pg[g][0] = __ffma2_rn(w, d[g][0], pg[g][0]);
                pg[g][1] = __ffma2_rn(w, d[g][1], pg[g][1]);
                pg[g][2] = __ffma2_rn(w, d[g][2], pg[g][2]);
                jx = __ffma2_rn(w, d[g][0], jx);
                jy = __ffma2_rn(w, d[g][1], jy);
                jz = __ffma2_rn(w, d[g][2], jz);
            }
            // rotate j (position and both halves of the reaction) to the next lane
            if (!LDSJ) {
                xj.x = __shfl_sync(0xffffffffu, xj.x, src);
                xj.y = __shfl_sync(0xffffffffu, xj.y, src);
                xj.z = __shfl_sync(0xffffffffu, xj.z, src);
            }
            jx.x = __shfl_sync(0xffffffffu, jx.x, src);
            jx.y = __shfl_sync(0xffffffffu, jx.y, src);
            jy.x = __shfl_sync(0xffffffffu, jy.x, src);
            jy.y = __shfl_sync(0xffffffffu, jy.y, src);
            jz.x = __shfl_sync(0xffffffffu, jz.x, src);
            jz.y = __shfl_sync(0xffffffffu, jz.y, src);
        }
        float *q = sjacc[ch * 32 + lane];
        atomicAdd(q + 0, jx.x + jx.y);
        atomicAdd(q + 1, jy.x + jy.y);
        atomicAdd(q + 2, jz.x + jz.y);
    }
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
        for (int k = 0; k < 3; ++k) {     // p is zero on entry
            p[2 * g][k] = pg[g][k].x;
            p[2 * g + 1][k] = pg[g][k].y;
        }
    pe = pe2.x + pe2.y;
}

// MODE 0: scalar FP32, i-force accumulators in registers; 1: packed FP32x2,
// accumulators in shared memory; 2: as 1 with j positions read from shared
// memory (LDSJ).
// W: warps per CTA (i-tile = 32 R W particles).  PD: degree of the Ewald erfc
// polynomial of the packed forms (kErfcH5 only where PairConsts::erfc5_ok).
template <bool ENERGY, int R, int UNROLL, int MINB, bool BATCH, int MODE = 0, int W = kN3Warps, bool RDF = false,
          int PD = kErfcH6>
__global__ void __launch_bounds__(32 * W, MINB) pair_n3_kernel(const N3Args a) {
    static_assert(W >= 1, "at least one warp per CTA");
    static_assert(!RDF || (MODE >= 1 && !BATCH), "RDF histograms: packed single-system forms");
    static_assert(PD == kErfcH6 || MODE >= 1, "the degree-5 erfc exists in the packed forms");
    static_assert((32 * R * W) % kN3Sub == 0, "i-tiles hold whole j-subtiles");
    constexpr int NT = 32 * W;
    constexpr bool X2 = MODE >= 1;
    constexpr bool SACC = MODE >= 1;
    constexpr int TILE = 32 * R * W;
    constexpr int SPT = TILE / kN3Sub;
    __shared__ __align__(128) int4 tiles[kN3Stages][kN3Sub];
    __shared__ __align__(8) uint64_t bars[kN3Stages];
    __shared__ float sjacc[kN3Sub][3];
    __shared__ double red[32];
    // the item of each ring slot, decoded once by thread 0 (s_I < 0: no item)
    __shared__ int s_rep[kN3Stages], s_I[kN3Stages], s_S[kN3Stages];
    __shared__ unsigned hist[RDF ? kRdfSpare + 32 : 1];
    // per-thread TwoSum (hi, lo) i-force accumulators, touched once per item:
    // in shared memory ([slot][thread], conflict-free) for the packed forms,
    // whose constant pairs need the registers
    __shared__ float sacc[SACC ? 2 * 3 * R : 1][SACC ? NT : 1];
    __shared__ __align__(16) int4 jbuf[MODE == 2 ? W : 1][MODE == 2 ? 64 : 1];
    float hi[SACC ? 1 : R][3], lo[SACC ? 1 : R][3];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int k = tid; k < kN3Sub * 3; k += NT) (&sjacc[0][0])[k] = 0.f;
    if (RDF)
        for (int k = tid; k < kRdfSpare + 32; k += NT) hist[k] = 0u;
    if (tid == 0) {
        for (int s = 0; s < kN3Stages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    // Guided self-scheduling: thread 0 claims chunks of consecutive items
    // (a.chunks, shorter towards the end of the list) from the counter, so the
    // CTAs end together whatever their items cost, and the i-tile stays in
    // registers along the long early chunks.  It decodes each item once,
    // publishes it in the ring slot of its subtile copy and issues the copy
    // kN3Stages items ahead of the one being processed.
    long long cur = 0, cend = 0;   // thread 0: the rest of the current chunk
    bool drained = false;          // thread 0: the chunk list is exhausted
    int last_filled = -1;          // thread 0: ring index of the last item with a copy
    auto fill = [&](int k) {       // ring index k (slot k % kN3Stages), thread 0
        const int stage = k % kN3Stages;
        if (!drained && cur == cend) {
            const unsigned j = atomicAdd(a.counter, 1u);
            if (j < a.nchunks) {
                cur = a.chunks[j];
                cend = a.chunks[j + 1];
            } else {
                drained = true;
            }
        }
        if (drained) {
            s_I[stage] = -1;
            return;
        }
        int rep, I_, S_;
        n3_locate<TILE, BATCH>(a, cur++, rep, I_, S_);
        s_rep[stage] = rep;
        s_I[stage] = I_;
        s_S[stage] = S_;
        last_filled = k;
        if (a.inject_skip && blockIdx.x == 0 && k == 0) return;   // test hook: the copy never comes
        const N3Geom &g = n3_geom<BATCH>(a, rep);
        int js, jc, jsp;
        n3_sub(g, S_, js, jc, jsp);
        const uint32_t bytes = (uint32_t)jc * sizeof(int4);
        mbar_arrive_expect_tx(&bars[stage], bytes);
        bulk_g2s(tiles[stage], a.xq + g.off + js, bytes, &bars[stage]);
    };
    if (tid == 0)
        for (int k = 0; k < kN3Stages; ++k) fill(k);

    double etot = 0.0;
    int curRep = -1, curI = -1, istart = 0, iend = 0, isp = 0, ifirst = 0, ioff = 0;
    int4 xi[R];
    int ibase = 0;           // i-particle 0 of this lane; particle r is ibase + 32 r
    float eh = 0.f, el = 0.f;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        xi[r] = make_int4(0, 0, 0, 0);
    }
    if constexpr (SACC) {
#pragma unroll
        for (int q = 0; q < 6 * R; ++q) sacc[q][tid] = 0.f;   // slot 6r+2k: hi, 6r+2k+1: lo
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) hi[r][0] = hi[r][1] = hi[r][2] = lo[r][0] = lo[r][1] = lo[r][2] = 0.f;
    }

    // i-forces of the current row to global memory (all threads, uniform)
    auto flush_i = [&]() {
        if (curI < 0) return;
#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float &h = SACC ? sacc[6 * r + 2 * k][tid] : hi[SACC ? 0 : r][k];
                float &l = SACC ? sacc[6 * r + 2 * k + 1][tid] : lo[SACC ? 0 : r][k];
                if (ibase + 32 * r < iend)
                    atomicAdd(&a.facc[(size_t)k * a.ntot + ioff + ibase + 32 * r], kEps * ((double)h + (double)l));
                h = 0.f;
                l = 0.f;
            }
        }
        if (ENERGY) {
            if (BATCH) {
                const double t = block_sum((double)eh + (double)el, red);
                if (tid == 0) atomicAdd(&a.ur_rep[curRep], t);
            } else {
                etot += (double)eh + (double)el;
            }
        }
        eh = el = 0.f;
    };

    // process the item (replica rep, row I_, subtile S_) of ring index k;
    // false on timeout
    auto process = [&](int k, int rep, int I_, int S_) -> bool {
        const N3Geom &g = n3_geom<BATCH>(a, rep);
        if (I_ != curI || rep != curRep) {
            flush_i();
            curI = I_;
            curRep = rep;
            ioff = g.off;
            n3_itile<TILE>(g, I_, istart, iend, isp, ifirst);
            ibase = istart + warp * 32 * R + lane;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ir = istart + warp * 32 * R + r * 32 + lane;
                xi[r] = a.xq[ioff + (ir < iend ? ir : istart)];
            }
        }
        int jstart, cnt, jsp;
        n3_sub(g, S_, jstart, cnt, jsp);
        const int pt = isp + jsp;
        const bool masked = (S_ < ifirst + SPT && jsp == isp) || cnt < kN3Sub || (iend - istart) < TILE;
        const int stage = k % kN3Stages;
        const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / kN3Stages) & 1), kWaitLimitCycles);
        const PairConsts &c = n3_consts<BATCH>(a, rep);
        float p[R][3], pe = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r) p[r][0] = p[r][1] = p[r][2] = 0.f;
        const int kind = pt == 1 ? (c.ei_model == TCP_EI_DEUTSCH ? 1 : (c.ei_model == TCP_EI_KELBG ? 2 : 0)) : 0;
        N3Rdf rh;
        if (RDF) rh = N3Rdf{hist, pt * kNbin, pt, c.u_inv_dx[pt], c.u_rc2, a.rdf_edges};
#define TCP_N3_ITEM(KIND, MASKED)                                                                      \
    do {                                                                                                \
        if (X2)                                                                                         \
            n3_item_x2<KIND, ENERGY, MASKED, UNROLL, R, MODE == 2, RDF, PD>(c, tiles[stage], cnt, jstart, xi, ibase, iend, sjacc, p, pe, jbuf[MODE == 2 ? warp : 0], &rh); \
        else                                                                                            \
            n3_item<KIND, ENERGY, MASKED, UNROLL, R>(c, tiles[stage], cnt, jstart, xi, ibase, iend, sjacc, p, pe);    \
    } while (0)
        if (masked) {
            if (kind == 1) TCP_N3_ITEM(1, true);
            else if (kind == 2) TCP_N3_ITEM(2, true);
            else TCP_N3_ITEM(0, true);
        } else {
            if (kind == 1) TCP_N3_ITEM(1, false);
            else if (kind == 2) TCP_N3_ITEM(2, false);
            else TCP_N3_ITEM(0, false);
        }
#undef TCP_N3_ITEM
        const float qf = c.u_qq_force[pt];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if constexpr (SACC) {
                    float h = sacc[6 * r + 2 * k][tid], l = sacc[6 * r + 2 * k + 1][tid];
                    acc2(h, l, p[r][k] * qf);
                    sacc[6 * r + 2 * k][tid] = h;
                    sacc[6 * r + 2 * k + 1][tid] = l;
                } else {
                    acc2(hi[r][k], lo[r][k], p[r][k] * qf);
                }
            }
        if (ENERGY) acc2(eh, el, pe * c.u_qq_energy[pt]);
        // all warps are done with this subtile and its reaction sums
        const bool timeout = __syncthreads_or(!ok);
        if constexpr (NT >= kN3Sub) {
            if (!timeout && tid < cnt) {
                const double sc = -kEps * (double)qf;
                const size_t j = (size_t)ioff + jstart + tid;
                atomicAdd(&a.facc[j], sc * (double)sjacc[tid][0]);
                atomicAdd(&a.facc[(size_t)a.ntot + j], sc * (double)sjacc[tid][1]);
                atomicAdd(&a.facc[2 * (size_t)a.ntot + j], sc * (double)sjacc[tid][2]);
            }
            if (tid < kN3Sub) sjacc[tid][0] = sjacc[tid][1] = sjacc[tid][2] = 0.f;
        } else {   // fewer threads than subtile particles: each flushes several
            for (int t = tid; t < kN3Sub; t += NT) {
                if (!timeout && t < cnt) {
                    const double sc = -kEps * (double)qf;
                    const size_t j = (size_t)ioff + jstart + t;
                    atomicAdd(&a.facc[j], sc * (double)sjacc[t][0]);
                    atomicAdd(&a.facc[(size_t)a.ntot + j], sc * (double)sjacc[t][1]);
                    atomicAdd(&a.facc[2 * (size_t)a.ntot + j], sc * (double)sjacc[t][2]);
                }
                sjacc[t][0] = sjacc[t][1] = sjacc[t][2] = 0.f;
            }
        }
        return !timeout;
    };

    __syncthreads();   // the first slots are published
    bool good = true;
    int k = 0;
    for (;; ++k) {
        const int stage = k % kN3Stages;
        const int I_ = s_I[stage];
        if (I_ < 0) break;
        if (!process(k, s_rep[stage], I_, s_S[stage])) {   // ends with a CTA barrier
            good = false;
            break;
        }
        if (tid == 0) fill(k + kN3Stages);
        __syncthreads();
    }
    if (!good) {
        if (tid == 0) {
            atomicOr(a.status, kStatusTmaTimeout);
            for (int kk = k; kk <= last_filled; ++kk)   // copies possibly still in flight
                mbar_wait_bounded(&bars[kk % kN3Stages], (uint32_t)((kk / kN3Stages) & 1), kWaitLimitCycles);
        }
        __syncthreads();
        return;
    }
    flush_i();
    if (ENERGY && !BATCH) {
        const double tot = block_sum(etot, red);
        if (tid == 0) a.upart[blockIdx.x] = tot;
    }
    if (RDF) {
        __syncthreads();
        for (int q = tid; q < 3 * kNbin; q += NT)
            if (hist[q]) atomicAdd(&a.rdf[q], (unsigned long long)hist[q]);
    }
}

// ---------------------------------------------------------------------------
static int cdiv(int x, int y) { return (x + y - 1) / y; }

bool n3_applicable(const tcp_ctx *c) {
    return c->p.precision == TCP_PREC_FP32C && c->pc.cubic && c->n >= 2 && c->pair_variant > 0 &&
           !(c->flags & TCP_FLAG_DETERMINISTIC);
}

// Variants 1..V (0 = the ordered-pair kernel): i-particles per lane x unroll
// depth of the rotation loop x CTAs per SM.
typedef void (*N3Kernel)(const N3Args);
struct N3Variant {
    N3Kernel energy, plain;
    int R, W;
    const char *name;
    bool erfc5 = false;   // degree-5 Ewald erfc: only where PairConsts::erfc5_ok
};
static const N3Variant kVariants[] = {
    // degree-6 Ewald erfc (any alpha rc)
    {pair_n3_kernel<true, 4, 2, 2, false>, pair_n3_kernel<false, 4, 2, 2, false>, 4, 8, "n3_r4_u2_b2"},
    {pair_n3_kernel<true, 4, 2, 2, false, 1>, pair_n3_kernel<false, 4, 2, 2, false, 1>, 4, 8, "n3_r4_u2_b2_x2"},
    {pair_n3_kernel<true, 4, 1, 5, false, 1, 4>, pair_n3_kernel<false, 4, 1, 5, false, 1, 4>, 4, 4, "n3_r4_u1_w4b5_x2"},
    {pair_n3_kernel<true, 4, 1, 3, false, 2>, pair_n3_kernel<false, 4, 1, 3, false, 2>, 4, 8, "n3_r4_u1_b3_x2l"},
    {pair_n3_kernel<true, 4, 2, 4, false, 1, 4>, pair_n3_kernel<false, 4, 2, 4, false, 1, 4>, 4, 4, "n3_r4_u2_w4b4_x2"},
    // degree-5 Ewald erfc (alpha rc <= kErfc5Xmax)
    {pair_n3_kernel<true, 4, 1, 3, false, 2, 8, false, kErfcH5>,
     pair_n3_kernel<false, 4, 1, 3, false, 2, 8, false, kErfcH5>, 4, 8, "n3_r4_u1_b3_x2l_p5", true},
    {pair_n3_kernel<true, 4, 2, 2, false, 1, 8, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 2, false, 1, 8, false, kErfcH5>, 4, 8, "n3_r4_u2_b2_x2_p5", true},
    {pair_n3_kernel<true, 4, 2, 5, false, 1, 4, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 5, false, 1, 4, false, kErfcH5>, 4, 4, "n3_r4_u2_w4b5_x2_p5", true},
    {pair_n3_kernel<true, 4, 2, 5, false, 2, 4, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 5, false, 2, 4, false, kErfcH5>, 4, 4, "n3_r4_u2_w4b5_x2l_p5", true},
    {pair_n3_kernel<true, 4, 2, 4, false, 1, 4, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 4, false, 1, 4, false, kErfcH5>, 4, 4, "n3_r4_u2_w4b4_x2_p5", true},
    {pair_n3_kernel<true, 4, 4, 4, false, 1, 4, false, kErfcH5>,
     pair_n3_kernel<false, 4, 4, 4, false, 1, 4, false, kErfcH5>, 4, 4, "n3_r4_u4_w4b4_x2_p5", true},
    {pair_n3_kernel<true, 6, 1, 4, false, 1, 4, false, kErfcH5>,
     pair_n3_kernel<false, 6, 1, 4, false, 1, 4, false, kErfcH5>, 6, 4, "n3_r6_u1_w4b4_x2_p5", true},
    {pair_n3_kernel<true, 6, 2, 3, false, 1, 4, false, kErfcH5>,
     pair_n3_kernel<false, 6, 2, 3, false, 1, 4, false, kErfcH5>, 6, 4, "n3_r6_u2_w4b3_x2_p5", true},
    // 2 warps per CTA: 256-particle i-tiles at the per-lane work of R = 4, so
    // that small systems end with a short tail
    {pair_n3_kernel<true, 4, 2, 8, false, 1, 2, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 8, false, 1, 2, false, kErfcH5>, 4, 2, "n3_r4_u2_w2b8_x2_p5", true},
    {pair_n3_kernel<true, 4, 2, 8, false, 2, 2, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 8, false, 2, 2, false, kErfcH5>, 4, 2, "n3_r4_u2_w2b8_x2l_p5", true},
    // one warp per CTA: 128-particle i-tiles, no cross-warp reaction sum
    {pair_n3_kernel<true, 4, 2, 16, false, 1, 1, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 16, false, 1, 1, false, kErfcH5>, 4, 1, "n3_r4_u2_w1b16_x2_p5", true},
    // the 2-warp form with the degree-6 erfc (any alpha rc)
    {pair_n3_kernel<true, 4, 2, 8, false, 1, 2>, pair_n3_kernel<false, 4, 2, 8, false, 1, 2>, 4, 2,
     "n3_r4_u2_w2b8_x2"},
    {pair_n3_kernel<true, 4, 4, 8, false, 1, 2, false, kErfcH5>,
     pair_n3_kernel<false, 4, 4, 8, false, 1, 2, false, kErfcH5>, 4, 2, "n3_r4_u4_w2b8_x2_p5", true},
};
constexpr int kN3Variants = sizeof(kVariants) / sizeof(kVariants[0]);

// Forms that also accumulate the RDF histograms (steps with TCP_FLAG_RDF,
// which the reference accumulates in every force call): the 2-warp form of
// the variants above with the degree-5 (0, the default where alpha rc allows
// it) or degree-6 (1, the default otherwise) erfc, and two 8-warp forms: RDF
// steps of 4.25 / 4.30 / 4.59 / 4.52 ms at N = 65,536; TCP_RDF_VARIANT=k picks
// one.
static const N3Variant kRdfVariants[] = {
    {pair_n3_kernel<true, 4, 2, 8, false, 1, 2, true, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 8, false, 1, 2, true, kErfcH5>, 4, 2, "n3_r4_u2_w2b8_x2_p5_rdf", true},
    {pair_n3_kernel<true, 4, 2, 8, false, 1, 2, true>, pair_n3_kernel<false, 4, 2, 8, false, 1, 2, true>, 4, 2,
     "n3_r4_u2_w2b8_x2_rdf"},
    {pair_n3_kernel<true, 4, 1, 3, false, 2, 8, true>, pair_n3_kernel<false, 4, 1, 3, false, 2, 8, true>, 4, 8,
     "n3_r4_u1_b3_x2l_rdf"},
    {pair_n3_kernel<true, 4, 1, 2, false, 1, 8, true>, pair_n3_kernel<false, 4, 1, 2, false, 1, 8, true>, 4, 8,
     "n3_r4_u1_b2_x2_rdf"},
};
constexpr int kN3RdfVariants = sizeof(kRdfVariants) / sizeof(kRdfVariants[0]);

int n3_variant_count() { return kN3Variants; }
bool n3_variant_usable(const tcp_ctx *c, int v) {
    return v >= 1 && v <= kN3Variants && (!kVariants[v - 1].erfc5 || c->pc.erfc5_ok);
}
const char *n3_variant_name(int v) { return v >= 1 && v <= kN3Variants ? kVariants[v - 1].name : "ordered"; }

int n3_grid_for(const tcp_ctx *c, int v) {
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kVariants[v - 1].energy, 32 * kVariants[v - 1].W, 0);
    return std::max(1, c->num_sms * std::max(1, bps));
}

static int kernel_grid(const tcp_ctx *c, N3Kernel k, int threads) {
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, threads, 0);
    return std::max(1, c->num_sms * std::max(1, bps));
}

int n3_grid(const tcp_ctx *c) {
    int g = 1;
    for (int v = 1; v <= kN3Variants; ++v) g = std::max(g, n3_grid_for(c, v));
    for (int v = 0; v < kN3RdfVariants; ++v) g = std::max(g, kernel_grid(c, kRdfVariants[v].energy, 32 * kRdfVariants[v].W));
    return g;
}

// Tile geometry of a system of nel + nion particles for i-tiles of `tile`.
N3Geom n3_geometry(int off, int nel, int nion, int tile, long long item0, long long *items) {
    N3Geom g;
    const int spt = tile / kN3Sub;
    g.off = off;
    g.nel = nel;
    g.n = nel + nion;
    g.nIe = cdiv(nel, tile);
    g.nI = g.nIe + cdiv(nion, tile);
    g.nSe = cdiv(nel, kN3Sub);
    g.nS = g.nSe + cdiv(nion, kN3Sub);
    g.item0 = item0;
    long long total = 0;
    for (int I = 0; I < g.nI; ++I) total += g.nS - (I < g.nIe ? I * spt : g.nSe + (I - g.nIe) * spt);
    *items = total;
    return g;
}

void n3_chunk_table(long long total, int ctas, std::vector<long long> &starts) {
    starts.assign(1, 0);
    const long long div = 2LL * std::max(1, ctas);
    for (long long at = 0; at < total;) {
        at += std::max(1LL, (total - at + div - 1) / div);
        starts.push_back(std::min(at, total));
    }
}

// Chunk tables of every i-tile size the variants use, in one device array
// (c->n3_chunks; c->n3_chunk_meta holds tile, items, offset, chunks per
// table).  Built on the host when the pair constants change, outside any
// stream capture, each for the largest persistent grid among the variants of
// that i-tile.
int n3_prepare_chunks(tcp_ctx *c) {
    std::vector<int> tiles;
    for (const N3Variant &v : kVariants) tiles.push_back(32 * v.R * v.W);
    for (const N3Variant &v : kRdfVariants) tiles.push_back(32 * v.R * v.W);
    std::sort(tiles.begin(), tiles.end());
    tiles.erase(std::unique(tiles.begin(), tiles.end()), tiles.end());
    std::vector<long long> all, meta, t;
    for (const int tile : tiles) {
        int ctas = 1;
        for (int v = 1; v <= kN3Variants; ++v)
            if (32 * kVariants[v - 1].R * kVariants[v - 1].W == tile) ctas = std::max(ctas, n3_grid_for(c, v));
        for (const N3Variant &v : kRdfVariants)
            if (32 * v.R * v.W == tile) ctas = std::max(ctas, kernel_grid(c, v.energy, 32 * v.W));
        long long total = 0;
        n3_geometry(0, c->nel, c->nion, tile, 0, &total);
        n3_chunk_table(total, ctas, t);
        meta.insert(meta.end(), {(long long)tile, total, (long long)all.size(), (long long)t.size() - 1});
        all.insert(all.end(), t.begin(), t.end());
    }
    if (c->n3_chunks) cudaFree(c->n3_chunks);
    c->n3_chunks = nullptr;
    TCP_CUDA(cudaMalloc(&c->n3_chunks, sizeof(long long) * all.size()));
    TCP_CUDA(cudaMemcpy(c->n3_chunks, all.data(), sizeof(long long) * all.size(), cudaMemcpyHostToDevice));
    c->n3_chunk_meta = meta;
    return TCP_OK;
}

// the arguments, grid and kernel of a rejoin launch (not yet pending)
static void n3_rejoin_set(N3Rejoin &r, const N3Args &a, int grid, int threads, const void *fn) {
    if (!r.args) r.args = new N3Args;
    *r.args = a;
    r.args->inject_skip = 0;
    r.grid = grid;
    r.threads = threads;
    r.fn = fn;
}

int launch_pair_n3(tcp_ctx *c, bool energy, bool rdf) {
    int rv = c->pc.erfc5_ok ? 0 : 1;   // the 2-warp forms: the fastest RDF steps measured
    if (const char *forced = getenv("TCP_RDF_VARIANT")) rv = std::min(std::max(atoi(forced), 0), kN3RdfVariants - 1);
    if (kRdfVariants[rv].erfc5 && !c->pc.erfc5_ok) rv = 1;
    const int v = std::min(std::max(c->pair_variant, 1), kN3Variants);
    const N3Variant &K = rdf ? kRdfVariants[rv] : kVariants[v - 1];
    const int tile = 32 * K.R * K.W;
    const int nt = 32 * K.W;
    N3Args a;
    std::memset(&a, 0, sizeof a);
    long long total = 0;
    a.g = n3_geometry(0, c->nel, c->nion, tile, 0, &total);
    a.xq = c->xq;
    a.total = total;
    for (size_t m = 0; m + 3 < c->n3_chunk_meta.size(); m += 4)
        if (c->n3_chunk_meta[m] == tile && c->n3_chunk_meta[m + 1] == total) {
            a.chunks = c->n3_chunks + c->n3_chunk_meta[m + 2];
            a.nchunks = (unsigned)c->n3_chunk_meta[m + 3];
        }
    if (!a.chunks) return set_error(TCP_ERR_STATE, "no Newton-3 chunk table for this geometry");
    a.ntot = c->n;
    a.facc = c->fpart;
    a.upart = c->upart;
    a.status = c->status;
    a.counter = c->counter;
    a.c = c->pc;
    a.inject_skip = inject_fault("tile_wait") ? 1 : 0;
    a.rdf = c->rdf;
    a.rdf_edges = c->rdf_edges;
    // CTAs left free for the reciprocal chain when it runs beside this launch;
    // they rejoin it after the chain (launch_pair_n3_rejoin)
    c->rejoin.pending = false;
    const int reserve = c->recip_beside ? c->pair_reserve : 0;
    const int full = rdf ? kernel_grid(c, K.energy, nt) : n3_grid_for(c, v);
    const int grid = (int)std::min<long long>(std::max(1, full - reserve), total);
    const int rejoin = (int)std::min<long long>(full - grid, total - grid);
    if (grid + std::max(rejoin, 0) > c->n_upart)
        return set_error(TCP_ERR_STATE, "energy partial buffer smaller than the Newton-3 grid");
    TCP_CUDA(cudaMemsetAsync(c->fpart, 0, sizeof(double) * 3 * (size_t)c->n, c->stream));
    TCP_CUDA(cudaMemsetAsync(c->counter, 0, sizeof(unsigned), c->stream));
    if (energy) TCP_CUDA(cudaMemsetAsync(c->upart, 0, sizeof(double) * (size_t)c->n_upart, c->stream));
    if (rejoin > 0) {
        TCP_CUDA(cudaEventRecord(c->ev_pair_ready, c->stream));
        N3Args r = a;
        r.upart = c->upart + grid;   // its CTAs' energy partials follow the first launch's
        n3_rejoin_set(c->rejoin, r, rejoin, nt, reinterpret_cast<const void *>(energy ? K.energy : K.plain));
    }
    if (energy)
        K.energy<<<grid, nt, 0, c->stream>>>(a);
    else
        K.plain<<<grid, nt, 0, c->stream>>>(a);
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    c->rejoin.pending = rejoin > 0;
    return TCP_OK;
}

// The CTAs a Newton-3 launch left to the reciprocal chain, launched on the
// chain's stream after it: the same kernel and arguments, claiming whatever
// chunks remain from the shared counter (none if the first launch has taken
// them all, and its CTAs then leave at once).  It waits for the clearing of
// the counter and accumulators that preceded the first launch.
int n3_rejoin_launch(N3Rejoin &r, cudaStream_t st, cudaEvent_t ready, long long *launches) {
    if (!r.pending) return TCP_OK;
    r.pending = false;
    TCP_CUDA(cudaStreamWaitEvent(st, ready, 0));
    void *args[] = {r.args};
    TCP_CUDA(cudaLaunchKernel(r.fn, dim3(r.grid), dim3(r.threads), args, 0, st));
    if (launches) ++*launches;
    return TCP_OK;
}

int launch_pair_n3_rejoin(tcp_ctx *c, cudaStream_t st) {
    return n3_rejoin_launch(c->rejoin, st, c->ev_pair_ready, &c->launches);
}

void n3_rejoin_free(N3Rejoin &r) {
    delete r.args;
    r.args = nullptr;
    r.pending = false;
}

void n3_free(tcp_ctx *c) { n3_rejoin_free(c->rejoin); }

// ---- batch of replicas -------------------------------------------------------
// Variants of the batched launch (the batch autotuner picks one per batch):
// i-particles per lane x packed FP32 x CTAs per SM.
struct N3BatchVariant {
    N3Kernel energy, plain;
    int R, W;
    const char *name;
    bool erfc5 = false;   // degree-5 Ewald erfc: only where every replica's alpha rc allows it
};
static const N3BatchVariant kBatchVariants[] = {
    {pair_n3_kernel<true, 2, 2, 2, true>, pair_n3_kernel<false, 2, 2, 2, true>, 2, 8, "b_r2_u2_b2"},
    {pair_n3_kernel<true, 4, 1, 2, true, 1>, pair_n3_kernel<false, 4, 1, 2, true, 1>, 4, 8, "b_r4_u1_b2_x2"},
    {pair_n3_kernel<true, 2, 2, 3, true, 1>, pair_n3_kernel<false, 2, 2, 3, true, 1>, 2, 8, "b_r2_u2_b3_x2"},
    {pair_n3_kernel<true, 4, 1, 3, true, 1>, pair_n3_kernel<false, 4, 1, 3, true, 1>, 4, 8, "b_r4_u1_b3_x2"},
    {pair_n3_kernel<true, 4, 1, 3, true, 2>, pair_n3_kernel<false, 4, 1, 3, true, 2>, 4, 8, "b_r4_u1_b3_x2l"},
    {pair_n3_kernel<true, 2, 2, 3, true, 2>, pair_n3_kernel<false, 2, 2, 3, true, 2>, 2, 8, "b_r2_u2_b3_x2l"},
    {pair_n3_kernel<true, 2, 2, 6, true, 2, 4>, pair_n3_kernel<false, 2, 2, 6, true, 2, 4>, 2, 4, "b_r2_u2_w4b6_x2l"},
    {pair_n3_kernel<true, 4, 1, 6, true, 2, 4>, pair_n3_kernel<false, 4, 1, 6, true, 2, 4>, 4, 4, "b_r4_u1_w4b6_x2l"},
    // 1- and 2-warp CTAs: 128- and 256-particle i-tiles
    {pair_n3_kernel<true, 4, 2, 8, true, 1, 2>, pair_n3_kernel<false, 4, 2, 8, true, 1, 2>, 4, 2, "b_r4_u2_w2b8_x2"},
    {pair_n3_kernel<true, 2, 2, 12, true, 2, 2>, pair_n3_kernel<false, 2, 2, 12, true, 2, 2>, 2, 2,
     "b_r2_u2_w2b12_x2l"},
    {pair_n3_kernel<true, 2, 2, 12, true, 1, 2>, pair_n3_kernel<false, 2, 2, 12, true, 1, 2>, 2, 2,
     "b_r2_u2_w2b12_x2"},
    {pair_n3_kernel<true, 4, 2, 16, true, 1, 1>, pair_n3_kernel<false, 4, 2, 16, true, 1, 1>, 4, 1, "b_r4_u2_w1b16_x2"},
    // the degree-5 Ewald erfc (every replica with alpha rc <= kErfc5Xmax)
    {pair_n3_kernel<true, 2, 2, 12, true, 2, 2, false, kErfcH5>,
     pair_n3_kernel<false, 2, 2, 12, true, 2, 2, false, kErfcH5>, 2, 2, "b_r2_u2_w2b12_x2l_p5", true},
    {pair_n3_kernel<true, 4, 2, 8, true, 1, 2, false, kErfcH5>,
     pair_n3_kernel<false, 4, 2, 8, true, 1, 2, false, kErfcH5>, 4, 2, "b_r4_u2_w2b8_x2_p5", true},
};
constexpr int kN3BatchVariants = sizeof(kBatchVariants) / sizeof(kBatchVariants[0]);

int n3_batch_variant_count() { return kN3BatchVariants; }
bool n3_batch_variant_erfc5(int v) { return kBatchVariants[std::min(std::max(v, 0), kN3BatchVariants - 1)].erfc5; }
const char *n3_batch_variant_name(int v) { return kBatchVariants[std::min(std::max(v, 0), kN3BatchVariants - 1)].name; }
int n3_batch_tile(int v) {
    const N3BatchVariant &k = kBatchVariants[std::min(std::max(v, 0), kN3BatchVariants - 1)];
    return 32 * k.R * k.W;
}
size_t n3_rep_bytes() { return sizeof(N3Rep); }

// Fills reps (host) for replicas with the given offsets/counts/constants and
// the i-tile of the variant.
long long n3_batch_fill(void *reps_host, int nrep, const int *off, const int *nel, const int *nion,
                        const PairConsts *pc, int tile) {
    N3Rep *r = static_cast<N3Rep *>(reps_host);
    long long item0 = 0;
    for (int k = 0; k < nrep; ++k) {
        long long items = 0;
        r[k].g = n3_geometry(off[k], nel[k], nion[k], tile, item0, &items);
        r[k].c = pc[k];
        item0 += items;
    }
    return item0;
}

static int n3_batch_grid(int num_sms, int v) {
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kBatchVariants[v].energy, 32 * kBatchVariants[v].W, 0);
    return std::max(1, num_sms * std::max(1, bps));
}

int n3_batch_ctas(int num_sms, int v) { return n3_batch_grid(num_sms, std::min(std::max(v, 0), kN3BatchVariants - 1)); }

int launch_pair_n3_batch(cudaStream_t st, const int4 *xq, int ntot, double *facc, const void *reps_dev, int nrep,
                         long long total, const long long *chunks, unsigned nchunks, double *ur_rep, unsigned *status,
                         unsigned *counter, int num_sms, bool energy, int variant, int reserve, N3Rejoin *rejoin,
                         cudaEvent_t ready) {
    const int v = std::min(std::max(variant, 0), kN3BatchVariants - 1);
    N3Args a;
    std::memset(&a, 0, sizeof a);
    a.xq = xq;
    a.total = total;
    a.chunks = chunks;
    a.nchunks = nchunks;
    a.ntot = ntot;
    a.facc = facc;
    a.status = status;
    a.counter = counter;
    a.reps = static_cast<const N3Rep *>(reps_dev);
    a.nrep = nrep;
    a.ur_rep = ur_rep;
    const int full = n3_batch_grid(num_sms, v);
    if (rejoin) rejoin->pending = false;
    const int res = rejoin && ready ? std::max(reserve, 0) : 0;
    const int grid = (int)std::min<long long>(std::max(1, full - res), total);
    const int extra = (int)std::min<long long>(full - grid, total - grid);   // rejoin CTAs
    const int nt = 32 * kBatchVariants[v].W;
    TCP_CUDA(cudaMemsetAsync(facc, 0, sizeof(double) * 3 * (size_t)ntot, st));
    TCP_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    if (energy) TCP_CUDA(cudaMemsetAsync(ur_rep, 0, sizeof(double) * (size_t)nrep, st));
    if (res > 0 && extra > 0) {   // the batched kernels add Ur per replica by atomics
        TCP_CUDA(cudaEventRecord(ready, st));
        n3_rejoin_set(*rejoin, a, extra, nt,
                      reinterpret_cast<const void *>(energy ? kBatchVariants[v].energy : kBatchVariants[v].plain));
    }
    if (energy)
        kBatchVariants[v].energy<<<grid, nt, 0, st>>>(a);
    else
        kBatchVariants[v].plain<<<grid, nt, 0, st>>>(a);
    TCP_CUDA(cudaGetLastError());
    if (rejoin) rejoin->pending = res > 0 && extra > 0;
    return TCP_OK;
}

}  // namespace tcp

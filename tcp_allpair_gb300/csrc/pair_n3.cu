// pair_n3.cu -- the compensated-FP32 real-space sum with Newton's third law:
// every unique pair (i < j) is evaluated once and its force is added to both
// particles (Force_direct_self / _ext / _sum of force.f90:52-372, whose
// triangular loops also evaluate each pair once).
//
// Work: particles are split per species into i-tiles of kN3Tile = 512 and
// j-subtiles of kN3Sub = 128 (tiles never straddle the e/i boundary).  An
// item is (i-tile I, j-subtile S) with S at or after I's first subtile; items
// are enumerated row by row and a persistent grid splits the list evenly (each
// CTA a contiguous range), so the triangular work is balanced to one item.
//
// CTA = 8 warps; a lane holds two i-particles (i-chunks of 32 at warp*64 and
// warp*64+32).  A j-subtile is copied into shared memory by the bulk-copy
// engine (cp.async.bulk + mbarrier, kN3Stages-deep ring, prefetched across
// items).  Each warp takes the subtile in chunks of 32: lane l loads j = l,
// and for 32 steps computes the pairs (i_A, j) and (i_B, j) and rotates j's
// position and reaction accumulator to the next lane with shuffles, so after
// 32 steps every lane holds the reaction of its own j again.  Reactions are
// summed over the warps in shared memory and added to the global FP64 force
// with one atomic per j and component per item; i-forces are folded per item
// into TwoSum (hi, lo) accumulators and added with atomics when the CTA
// leaves the row.  Subtiles inside the i-tile (the diagonal) and partial tiles
// use an index mask i < j; all others run unmasked except for the cut-off.
//
// Pair arithmetic is that of pair_fp32c_kernel (fixed-point differences in
// units of L/2^32, SFU rsqrt/rcp/ex2, erfc = exp(-x^2) t Q(t)).  Cubic boxes
// only; other boxes use the ordered-pair kernel.
#include <algorithm>

#include "device_util.cuh"
#include "pair_math.cuh"
#include "tcp_internal.h"

namespace tcp {

constexpr int kN3Warps = 8;
constexpr int kN3Threads = 32 * kN3Warps;
constexpr int kN3Tile = 64 * kN3Warps;     // i-particles per CTA (2 per lane)
constexpr int kN3Sub = 128;                // j-subtile
constexpr int kN3SubPerTile = kN3Tile / kN3Sub;
constexpr int kN3Stages = 3;

struct N3Args {
    const int4 *xq;
    int nel, n;
    int nIe, nI;          // i-tiles, electron tiles first
    int nSe, nS;          // j-subtiles, electron subtiles first
    long long total;      // items
    double *facc;         // [3][n], zeroed before the launch
    double *upart;        // [gridDim.x]
    unsigned *status;
    PairConsts c;
};

__device__ __forceinline__ void n3_itile(const N3Args &a, int I, int &start, int &end, int &sp, int &first) {
    if (I < a.nIe) {
        sp = 0;
        start = I * kN3Tile;
        end = min(start + kN3Tile, a.nel);
        first = I * kN3SubPerTile;
    } else {
        sp = 1;
        start = a.nel + (I - a.nIe) * kN3Tile;
        end = min(start + kN3Tile, a.n);
        first = a.nSe + (I - a.nIe) * kN3SubPerTile;
    }
}

__device__ __forceinline__ void n3_sub(const N3Args &a, int S, int &start, int &cnt, int &sp) {
    if (S < a.nSe) {
        sp = 0;
        start = S * kN3Sub;
        cnt = min(kN3Sub, a.nel - start);
    } else {
        sp = 1;
        start = a.nel + (S - a.nSe) * kN3Sub;
        cnt = min(kN3Sub, a.n - start);
    }
}

// first item of row I
__device__ __forceinline__ void n3_advance(const N3Args &a, int &I, int &S) {
    if (++S == a.nS) {
        ++I;
        int st, en, sp, first;
        if (I < a.nI) {
            n3_itile(a, I, st, en, sp, first);
            S = first;
        }
    }
}

// One pair in units of u = L/2^32.  Returns the force weight w (force on i is
// eps qq/u^2 * w * d) and, with ENERGY, adds the energy term / r to pe.
//   er = erfc(ar)/r is shared by the energy and by
//   w  = [erfc(ar)/r + 2a/sqrt(pi) exp(-a^2r^2) (- e-i terms)] / r^2.
// KIND 2 (Kelbg) adds its Gaussian terms only when `near_any` (a warp vote
// taken by the caller for both i-particles of the lane) is set.
template <int KIND, bool ENERGY>
__device__ __forceinline__ float n3_pair(const PairConsts &c, float r2, bool ok, bool near_any, float &pe) {
    const float rinv = rsqrt_approx(r2);
    const float r = r2 * rinv;
    const float t = rcp_approx(fmaf(c.u_p_alpha, r, 1.0f));
    const float e = ex2_approx(c.u_c_exp * r2);
    const float er = (e * erfc_poly(t)) * rinv;          // erfc(ar)/r
    float s = fmaf(c.u_c_gauss, e, er);                   // (erfc(ar) + 2ar/sqrt(pi) e^{-a^2r^2}) / r
    float u = er;
    if (KIND == 1) {                                      // Deutsch, force.f90:136-139
        const float y = ex2_approx(c.u_c_rs * r);         // exp(-r/rs)
        s = fmaf(-y, rinv + c.u_inv_rs, s);
        if (ENERGY) u = fmaf(-y, rinv, u);
    }
    if (KIND == 2 && near_any) {                          // Kelbg
        const bool near = ok && (r2 < c.u_rshort2);
        const float g = near ? ex2_approx(c.u_c_lam * r2) : 0.0f;   // exp(-r^2/lambda^2)
        s = fmaf(-g, rinv, s);
        if (ENERGY) {
            const float t2 = rcp_approx(fmaf(c.u_p_lam, r, 1.0f));
            const float erfc_rl = g * erfc_poly(t2);      // erfc(r/lambda)
            u += fmaf(c.u_sqrtpi_lam, erfc_rl, -g * rinv);
        }
    }
    if (ENERGY) pe += ok ? u : 0.0f;
    const float w = s * (rinv * rinv);
    return ok ? w : 0.0f;
}

// One item: the two i-particles of this lane against a j-subtile in shared
// memory.  MASKED: apply validity and i < j index masks.
template <int KIND, bool ENERGY, bool MASKED, int UNROLL>
__device__ __forceinline__ void n3_item(const PairConsts &c, const int4 *__restrict__ tj, int cnt, int jstart,
                                        int4 xa, int4 xb, int ia, int ib, bool va, bool vb, float (*sjacc)[3],
                                        float &pax, float &pay, float &paz, float &pbx, float &pby, float &pbz,
                                        float &pe) {
    const int lane = threadIdx.x & 31;
    const int src = (lane + 1) & 31;
    for (int ch = 0; ch * 32 < cnt; ++ch) {
        int4 xj = tj[ch * 32 + lane];
        float jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll UNROLL
        for (int s = 0; s < 32; ++s) {
            bool oka = true, okb = true;
            if (MASKED) {
                const int jo = ch * 32 + ((lane + s) & 31);
                const bool jv = jo < cnt;
                const int jidx = jstart + jo;
                oka = va && jv && (ia < jidx);
                okb = vb && jv && (ib < jidx);
            }
            const float dax = (float)(xa.x - xj.x), day = (float)(xa.y - xj.y), daz = (float)(xa.z - xj.z);
            const float dbx = (float)(xb.x - xj.x), dby = (float)(xb.y - xj.y), dbz = (float)(xb.z - xj.z);
            const float r2a = fmaf(dax, dax, fmaf(day, day, daz * daz));
            const float r2b = fmaf(dbx, dbx, fmaf(dby, dby, dbz * dbz));
            oka = oka && (r2a < c.u_rc2);
            okb = okb && (r2b < c.u_rc2);
            bool near_any = false;
            if (KIND == 2)
                near_any = __any_sync(0xffffffffu, (oka && r2a < c.u_rshort2) || (okb && r2b < c.u_rshort2));
            const float wa = n3_pair<KIND, ENERGY>(c, r2a, oka, near_any, pe);
            const float wb = n3_pair<KIND, ENERGY>(c, r2b, okb, near_any, pe);
            pax = fmaf(wa, dax, pax);
            pay = fmaf(wa, day, pay);
            paz = fmaf(wa, daz, paz);
            pbx = fmaf(wb, dbx, pbx);
            pby = fmaf(wb, dby, pby);
            pbz = fmaf(wb, dbz, pbz);
            jx = fmaf(wb, dbx, fmaf(wa, dax, jx));
            jy = fmaf(wb, dby, fmaf(wa, day, jy));
            jz = fmaf(wb, dbz, fmaf(wa, daz, jz));
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

template <bool ENERGY, int UNROLL, int MINB>
__global__ void __launch_bounds__(kN3Threads, MINB) pair_n3_kernel(const N3Args a) {
    __shared__ __align__(128) int4 tiles[kN3Stages][kN3Sub];
    __shared__ __align__(8) uint64_t bars[kN3Stages];
    __shared__ float sjacc[kN3Sub][3];
    __shared__ double red[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    const long long it0 = a.total * (long long)blockIdx.x / gridDim.x;
    const long long it1 = a.total * (long long)(blockIdx.x + 1) / gridDim.x;
    const int nitems = (int)(it1 - it0);

    // locate the first item: row I and subtile S
    int I = 0, S = 0;
    {
        long long acc = 0;
        int st, en, sp, first;
        for (I = 0; I < a.nI; ++I) {
            n3_itile(a, I, st, en, sp, first);
            const long long len = a.nS - first;
            if (it0 < acc + len) {
                S = first + (int)(it0 - acc);
                break;
            }
            acc += len;
        }
    }
    for (int k = tid; k < kN3Sub * 3; k += kN3Threads) (&sjacc[0][0])[k] = 0.f;
    if (tid == 0) {
        for (int s = 0; s < kN3Stages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // producer cursor (thread 0 only)
    int pI = I, pS = S;
    if (tid == 0) {
        for (int k = 0; k < min(kN3Stages, nitems); ++k) {
            int js, jc, jsp;
            n3_sub(a, pS, js, jc, jsp);
            const uint32_t bytes = (uint32_t)jc * sizeof(int4);
            mbar_arrive_expect_tx(&bars[k], bytes);
            bulk_g2s(tiles[k], a.xq + js, bytes, &bars[k]);
            n3_advance(a, pI, pS);
        }
    }

    double etot = 0.0;
    int curI = -1, istart = 0, iend = 0, isp = 0, ifirst = 0;
    int ia = 0, ib = 0;
    bool va = false, vb = false;
    int4 xa = make_int4(0, 0, 0, 0), xb = xa;
    float hax = 0.f, lax = 0.f, hay = 0.f, lay = 0.f, haz = 0.f, laz = 0.f;
    float hbx = 0.f, lbx = 0.f, hby = 0.f, lby = 0.f, hbz = 0.f, lbz = 0.f;
    float eh = 0.f, el = 0.f;

    auto flush_i = [&]() {
        if (curI < 0) return;
        if (va) {
            atomicAdd(&a.facc[ia], kEps * ((double)hax + (double)lax));
            atomicAdd(&a.facc[(size_t)a.n + ia], kEps * ((double)hay + (double)lay));
            atomicAdd(&a.facc[2 * (size_t)a.n + ia], kEps * ((double)haz + (double)laz));
        }
        if (vb) {
            atomicAdd(&a.facc[ib], kEps * ((double)hbx + (double)lbx));
            atomicAdd(&a.facc[(size_t)a.n + ib], kEps * ((double)hby + (double)lby));
            atomicAdd(&a.facc[2 * (size_t)a.n + ib], kEps * ((double)hbz + (double)lbz));
        }
        etot += (double)eh + (double)el;
        hax = lax = hay = lay = haz = laz = 0.f;
        hbx = lbx = hby = lby = hbz = lbz = 0.f;
        eh = el = 0.f;
    };

    int k = 0;
    for (; k < nitems; ++k) {
        if (I != curI) {
            flush_i();
            curI = I;
            n3_itile(a, I, istart, iend, isp, ifirst);
            ia = istart + warp * 64 + lane;
            ib = ia + 32;
            va = ia < iend;
            vb = ib < iend;
            xa = a.xq[va ? ia : istart];
            xb = a.xq[vb ? ib : istart];
        }
        int jstart, cnt, jsp;
        n3_sub(a, S, jstart, cnt, jsp);
        const int pt = isp + jsp;
        const bool masked = (S < ifirst + kN3SubPerTile && jsp == isp) || cnt < kN3Sub || (iend - istart) < kN3Tile;
        const int stage = k % kN3Stages;
        const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / kN3Stages) & 1), kWaitLimitCycles);
        float pax = 0.f, pay = 0.f, paz = 0.f, pbx = 0.f, pby = 0.f, pbz = 0.f, pe = 0.f;
        const int kind = pt == 1 ? (a.c.ei_model == TCP_EI_DEUTSCH ? 1 : (a.c.ei_model == TCP_EI_KELBG ? 2 : 0)) : 0;
#define TCP_N3_ITEM(KIND, MASKED)                                                                             \
    n3_item<KIND, ENERGY, MASKED, UNROLL>(a.c, tiles[stage], cnt, jstart, xa, xb, ia, ib, va, vb, sjacc, pax, pay, paz, \
                                  pbx, pby, pbz, pe)
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
        const float qf = a.c.u_qq_force[pt];
        acc2(hax, lax, pax * qf);
        acc2(hay, lay, pay * qf);
        acc2(haz, laz, paz * qf);
        acc2(hbx, lbx, pbx * qf);
        acc2(hby, lby, pby * qf);
        acc2(hbz, lbz, pbz * qf);
        if (ENERGY) acc2(eh, el, pe * a.c.u_qq_energy[pt]);
        // all warps done with this subtile and its reaction sums
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(a.status, kStatusTmaTimeout);
            break;
        }
        if (tid < cnt) {
            const double sc = -kEps * (double)qf;
            atomicAdd(&a.facc[jstart + tid], sc * (double)sjacc[tid][0]);
            atomicAdd(&a.facc[(size_t)a.n + jstart + tid], sc * (double)sjacc[tid][1]);
            atomicAdd(&a.facc[2 * (size_t)a.n + jstart + tid], sc * (double)sjacc[tid][2]);
        }
        if (tid < kN3Sub) sjacc[tid][0] = sjacc[tid][1] = sjacc[tid][2] = 0.f;
        if (tid == 0 && k + kN3Stages < nitems) {
            int js, jc, jsp2;
            n3_sub(a, pS, js, jc, jsp2);
            const uint32_t bytes = (uint32_t)jc * sizeof(int4);
            mbar_arrive_expect_tx(&bars[stage], bytes);
            bulk_g2s(tiles[stage], a.xq + js, bytes, &bars[stage]);
            n3_advance(a, pI, pS);
        }
        __syncthreads();
        n3_advance(a, I, S);
    }
    if (k < nitems) {
        if (tid == 0)
            for (int kk = k; kk < min(nitems, k + kN3Stages); ++kk)
                mbar_wait_bounded(&bars[kk % kN3Stages], (uint32_t)((kk / kN3Stages) & 1), kWaitLimitCycles);
        __syncthreads();
        return;
    }
    flush_i();
    if (ENERGY) {
        const double tot = block_sum(etot, red);
        if (tid == 0) a.upart[blockIdx.x] = tot;
    }
}

// ---------------------------------------------------------------------------
static int cdiv(int x, int y) { return (x + y - 1) / y; }

bool n3_applicable(const tcp_ctx *c) {
    return c->p.precision == TCP_PREC_FP32C && c->pc.cubic && c->n >= 2 && c->pair_variant > 0;
}

// Variants: 1..kN3Variants (index - 1 into the table below); 0 = ordered-pair kernel.
typedef void (*N3Kernel)(const N3Args);
struct N3Variant {
    N3Kernel energy, plain;
    const char *name;
};
static const N3Variant kVariants[] = {
    {pair_n3_kernel<true, 2, 3>, pair_n3_kernel<false, 2, 3>, "n3_u2_b3"},
    {pair_n3_kernel<true, 4, 3>, pair_n3_kernel<false, 4, 3>, "n3_u4_b3"},
    {pair_n3_kernel<true, 2, 4>, pair_n3_kernel<false, 2, 4>, "n3_u2_b4"},
    {pair_n3_kernel<true, 1, 4>, pair_n3_kernel<false, 1, 4>, "n3_u1_b4"},
};
constexpr int kN3Variants = sizeof(kVariants) / sizeof(kVariants[0]);

int n3_variant_count() { return kN3Variants; }
const char *n3_variant_name(int v) { return v >= 1 && v <= kN3Variants ? kVariants[v - 1].name : "ordered"; }

int n3_grid_for(const tcp_ctx *c, int v) {
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kVariants[v - 1].energy, kN3Threads, 0);
    return std::max(1, c->num_sms * std::max(1, bps));
}

int n3_grid(const tcp_ctx *c) {
    int g = 1;
    for (int v = 1; v <= kN3Variants; ++v) g = std::max(g, n3_grid_for(c, v));
    return g;
}

int launch_pair_n3(tcp_ctx *c, bool energy) {
    N3Args a;
    a.xq = c->xq;
    a.nel = c->nel;
    a.n = c->n;
    a.nIe = cdiv(c->nel, kN3Tile);
    a.nI = a.nIe + cdiv(c->nion, kN3Tile);
    a.nSe = cdiv(c->nel, kN3Sub);
    a.nS = a.nSe + cdiv(c->nion, kN3Sub);
    long long total = 0;
    for (int I = 0; I < a.nI; ++I) {
        const int first = I < a.nIe ? I * kN3SubPerTile : a.nSe + (I - a.nIe) * kN3SubPerTile;
        total += a.nS - first;
    }
    a.total = total;
    a.facc = c->fpart;
    a.upart = c->upart;
    a.status = c->status;
    a.c = c->pc;
    const int v = std::min(std::max(c->pair_variant, 1), kN3Variants);
    const int grid = (int)std::min<long long>(n3_grid_for(c, v), total);
    if (grid > c->n_upart) return set_error(TCP_ERR_STATE, "energy partial buffer smaller than the Newton-3 grid");
    TCP_CUDA(cudaMemsetAsync(c->fpart, 0, sizeof(double) * 3 * (size_t)c->n, c->stream));
    if (energy) {
        TCP_CUDA(cudaMemsetAsync(c->upart, 0, sizeof(double) * (size_t)c->n_upart, c->stream));
        kVariants[v - 1].energy<<<grid, kN3Threads, 0, c->stream>>>(a);
    } else {
        kVariants[v - 1].plain<<<grid, kN3Threads, 0, c->stream>>>(a);
    }
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

}  // namespace tcp

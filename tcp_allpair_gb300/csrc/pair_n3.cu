// pair_n3.cu -- the compensated-FP32 real-space sum with Newton's third law:
// every unique pair (i < j) is evaluated once and its force is added to both
// particles (Force_direct_self / _ext / _sum of force.f90:52-372, whose
// triangular loops also evaluate each pair once).
//
// Work: particles are split per species into i-tiles of TILE = 32 R W
// particles (W warps, R i-particles per lane) and j-subtiles of kN3Sub = 128
// (tiles never straddle the e/i boundary).  An item is (i-tile I, j-subtile
// S) with S at or after I's first subtile; items are enumerated row by row.
// A persistent grid takes the first ~90 % of the list in equal contiguous
// shares (the i-tile stays in registers along a row) and the rest one item
// at a time from an atomic counter, which absorbs the cost differences
// between items (pair types, masked items).
//
// A lane holds R i-particles (R i-chunks of 32 per warp).  A j-subtile is
// copied into shared memory by the bulk-copy engine (cp.async.bulk +
// mbarrier, kN3Stages-deep ring, prefetched along the static share).  Each
// warp takes the subtile in chunks of 32: lane l loads j = l, and for 32
// steps computes the R pairs (i_r, j) and rotates j's position and reaction
// accumulator to the next lane with shuffles, so after 32 steps every lane
// holds the reaction of its own j again.  Reactions are summed over the
// warps in shared memory and added to the global FP64 force with one atomic
// per j and component per item; i-forces are folded per item into TwoSum
// (hi, lo) accumulators and added with atomics when the CTA leaves the row.
// Subtiles inside the i-tile (the diagonal) and partial tiles use an index
// mask i < j; all others run unmasked except for the cut-off.
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
constexpr int kN3Sub = 128;                // j-subtile
constexpr int kN3Stages = 3;
constexpr int kN3DynPercent = 10;          // share of the items handed out dynamically

struct N3Args {
    const int4 *xq;
    int nel, n;
    int nIe, nI;          // i-tiles, electron tiles first
    int nSe, nS;          // j-subtiles, electron subtiles first
    long long total;      // items
    long long nstatic;    // items [0, nstatic) split statically
    double *facc;         // [3][n], zeroed before the launch
    double *upart;        // [gridDim.x]
    unsigned *status;
    unsigned *counter;    // dynamic item counter, zeroed before the launch
    PairConsts c;
};

template <int TILE>
__device__ __forceinline__ void n3_itile(const N3Args &a, int I, int &start, int &end, int &sp, int &first) {
    constexpr int SPT = TILE / kN3Sub;
    if (I < a.nIe) {
        sp = 0;
        start = I * TILE;
        end = min(start + TILE, a.nel);
        first = I * SPT;
    } else {
        sp = 1;
        start = a.nel + (I - a.nIe) * TILE;
        end = min(start + TILE, a.n);
        first = a.nSe + (I - a.nIe) * SPT;
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

// item index -> (row I, subtile S)
template <int TILE>
__device__ __forceinline__ void n3_decode(const N3Args &a, long long it, int &I, int &S) {
    long long acc = 0;
    int st, en, sp, first;
    for (I = 0; I < a.nI; ++I) {
        n3_itile<TILE>(a, I, st, en, sp, first);
        const long long len = a.nS - first;
        if (it < acc + len) {
            S = first + (int)(it - acc);
            return;
        }
        acc += len;
    }
    S = a.nS;
}

template <int TILE>
__device__ __forceinline__ void n3_advance(const N3Args &a, int &I, int &S) {
    if (++S == a.nS) {
        ++I;
        int st, en, sp, first;
        if (I < a.nI) {
            n3_itile<TILE>(a, I, st, en, sp, first);
            S = first;
        }
    }
}

// One pair in units of u = L/2^32.  Returns the force weight w (force on i is
// eps qq/u^2 * w * d) and, with ENERGY, adds the energy term / r to pe.
//   er = erfc(ar)/r is shared by the energy and by
//   w  = [erfc(ar)/r + 2a/sqrt(pi) exp(-a^2r^2) (- e-i terms)] / r^2.
// KIND 2 (Kelbg) adds its Gaussian terms only when `near_any` (a warp vote
// taken by the caller for all i-particles of the lane) is set.
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

// One item: the R i-particles of this lane against a j-subtile in shared
// memory.  MASKED: apply validity and i < j index masks.
template <int KIND, bool ENERGY, bool MASKED, int UNROLL, int R>
__device__ __forceinline__ void n3_item(const PairConsts &c, const int4 *__restrict__ tj, int cnt, int jstart,
                                        const int4 (&xi)[R], const int (&ii)[R], const bool (&vi)[R],
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
                    ok[r] = ok[r] && vi[r] && (jo < cnt) && (ii[r] < jstart + jo);
                }
                if (KIND == 2) r2min = fminf(r2min, r2[r]);
            }
            // a vote without the masks: a false positive only runs the branch
            bool near_any = false;
            if (KIND == 2) near_any = __any_sync(0xffffffffu, r2min < c.u_rshort2);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float w = n3_pair<KIND, ENERGY>(c, r2[r], ok[r], near_any, pe);
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

template <bool ENERGY, int R, int UNROLL, int MINB>
__global__ void __launch_bounds__(kN3Threads, MINB) pair_n3_kernel(const N3Args a) {
    constexpr int TILE = 32 * R * kN3Warps;
    constexpr int SPT = TILE / kN3Sub;
    __shared__ __align__(128) int4 tiles[kN3Stages][kN3Sub];
    __shared__ __align__(8) uint64_t bars[kN3Stages];
    __shared__ float sjacc[kN3Sub][3];
    __shared__ double red[32];
    __shared__ long long s_next;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    const long long it0 = a.nstatic * (long long)blockIdx.x / gridDim.x;
    const long long it1 = a.nstatic * (long long)(blockIdx.x + 1) / gridDim.x;
    const int nst = (int)(it1 - it0);

    for (int k = tid; k < kN3Sub * 3; k += kN3Threads) (&sjacc[0][0])[k] = 0.f;
    if (tid == 0) {
        for (int s = 0; s < kN3Stages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    int I = 0, S = 0;
    if (nst > 0) n3_decode<TILE>(a, it0, I, S);
    int pI = I, pS = S;   // producer cursor (thread 0)
    auto issue = [&](int stage, int si) {
        int js, jc, jsp;
        n3_sub(a, si, js, jc, jsp);
        const uint32_t bytes = (uint32_t)jc * sizeof(int4);
        mbar_arrive_expect_tx(&bars[stage], bytes);
        bulk_g2s(tiles[stage], a.xq + js, bytes, &bars[stage]);
    };
    if (tid == 0)
        for (int k = 0; k < min(kN3Stages, nst); ++k) {
            issue(k, pS);
            n3_advance<TILE>(a, pI, pS);
        }

    double etot = 0.0;
    int curI = -1, istart = 0, iend = 0, isp = 0, ifirst = 0;
    int4 xi[R];
    int ii[R];
    bool vi[R];
    float hi[R][3], lo[R][3];
    float eh = 0.f, el = 0.f;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        xi[r] = make_int4(0, 0, 0, 0);
        ii[r] = 0;
        vi[r] = false;
        hi[r][0] = hi[r][1] = hi[r][2] = lo[r][0] = lo[r][1] = lo[r][2] = 0.f;
    }

    auto flush_i = [&]() {
        if (curI < 0) return;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (vi[r])
                for (int k = 0; k < 3; ++k)
                    atomicAdd(&a.facc[(size_t)k * a.n + ii[r]], kEps * ((double)hi[r][k] + (double)lo[r][k]));
            hi[r][0] = hi[r][1] = hi[r][2] = lo[r][0] = lo[r][1] = lo[r][2] = 0.f;
        }
        etot += (double)eh + (double)el;
        eh = el = 0.f;
    };

    // process item k (ring stage k % kN3Stages) of row I_, subtile S_; false on timeout
    auto process = [&](int k, int I_, int S_) -> bool {
        if (I_ != curI) {
            flush_i();
            curI = I_;
            n3_itile<TILE>(a, I_, istart, iend, isp, ifirst);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                ii[r] = istart + warp * 32 * R + r * 32 + lane;
                vi[r] = ii[r] < iend;
                xi[r] = a.xq[vi[r] ? ii[r] : istart];
            }
        }
        int jstart, cnt, jsp;
        n3_sub(a, S_, jstart, cnt, jsp);
        const int pt = isp + jsp;
        const bool masked = (S_ < ifirst + SPT && jsp == isp) || cnt < kN3Sub || (iend - istart) < TILE;
        const int stage = k % kN3Stages;
        const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / kN3Stages) & 1), kWaitLimitCycles);
        float p[R][3], pe = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r) p[r][0] = p[r][1] = p[r][2] = 0.f;
        const int kind = pt == 1 ? (a.c.ei_model == TCP_EI_DEUTSCH ? 1 : (a.c.ei_model == TCP_EI_KELBG ? 2 : 0)) : 0;
#define TCP_N3_ITEM(KIND, MASKED) \
    n3_item<KIND, ENERGY, MASKED, UNROLL, R>(a.c, tiles[stage], cnt, jstart, xi, ii, vi, sjacc, p, pe)
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
#pragma unroll
        for (int r = 0; r < R; ++r) {
            acc2(hi[r][0], lo[r][0], p[r][0] * qf);
            acc2(hi[r][1], lo[r][1], p[r][1] * qf);
            acc2(hi[r][2], lo[r][2], p[r][2] * qf);
        }
        if (ENERGY) acc2(eh, el, pe * a.c.u_qq_energy[pt]);
        // all warps are done with this subtile and its reaction sums
        const bool timeout = __syncthreads_or(!ok);
        if (!timeout && tid < cnt) {
            const double sc = -kEps * (double)qf;
            atomicAdd(&a.facc[jstart + tid], sc * (double)sjacc[tid][0]);
            atomicAdd(&a.facc[(size_t)a.n + jstart + tid], sc * (double)sjacc[tid][1]);
            atomicAdd(&a.facc[2 * (size_t)a.n + jstart + tid], sc * (double)sjacc[tid][2]);
        }
        if (tid < kN3Sub) sjacc[tid][0] = sjacc[tid][1] = sjacc[tid][2] = 0.f;
        return !timeout;
    };

    bool good = true;
    int k = 0;
    int issued = min(kN3Stages, nst);   // items whose subtile copy has been issued (thread 0's view)
    // static share: contiguous items, subtiles prefetched kN3Stages ahead
    for (; k < nst; ++k) {
        if (!process(k, I, S)) {
            good = false;
            break;
        }
        if (k + kN3Stages < nst) {
            if (tid == 0) {
                issue(k % kN3Stages, pS);
                n3_advance<TILE>(a, pI, pS);
            }
            issued = k + kN3Stages + 1;
        }
        __syncthreads();
        n3_advance<TILE>(a, I, S);
    }
    // dynamic share: one item at a time from the counter
    while (good) {
        if (tid == 0) {
            const long long it = a.nstatic + (long long)atomicAdd(a.counter, 1u);
            s_next = it;
            if (it < a.total) {
                int dI, dS;
                n3_decode<TILE>(a, it, dI, dS);
                issue(k % kN3Stages, dS);
            }
        }
        __syncthreads();
        const long long it = s_next;
        if (it >= a.total) break;
        issued = k + 1;
        int dI, dS;
        n3_decode<TILE>(a, it, dI, dS);
        if (!process(k, dI, dS)) {
            good = false;
            break;
        }
        __syncthreads();
        ++k;
    }
    if (!good) {
        if (tid == 0) {
            atomicOr(a.status, kStatusTmaTimeout);
            for (int kk = k; kk < issued; ++kk)   // copies possibly still in flight
                mbar_wait_bounded(&bars[kk % kN3Stages], (uint32_t)((kk / kN3Stages) & 1), kWaitLimitCycles);
        }
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

// Variants 1..V (0 = the ordered-pair kernel): i-particles per lane x unroll
// depth of the rotation loop x CTAs per SM.
typedef void (*N3Kernel)(const N3Args);
struct N3Variant {
    N3Kernel energy, plain;
    int R;
    const char *name;
};
static const N3Variant kVariants[] = {
    {pair_n3_kernel<true, 2, 2, 3>, pair_n3_kernel<false, 2, 2, 3>, 2, "n3_r2_u2_b3"},
    {pair_n3_kernel<true, 2, 1, 3>, pair_n3_kernel<false, 2, 1, 3>, 2, "n3_r2_u1_b3"},
    {pair_n3_kernel<true, 4, 1, 2>, pair_n3_kernel<false, 4, 1, 2>, 4, "n3_r4_u1_b2"},
    {pair_n3_kernel<true, 4, 2, 2>, pair_n3_kernel<false, 4, 2, 2>, 4, "n3_r4_u2_b2"},
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
    const int v = std::min(std::max(c->pair_variant, 1), kN3Variants);
    const int tile = 32 * kVariants[v - 1].R * kN3Warps;
    const int spt = tile / kN3Sub;
    N3Args a;
    a.xq = c->xq;
    a.nel = c->nel;
    a.n = c->n;
    a.nIe = cdiv(c->nel, tile);
    a.nI = a.nIe + cdiv(c->nion, tile);
    a.nSe = cdiv(c->nel, kN3Sub);
    a.nS = a.nSe + cdiv(c->nion, kN3Sub);
    long long total = 0;
    for (int I = 0; I < a.nI; ++I) {
        const int first = I < a.nIe ? I * spt : a.nSe + (I - a.nIe) * spt;
        total += a.nS - first;
    }
    a.total = total;
    a.nstatic = total - total * kN3DynPercent / 100;
    a.facc = c->fpart;
    a.upart = c->upart;
    a.status = c->status;
    a.counter = c->counter;
    a.c = c->pc;
    const int grid = (int)std::min<long long>(n3_grid_for(c, v), total);
    if (grid > c->n_upart) return set_error(TCP_ERR_STATE, "energy partial buffer smaller than the Newton-3 grid");
    TCP_CUDA(cudaMemsetAsync(c->fpart, 0, sizeof(double) * 3 * (size_t)c->n, c->stream));
    TCP_CUDA(cudaMemsetAsync(c->counter, 0, sizeof(unsigned), c->stream));
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

// pair_n3_f64.cu -- the FP64 real-space sum with Newton's third law: every
// unique pair (i < j) is evaluated once in FP64 and its force is added to both
// particles (Force_direct_self / _ext / _sum of force.f90:52-372, whose
// triangular loops also evaluate each pair once).
//
// The items are those of the compensated-FP32 Newton-3 kernel (pair_n3.cuh:
// i-tiles of 32 R W particles x j-subtiles of kN3Sub, bulk copies into a
// kN3Stages-deep ring), all taken one at a time from an atomic counter; the
// warp-rotation of j (position and reaction) runs on doubles.  Forces and
// energies are summed in FP64: per item in registers, then i-forces into
// registers along the row and j-reactions through shared-memory FP64 atomics,
// both added to the global FP64 force with one atomic per particle and
// component.  The order of those atomics varies from run to run, so results
// vary in the last bits; TCP_FLAG_DETERMINISTIC selects the ordered-pair
// kernel with its fixed-order reduction instead.
//
// Pair arithmetic follows force.f90:87-141 in FP64 without divisions: the
// minimum image (force.f90:92) is the wrapped difference of 64-bit fixed-point
// coordinates (2^64 per box length, refreshed with every position update),
// exact and then rounded once to FP64 (the sign choice at |d| = box/2 exactly
// differs from DNINT's, where r >= rc), 1/r and 1/r^3 come from one
// rsqrt_nr, the exponentials from the table-driven exp_neg_tab (2e-16
// relative), and the Ewald force term erfc(ar) + 2ar/sqrt(pi) exp(-a^2 r^2)
// (the reference's 1 - erf(ar)) is the Gaussian exp(-a^2 r^2), which the force
// needs anyway, times the segment polynomial of erfcx(x) + 2x/sqrt(pi)
// (ewald_q; 2e-16 relative, fit_erfcx64.py).  The
// cut-off and Kelbg range tests compare the bit patterns of non-negative
// doubles, which order as their values.
#include <algorithm>
#include <cstring>

#include "device_util.cuh"
#include "pair_n3.cuh"

namespace tcp {

constexpr int kF64R = 1;   // i-particles per lane

// The Kelbg Gaussian terms exp(-r^2/lambda^2) and erfc(r/lambda) are skipped
// beyond r = kKelbgFar lambda, where both are below 1e-31 of the pair's
// Coulomb terms.
constexpr double kKelbgFar = 8.5;

// One pair at squared distance r2 (> 0).  Returns the force weight w, with the
// force on i = eps qq w d, and adds the energy term (energy = qq pe) with ENERGY.
template <int KIND, bool ENERGY>
__device__ __forceinline__ double n3_pair_f64(const PairConsts &c, double r2, bool ok, double &pe, const F64Tab &tb) {
    const double rinv = rsqrt_nr(r2);
    const double r = r2 * rinv;
    const double rinv_m = ok ? rinv : 0.0;
    const double e = exp_neg_tab(c.alpha2 * r2, tb);
    double s = e * ewald_q(c.alpha * r, tb);              // erfc(ar) + 2ar/sqrt(pi) exp(-a^2 r^2), force.f90:104-106
    // the Ewald energy term erfc(ar)/r (force.f90:105, 1 - erf) = s/r - 2a/sqrt(pi) exp(-a^2 r^2)
    if (ENERGY) pe = fma(s, rinv_m, fma(-c.c_gauss_d, ok ? e : 0.0, pe));
    if (KIND == 2) {                                      // Kelbg, e-i pairs
        if (__double_as_longlong(r2) < __double_as_longlong(c.kelbg_far2)) {   // r < 8.5 lambda
            const double g = exp_neg_tab(r2 * c.inv_lam2, tb);
            s -= g;
            if (ENERGY && ok) pe += c.sqrtpi_lam_d * erfc_tab(r * c.inv_lam, g, tb) - g * rinv;
        }
    } else if (KIND == 1) {                               // Deutsch, force.f90:136-139
        const double y = exp_neg_tab(r * c.inv_rs_d, tb);
        s = s - y - y * r * c.inv_rs_d;
        if (ENERGY) pe = fma(-y, rinv_m, pe);
    }
    return s * (rinv_m * rinv * rinv);
}

// minimum-image separation from 64-bit fixed-point coordinates (2^64 per box
// length): the wrapped integer difference, exact, then one rounding to FP64
__device__ __forceinline__ double fixed_diff(long long a, long long b, double scale) {
    return (double)(long long)((unsigned long long)a - (unsigned long long)b) * scale;
}

// One item: the R i-particles of this lane against a j-subtile in shared
// memory.  MASKED: apply validity and i < j index masks.  CUBIC: the
// separations stay in units of L/2^64 (r^2 scaled once, the force and reaction
// sums once per item by the caller) instead of three scalings per pair.
// RDF: +2 per unique pair inside rc in bin INT(r/dx) of its type, r from sqrt
// as in the ordered FP64 kernel (force.f90:99-103)
template <int KIND, bool ENERGY, bool MASKED, int R, bool RDF, bool CUBIC>
__device__ __forceinline__ void n3_item_f64(const PairConsts &c, const longlong4_32a *__restrict__ tj, int cnt,
                                            int jstart, const longlong3 (&xi)[R], int ibase, int iend,
                                            double (*sjacc)[3], double (&p)[R][3], double &pe,
                                            const F64Tab &tb, unsigned *hist = nullptr, double inv_dx = 0.0) {
    const int lane = threadIdx.x & 31;
    const int src = (lane + 1) & 31;
    for (int ch = 0; ch * 32 < cnt; ++ch) {
        const int jl = ch * 32 + lane;
        longlong3 xj = make_longlong3(0, 0, 0);           // padding lanes: masked below
        if (jl < cnt) {
            const longlong4_32a t = tj[jl];
            xj = make_longlong3(t.x, t.y, t.z);
        }
        double jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll 1
        for (int s = 0; s < 32; ++s) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double dx = fixed_diff(xi[r].x, xj.x, CUBIC ? 1.0 : c.sl[0]);
                const double dy = fixed_diff(xi[r].y, xj.y, CUBIC ? 1.0 : c.sl[1]);
                const double dz = fixed_diff(xi[r].z, xj.z, CUBIC ? 1.0 : c.sl[2]);
                const double r2 = CUBIC ? fma(dx, dx, fma(dy, dy, dz * dz)) * c.sl2 : fma(dx, dx, fma(dy, dy, dz * dz));
                // 0 < r2 < rc^2 on the bit patterns (r2 >= 0: they order as the values)
                const long long rb = __double_as_longlong(r2);
                bool ok = rb > 0 && rb < __double_as_longlong(c.rc2);
                if (MASKED) {
                    const int jo = ch * 32 + ((lane + s) & 31);
                    const int ir = ibase + 32 * r;
                    ok = ok && (ir < iend) && (jo < cnt) && (ir < jstart + jo);
                }
                if (RDF && ok) {
                    const double tb = sqrt(r2) * inv_dx;
                    if (tb < (double)kNbin) atomicAdd(&hist[(int)tb], 2u);
                }
                const double w = n3_pair_f64<KIND, ENERGY>(c, ok ? r2 : 1.0, ok, pe, tb);
                p[r][0] = fma(w, dx, p[r][0]);
                p[r][1] = fma(w, dy, p[r][1]);
                p[r][2] = fma(w, dz, p[r][2]);
                jx = fma(w, dx, jx);
                jy = fma(w, dy, jy);
                jz = fma(w, dz, jz);
            }
            xj.x = __shfl_sync(0xffffffffu, xj.x, src);
            xj.y = __shfl_sync(0xffffffffu, xj.y, src);
            xj.z = __shfl_sync(0xffffffffu, xj.z, src);
            jx = __shfl_sync(0xffffffffu, jx, src);
            jy = __shfl_sync(0xffffffffu, jy, src);
            jz = __shfl_sync(0xffffffffu, jz, src);
        }
        // back home: lane l holds the reaction sum of j = ch*32 + l
        if (jl < cnt) {
            atomicAdd(&sjacc[jl][0], jx);
            atomicAdd(&sjacc[jl][1], jy);
            atomicAdd(&sjacc[jl][2], jz);
        }
    }
}

template <bool ENERGY, int R, bool RDF = false>
__global__ void __launch_bounds__(kN3Threads, 2) pair_n3_f64_kernel(const N3Args a) {
    constexpr int TILE = 32 * R * kN3Warps;
    __shared__ __align__(128) longlong4_32a tiles[kN3Stages][kN3Sub];
    __shared__ __align__(8) uint64_t bars[kN3Stages];
    __shared__ double sjacc[kN3Sub][3];
    __shared__ double red[32];
    __shared__ long long s_next;
    __shared__ unsigned hist[RDF ? 3 * kNbin : 1];
    __shared__ F64Tab tab;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (RDF)
        for (int k = tid; k < 3 * kNbin; k += kN3Threads) hist[k] = 0u;

    const long long it0 = a.nstatic * (long long)blockIdx.x / gridDim.x;
    const long long it1 = a.nstatic * (long long)(blockIdx.x + 1) / gridDim.x;
    const int nst = (int)(it1 - it0);

    for (int k = tid; k < kN3Sub * 3; k += kN3Threads) (&sjacc[0][0])[k] = 0.0;
    load_f64_tab(tab);
    if (tid == 0) {
        for (int s = 0; s < kN3Stages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    // subtile copy of item `it` into ring stage `stage` (thread 0)
    auto issue = [&](int stage, long long it) {
        int rep, I_, S_;
        n3_locate<TILE, false>(a, it, rep, I_, S_);
        int js, jc, jsp;
        n3_sub(a.g, S_, js, jc, jsp);
        const uint32_t bytes = (uint32_t)jc * sizeof(longlong4_32a);
        mbar_arrive_expect_tx(&bars[stage], bytes);
        bulk_g2s(tiles[stage], a.xl + js, bytes, &bars[stage]);
    };
    if (tid == 0)
        for (int k = 0; k < min(kN3Stages, nst); ++k)
            if (!(a.inject_skip && blockIdx.x == 0 && k == 0)) issue(k, it0 + k);

    double etot = 0.0;
    int curI = -1, istart = 0, iend = 0, isp = 0, ifirst = 0;
    longlong3 xi[R];
    double fi[R][3];
    int ibase = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        xi[r] = make_longlong3(0, 0, 0);
        fi[r][0] = fi[r][1] = fi[r][2] = 0.0;
    }

    auto flush_i = [&]() {
        if (curI < 0) return;
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (ibase + 32 * r < iend) atomicAdd(&a.facc[(size_t)k * a.ntot + ibase + 32 * r], kEps * fi[r][k]);
                fi[r][k] = 0.0;
            }
    };

    auto process = [&](int k, long long it) -> bool {
        int rep, I_, S_;
        n3_locate<TILE, false>(a, it, rep, I_, S_);
        if (I_ != curI) {
            flush_i();
            curI = I_;
            n3_itile<TILE>(a.g, I_, istart, iend, isp, ifirst);
            ibase = istart + warp * 32 * R + lane;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ir = ibase + 32 * r;
                const longlong4_32a t = a.xl[ir < iend ? ir : istart];
                xi[r] = make_longlong3(t.x, t.y, t.z);
            }
        }
        int jstart, cnt, jsp;
        n3_sub(a.g, S_, jstart, cnt, jsp);
        const int pt = isp + jsp;
        const bool masked = (S_ < ifirst + TILE / kN3Sub && jsp == isp) || cnt < kN3Sub || (iend - istart) < TILE;
        const int stage = k % kN3Stages;
        const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / kN3Stages) & 1), kWaitLimitCycles);
        const PairConsts &c = a.c;
        double p[R][3], pe = 0.0;
#pragma unroll
        for (int r = 0; r < R; ++r) p[r][0] = p[r][1] = p[r][2] = 0.0;
        const int kind = pt == 1 ? (c.ei_model == TCP_EI_DEUTSCH ? 1 : (c.ei_model == TCP_EI_KELBG ? 2 : 0)) : 0;
        if (ok) {
#define TCP_N3D_ITEM2(KIND, MASKED, CUBIC) \
    n3_item_f64<KIND, ENERGY, MASKED, R, RDF, CUBIC>(c, tiles[stage], cnt, jstart, xi, ibase, iend, sjacc, p, pe, \
                                                     tab, RDF ? hist + pt * kNbin : nullptr, RDF ? c.inv_dxd[pt] : 0.0)
#define TCP_N3D_ITEM(KIND, MASKED) \
    do {                                   \
        if (c.cubic)                       \
            TCP_N3D_ITEM2(KIND, MASKED, true); \
        else                               \
            TCP_N3D_ITEM2(KIND, MASKED, false); \
    } while (0)
            if (masked) {
                if (kind == 1) TCP_N3D_ITEM(1, true);
                else if (kind == 2) TCP_N3D_ITEM(2, true);
                else TCP_N3D_ITEM(0, true);
            } else {
                if (kind == 1) TCP_N3D_ITEM(1, false);
                else if (kind == 2) TCP_N3D_ITEM(2, false);
                else TCP_N3D_ITEM(0, false);
            }
#undef TCP_N3D_ITEM
#undef TCP_N3D_ITEM2
        }
        const double qq = c.qq[pt];
        const double us = c.cubic ? c.sl[0] : 1.0;   // units of the item's sums
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) fi[r][kk] = fma(qq * us, p[r][kk], fi[r][kk]);
        if (ENERGY) etot = fma(qq, pe, etot);
        // all warps are done with this subtile and its reaction sums
        const bool timeout = __syncthreads_or(!ok);
        if (!timeout && tid < cnt) {
            const double sc = -kEps * qq * us;
            const size_t j = (size_t)jstart + tid;
            atomicAdd(&a.facc[j], sc * sjacc[tid][0]);
            atomicAdd(&a.facc[(size_t)a.ntot + j], sc * sjacc[tid][1]);
            atomicAdd(&a.facc[2 * (size_t)a.ntot + j], sc * sjacc[tid][2]);
        }
        if (tid < kN3Sub) sjacc[tid][0] = sjacc[tid][1] = sjacc[tid][2] = 0.0;
        return !timeout;
    };

    bool good = true;
    int k = 0;
    int issued = min(kN3Stages, nst);
    for (; k < nst; ++k) {
        if (!process(k, it0 + k)) {
            good = false;
            break;
        }
        if (k + kN3Stages < nst) {
            if (tid == 0) issue(k % kN3Stages, it0 + k + kN3Stages);
            issued = k + kN3Stages + 1;
        }
        __syncthreads();
    }
    while (good) {
        if (tid == 0) {
            const long long it = a.nstatic + (long long)atomicAdd(a.counter, 1u);
            s_next = it;
            if (it < a.total && !(a.inject_skip && blockIdx.x == 0 && k == 0)) issue(k % kN3Stages, it);
        }
        __syncthreads();
        const long long it = s_next;
        if (it >= a.total) break;
        issued = k + 1;
        if (!process(k, it)) {
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
    if (RDF) {
        __syncthreads();
        for (int q = tid; q < 3 * kNbin; q += kN3Threads)
            if (hist[q]) atomicAdd(&a.rdf[q], (unsigned long long)hist[q]);
    }
}

// ---------------------------------------------------------------------------
bool n3_f64_applicable(const tcp_ctx *c) {
    return c->p.precision == TCP_PREC_FP64 && c->n >= 2 && !(c->flags & TCP_FLAG_DETERMINISTIC);
}

int n3_f64_grid(const tcp_ctx *c) {
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pair_n3_f64_kernel<true, kF64R>, kN3Threads, 0);
    return std::max(1, c->num_sms * std::max(1, bps));
}

int launch_pair_n3_f64(tcp_ctx *c, bool energy, bool rdf) {
    constexpr int tile = 32 * kF64R * kN3Warps;
    N3Args a;
    std::memset(&a, 0, sizeof a);
    long long total = 0;
    a.g = n3_geometry(0, c->nel, c->nion, tile, 0, &total);
    a.xl = c->xl;
    a.total = total;
    // all items from the counter: an FP64 item takes milliseconds, so the
    // per-item copy latency is negligible and the tail is at most one item
    a.nstatic = 0;
    a.ntot = c->n;
    a.facc = c->fpart;
    a.upart = c->upart;
    a.status = c->status;
    a.counter = c->counter;
    a.c = c->pc;
    a.inject_skip = inject_fault("tile_wait") ? 1 : 0;
    a.rdf = c->rdf;
    const int grid = (int)std::min<long long>(n3_f64_grid(c), total);
    if (grid > c->n_upart) return set_error(TCP_ERR_STATE, "energy partial buffer smaller than the Newton-3 grid");
    TCP_CUDA(cudaMemsetAsync(c->fpart, 0, sizeof(double) * 3 * (size_t)c->n, c->stream));
    TCP_CUDA(cudaMemsetAsync(c->counter, 0, sizeof(unsigned), c->stream));
    if (energy) {
        TCP_CUDA(cudaMemsetAsync(c->upart, 0, sizeof(double) * (size_t)c->n_upart, c->stream));
        if (rdf) pair_n3_f64_kernel<true, kF64R, true><<<grid, kN3Threads, 0, c->stream>>>(a);
        else pair_n3_f64_kernel<true, kF64R><<<grid, kN3Threads, 0, c->stream>>>(a);
    } else {
        if (rdf) pair_n3_f64_kernel<false, kF64R, true><<<grid, kN3Threads, 0, c->stream>>>(a);
        else pair_n3_f64_kernel<false, kF64R><<<grid, kN3Threads, 0, c->stream>>>(a);
    }
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

}  // namespace tcp

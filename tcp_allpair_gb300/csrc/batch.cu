// batch.cu -- many independent systems (replicas) in one context: one
// persistent Newton-3 pair launch over the items of all replicas, SPME with
// one batched cuFFT plan per distinct mesh, and replica-aware integrator and
// reduction kernels, captured together as one CUDA graph per MD step.
//
// Each replica is a complete system of the reference (its own box, charges,
// masses, Ewald alpha, e-i model and length, SPME mesh, thermostat target),
// stepped exactly as main.f90:81-153 steps one system.  Particles of all
// replicas are concatenated (replica r at [off_r, off_r + n_r), electrons
// first inside it) in SoA FP64 arrays; rep_of[i] maps a particle to its
// replica.  Requirements: compensated-FP32 precision, SPME, cubic boxes, one
// B-spline order for the batch, NOTEMP / ISOKIN / BEREND thermostats applied
// every step, one time step for all replicas.
//
// Per-replica sums (Ur, Um, sum m v^2, sum f) are accumulated with FP64
// atomics, warp-reduced first when a warp holds one replica.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "device_util.cuh"
#include "spme_math.cuh"
#include "tcp_internal.h"

namespace tcp {

struct BRep {
    int off, n, nel;
    double L[3];
    double iL[3], KL[3];     // 1/L, K/L (the kernels multiply: GB300's FP64 division is slow)
    double xm[2], q[2];      // masses, scaled charges
    double ixm[2];           // 1/xm
    int K[3], Kh;
    long long mesh_off, half_off;
    int bin_off, grp_off;    // first spreading bin (K2 K3 per replica) and first 8-row group
    double V;
    double Te, Ti, tau;
    int thermo;
};

constexpr int kBThreads = 256;

// accumulator block: ur[nrep] | um[nrep] | mv0[2 nrep] | mv1[2 nrep] | fsum[3 nrep]
struct BAcc {
    double *ur, *um, *mv0, *mv1, *fsum;
};


// add v to acc[key] with one atomic per warp when the warp shares the key
__device__ __forceinline__ void keyed_add(double *acc, int key, double v) {
    const unsigned all = __activemask();
    const int k0 = __shfl_sync(all, key, __ffs(all) - 1);
    if (__all_sync(all, key == k0) && all == 0xffffffffu) {
        v = warp_sum(v);
        if ((threadIdx.x & 31) == 0) atomicAdd(acc + key, v);
    } else {
        atomicAdd(acc + key, v);
    }
}

struct BParticles {
    double *x, *v, *f, *frec, *facc;
    int4 *xq;
    const int *rep_of;
    const BRep *reps;
    int ntot;
};

// VVerletNotemp1 (vverlet.f90:148-167) per replica
__global__ void b_vverlet1_kernel(const BParticles a, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.ntot) return;
    const BRep &R = a.reps[a.rep_of[i]];
    const double ixm = (i - R.off) < R.nel ? R.ixm[0] : R.ixm[1];
    int q[3];
    for (int k = 0; k < 3; ++k) {
        const size_t o = (size_t)k * a.ntot + i;
        const double vk = a.v[o] + 0.5 * dt * a.f[o] * ixm;
        a.v[o] = vk;
        const double y = wrap_box(a.x[o] + dt * vk, R.L[k], R.iL[k]);
        a.x[o] = y;
        q[k] = fixed_coord(y, R.iL[k]);
    }
    a.xq[i] = make_int4(q[0], q[1], q[2], 0);
}

__global__ void b_refresh_kernel(const BParticles a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.ntot) return;
    const BRep &R = a.reps[a.rep_of[i]];
    a.xq[i] = make_int4(fixed_coord(a.x[i], R.iL[0]), fixed_coord(a.x[(size_t)a.ntot + i], R.iL[1]),
                        fixed_coord(a.x[2 * (size_t)a.ntot + i], R.iL[2]), 0);
}

// ---- atomic-free spreading, cell-sorted per replica ------------------------------
// The single-system scheme of spme.cu over all replicas: particles are binned by
// the (y, z) mesh column of their spline base (replica r owns bins
// [bin_off, bin_off + K2 K3)), the bins are index-ordered, and a warp gathers 8
// mesh rows of one replica from the bins that reach them, summing in
// compensated two-float FP32 (no atomics; the same order on every call).
constexpr int kBRows = 8;
constexpr int kBRowWarps = 4;

template <int P>
__global__ void b_bin_count_kernel(const BParticles a, SpreadBins bins) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.ntot) return;
    const BRep &R = a.reps[a.rep_of[i]];
    int base[3];
#pragma unroll
    for (int d = 1; d < 3; ++d) {
        const double u = (a.x[(size_t)d * a.ntot + i] + R.L[d] * .5) * R.KL[d];
        base[d] = wrapi((int)trunc(u) - (P - 3), R.K[d]);
    }
    const int bin = R.bin_off + base[1] + R.K[1] * base[2];
    bins.rank[i] = atomicAdd(&bins.count[bin], 1);
    bins.ebx[i] = bin;
}

template <int P>
__global__ void b_bin_weights_kernel(const BParticles a, SpreadBins bins) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= a.ntot) return;
    const int i = bins.list[pos];
    const BRep &R = a.reps[a.rep_of[i]];
    float *w = static_cast<float *>(bins.ew) + (size_t)pos * 3 * P;
    float W[P], dW[P];
    int base[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = (a.x[(size_t)d * a.ntot + i] + R.L[d] * .5) * R.KL[d];
        spline_w<P, float>(u, W, dW);
#pragma unroll
        for (int j = 0; j < P; ++j) w[d * P + j] = W[j];
        base[d] = wrapi((int)trunc(u) - (P - 3), R.K[d]);
    }
    bins.ebx[pos] = base[0];
    bins.eby[pos] = base[1];
    static_cast<float *>(bins.eq)[pos] = (float)((i - R.off) < R.nel ? R.q[0] : R.q[1]);
}

__host__ __device__ constexpr size_t b_row_warp_bytes(int P, int k1max) {
    return (size_t)kBRows * k1max * 8 + 32 * (8 + (1 + 3 * P) * 4);
}

template <int P>
__global__ void __launch_bounds__(32 * kBRowWarps) b_row_spread_kernel(const BParticles a, const SpreadBins bins,
                                                                       int nrep, int ngroups, int k1max,
                                                                       float *__restrict__ Qf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = blockIdx.x * (blockDim.x >> 5) + warp;
    if (g >= ngroups) return;                                     // warp-uniform
    int lo = 0, hi_ = nrep - 1;
    while (lo < hi_) {
        const int mid = (lo + hi_ + 1) >> 1;
        if (a.reps[mid].grp_off <= g) lo = mid; else hi_ = mid - 1;
    }
    const BRep &R = a.reps[lo];
    const int K1 = R.K[0], K2 = R.K[1], K3 = R.K[2];
    const int ngy = (K2 + kBRows - 1) / kBRows, lg = g - R.grp_off;
    const int y0 = (lg % ngy) * kBRows, z = lg / ngy;
    const int nrow = min(kBRows, K2 - y0);
    unsigned char *base = smem + (size_t)warp * b_row_warp_bytes(P, k1max);
    float *hi = reinterpret_cast<float *>(base);                    // [kBRows][K1]
    float *lo_ = hi + (size_t)kBRows * k1max;
    float *sw = lo_ + (size_t)kBRows * k1max;                       // [32][3P]
    float *sq = sw + 32 * 3 * P;
    int *sbx = reinterpret_cast<int *>(sq + 32), *sby = sbx + 32;
    for (int k = lane; k < kBRows * K1; k += 32) {
        hi[k] = 0.f;
        lo_[k] = 0.f;
    }
    __syncwarp();
    const float *ew = static_cast<const float *>(bins.ew);
    const float *eq = static_cast<const float *>(bins.eq);
    const int nb = nrow + P - 1;
    for (int jz = 0; jz < P; ++jz) {
        int bz = z - jz;
        bz += bz < 0 ? K3 : 0;
        int by0 = y0 - P + 1, len0 = nb, len1 = 0;
        if (by0 < 0) {
            by0 += K2;
            len0 = min(nb, K2 - by0);
            len1 = nb - len0;
        }
        if (nb >= K2) {
            by0 = 0;
            len0 = K2;
            len1 = 0;
        }
        for (int piece = 0; piece < 2; ++piece) {
            const int blo = R.bin_off + (piece == 0 ? by0 : 0) + K2 * bz, len = piece == 0 ? len0 : len1;
            if (len <= 0) continue;
            const int p0 = bins.start[blo], p1 = bins.start[blo + len];
            for (int c0 = p0; c0 < p1; c0 += 32) {
                const int ne = min(32, p1 - c0);
                if (lane < ne) {
                    const int pos = c0 + lane;
#pragma unroll
                    for (int j = 0; j < 3 * P; ++j) sw[lane * 3 * P + j] = ew[(size_t)pos * 3 * P + j];
                    sq[lane] = eq[pos];
                    sbx[lane] = bins.ebx[pos];
                    sby[lane] = bins.eby[pos];
                }
                __syncwarp();
                for (int e = 0; e < ne; ++e) {
                    const float *w = sw + e * 3 * P;
                    const float qz = sq[e] * w[2 * P + jz];
                    const int bx = sbx[e], by = sby[e];
                    for (int l = lane; l < P * P; l += 32) {
                        const int jy = l / P, jx = l - jy * P;
                        int rl = by + jy - y0;
                        rl += rl < 0 ? K2 : 0;
                        rl -= rl >= K2 ? K2 : 0;
                        if (rl < nrow) {
                            int x = bx + jx;
                            x -= x >= K1 ? K1 : 0;
                            const float v = qz * w[P + jy] * w[jx];
                            const int k = rl * K1 + x;
                            const float sum = hi[k] + v, bp = sum - hi[k];
                            lo_[k] += (hi[k] - (sum - bp)) + (v - bp);
                            hi[k] = sum;
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    float *mesh = Qf + R.mesh_off;
    for (int k = lane; k < nrow * K1; k += 32) {
        const int rl = k / K1, x = k - rl * K1;
        mesh[(size_t)K1 * ((y0 + rl) + (size_t)K2 * z) + x] = hi[k] + lo_[k];
    }
}

// influence multiply; blocks [blk0[r], blk0[r+1]) belong to replica r
__global__ void b_influence_kernel(cufftComplex *__restrict__ Qk, const float *__restrict__ infl,
                                   const BRep *__restrict__ reps, const int *__restrict__ blk0, int nrep,
                                   double *__restrict__ um) {
    __shared__ double red[32];
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (blk0[mid] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const BRep &R = reps[lo];
    const int nb = blk0[lo + 1] - blk0[lo], lb = blockIdx.x - blk0[lo];
    const int total = R.K[2] * R.K[1] * R.Kh;
    // energy terms in FP32 per thread, FP64 across threads; the half-spectrum
    // column advances by the stride modulo Kh (no division per element)
    float e = 0.0f;
    const int stride = nb * blockDim.x;
    int idx = lb * blockDim.x + threadIdx.x;
    int kx = idx % R.Kh;
    const int dkx = stride % R.Kh;
    for (; idx < total; idx += stride) {
        const float g = infl[R.half_off + idx];
        cufftComplex z = Qk[R.half_off + idx];
        const float wgt = (kx == 0 || (2 * kx == R.K[0])) ? 1.0f : 2.0f;
        e = fmaf(wgt * g, fmaf(z.x, z.x, z.y * z.y), e);
        z.x *= g;
        z.y *= g;
        Qk[R.half_off + idx] = z;
        kx += dkx;
        if (kx >= R.Kh) kx -= R.Kh;
    }
    const double t = block_sum((double)e, red);
    if (threadIdx.x == 0) atomicAdd(&um[lo], t * kEps / (2.0 * kPi * R.V));
}

// Particles in the cell-sort order of the spread (order[t]): the lanes of a
// warp share replicas and mesh columns; mesh indices wrap by comparison.
template <int P>
__global__ void b_gather_kernel(const BParticles a, const float *__restrict__ phi, const int *__restrict__ order) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.ntot) return;
    const int i = order[t];
    const BRep &R = a.reps[a.rep_of[i]];
    const double q = (i - R.off) < R.nel ? R.q[0] : R.q[1];
    float W[3][P], dW[3][P];
    int base[3];
    for (int d = 0; d < 3; ++d) {
        const double u = (a.x[(size_t)d * a.ntot + i] + R.L[d] * .5) * R.KL[d];
        spline_w<P, float>(u, W[d], dW[d]);
        base[d] = wrapi((int)trunc(u) - (P - 3), R.K[d]);
    }
    const float *mesh = phi + R.mesh_off;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    int iz = base[2];
#pragma unroll 1
    for (int k = 0; k < P; ++k) {
        int iy = base[1];
#pragma unroll 1
        for (int j = 0; j < P; ++j) {
            const float *row = mesh + (size_t)R.K[0] * (iy + (size_t)R.K[1] * iz);
            float sx = 0.f, sd = 0.f;
            int ix = base[0];
#pragma unroll
            for (int ii = 0; ii < P; ++ii) {
                const float ph = row[ix];
                sx += dW[0][ii] * ph;
                sd += W[0][ii] * ph;
                ix = ix + 1 == R.K[0] ? 0 : ix + 1;
            }
            gx += sx * W[1][j] * W[2][k];
            gy += sd * dW[1][j] * W[2][k];
            gz += sd * W[1][j] * dW[2][k];
            iy = iy + 1 == R.K[1] ? 0 : iy + 1;
        }
        iz = iz + 1 == R.K[2] ? 0 : iz + 1;
    }
    const double coef = kEps / (kPi * R.V);
    a.frec[i] = -coef * q * (double)gx * R.KL[0];
    a.frec[(size_t)a.ntot + i] = -coef * q * (double)gy * R.KL[1];
    a.frec[2 * (size_t)a.ntot + i] = -coef * q * (double)gz * R.KL[2];
}

// f = real-space + reciprocal (SPME_SUM); per-replica sum f (REMOVE_RIGIDMTN)
__global__ void b_finalize_kernel(const BParticles a, double *__restrict__ fsum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.ntot;
    const int r = valid ? a.rep_of[i] : a.rep_of[a.ntot - 1];
    for (int k = 0; k < 3; ++k) {
        double fk = 0.0;
        if (valid) {
            const size_t o = (size_t)k * a.ntot + i;
            fk = a.facc[o] + a.frec[o];
            a.f[o] = fk;
        }
        keyed_add(fsum, 3 * r + k, fk);
    }
}

// second half kick with the net force removed (vverlet.f90:194-219,
// force.f90:996-1004); sum m v^2 per replica and species into mv
__global__ void b_kick2_kernel(const BParticles a, double dt, const double *__restrict__ fsum,
                               double *__restrict__ mv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.ntot;
    const int ic = valid ? i : a.ntot - 1;
    const int r = a.rep_of[ic];
    const BRep &R = a.reps[r];
    const int s = (ic - R.off) < R.nel ? 0 : 1;
    double mv2 = 0.0;
    if (valid) {
        const double xm = R.xm[s], ixm = R.ixm[s], in = 1.0 / (double)R.n;
        double vv[3];
        for (int k = 0; k < 3; ++k) {
            const size_t o = (size_t)k * a.ntot + i;
            const double fk = a.f[o] - fsum[3 * r + k] * in;
            a.f[o] = fk;
            vv[k] = a.v[o] + 0.5 * dt * fk * ixm;
            a.v[o] = vv[k];
        }
        mv2 = (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]) * xm;
    }
    keyed_add(mv, 2 * r + s, mv2);
}

// ISOKIN / BEREND rescale (vverlet.f90:331-344, 257-270); lambda = 1 for NOTEMP
__global__ void b_rescale_kernel(const BParticles a, double dt, const double *__restrict__ mv_in,
                                 double *__restrict__ mv_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.ntot;
    const int ic = valid ? i : a.ntot - 1;
    const int r = a.rep_of[ic];
    const BRep &R = a.reps[r];
    const int s = (ic - R.off) < R.nel ? 0 : 1;
    const int cnt = s == 0 ? R.nel : R.n - R.nel;
    double lam = 1.0;
    if (R.thermo == TCP_THERMO_ISOKIN || R.thermo == TCP_THERMO_BEREND) {
        const double T0 = mv_in[2 * r + s] / (double)(3 * cnt);
        const double T = s == 0 ? R.Te : R.Ti;
        lam = R.thermo == TCP_THERMO_ISOKIN ? sqrt(T / T0) : sqrt(1.0 + dt * (T / T0 - 1.0) / R.tau);
    }
    double mv2 = 0.0;
    if (valid) {
        double vv[3];
        for (int k = 0; k < 3; ++k) {
            const size_t o = (size_t)k * a.ntot + i;
            vv[k] = a.v[o] * lam;
            a.v[o] = vv[k];
        }
        mv2 = (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]) * R.xm[s];
    }
    keyed_add(mv_out, 2 * r + s, mv2);
}

}  // namespace tcp

// ---------------------------------------------------------------------------
struct tcp_batch {
    int nrep = 0, ntot = 0, device = 0, num_sms = 0, order = 4;
    std::vector<tcp_params> p;
    std::vector<int> nel, nion, off;
    std::vector<double> alpha, Uo;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;     // the SPME chain of a step, beside the pair launch
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_ready = nullptr;     // the pair launch's counter and accumulators are cleared
    cudaEvent_t ev[5] = {};             // phase marks of a step (event nodes in the step graph)
    void *l2_flush = nullptr;           // written between timed steps (tcp_batch_time_steps)
    size_t l2_flush_bytes = 0;
    // CTAs of the persistent pair grid left to the SPME chains; they rejoin the
    // pair launch on stream2 once the chains are done (chosen by the autotuner)
    int pair_reserve = 0;
    double reserve_ms[8] = {};
    tcp::N3Rejoin rejoin;
    double *x = nullptr, *v = nullptr, *f = nullptr, *frec = nullptr, *facc = nullptr;
    int4 *xq = nullptr;
    int *rep_of = nullptr;
    tcp::BRep *reps = nullptr;          // device table
    std::vector<tcp::BRep> h_reps;
    void *n3reps = nullptr;             // device Newton-3 table
    long long n3_items = 0;
    long long *n3_chunks = nullptr;     // chunk table of the guided schedule (device)
    unsigned n3_nchunks = 0;
    std::vector<tcp::PairConsts> pcs;   // per-replica pair constants (the table is refilled per variant)
    int pair_variant = 0;               // batched Newton-3 variant (batch autotuner)
    bool tuned = false;
    double variant_ms[16] = {};
    double *acc = nullptr;              // accumulator block
    double *h_acc = nullptr;            // pinned copy
    unsigned *status = nullptr, *counter = nullptr;
    // SPME
    float *Qf = nullptr, *infl = nullptr;
    // cell-sorted spreading
    int *bin_count = nullptr, *bin_start = nullptr, *bin_bsum = nullptr, *bin_rank = nullptr;
    int *bin_list = nullptr, *bin_ebx = nullptr, *bin_eby = nullptr;
    float *bin_ew = nullptr, *bin_eq = nullptr;
    int nbins = 0, ngroups = 0, k1max = 0;
    cufftComplex *Qk = nullptr;
    long long mesh_total = 0, half_total = 0;
    int *blk0 = nullptr;
    int infl_blocks = 0;
    struct Group {
        int K[3];
        long long mesh_off, half_off;
        int count;
        cufftHandle fwd, inv;
    };
    std::vector<Group> groups;
    // the transforms of mesh-size group k >= 1 run on gstream[k - 1] beside group 0's on stream2
    std::vector<cudaStream_t> gstream;
    cudaEvent_t ev_fft[2] = {};                 // forks: after the spread, after the influence multiply
    std::vector<cudaEvent_t> ev_gdone[2];       // joins of groups 1.. (each direction)
    bool ready = false;
    cudaGraphExec_t graph = nullptr;
    double graph_dt = 0;
    int graph_kernels = 0;
    long long launches = 0;
};

namespace tcp {

static BAcc acc_of(tcp_batch *b) {
    BAcc a;
    a.ur = b->acc;
    a.um = b->acc + b->nrep;
    a.mv0 = b->acc + 2 * b->nrep;
    a.mv1 = b->acc + 4 * b->nrep;
    a.fsum = b->acc + 6 * b->nrep;
    return a;
}

static BParticles parts(tcp_batch *b) {
    BParticles a;
    a.x = b->x;
    a.v = b->v;
    a.f = b->f;
    a.frec = b->frec;
    a.facc = b->facc;
    a.xq = b->xq;
    a.rep_of = b->rep_of;
    a.reps = b->reps;
    a.ntot = b->ntot;
    return a;
}

static SpreadBins b_bins(tcp_batch *b) {
    SpreadBins s;
    s.count = b->bin_count;
    s.start = b->bin_start;
    s.bsum = b->bin_bsum;
    s.rank = b->bin_rank;
    s.list = b->bin_list;
    s.ebx = b->bin_ebx;
    s.eby = b->bin_eby;
    s.ew = b->bin_ew;
    s.eq = b->bin_eq;
    return s;
}

template <int P>
static void b_spme_launch(tcp_batch *b, bool gather, cudaStream_t st) {
    const int blocks = (b->ntot + 127) / 128;
    if (gather) {
        b_gather_kernel<P><<<blocks, 128, 0, st>>>(parts(b), b->Qf, b->bin_list);   // sorted by the spread
        return;
    }
    const SpreadBins bins = b_bins(b);
    cudaMemsetAsync(b->bin_count, 0, sizeof(int) * (size_t)b->nbins, st);
    b_bin_count_kernel<P><<<blocks, 128, 0, st>>>(parts(b), bins);
    b->launches += launch_bin_sort(st, b->ntot, b->nbins, bins) - 5;   // the step's count assumes five
    b_bin_weights_kernel<P><<<blocks, 128, 0, st>>>(parts(b), bins);
    const size_t sm = kBRowWarps * b_row_warp_bytes(P, b->k1max);   // attribute set at tcp_batch_create
    b_row_spread_kernel<P><<<(b->ngroups + kBRowWarps - 1) / kBRowWarps, 32 * kBRowWarps, sm, st>>>(
        parts(b), bins, b->nrep, b->ngroups, b->k1max, b->Qf);
}

template <int P>
static int b_prepare_spread_p(tcp_batch *b) {
    TCP_CUDA(cudaFuncSetAttribute(b_row_spread_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(kBRowWarps * b_row_warp_bytes(P, b->k1max))));
    return TCP_OK;
}

static int b_prepare_spread(tcp_batch *b) {
    switch (b->order) {
        case 4: return b_prepare_spread_p<4>(b);
        case 5: return b_prepare_spread_p<5>(b);
        case 6: return b_prepare_spread_p<6>(b);
        case 7: return b_prepare_spread_p<7>(b);
        default: return b_prepare_spread_p<8>(b);
    }
}

static void b_spme(tcp_batch *b, bool gather, cudaStream_t st) {
    switch (b->order) {
        case 4: b_spme_launch<4>(b, gather, st); break;
        case 5: b_spme_launch<5>(b, gather, st); break;
        case 6: b_spme_launch<6>(b, gather, st); break;
        case 7: b_spme_launch<7>(b, gather, st); break;
        default: b_spme_launch<8>(b, gather, st); break;
    }
}

// The batched R2C (dir 0) or C2R (dir 1) of every mesh-size group.  The groups
// are independent and each transform leaves most of the GPU idle, so group 0
// runs on stream2 and group k >= 1 on gstream[k - 1], forked from stream2 and
// joined back into it.
static int b_fft_groups(tcp_batch *b, int dir) {
    const size_t ng = b->groups.size();
    if (ng > 1) {
        TCP_CUDA(cudaEventRecord(b->ev_fft[dir], b->stream2));
        for (size_t k = 1; k < ng; ++k) TCP_CUDA(cudaStreamWaitEvent(b->gstream[k - 1], b->ev_fft[dir], 0));
    }
    for (size_t k = 0; k < ng; ++k) {
        const auto &g = b->groups[k];
        const cudaStream_t st = k ? b->gstream[k - 1] : b->stream2;
        if (dir == 0) {
            cufftSetStream(g.fwd, st);
            if (cufftExecR2C(g.fwd, b->Qf + g.mesh_off, b->Qk + g.half_off) != CUFFT_SUCCESS)
                return set_error(TCP_ERR_CUFFT, "batched cufftExecR2C failed");
        } else {
            cufftSetStream(g.inv, st);
            if (cufftExecC2R(g.inv, b->Qk + g.half_off, b->Qf + g.mesh_off) != CUFFT_SUCCESS)
                return set_error(TCP_ERR_CUFFT, "batched cufftExecC2R failed");
        }
    }
    for (size_t k = 1; k < ng; ++k) {
        TCP_CUDA(cudaEventRecord(b->ev_gdone[dir][k - 1], b->gstream[k - 1]));
        TCP_CUDA(cudaStreamWaitEvent(b->stream2, b->ev_gdone[dir][k - 1], 0));
    }
    return TCP_OK;
}

// The SPME chain of every replica (spread, batched R2C per mesh size,
// influence multiply + energy, C2R, gather into frec), forked onto stream2
// after the work queued on the main stream, so that it runs beside the
// real-space launch; b_recip_join makes the main stream wait for it.
static int b_recip_fork(tcp_batch *b, const BAcc &A) {
    TCP_CUDA(cudaEventRecord(b->ev_fork, b->stream));
    TCP_CUDA(cudaStreamWaitEvent(b->stream2, b->ev_fork, 0));
    b_spme(b, false, b->stream2);                       // atomic-free, every mesh point written
    if (int rc = b_fft_groups(b, 0)) return rc;
    b_influence_kernel<<<b->infl_blocks, 256, 0, b->stream2>>>(b->Qk, b->infl, b->reps, b->blk0, b->nrep, A.um);
    if (int rc = b_fft_groups(b, 1)) return rc;
    b_spme(b, true, b->stream2);
    return TCP_OK;
}

// Phase mark k of a step: an event-record node while the stream is captured,
// a plain record otherwise (the External flag is valid during capture only).
// 0 step start, 1 after the first half kick, 2 end of the SPME chains (stream2),
// 3 end of the pair launch on the main stream, 4 step end.
static int b_mark(tcp_batch *b, int k, cudaStream_t s) {
    if (!b->ev[k]) return TCP_OK;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    TCP_CUDA(cudaStreamIsCapturing(s, &st));
    if (st == cudaStreamCaptureStatusActive)
        TCP_CUDA(cudaEventRecordWithFlags(b->ev[k], s, cudaEventRecordExternal));
    else
        TCP_CUDA(cudaEventRecord(b->ev[k], s));
    return TCP_OK;
}

static int b_recip_join(tcp_batch *b) {
    if (int rc = b_mark(b, 2, b->stream2)) return rc;
    if (int rc = n3_rejoin_launch(b->rejoin, b->stream2, b->ev_ready, &b->launches)) return rc;
    TCP_CUDA(cudaEventRecord(b->ev_join, b->stream2));
    TCP_CUDA(cudaStreamWaitEvent(b->stream, b->ev_join, 0));
    return TCP_OK;
}

// One batched MD step (main.f90:81-153 for every replica) on b->stream.
static int b_step(tcp_batch *b, double dt) {
    const BAcc A = acc_of(b);
    const int nb = (b->ntot + kBThreads - 1) / kBThreads;
    int rc;
    if ((rc = b_mark(b, 0, b->stream))) return rc;
    TCP_CUDA(cudaMemsetAsync(A.um, 0, sizeof(double) * 8 * (size_t)b->nrep, b->stream));   // um, mv0, mv1, fsum
    b_vverlet1_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b), dt);
    if ((rc = b_mark(b, 1, b->stream))) return rc;
    rc = b_recip_fork(b, A);
    if (!rc)
        rc = launch_pair_n3_batch(b->stream, b->xq, b->ntot, b->facc, b->n3reps, b->nrep, b->n3_items, b->n3_chunks, b->n3_nchunks, A.ur,
                                  b->status, b->counter, b->num_sms, true, b->pair_variant, b->pair_reserve,
                                  &b->rejoin, b->ev_ready);
    if (!rc) rc = b_mark(b, 3, b->stream);
    if (int jrc = b_recip_join(b)) return jrc;
    if (rc) return rc;
    b_finalize_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b), A.fsum);
    b_kick2_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b), dt, A.fsum, A.mv0);
    b_rescale_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b), dt, A.mv0, A.mv1);
    b->launches += 15;
    TCP_CUDA(cudaGetLastError());
    return b_mark(b, 4, b->stream);
}

// Newton-3 item table for variant v (its i-tile), uploaded on the stream
static int b_fill_n3(tcp_batch *b, int v) {
    std::vector<unsigned char> n3h(n3_rep_bytes() * b->nrep);
    b->n3_items = n3_batch_fill(n3h.data(), b->nrep, b->off.data(), b->nel.data(), b->nion.data(), b->pcs.data(),
                                n3_batch_tile(v));
    TCP_CUDA(cudaMemcpyAsync(b->n3reps, n3h.data(), n3h.size(), cudaMemcpyHostToDevice, b->stream));
    std::vector<long long> chunks;
    n3_chunk_table(b->n3_items, n3_batch_ctas(b->num_sms, v), chunks);
    cudaFree(b->n3_chunks);
    b->n3_chunks = nullptr;
    TCP_CUDA(cudaMalloc(&b->n3_chunks, sizeof(long long) * chunks.size()));
    TCP_CUDA(cudaMemcpyAsync(b->n3_chunks, chunks.data(), sizeof(long long) * chunks.size(), cudaMemcpyHostToDevice,
                             b->stream));
    b->n3_nchunks = (unsigned)chunks.size() - 1;
    TCP_CUDA(cudaStreamSynchronize(b->stream));
    b->pair_variant = v;
    return TCP_OK;
}

// CTAs of the persistent pair grid left to the SPME chains, which run beside
// it on stream2 and find no registers free otherwise; they rejoin the pair
// launch once the chains are done.  Each candidate is timed as the chains and
// the pair launch beside them, up to the join, over four graph replays; the
// smallest reserve within 0.3 % of the fastest is kept (TCP_BATCH_RESERVE
// forces one).
static constexpr int kBReserveCandidates[] = {0, 16, 32, 64, 128, 256, 512};
static int b_choose_reserve(tcp_batch *b) {
    b->pair_reserve = 0;
    if (const char *forced = getenv("TCP_BATCH_RESERVE")) {
        b->pair_reserve = std::max(atoi(forced), 0);
        return TCP_OK;
    }
    const BAcc A = acc_of(b);
    cudaEvent_t e0, e1;
    TCP_CUDA(cudaEventCreate(&e0));
    TCP_CUDA(cudaEventCreate(&e1));
    int rc = TCP_OK, k = 0;
    double best = 1e300;
    const long long before = b->launches;
    auto once = [&]() -> int {
        int r = b_recip_fork(b, A);
        if (!r)
            r = launch_pair_n3_batch(b->stream, b->xq, b->ntot, b->facc, b->n3reps, b->nrep, b->n3_items, b->n3_chunks,
                                     b->n3_nchunks, A.ur, b->status, b->counter, b->num_sms, true, b->pair_variant,
                                     b->pair_reserve, &b->rejoin, b->ev_ready);
        if (int j = b_recip_join(b)) return j;
        return r;
    };
    // each candidate captured as one graph and replayed, as it runs inside the
    // step graph (launched one by one, the chains would run ahead on an idle
    // GPU while the host is still issuing the pair launch)
    auto graph_of = [&](cudaGraphExec_t *ge) -> int {
        cudaGraph_t g = nullptr;
        TCP_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int r = once();
        const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (!r && ce != cudaSuccess) r = cuda_check(ce, "cudaStreamEndCapture");
        if (!r) {
            const cudaError_t ie = cudaGraphInstantiate(ge, g, 0);
            if (ie != cudaSuccess) r = cuda_check(ie, "cudaGraphInstantiate");
        }
        if (g) cudaGraphDestroy(g);
        return r;
    };
    for (const int r : kBReserveCandidates) {
        b->pair_reserve = r;
        cudaGraphExec_t ge = nullptr;
        if ((rc = graph_of(&ge))) break;
        cudaError_t le = cudaGraphLaunch(ge, b->stream);
        cudaEventRecord(e0, b->stream);
        for (int t = 0; t < 4 && le == cudaSuccess; ++t) le = cudaGraphLaunch(ge, b->stream);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        cudaGraphExecDestroy(ge);
        if (le != cudaSuccess) rc = cuda_check(le, "cudaGraphLaunch");
        if (rc) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        b->reserve_ms[k++] = ms / 4;
        best = std::min(best, (double)ms / 4);
    }
    b->launches = before;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    b->pair_reserve = kBReserveCandidates[0];
    for (int j = k - 1; j >= 0; --j)
        if (b->reserve_ms[j] <= best * 1.003) b->pair_reserve = kBReserveCandidates[j];
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

// Batch autotuner: times every batched Newton-3 variant on this batch's items
// (one warm-up and two timed launches each, CUDA events) and keeps the
// fastest; TCP_BATCH_VARIANT forces one.  Runs before the step graph is captured.
static int b_autotune(tcp_batch *b) {
    if (b->tuned) return TCP_OK;
    b->tuned = true;
    const int nv = n3_batch_variant_count();
    bool erfc5_ok = true;   // the degree-5 erfc variants need it in every replica
    for (const PairConsts &pc : b->pcs) erfc5_ok = erfc5_ok && pc.erfc5_ok;
    if (const char *forced = getenv("TCP_BATCH_VARIANT")) {
        int v = std::min(std::max(atoi(forced), 0), nv - 1);
        if (n3_batch_variant_erfc5(v) && !erfc5_ok) v = 0;
        if (int rc = b_fill_n3(b, v)) return rc;
        return b_choose_reserve(b);
    }
    const BAcc A = acc_of(b);
    const int nb = (b->ntot + kBThreads - 1) / kBThreads;
    b_refresh_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b));
    cudaEvent_t e0, e1;
    TCP_CUDA(cudaEventCreate(&e0));
    TCP_CUDA(cudaEventCreate(&e1));
    double best = 1e300;
    int best_v = 0, rc = TCP_OK;
    for (int v = 0; v < nv && v < 16 && !rc; ++v) {
        if (n3_batch_variant_erfc5(v) && !erfc5_ok) continue;   // ms stays 0: not timed
        if ((rc = b_fill_n3(b, v))) break;
        rc = launch_pair_n3_batch(b->stream, b->xq, b->ntot, b->facc, b->n3reps, b->nrep, b->n3_items, b->n3_chunks, b->n3_nchunks, A.ur,
                                  b->status, b->counter, b->num_sms, true, v);
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < 2 && !rc; ++r)
            rc = launch_pair_n3_batch(b->stream, b->xq, b->ntot, b->facc, b->n3reps, b->nrep, b->n3_items, b->n3_chunks, b->n3_nchunks, A.ur,
                                      b->status, b->counter, b->num_sms, true, v);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        b->variant_ms[v] = ms / 2;
        if (ms / 2 < best) {
            best = ms / 2;
            best_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = b_fill_n3(b, best_v))) return rc;
    return b_choose_reserve(b);
}

static int b_sync(tcp_batch *b) {
    TCP_CUDA(cudaMemcpyAsync(b->h_acc, b->acc, sizeof(double) * 9 * (size_t)b->nrep, cudaMemcpyDeviceToHost,
                             b->stream));
    unsigned st = 0;
    TCP_CUDA(cudaMemcpyAsync(&st, b->status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    TCP_CUDA(cudaStreamSynchronize(b->stream));
    if (st & kStatusTmaTimeout) {
        cudaMemsetAsync(b->status, 0, sizeof(unsigned), b->stream);
        return set_error(TCP_ERR_TIMEOUT, "a pair-kernel tile wait exceeded its bound");
    }
    return TCP_OK;
}

static void b_energies(tcp_batch *b, tcp_energies *e) {
    if (!e) return;
    for (int r = 0; r < b->nrep; ++r) {
        e[r].Ur = b->h_acc[r];
        e[r].Um = b->h_acc[b->nrep + r];
        e[r].Uo = b->Uo[r];
        e[r].Epot = (e[r].Ur + e[r].Uo) * kEps;
        e[r].mv2el = b->h_acc[4 * b->nrep + 2 * r];
        e[r].mv2ion = b->h_acc[4 * b->nrep + 2 * r + 1];
    }
}

}  // namespace tcp

using namespace tcp;

extern "C" {

int tcp_batch_destroy(tcp_batch *b) {
    if (!b) return TCP_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto &g : b->groups) {
        cufftDestroy(g.fwd);
        cufftDestroy(g.inv);
    }
    for (void *ptr : {(void *)b->x, (void *)b->v, (void *)b->f, (void *)b->frec, (void *)b->facc, (void *)b->xq,
                      (void *)b->rep_of, (void *)b->reps, b->n3reps, (void *)b->n3_chunks, (void *)b->acc, (void *)b->status,
                      (void *)b->counter, (void *)b->Qf, (void *)b->infl, (void *)b->Qk, (void *)b->blk0,
                      (void *)b->bin_count, (void *)b->bin_start, (void *)b->bin_bsum, (void *)b->bin_rank,
                      (void *)b->bin_list, (void *)b->bin_ebx, (void *)b->bin_eby, (void *)b->bin_ew,
                      (void *)b->bin_eq})
        cudaFree(ptr);
    if (b->h_acc) cudaFreeHost(b->h_acc);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->ev_ready) cudaEventDestroy(b->ev_ready);
    for (cudaEvent_t &e : b->ev)
        if (e) cudaEventDestroy(e);
    cudaFree(b->l2_flush);
    n3_rejoin_free(b->rejoin);
    for (cudaStream_t st : b->gstream) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (int d = 0; d < 2; ++d) {
        if (b->ev_fft[d]) cudaEventDestroy(b->ev_fft[d]);
        for (cudaEvent_t e : b->ev_gdone[d]) cudaEventDestroy(e);
    }
    if (b->stream2) {
        cudaStreamSynchronize(b->stream2);
        cudaStreamDestroy(b->stream2);
    }
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return TCP_OK;
}

int tcp_batch_create(const tcp_params *params, const int *nel, const int *nion, int nrep, int device,
                     tcp_batch **out) {
    TCP_TRACE("tcp_batch_create");
    if (!out || !params || !nel || !nion || nrep <= 0) return set_error(TCP_ERR_BAD_PARAM, "bad arguments");
    *out = nullptr;
    for (int r = 0; r < nrep; ++r) {
        const tcp_params &p = params[r];
        if (p.precision != TCP_PREC_FP32C || p.reciprocal != TCP_RECIP_SPME)
            return set_error(TCP_ERR_BAD_PARAM, "batch replicas need TCP_PREC_FP32C and TCP_RECIP_SPME");
        if (!(p.box[0] > 0) || p.box[0] != p.box[1] || p.box[1] != p.box[2])
            return set_error(TCP_ERR_BAD_PARAM, "batch replicas need cubic boxes");
        if (p.order != params[0].order || p.order < 4 || p.order > kMaxOrder)
            return set_error(TCP_ERR_BAD_PARAM, "batch replicas need one B-spline order in 4..8");
        for (int d = 0; d < 3; ++d)
            if (p.K[d] < p.order) return set_error(TCP_ERR_BAD_PARAM, "SPME mesh must be >= order");
        if (nel[r] < 0 || nion[r] < 0 || nel[r] + nion[r] < 2) return set_error(TCP_ERR_BAD_PARAM, "bad particle counts");
        if (p.thermo == TCP_THERMO_STOCH) return set_error(TCP_ERR_BAD_PARAM, "STOCH is not batched");
        if (!(p.rc > 0.0) || !(p.xm[0] > 0) || !(p.xm[1] > 0)) return set_error(TCP_ERR_BAD_PARAM, "bad rc or masses");
        if (p.ei_model == TCP_EI_KELBG && !(p.lambda_ei > 0)) return set_error(TCP_ERR_BAD_PARAM, "Kelbg needs lambda_ei > 0");
        if (p.ei_model == TCP_EI_DEUTSCH && !(p.rs > 0)) return set_error(TCP_ERR_BAD_PARAM, "Deutsch needs rs > 0");
    }
    cudaDeviceProp prop;
    TCP_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3) return set_error(TCP_ERR_NO_DEVICE, "libtcpgpu is built for sm_103a");
    TCP_CUDA(cudaSetDevice(device));
    tcp_batch *b = new tcp_batch();
    b->nrep = nrep;
    b->device = device;
    b->num_sms = prop.multiProcessorCount;
    b->order = params[0].order;
    b->p.assign(params, params + nrep);
    for (auto &p : b->p)
        if (p.charge_scale == 0.0) p.charge_scale = 1.0;
    b->nel.assign(nel, nel + nrep);
    b->nion.assign(nion, nion + nrep);
    b->off.resize(nrep);
    for (int r = 0; r < nrep; ++r) {
        b->off[r] = b->ntot;
        b->ntot += nel[r] + nion[r];
    }
    auto fail = [&](int code) {
        tcp_batch_destroy(b);
        return code;
    };
    const size_t n = b->ntot;
#define TCP_BALLOC(ptr, bytes)                                                      \
    do {                                                                            \
        cudaError_t _e = cudaMalloc(&(ptr), (bytes));                               \
        if (_e != cudaSuccess) return fail(cuda_check(_e, "cudaMalloc " #ptr));     \
    } while (0)
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess ||
        cudaEventCreate(&b->ev[2]) != cudaSuccess || cudaEventCreate(&b->ev[3]) != cudaSuccess ||
        cudaEventCreate(&b->ev[4]) != cudaSuccess)
        return fail(cuda_check(cudaGetLastError(), "cudaStreamCreate"));
    TCP_BALLOC(b->x, sizeof(double) * 3 * n);
    TCP_BALLOC(b->v, sizeof(double) * 3 * n);
    TCP_BALLOC(b->f, sizeof(double) * 3 * n);
    TCP_BALLOC(b->frec, sizeof(double) * 3 * n);
    TCP_BALLOC(b->facc, sizeof(double) * 3 * n);
    TCP_BALLOC(b->xq, sizeof(int4) * n);
    TCP_BALLOC(b->rep_of, sizeof(int) * n);
    TCP_BALLOC(b->reps, sizeof(BRep) * nrep);
    TCP_BALLOC(b->n3reps, n3_rep_bytes() * nrep);
    TCP_BALLOC(b->acc, sizeof(double) * 9 * nrep);
    TCP_BALLOC(b->status, sizeof(unsigned));
    TCP_BALLOC(b->counter, sizeof(unsigned));
    if (cudaMallocHost(&b->h_acc, sizeof(double) * 9 * nrep) != cudaSuccess)
        return fail(cuda_check(cudaGetLastError(), "cudaMallocHost"));
    std::vector<int> rep_of(n);
    for (int r = 0; r < nrep; ++r)
        for (int i = 0; i < nel[r] + nion[r]; ++i) rep_of[b->off[r] + i] = r;
    TCP_CUDA(cudaMemcpyAsync(b->rep_of, rep_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
    for (double *ptr : {b->x, b->v, b->f, b->frec, b->facc})
        cudaMemsetAsync(ptr, 0, sizeof(double) * 3 * n, b->stream);
    cudaMemsetAsync(b->acc, 0, sizeof(double) * 9 * nrep, b->stream);
    cudaMemsetAsync(b->status, 0, sizeof(unsigned), b->stream);
    // SPME meshes grouped by size: replicas of one group are contiguous so that
    // one batched plan transforms them all
    std::map<std::tuple<int, int, int>, std::vector<int>> by_mesh;
    for (int r = 0; r < nrep; ++r) by_mesh[{params[r].K[0], params[r].K[1], params[r].K[2]}].push_back(r);
    b->h_reps.resize(nrep);
    for (auto &kv : by_mesh) {
        tcp_batch::Group g;
        g.K[0] = std::get<0>(kv.first);
        g.K[1] = std::get<1>(kv.first);
        g.K[2] = std::get<2>(kv.first);
        g.mesh_off = b->mesh_total;
        g.half_off = b->half_total;
        g.count = (int)kv.second.size();
        const long long nreal = (long long)g.K[0] * g.K[1] * g.K[2];
        const long long nhalf = (long long)(g.K[0] / 2 + 1) * g.K[1] * g.K[2];
        for (int k = 0; k < g.count; ++k) {
            BRep &R = b->h_reps[kv.second[k]];
            R.mesh_off = b->mesh_total + k * nreal;
            R.half_off = b->half_total + k * nhalf;
        }
        b->mesh_total += nreal * g.count;
        b->half_total += nhalf * g.count;
        int nfwd[3] = {g.K[2], g.K[1], g.K[0]};
        if (cufftPlanMany(&g.fwd, 3, nfwd, nullptr, 1, (int)nreal, nullptr, 1, (int)nhalf, CUFFT_R2C, g.count) !=
                CUFFT_SUCCESS ||
            cufftPlanMany(&g.inv, 3, nfwd, nullptr, 1, (int)nhalf, nullptr, 1, (int)nreal, CUFFT_C2R, g.count) !=
                CUFFT_SUCCESS)
            return fail(set_error(TCP_ERR_CUFFT, "cufftPlanMany failed"));
        cufftSetStream(g.fwd, b->stream);
        cufftSetStream(g.inv, b->stream);
        b->groups.push_back(g);
    }
    for (size_t k = 1; k < b->groups.size(); ++k) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
            return fail(cuda_check(cudaGetLastError(), "cudaStreamCreate"));
        b->gstream.push_back(st);
        for (int d = 0; d < 2; ++d) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                return fail(cuda_check(cudaGetLastError(), "cudaEventCreate"));
            b->ev_gdone[d].push_back(e);
        }
    }
    for (int d = 0; d < 2 && b->groups.size() > 1; ++d)
        if (cudaEventCreateWithFlags(&b->ev_fft[d], cudaEventDisableTiming) != cudaSuccess)
            return fail(cuda_check(cudaGetLastError(), "cudaEventCreate"));
    TCP_BALLOC(b->Qf, sizeof(float) * (size_t)b->mesh_total);
    // spreading bins (K2 K3 per replica) and 8-row groups (ceil(K2/8) K3 per replica)
    for (int r = 0; r < nrep; ++r) {
        BRep &R = b->h_reps[r];
        R.bin_off = b->nbins;
        R.grp_off = b->ngroups;
        b->nbins += b->p[r].K[1] * b->p[r].K[2];
        b->ngroups += ((b->p[r].K[1] + kBRows - 1) / kBRows) * b->p[r].K[2];
        b->k1max = std::max(b->k1max, b->p[r].K[0]);
    }
    TCP_BALLOC(b->bin_count, sizeof(int) * ((size_t)b->nbins + 1));
    TCP_BALLOC(b->bin_start, sizeof(int) * ((size_t)b->nbins + 1));
    TCP_BALLOC(b->bin_bsum, sizeof(int) * (size_t)((b->nbins + bin_scan_block() - 1) / bin_scan_block()));
    TCP_BALLOC(b->bin_rank, sizeof(int) * (size_t)b->ntot);
    TCP_BALLOC(b->bin_list, sizeof(int) * (size_t)b->ntot);
    TCP_BALLOC(b->bin_ebx, sizeof(int) * (size_t)b->ntot);
    TCP_BALLOC(b->bin_eby, sizeof(int) * (size_t)b->ntot);
    TCP_BALLOC(b->bin_ew, sizeof(float) * 3 * kMaxOrder * (size_t)b->ntot);
    TCP_BALLOC(b->bin_eq, sizeof(float) * (size_t)b->ntot);
    if (b_prepare_spread(b)) return fail(TCP_ERR_CUDA);
    TCP_BALLOC(b->infl, sizeof(float) * (size_t)b->half_total);
    TCP_BALLOC(b->Qk, sizeof(cufftComplex) * (size_t)b->half_total);
    TCP_BALLOC(b->blk0, sizeof(int) * (nrep + 1));
#undef TCP_BALLOC
    TCP_CUDA(cudaStreamSynchronize(b->stream));
    *out = b;
    return TCP_OK;
}

int tcp_batch_ewald_self(tcp_batch *b, double *Uo) {
    if (!b) return set_error(TCP_ERR_BAD_PARAM, "batch is NULL");
    cudaSetDevice(b->device);
    const int nrep = b->nrep;
    b->alpha.assign(nrep, 0.0);
    b->Uo.assign(nrep, 0.0);
    std::vector<PairConsts> pcs(nrep);
    std::vector<int> blk0(nrep + 1, 0);
    std::vector<float> infl((size_t)b->half_total);
    for (int r = 0; r < nrep; ++r) {
        const tcp_params &p = b->p[r];
        if (p.rc > p.box[0] / 2.0) return set_error(TCP_ERR_CUTOFF, "replica " + std::to_string(r) + ": rc > L/2");
        const double alpha = p.a > 0.0 ? p.a : 3.1 / p.rc;                     // force.f90:23
        b->alpha[r] = alpha;
        const double s = p.charge_scale;
        b->Uo[r] = ewald_constant_energy(p, b->nel[r], b->nion[r], alpha);   // force.f90:44-45 + background
        tcp_ctx tmp;
        tmp.p = p;
        tmp.nel = b->nel[r];
        tmp.nion = b->nion[r];
        tmp.n = tmp.nel + tmp.nion;
        tmp.alpha = alpha;
        tmp.rc2 = p.rc * p.rc;
        make_pair_consts(&tmp);
        pcs[r] = tmp.pc;
        BRep &R = b->h_reps[r];
        R.off = b->off[r];
        R.n = b->nel[r] + b->nion[r];
        R.nel = b->nel[r];
        for (int d = 0; d < 3; ++d) {
            R.L[d] = p.box[d];
            R.iL[d] = 1.0 / p.box[d];
            R.K[d] = p.K[d];
            R.KL[d] = (double)p.K[d] / p.box[d];
        }
        R.Kh = p.K[0] / 2 + 1;
        R.xm[0] = p.xm[0];
        R.xm[1] = p.xm[1];
        R.ixm[0] = 1.0 / p.xm[0];
        R.ixm[1] = 1.0 / p.xm[1];
        R.q[0] = s * p.q[0];
        R.q[1] = s * p.q[1];
        R.V = p.box[0] * p.box[1] * p.box[2];
        R.Te = p.Te;
        R.Ti = p.Ti;
        R.tau = p.tau;
        R.thermo = p.thermo;
        // influence function theta(m) |b(m)|^-2 on the half spectrum (EWALD_SELF, force.f90:27-42)
        std::vector<double> bx = bspline_moduli(p.order, p.K[0]), by = bspline_moduli(p.order, p.K[1]),
                            bz = bspline_moduli(p.order, p.K[2]);
        for (int k = 0; k < p.K[2]; ++k) {
            const int iz = (k + p.K[2] / 2) % p.K[2] - p.K[2] / 2;
            for (int j = 0; j < p.K[1]; ++j) {
                const int iy = (j + p.K[1] / 2) % p.K[1] - p.K[1] / 2;
                for (int i = 0; i < R.Kh; ++i) {
                    const int ix = (i + p.K[0] / 2) % p.K[0] - p.K[0] / 2;
                    const size_t idx = R.half_off + i + (size_t)R.Kh * (j + (size_t)p.K[1] * k);
                    if (ix == 0 && iy == 0 && iz == 0) {
                        infl[idx] = 0.f;
                        continue;
                    }
                    const double m2 = (double)ix * ix / (p.box[0] * p.box[0]) + (double)iy * iy / (p.box[1] * p.box[1]) +
                                      (double)iz * iz / (p.box[2] * p.box[2]);
                    infl[idx] = (float)(std::exp(-m2 * kPi * kPi / (alpha * alpha)) / m2 * bx[i] * by[j] * bz[k]);
                }
            }
        }
        const long long half = (long long)R.Kh * p.K[1] * p.K[2];
        // a few blocks per replica: each block adds its energy partial to the
        // replica's Um with one FP64 atomic, and hundreds of atomics on one
        // address serialise (512 blocks a replica: 80 us for the 64 replicas)
        blk0[r + 1] = blk0[r] + (int)std::max<long long>(1, std::min<long long>((half + 255) / 256, 16));
    }
    b->infl_blocks = blk0[nrep];
    b->pcs = pcs;
    b->tuned = false;
    int frc = b_fill_n3(b, b->pair_variant);
    if (frc) return frc;
    TCP_CUDA(cudaMemcpyAsync(b->reps, b->h_reps.data(), sizeof(BRep) * nrep, cudaMemcpyHostToDevice, b->stream));
    TCP_CUDA(cudaMemcpyAsync(b->blk0, blk0.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice, b->stream));
    TCP_CUDA(cudaMemcpyAsync(b->infl, infl.data(), sizeof(float) * infl.size(), cudaMemcpyHostToDevice, b->stream));
    TCP_CUDA(cudaStreamSynchronize(b->stream));
    if (Uo)
        for (int r = 0; r < nrep; ++r) Uo[r] = b->Uo[r];
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->ready = true;
    return TCP_OK;
}

int tcp_batch_upload(tcp_batch *b, int rep, const double *x, const double *v, const double *f) {
    if (!b || rep < 0 || rep >= b->nrep) return set_error(TCP_ERR_BAD_PARAM, "bad batch or replica");
    cudaSetDevice(b->device);
    const int n = b->nel[rep] + b->nion[rep];
    std::vector<double> soa(3 * (size_t)n);
    double *dst[3] = {b->x, b->v, b->f};
    const double *src[3] = {x, v, f};
    for (int q = 0; q < 3; ++q) {
        if (!src[q]) continue;
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) soa[(size_t)k * n + i] = src[q][3 * (size_t)i + k];
        for (int k = 0; k < 3; ++k)
            TCP_CUDA(cudaMemcpyAsync(dst[q] + (size_t)k * b->ntot + b->off[rep], soa.data() + (size_t)k * n,
                                     sizeof(double) * n, cudaMemcpyHostToDevice, b->stream));
        TCP_CUDA(cudaStreamSynchronize(b->stream));
    }
    if (x && b->ready) {
        b_refresh_kernel<<<(b->ntot + 255) / 256, 256, 0, b->stream>>>(parts(b));
        TCP_CUDA(cudaGetLastError());
    }
    TCP_CUDA(cudaStreamSynchronize(b->stream));
    return TCP_OK;
}

int tcp_batch_download(tcp_batch *b, int rep, double *x, double *v, double *f) {
    if (!b || rep < 0 || rep >= b->nrep) return set_error(TCP_ERR_BAD_PARAM, "bad batch or replica");
    cudaSetDevice(b->device);
    const int n = b->nel[rep] + b->nion[rep];
    std::vector<double> soa(3 * (size_t)n);
    const double *src[3] = {b->x, b->v, b->f};
    double *dst[3] = {x, v, f};
    for (int q = 0; q < 3; ++q) {
        if (!dst[q]) continue;
        for (int k = 0; k < 3; ++k)
            TCP_CUDA(cudaMemcpyAsync(soa.data() + (size_t)k * n, src[q] + (size_t)k * b->ntot + b->off[rep],
                                     sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream));
        TCP_CUDA(cudaStreamSynchronize(b->stream));
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) dst[q][3 * (size_t)i + k] = soa[(size_t)k * n + i];
    }
    return TCP_OK;
}

// Forces of all replicas at the current positions (main.f90:100-141 per
// replica): SPME, real-space sum, SPME_SUM and REMOVE_RIGIDMTN.
int tcp_batch_force(tcp_batch *b, tcp_energies *e) {
    TCP_TRACE("tcp_batch_force");
    if (!b || !b->ready) return set_error(TCP_ERR_STATE, "tcp_batch_ewald_self must be called first");
    cudaSetDevice(b->device);
    if (int arc = b_autotune(b)) return arc;
    const BAcc A = acc_of(b);
    const int nb = (b->ntot + kBThreads - 1) / kBThreads;
    b_refresh_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b));
    TCP_CUDA(cudaMemsetAsync(A.um, 0, sizeof(double) * 8 * (size_t)b->nrep, b->stream));
    int rc = b_recip_fork(b, A);
    if (!rc)
        rc = launch_pair_n3_batch(b->stream, b->xq, b->ntot, b->facc, b->n3reps, b->nrep, b->n3_items, b->n3_chunks, b->n3_nchunks, A.ur,
                                  b->status, b->counter, b->num_sms, true, b->pair_variant, b->pair_reserve,
                                  &b->rejoin, b->ev_ready);
    if (int jrc = b_recip_join(b)) return jrc;
    if (rc) return rc;
    b_finalize_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b), A.fsum);
    // the net-force removal of the step is fused into the kick; here apply it alone
    b_kick2_kernel<<<nb, kBThreads, 0, b->stream>>>(parts(b), 0.0, A.fsum, A.mv0);
    TCP_CUDA(cudaGetLastError());
    if ((rc = b_sync(b))) return rc;
    b_energies(b, e);
    return TCP_OK;
}

// nsteps MD steps of every replica, one CUDA graph per step.
int tcp_batch_md_steps(tcp_batch *b, double dt, int nsteps, tcp_energies *e) {
    TCP_TRACE("tcp_batch_md_steps");
    if (!b || !b->ready) return set_error(TCP_ERR_STATE, "tcp_batch_ewald_self must be called first");
    if (nsteps < 0) return set_error(TCP_ERR_BAD_PARAM, "nsteps < 0");
    cudaSetDevice(b->device);
    int rc;
    if ((rc = b_autotune(b))) return rc;                // timing launches cannot run inside a capture
    if (!b->graph || b->graph_dt != dt) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g;
        const long long before = b->launches;
        TCP_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        rc = b_step(b, dt);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (rc) return rc;
        if (ce != cudaSuccess) return cuda_check(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_check(ce, "cudaGraphInstantiate");
        b->graph_kernels = (int)(b->launches - before);
        b->launches = before;
        b->graph_dt = dt;
    }
    for (int s = 0; s < nsteps; ++s) {
        TCP_CUDA(cudaGraphLaunch(b->graph, b->stream));
        b->launches += b->graph_kernels;
    }
    if ((rc = b_sync(b))) return rc;
    b_energies(b, e);
    return TCP_OK;
}

int tcp_batch_autotune_report(tcp_batch *b, int *variant, double *ms, int nmax) {
    if (!b) return set_error(TCP_ERR_BAD_PARAM, "batch is NULL");
    if (variant) *variant = b->pair_variant;
    for (int k = 0; ms && k < nmax && k < 16; ++k) ms[k] = b->variant_ms[k];
    return TCP_OK;
}

int tcp_batch_overlap_report(tcp_batch *b, int *reserve, int *candidates, double *ms, int nmax) {
    if (!b) return set_error(TCP_ERR_BAD_PARAM, "batch is NULL");
    if (reserve) *reserve = b->pair_reserve;
    constexpr int nc = (int)(sizeof kBReserveCandidates / sizeof kBReserveCandidates[0]);
    for (int k = 0; k < nmax && k < nc; ++k) {
        if (candidates) candidates[k] = kBReserveCandidates[k];
        if (ms) ms[k] = b->reserve_ms[k];
    }
    return TCP_OK;
}

int tcp_batch_time_component(tcp_batch *b, int which, int reps, double *ms_per_launch) {
    if (!b || !b->ready) return set_error(TCP_ERR_STATE, "tcp_batch_ewald_self must be called first");
    if (reps <= 0 || !ms_per_launch || which < 0 || which > 1) return set_error(TCP_ERR_BAD_PARAM, "bad arguments");
    cudaSetDevice(b->device);
    int rc;
    if ((rc = b_autotune(b))) return rc;
    const BAcc A = acc_of(b);
    cudaEvent_t e0, e1;
    TCP_CUDA(cudaEventCreate(&e0));
    TCP_CUDA(cudaEventCreate(&e1));
    auto one = [&]() -> int {
        if (which == 0)   // clears its accumulators itself
            return launch_pair_n3_batch(b->stream, b->xq, b->ntot, b->facc, b->n3reps, b->nrep, b->n3_items,
                                        b->n3_chunks, b->n3_nchunks, A.ur, b->status, b->counter, b->num_sms, true,
                                        b->pair_variant);
        TCP_CUDA(cudaMemsetAsync(A.um, 0, sizeof(double) * (size_t)b->nrep, b->stream));
        if (int r = b_recip_fork(b, A)) return r;
        return b_recip_join(b);
    };
    rc = one();   // warm-up
    cudaEventRecord(e0, b->stream);
    for (int r = 0; r < reps && !rc; ++r) rc = one();
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = b_sync(b))) return rc;
    *ms_per_launch = (double)t / reps;
    return TCP_OK;
}

int tcp_batch_time_steps(tcp_batch *b, double dt, int nsteps, int flush_l2, double *out) {
    if (!b || !out || nsteps <= 0) return set_error(TCP_ERR_BAD_PARAM, "bad arguments");
    int rc = tcp_batch_md_steps(b, dt, 1, nullptr);   // builds the graph
    if (rc) return rc;
    if (flush_l2 && !b->l2_flush) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->device);
        b->l2_flush_bytes = 2 * (size_t)std::max(l2, 64 << 20);
        TCP_CUDA(cudaMalloc(&b->l2_flush, b->l2_flush_bytes));
    }
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    for (int s = 0; s < nsteps; ++s) {
        if (flush_l2) TCP_CUDA(cudaMemsetAsync(b->l2_flush, s & 0xff, b->l2_flush_bytes, b->stream));
        TCP_CUDA(cudaGraphLaunch(b->graph, b->stream));
        b->launches += b->graph_kernels;
        TCP_CUDA(cudaEventSynchronize(b->ev[4]));
        // step; first kick (0-1); SPME chains (1-2, stream2); pair launch (1-3,
        // beside the chains); epilogue (from the later of 2 and 3 to 4)
        float t[5], e2, e3;
        cudaEventElapsedTime(&t[0], b->ev[0], b->ev[4]);
        cudaEventElapsedTime(&t[1], b->ev[0], b->ev[1]);
        cudaEventElapsedTime(&t[2], b->ev[1], b->ev[2]);
        cudaEventElapsedTime(&t[3], b->ev[1], b->ev[3]);
        cudaEventElapsedTime(&e2, b->ev[2], b->ev[4]);
        cudaEventElapsedTime(&e3, b->ev[3], b->ev[4]);
        t[4] = std::min(e2, e3);
        for (int k = 0; k < 5; ++k) out[k] += t[k];
        out[5] += 1.0;
    }
    return b_sync(b);
}

}  // extern "C"

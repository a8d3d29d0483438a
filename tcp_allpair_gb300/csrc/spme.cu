// spme.cu -- reciprocal-space sums: smooth PME (Force_SPME4, force.f90:652-929,
// generalised to B-spline order 4..8) and the plain Ewald k-sum.
//
// Mesh layout: Q[iz][iy][ix] (ix fastest, the Fortran order of Q(ix,iy,iz)),
// FP64.  The 3-D FFT is cuFFT D2Z / Z2D on that layout (the only library
// call of the path); spreading (cell-sorted and atomic-free), the
// influence-function multiply fused with the energy reduction, and the force
// gather are kernels of this file.
// In the compensated-FP32 mode the charge mesh is summed in two-float FP32
// and written as FP32 for R2C / C2R transforms, the influence multiply
// (energy summed in FP64) and the force gather: on GB300 FP64 runs at 1/64 of
// the FP32 rate, which makes a 128^3 FP64 transform compute-bound.
// TCP_PREC_FP32C_R64 keeps the FP32C real-space sum and runs this chain in
// FP64 as in TCP_PREC_FP64.
//
// Normalisation: both transforms are unnormalised, so the real mesh after the
// inverse transform is phi = K^3 Qfin of the reference; its 1/K^3 (FFTE
// iopt=+1) and K^3 (force.f90:864-865) cancel, giving
//   Um = eps/(2 pi V) sum_m theta(m) B(m) |S(m)|^2          (force.f90:921)
//   F_i = -eps/(pi V) sum_k dQ(k)/dx_i phi(k)              (force.f90:882-887)
#include <algorithm>
#include <cmath>
#include <vector>

#include "device_util.cuh"
#include "spme_math.cuh"
#include "tcp_internal.h"

namespace tcp {

struct SpmeArgs {
    const double *x;     // SoA [3][n]
    int nel, n;
    double q0, q1;       // scaled charges per species
    double box0, box1, box2;
    double kl0, kl1, kl2;   // K/L: the step's kernels multiply (GB300's FP64 division is slow)
    int K1, K2, K3;
};

// ---- atomic-free charge spreading (cell-sorted) --------------------------------
// A particle's support is the P^3 mesh points from its base index
// b = INT(u)-(P-3) (force.f90:742-744).  Particles are counting-sorted by the
// (y, z) mesh column of their base (bin = by + K2 bz); each bin is put in
// particle-index order and the B-spline weights of every particle are stored
// once, in sorted order.  The spread is then a gather by mesh rows: a warp
// owns ROWS consecutive rows (y0 .. y0 + ROWS - 1, z) in shared memory (ROWS
// = 8, or 4 / 2 on small meshes) and visits, for jz < P, the bins
// (y0 - P + 1 .. y0 + ROWS - 1, z - jz) -- a
// contiguous (or wrapped) range of the sorted list, staged 32 particles at a
// time.  For one particle its lanes cover the P x P points (jy, jx) of plane
// z, so no two lanes and no two warps touch the same point: no atomics, and
// every mesh point is summed in the same order (jz, bins, particle index) on
// every call.  The bin counts and slots come from integer atomics; the sum
// does not depend on them.  FP64 mode adds FP64 products in FP64; FP32C mode
// adds FP32 products in compensated two-float FP32 (TwoSum hi/lo) and writes
// the FP32 mesh read by the FP32 transforms (GB300's FP64 rate is 1/64 of
// FP32).
constexpr int kRows = 8;                 // mesh rows per warp (fewer for small meshes: spread_rows)
constexpr int kRowWarps = 4;             // warps per CTA (fewer when the rows of a large mesh need the space)
constexpr int kScanBlock = 1024;         // bins per block of the prefix sum
constexpr int kSortReg = 8;              // bins up to this size are sorted in registers


template <int P>
__global__ void spme_bin_count_kernel(const SpmeArgs a, SpreadBins b) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.n) return;
    const double L[3] = {a.box0, a.box1, a.box2};
    const double KL[3] = {a.kl0, a.kl1, a.kl2};
    const int K[3] = {a.K1, a.K2, a.K3};
    int base[3];
#pragma unroll
    for (int d = 1; d < 3; ++d) {
        const double u = (a.x[(size_t)d * a.n + m] + L[d] * .5) * KL[d];   // force.f90:700-702, K/L precomputed
        base[d] = wrapi((int)trunc(u) - (P - 3), K[d]);
    }
    const int bin = base[1] + a.K2 * base[2];
    b.rank[m] = atomicAdd(&b.count[bin], 1);
    b.ebx[m] = bin;                      // the bin of particle m (read back by the scatter)
}

// exclusive prefix sum of count[0..nbins) into start[0..nbins], in three steps
__global__ void scan_block_kernel(const int *__restrict__ count, int nbins, int *__restrict__ start,
                                  int *__restrict__ bsum) {
    __shared__ int ws[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < nbins ? count[i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    const int incl = x + (w > 0 ? ws[w - 1] : 0);
    if (i < nbins) start[i] = incl - v;
    if (threadIdx.x == kScanBlock - 1) bsum[blockIdx.x] = incl;
}

// One CTA for up to kScanBlock * kScanPer bins: each thread sums its run of
// consecutive bins, the CTA scans the run sums, and each thread writes its
// run's exclusive prefix; start[nbins] = total.  Above 8,192 bins the runs
// are long enough that the three-launch scan is faster (16,384 bins: 17.7
// against 8.4 us under ncu).
constexpr int kScanPer = 8;
__global__ void __launch_bounds__(kScanBlock) scan_single_kernel(const int *__restrict__ count, int nbins,
                                                                 int *__restrict__ start, int total) {
    __shared__ int ws[32];
    const int per = (nbins + kScanBlock - 1) / kScanBlock;
    const int b0 = min(nbins, (int)threadIdx.x * per), b1 = min(nbins, b0 + per);
    int v = 0;
    for (int k = b0; k < b1; ++k) v += count[k];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    int run = x - v + (w > 0 ? ws[w - 1] : 0);
    for (int k = b0; k < b1; ++k) {
        const int t = count[k];
        start[k] = run;
        run += t;
    }
    if (threadIdx.x == 0) start[nbins] = total;
}

__global__ void scan_sums_kernel(int *__restrict__ bsum, int nblocks) {
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < nblocks; ++k) {
            const int t = bsum[k];
            bsum[k] = acc;
            acc += t;
        }
    }
}

__global__ void scan_add_kernel(int *__restrict__ start, int nbins, const int *__restrict__ bsum, int total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nbins) start[i] += bsum[i / kScanBlock];
    if (i == 0) start[nbins] = total;
}

__global__ void spme_bin_scatter_kernel(int n, SpreadBins b) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    b.list[b.start[b.ebx[m]] + b.rank[m]] = m;
}

// each bin in particle-index order: small bins by a register sorting pass,
// larger ones by insertion sort in place
__global__ void spme_bin_sort_kernel(SpreadBins b, int nbins) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nbins) return;
    const int s = b.start[k], e = b.start[k + 1], cnt = e - s;
    if (cnt <= 1) return;
    if (cnt <= kSortReg) {
        int v[kSortReg];
#pragma unroll
        for (int i = 0; i < kSortReg; ++i) v[i] = i < cnt ? b.list[s + i] : 0x7fffffff;
#pragma unroll
        for (int i = 0; i < kSortReg; ++i)            // odd-even transposition sort
#pragma unroll
            for (int j = i & 1; j + 1 < kSortReg; j += 2)
                if (v[j] > v[j + 1]) {
                    const int t = v[j];
                    v[j] = v[j + 1];
                    v[j + 1] = t;
                }
#pragma unroll
        for (int i = 0; i < kSortReg; ++i)
            if (i < cnt) b.list[s + i] = v[i];
        return;
    }
    for (int i = s + 1; i < e; ++i) {
        const int v = b.list[i];
        int j = i - 1;
        while (j >= s && b.list[j] > v) {
            b.list[j + 1] = b.list[j];
            --j;
        }
        b.list[j + 1] = v;
    }
}

template <int P, typename T>
__global__ void spme_bin_weights_kernel(const SpmeArgs a, SpreadBins b) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= a.n) return;
    const int m = b.list[pos];
    const double L[3] = {a.box0, a.box1, a.box2};
    const double KL[3] = {a.kl0, a.kl1, a.kl2};
    const int K[3] = {a.K1, a.K2, a.K3};
    T *w = static_cast<T *>(b.ew) + (size_t)pos * 3 * P;
    T W[P], dW[P];
    int base[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = (a.x[(size_t)d * a.n + m] + L[d] * .5) * KL[d];
        spline_w<P, T>(u, W, dW);
#pragma unroll
        for (int j = 0; j < P; ++j) w[d * P + j] = W[j];
        base[d] = wrapi((int)trunc(u) - (P - 3), K[d]);
    }
    b.ebx[pos] = base[0];
    b.eby[pos] = base[1];
    static_cast<T *>(b.eq)[pos] = (T)(m < a.nel ? a.q0 : a.q1);
}

// Shared memory of one warp: ROWS rows of hi (T) [and lo (float)] of K1
// points, then 32 staged particles (bx, by, q, weights).
template <int P, typename T, int ROWS = kRows>
__host__ __device__ constexpr size_t row_warp_bytes(int K1) {
    return (size_t)ROWS * K1 * (sizeof(T) + (sizeof(T) == 4 ? 4 : 0)) + 32 * (2 * sizeof(int) + (1 + 3 * P) * sizeof(T));
}

template <int P, typename T, int ROWS>
__global__ void __launch_bounds__(32 * kRowWarps) spme_row_spread_kernel(const SpmeArgs a, const SpreadBins b,
                                                                         double *__restrict__ Q,
                                                                         float *__restrict__ Qf) {
    constexpr bool F32 = sizeof(T) == 4;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ngy = (a.K2 + ROWS - 1) / ROWS;
    const long grp = (long)blockIdx.x * (blockDim.x >> 5) + warp;  // (row group, z)
    if (grp >= (long)ngy * a.K3) return;                          // warp-uniform
    const int y0 = (int)(grp % ngy) * ROWS, z = (int)(grp / ngy);
    const int nrow = min(ROWS, a.K2 - y0);
    unsigned char *base = smem + (size_t)warp * row_warp_bytes<P, T, ROWS>(a.K1);
    T *hi = reinterpret_cast<T *>(base);                            // [ROWS][K1]
    float *lo = reinterpret_cast<float *>(base + (size_t)ROWS * a.K1 * sizeof(T));
    unsigned char *st = base + (size_t)ROWS * a.K1 * (sizeof(T) + (F32 ? 4 : 0));
    T *sw = reinterpret_cast<T *>(st);                              // [32][3P]
    T *sq = sw + 32 * 3 * P;                                        // [32]
    int *sbx = reinterpret_cast<int *>(sq + 32), *sby = sbx + 32;   // [32], [32]
    for (int k = lane; k < ROWS * a.K1; k += 32) {
        hi[k] = (T)0;
        if (F32) lo[k] = 0.f;
    }
    __syncwarp();
    const int nb = nrow + P - 1;                                    // bins by = y0-P+1 .. y0+nrow-1
    for (int jz = 0; jz < P; ++jz) {
        int bz = z - jz;
        bz += bz < 0 ? a.K3 : 0;
        // the by range as at most two contiguous pieces of the sorted list
        int by0 = y0 - P + 1, len0 = nb, len1 = 0;
        if (by0 < 0) {
            by0 += a.K2;
            len0 = min(nb, a.K2 - by0);
            len1 = nb - len0;
        }
        if (nb >= a.K2) {                                           // the range covers every bin
            by0 = 0;
            len0 = a.K2;
            len1 = 0;
        }
        for (int piece = 0; piece < 2; ++piece) {
            const int blo = (piece == 0 ? by0 : 0) + a.K2 * bz, len = piece == 0 ? len0 : len1;
            if (len <= 0) continue;
            const int p0 = b.start[blo], p1 = b.start[blo + len];
            for (int c0 = p0; c0 < p1; c0 += 32) {
                const int ne = min(32, p1 - c0);
                if (lane < ne) {
                    const int pos = c0 + lane;
                    const T *w = static_cast<const T *>(b.ew) + (size_t)pos * 3 * P;
#pragma unroll
                    for (int j = 0; j < 3 * P; ++j) sw[lane * 3 * P + j] = w[j];
                    sq[lane] = static_cast<const T *>(b.eq)[pos];
                    sbx[lane] = b.ebx[pos];
                    sby[lane] = b.eby[pos];
                }
                __syncwarp();
                for (int e = 0; e < ne; ++e) {
                    const T *w = sw + e * 3 * P;
                    const T qz = sq[e] * w[2 * P + jz];
                    const int bx = sbx[e], by = sby[e];
                    for (int l = lane; l < P * P; l += 32) {
                        const int jy = l / P, jx = l - jy * P;
                        int rl = by + jy - y0;                      // owned row of point (jy, jx)
                        rl += rl < 0 ? a.K2 : 0;
                        rl -= rl >= a.K2 ? a.K2 : 0;
                        if (rl < nrow) {
                            int x = bx + jx;
                            x -= x >= a.K1 ? a.K1 : 0;
                            const T v = qz * w[P + jy] * w[jx];
                            const int k = rl * a.K1 + x;
                            if (F32) {
                                const T s = hi[k] + v, bp = s - hi[k];
                                lo[k] += (hi[k] - (s - bp)) + (v - bp);
                                hi[k] = s;
                            } else {
                                hi[k] += v;
                            }
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    for (int k = lane; k < nrow * a.K1; k += 32) {
        const int rl = k / a.K1, x = k - rl * a.K1;
        const size_t g = (size_t)a.K1 * ((y0 + rl) + (size_t)a.K2 * z) + x;
        if (F32) Qf[g] = (float)(hi[k] + lo[k]);
        else Q[g] = (double)hi[k];
    }
}

// Qk *= theta B; energy partial sum_m w_m theta B |Qk|^2 (w = 2 for the
// kx columns that stand for a conjugate pair in the half spectrum).
__global__ void spme_influence_kernel(cufftDoubleComplex *__restrict__ Qk, const double *__restrict__ infl,
                                      long total, int Kh, int K1, double *__restrict__ epart, bool energy) {
    __shared__ double red[32];
    double e = 0.0;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const double g = infl[idx];
        cufftDoubleComplex z = Qk[idx];
        if (energy) {
            const int kx = (int)(idx % Kh);
            const double wgt = (kx == 0 || (2 * kx == K1)) ? 1.0 : 2.0;
            e += wgt * g * (z.x * z.x + z.y * z.y);
        }
        z.x *= g;
        z.y *= g;
        Qk[idx] = z;
    }
    if (energy) {
        const double t = block_sum(e, red);
        if (threadIdx.x == 0) epart[blockIdx.x] = t;
    }
}

// force gather, force.f90:868-919.  T = double (FP64 mode) or float (FP32C
// mode: FP32 mesh and weights, the per-particle sum in FP32, force in FP64).
template <int P, typename T>
__global__ void spme_gather_kernel(const SpmeArgs a, const T *__restrict__ phi, double coef,
                                   double *__restrict__ frec, const int *__restrict__ order) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    // particles in the cell-sort order of the spread: the lanes of a warp share
    // their (y, z) mesh columns, so their mesh rows are read together
    const int m = order ? order[t] : t;
    const double q = m < a.nel ? a.q0 : a.q1;
    const double L[3] = {a.box0, a.box1, a.box2};
    const double KL[3] = {a.kl0, a.kl1, a.kl2};
    const int K[3] = {a.K1, a.K2, a.K3};
    T W[3][P], dW[3][P];
    int base[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = (a.x[(size_t)d * a.n + m] + L[d] * .5) * KL[d];
        spline_w<P, T>(u, W[d], dW[d]);
        base[d] = wrapi((int)trunc(u) - (P - 3), K[d]);    // first mesh index, wrapped once
    }
    T gx = 0, gy = 0, gz = 0;
    int iz = base[2];
#pragma unroll 1
    for (int k = 0; k < P; ++k) {
        int iy = base[1];
#pragma unroll 1
        for (int j = 0; j < P; ++j) {
            const T *row = phi + (size_t)a.K1 * (iy + (size_t)a.K2 * iz);
            T sx = 0, sd = 0;
            int ix = base[0];
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const T ph = row[ix];
                sx += dW[0][i] * ph;
                sd += W[0][i] * ph;
                ix = ix + 1 == a.K1 ? 0 : ix + 1;
            }
            gx += sx * W[1][j] * W[2][k];
            gy += sd * dW[1][j] * W[2][k];
            gz += sd * W[1][j] * dW[2][k];
            iy = iy + 1 == a.K2 ? 0 : iy + 1;
        }
        iz = iz + 1 == a.K3 ? 0 : iz + 1;
    }
    // F = -eps/(pi V) q (K_d/L_d) sum dW W W phi
    frec[m] = -coef * q * (double)gx * a.kl0;
    frec[(size_t)a.n + m] = -coef * q * (double)gy * a.kl1;
    frec[2 * (size_t)a.n + m] = -coef * q * (double)gz * a.kl2;
}

// FP32C influence multiply.  Energy terms are summed in FP32 per thread (a
// few elements each) and in FP64 across threads and blocks.  The half-spectrum
// column kx of element idx advances by the grid stride modulo Kh, so no
// division runs per element.
__global__ void spme_influence_f_kernel(cufftComplex *__restrict__ Qk, const float *__restrict__ infl, int total,
                                        int Kh, int K1, double *__restrict__ epart, bool energy) {
    __shared__ double red[32];
    float e = 0.0f;
    const int stride = gridDim.x * blockDim.x;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    int kx = idx % Kh;
    const int dkx = stride % Kh;
    for (; idx < total; idx += stride) {
        const float g = infl[idx];
        cufftComplex z = Qk[idx];
        if (energy) {
            const float wgt = (kx == 0 || (2 * kx == K1)) ? 1.0f : 2.0f;
            e = fmaf(wgt * g, fmaf(z.x, z.x, z.y * z.y), e);
        }
        z.x *= g;
        z.y *= g;
        Qk[idx] = z;
        kx += dkx;
        if (kx >= Kh) kx -= Kh;
    }
    if (energy) {
        const double t = block_sum((double)e, red);
        if (threadIdx.x == 0) epart[blockIdx.x] = t;
    }
}

__global__ void sum_partials_kernel(const double *__restrict__ part, int np, double scale,
                                    double *__restrict__ out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = s * scale;
}

// ---- plain Ewald k-sum ------------------------------------------------------
// S(m) = sum_j q_j exp(2 pi i m.x_j) per k-vector (one CTA per vector)
__global__ void ewald_sfac_kernel(const double *__restrict__ x, int nel, int n, double q0, double q1,
                                  const double *__restrict__ kvec, double *__restrict__ ksum,
                                  double *__restrict__ epart) {
    __shared__ double red[32];
    const double mx = kvec[4 * blockIdx.x], my = kvec[4 * blockIdx.x + 1], mz = kvec[4 * blockIdx.x + 2];
    double sr = 0.0, si = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double q = j < nel ? q0 : q1;
        const double ph = 2.0 * kPi * (mx * x[j] + my * x[(size_t)n + j] + mz * x[2 * (size_t)n + j]);
        double s, c;
        sincos(ph, &s, &c);
        sr += q * c;
        si += q * s;
    }
    sr = block_sum(sr, red);
    si = block_sum(si, red);
    if (threadIdx.x == 0) {
        ksum[2 * blockIdx.x] = sr;
        ksum[2 * blockIdx.x + 1] = si;
        epart[blockIdx.x] = kvec[4 * blockIdx.x + 3] * (sr * sr + si * si);
    }
}

// F_i = (2 eps q_i / V) sum_m theta m Im(conj(S) e^{i phase})
__global__ void ewald_force_kernel(const double *__restrict__ x, int nel, int n, double q0, double q1,
                                   const double *__restrict__ kvec, const double *__restrict__ ksum, int nk,
                                   double coef, double *__restrict__ frec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double q = i < nel ? q0 : q1;
    const double xi = x[i], yi = x[(size_t)n + i], zi = x[2 * (size_t)n + i];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int k = 0; k < nk; ++k) {
        const double mx = kvec[4 * k], my = kvec[4 * k + 1], mz = kvec[4 * k + 2], th = kvec[4 * k + 3];
        double s, c;
        sincos(2.0 * kPi * (mx * xi + my * yi + mz * zi), &s, &c);
        const double im = (ksum[2 * k] * s - ksum[2 * k + 1] * c) * th;
        fx += im * mx;
        fy += im * my;
        fz += im * mz;
    }
    frec[i] = coef * q * fx;
    frec[(size_t)n + i] = coef * q * fy;
    frec[2 * (size_t)n + i] = coef * q * fz;
}

// ---------------------------------------------------------------------------
static double bspline_M(int n, double y) {
    if (y <= 0.0 || y >= (double)n) return 0.0;
    if (n == 2) return 1.0 - std::fabs(y - 1.0);
    return (y * bspline_M(n - 1, y) + ((double)n - y) * bspline_M(n - 1, y - 1.0)) / (double)(n - 1);
}

// |b(m)|^-2 per axis (36/(4+2cos)^2 for order 4, force.f90:834-839); odd
// orders vanish at the Nyquist index, where the mean of the neighbours is used.
std::vector<double> bspline_moduli(int order, int K) {
    std::vector<double> den(K), out(K);
    for (int m = 0; m < K; ++m) {
        if (order == 4) {
            const double z = 4.0 + 2.0 * std::cos(2.0 * kPi * m / K);
            den[m] = z * z / 36.0;
            continue;
        }
        double re = 0.0, im = 0.0;
        for (int k = 0; k <= order - 2; ++k) {
            const double mk = bspline_M(order, (double)(k + 1));
            re += mk * std::cos(2.0 * kPi * m * k / K);
            im += mk * std::sin(2.0 * kPi * m * k / K);
        }
        den[m] = re * re + im * im;
    }
    for (int m = 0; m < K; ++m)
        if (den[m] < 1e-7) den[m] = 0.5 * (den[(m - 1 + K) % K] + den[(m + 1) % K]);
    for (int m = 0; m < K; ++m) out[m] = 1.0 / den[m];
    return out;
}

int spme_free(tcp_ctx *c) {
    if (c->plans) {
        cufftDestroy(c->plan_f);
        cufftDestroy(c->plan_b);
        c->plans = false;
    }
    int **ib[] = {&c->bin_count, &c->bin_start, &c->bin_bsum, &c->bin_rank, &c->bin_list, &c->bin_ebx, &c->bin_eby};
    for (int **q : ib) {
        cudaFree(*q);
        *q = nullptr;
    }
    cudaFree(c->bin_ew);
    cudaFree(c->bin_eq);
    c->bin_ew = c->bin_eq = nullptr;
    cudaFree(c->Q);
    cudaFree(c->Qk);
    cudaFree(c->infl);
    cudaFree(c->Qf);
    cudaFree(c->Qkf);
    cudaFree(c->infl_f);
    c->Q = nullptr;
    c->Qk = nullptr;
    c->infl = nullptr;
    c->Qf = nullptr;
    c->Qkf = nullptr;
    c->infl_f = nullptr;
    return TCP_OK;
}

// blocks of 256 threads for the influence multiply: about four elements per
// thread, at most 4096 blocks (the size of the energy partial array)
static int spme_energy_blocks(const tcp_ctx *c) {
    const long total = (long)c->K3 * c->K2 * c->Kh;
    return (int)std::max<long>(1, std::min<long>((total + 1023) / 1024, 4096));
}

static int prepare_cell_spread(tcp_ctx *c);

int spme_setup(tcp_ctx *c) {
    const tcp_params &p = c->p;
    c->K1 = p.K[0];
    c->K2 = p.K[1];
    c->K3 = p.K[2];
    c->Kh = c->K1 / 2 + 1;
    const size_t nreal = (size_t)c->K1 * c->K2 * c->K3;
    const size_t nhalf = (size_t)c->Kh * c->K2 * c->K3;
    c->spme_fp32 = c->p.precision == TCP_PREC_FP32C && !c->recip_fp64;
    if (!c->Q) {
        const size_t nbins = (size_t)c->K2 * c->K3;
        if (cudaMalloc(&c->bin_count, sizeof(int) * (nbins + 1)) != cudaSuccess ||
            cudaMalloc(&c->bin_start, sizeof(int) * (nbins + 1)) != cudaSuccess ||
            cudaMalloc(&c->bin_bsum, sizeof(int) * ((nbins + kScanBlock - 1) / kScanBlock)) != cudaSuccess ||
            cudaMalloc(&c->bin_rank, sizeof(int) * (size_t)c->n) != cudaSuccess ||
            cudaMalloc(&c->bin_list, sizeof(int) * (size_t)c->n) != cudaSuccess ||
            cudaMalloc(&c->bin_ebx, sizeof(int) * (size_t)c->n) != cudaSuccess ||
            cudaMalloc(&c->bin_eby, sizeof(int) * (size_t)c->n) != cudaSuccess ||
            cudaMalloc(&c->bin_ew, sizeof(double) * 3 * kMaxOrder * (size_t)c->n) != cudaSuccess ||
            cudaMalloc(&c->bin_eq, sizeof(double) * (size_t)c->n) != cudaSuccess ||
            cudaMalloc(&c->Q, sizeof(double) * nreal) != cudaSuccess ||
            cudaMalloc(&c->Qk, sizeof(cufftDoubleComplex) * nhalf) != cudaSuccess ||
            cudaMalloc(&c->infl, sizeof(double) * nhalf) != cudaSuccess)
            return set_error(TCP_ERR_NOMEM, "SPME mesh allocation failed");
        if (c->spme_fp32 && (cudaMalloc(&c->Qf, sizeof(float) * nreal) != cudaSuccess ||
                             cudaMalloc(&c->Qkf, sizeof(cufftComplex) * nhalf) != cudaSuccess ||
                             cudaMalloc(&c->infl_f, sizeof(float) * nhalf) != cudaSuccess))
            return set_error(TCP_ERR_NOMEM, "SPME FP32 mesh allocation failed");
    }
    if (!c->plans) {
        if (inject_fault("cufft_plan")) return set_error(TCP_ERR_CUFFT, "injected: cufftPlan3d failed");
        const cufftType tf = c->spme_fp32 ? CUFFT_R2C : CUFFT_D2Z;
        const cufftType tb = c->spme_fp32 ? CUFFT_C2R : CUFFT_Z2D;
        if (cufftPlan3d(&c->plan_f, c->K3, c->K2, c->K1, tf) != CUFFT_SUCCESS)
            return set_error(TCP_ERR_CUFFT, "cufftPlan3d forward failed");
        if (cufftPlan3d(&c->plan_b, c->K3, c->K2, c->K1, tb) != CUFFT_SUCCESS) {
            cufftDestroy(c->plan_f);
            return set_error(TCP_ERR_CUFFT, "cufftPlan3d inverse failed");
        }
        cufftSetStream(c->plan_f, c->stream);
        cufftSetStream(c->plan_b, c->stream);
        c->plans = true;
    }
    if (int rc = prepare_cell_spread(c)) return rc;
    // theta(m) = exp(-pi^2 m^2/a^2)/m^2 (EWALD_SELF, force.f90:27-42) times
    // the B-spline moduli, on the half spectrum; theta(0) = 0.
    std::vector<double> bx = bspline_moduli(p.order, c->K1), by = bspline_moduli(p.order, c->K2),
                        bz = bspline_moduli(p.order, c->K3);
    std::vector<double> h(nhalf);
    const double a2 = c->alpha * c->alpha;
    for (int k = 0; k < c->K3; ++k) {
        const int iz = (k + c->K3 / 2) % c->K3 - c->K3 / 2;
        for (int j = 0; j < c->K2; ++j) {
            const int iy = (j + c->K2 / 2) % c->K2 - c->K2 / 2;
            for (int i = 0; i < c->Kh; ++i) {
                const int ix = (i + c->K1 / 2) % c->K1 - c->K1 / 2;
                const size_t idx = i + (size_t)c->Kh * (j + (size_t)c->K2 * k);
                if (ix == 0 && iy == 0 && iz == 0) {
                    h[idx] = 0.0;
                    continue;
                }
                const double m2 = (double)ix * ix / (p.box[0] * p.box[0]) + (double)iy * iy / (p.box[1] * p.box[1]) +
                                  (double)iz * iz / (p.box[2] * p.box[2]);
                h[idx] = std::exp(-m2 * kPi * kPi / a2) / m2 * bx[i] * by[j] * bz[k];
            }
        }
    }
    TCP_CUDA(cudaMemcpyAsync(c->infl, h.data(), sizeof(double) * nhalf, cudaMemcpyHostToDevice, c->stream));
    if (c->spme_fp32) {
        std::vector<float> hf(h.begin(), h.end());
        TCP_CUDA(cudaMemcpyAsync(c->infl_f, hf.data(), sizeof(float) * nhalf, cudaMemcpyHostToDevice, c->stream));
        TCP_CUDA(cudaStreamSynchronize(c->stream));
    }
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

static SpmeArgs spme_args(const tcp_ctx *c) {
    SpmeArgs a;
    a.x = c->x;
    a.nel = c->nel;
    a.n = c->n;
    a.q0 = c->p.charge_scale * c->p.q[0];
    a.q1 = c->p.charge_scale * c->p.q[1];
    a.box0 = c->p.box[0];
    a.box1 = c->p.box[1];
    a.box2 = c->p.box[2];
    a.K1 = c->K1;
    a.K2 = c->K2;
    a.K3 = c->K3;
    a.kl0 = (double)c->K1 / c->p.box[0];
    a.kl1 = (double)c->K2 / c->p.box[1];
    a.kl2 = (double)c->K3 / c->p.box[2];
    return a;
}

// prefix sum of the bin counts, placement by the counting-sort slots, and
// each bin in particle-index order (shared by the single-system and batched paths)
int launch_bin_sort(cudaStream_t st, int n, int nbins, const SpreadBins &b) {
    const int threads = 256;
    const int sblocks = (nbins + kScanBlock - 1) / kScanBlock;
    const bool single = nbins <= kScanBlock * kScanPer;   // up to 8,192 (y, z) columns: one launch
    if (single) {
        scan_single_kernel<<<1, kScanBlock, 0, st>>>(b.count, nbins, b.start, n);
    } else {
        scan_block_kernel<<<sblocks, kScanBlock, 0, st>>>(b.count, nbins, b.start, b.bsum);
        scan_sums_kernel<<<1, 32, 0, st>>>(b.bsum, sblocks);
        scan_add_kernel<<<(nbins + threads - 1) / threads, threads, 0, st>>>(b.start, nbins, b.bsum, n);
    }
    spme_bin_scatter_kernel<<<(n + threads - 1) / threads, threads, 0, st>>>(n, b);
    spme_bin_sort_kernel<<<(nbins + threads - 1) / threads, threads, 0, st>>>(b, nbins);
    return single ? 3 : 5;
}

int bin_scan_block() { return kScanBlock; }

// atomic-free spread into Q (FP64) or straight into Qf (FP32C mode)
static SpreadBins spread_bins(tcp_ctx *c) {
    SpreadBins b;
    b.count = c->bin_count;
    b.start = c->bin_start;
    b.bsum = c->bin_bsum;
    b.rank = c->bin_rank;
    b.list = c->bin_list;
    b.ebx = c->bin_ebx;
    b.eby = c->bin_eby;
    b.ew = c->bin_ew;
    b.eq = c->bin_eq;
    return b;
}

// Mesh rows per warp of the spread: 8, or 4 / 2 on meshes of fewer (y, z)
// columns, so that the kernel keeps about 2,048 warps (13 per SM) where a
// small mesh would leave a few warps per SM with long serial loops.  A warp
// visits the particles of ROWS + P - 1 bin rows for ROWS mesh rows.
static int spread_rows(const tcp_ctx *c) {
    const long cols = (long)c->K2 * c->K3;
    return cols >= 16384 ? kRows : (cols >= 8192 ? 4 : 2);
}

template <int P, typename T, int ROWS>
static void launch_row_spread(tcp_ctx *c, const SpmeArgs &a, const SpreadBins &b, double *Q, float *Qf) {
    const long groups = (long)((c->K2 + ROWS - 1) / ROWS) * c->K3;
    const size_t per_warp = row_warp_bytes<P, T, ROWS>(c->K1);
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(kRowWarps, (200u << 10) / per_warp));
    const size_t sm = warps * per_warp;
    const int rblocks = (int)((groups + warps - 1) / warps);
    spme_row_spread_kernel<P, T, ROWS><<<rblocks, 32 * warps, sm, c->rstream>>>(a, b, Q, Qf);
}

template <int P>
static int launch_cell_spread(tcp_ctx *c, const SpmeArgs &a, double *Q, float *Qf) {
    const SpreadBins b = spread_bins(c);
    const int threads = 256, pblocks = (c->n + threads - 1) / threads;
    const int nbins = c->K2 * c->K3;
    TCP_CUDA(cudaMemsetAsync(c->bin_count, 0, sizeof(int) * (size_t)nbins, c->rstream));
    spme_bin_count_kernel<P><<<pblocks, threads, 0, c->rstream>>>(a, b);
    const int sort_kernels = launch_bin_sort(c->rstream, c->n, nbins, b);
    if (Qf) {
        spme_bin_weights_kernel<P, float><<<pblocks, threads, 0, c->rstream>>>(a, b);
        switch (spread_rows(c)) {
            case 2: launch_row_spread<P, float, 2>(c, a, b, nullptr, Qf); break;
            case 4: launch_row_spread<P, float, 4>(c, a, b, nullptr, Qf); break;
            default: launch_row_spread<P, float, kRows>(c, a, b, nullptr, Qf); break;
        }
    } else {
        spme_bin_weights_kernel<P, double><<<pblocks, threads, 0, c->rstream>>>(a, b);
        switch (spread_rows(c)) {
            case 2: launch_row_spread<P, double, 2>(c, a, b, Q, nullptr); break;
            case 4: launch_row_spread<P, double, 4>(c, a, b, Q, nullptr); break;
            default: launch_row_spread<P, double, kRows>(c, a, b, Q, nullptr); break;
        }
    }
    c->launches += 3 + sort_kernels;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

// shared-memory limits of the spread kernels for this mesh (set once, outside
// any stream capture; a launch uses at most kRowWarps warps' worth)
template <int P, typename T, int ROWS>
static int prepare_row_spread(tcp_ctx *c) {
    const size_t s = std::min<size_t>(kRowWarps * row_warp_bytes<P, T, ROWS>(c->K1), 200u << 10);
    TCP_CUDA(cudaFuncSetAttribute(spme_row_spread_kernel<P, T, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::max(s, row_warp_bytes<P, T, ROWS>(c->K1))));
    return TCP_OK;
}

template <int P>
static int prepare_cell_spread_p(tcp_ctx *c) {
    for (int rc : {prepare_row_spread<P, float, 2>(c), prepare_row_spread<P, float, 4>(c),
                   prepare_row_spread<P, float, kRows>(c), prepare_row_spread<P, double, 2>(c),
                   prepare_row_spread<P, double, 4>(c), prepare_row_spread<P, double, kRows>(c)})
        if (rc) return rc;
    return TCP_OK;
}

static int prepare_cell_spread(tcp_ctx *c) {
    switch (c->p.order) {
        case 4: return prepare_cell_spread_p<4>(c);
        case 5: return prepare_cell_spread_p<5>(c);
        case 6: return prepare_cell_spread_p<6>(c);
        case 7: return prepare_cell_spread_p<7>(c);
        default: return prepare_cell_spread_p<8>(c);
    }
}

static int cell_spread(tcp_ctx *c, const SpmeArgs &a, double *Q, float *Qf) {
    switch (c->p.order) {
        case 4: return launch_cell_spread<4>(c, a, Q, Qf);
        case 5: return launch_cell_spread<5>(c, a, Q, Qf);
        case 6: return launch_cell_spread<6>(c, a, Q, Qf);
        case 7: return launch_cell_spread<7>(c, a, Q, Qf);
        default: return launch_cell_spread<8>(c, a, Q, Qf);
    }
}

template <int P>
static void launch_gather(tcp_ctx *c, const SpmeArgs &a, double coef) {
    const int threads = 128, blocks = (c->n + threads - 1) / threads;
    const int *order = c->bin_list;      // the spread of this chain sorted the particles
    if (c->spme_fp32)
        spme_gather_kernel<P, float><<<blocks, threads, 0, c->rstream>>>(a, c->Qf, coef, c->frec, order);
    else
        spme_gather_kernel<P, double><<<blocks, threads, 0, c->rstream>>>(a, c->Q, coef, c->frec, order);
}

static void gather(tcp_ctx *c, const SpmeArgs &a, double coef) {
    switch (c->p.order) {
        case 4: launch_gather<4>(c, a, coef); break;
        case 5: launch_gather<5>(c, a, coef); break;
        case 6: launch_gather<6>(c, a, coef); break;
        case 7: launch_gather<7>(c, a, coef); break;
        default: launch_gather<8>(c, a, coef); break;
    }
}

// the red[] region after the force and kinetic partials holds the energy partials
double *recip_epart(tcp_ctx *c);

int launch_spme(tcp_ctx *c, bool energy) {
    const SpmeArgs a = spme_args(c);
    // charge accumulation, atomic-free (every mesh point is written)
    int rcs = cell_spread(c, a, c->spme_fp32 ? nullptr : c->Q, c->spme_fp32 ? c->Qf : nullptr);
    if (rcs) return rcs;
    const long total = (long)c->K3 * c->K2 * c->Kh;
    const int eb = spme_energy_blocks(c);
    double *epart = recip_epart(c);
    cufftSetStream(c->plan_f, c->rstream);
    cufftSetStream(c->plan_b, c->rstream);
    if (c->spme_fp32) {
        if (cufftExecR2C(c->plan_f, c->Qf, c->Qkf) != CUFFT_SUCCESS) return set_error(TCP_ERR_CUFFT, "cufftExecR2C failed");
        spme_influence_f_kernel<<<eb, 256, 0, c->rstream>>>(c->Qkf, c->infl_f, (int)total, c->Kh, c->K1, epart, energy);
        c->launches++;
        if (cufftExecC2R(c->plan_b, c->Qkf, c->Qf) != CUFFT_SUCCESS) return set_error(TCP_ERR_CUFFT, "cufftExecC2R failed");
    } else {
        if (cufftExecD2Z(c->plan_f, c->Q, c->Qk) != CUFFT_SUCCESS) return set_error(TCP_ERR_CUFFT, "cufftExecD2Z failed");
        spme_influence_kernel<<<eb, 256, 0, c->rstream>>>(c->Qk, c->infl, total, c->Kh, c->K1, epart, energy);
        c->launches++;
        if (cufftExecZ2D(c->plan_b, c->Qk, c->Q) != CUFFT_SUCCESS) return set_error(TCP_ERR_CUFFT, "cufftExecZ2D failed");
    }
    gather(c, a, kEps / (kPi * c->V));
    c->launches++;
    if (energy) {
        sum_partials_kernel<<<1, 1024, 0, c->rstream>>>(epart, eb, kEps / (2.0 * kPi * c->V), c->scal + kScalUm);
        c->launches++;
    }
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

int ewald_setup(tcp_ctx *c) {
    const tcp_params &p = c->p;
    const int nmax2 = p.ewald_nmax2;
    const int nm = (int)std::floor(std::sqrt((double)nmax2));
    std::vector<double> kv;
    for (int n3 = -nm; n3 <= nm; ++n3)
        for (int n2 = -nm; n2 <= nm; ++n2)
            for (int n1 = -nm; n1 <= nm; ++n1) {
                const int nn = n1 * n1 + n2 * n2 + n3 * n3;
                if (nn == 0 || nn > nmax2) continue;
                const double m[3] = {n1 / p.box[0], n2 / p.box[1], n3 / p.box[2]};
                const double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
                kv.push_back(m[0]);
                kv.push_back(m[1]);
                kv.push_back(m[2]);
                kv.push_back(std::exp(-m2 * kPi * kPi / (c->alpha * c->alpha)) / m2);
            }
    c->nk = (int)(kv.size() / 4);
    if (c->nk > c->red_cap - 7 * kick_blocks(c->n))
        return set_error(TCP_ERR_BAD_PARAM, "ewald_nmax2 too large: more k-vectors than the energy buffer holds");
    cudaFree(c->kvec);
    cudaFree(c->ksum);
    cudaFree(c->kS4);
    c->kvec = nullptr;
    c->ksum = nullptr;
    c->kS4 = nullptr;
    if (c->nk == 0) return TCP_OK;
    TCP_CUDA(cudaMalloc(&c->kvec, sizeof(double) * kv.size()));
    TCP_CUDA(cudaMalloc(&c->ksum, sizeof(double) * 2 * (size_t)c->nk));
    TCP_CUDA(cudaMemcpyAsync(c->kvec, kv.data(), sizeof(double) * kv.size(), cudaMemcpyHostToDevice, c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int launch_ewald(tcp_ctx *c, bool energy) {
    if (c->nk == 0) {
        TCP_CUDA(cudaMemsetAsync(c->frec, 0, sizeof(double) * 3 * (size_t)c->n, c->rstream));
        TCP_CUDA(cudaMemsetAsync(c->scal + kScalUm, 0, sizeof(double), c->rstream));
        return TCP_OK;
    }
    const double q0 = c->p.charge_scale * c->p.q[0], q1 = c->p.charge_scale * c->p.q[1];
    double *epart = recip_epart(c);
    ewald_sfac_kernel<<<c->nk, 256, 0, c->rstream>>>(c->x, c->nel, c->n, q0, q1, c->kvec, c->ksum, epart);
    ewald_force_kernel<<<(c->n + 127) / 128, 128, 0, c->rstream>>>(c->x, c->nel, c->n, q0, q1, c->kvec, c->ksum,
                                                                  c->nk, 2.0 * kEps / c->V, c->frec);
    c->launches += 2;
    if (energy) {
        sum_partials_kernel<<<1, 1024, 0, c->rstream>>>(epart, c->nk, kEps / (2.0 * kPi * c->V), c->scal + kScalUm);
        c->launches++;
    }
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

// ---- reciprocal-space Hessian-vector products -------------------------------
// With Q(k) = sum_j q_j W_j(k), phi = A Q (the convolution of launch_spme) and
// E = c/2 Q.phi, c = eps/(pi V):
//   (H w)_i = c q_i [sum_k (hess W_i(k) w_i) phi(k) + sum_k grad W_i(k) dphi(k)],
//   dphi = A dQ, dQ(k) = sum_j q_j grad W_j(k) . w_j.
// Always FP64 (meshes hQ / hdQ, own D2Z / Z2D plans), whatever the precision
// of the force path.

// dQ(k) += q_j grad W_j(k) . w_j
template <int P>
__global__ void spme_spread_dipole_kernel(const SpmeArgs a, const double *__restrict__ w, double *__restrict__ dQ) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.n) return;
    const double q = m < a.nel ? a.q0 : a.q1;
    const double L[3] = {a.box0, a.box1, a.box2};
    const int K[3] = {a.K1, a.K2, a.K3};
    double W[3][P], dW[3][P];
    int base[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = (double)K[d] * (a.x[(size_t)d * a.n + m] + L[d] * .5) / L[d];
        spline_w<P, double>(u, W[d], dW[d]);
        base[d] = (int)trunc(u) - (P - 3);
    }
    const double wx = q * w[m] * ((double)a.K1 / a.box0), wy = q * w[(size_t)a.n + m] * ((double)a.K2 / a.box1),
                 wz = q * w[2 * (size_t)a.n + m] * ((double)a.K3 / a.box2);
#pragma unroll 1
    for (int k = 0; k < P; ++k) {
        const int iz = wrapi(base[2] + k, a.K3);
#pragma unroll 1
        for (int j = 0; j < P; ++j) {
            const int iy = wrapi(base[1] + j, a.K2);
            const double cx = wx * W[1][j] * W[2][k];
            const double cyz = wy * dW[1][j] * W[2][k] + wz * W[1][j] * dW[2][k];
            double *row = dQ + (size_t)a.K1 * (iy + (size_t)a.K2 * iz);
#pragma unroll
            for (int i = 0; i < P; ++i) atomicAdd(row + wrapi(base[0] + i, a.K1), cx * dW[0][i] + cyz * W[0][i]);
        }
    }
}

template <int P>
__global__ void spme_gather_hvp_kernel(const SpmeArgs a, const double *__restrict__ phi,
                                       const double *__restrict__ dphi, const double *__restrict__ w, double coef,
                                       double *__restrict__ hw) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.n) return;
    const double q = m < a.nel ? a.q0 : a.q1;
    const double L[3] = {a.box0, a.box1, a.box2};
    const int K[3] = {a.K1, a.K2, a.K3};
    double W[3][P], dW[3][P], d2W[3][P];
    int base[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = (double)K[d] * (a.x[(size_t)d * a.n + m] + L[d] * .5) / L[d];
        spline_w2<P>(u, W[d], dW[d], d2W[d]);
        const double kl = (double)K[d] / L[d];
#pragma unroll
        for (int j = 0; j < P; ++j) {
            dW[d][j] *= kl;
            d2W[d][j] *= kl * kl;
        }
        base[d] = (int)trunc(u) - (P - 3);
    }
    const double w0 = w[m], w1 = w[(size_t)a.n + m], w2 = w[2 * (size_t)a.n + m];
    double h0 = 0.0, h1 = 0.0, h2 = 0.0;
#pragma unroll 1
    for (int k = 0; k < P; ++k) {
        const int iz = wrapi(base[2] + k, a.K3);
#pragma unroll 1
        for (int j = 0; j < P; ++j) {
            const int iy = wrapi(base[1] + j, a.K2);
            const size_t ro = (size_t)a.K1 * (iy + (size_t)a.K2 * iz);
            // per row: sums over i of W, dW, d2W times phi and dphi
            double sp = 0, sdp = 0, sd2p = 0, sq = 0, sdq = 0;
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const size_t idx = ro + wrapi(base[0] + i, a.K1);
                const double ph = phi[idx], dph = dphi[idx];
                sp += W[0][i] * ph;
                sdp += dW[0][i] * ph;
                sd2p += d2W[0][i] * ph;
                sq += W[0][i] * dph;
                sdq += dW[0][i] * dph;
            }
            const double Wy = W[1][j], dWy = dW[1][j], d2Wy = d2W[1][j];
            const double Wz = W[2][k], dWz = dW[2][k], d2Wz = d2W[2][k];
            // Hessian of W x gradient rows, times w, times phi; gradient times dphi
            const double hxx = sd2p * Wy * Wz, hyy = sp * d2Wy * Wz, hzz = sp * Wy * d2Wz;
            const double hxy = sdp * dWy * Wz, hxz = sdp * Wy * dWz, hyz = sp * dWy * dWz;
            h0 += hxx * w0 + hxy * w1 + hxz * w2 + sdq * Wy * Wz;
            h1 += hxy * w0 + hyy * w1 + hyz * w2 + sq * dWy * Wz;
            h2 += hxz * w0 + hyz * w1 + hzz * w2 + sq * Wy * dWz;
        }
    }
    hw[m] += coef * q * h0;
    hw[(size_t)a.n + m] += coef * q * h1;
    hw[2 * (size_t)a.n + m] += coef * q * h2;
}

template <int P>
static void launch_hvp_kernels(tcp_ctx *c, const SpmeArgs &a, const double *w, double *hw, int which) {
    const int threads = 128, blocks = (c->n + threads - 1) / threads;
    if (which == 0) (void)launch_cell_spread<P>(c, a, c->hQ, nullptr);
    else if (which == 1) spme_spread_dipole_kernel<P><<<blocks, threads, 0, c->stream>>>(a, w, c->hdQ);
    else spme_gather_hvp_kernel<P><<<blocks, threads, 0, c->stream>>>(a, c->hQ, c->hdQ, w, kEps / (kPi * c->V), hw);
}

static void hvp_kernels(tcp_ctx *c, const SpmeArgs &a, const double *w, double *hw, int which) {
    switch (c->p.order) {
        case 4: launch_hvp_kernels<4>(c, a, w, hw, which); break;
        case 5: launch_hvp_kernels<5>(c, a, w, hw, which); break;
        case 6: launch_hvp_kernels<6>(c, a, w, hw, which); break;
        case 7: launch_hvp_kernels<7>(c, a, w, hw, which); break;
        default: launch_hvp_kernels<8>(c, a, w, hw, which); break;
    }
}

void spme_hvp_free(tcp_ctx *c) {
    if (c->hplans) {
        cufftDestroy(c->hplan_f);
        cufftDestroy(c->hplan_b);
        c->hplans = false;
    }
    cudaFree(c->hQ);
    cudaFree(c->hdQ);
    cudaFree(c->hQk);
    cudaFree(c->kS4);
    c->hQ = c->hdQ = nullptr;
    c->hQk = nullptr;
    c->kS4 = nullptr;
}

int launch_spme_hvp(tcp_ctx *c, const double *w, double *hw) {
    const size_t nreal = (size_t)c->K1 * c->K2 * c->K3;
    const size_t nhalf = (size_t)c->Kh * c->K2 * c->K3;
    if (!c->hQ) {
        if (cudaMalloc(&c->hQ, sizeof(double) * nreal) != cudaSuccess ||
            cudaMalloc(&c->hdQ, sizeof(double) * nreal) != cudaSuccess ||
            cudaMalloc(&c->hQk, sizeof(cufftDoubleComplex) * nhalf) != cudaSuccess)
            return set_error(TCP_ERR_NOMEM, "SPME Hessian mesh allocation failed");
    }
    if (!c->hplans) {
        if (cufftPlan3d(&c->hplan_f, c->K3, c->K2, c->K1, CUFFT_D2Z) != CUFFT_SUCCESS)
            return set_error(TCP_ERR_CUFFT, "cufftPlan3d D2Z failed");
        if (cufftPlan3d(&c->hplan_b, c->K3, c->K2, c->K1, CUFFT_Z2D) != CUFFT_SUCCESS) {
            cufftDestroy(c->hplan_f);
            return set_error(TCP_ERR_CUFFT, "cufftPlan3d Z2D failed");
        }
        cufftSetStream(c->hplan_f, c->stream);
        cufftSetStream(c->hplan_b, c->stream);
        c->hplans = true;
    }
    const SpmeArgs a = spme_args(c);
    const long total = (long)nhalf;
    const int eb = spme_energy_blocks(c);
    double *mesh[2] = {c->hQ, c->hdQ};
    for (int pass = 0; pass < 2; ++pass) {    // phi = A Q, then dphi = A dQ
        if (pass == 1) TCP_CUDA(cudaMemsetAsync(mesh[pass], 0, sizeof(double) * nreal, c->stream));
        hvp_kernels(c, a, w, hw, pass);
        if (cufftExecD2Z(c->hplan_f, mesh[pass], c->hQk) != CUFFT_SUCCESS) return set_error(TCP_ERR_CUFFT, "cufftExecD2Z failed");
        spme_influence_kernel<<<eb, 256, 0, c->stream>>>(c->hQk, c->infl, total, c->Kh, c->K1, nullptr, false);
        if (cufftExecZ2D(c->hplan_b, c->hQk, mesh[pass]) != CUFFT_SUCCESS) return set_error(TCP_ERR_CUFFT, "cufftExecZ2D failed");
        c->launches += 2;
    }
    hvp_kernels(c, a, w, hw, 2);
    c->launches++;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

// plain Ewald: S(m) and dS(m) = sum_j q_j (2 pi i m.w_j) e^{i ph_j} per k-vector
__global__ void ewald_dsfac_kernel(const double *__restrict__ x, const double *__restrict__ w, int nel, int n,
                                   double q0, double q1, const double *__restrict__ kvec, double *__restrict__ kS4) {
    __shared__ double red[32];
    const double mx = kvec[4 * blockIdx.x], my = kvec[4 * blockIdx.x + 1], mz = kvec[4 * blockIdx.x + 2];
    double sr = 0.0, si = 0.0, dr = 0.0, di = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double q = j < nel ? q0 : q1;
        const double ph = 2.0 * kPi * (mx * x[j] + my * x[(size_t)n + j] + mz * x[2 * (size_t)n + j]);
        const double mw = 2.0 * kPi * (mx * w[j] + my * w[(size_t)n + j] + mz * w[2 * (size_t)n + j]);
        double s, c;
        sincos(ph, &s, &c);
        sr += q * c;
        si += q * s;
        dr -= q * mw * s;
        di += q * mw * c;
    }
    sr = block_sum(sr, red);
    si = block_sum(si, red);
    dr = block_sum(dr, red);
    di = block_sum(di, red);
    if (threadIdx.x == 0) {
        kS4[4 * blockIdx.x] = sr;
        kS4[4 * blockIdx.x + 1] = si;
        kS4[4 * blockIdx.x + 2] = dr;
        kS4[4 * blockIdx.x + 3] = di;
    }
}

// (H w)_i = -(2 eps/V) q_i sum_m theta m [Im(conj(dS) e^{i ph_i}) + 2 pi (m.w_i) Re(conj(S) e^{i ph_i})]
__global__ void ewald_hvp_kernel(const double *__restrict__ x, const double *__restrict__ w, int nel, int n,
                                 double q0, double q1, const double *__restrict__ kvec,
                                 const double *__restrict__ kS4, int nk, double coef, double *__restrict__ hw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double q = i < nel ? q0 : q1;
    const double xi = x[i], yi = x[(size_t)n + i], zi = x[2 * (size_t)n + i];
    const double wx = w[i], wy = w[(size_t)n + i], wz = w[2 * (size_t)n + i];
    double h0 = 0.0, h1 = 0.0, h2 = 0.0;
    for (int k = 0; k < nk; ++k) {
        const double mx = kvec[4 * k], my = kvec[4 * k + 1], mz = kvec[4 * k + 2], th = kvec[4 * k + 3];
        double s, c;
        sincos(2.0 * kPi * (mx * xi + my * yi + mz * zi), &s, &c);
        const double mw = 2.0 * kPi * (mx * wx + my * wy + mz * wz);
        const double im_d = kS4[4 * k + 2] * s - kS4[4 * k + 3] * c;
        const double re_s = kS4[4 * k] * c + kS4[4 * k + 1] * s;
        const double t = th * (im_d + mw * re_s);
        h0 += t * mx;
        h1 += t * my;
        h2 += t * mz;
    }
    hw[i] += coef * q * h0;
    hw[(size_t)n + i] += coef * q * h1;
    hw[2 * (size_t)n + i] += coef * q * h2;
}

int launch_ewald_hvp(tcp_ctx *c, const double *w, double *hw) {
    if (c->nk == 0) return TCP_OK;
    if (!c->kS4 && cudaMalloc(&c->kS4, sizeof(double) * 4 * (size_t)c->nk) != cudaSuccess)
        return set_error(TCP_ERR_NOMEM, "Ewald Hessian buffer allocation failed");
    const double q0 = c->p.charge_scale * c->p.q[0], q1 = c->p.charge_scale * c->p.q[1];
    ewald_dsfac_kernel<<<c->nk, 256, 0, c->stream>>>(c->x, w, c->nel, c->n, q0, q1, c->kvec, c->kS4);
    ewald_hvp_kernel<<<(c->n + 127) / 128, 128, 0, c->stream>>>(c->x, w, c->nel, c->n, q0, q1, c->kvec, c->kS4,
                                                                c->nk, -2.0 * kEps / c->V, hw);
    c->launches += 2;
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

}  // namespace tcp

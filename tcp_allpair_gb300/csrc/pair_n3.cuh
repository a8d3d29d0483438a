// pair_n3.cuh -- the Newton-3 item schedule shared by the compensated-FP32
// (pair_n3.cu) and the FP64 (pair_n3_f64.cu) real-space kernels.
//
// Particles are split per species into i-tiles of TILE particles and
// j-subtiles of kN3Sub (tiles never straddle the e/i boundary).  An item is
// (i-tile I, j-subtile S) with S at or after I's first subtile; items are
// enumerated row by row, system by system for a batch.
#pragma once

#include "pair_math.cuh"
#include "tcp_internal.h"

namespace tcp {

constexpr int kN3Warps = 8;
constexpr int kN3Threads = 32 * kN3Warps;
constexpr int kN3Sub = 128;                // j-subtile
constexpr int kN3Stages = 3;

// Tile geometry of one system (a replica of a batch, or the only system).
struct N3Geom {
    int off;              // first particle in the global arrays
    int nel, n;           // electrons, particles
    int nIe, nI;          // i-tiles, electron tiles first
    int nSe, nS;          // j-subtiles, electron subtiles first
    long long item0;      // first item of this system in the global item list
};

struct N3Rep {
    N3Geom g;
    PairConsts c;
};

struct N3Args {
    const int4 *xq;                // fixed-point positions (FP32C kernels)
    const double4_32a *xd;         // FP64 positions
    const longlong4_32a *xl;       // 64-bit fixed-point positions (FP64 kernel)
    long long total;      // items (all systems)
    long long nstatic;    // FP64: items [0, nstatic) split statically (0: all from the counter)
    int ntot;             // stride of facc
    double *facc;         // [3][ntot], zeroed before the launch
    double *upart;        // [gridDim.x] (single system)
    unsigned *status;
    unsigned *counter;    // chunk counter (FP32C) / item counter (FP64), zeroed before the launch
    const long long *chunks;   // FP32C: chunk c holds items [chunks[c], chunks[c+1])
    unsigned nchunks;
    N3Geom g;             // single system
    PairConsts c;
    const N3Rep *reps;    // batch: one entry per replica
    int nrep;
    double *ur_rep;       // batch: Ur per replica (zeroed before the launch)
    int inject_skip;      // test hook: CTA 0 never issues the copy of its first item (its bounded wait runs out)
    unsigned long long *rdf;   // RDF variants: [3][kNbin] pair counts, +2 per unique pair (force.f90:99-103)
    const RdfEdges *rdf_edges; // exact bin edges (RDF variants)
};

template <int TILE>
__device__ __forceinline__ void n3_itile(const N3Geom &a, int I, int &start, int &end, int &sp, int &first) {
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

__device__ __forceinline__ void n3_sub(const N3Geom &a, int S, int &start, int &cnt, int &sp) {
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

// local item index of one system -> (row I, subtile S), in closed form.
// Electron row k (k < nIe) holds nS - k SPT items and starts at item
// k nS - SPT k (k - 1) / 2; ion row nIe + k holds n0 - k SPT items
// (n0 = nS - nSe) and starts at E + k n0 - SPT k (k - 1) / 2, E the items of
// the electron rows.  k comes from the root of that quadratic in FP32 and is
// corrected by exact integer comparisons.  An item at or past the end gives
// S = nS.
template <int TILE>
__device__ __forceinline__ void n3_decode(const N3Geom &a, long long it, int &I, int &S) {
    constexpr int SPT = TILE / kN3Sub;
    const long long E = (long long)a.nIe * a.nS - (long long)SPT * a.nIe * (a.nIe - 1) / 2;
    const bool ion = it >= E;
    const long long x = ion ? it - E : it;
    const int n0 = ion ? a.nS - a.nSe : a.nS;
    const int rows = ion ? a.nI - a.nIe : a.nIe;
    auto start = [&](int k) { return (long long)k * n0 - (long long)SPT * k * (k - 1) / 2; };
    const float b = (float)n0 + 0.5f * (float)SPT;
    int k = (int)((b - sqrtf(fmaxf(b * b - 2.0f * (float)SPT * (float)x, 0.0f))) / (float)SPT);
    k = max(0, min(k, rows - 1));
    while (k > 0 && start(k) > x) --k;
    while (k + 1 < rows && start(k + 1) <= x) ++k;
    if (rows <= 0 || x - start(k) >= (long long)(n0 - k * SPT)) {   // past the end
        I = a.nI;
        S = a.nS;
        return;
    }
    I = (ion ? a.nIe : 0) + k;
    S = (ion ? a.nSe : 0) + k * SPT + (int)(x - start(k));
}

// global item -> replica (0 for a single system), row and subtile
template <int TILE, bool BATCH>
__device__ __forceinline__ void n3_locate(const N3Args &a, long long it, int &rep, int &I, int &S) {
    rep = 0;
    if (BATCH) {
        int lo = 0, hi = a.nrep - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.reps[mid].g.item0 <= it) lo = mid; else hi = mid - 1;
        }
        rep = lo;
        n3_decode<TILE>(a.reps[rep].g, it - a.reps[rep].g.item0, I, S);
    } else {
        n3_decode<TILE>(a.g, it, I, S);
    }
}

template <bool BATCH>
__device__ __forceinline__ const N3Geom &n3_geom(const N3Args &a, int rep) {
    return BATCH ? a.reps[rep].g : a.g;
}

template <bool BATCH>
__device__ __forceinline__ const PairConsts &n3_consts(const N3Args &a, int rep) {
    return BATCH ? a.reps[rep].c : a.c;
}

// Tile geometry of a system of nel + nion particles for i-tiles of `tile`.
N3Geom n3_geometry(int off, int nel, int nion, int tile, long long item0, long long *items);

// Chunk boundaries of guided self-scheduling over `total` items for up to
// `ctas` CTAs: chunk sizes ceil(rest / (2 ctas)), at least one item, so the
// first chunks are long runs of one row and the last ones single items.
void n3_chunk_table(long long total, int ctas, std::vector<long long> &starts);

}  // namespace tcp

// tcp_internal.h -- device data layout, context and kernel interfaces of
// libtcpgpu.so (not part of the public ABI; see include/tcp_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "tcp_gpu.h"

namespace tcp {

constexpr double kEps = 14.399644154020082;     // data.f90:21
constexpr double kPi = 3.1415926535897931;       // data.f90:23
constexpr double kSqrtPi = 1.7724538509055159;   // data.f90:24
constexpr int kNdist = 500;                      // data.f90:16
constexpr int kNbin = kNdist + 1;
constexpr int kMaxOrder = 8;

// status word bits written by kernels (ctx->d_status)
constexpr unsigned kStatusTmaTimeout = 1u;

// ---------------------------------------------------------------------------
// Exact RDF bins of the FP32C kernels.  Bin k of pair type t (ee, ei, ii)
// holds the pairs with k dx_t <= r < (k+1) dx_t inside rc (force.f90:99-103).
// The kernels bin from their FP32 r and send the pairs whose r/dx_t lies
// within kRdfEdge of an integer, or whose r^2 lies within kRdfEdge of rc^2
// (relative), to an exact test.  In a cubic box r^2 in units of u^2
// (u = L/2^32) is an integer, the sum of the squared fixed-point
// separations, and is compared with e[t][k] = ceil((k dx_t/u)^2) and
// rc2 = ceil(rc^2/u^2).  Other boxes square the separations in FP64 (the
// scaling by L/2^32 is exact) against d[t][k] = (k dx_t)^2 and rc2d.
constexpr float kRdfEdge = 1.0f / 4096.0f;   // 8x the FP32 error of r/dx at r/dx = 500
struct RdfEdges {
    unsigned long long e[3][kNbin + 1];
    unsigned long long rc2;
    double d[3][kNbin + 1];
    double rc2d;
};

// ---------------------------------------------------------------------------
// Pair-kernel constants (host-computed once per parameter change).
struct PairConsts {
    // FP32 path: fixed-point positions are 2^32 units per box length
    float sx, sy, sz;          // box / 2^32
    float rc2f;                // cut-off^2
    float c_exp;               // -alpha^2 log2(e): exp(-a^2 r^2) = ex2(c_exp r^2)
    float p_alpha;             // P alpha: t = 1/(1 + P alpha r), P = kErfcP (pair_math.cuh)
    float c_gauss;             // 2 alpha / sqrt(pi)
    float c_rs;                // Deutsch: -log2(e)/rs
    float inv_rs;              // 1/rs
    float c_lam;               // Kelbg: -log2(e)/lambda^2
    float p_lam;               // P/lambda
    float sqrtpi_lam;          // sqrt(pi)/lambda
    float rshort2;             // (6 lambda)^2: Kelbg Gaussian terms below FP64 resolution beyond
    float close2;              // Kelbg close pairs (series form, kelbg_close): min(lambda^2/4, 1/(4 alpha^2))
    float inv_lam2f, alphaf;   // 1/lambda^2, alpha
    float inv_dx[3];           // RDF 1/dx per pair type ee|ei|ii
    float qqf[3];              // q_i q_j s^2 per pair type (energy/force sign and scale)
    // the same constants for cubic boxes in units of u = L/2^32 (the fixed-point
    // difference used unscaled): lengths / u, and the per-tile factors q_i q_j / u^2
    // (force) and q_i q_j / u (energy)
    int cubic;
    float u_rc2, u_p_alpha, u_c_exp, u_c_gauss, u_c_rs, u_inv_rs, u_c_lam, u_p_lam, u_sqrtpi_lam, u_rshort2;
    float u_close2, u_inv_lam2, u_alpha;
    float u_p_alpha5;          // kErfc5P alpha u: the degree-5 erfc of the Newton-3 kernels
    int erfc5_ok;              // alpha rc <= kErfc5Xmax: the degree-5 fit covers the Ewald term
    float u_inv_dx[3], u_qq_force[3], u_qq_energy[3];
    // FP64 path
    double box[3];
    double rc2, alpha, rs, lambda;
    double inv_box[3];         // 1/box (minimum image by multiplication)
    double sl[3];              // box / 2^64: the 64-bit fixed-point difference in A
    double sl2;                // sl[0]^2 (cubic boxes: r^2 from the unscaled differences)
    double alpha2;             // alpha^2
    double c_gauss_d;          // 2 alpha / sqrt(pi)
    double inv_rs_d;           // 1/rs
    double inv_lam2;           // 1/lambda^2
    double inv_lam;            // 1/lambda
    double sqrtpi_lam_d;       // sqrt(pi)/lambda
    double kelbg_far2;         // (8.5 lambda)^2: beyond, the Kelbg Gaussian terms are below 1e-31
    double inv_dxd[3];
    double qq[3];
    int ei_model;
};

// EWALD_SELF's constant energy, without eps: the self term
// -alpha/sqrt(pi) sum q_i^2 (force.f90:44-45) plus, for a system with net
// charge Q = sum q_i, the energy of the uniform neutralising background that
// the Ewald sum implies, -pi Q^2 / (2 V alpha^2).  The reference has no
// background term; its systems are neutral, where the term is zero.  Both
// terms are in FP64 and scale with the charge scale s squared.
inline double ewald_constant_energy(const tcp_params &p, int nel, int nion, double alpha) {
    const double s = p.charge_scale;
    const double q0 = s * p.q[0], q1 = s * p.q[1];
    const double self = (-(double)nel * q0 * q0 - (double)nion * q1 * q1) * alpha / kSqrtPi;
    const double Q = (double)nel * q0 + (double)nion * q1;
    const double V = p.box[0] * p.box[1] * p.box[2];
    return self - kPi * Q * Q / (2.0 * V * alpha * alpha);
}

// ---------------------------------------------------------------------------
struct Ctx;
struct N3Args;

// The CTAs a persistent Newton-3 launch left to the reciprocal chain, launched
// again with the same arguments on the chain's stream after it (pair_n3.cu)
struct N3Rejoin {
    N3Args *args = nullptr;
    bool pending = false;
    int grid = 0, threads = 0;
    const void *fn = nullptr;
};

}  // namespace tcp

struct tcp_ctx {
    tcp_params p;
    int nel = 0, nion = 0, n = 0;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // the reciprocal chain's stream: `stream`, or `stream2` while a step runs the
    // reciprocal sum concurrently with the real-space kernel (fork/join events)
    cudaStream_t rstream = nullptr, stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_pair_ready = nullptr;   // the Newton-3 launch's counter and accumulators are cleared
    unsigned flags = TCP_FLAG_ENERGY;
    bool ewald_ready = false;
    double alpha = 0, rc2 = 0, Uo = 0, V = 0;
    tcp::PairConsts pc{};

    // particle state, SoA [3][n]
    double *x = nullptr, *v = nullptr, *f = nullptr, *frec = nullptr;
    int4 *xq = nullptr;        // fixed-point positions for the FP32 pair kernel
    double4_32a *xd = nullptr;     // FP64 positions for the FP64 pair kernel
    longlong4_32a *xl = nullptr;   // 64-bit fixed-point positions (2^64 per box length) for the FP64 Newton-3 kernel
    // pair-kernel partials
    int jsplit = 1;
    int fpart_splits = 1;      // splits written by the last pair launch
    int pair_variant = 1;      // FP32C real-space kernel: 0 ordered pairs, >= 1 Newton-3 variant
    bool tuned = false;        // autotuner ran for the current parameters
    double pair_variant_ms[32] = {};   // autotuner timings per variant
    // CTAs of the persistent Newton-3 grid left free so that the reciprocal
    // chain, which runs beside the pair kernel in a step, finds room on the
    // SMs (chosen by the autotuner from kReserveCandidates)
    int pair_reserve = 0;
    double pair_reserve_ms[8] = {};
    bool recip_beside = false;          // the reciprocal chain is running on stream2
    // The reserved CTAs rejoin the Newton-3 launch once the chain is done: a second
    // launch of the same kernel on stream2 after the chain, claiming the remaining
    // chunks from the same counter (pair_n3.cu launch_pair_n3_rejoin)
    tcp::N3Rejoin rejoin;
    double *fpart = nullptr;   // [jsplit][3][n]
    double *upart = nullptr;   // energy partial per pair block
    int n_upart = 0;
    // reductions
    double *red = nullptr;     // block partials (size red_cap)
    int red_cap = 0;
    double *scal = nullptr;    // device scalars, see kScal* below
    double *h_scal = nullptr;  // pinned host copy
    unsigned *status = nullptr;
    unsigned *counter = nullptr;        // dynamic work counter of the Newton-3 kernel
    unsigned long long *rdf = nullptr;  // [3][kNbin]
    unsigned long long *vdf = nullptr;  // [2][kNbin]
    tcp::RdfEdges *rdf_edges = nullptr; // exact bin edges of the FP32C RDF
    long long *n3_chunks = nullptr;     // chunk tables of the FP32C Newton-3 schedule
    std::vector<long long> n3_chunk_meta;   // per table: i-tile, items, offset, chunks
    // staging for host transfers
    unsigned char *d_stage = nullptr;
    size_t d_stage_bytes = 0;
    double *h_stage = nullptr;          // pinned
    size_t h_stage_bytes = 0;
    // the device reads and writes the caller's (pageable) host arrays directly:
    // cudaDevAttrPageableMemoryAccess (coherent NVLink-C2C on Grace hosts)
    bool host_direct = false;
    // SPME
    int K1 = 0, K2 = 0, K3 = 0, Kh = 0; // Kh = K1/2+1
    // cell-sorted spreading: counting sort by the (y, z) mesh column of the spline base
    int *bin_count = nullptr, *bin_start = nullptr, *bin_bsum = nullptr;   // [K2 K3 (+1)], block sums
    int *bin_rank = nullptr, *bin_list = nullptr, *bin_ebx = nullptr, *bin_eby = nullptr;   // [n]
    void *bin_ew = nullptr, *bin_eq = nullptr;                               // weights [n][3][P], charges [n]
    double *Q = nullptr;                // real mesh [K3][K2][K1]
    cufftDoubleComplex *Qk = nullptr;   // [K3][K2][Kh]
    double *infl = nullptr;             // theta * |b|^-2 on the half mesh
    bool spme_fp32 = false;             // FP32C mode: FP32 transforms, influence and gather
    bool recip_fp64 = false;            // TCP_PREC_FP32C_R64: p.precision is FP32C, the reciprocal chain FP64
    float *Qf = nullptr;                // FP32 real mesh [K3][K2][K1]
    cufftComplex *Qkf = nullptr;        // FP32 half spectrum
    float *infl_f = nullptr;
    cufftHandle plan_f = 0, plan_b = 0;
    bool plans = false;
    // plain Ewald
    int nk = 0;
    double *kvec = nullptr;             // [nk][4]: m_x, m_y, m_z, theta
    double *ksum = nullptr;             // [nk][2]: S re, im
    // graph of one md step
    cudaGraphExec_t graph = nullptr;
    double graph_dt = 0.0;
    unsigned graph_flags = 0;
    int graph_kernels = 0;
    long long launches = 0;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // step phase marks
    void *l2_flush = nullptr;
    size_t l2_flush_bytes = 0;
    long long step_index = 0;
    tcp_energies last{};
    // derivatives (allocated on first use): vectors SoA [3][n]
    double *adj_w = nullptr, *adj_hw = nullptr;       // Hessian-vector product input / output
    double *adj_xb = nullptr, *adj_vb = nullptr, *adj_fb = nullptr;   // reverse-mode adjoints
    double *adj_save = nullptr;        // [3][3][n] x, v, f after the forward pass
    double *adj_io = nullptr;          // [3][n] host-layout staging
    double *adj_scal = nullptr;        // kAdj* scalars
    double *adj_part = nullptr;        // per-block partial sums
    double *adj_ck = nullptr;          // checkpoints [nck][2][3][n]
    int adj_ck_cap = 0;
    double *adj_seg = nullptr;         // recomputed segment [M+1][2][3][n]
    int adj_seg_cap = 0;
    double *hQ = nullptr, *hdQ = nullptr;   // FP64 meshes phi and dphi of the reciprocal HVP
    cufftDoubleComplex *hQk = nullptr;
    cufftHandle hplan_f = 0, hplan_b = 0;
    bool hplans = false;
    double *kS4 = nullptr;             // plain Ewald HVP: [nk][4] S re, S im, dS re, dS im
};

namespace tcp {

// indices into ctx->scal
enum {
    kScalUr = 0, kScalUm = 1, kScalMv2e = 2, kScalMv2i = 3,
    kScalFx = 4, kScalFy = 5, kScalFz = 6, kScalLamE = 7, kScalLamI = 8, kScalStep = 9,
    kScalCount = 16
};

int set_error(int code, const std::string &msg);

// Tracing: an NVTX range per C-ABI call (visible in nsys / ncu timelines;
// a no-op when no tool is attached).
struct TraceRange {
    explicit TraceRange(const char *name);
    ~TraceRange();
};
#define TCP_TRACE(name) tcp::TraceRange tcp_trace_range_(name)

// Fault injection for tests: TCP_INJECT_FAULT=<site>.  Host sites make the
// named call report failure ("alloc" in tcp_create, "cufft_plan" in the SPME
// setup); "tile_wait" makes CTA 0 of the Newton-3 kernel skip its first
// subtile copy, so its bounded mbarrier wait runs out (about 2 s), the kernel
// sets the timeout status and returns, and the call reports TCP_ERR_TIMEOUT.
bool inject_fault(const char *site);
int cuda_check(cudaError_t e, const char *what);
#define TCP_CUDA(call)                                        \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return tcp::cuda_check(_e, #call); \
    } while (0)

// pair.cu
void make_pair_consts(tcp_ctx *c);                 // c->pc from c->p, c->alpha, c->rc2
int pair_setup(tcp_ctx *c);                        // constants, jsplit, partial buffers
int launch_pair(tcp_ctx *c, bool energy, bool rdf);
int launch_force_finalize(tcp_ctx *c, bool add_rec);
// pair_n3.cu
bool n3_applicable(const tcp_ctx *c);
bool n3_f64_applicable(const tcp_ctx *c);
int n3_f64_grid(const tcp_ctx *c);
int launch_pair_n3_f64(tcp_ctx *c, bool energy, bool rdf);
int n3_grid(const tcp_ctx *c);
int n3_variant_count();
const char *n3_variant_name(int v);
bool n3_variant_usable(const tcp_ctx *c, int v);
int autotune_pair(tcp_ctx *c);
int time_pair_with_recip(tcp_ctx *c, int reps, double *ms);   // ctx.cu
int launch_pair_n3(tcp_ctx *c, bool energy, bool rdf);
int launch_pair_n3_rejoin(tcp_ctx *c, cudaStream_t st);   // on stream2, after the reciprocal chain
void n3_free(tcp_ctx *c);
int n3_rejoin_launch(N3Rejoin &r, cudaStream_t st, cudaEvent_t ready, long long *launches);
void n3_rejoin_free(N3Rejoin &r);
int n3_batch_variant_count();
bool n3_batch_variant_erfc5(int v);   // the variant needs every replica's PairConsts::erfc5_ok
const char *n3_batch_variant_name(int v);
int n3_batch_tile(int variant);
size_t n3_rep_bytes();
long long n3_batch_fill(void *reps_host, int nrep, const int *off, const int *nel, const int *nion,
                        const PairConsts *pc, int tile);
// reserve > 0 with a rejoin: that many CTAs are left out of the persistent
// grid for the reciprocal chain and set up in *rejoin (ready is recorded on st
// once the launch's counter and accumulators are cleared)
int launch_pair_n3_batch(cudaStream_t st, const int4 *xq, int ntot, double *facc, const void *reps_dev, int nrep,
                         long long total, const long long *chunks, unsigned nchunks, double *ur_rep, unsigned *status,
                         unsigned *counter, int num_sms, bool energy, int variant, int reserve = 0,
                         N3Rejoin *rejoin = nullptr, cudaEvent_t ready = nullptr);
int n3_batch_ctas(int num_sms, int v);
void n3_chunk_table(long long total, int ctas, std::vector<long long> &starts);
int n3_prepare_chunks(tcp_ctx *c);
// spme.cu
int spme_setup(tcp_ctx *c);                        // meshes, plans, influence function
std::vector<double> bspline_moduli(int order, int K);
int spme_free(tcp_ctx *c);
int launch_spme(tcp_ctx *c, bool energy);
int ewald_setup(tcp_ctx *c);
int launch_ewald(tcp_ctx *c, bool energy);
// integrate.cu
double *fsum_part(tcp_ctx *c);
double *mv_part(tcp_ctx *c, int pass);
double *recip_epart(tcp_ctx *c);
int red_capacity(int n, int extra);
int kick_blocks(int n);
int launch_refresh_positions(tcp_ctx *c);
int launch_shift(tcp_ctx *c, double sdt);
int launch_vverlet1(tcp_ctx *c, double dt, double unused);
int launch_spme_sum(tcp_ctx *c);
int launch_fsum(tcp_ctx *c);
int launch_remove_rigid(tcp_ctx *c);
int launch_kick2(tcp_ctx *c, double dt, bool remove_net, bool apply_thermo, bool vdf, int *final_pass);
int launch_reduce(tcp_ctx *c, int mask, int pass);
int launch_extract(tcp_ctx *c, const unsigned char *src, int first, int count, long stride, long off_x, long off_v,
                   long off_f, cudaStream_t st = nullptr);   // st: c->stream when null
int launch_scatter(tcp_ctx *c, unsigned char *dst, int first, int count, long stride, long off_x, long off_v,
                   long off_f, const double *fsrc, cudaStream_t st = nullptr);
int launch_pack(tcp_ctx *c, int first, int count, bool x, bool v, bool f, bool frec, int *nf);
int launch_fp32_peak(int device, double *tffma);

// spme.cu: cell sort of the atomic-free spread (single system and batch)
struct SpreadBins {
    int *count, *start, *bsum, *rank, *list, *ebx, *eby;
    void *ew, *eq;                       // [n][3][P] weights, [n] charges (float or double)
};
// start = exclusive prefix of count (plus start[nbins] = n), list = particles
// by bin (ebx[m] holds the bin of particle m on entry), each bin index-ordered
int launch_bin_sort(cudaStream_t st, int n, int nbins, const SpreadBins &b);   // returns its kernel count
int bin_scan_block();

// ctx.cu: step and force composition for the derivative routines
int force_eval(tcp_ctx *c, bool remove_net);        // main.f90:100-141 on the stream
int md_advance(tcp_ctx *c, double dt, int nsteps);  // nsteps MD steps (graph), no host sync
int md_finish(tcp_ctx *c);                          // sync scalars, fill c->last
// spme.cu: reciprocal Hessian-vector products, hw += H_rec w (w, hw SoA [3][n])
int launch_spme_hvp(tcp_ctx *c, const double *w, double *hw);
int launch_ewald_hvp(tcp_ctx *c, const double *w, double *hw);
void spme_hvp_free(tcp_ctx *c);
// adjoint.cu
void adjoint_free(tcp_ctx *c);

// reduce targets for launch_reduce
enum { kRedUr = 1, kRedMv2 = 4 };

}  // namespace tcp

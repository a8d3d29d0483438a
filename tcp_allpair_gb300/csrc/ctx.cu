// ctx.cu -- the C ABI of libtcpgpu.so (include/tcp_gpu.h): context
// lifecycle, host transfers, the reference-named step routines and the CUDA
// graph of one MD step.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "tcp_internal.h"

namespace tcp {

static thread_local std::string g_err;

TraceRange::TraceRange(const char *name) { nvtxRangePushA(name); }
TraceRange::~TraceRange() { nvtxRangePop(); }

bool inject_fault(const char *site) {
    const char *e = getenv("TCP_INJECT_FAULT");
    return e && std::strcmp(e, site) == 0;
}

int set_error(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int cuda_check(cudaError_t e, const char *what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? TCP_ERR_NOMEM : TCP_ERR_CUDA;
}

static int validate(const tcp_params *p, int nel, int nion) {
    if (!p) return set_error(TCP_ERR_BAD_PARAM, "params is NULL");
    if (nel < 0 || nion < 0 || nel + nion < 2) return set_error(TCP_ERR_BAD_PARAM, "need nel, nion >= 0 and nel+nion >= 2");
    for (int d = 0; d < 3; ++d)
        if (!(p->box[d] > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "box lengths must be positive");
    if (!(p->rc > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "rc must be positive");
    if (!(p->xm[0] > 0.0) || !(p->xm[1] > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "masses must be positive");
    if (p->precision != TCP_PREC_FP64 && p->precision != TCP_PREC_FP32C && p->precision != TCP_PREC_FP32C_R64)
        return set_error(TCP_ERR_BAD_PARAM, "unknown precision");
    if (p->ei_model < TCP_EI_DEUTSCH || p->ei_model > TCP_EI_COULOMB) return set_error(TCP_ERR_BAD_PARAM, "unknown ei_model");
    if (p->ei_model == TCP_EI_DEUTSCH && !(p->rs > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "Deutsch model needs rs > 0");
    if (p->ei_model == TCP_EI_KELBG && !(p->lambda_ei > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "Kelbg model needs lambda_ei > 0");
    if (p->reciprocal < TCP_RECIP_NONE || p->reciprocal > TCP_RECIP_EWALD) return set_error(TCP_ERR_BAD_PARAM, "unknown reciprocal");
    if (p->reciprocal == TCP_RECIP_SPME) {
        if (p->order < 4 || p->order > kMaxOrder) return set_error(TCP_ERR_BAD_PARAM, "SPME order must be in 4..8");
        for (int d = 0; d < 3; ++d)
            if (p->K[d] < p->order || p->K[d] > 1024)
                return set_error(TCP_ERR_BAD_PARAM, "SPME mesh must be in [order, 1024] in every dimension");
    }
    if (p->reciprocal == TCP_RECIP_EWALD && p->ewald_nmax2 < 0) return set_error(TCP_ERR_BAD_PARAM, "ewald_nmax2 < 0");
    if (p->thermo < TCP_THERMO_NOTEMP || p->thermo > TCP_THERMO_STOCH) return set_error(TCP_ERR_BAD_PARAM, "unknown thermo");
    if (p->thermo == TCP_THERMO_BEREND && !(p->tau > 0.0)) return set_error(TCP_ERR_BAD_PARAM, "Berendsen needs tau > 0");
    return TCP_OK;
}

static void normalise(tcp_params *p) {
    if (p->charge_scale == 0.0) p->charge_scale = 1.0;
    if (p->thermo_period <= 0) p->thermo_period = 1;
}

static int sync_scalars(tcp_ctx *c) {
    TCP_CUDA(cudaMemcpyAsync(c->h_scal, c->scal, sizeof(double) * kScalCount, cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaMemcpyAsync(c->h_scal + kScalCount, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    const unsigned st = *reinterpret_cast<unsigned *>(c->h_scal + kScalCount);
    if (st & kStatusTmaTimeout) {
        cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream);
        return set_error(TCP_ERR_TIMEOUT, "a pair-kernel tile wait exceeded its bound");
    }
    return TCP_OK;
}

static void invalidate_graph(tcp_ctx *c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
}

static int ensure_stage(tcp_ctx *c, size_t bytes) {
    if (c->d_stage_bytes < bytes) {
        cudaFree(c->d_stage);
        c->d_stage = nullptr;
        c->d_stage_bytes = 0;
        TCP_CUDA(cudaMalloc(&c->d_stage, bytes));
        c->d_stage_bytes = bytes;
    }
    if (c->h_stage_bytes < bytes) {
        cudaFreeHost(c->h_stage);
        c->h_stage = nullptr;
        c->h_stage_bytes = 0;
        TCP_CUDA(cudaMallocHost(&c->h_stage, bytes));
        c->h_stage_bytes = bytes;
    }
    return TCP_OK;
}

static bool energy_on(const tcp_ctx *c) { return (c->flags & TCP_FLAG_ENERGY) != 0; }

static int recip_launch(tcp_ctx *c) {
    if (c->p.reciprocal == TCP_RECIP_SPME) return launch_spme(c, energy_on(c));
    if (c->p.reciprocal == TCP_RECIP_EWALD) return launch_ewald(c, energy_on(c));
    return TCP_OK;
}

// The reciprocal chain forked onto stream2 (after the work queued so far on
// the main stream) so that it overlaps the real-space kernel; recip_join makes
// the main stream wait for it.  Inside a stream capture the two events become
// graph edges.
static int recip_fork(tcp_ctx *c) {
    if (c->p.reciprocal == TCP_RECIP_NONE) return TCP_OK;
    TCP_CUDA(cudaEventRecord(c->ev_fork, c->stream));
    TCP_CUDA(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
    c->rstream = c->stream2;
    const int rc = recip_launch(c);
    c->rstream = c->stream;
    c->recip_beside = rc == TCP_OK;
    return rc;
}

static int recip_join(tcp_ctx *c) {
    c->recip_beside = false;
    if (c->p.reciprocal == TCP_RECIP_NONE) return TCP_OK;
    if (int rc = launch_pair_n3_rejoin(c, c->stream2)) return rc;
    TCP_CUDA(cudaEventRecord(c->ev_join, c->stream2));
    TCP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    return TCP_OK;
}

// Mean time of the real-space launch with the reciprocal chain beside it on
// stream2, as inside a step (the autotuner's measure for the grid reserve).
int time_pair_with_recip(tcp_ctx *c, int reps, double *ms) {
    // The fork, the pair launch and the join are captured as one graph and
    // replayed, as they run inside the step graph: both branches become ready
    // together.  Launched one by one, the chain's kernels would run ahead on
    // an idle GPU while the host is still issuing the rest.
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    TCP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = recip_fork(c);
    if (!rc) rc = launch_pair(c, energy_on(c), false);
    const int jrc = recip_join(c);
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (!rc) rc = jrc;
    if (!rc && ce != cudaSuccess) rc = cuda_check(ce, "cudaStreamEndCapture");
    if (!rc) {
        const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
        if (ie != cudaSuccess) rc = cuda_check(ie, "cudaGraphInstantiate");
    }
    if (g) cudaGraphDestroy(g);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    TCP_CUDA(cudaEventCreate(&e0));
    TCP_CUDA(cudaEventCreate(&e1));
    cudaError_t le = cudaGraphLaunch(ge, c->stream);   // warm-up
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && le == cudaSuccess; ++r) le = cudaGraphLaunch(ge, c->stream);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    if (le != cudaSuccess) return cuda_check(le, "cudaGraphLaunch");
    *ms = t / std::max(reps, 1);
    TCP_CUDA(cudaGetLastError());
    return TCP_OK;
}

// Force evaluation of main.f90:100-141 without host synchronisation.
static int force_chain(tcp_ctx *c, bool remove_net) {
    int rc;
    if ((rc = recip_fork(c))) return rc;
    rc = launch_pair(c, energy_on(c), (c->flags & TCP_FLAG_RDF) != 0);
    if (int jrc = recip_join(c)) return jrc;
    if (rc) return rc;
    if ((rc = launch_force_finalize(c, c->p.reciprocal != TCP_RECIP_NONE))) return rc;
    if (remove_net && (rc = launch_remove_rigid(c))) return rc;
    if (energy_on(c) && (rc = launch_reduce(c, kRedUr, 0))) return rc;
    return TCP_OK;
}

static void fill_energies(tcp_ctx *c, tcp_energies *e) {
    c->last.Ur = c->h_scal[kScalUr];
    c->last.Um = c->p.reciprocal == TCP_RECIP_NONE ? 0.0 : c->h_scal[kScalUm];
    c->last.Uo = c->Uo;
    c->last.Epot = (c->last.Ur + c->Uo) * kEps;      // main.f90:138
    if (e) *e = c->last;
}

static bool thermostat_due(const tcp_ctx *c) {
    return ((c->step_index + 1) % c->p.thermo_period) == 0;
}

// One MD step (main.f90:81-153) on the stream; *pass = kinetic partial set.
// Phase mark k: an event-record node when the stream is being captured, a
// plain record otherwise (the External flag is only valid during capture).
static int mark_on(tcp_ctx *c, int k, cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    TCP_CUDA(cudaStreamIsCapturing(s, &st));
    if (st == cudaStreamCaptureStatusActive)
        TCP_CUDA(cudaEventRecordWithFlags(c->ev[k], s, cudaEventRecordExternal));
    else
        TCP_CUDA(cudaEventRecord(c->ev[k], s));
    return TCP_OK;
}

static int mark(tcp_ctx *c, int k) { return mark_on(c, k, c->stream); }

// Phase marks ev[0..4] (event nodes in the graph): 0 step start, 1 after
// the first half kick, 2 end of the reciprocal chain (on stream2, concurrent
// with the pair kernel), 3 end of the pair launch on the main stream (the
// reserved CTAs that rejoin it after the chain drain the same chunk counter,
// so they end within a chunk of it), 4 step end.
static int step_chain(tcp_ctx *c, double dt, bool apply, int *pass) {
    int rc;
    if ((rc = mark(c, 0))) return rc;
    if ((rc = launch_vverlet1(c, dt, 0.0))) return rc;
    if ((rc = mark(c, 1))) return rc;
    if ((rc = recip_fork(c))) return rc;
    if (c->p.reciprocal != TCP_RECIP_NONE) {
        if ((rc = mark_on(c, 2, c->stream2))) return rc;
    } else if ((rc = mark(c, 2))) {
        return rc;
    }
    if ((rc = launch_pair(c, energy_on(c), (c->flags & TCP_FLAG_RDF) != 0))) return rc;
    if ((rc = mark(c, 3))) return rc;
    if ((rc = recip_join(c))) return rc;
    if ((rc = launch_force_finalize(c, c->p.reciprocal != TCP_RECIP_NONE))) return rc;
    if ((rc = launch_kick2(c, dt, true, apply, (c->flags & TCP_FLAG_VDF) != 0, pass))) return rc;
    if ((rc = launch_reduce(c, (energy_on(c) ? kRedUr : 0) | kRedMv2, *pass))) return rc;
    if ((rc = mark(c, 4))) return rc;
    return TCP_OK;
}

// ---- composition used by the derivative routines (adjoint.cu) ----------------
int force_eval(tcp_ctx *c, bool remove_net) { return force_chain(c, remove_net); }

int md_finish(tcp_ctx *c) {
    int rc;
    if ((rc = sync_scalars(c))) return rc;
    fill_energies(c, nullptr);
    c->last.mv2el = c->h_scal[kScalMv2e];
    c->last.mv2ion = c->h_scal[kScalMv2i];
    return TCP_OK;
}

}  // namespace tcp

using namespace tcp;

extern "C" {

const char *tcp_last_error(void) { return g_err.c_str(); }

const char *tcp_status_string(int code) {
    switch (code) {
        case TCP_OK: return "ok";
        case TCP_ERR_BAD_PARAM: return "bad parameter";
        case TCP_ERR_CUTOFF: return "cut-off radius larger than half the box";
        case TCP_ERR_CUDA: return "CUDA error";
        case TCP_ERR_CUFFT: return "cuFFT error";
        case TCP_ERR_TIMEOUT: return "device wait timed out";
        case TCP_ERR_NO_DEVICE: return "no usable sm_103 device";
        case TCP_ERR_STATE: return "call order";
        case TCP_ERR_NOMEM: return "device allocation failed";
        default: return "unknown status";
    }
}

int tcp_version(int *major, int *minor, int *arch) {
    if (major) *major = 0;
    if (minor) *minor = 1;
    if (arch) *arch = 103;
    return TCP_OK;
}

int tcp_create(const tcp_params *p_in, int nel, int nion, int device, tcp_ctx **out) {
    TCP_TRACE("tcp_create");
    if (!out) return set_error(TCP_ERR_BAD_PARAM, "out is NULL");
    *out = nullptr;
    int rc = validate(p_in, nel, nion);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(TCP_ERR_NO_DEVICE, "no CUDA device visible");
    }
    if (device < 0 || device >= ndev) return set_error(TCP_ERR_BAD_PARAM, "device index out of range");
    cudaDeviceProp prop;
    TCP_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return set_error(TCP_ERR_NO_DEVICE, "libtcpgpu is built for sm_103a (GB300); device is sm_" +
                                                std::to_string(prop.major) + std::to_string(prop.minor));
    TCP_CUDA(cudaSetDevice(device));
    if (inject_fault("alloc")) return set_error(TCP_ERR_NOMEM, "injected: device allocation failed");
    tcp_ctx *c = new tcp_ctx();
    c->p = *p_in;
    normalise(&c->p);
    // TCP_PREC_FP32C_R64 is the FP32C context with an FP64 reciprocal chain
    c->recip_fp64 = c->p.precision == TCP_PREC_FP32C_R64;
    if (c->recip_fp64) c->p.precision = TCP_PREC_FP32C;
    c->nel = nel;
    c->nion = nion;
    c->n = nel + nion;
    c->device = device;
    c->num_sms = prop.multiProcessorCount;
    {
        int pageable = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
        const char *env = getenv("TCP_HOST_DIRECT");
        c->host_direct = pageable == 1 && !(env && env[0] == '0');
    }
    const size_t n = c->n;
    auto fail = [&](int code) {
        tcp_destroy(c);
        return code;
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(cuda_check(cudaGetLastError(), "cudaStreamCreate"));
    if (cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_pair_ready, cudaEventDisableTiming) != cudaSuccess)
        return fail(cuda_check(cudaGetLastError(), "cudaStreamCreate (reciprocal stream)"));
    c->rstream = c->stream;
    for (auto &e : c->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(cuda_check(cudaGetLastError(), "cudaEventCreate"));
#define TCP_ALLOC(ptr, bytes)                                                            \
    do {                                                                                 \
        cudaError_t _e = cudaMalloc(&(ptr), (bytes));                                    \
        if (_e != cudaSuccess) return fail(cuda_check(_e, "cudaMalloc " #ptr));          \
    } while (0)
    TCP_ALLOC(c->x, sizeof(double) * 3 * n);
    TCP_ALLOC(c->v, sizeof(double) * 3 * n);
    TCP_ALLOC(c->f, sizeof(double) * 3 * n);
    TCP_ALLOC(c->frec, sizeof(double) * 3 * n);
    TCP_ALLOC(c->xq, sizeof(int4) * n);
    TCP_ALLOC(c->xd, sizeof(double4_32a) * n);
    TCP_ALLOC(c->xl, sizeof(longlong4_32a) * n);
    c->red_cap = red_capacity(c->n, 8192 + 65536);
    TCP_ALLOC(c->red, sizeof(double) * (size_t)c->red_cap);
    TCP_ALLOC(c->scal, sizeof(double) * kScalCount);
    TCP_ALLOC(c->status, sizeof(unsigned));
    TCP_ALLOC(c->counter, sizeof(unsigned));
    TCP_ALLOC(c->rdf, sizeof(unsigned long long) * 3 * kNbin);
    TCP_ALLOC(c->vdf, sizeof(unsigned long long) * 2 * kNbin);
    TCP_ALLOC(c->rdf_edges, sizeof(RdfEdges));
#undef TCP_ALLOC
    if (cudaMallocHost(&c->h_scal, sizeof(double) * (kScalCount + 1)) != cudaSuccess)
        return fail(cuda_check(cudaGetLastError(), "cudaMallocHost"));
    cudaMemsetAsync(c->x, 0, sizeof(double) * 3 * n, c->stream);
    cudaMemsetAsync(c->v, 0, sizeof(double) * 3 * n, c->stream);
    cudaMemsetAsync(c->f, 0, sizeof(double) * 3 * n, c->stream);
    cudaMemsetAsync(c->frec, 0, sizeof(double) * 3 * n, c->stream);
    cudaMemsetAsync(c->scal, 0, sizeof(double) * kScalCount, c->stream);
    cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream);
    cudaMemsetAsync(c->rdf, 0, sizeof(unsigned long long) * 3 * kNbin, c->stream);
    cudaMemsetAsync(c->vdf, 0, sizeof(unsigned long long) * 2 * kNbin, c->stream);
    if ((rc = launch_refresh_positions(c))) return fail(rc);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(cuda_check(cudaGetLastError(), "create sync"));
    *out = c;
    return TCP_OK;
}

int tcp_destroy(tcp_ctx *c) {
    TCP_TRACE("tcp_destroy");
    if (!c) return TCP_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    invalidate_graph(c);
    adjoint_free(c);
    spme_hvp_free(c);
    spme_free(c);
    cudaFree(c->x);
    cudaFree(c->v);
    cudaFree(c->f);
    cudaFree(c->frec);
    cudaFree(c->xq);
    cudaFree(c->xd);
    cudaFree(c->xl);
    cudaFree(c->fpart);
    cudaFree(c->upart);
    cudaFree(c->red);
    cudaFree(c->scal);
    cudaFree(c->status);
    cudaFree(c->counter);
    cudaFree(c->rdf);
    cudaFree(c->vdf);
    cudaFree(c->rdf_edges);
    cudaFree(c->n3_chunks);
    cudaFree(c->d_stage);
    cudaFree(c->kvec);
    cudaFree(c->ksum);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->h_scal) cudaFreeHost(c->h_scal);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    cudaFree(c->l2_flush);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_pair_ready) cudaEventDestroy(c->ev_pair_ready);
    n3_free(c);
    if (c->stream2) {
        cudaStreamSynchronize(c->stream2);
        cudaStreamDestroy(c->stream2);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TCP_OK;
}

int tcp_ewald_self(tcp_ctx *c, double *alpha_out, double *Uo_out) {
    TCP_TRACE("tcp_ewald_self");
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    cudaSetDevice(c->device);
    const tcp_params &p = c->p;
    const double rc_cut = std::min(std::min(p.box[0], p.box[1]), p.box[2]) / 2.0;   // force.f90:18
    if (p.rc > rc_cut) return set_error(TCP_ERR_CUTOFF, " *** error at cut-off radius *** (rc > min(box)/2)");
    c->alpha = p.a > 0.0 ? p.a : 3.1 / p.rc;                                       // force.f90:23
    c->rc2 = p.rc * p.rc;                                                           // force.f90:24
    c->V = p.box[0] * p.box[1] * p.box[2];
    c->Uo = ewald_constant_energy(p, c->nel, c->nion, c->alpha);                   // force.f90:44-45 + background
    int rc;
    if ((rc = pair_setup(c))) return rc;
    if (p.reciprocal == TCP_RECIP_SPME && (rc = spme_setup(c))) return rc;
    if (p.reciprocal == TCP_RECIP_EWALD && (rc = ewald_setup(c))) return rc;
    invalidate_graph(c);
    c->tuned = false;
    c->ewald_ready = true;
    if (alpha_out) *alpha_out = c->alpha;
    if (Uo_out) *Uo_out = c->Uo;
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_set_params(tcp_ctx *c, const tcp_params *p) {
    TCP_TRACE("tcp_set_params");
    if (!c || !p) return set_error(TCP_ERR_BAD_PARAM, "NULL argument");
    int rc = validate(p, c->nel, c->nion);
    if (rc) return rc;
    tcp_params q = *p;
    normalise(&q);
    for (int d = 0; d < 3; ++d)
        if (q.box[d] != c->p.box[d] || q.K[d] != c->p.K[d])
            return set_error(TCP_ERR_BAD_PARAM, "box and mesh are fixed at tcp_create");
    const bool q_r64 = q.precision == TCP_PREC_FP32C_R64;
    if (q_r64) q.precision = TCP_PREC_FP32C;
    if (q.order != c->p.order || q.precision != c->p.precision || q_r64 != c->recip_fp64 ||
        q.reciprocal != c->p.reciprocal || q.ewald_nmax2 != c->p.ewald_nmax2)
        return set_error(TCP_ERR_BAD_PARAM, "order, precision and reciprocal method are fixed at tcp_create");
    const bool alpha_changed = q.a != c->p.a || q.rc != c->p.rc;
    c->p = q;
    invalidate_graph(c);
    if (c->ewald_ready && (alpha_changed || true)) return tcp_ewald_self(c, nullptr, nullptr);
    return TCP_OK;
}

int tcp_set_flags(tcp_ctx *c, unsigned flags) {
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    if (flags != c->flags) invalidate_graph(c);
    c->flags = flags;
    return TCP_OK;
}

// ---- transfers ---------------------------------------------------------------
// One species' fields in its records: the lowest field address, the byte
// offset of xx, xv, ff from it (-1: skipped) and the span of bytes touched.
struct RecSpan {
    const char *base = nullptr;
    long off[3] = {-1, -1, -1};
    size_t span = 0;
};

static int record_span(int count, const double *xx, const double *xv, const double *ff, long stride, RecSpan &rs) {
    rs = RecSpan();
    const double *ptrs[3] = {xx, xv, ff};
    const char *top = nullptr;
    for (const double *q : ptrs)
        if (q) {
            const char *b = reinterpret_cast<const char *>(q);
            if (!rs.base || b < rs.base) rs.base = b;
            if (!top || b > top) top = b;
        }
    if (!rs.base || count == 0) return TCP_OK;
    if (stride < 24 || stride % 8 || (top - rs.base) + 24 > (count > 1 ? stride : (top - rs.base) + 24))
        return set_error(TCP_ERR_BAD_PARAM, "stride must be a multiple of 8 and cover the three fields");
    for (int k = 0; k < 3; ++k) {
        rs.off[k] = ptrs[k] ? (long)(reinterpret_cast<const char *>(ptrs[k]) - rs.base) : -1;
        if (rs.off[k] >= 0 && rs.off[k] % 8) return set_error(TCP_ERR_BAD_PARAM, "fields must be 8-byte aligned");
    }
    rs.span = (size_t)(count - 1) * stride + (size_t)(top - rs.base) + 24;
    return TCP_OK;
}

static int species_range(const tcp_ctx *c, int species, int &first, int &count) {
    if (species != 0 && species != 1) return set_error(TCP_ERR_BAD_PARAM, "bad species");
    count = species == 0 ? c->nel : c->nion;
    first = species == 0 ? 0 : c->nel;
    return TCP_OK;
}

// records -> device arrays, queued on the stream (no wait)
static int enqueue_upload(tcp_ctx *c, int first, int count, const RecSpan &rs, long stride,
                          cudaStream_t st = nullptr) {
    if (count == 0 || !rs.base) return TCP_OK;
    const unsigned char *src = reinterpret_cast<const unsigned char *>(rs.base);
    int rc;
    if (!c->host_direct) {      // staged: one copy of the record span, then the same gather
        if ((rc = ensure_stage(c, rs.span))) return rc;
        TCP_CUDA(cudaMemcpyAsync(c->d_stage, rs.base, rs.span, cudaMemcpyHostToDevice, c->stream));
        src = c->d_stage;
        st = nullptr;
    }
    return launch_extract(c, src, first, count, stride, rs.off[0], rs.off[1], rs.off[2], st);   // refreshes xq, xd
}

// device arrays -> records the device writes in place (host_direct), queued
static int enqueue_download_direct(tcp_ctx *c, int first, int count, const RecSpan &rs, long stride,
                                   cudaStream_t st = nullptr) {
    if (count == 0 || !rs.base) return TCP_OK;
    return launch_scatter(c, reinterpret_cast<unsigned char *>(const_cast<char *>(rs.base)), first, count, stride,
                          rs.off[0], rs.off[1], rs.off[2], c->f, st);
}

// The two species' records read or written concurrently over the host link:
// the electrons' on the main stream, the ions' on stream2 between a fork and a
// join (one launch alone leaves most SMs waiting on the link)
static int records_both(tcp_ctx *c, const RecSpan *rs, long el_stride, long ion_stride, bool upload) {
    int rc;
    TCP_CUDA(cudaEventRecord(c->ev_fork, c->stream));
    TCP_CUDA(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
    if (upload) {
        if ((rc = enqueue_upload(c, 0, c->nel, rs[0], el_stride))) return rc;
        if ((rc = enqueue_upload(c, c->nel, c->nion, rs[1], ion_stride, c->stream2))) return rc;
    } else {
        if ((rc = enqueue_download_direct(c, 0, c->nel, rs[0], el_stride))) return rc;
        if ((rc = enqueue_download_direct(c, c->nel, c->nion, rs[1], ion_stride, c->stream2))) return rc;
    }
    TCP_CUDA(cudaEventRecord(c->ev_join, c->stream2));
    TCP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    return TCP_OK;
}

// device arrays -> records through the pinned stage; waits for the device
static int download_staged(tcp_ctx *c, int first, int count, double *xx, double *xv, double *ff, long stride) {
    if (count == 0 || (!xx && !xv && !ff)) return TCP_OK;
    int nf = 0, rc;
    if ((rc = ensure_stage(c, (size_t)count * 4 * 3 * sizeof(double)))) return rc;
    if ((rc = launch_pack(c, first, count, xx != nullptr, xv != nullptr, ff != nullptr, false, &nf))) return rc;
    TCP_CUDA(cudaMemcpyAsync(c->h_stage, c->d_stage, (size_t)count * nf * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    double *dst[3] = {xx, xv, ff};
    int slot = 0;
    for (int q = 0; q < 3; ++q) {
        if (!dst[q]) continue;
        char *b = reinterpret_cast<char *>(dst[q]);
        for (int r = 0; r < count; ++r)
            std::memcpy(b + (size_t)r * stride, c->h_stage + ((size_t)r * nf + slot) * 3, 3 * sizeof(double));
        ++slot;
    }
    return TCP_OK;
}

int tcp_upload(tcp_ctx *c, int species, const double *xx, const double *xv, const double *ff, long stride) {
    TCP_TRACE("tcp_upload");
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    cudaSetDevice(c->device);
    int first, count, rc;
    RecSpan rs;
    if ((rc = species_range(c, species, first, count))) return rc;
    if ((rc = record_span(count, xx, xv, ff, stride, rs))) return rc;
    if ((rc = enqueue_upload(c, first, count, rs, stride))) return rc;
    // the step graph reads the device arrays in place: new data needs no new graph
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_download(tcp_ctx *c, int species, double *xx, double *xv, double *ff, long stride) {
    TCP_TRACE("tcp_download");
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    cudaSetDevice(c->device);
    int first, count, rc;
    RecSpan rs;
    if ((rc = species_range(c, species, first, count))) return rc;
    if ((rc = record_span(count, xx, xv, ff, stride, rs))) return rc;
    if (!c->host_direct) return download_staged(c, first, count, xx, xv, ff, stride);
    if ((rc = enqueue_download_direct(c, first, count, rs, stride))) return rc;   // written in place
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_upload_soa(tcp_ctx *c, const double *x, const double *v, const double *f) {
    TCP_TRACE("tcp_upload_soa");
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    cudaSetDevice(c->device);
    int rc;
    if ((rc = ensure_stage(c, (size_t)c->n * 3 * sizeof(double)))) return rc;
    const double *src[3] = {x, v, f};
    for (int q = 0; q < 3; ++q) {
        if (!src[q]) continue;
        const unsigned char *from = reinterpret_cast<const unsigned char *>(src[q]);
        if (!c->host_direct) {
            // the stream is in order: the previous extract has read d_stage before this copy lands
            TCP_CUDA(cudaMemcpyAsync(c->d_stage, src[q], (size_t)c->n * 3 * sizeof(double), cudaMemcpyHostToDevice,
                                     c->stream));
            from = c->d_stage;
        }
        if ((rc = launch_extract(c, from, 0, c->n, 24, q == 0 ? 0 : -1, q == 1 ? 0 : -1, q == 2 ? 0 : -1))) return rc;
    }
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_download_soa(tcp_ctx *c, double *x, double *v, double *f, double *frec) {
    TCP_TRACE("tcp_download_soa");
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    cudaSetDevice(c->device);
    int nf = 0, rc;
    if (c->host_direct) {
        // (n, 3) row-major host arrays are records of stride 24 with one field
        if (x && (rc = launch_scatter(c, reinterpret_cast<unsigned char *>(x), 0, c->n, 24, 0, -1, -1, c->f))) return rc;
        if (v && (rc = launch_scatter(c, reinterpret_cast<unsigned char *>(v), 0, c->n, 24, -1, 0, -1, c->f))) return rc;
        if (f && (rc = launch_scatter(c, reinterpret_cast<unsigned char *>(f), 0, c->n, 24, -1, -1, 0, c->f))) return rc;
        if (frec && (rc = launch_scatter(c, reinterpret_cast<unsigned char *>(frec), 0, c->n, 24, -1, -1, 0, c->frec)))
            return rc;
        TCP_CUDA(cudaStreamSynchronize(c->stream));
        return TCP_OK;
    }
    if ((rc = ensure_stage(c, (size_t)c->n * 4 * 3 * sizeof(double)))) return rc;
    if ((rc = launch_pack(c, 0, c->n, x != nullptr, v != nullptr, f != nullptr, frec != nullptr, &nf))) return rc;
    if (nf == 0) return TCP_OK;
    TCP_CUDA(cudaMemcpyAsync(c->h_stage, c->d_stage, (size_t)c->n * nf * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    double *dst[4] = {x, v, f, frec};
    int slot = 0;
    for (int q = 0; q < 4; ++q) {
        if (!dst[q]) continue;
        for (int r = 0; r < c->n; ++r)
            for (int d = 0; d < 3; ++d) dst[q][3 * (size_t)r + d] = c->h_stage[((size_t)r * nf + slot) * 3 + d];
        ++slot;
    }
    return TCP_OK;
}

// ---- force routines ------------------------------------------------------------
#define TCP_REQUIRE_READY(c)                                                                     \
    do {                                                                                         \
        if (!(c)) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");                           \
        if (!(c)->ewald_ready) return set_error(TCP_ERR_STATE, "tcp_ewald_self must be called first"); \
        cudaSetDevice((c)->device);                                                              \
    } while (0)

int tcp_force_direct(tcp_ctx *c, double *Ur) {
    TCP_TRACE("tcp_force_direct");
    TCP_REQUIRE_READY(c);
    int rc;
    if ((rc = autotune_pair(c))) return rc;
    if ((rc = launch_pair(c, energy_on(c), (c->flags & TCP_FLAG_RDF) != 0))) return rc;
    if ((rc = launch_force_finalize(c, false))) return rc;
    if (energy_on(c) && (rc = launch_reduce(c, kRedUr, 0))) return rc;
    if ((rc = sync_scalars(c))) return rc;
    if (Ur) *Ur = energy_on(c) ? c->h_scal[kScalUr] : 0.0;
    return TCP_OK;
}

int tcp_force_spme(tcp_ctx *c, double *Um) {
    TCP_TRACE("tcp_force_spme");
    TCP_REQUIRE_READY(c);
    int rc;
    if (c->p.reciprocal == TCP_RECIP_NONE) {
        TCP_CUDA(cudaMemsetAsync(c->frec, 0, sizeof(double) * 3 * (size_t)c->n, c->stream));
        TCP_CUDA(cudaMemsetAsync(c->scal + kScalUm, 0, sizeof(double), c->stream));
    } else if ((rc = recip_launch(c))) {
        return rc;
    }
    if ((rc = sync_scalars(c))) return rc;
    if (Um) *Um = c->h_scal[kScalUm];
    return TCP_OK;
}

int tcp_spme_sum(tcp_ctx *c) {
    TCP_TRACE("tcp_spme_sum");
    TCP_REQUIRE_READY(c);
    int rc;
    if ((rc = launch_spme_sum(c))) return rc;
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_remove_rigidmtn(tcp_ctx *c) {
    TCP_TRACE("tcp_remove_rigidmtn");
    TCP_REQUIRE_READY(c);
    int rc;
    if ((rc = launch_fsum(c))) return rc;
    if ((rc = launch_remove_rigid(c))) return rc;
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_force(tcp_ctx *c, tcp_energies *e) {
    TCP_TRACE("tcp_force");
    TCP_REQUIRE_READY(c);
    int rc;
    if ((rc = autotune_pair(c))) return rc;
    if ((rc = force_chain(c, true))) return rc;
    if ((rc = sync_scalars(c))) return rc;
    fill_energies(c, e);
    return TCP_OK;
}

int tcp_vverlet1(tcp_ctx *c, double dt) {
    TCP_TRACE("tcp_vverlet1");
    TCP_REQUIRE_READY(c);
    int rc;
    if ((rc = launch_vverlet1(c, dt, 0.0))) return rc;
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    return TCP_OK;
}

int tcp_vverlet2(tcp_ctx *c, double dt, double *mv2el, double *mv2ion) {
    TCP_TRACE("tcp_vverlet2");
    TCP_REQUIRE_READY(c);
    int rc, pass = 0;
    if ((rc = launch_kick2(c, dt, false, thermostat_due(c), (c->flags & TCP_FLAG_VDF) != 0, &pass))) return rc;
    if ((rc = launch_reduce(c, kRedMv2, pass))) return rc;
    if ((rc = sync_scalars(c))) return rc;
    c->step_index++;
    c->last.mv2el = c->h_scal[kScalMv2e];
    c->last.mv2ion = c->h_scal[kScalMv2i];
    if (mv2el) *mv2el = c->last.mv2el;
    if (mv2ion) *mv2ion = c->last.mv2ion;
    return TCP_OK;
}

int tcp_finit(tcp_ctx *c, double dt, tcp_energies *e) {
    TCP_TRACE("tcp_finit");
    TCP_REQUIRE_READY(c);
    int rc;
    if ((rc = autotune_pair(c))) return rc;
    if ((rc = launch_shift(c, -dt))) return rc;                  // init.f90:171-185
    if ((rc = force_chain(c, true))) return rc;                  // init.f90:193-220
    if ((rc = launch_shift(c, dt))) return rc;                   // init.f90:223-237
    if ((rc = sync_scalars(c))) return rc;
    fill_energies(c, e);
    return TCP_OK;
}

static int build_graph(tcp_ctx *c, double dt, bool apply, cudaGraphExec_t *out, int *kernels) {
    cudaGraph_t g;
    const long long before = c->launches;
    TCP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int pass = 0;
    int rc = step_chain(c, dt, apply, &pass);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_check(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_check(ce, "cudaGraphInstantiate");
    *kernels = (int)(c->launches - before);
    c->launches = before;
    return TCP_OK;
}

static int ensure_graph(tcp_ctx *c, double dt) {
    int arc = autotune_pair(c);   // timing launches cannot run inside a capture
    if (arc) return arc;
    const bool has_thermo = c->p.thermo == TCP_THERMO_ISOKIN || c->p.thermo == TCP_THERMO_BEREND;
    // c->graph holds the step without the thermostat rescale; the rescale step
    // (ISOKIN/BEREND, every thermo_period-th step) is launched eagerly.
    if (!c->graph || c->graph_dt != dt || c->graph_flags != c->flags) {
        invalidate_graph(c);
        int rc = build_graph(c, dt, !has_thermo, &c->graph, &c->graph_kernels);
        if (rc) return rc;
        c->graph_dt = dt;
        c->graph_flags = c->flags;
    }
    return TCP_OK;
}

static int launch_step(tcp_ctx *c, double dt) {
    const bool has_thermo = c->p.thermo == TCP_THERMO_ISOKIN || c->p.thermo == TCP_THERMO_BEREND;
    int rc;
    if (has_thermo && thermostat_due(c)) {
        int pass = 0;
        if ((rc = step_chain(c, dt, true, &pass))) return rc;
    } else {
        TCP_CUDA(cudaGraphLaunch(c->graph, c->stream));
        c->launches += c->graph_kernels;
    }
    c->step_index++;
    return TCP_OK;
}

int tcp_md_steps(tcp_ctx *c, double dt, int nsteps, tcp_energies *e) {
    TCP_TRACE("tcp_md_steps");
    TCP_REQUIRE_READY(c);
    if (nsteps < 0) return set_error(TCP_ERR_BAD_PARAM, "nsteps < 0");
    int rc;
    if ((rc = ensure_graph(c, dt))) return rc;
    for (int s = 0; s < nsteps; ++s)
        if ((rc = launch_step(c, dt))) return rc;
    if ((rc = sync_scalars(c))) return rc;
    fill_energies(c, nullptr);
    c->last.mv2el = c->h_scal[kScalMv2e];
    c->last.mv2ion = c->h_scal[kScalMv2i];
    if (e) *e = c->last;
    return TCP_OK;
}

int tcp_md_steps_records(tcp_ctx *c, double dt, int nsteps, double *el_xx, double *el_xv, double *el_ff,
                         long el_stride, double *ion_xx, double *ion_xv, double *ion_ff, long ion_stride,
                         tcp_energies *e) {
    TCP_TRACE("tcp_md_steps_records");
    TCP_REQUIRE_READY(c);
    if (nsteps < 0) return set_error(TCP_ERR_BAD_PARAM, "nsteps < 0");
    RecSpan rs[2];
    int rc;
    // every argument is checked before anything is queued
    if ((rc = record_span(c->nel, el_xx, el_xv, el_ff, el_stride, rs[0]))) return rc;
    if ((rc = record_span(c->nion, ion_xx, ion_xv, ion_ff, ion_stride, rs[1]))) return rc;
    if (c->host_direct) {
        if ((rc = records_both(c, rs, el_stride, ion_stride, true))) return rc;
    } else {
        if ((rc = enqueue_upload(c, 0, c->nel, rs[0], el_stride))) return rc;
        if ((rc = enqueue_upload(c, c->nel, c->nion, rs[1], ion_stride))) return rc;
    }
    if ((rc = ensure_graph(c, dt))) return rc;
    for (int s = 0; s < nsteps; ++s)
        if ((rc = launch_step(c, dt))) return rc;
    if (c->host_direct && (rc = records_both(c, rs, el_stride, ion_stride, false))) return rc;   // before the one wait below
    if ((rc = sync_scalars(c))) return rc;
    if (!c->host_direct) {
        if ((rc = download_staged(c, 0, c->nel, el_xx, el_xv, el_ff, el_stride))) return rc;
        if ((rc = download_staged(c, c->nel, c->nion, ion_xx, ion_xv, ion_ff, ion_stride))) return rc;
    }
    fill_energies(c, nullptr);
    c->last.mv2el = c->h_scal[kScalMv2e];
    c->last.mv2ion = c->h_scal[kScalMv2i];
    if (e) *e = c->last;
    return TCP_OK;
}

int tcp_energies_get(tcp_ctx *c, tcp_energies *e) {
    if (!c || !e) return set_error(TCP_ERR_BAD_PARAM, "NULL argument");
    *e = c->last;
    return TCP_OK;
}

int tcp_histograms(tcp_ctx *c, double *rdf, double *vdf, int reset) {
    if (!c) return set_error(TCP_ERR_BAD_PARAM, "ctx is NULL");
    cudaSetDevice(c->device);
    std::vector<unsigned long long> h(5 * kNbin);
    TCP_CUDA(cudaMemcpyAsync(h.data(), c->rdf, sizeof(unsigned long long) * 3 * kNbin, cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaMemcpyAsync(h.data() + 3 * kNbin, c->vdf, sizeof(unsigned long long) * 2 * kNbin,
                             cudaMemcpyDeviceToHost, c->stream));
    TCP_CUDA(cudaStreamSynchronize(c->stream));
    // ordered pairs are counted once each: +2 per unordered pair as force.f90:102
    if (rdf)
        for (int k = 0; k < 3 * kNbin; ++k) rdf[k] = (double)h[k];
    if (vdf)
        for (int k = 0; k < 2 * kNbin; ++k) vdf[k] = (double)h[3 * kNbin + k];
    if (reset) {
        TCP_CUDA(cudaMemsetAsync(c->rdf, 0, sizeof(unsigned long long) * 3 * kNbin, c->stream));
        TCP_CUDA(cudaMemsetAsync(c->vdf, 0, sizeof(unsigned long long) * 2 * kNbin, c->stream));
        TCP_CUDA(cudaStreamSynchronize(c->stream));
    }
    return TCP_OK;
}

int tcp_time_component(tcp_ctx *c, int which, int reps, double dt, double *ms) {
    TCP_REQUIRE_READY(c);
    if (reps <= 0 || !ms) return set_error(TCP_ERR_BAD_PARAM, "reps must be positive");
    cudaEvent_t e0, e1;
    TCP_CUDA(cudaEventCreate(&e0));
    TCP_CUDA(cudaEventCreate(&e1));
    int rc = TCP_OK;
    if ((rc = autotune_pair(c))) return rc;
    auto one = [&]() -> int {
        if (which == 0) return launch_pair(c, energy_on(c), (c->flags & TCP_FLAG_RDF) != 0);
        return recip_launch(c);
    };
    if (which == 2 && (rc = ensure_graph(c, dt))) return rc;
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && !rc; ++r) rc = which == 2 ? launch_step(c, dt) : one();
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = sync_scalars(c))) return rc;
    *ms = (double)t / reps;
    return TCP_OK;
}

int tcp_time_steps(tcp_ctx *c, double dt, int nsteps, int flush_l2, double *out) {
    TCP_TRACE("tcp_time_steps");
    TCP_REQUIRE_READY(c);
    if (nsteps <= 0 || !out) return set_error(TCP_ERR_BAD_PARAM, "nsteps must be positive");
    int rc;
    if (flush_l2 && !c->l2_flush) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device);
        c->l2_flush_bytes = 2 * (size_t)std::max(l2, 64 << 20);
        TCP_CUDA(cudaMalloc(&c->l2_flush, c->l2_flush_bytes));
    }
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    if ((rc = ensure_graph(c, dt))) return rc;
    for (int s = 0; s < nsteps; ++s) {
        if (flush_l2) TCP_CUDA(cudaMemsetAsync(c->l2_flush, s & 0xff, c->l2_flush_bytes, c->stream));
        if ((rc = launch_step(c, dt))) return rc;
        TCP_CUDA(cudaEventSynchronize(c->ev[4]));
        // step; first kick (0-1); reciprocal (1-2, stream2); pair (1-3, concurrent
        // with the reciprocal chain); epilogue (from the later of 2 and 3 to 4)
        float t[5], e2, e3;
        cudaEventElapsedTime(&t[0], c->ev[0], c->ev[4]);
        cudaEventElapsedTime(&t[1], c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&t[2], c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&t[3], c->ev[1], c->ev[3]);
        cudaEventElapsedTime(&e2, c->ev[2], c->ev[4]);
        cudaEventElapsedTime(&e3, c->ev[3], c->ev[4]);
        t[4] = std::min(e2, e3);
        for (int k = 0; k < 5; ++k) out[k] += t[k];
        out[5] += 1.0;
    }
    if ((rc = sync_scalars(c))) return rc;
    fill_energies(c, nullptr);
    c->last.mv2el = c->h_scal[kScalMv2e];
    c->last.mv2ion = c->h_scal[kScalMv2i];
    return TCP_OK;
}

int tcp_launch_count(tcp_ctx *c, long long *count) {
    if (!c || !count) return set_error(TCP_ERR_BAD_PARAM, "NULL argument");
    *count = c->launches;
    return TCP_OK;
}

int tcp_fp32_peak(int device, double *tffma) {
    if (!tffma) return set_error(TCP_ERR_BAD_PARAM, "NULL argument");
    TCP_CUDA(cudaSetDevice(device));
    return launch_fp32_peak(device, tffma);
}

}  // extern "C"

namespace tcp {
int md_advance(tcp_ctx *c, double dt, int nsteps) {
    int rc;
    if ((rc = ::ensure_graph(c, dt))) return rc;
    for (int s = 0; s < nsteps; ++s)
        if ((rc = ::launch_step(c, dt))) return rc;
    return TCP_OK;
}
}  // namespace tcp

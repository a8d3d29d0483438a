/*
 * tcp_gpu.h -- C ABI of libtcpgpu.so, the GB300 (sm_103a) implementation of
 * the TCP_allpair force-and-integrate step.
 *
 * The reference drives this path through Fortran subroutines with implicit
 * interfaces and derived-type arguments (force.f90, vverlet.f90, init.f90).
 * Every entry point below replaces one of them; the comment above each
 * declaration names the routine and its file:line.  A Fortran caller binds
 * these with ISO_C_BINDING (fortran/tcp_gpu_mod.f90 in the package); other
 * callers use the same plain C types: no C++ and no CUDA types cross this
 * boundary.
 *
 * State model.  A tcp_ctx owns one system on one GPU: device-resident SoA
 * FP64 positions, velocities and forces (plus the 32-bit fixed-point position
 * copy of the FP32 pair kernel), the SPME meshes and cuFFT plans, the RDF/VDF
 * histograms and a CUDA stream.  Host arrays are authoritative only after
 * tcp_download().  Particles are ordered as in the reference: species 0
 * (electrons, "qel") first, then species 1 (ions, "qion").
 *
 * Units are the reference's (data.f90:21-24): Angstrom, eV, amu, time in
 * units of 10.18 fs, eps = 14.399644154020082 eV*A.
 *
 * Errors.  Every function returns 0 (TCP_OK) or a TCP_ERR_* code; the
 * reference STOPs instead (force.f90:19-22, main.f90:222-225).
 * tcp_last_error() gives a one-line message for the calling thread.
 * Contexts are not re-entrant: one host thread per context at a time.
 */
#ifndef TCP_GPU_H
#define TCP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define TCP_OK 0
#define TCP_ERR_BAD_PARAM 1     /* invalid argument or parameter combination   */
#define TCP_ERR_CUTOFF 2        /* rc > min(box)/2, force.f90:18-22            */
#define TCP_ERR_CUDA 3          /* CUDA runtime error (message has details)    */
#define TCP_ERR_CUFFT 4         /* cuFFT plan or execution failure             */
#define TCP_ERR_TIMEOUT 5       /* a bounded device-side wait gave up          */
#define TCP_ERR_NO_DEVICE 6     /* no usable sm_103 device                     */
#define TCP_ERR_STATE 7         /* call order (e.g. force before ewald_self)   */
#define TCP_ERR_NOMEM 8         /* device allocation failed                    */

/* ---- enumerations ------------------------------------------------------ */
#define TCP_PREC_FP64 0         /* plain FP64 pair kernel (the drop-in)        */
#define TCP_PREC_FP32C 1        /* FP32 pair arithmetic, compensated sums      */
#define TCP_PREC_FP32C_R64 2    /* TCP_PREC_FP32C real-space sum with the whole
                                 * reciprocal chain (spread, transforms,
                                 * influence, gather) in FP64                  */

#define TCP_EI_DEUTSCH 0        /* reference e-i term (erfc(ar)-exp(-r/rs))/r, force.f90:135-139 */
#define TCP_EI_KELBG 1          /* Kelbg e-i potential with length lambda_ei   */
#define TCP_EI_COULOMB 2        /* bare Coulomb for every pair                 */

#define TCP_THERMO_NOTEMP 0     /* vverlet.f90:174-223 */
#define TCP_THERMO_ISOKIN 1     /* vverlet.f90:301-372 */
#define TCP_THERMO_BEREND 2     /* vverlet.f90:227-298 */
#define TCP_THERMO_STOCH 3      /* vverlet.f90:9-127 (counter-based RNG)       */

#define TCP_RECIP_NONE 0        /* real-space sum only                         */
#define TCP_RECIP_SPME 1        /* smooth PME, force.f90:652-929               */
#define TCP_RECIP_EWALD 2       /* plain Ewald k-space sum, |n|^2 <= ewald_nmax2 */

/* tcp_set_flags bits */
#define TCP_FLAG_RDF 1u         /* accumulate RDF histograms in the pair sum   */
#define TCP_FLAG_VDF 2u         /* accumulate VDF histograms in the 2nd kick   */
#define TCP_FLAG_ENERGY 4u      /* compute Ur/Um (default on)                  */
#define TCP_FLAG_DETERMINISTIC 8u /* ordered-pair real-space kernels with a fixed
                                   * summation order: bitwise reproducible forces
                                   * and energies (the Newton-3 kernels add with
                                   * atomics in a varying order)               */

/* Parameters: the fields of TYPE PM (data.f90:68-74), the histogram
 * spacings of TYPE NM (data.f90:99) and the GPU build's own knobs. */
typedef struct tcp_params {
    double xm[2];           /* masses [amu] (PM%xm)                          */
    double q[2];            /* charges [e] (PM%q)                            */
    double tau;             /* Berendsen time constant (PM%tau)              */
    double alpha_lgv;       /* Langevin damping (PM%alpha)                   */
    double a;               /* Ewald alpha; <= 0 selects 3.1/rc (force.f90:23) */
    double box[3];          /* box lengths [A] (PM%box)                      */
    double Te, Ti;          /* target temperatures [eV]                      */
    double rs;              /* Deutsch length [A] (PM%rs)                    */
    double rc;              /* real-space cut-off [A] (PM%rc)                */
    int K[3];               /* SPME mesh (PM%K)                              */
    int order;              /* B-spline order, 4 (reference) .. 8            */
    double dx_ee, dx_ei, dx_ii;  /* RDF bin widths (NM%dx_*)                 */
    double dv_e, dv_i;      /* VDF bin widths (NM%dv_*, main.f90:286-287)    */
    int ei_model;           /* TCP_EI_*                                      */
    double lambda_ei;       /* Kelbg length [A]                              */
    double charge_scale;    /* q -> s q in every energy and force (1 = reference) */
    int precision;          /* TCP_PREC_*                                    */
    int reciprocal;         /* TCP_RECIP_*                                   */
    int ewald_nmax2;        /* plain Ewald: |n|^2 bound                      */
    int thermo;             /* TCP_THERMO_*                                  */
    int thermo_period;      /* apply ISOKIN/BEREND every n-th step (1 = reference) */
    uint64_t seed;          /* STOCH random stream                           */
} tcp_params;

/* Energies of the last force evaluation / step (TYPE ST, data.f90:89-92). */
typedef struct tcp_energies {
    double Ur;              /* real-space energy WITHOUT eps (sys%Ur)        */
    double Uo;              /* self energy WITHOUT eps (sys%Uo), plus the
                             * neutralising-background energy
                             * -pi Q^2/(2 V alpha^2) of a system with net
                             * charge Q (0 for neutral systems; the reference
                             * has no such term)                             */
    double Um;              /* reciprocal energy WITH eps (sys%Um)           */
    double Epot;            /* (Ur + Uo) * eps, main.f90:138                 */
    double mv2el, mv2ion;   /* sum m v^2 per species (sys%mv2el/mv2ion)      */
} tcp_energies;

typedef struct tcp_ctx tcp_ctx;

/* ---- lifecycle ------------------------------------------------------- */
/* Allocates the device state for nel electrons + nion ions on `device`.
 * Replaces the ALLOCATE of main.f90:45 / :335 for the GPU-resident arrays. */
int tcp_create(const tcp_params *p, int nel, int nion, int device, tcp_ctx **out);
int tcp_destroy(tcp_ctx *ctx);
const char *tcp_last_error(void);
const char *tcp_status_string(int code);
/* Library version and the compute capability it was built for (103). */
int tcp_version(int *major, int *minor, int *arch);

/* EWALD_SELF(NS,param,sys,PSI,COMM), force.f90:4-49: checks rc <= L/2,
 * sets alpha (3.1/rc unless p->a > 0) and rc^2, fills the influence mesh and
 * returns Uo (no eps): -alpha/sqrt(pi) sum q^2 (force.f90:44-45) plus, for a
 * net charge Q, the background term -pi Q^2/(2 V alpha^2).  Must precede
 * every force call. */
int tcp_ewald_self(tcp_ctx *ctx, double *alpha_out, double *Uo_out);

/* The GPU build's own parameters for callers that fill tcp_params from the
 * reference's tcp.prm (main.f90:221-294), which has no field for them; no
 * counterpart in the reference.  Keys and values, read first from the file
 * named by $TCP_GPU_PRM, else ./tcp_gpu.prm if it exists ("key value" or
 * "key = value" per line, '#' or '!' starts a comment), then from the
 * environment variables TCP_GPU_<KEY>, later ones overriding earlier ones:
 *   precision     fp64 | fp32c | fp32c_r64      -> p->precision
 *   ei_model      deutsch | kelbg | coulomb     -> p->ei_model
 *   reciprocal    none | spme | ewald           -> p->reciprocal
 *   order         4..8                          -> p->order
 *   alpha         Ewald alpha [1/A], 0 = 3.1/rc -> p->a
 *   lambda_ei     Kelbg length [A]              -> p->lambda_ei
 *   ewald_nmax2, thermo_period, seed, charge_scale -> the fields of that name
 *   device        GPU index                     -> *device (may be NULL)
 *   sync_every    host records refreshed every n steps by the Fortran
 *                 module's second half kick (0 = never) -> *sync_every
 * Fields without a key are left as they are.  An unknown key, a bad value
 * or an unreadable $TCP_GPU_PRM returns TCP_ERR_BAD_PARAM naming the line or
 * variable.  Touches no device. */
int tcp_params_from_env(tcp_params *p, int *device, int *sync_every);

/* Updates the parameters that may change between steps (temperatures,
 * thermostat, tau, charge scale, e-i length).  Box, mesh, order, counts and
 * precision are fixed at tcp_create. */
int tcp_set_params(tcp_ctx *ctx, const tcp_params *p);
int tcp_set_flags(tcp_ctx *ctx, unsigned flags);

/* ---- host <-> device ------------------------------------------------- */
/* Copy one species' records from host memory.  xx, xv, ff point at the first
 * record's xx(1), xv(1), ff(1) of a PT array (data.f90:32-35); stride_bytes
 * is the distance between consecutive records (104 for gfortran/ifort), so a
 * Fortran caller passes C_LOC(qel(1)%xx) and C_LOC(qel(2)) - C_LOC(qel(1)).
 * A NULL pointer skips that field.  species: 0 = qel, 1 = qion. */
int tcp_upload(tcp_ctx *ctx, int species, const double *xx, const double *xv,
               const double *ff, long stride_bytes);
int tcp_download(tcp_ctx *ctx, int species, double *xx, double *xv, double *ff,
                 long stride_bytes);
/* Plain (N,3) row-major arrays for all particles (electrons then ions);
 * NULL skips a field.  frec: the reciprocal (pme) forces of the last SPME call. */
int tcp_upload_soa(tcp_ctx *ctx, const double *x, const double *v, const double *f);
int tcp_download_soa(tcp_ctx *ctx, double *x, double *v, double *f, double *frec);

/* No counterpart in the reference.  The real-space sum of tcp_force_direct
 * for callers that cannot allocate device memory: programs whose device
 * memory belongs to another allocator (a pool that reserved the free HBM at
 * start-up) and step loops that forbid allocation after set-up because
 * cudaMalloc/cudaFree can synchronise the whole device.  No context and no
 * allocation: every temporary lives in one static 8 MiB device array that each
 * GPU loading the library holds until exit, so n is limited to what fits
 * (about 200,000 particles for TCP_PREC_FP32C, 140,000 for TCP_PREC_FP64);
 * larger n returns TCP_ERR_BAD_PARAM.  x and f are device arrays, SoA [3][n]
 * (electrons first); *Ur (host, may be NULL) gets Ur without eps.  Runs on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and returns when the
 * forces are written.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) with the caller's current device, which allocates
 * nothing.  Calls share the array: calls that overlap on the GPU race and
 * must be serialised.  After a non-zero return the contents of f are
 * undefined. */
int tcp_force_direct_noalloc(const tcp_params *p, int nel, int nion, const double *x, double *f,
                             double *Ur, void *stream);

/* ---- the force evaluation (main.f90:100-141) --------------------------- */
/* Force_direct_self + Force_direct_ext + Force_direct_sum for the whole
 * system (force.f90:52-372, main.f90:105-130): f is overwritten with the
 * real-space forces, *Ur (no eps) returned, RDF accumulated if enabled. */
int tcp_force_direct(tcp_ctx *ctx, double *Ur);
/* Force_SPME4(NS,param,sys,COMM,PSI,gsend,pme), force.f90:652-929: the
 * reciprocal forces (kept on the device, the pme array) and *Um (with eps).
 * With reciprocal == TCP_RECIP_EWALD the plain Ewald sum is used instead. */
int tcp_force_spme(tcp_ctx *ctx, double *Um);
/* SPME_SUM(NS,qel,qion,sys,COMM,pme,grec), force.f90:932-969: f += pme. */
int tcp_spme_sum(tcp_ctx *ctx);
/* REMOVE_RIGIDMTN(NS,qel,qion,COMM), force.f90:974-1007: f -= sum(f)/N. */
int tcp_remove_rigidmtn(tcp_ctx *ctx);
/* The four calls above in the order of main.f90:100-141, plus
 * Epot = (Ur+Uo)*eps (main.f90:138). */
int tcp_force(tcp_ctx *ctx, tcp_energies *e);

/* ---- integration (vverlet.f90) ----------------------------------------- */
/* VVerletNotemp1(NS,qel,qion,param,dt,gsend), vverlet.f90:132-171 (also the
 * first half of ISOKIN/BEREND, main.f90:88-92); VVerletStoch1
 * (vverlet.f90:9-59) when thermo == TCP_THERMO_STOCH. */
int tcp_vverlet1(tcp_ctx *ctx, double dt);
/* VVerletNotemp2 / VVerletIsokin2 / VVerletBerend2 / VVerletStoch2
 * (vverlet.f90:174-223, 301-372, 227-298, 62-127) selected by thermo;
 * returns sum m v^2 per species. */
int tcp_vverlet2(tcp_ctx *ctx, double dt, double *mv2el, double *mv2ion);
/* Finit(...), init.f90:152-239: forces at x - dt v (the reference's quirk),
 * positions restored. */
int tcp_finit(tcp_ctx *ctx, double dt, tcp_energies *e);

/* ---- the step (main.f90:81-153) ---------------------------------------- */
/* nsteps MD steps (vverlet1, SPME, direct sum, SPME_SUM, Epot, net-force
 * removal, vverlet2+thermostat), captured once as a CUDA graph and replayed.
 * e receives the energies of the last step (NULL: not read back). */
int tcp_md_steps(tcp_ctx *ctx, double dt, int nsteps, tcp_energies *e);
/* The same steps on the caller's PT records, which main.f90:81-153 updates in
 * place: the fields given (xx, xv, ff as for tcp_upload; NULL skips one) are
 * read from the qel and qion records, nsteps steps run, and the same fields
 * are written back.  Equal to tcp_upload(0) + tcp_upload(1) + tcp_md_steps +
 * tcp_download(0) + tcp_download(1) with one wait for the device instead of
 * five.  Every argument is checked before anything runs. */
int tcp_md_steps_records(tcp_ctx *ctx, double dt, int nsteps,
                         double *el_xx, double *el_xv, double *el_ff, long el_stride_bytes,
                         double *ion_xx, double *ion_xv, double *ion_ff, long ion_stride_bytes,
                         tcp_energies *e);
/* Energies of the most recent evaluation without launching anything. */
int tcp_energies_get(tcp_ctx *ctx, tcp_energies *e);

/* ---- histograms (NS%RDF_*, NS%VDF_*, data.f90:100-101) ----------------- */
/* rdf: 3*(Ndist+1) doubles ee|ei|ii; vdf: 2*(Ndist+1) doubles e|i.  Counts
 * follow the reference (+2 per pair, +1 per particle).  reset != 0 zeroes
 * the device copies afterwards (DUMP does so, result.f90:264-268). */
int tcp_histograms(tcp_ctx *ctx, double *rdf, double *vdf, int reset);

/* ---- many independent systems in one context ---------------------------------- */
/* No single counterpart in the reference, which runs one system per job
 * (main.f90): a batch steps nrep independent replicas, each exactly as
 * main.f90:81-153 steps one system, with one persistent real-space launch
 * over all replicas, batched SPME transforms per mesh size and one CUDA graph
 * per step.  params[r], nel[r], nion[r] describe replica r; all replicas use
 * TCP_PREC_FP32C, TCP_RECIP_SPME, cubic boxes, one B-spline order, and a
 * NOTEMP / ISOKIN / BEREND thermostat applied every step. */
typedef struct tcp_batch tcp_batch;
int tcp_batch_create(const tcp_params *params, const int *nel, const int *nion, int nrep, int device,
                     tcp_batch **out);
int tcp_batch_destroy(tcp_batch *b);
/* EWALD_SELF for every replica; Uo[nrep] (no eps) may be NULL. */
int tcp_batch_ewald_self(tcp_batch *b, double *Uo);
/* (n_r, 3) row-major host arrays of replica r; NULL skips a field. */
int tcp_batch_upload(tcp_batch *b, int rep, const double *x, const double *v, const double *f);
int tcp_batch_download(tcp_batch *b, int rep, double *x, double *v, double *f);
/* Forces and energies (e[nrep], may be NULL) of all replicas at the current positions. */
int tcp_batch_force(tcp_batch *b, tcp_energies *e);
/* nsteps MD steps of every replica with time step dt; e[nrep] may be NULL. */
int tcp_batch_md_steps(tcp_batch *b, double dt, int nsteps, tcp_energies *e);
/* The batched real-space kernel the batch autotuner picked (variant index) and
 * the per-candidate times in ms (0 when not timed), up to nmax entries. */
int tcp_batch_autotune_report(tcp_batch *b, int *variant, double *ms, int nmax);
/* Name of batched real-space variant `variant` (NULL past the last): "b_", i-particles per
 * lane, unroll, warps and CTAs per SM, packed forms ("x2", "x2l"). */
const char *tcp_batch_variant_name(int variant);
/* The CTAs the batch autotuner left out of the persistent batched pair grid so
 * that the replicas' SPME chains, which run beside it, find room on the SMs
 * (they join the pair launch's work once the chains are done); the candidates
 * and the time of the pair launch with the chains beside it for each, up to
 * the join, replayed as one captured graph (ms, 0 when not timed), up to nmax
 * entries.  TCP_BATCH_RESERVE=k forces k. */
int tcp_batch_overlap_report(tcp_batch *b, int *reserve, int *candidates, double *ms, int nmax);
/* Mean device time of one launch of a batch component over `reps` launches
 * on the batch's stream (CUDA events), after one untimed launch: which 0 =
 * the batched real-space pair launch alone, 1 = the SPME chains of every
 * replica alone (forked onto the second stream and joined back). */
int tcp_batch_time_component(tcp_batch *b, int which, int reps, double *ms_per_launch);
/* Device time of nsteps batched steps, one graph replay each, with the L2
 * cache overwritten before each when flush_l2 is set: out[6] = summed ms of
 * the step, the first half kick, the SPME chains (beside the pair launch),
 * the pair launch, the epilogue after the later of the two, and the step
 * count (CUDA events recorded inside the step graph). */
int tcp_batch_time_steps(tcp_batch *b, double dt, int nsteps, int flush_l2, double *out);

/* ---- derivatives ---------------------------------------------------------
 * No counterpart in the reference (it computes no derivatives): the analytic
 * derivatives of the energy of force.f90 / EWALD_SELF and of the NOTEMP step
 * of vverlet.f90, for the context's parameters and precision (the real-space
 * part in the context's precision; the reciprocal part in FP64).  "lambda" is
 * lambda_ei for TCP_EI_KELBG and rs for TCP_EI_DEUTSCH; every lambda
 * derivative is 0 for TCP_EI_COULOMB. */

/* At the current positions: *E = Epot + Um (eV, the potential energy of the
 * ener files), *dE_dlambda (eV/A) and *dE_dscale = dE/ds for charges s q
 * (every term is quadratic in s, so 2E/s).  The stored forces are kept (the
 * energy evaluation writes them to scratch first).  Any pointer may be NULL. */
int tcp_adjoint_energy(tcp_ctx *ctx, double *E, double *dE_dlambda, double *dE_dscale);

/* Hessian-vector product of the potential energy at the current positions:
 * hw = (d^2 E / dx dx) w, w and hw host arrays [N][3] in particle order
 * (electrons, then ions), hw in eV/A^2 times the unit of w.  The mean-force
 * removal of REMOVE_RIGIDMTN is not applied.  *dF_dlambda_w (may be NULL)
 * = sum_i dF_i/dlambda . w_i with F = -grad E. */
int tcp_hvp(tcp_ctx *ctx, const double *w, double *hw, double *dF_dlambda_w);

/* Reverse mode through nsteps NOTEMP steps of tcp_md_steps from the current
 * x, v (the start forces are recomputed, f_0 = F(x_0; lambda)):
 *   *J = (1/K) sum_{k=1..K} (mv2el_k + mv2ion_k) / (3N)   (K = nsteps)
 * and *dJ_dlambda by the discrete adjoint of the step, with checkpoints of
 * (x, v) every `every` steps and the steps in between recomputed.  On return
 * the context holds the state after step K, as after tcp_md_steps.
 * TCP_ERR_BAD_PARAM unless thermo = TCP_THERMO_NOTEMP. */
int tcp_reverse_md(tcp_ctx *ctx, double dt, int nsteps, int every, double *J, double *dJ_dlambda);

/* ---- measurement hooks ---------------------------------------------------- */
/* Runs `reps` launches of one component on the context's stream and returns
 * the mean device time per launch from CUDA events recorded on that stream.
 * which: 0 = real-space pair kernel (the RDF-binning form when the context's
 * flags hold TCP_FLAG_RDF), 1 = SPME chain, 2 = full md step. */
int tcp_time_component(tcp_ctx *ctx, int which, int reps, double dt, double *ms_per_launch);
/* Times nsteps MD steps one by one with CUDA events recorded on the
 * context's stream (also inside the captured step graph), optionally writing
 * a buffer of twice the L2 size between steps (outside the timed spans).
 * out[6] receives the summed milliseconds of: whole steps, first half kick,
 * reciprocal sum (its span on the second stream, where it runs concurrently
 * with the pair kernel), real-space pair kernel, force epilogue + second half
 * kick (from the later of the two to the step end), and the number of steps
 * timed. */
int tcp_time_steps(tcp_ctx *ctx, double dt, int nsteps, int flush_l2, double *out);
/* The FP32C real-space kernel the autotuner picked for this context (0 =
 * ordered pairs, >= 1 = Newton-3 variants) and the per-candidate times in ms
 * (ms[k] for variant k, 0 when not timed), up to nmax entries. */
int tcp_autotune_report(tcp_ctx *ctx, int *variant, double *ms, int nmax);
/* Name of FP32C real-space variant `variant` ("ordered" for 0, NULL past the
 * last): i-particles per lane, unroll, warps and CTAs per SM, packed forms
 * ("x2", "x2l": shared-memory j positions) and "_p5" for the degree-5 Ewald
 * erfc polynomial (one FMA fewer per pair than degree 6). */
const char *tcp_pair_variant_name(int variant);
/* The number of CTAs the autotuner left out of the persistent Newton-3 grid
 * so that the reciprocal chain, which runs beside the pair kernel in a step,
 * finds room on the SMs (they join the pair kernel's work once the chain is
 * done); the candidates and the time of the pair kernel with the chain
 * beside it for each, up to the join of both, replayed as one captured graph
 * (ms, 0 when not timed), up to nmax entries.  TCP_PAIR_RESERVE=k forces k. */
int tcp_overlap_report(tcp_ctx *ctx, int *reserve, int *candidates, double *ms, int nmax);
/* Kernel launches issued by the context so far (all kernels of this library). */
int tcp_launch_count(tcp_ctx *ctx, long long *count);
/* Measured FP32 FFMA issue rate of the device: a calibration kernel of
 * dependent-chain-free FFMAs, returned in 1e12 FFMA/s. */
int tcp_fp32_peak(int device, double *tffma_per_s);

#ifdef __cplusplus
}
#endif
#endif

/*
 * tcp_oracle.h -- FP64 CPU restatement of the TCP_allpair force-and-integrate
 * path.  TEST INFRASTRUCTURE ONLY: this library is the checker that the CUDA
 * library (libtcpgpu.so) is compared against, and the timed CPU baseline of the
 * benchmark.  It is never linked into, loaded by or called from the product.
 *
 * Parity status: the reference (Fortran 90 + MPI + FFTE) has no tests, no
 * fixtures and cannot be compiled where this code is built, so the restatement
 * is NOT pinned by reference-generated goldens ("parity unpinned" by the
 * reference).  It is pinned by analytic known answers instead: closed-form pair
 * forces, Madelung constants of NaCl/CsCl lattices, SPME -> plain Ewald
 * convergence, force = -grad(energy) by central differences, E(s q) = s^2 E(q),
 * sum of forces = 0 (tests/test_oracle_*.py, tests/golden/).
 *
 * Units and conventions are the reference's (data.f90:21-24): lengths in
 * Angstrom, energies in eV, masses in amu, time in units of tps = 10.18 fs,
 * eps = e^2/(4 pi eps0) = 14.399644154020082 eV*A.  Particles are ordered
 * electrons first (species 0), then ions (species 1), positions AoS x[3*i+k].
 */
#ifndef TCP_ORACLE_H
#define TCP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NDIST 500          /* data.f90:16 Ndist; histograms have Ndist+1 bins */
#define ORC_EPS 14.399644154020082
#define ORC_TPS 10.180505306645389
#define ORC_PI 3.1415926535897931
#define ORC_SQRTPI 1.7724538509055159

/* e-i real-space model */
#define ORC_EI_DEUTSCH 0   /* reference: q1q2 (erfc(ar) - exp(-r/rs))/r, force.f90:135-139 */
#define ORC_EI_KELBG 1     /* q1q2 [erfc(ar)/r - exp(-r^2/l^2)/r + sqrt(pi) erfc(r/l)/l] */
#define ORC_EI_COULOMB 2   /* bare Ewald Coulomb for every pair (lattice known answers) */

/* thermostats, main.f90:88-92 and 145-153 */
#define ORC_NOTEMP 0
#define ORC_ISOKIN 1
#define ORC_BEREND 2
#define ORC_STOCH 3

/* Fields follow TYPE PM (data.f90:68-74) plus the histogram spacings of TYPE NM
 * (data.f90:97-101) and the extensions the GPU library also takes. */
typedef struct orc_params {
    double xm[2], q[2];        /* masses [amu], charges [e] per species        */
    double tau, alpha_lgv;     /* Berendsen tau, Langevin damping (PM%alpha)    */
    double a;                  /* Ewald alpha (PM%a), set by orc_ewald_self     */
    double box[3];             /* box lengths [A]                               */
    double Te, Ti;             /* target temperatures [eV]                      */
    double rs, rc, rc2;        /* Deutsch length, cut-off, cut-off^2            */
    int K[3];                  /* SPME mesh                                     */
    int order;                 /* B-spline order (reference: 4)                 */
    double dx_ee, dx_ei, dx_ii;/* RDF bin widths                                */
    double dv_e, dv_i;         /* VDF bin widths (main.f90:286-287)             */
    int ei_model;              /* ORC_EI_*                                      */
    double lambda_ei;          /* Kelbg lambda [A]                              */
    double charge_scale;       /* q -> s q for all pair / mesh charges (1 = ref) */
} orc_params;

/* EWALD_SELF (force.f90:4-49).  Sets p->a (3.1/rc when alpha_override <= 0,
 * force.f90:23) and p->rc2 (force.f90:24); fills psi[K1*K2*K3] (Fortran
 * order, ix fastest) with exp(-pi^2 m^2/a^2)/m^2 and psi[0] = 0 (the
 * reference leaves PSI(1,1,1) unset); returns Uo = -(a/sqrtpi) sum q^2
 * without eps (force.f90:44-45).  Returns -1 when rc > min(box)/2
 * (force.f90:18-22), else 0.  psi may be NULL. */
int orc_ewald_self(orc_params *p, int nel, int nion, double alpha_override,
                   double *psi, double *Uo);

/* Force_direct_self (force.f90:52-180) over the whole system, i.e. the
 * union of Force_direct_self + Force_direct_ext + Force_direct_sum of all
 * ranks (main.f90:105-130) on one rank.  f is overwritten, Ur is the
 * real-space energy WITHOUT eps (force.f90:105,137,169), rdf (3*(Ndist+1),
 * ee|ei|ii) is incremented by 2 per pair inside the cut-off when non-NULL.
 * nthreads <= 0 uses all OpenMP threads. */
void orc_force_direct(const orc_params *p, int nel, int nion, const double *x,
                      double *f, double *Ur, double *rdf, int nthreads);

/* Same pair sum restricted to rows [i0, i1) of the full (ordered) pair matrix:
 * f[3*(i-i0)+k] gets the force on particle i from every j != i; *Ur gets half
 * of the row energies (so summing over all row blocks gives the full Ur).
 * This is the sampled workload of the timed CPU baseline. */
void orc_force_direct_rows(const orc_params *p, int nel, int nion,
                           const double *x, int i0, int i1, double *f,
                           double *Ur, int nthreads);

/* Force_SPME4 (force.f90:652-929) generalised to B-spline order p->order.
 * frec = reciprocal force on every particle (pme%xx, eV/A), *Um with eps
 * (force.f90:921).  psi as filled by orc_ewald_self.  Order 4 uses the
 * reference's explicit cubic weights (force.f90:703-738); other orders the
 * Cox-de Boor recursion.  Returns 0. */
int orc_force_spme(const orc_params *p, int nel, int nion, const double *x,
                   const double *psi, double *frec, double *Um);

/* |b(m)|^-2 per axis for order p (the 36/(4+2cos)^2 of force.f90:834-839 for
 * p=4).  out[K] */
void orc_bspline_moduli(int order, int K, double *out);

/* Plain Ewald reciprocal sum over integer vectors n with |n|^2 <= nmax2
 * (m = n/L).  frec forces (eV/A), *Uk energy with eps.  Same influence
 * function as the SPME path without the B-spline approximation. */
void orc_ewald_ksum(const orc_params *p, int nel, int nion, const double *x,
                    int nmax2, double *frec, double *Uk, int nthreads);

/* SPME_SUM (force.f90:932-969): f += frec */
void orc_spme_sum(int n, double *f, const double *frec);

/* REMOVE_RIGIDMTN (force.f90:974-1007): f -= sum(f)/N */
void orc_remove_rigidmtn(int n, double *f);

/* VVerletNotemp1 (vverlet.f90:132-171): v += dt f/(2m); x += dt v; wrap */
void orc_vverlet1(const orc_params *p, int nel, int nion, double dt,
                  double *x, double *v, const double *f);

/* VVerletStoch1 (vverlet.f90:9-59): damped half kick, drift, wrap */
void orc_vverlet_stoch1(const orc_params *p, int nel, int nion, double dt,
                        double *x, double *v, const double *f);

/* Second half steps.  thermo = ORC_NOTEMP (vverlet.f90:174-223),
 * ORC_ISOKIN (vverlet.f90:301-372), ORC_BEREND (vverlet.f90:227-298),
 * ORC_STOCH (vverlet.f90:62-127, with the Gaussian numbers eta[3N] supplied
 * by the caller instead of the compiler RNG; f is modified as there).
 * apply_thermostat = 0 turns ISOKIN/BEREND into NOTEMP for this step (the
 * thermostat period extension).  mv2 = sum m v^2 per species (not halved),
 * vdf (2*(Ndist+1), e|i) incremented when non-NULL. */
void orc_vverlet2(const orc_params *p, int thermo, int apply_thermostat,
                  int nel, int nion, double dt, double *v, double *f,
                  const double *eta, double *mv2el, double *mv2ion,
                  double *vdf);

/* Full force evaluation (main.f90:100-141): SPME, direct sum, SPME_SUM,
 * REMOVE_RIGIDMTN.  reciprocal: 0 none, 1 SPME, 2 plain Ewald k-sum with
 * nmax2.  Outputs f (total, net force removed), *Ur (no eps), *Um (eps). */
int orc_force_total(const orc_params *p, int nel, int nion, const double *x,
                    const double *psi, int reciprocal, int nmax2, double *f,
                    double *Ur, double *Um, double *rdf, int nthreads);

/* Finit (init.f90:152-239): forces evaluated at x - dt v, x restored. */
int orc_finit(const orc_params *p, int nel, int nion, double dt, double *x,
              const double *v, const double *psi, double *f, double *Ur,
              double *Um, int nthreads);

/* One MD step in the order of main.f90:81-153 (NOTEMP/ISOKIN/BEREND);
 * reciprocal as in orc_force_total.
 * energies[5] = {Ur, Um, Epot=(Ur+Uo)*eps, mv2el, mv2ion}. */
int orc_md_step(const orc_params *p, int thermo, int apply_thermostat,
                int nel, int nion, double dt, double *x, double *v, double *f,
                const double *psi, double Uo, int reciprocal, int nmax2,
                double *energies, double *rdf, double *vdf, int nthreads);

/* ---- derivatives (no reference counterpart: the reference computes none).
 * Pinned by central finite differences of the routines above. ---- */

/* dE/dlambda (eV/A) of the total potential energy: lambda = lambda_ei
 * (Kelbg) or rs (Deutsch); only the e-i real-space term depends on it. */
void orc_adjoint_energy(const orc_params *p, int nel, int nion, const double *x,
                        double *dEdl, int nthreads);

/* hw = H w, H = d^2 E / dx dx of the total potential energy (real space +
 * reciprocal as in orc_force_total, without the mean-force removal);
 * *dFdl_w = sum_i dF_i/dlambda . w_i (F = -grad E).  AoS [3N] arrays. */
void orc_hvp(const orc_params *p, int nel, int nion, const double *x,
             const double *psi, int reciprocal, int nmax2, const double *w,
             double *hw, double *dFdl_w, int nthreads);

/* Reverse mode through K NOTEMP steps of orc_md_step from (x0, v0), f_0 =
 * F(x_0): J = mean over steps 1..K of (mv2el + mv2ion)/(3N) and dJ/dlambda,
 * checkpoints every M steps with recomputation in between.  Returns 0. */
int orc_reverse_md(const orc_params *p, int nel, int nion, const double *x0,
                   const double *v0, const double *psi, int reciprocal,
                   int nmax2, double dt, int K, int M, double *J, double *dJdl,
                   int nthreads);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif

/*
 * tcp_oracle.c -- FP64 CPU restatement of the TCP_allpair force-and-integrate
 * path (force.f90, vverlet.f90, init.f90).  TEST INFRASTRUCTURE ONLY: the
 * checker for the CUDA library and the timed CPU baseline; never part of the
 * product.  Parity is unpinned by reference goldens (the Fortran/MPI/FFTE
 * reference cannot be built here and ships no tests); it is pinned by the
 * analytic known answers listed in tcp_oracle.h.
 *
 * Each function cites the reference lines it restates.  Arithmetic is kept in
 * the reference's order where that is cheap (pair expressions, spline
 * polynomials, loop structure); the OpenMP reductions only change summation
 * order (FP64 rounding at the 1e-16 level).
 */
#include "tcp_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int nthreads_or_max(int nt) { return nt > 0 ? nt : orc_max_threads(); }

/* Fortran DNINT: round half away from zero (C round()). */
static inline double min_image(double x, double L) { return x - L * round(x / L); }

/* ------------------------------------------------------------------ */
/* EWALD_SELF, force.f90:4-49                                          */
/* ------------------------------------------------------------------ */
int orc_ewald_self(orc_params *p, int nel, int nion, double alpha_override,
                   double *psi, double *Uo) {
    double rc_cut = fmin(fmin(p->box[0], p->box[1]), p->box[2]) / 2.0; /* :18 */
    if (p->rc > rc_cut) return -1;                                       /* :19-22 */
    p->a = alpha_override > 0.0 ? alpha_override : 3.1 / p->rc;          /* :23 */
    p->rc2 = p->rc * p->rc;                                              /* :24 */
    if (psi) {
        const int K1 = p->K[0], K2 = p->K[1], K3 = p->K[2];
        for (int k = 0; k < K3; ++k) {
            int iz = (k + K3 / 2) % K3 - K3 / 2;                         /* :33 */
            for (int j = 0; j < K2; ++j) {
                int iy = (j + K2 / 2) % K2 - K2 / 2;                     /* :31 */
                for (int i = 0; i < K1; ++i) {
                    int ix = (i + K1 / 2) % K1 - K1 / 2;                 /* :29 */
                    long idx = i + (long)K1 * (j + (long)K2 * k);
                    int m = ix * ix + iy * iy + iz * iz;                 /* :34 */
                    if (m != 0) {
                        double m2 = (double)ix * ix / (p->box[0] * p->box[0]) +
                                    (double)iy * iy / (p->box[1] * p->box[1]) +
                                    (double)iz * iz / (p->box[2] * p->box[2]);
                        psi[idx] = exp(-m2 * ORC_PI * ORC_PI / (p->a * p->a)) / m2; /* :38 */
                    } else {
                        psi[idx] = 0.0; /* PSI(1,1,1) is never set by the reference */
                    }
                }
            }
        }
    }
    if (Uo) {
        double s = p->charge_scale;
        double u = -(double)nel * (s * p->q[0]) * (s * p->q[0]) -
                   (double)nion * (s * p->q[1]) * (s * p->q[1]);         /* :44 */
        /* net charge Q: the uniform neutralising background of the Ewald sum,
         * -pi Q^2 / (2 V alpha^2) (not in the reference; 0 for neutral systems) */
        double Q = (double)nel * s * p->q[0] + (double)nion * s * p->q[1];
        double V = p->box[0] * p->box[1] * p->box[2];
        *Uo = u * p->a / ORC_SQRTPI                                      /* :45 */
              - ORC_PI * Q * Q / (2.0 * V * p->a * p->a);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Pair terms of Force_direct_self, force.f90:87-178                   */
/* ------------------------------------------------------------------ */
/* Coulomb erfc pair (e-e :104-106, i-i :168-170).  Returns energy term
 * (no eps) and writes df (with eps). */
static inline double pair_coulomb(double a, double qq, double r2, double r, double *df) {
    double x = 1.0 - erf(a * r);                                         /* :104 */
    *df = ORC_EPS * qq * (2.0 * exp(-a * a * r2) * a * r / ORC_SQRTPI + x) / r2 / r; /* :106 */
    return qq * x / r;                                                   /* :105 */
}

/* Deutsch e-i pair, force.f90:135-139 */
static inline double pair_deutsch(double a, double rs, double qq, double r2, double r, double *df) {
    double x = 1.0 - erf(a * r);
    double y = exp(-r / rs);
    *df = ORC_EPS * qq * ((2.0 * exp(-a * a * r2) * a * r / ORC_SQRTPI + x - y) / r2 / r - y / r2 / rs);
    return qq * (x - y) / r;
}

/* Kelbg e-i pair (an extension of the reference, which has Deutsch):
 *   V = qq [erfc(ar)/r - exp(-r^2/l^2)/r + sqrt(pi) erfc(r/l)/l]
 *   -dV/dr / r = qq [erfc(ar) + 2ar/sqrt(pi) exp(-a^2 r^2) - exp(-r^2/l^2)] / r^3 */
static inline double pair_kelbg(double a, double lam, double qq, double r2, double r, double *df) {
    double x = erfc(a * r);
    double g = exp(-r2 / (lam * lam));
    *df = ORC_EPS * qq * (x + 2.0 * a * r / ORC_SQRTPI * exp(-a * a * r2) - g) / (r2 * r);
    return qq * (x / r - g / r + ORC_SQRTPI * erfc(r / lam) / lam);
}

static inline double pair_eval(const orc_params *p, int si, int sj, double qi, double qj,
                               double r2, double r, double *df) {
    double qq = qi * qj;
    if (si != sj) {
        if (p->ei_model == ORC_EI_DEUTSCH) return pair_deutsch(p->a, p->rs, qq, r2, r, df);
        if (p->ei_model == ORC_EI_KELBG) return pair_kelbg(p->a, p->lambda_ei, qq, r2, r, df);
    }
    return pair_coulomb(p->a, qq, r2, r, df);
}

static inline void rdf_add(double *rdf, double r, double dx) {
    /* idx = INT(r/dx)+1; IF (idx <= Ndist+1) RDF(idx) += 2, force.f90:99-103 */
    double t = r / dx;
    if (t < (double)(ORC_NDIST + 1)) {
        int b = (int)t;
        if (b <= ORC_NDIST) rdf[b] += 2.0;
    }
}

void orc_force_direct(const orc_params *p, int nel, int nion, const double *x,
                      double *f, double *Ur, double *rdf, int nthreads) {
    const int n = nel + nion;
    const int nt = nthreads_or_max(nthreads);
    const double s = p->charge_scale;
    const double qs[2] = {s * p->q[0], s * p->q[1]};
    const double dxs[3] = {p->dx_ee, p->dx_ei, p->dx_ii};
    double *fbuf = (double *)calloc((size_t)nt * 3 * n, sizeof(double));
    double *rbuf = rdf ? (double *)calloc((size_t)nt * 3 * (ORC_NDIST + 1), sizeof(double)) : NULL;
    double ur = 0.0;
#pragma omp parallel num_threads(nt) reduction(+ : ur)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *fl = fbuf + (size_t)tid * 3 * n;
        double *rl = rbuf ? rbuf + (size_t)tid * 3 * (ORC_NDIST + 1) : NULL;
        /* The three triangular loops e-e (:87-113), e-i (:118-147), i-i
         * (:151-178) are the unique pairs i<j of the species-ordered array. */
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < n - 1; ++i) {
            int si = i < nel ? 0 : 1;
            for (int j = i + 1; j < n; ++j) {
                int sj = j < nel ? 0 : 1;
                double xr[3], r2 = 0.0;
                for (int k = 0; k < 3; ++k) {                            /* :90-94 */
                    xr[k] = min_image(x[3 * i + k] - x[3 * j + k], p->box[k]);
                    r2 += xr[k] * xr[k];
                }
                if (r2 < p->rc2) {                                       /* :96 */
                    double r = sqrt(r2), df;
                    if (rl) rdf_add(rl + (si + sj) * (ORC_NDIST + 1), r, dxs[si + sj]);
                    ur += pair_eval(p, si, sj, qs[si], qs[sj], r2, r, &df);
                    for (int k = 0; k < 3; ++k) {                        /* :107-110 */
                        fl[3 * i + k] += df * xr[k];
                        fl[3 * j + k] -= df * xr[k];
                    }
                }
            }
        }
    }
    memset(f, 0, sizeof(double) * 3 * (size_t)n);                        /* :73-78 */
    for (int t = 0; t < nt; ++t)
        for (long i = 0; i < 3L * n; ++i) f[i] += fbuf[(size_t)t * 3 * n + i];
    if (rdf)
        for (int t = 0; t < nt; ++t)
            for (int i = 0; i < 3 * (ORC_NDIST + 1); ++i) rdf[i] += rbuf[(size_t)t * 3 * (ORC_NDIST + 1) + i];
    *Ur = ur;                                                            /* :79, main.f90:119 */
    free(fbuf);
    free(rbuf);
}

void orc_force_direct_rows(const orc_params *p, int nel, int nion, const double *x,
                           int i0, int i1, double *f, double *Ur, int nthreads) {
    const int n = nel + nion;
    const int nt = nthreads_or_max(nthreads);
    const double s = p->charge_scale;
    const double qs[2] = {s * p->q[0], s * p->q[1]};
    double ur = 0.0;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4) reduction(+ : ur)
    for (int i = i0; i < i1; ++i) {
        int si = i < nel ? 0 : 1;
        double fi[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            int sj = j < nel ? 0 : 1;
            double xr[3], r2 = 0.0;
            for (int k = 0; k < 3; ++k) {
                xr[k] = min_image(x[3 * i + k] - x[3 * j + k], p->box[k]);
                r2 += xr[k] * xr[k];
            }
            if (r2 < p->rc2) {
                double r = sqrt(r2), df;
                ur += 0.5 * pair_eval(p, si, sj, qs[si], qs[sj], r2, r, &df);
                for (int k = 0; k < 3; ++k) fi[k] += df * xr[k];
            }
        }
        for (int k = 0; k < 3; ++k) f[3 * (i - i0) + k] = fi[k];
    }
    *Ur = ur;
}

/* ------------------------------------------------------------------ */
/* SPME, force.f90:652-929                                            */
/* ------------------------------------------------------------------ */
/* Cardinal B-spline M_n(y), support [0, n] (Cox-de Boor recursion). */
static double bspline_M(int n, double y) {
    if (y <= 0.0 || y >= (double)n) return 0.0;
    if (n == 2) return 1.0 - fabs(y - 1.0);
    return (y * bspline_M(n - 1, y) + ((double)n - y) * bspline_M(n - 1, y - 1.0)) / (double)(n - 1);
}

/* Weights W[j] and dW/du[j], j = 0..p-1, on grid points floor(u) + j - (p-3).
 * Order 4 restates the explicit cubics of force.f90:703-738 (AX/AXX) whose
 * grid points are INT(u)+i-2, i=1..4 (force.f90:742-744). */
static void spline_weights(int p, double u, double *W, double *dW) {
    if (p == 4) {
        double z = trunc(u) - u + 1.0;                                   /* :703 */
        W[0] = z * z * z / 6.0;                                          /* :706 */
        dW[0] = -3. * z * z / 6.0;                                       /* :707 */
        z += 1.0;
        W[1] = (-3. * z * z * z + 12. * z * z - 12. * z + 4.) / 6.0;    /* :709 */
        dW[1] = (9. * z * z - 24. * z + 12.) / 6.0;                      /* :710 */
        z += 1.0;
        W[2] = (3. * z * z * z - 24. * z * z + 60. * z - 44.) / 6.0;    /* :712 */
        dW[2] = (-9. * z * z + 48. * z - 60.) / 6.0;                     /* :713 */
        z += 1.0;
        W[3] = (-z * z * z + 12. * z * z - 48. * z + 64.) / 6.0;        /* :715 */
        dW[3] = (3. * z * z - 24. * z + 48.) / 6.0;                      /* :716 */
        return;
    }
    double w = u - trunc(u);   /* u >= 0 for wrapped positions: trunc = floor */
    for (int j = 0; j < p; ++j) {
        double y = w + (double)(p - 1 - j);       /* = u - k + 2 for k = floor(u)+j-(p-3) */
        W[j] = bspline_M(p, y);
        dW[j] = bspline_M(p - 1, y) - bspline_M(p - 1, y - 1.0);
    }
}

void orc_bspline_moduli(int order, int K, double *out) {
    /* |b(m)|^-2 = 1/|sum_{k=0}^{p-2} M_p(k+1) exp(2 pi i m k/K)|^2.  For p=4 this
     * is 36/(4+2cos(2 pi m/K))^2 exactly as force.f90:834-839. */
    double *den = (double *)malloc(sizeof(double) * K);
    for (int m = 0; m < K; ++m) {
        if (order == 4) {
            double z = 4.0 + 2.0 * cos(2.0 * ORC_PI * m / K);
            den[m] = z * z / 36.0;
            continue;
        }
        double re = 0.0, im = 0.0;
        for (int k = 0; k <= order - 2; ++k) {
            double mk = bspline_M(order, (double)(k + 1));
            re += mk * cos(2.0 * ORC_PI * m * k / K);
            im += mk * sin(2.0 * ORC_PI * m * k / K);
        }
        den[m] = re * re + im * im;
    }
    /* odd orders vanish at the Nyquist index: use the mean of the neighbours */
    for (int m = 0; m < K; ++m)
        if (den[m] < 1e-7) den[m] = 0.5 * (den[(m - 1 + K) % K] + den[(m + 1) % K]);
    for (int m = 0; m < K; ++m) out[m] = 1.0 / den[m];
    free(den);
}

/* In-place 1-D complex DFT along a strided line, sign = -1 or +1, no
 * normalisation.  Radix-2 for powers of two, direct sum otherwise. */
static void dft_line(double complex *a, int n, long stride, int sign, double complex *tmp) {
    for (int i = 0; i < n; ++i) tmp[i] = a[i * stride];
    if ((n & (n - 1)) == 0) {
        for (int i = 1, j = 0; i < n; ++i) {
            int bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) { double complex t = tmp[i]; tmp[i] = tmp[j]; tmp[j] = t; }
        }
        for (int len = 2; len <= n; len <<= 1) {
            double ang = sign * 2.0 * ORC_PI / len;
            for (int i = 0; i < n; i += len)
                for (int k = 0; k < len / 2; ++k) {
                    double complex w = cos(ang * k) + I * sin(ang * k);
                    double complex u = tmp[i + k], v = tmp[i + k + len / 2] * w;
                    tmp[i + k] = u + v;
                    tmp[i + k + len / 2] = u - v;
                }
        }
        for (int i = 0; i < n; ++i) a[i * stride] = tmp[i];
    } else {
        for (int m = 0; m < n; ++m) {
            double complex s = 0.0;
            for (int k = 0; k < n; ++k) {
                double ang = sign * 2.0 * ORC_PI * (double)((long)m * k % n) / n;
                s += tmp[k] * (cos(ang) + I * sin(ang));
            }
            a[m * stride] = s;
        }
    }
}

static void fft3d(double complex *a, int K1, int K2, int K3, int sign) {
    int kmax = K1 > K2 ? (K1 > K3 ? K1 : K3) : (K2 > K3 ? K2 : K3);
#pragma omp parallel
    {
        double complex *tmp = (double complex *)malloc(sizeof(double complex) * kmax);
#pragma omp for collapse(2)
        for (int k = 0; k < K3; ++k)
            for (int j = 0; j < K2; ++j) dft_line(a + (long)K1 * (j + (long)K2 * k), K1, 1, sign, tmp);
#pragma omp for collapse(2)
        for (int k = 0; k < K3; ++k)
            for (int i = 0; i < K1; ++i) dft_line(a + i + (long)K1 * K2 * k, K2, K1, sign, tmp);
#pragma omp for collapse(2)
        for (int j = 0; j < K2; ++j)
            for (int i = 0; i < K1; ++i) dft_line(a + i + (long)K1 * j, K3, (long)K1 * K2, sign, tmp);
        free(tmp);
    }
}

int orc_force_spme(const orc_params *p, int nel, int nion, const double *x,
                   const double *psi, double *frec, double *Um) {
    const int n = nel + nion, P = p->order;
    const int K1 = p->K[0], K2 = p->K[1], K3 = p->K[2];
    const long KK = (long)K1 * K2 * K3;
    const double V = p->box[0] * p->box[1] * p->box[2];                 /* :692 */
    const double s = p->charge_scale;
    double *Q = (double *)calloc(KK, sizeof(double));
    double complex *A = (double complex *)malloc(sizeof(double complex) * KK);
    double *bx = (double *)malloc(sizeof(double) * K1), *by = (double *)malloc(sizeof(double) * K2),
           *bz = (double *)malloc(sizeof(double) * K3);
    double W[3][8], dW[3][8];
    /* charge spreading, force.f90:697-820 (serial: the mesh sum order is the
     * reference's particle order) */
    for (int m = 0; m < n; ++m) {
        double q1 = s * p->q[m < nel ? 0 : 1];                           /* :696, :759 */
        int base[3];
        for (int d = 0; d < 3; ++d) {
            double u = (double)p->K[d] * (x[3 * m + d] + p->box[d] * .5) / p->box[d]; /* :700-702 */
            spline_weights(P, u, W[d], dW[d]);
            base[d] = (int)trunc(u) - (P - 3);                           /* INT(u)+i-2 */
        }
        for (int k = 0; k < P; ++k) {
            int iz = ((base[2] + k) % K3 + K3) % K3;                     /* :744 */
            for (int j = 0; j < P; ++j) {
                int iy = ((base[1] + j) % K2 + K2) % K2;                 /* :743 */
                for (int i = 0; i < P; ++i) {
                    int ix = ((base[0] + i) % K1 + K1) % K1;             /* :742 */
                    Q[ix + (long)K1 * (iy + (long)K2 * iz)] += q1 * W[0][i] * W[1][j] * W[2][k]; /* :745 */
                }
            }
        }
    }
    /* FFT -> influence multiply -> FFT (force.f90:823-851).  The reference
     * takes Qinv = ZFFT3D(+1)(Q) normalised by 1/K^3 and undoes it with the
     * K^3 factors of :864-865; here both transforms are unnormalised, so
     * phi = K^3 Qfin and the 1/K^3 and K^3 cancel identically. */
    for (long i = 0; i < KK; ++i) A[i] = Q[i];
    fft3d(A, K1, K2, K3, -1);
    orc_bspline_moduli(P, K1, bx);
    orc_bspline_moduli(P, K2, by);
    orc_bspline_moduli(P, K3, bz);
    for (int k = 0; k < K3; ++k)
        for (int j = 0; j < K2; ++j)
            for (int i = 0; i < K1; ++i) {
                long idx = i + (long)K1 * (j + (long)K2 * k);
                A[idx] *= psi[idx] * bx[i] * by[j] * bz[k];              /* :839 */
            }
    fft3d(A, K1, K2, K3, +1);
    double epme = 0.0;                                                   /* :854-861 */
    for (long i = 0; i < KK; ++i) epme += Q[i] * creal(A[i]);
    *Um = ORC_EPS * epme / V / ORC_PI / 2.0;                             /* :921 */
    /* force gather, force.f90:868-919: F = -eps K^3 sum dQdx Qfin/(V pi) */
    const double q1f = ORC_EPS;                                          /* :865 with phi = K^3 Qfin */
#pragma omp parallel for private(W, dW) schedule(static)
    for (int m = 0; m < n; ++m) {
        double q1 = s * p->q[m < nel ? 0 : 1];
        int base[3];
        for (int d = 0; d < 3; ++d) {
            double u = (double)p->K[d] * (x[3 * m + d] + p->box[d] * .5) / p->box[d];
            spline_weights(P, u, W[d], dW[d]);
            base[d] = (int)trunc(u) - (P - 3);
        }
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int k = 0; k < P; ++k) {
            int iz = ((base[2] + k) % K3 + K3) % K3;
            for (int j = 0; j < P; ++j) {
                int iy = ((base[1] + j) % K2 + K2) % K2;
                for (int i = 0; i < P; ++i) {
                    int ix = ((base[0] + i) % K1 + K1) % K1;
                    double phi = creal(A[ix + (long)K1 * (iy + (long)K2 * iz)]);
                    /* dQdx(i,j,k,m,d), force.f90:746-751 */
                    double d1 = q1 * dW[0][i] * W[1][j] * W[2][k] * (double)K1 / p->box[0];
                    double d2 = q1 * W[0][i] * dW[1][j] * W[2][k] * (double)K2 / p->box[1];
                    double d3 = q1 * W[0][i] * W[1][j] * dW[2][k] * (double)K3 / p->box[2];
                    fx -= q1f * d1 * phi / V / ORC_PI;                   /* :882-887 */
                    fy -= q1f * d2 * phi / V / ORC_PI;
                    fz -= q1f * d3 * phi / V / ORC_PI;
                }
            }
        }
        frec[3 * m + 0] = fx;
        frec[3 * m + 1] = fy;
        frec[3 * m + 2] = fz;
    }
    free(Q); free(A); free(bx); free(by); free(bz);
    return 0;
}

void orc_ewald_ksum(const orc_params *p, int nel, int nion, const double *x, int nmax2,
                    double *frec, double *Uk, int nthreads) {
    const int n = nel + nion;
    const int nt = nthreads_or_max(nthreads);
    const double V = p->box[0] * p->box[1] * p->box[2];
    const double s = p->charge_scale;
    int nm = (int)floor(sqrt((double)nmax2));
    memset(frec, 0, sizeof(double) * 3 * (size_t)n);
    double e = 0.0;
    double *fb = (double *)calloc((size_t)nt * 3 * n, sizeof(double));
#pragma omp parallel num_threads(nt) reduction(+ : e)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *fl = fb + (size_t)tid * 3 * n;
        int side = 2 * nm + 1;
#pragma omp for schedule(dynamic, 1)
        for (int t = 0; t < side * side * side; ++t) {
            int n1 = t % side - nm, n2 = (t / side) % side - nm, n3 = t / (side * side) - nm;
            int nn = n1 * n1 + n2 * n2 + n3 * n3;
            if (nn == 0 || nn > nmax2) continue;
            double m[3] = {n1 / p->box[0], n2 / p->box[1], n3 / p->box[2]};
            double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
            double th = exp(-m2 * ORC_PI * ORC_PI / (p->a * p->a)) / m2;
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < n; ++j) {
                double q = s * p->q[j < nel ? 0 : 1];
                double ph = 2.0 * ORC_PI * (m[0] * x[3 * j] + m[1] * x[3 * j + 1] + m[2] * x[3 * j + 2]);
                sr += q * cos(ph);
                si += q * sin(ph);
            }
            e += th * (sr * sr + si * si);
            for (int j = 0; j < n; ++j) {
                double q = s * p->q[j < nel ? 0 : 1];
                double ph = 2.0 * ORC_PI * (m[0] * x[3 * j] + m[1] * x[3 * j + 1] + m[2] * x[3 * j + 2]);
                /* Im(conj(S) e^{i ph}) = sr sin(ph) - si cos(ph) */
                double im = sr * sin(ph) - si * cos(ph);
                double c = 2.0 * ORC_EPS * q / V * th * im;
                fl[3 * j] += c * m[0];
                fl[3 * j + 1] += c * m[1];
                fl[3 * j + 2] += c * m[2];
            }
        }
    }
    for (int t = 0; t < nt; ++t)
        for (long i = 0; i < 3L * n; ++i) frec[i] += fb[(size_t)t * 3 * n + i];
    free(fb);
    *Uk = ORC_EPS * e / (2.0 * ORC_PI * V);
}

/* SPME_SUM, force.f90:953-964 */
void orc_spme_sum(int n, double *f, const double *frec) {
    for (long i = 0; i < 3L * n; ++i) f[i] += frec[i];
}

/* REMOVE_RIGIDMTN, force.f90:986-1004 */
void orc_remove_rigidmtn(int n, double *f) {
    double F[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) F[k] += f[3 * i + k];
    for (int k = 0; k < 3; ++k) F[k] /= (double)n;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) f[3 * i + k] -= F[k];
}

/* ------------------------------------------------------------------ */
/* Integrators, vverlet.f90                                            */
/* ------------------------------------------------------------------ */
void orc_vverlet1(const orc_params *p, int nel, int nion, double dt, double *x, double *v,
                  const double *f) {
    for (int i = 0; i < nel + nion; ++i) {
        double xm = p->xm[i < nel ? 0 : 1];                              /* :148, :159 */
        for (int k = 0; k < 3; ++k) {
            v[3 * i + k] = v[3 * i + k] + 0.5 * dt * f[3 * i + k] / xm;  /* :151 */
            double xx = x[3 * i + k] + dt * v[3 * i + k];                /* :152 */
            x[3 * i + k] = min_image(xx, p->box[k]);                     /* :153 */
        }
    }
}

void orc_vverlet_stoch1(const orc_params *p, int nel, int nion, double dt, double *x,
                        double *v, const double *f) {
    for (int i = 0; i < nel + nion; ++i) {
        double xm = p->xm[i < nel ? 0 : 1];
        for (int k = 0; k < 3; ++k) {
            v[3 * i + k] = v[3 * i + k] * (1.0 - 0.5 * p->alpha_lgv * dt / xm) +
                           0.5 * dt * f[3 * i + k] / xm;                 /* :37-38 */
            double xx = x[3 * i + k] + dt * v[3 * i + k];
            x[3 * i + k] = min_image(xx, p->box[k]);
        }
    }
}

static inline void vdf_add(double *vdf, double mv2, double dv) {
    /* id = INT(mv2/3/dv)+1; IF (id <= Ndist+1) VDF(id) += 1, vverlet.f90:201-204 */
    double t = mv2 / 3.0 / dv;
    if (t < (double)(ORC_NDIST + 1)) {
        int b = (int)t;
        if (b <= ORC_NDIST) vdf[b] += 1.0;
    }
}

void orc_vverlet2(const orc_params *p, int thermo, int apply_thermostat, int nel, int nion,
                  double dt, double *v, double *f, const double *eta, double *mv2el,
                  double *mv2ion, double *vdf) {
    const int counts[2] = {nel, nion};
    const int start[2] = {0, nel};
    const double T[2] = {p->Te, p->Ti};
    const double dv[2] = {p->dv_e, p->dv_i};
    double out[2];
    for (int s = 0; s < 2; ++s) {
        const double xm = p->xm[s];
        double *vd = vdf ? vdf + s * (ORC_NDIST + 1) : NULL;
        double acc = 0.0;
        if (thermo == ORC_STOCH) {
            double beta = sqrt(2.0 * p->alpha_lgv * T[s] / dt);          /* :92, :110 */
            for (int i = start[s]; i < start[s] + counts[s]; ++i) {
                for (int k = 0; k < 3; ++k) {
                    f[3 * i + k] = f[3 * i + k] + eta[3 * i + k] * beta; /* :95 */
                    v[3 * i + k] = (v[3 * i + k] + 0.5 * dt * f[3 * i + k] / xm) /
                                   (1.0 + 0.5 * p->alpha_lgv * dt / xm); /* :96-97 */
                }
                double mv2 = (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) * xm;
                acc += mv2;
                if (vd) vdf_add(vd, mv2, dv[s]);
            }
            out[s] = acc;
            continue;
        }
        if ((thermo == ORC_ISOKIN || thermo == ORC_BEREND) && apply_thermostat) {
            /* kick + mv2 (:250-255), lambda (:257-258 / :331-332), rescale (:260-270) */
            for (int i = start[s]; i < start[s] + counts[s]; ++i)
                for (int k = 0; k < 3; ++k) {
                    v[3 * i + k] = v[3 * i + k] + 0.5 * dt * f[3 * i + k] / xm;
                    acc += xm * v[3 * i + k] * v[3 * i + k];
                }
            double T0 = acc / (double)(3 * counts[s]);
            double lambda = thermo == ORC_ISOKIN ? sqrt(T[s] / T0)
                                                 : sqrt(1.0 + dt * (T[s] / T0 - 1.0) / p->tau);
            acc = 0.0;
            for (int i = start[s]; i < start[s] + counts[s]; ++i) {
                for (int k = 0; k < 3; ++k) v[3 * i + k] = v[3 * i + k] * lambda;
                double mv2 = (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) * xm;
                acc += mv2;
                if (vd) vdf_add(vd, mv2, dv[s]);
            }
            out[s] = acc;
            continue;
        }
        /* NOTEMP, vverlet.f90:194-219 */
        for (int i = start[s]; i < start[s] + counts[s]; ++i) {
            for (int k = 0; k < 3; ++k) v[3 * i + k] = v[3 * i + k] + 0.5 * dt * f[3 * i + k] / xm;
            double mv2 = (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) * xm;
            acc += mv2;
            if (vd) vdf_add(vd, mv2, dv[s]);
        }
        out[s] = acc;
    }
    *mv2el = out[0];
    *mv2ion = out[1];
}

/* ------------------------------------------------------------------ */
/* Composition: main.f90:100-141, init.f90:152-239                    */
/* ------------------------------------------------------------------ */
int orc_force_total(const orc_params *p, int nel, int nion, const double *x, const double *psi,
                    int reciprocal, int nmax2, double *f, double *Ur, double *Um, double *rdf,
                    int nthreads) {
    const int n = nel + nion;
    double *frec = (double *)calloc(3 * (size_t)n, sizeof(double));
    double um = 0.0;
    if (reciprocal == 1) orc_force_spme(p, nel, nion, x, psi, frec, &um);       /* main.f90:100 */
    else if (reciprocal == 2) orc_ewald_ksum(p, nel, nion, x, nmax2, frec, &um, nthreads);
    orc_force_direct(p, nel, nion, x, f, Ur, rdf, nthreads);                    /* main.f90:106-130 */
    orc_spme_sum(n, f, frec);                                                   /* main.f90:136 */
    orc_remove_rigidmtn(n, f);                                                  /* main.f90:141 */
    *Um = um;
    free(frec);
    return 0;
}

int orc_finit(const orc_params *p, int nel, int nion, double dt, double *x, const double *v,
              const double *psi, double *f, double *Ur, double *Um, int nthreads) {
    const int n = nel + nion;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) x[3 * i + k] = min_image(x[3 * i + k] - dt * v[3 * i + k], p->box[k]); /* init.f90:171-185 */
    orc_force_total(p, nel, nion, x, psi, 1, 0, f, Ur, Um, NULL, nthreads);    /* init.f90:193-220 */
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) x[3 * i + k] = min_image(x[3 * i + k] + dt * v[3 * i + k], p->box[k]); /* init.f90:223-237 */
    return 0;
}

int orc_md_step(const orc_params *p, int thermo, int apply_thermostat, int nel, int nion,
                double dt, double *x, double *v, double *f, const double *psi, double Uo,
                int reciprocal, int nmax2, double *energies, double *rdf, double *vdf, int nthreads) {
    double Ur, Um, mv2el, mv2ion;
    orc_vverlet1(p, nel, nion, dt, x, v, f);                                    /* main.f90:91 */
    orc_force_total(p, nel, nion, x, psi, reciprocal, nmax2, f, &Ur, &Um, rdf, nthreads); /* main.f90:100-141 */
    orc_vverlet2(p, thermo, apply_thermostat, nel, nion, dt, v, f, NULL, &mv2el, &mv2ion, vdf); /* main.f90:145-153 */
    energies[0] = Ur;
    energies[1] = Um;
    energies[2] = (Ur + Uo) * ORC_EPS;                                          /* main.f90:138 */
    energies[3] = mv2el;
    energies[4] = mv2ion;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Derivatives of the path (adjoint).  The reference computes none: these
 * are the analytic derivatives of the energy and of the discrete MD map
 * restated above, pinned by central finite differences of those routines. */
/* ------------------------------------------------------------------ */

/* Radial functions of one pair term phi(r) (without eps and q_i q_j):
 *   G1 = -phi'(r)/r          (force on i = eps qq G1 u, u = x_i - x_j)
 *   G2 = -G1'(r)/r           (pair Hessian = eps qq (-G1 I + G2 u u^T))
 *   dl = d phi / d lambda    (lambda = lambda_ei for Kelbg, rs for Deutsch)
 *   gl = d G1 / d lambda
 * kind 0: erfc(ar)/r; 1: Deutsch e-i (force.f90:135-139); 2: Kelbg e-i. */
static void pair_radial(const orc_params *p, int kind, double r2, double r, double *G1, double *G2,
                        double *dl, double *gl) {
    const double a = p->a, c = 2.0 * a / ORC_SQRTPI;
    const double e = exp(-a * a * r2);
    const double w0 = (erfc(a * r) / r + c * e) / r2;
    double g1 = w0, g2 = (3.0 * w0 + 2.0 * a * a * c * e) / r2, d = 0.0, gg = 0.0;
    if (kind == 1) {
        const double rs = p->rs, y = exp(-r / rs);
        g1 -= y * (1.0 / (rs * r2) + 1.0 / (r2 * r));
        g2 -= y * (3.0 / (rs * r2) + 3.0 / (r2 * r) + 1.0 / (rs * rs * r)) / r2;
        d = -y / (rs * rs);
        gg = -y / (rs * rs * rs * r);
    } else if (kind == 2) {
        const double l = p->lambda_ei, g = exp(-r2 / (l * l));
        g1 -= g / (r2 * r);
        g2 -= g * (3.0 / (r2 * r) + 2.0 / (l * l * r)) / r2;
        d = -ORC_SQRTPI * erfc(r / l) / (l * l);
        gg = -2.0 * g / (l * l * l * r);
    }
    *G1 = g1;
    *G2 = g2;
    *dl = d;
    *gl = gg;
}

static int pair_kind(const orc_params *p, int si, int sj) {
    if (si == sj) return 0;
    if (p->ei_model == ORC_EI_DEUTSCH) return 1;
    if (p->ei_model == ORC_EI_KELBG) return 2;
    return 0;
}

/* Real-space part: hw += H_real w, *dEdl = dE/dlambda (eV/A), *dFdl_w =
 * sum_i dF_i/dlambda . w_i (F unprojected).  w or hw may be NULL. */
static void real_adjoint(const orc_params *p, int nel, int nion, const double *x, const double *w, double *hw,
                         double *dEdl, double *dFdl_w, int nthreads) {
    const int n = nel + nion;
    const int nt = nthreads_or_max(nthreads);
    const double s = p->charge_scale;
    const double qs[2] = {s * p->q[0], s * p->q[1]};
    double *hb = hw ? (double *)calloc((size_t)nt * 3 * n, sizeof(double)) : NULL;
    double el = 0.0, fl = 0.0;
#pragma omp parallel num_threads(nt) reduction(+ : el, fl)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *hl = hb ? hb + (size_t)tid * 3 * n : NULL;
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < n - 1; ++i) {
            int si = i < nel ? 0 : 1;
            for (int j = i + 1; j < n; ++j) {
                int sj = j < nel ? 0 : 1;
                double u[3], r2 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    u[k] = min_image(x[3 * i + k] - x[3 * j + k], p->box[k]);
                    r2 += u[k] * u[k];
                }
                if (r2 >= p->rc2) continue;
                const double r = sqrt(r2), qq = ORC_EPS * qs[si] * qs[sj];
                double G1, G2, dl, gl;
                pair_radial(p, pair_kind(p, si, sj), r2, r, &G1, &G2, &dl, &gl);
                el += qq * dl;
                if (!w) continue;
                double dw[3], ud = 0.0;
                for (int k = 0; k < 3; ++k) {
                    dw[k] = w[3 * i + k] - w[3 * j + k];
                    ud += u[k] * dw[k];
                }
                fl += qq * gl * ud;
                if (hl)
                    for (int k = 0; k < 3; ++k) {
                        const double t = qq * (-G1 * dw[k] + G2 * ud * u[k]);
                        hl[3 * i + k] += t;
                        hl[3 * j + k] -= t;
                    }
            }
        }
    }
    if (hw)
        for (int t = 0; t < nt; ++t)
            for (long i = 0; i < 3L * n; ++i) hw[i] += hb[(size_t)t * 3 * n + i];
    free(hb);
    if (dEdl) *dEdl = el;
    if (dFdl_w) *dFdl_w = fl;
}

/* SPME part: hw += H_rec w.  With Q(m) = sum_j q_j W_j(m), phi = A Q and
 * E = c/2 Q.phi (c = eps/(pi V)):
 *   grad_i E = c q_i sum_m grad W_i(m) phi(m)
 *   (H w)_i  = c q_i [sum_m (hess W_i(m) w_i) phi(m) + sum_m grad W_i(m) dphi(m)],
 *   dphi = A dQ,  dQ(m) = sum_j q_j grad W_j(m) . w_j. */
static void spme_hvp(const orc_params *p, int nel, int nion, const double *x, const double *psi, const double *w,
                     double *hw) {
    const int n = nel + nion, P = p->order;
    const int K1 = p->K[0], K2 = p->K[1], K3 = p->K[2];
    const int K[3] = {K1, K2, K3};
    const long KK = (long)K1 * K2 * K3;
    const double V = p->box[0] * p->box[1] * p->box[2];
    const double s = p->charge_scale;
    double complex *A = (double complex *)calloc(KK, sizeof(double complex));
    double complex *B = (double complex *)calloc(KK, sizeof(double complex));
    double *bm[3];
    for (int d = 0; d < 3; ++d) {
        bm[d] = (double *)malloc(sizeof(double) * K[d]);
        orc_bspline_moduli(P, K[d], bm[d]);
    }
    double W[3][8], dW[3][8], d2W[3][8];
    int base[3];
    /* weights, first and second derivatives w.r.t. x (chain factor K/L) */
#define ORC_WEIGHTS(m)                                                                          \
    for (int d = 0; d < 3; ++d) {                                                               \
        double u = (double)K[d] * (x[3 * (m) + d] + p->box[d] * .5) / p->box[d];                \
        spline_weights(P, u, W[d], dW[d]);                                                      \
        double fr = u - trunc(u), kl = (double)K[d] / p->box[d];                                \
        for (int j = 0; j < P; ++j) {                                                           \
            double y = fr + (double)(P - 1 - j);                                                \
            d2W[d][j] = (bspline_M(P - 2, y) - 2.0 * bspline_M(P - 2, y - 1.0) +                 \
                         bspline_M(P - 2, y - 2.0)) * kl * kl;                                   \
            dW[d][j] *= kl;                                                                     \
        }                                                                                       \
        base[d] = (int)trunc(u) - (P - 3);                                                      \
    }
    for (int m = 0; m < n; ++m) {
        const double q = s * p->q[m < nel ? 0 : 1];
        ORC_WEIGHTS(m)
        for (int k = 0; k < P; ++k) {
            int iz = ((base[2] + k) % K3 + K3) % K3;
            for (int j = 0; j < P; ++j) {
                int iy = ((base[1] + j) % K2 + K2) % K2;
                for (int i = 0; i < P; ++i) {
                    int ix = ((base[0] + i) % K1 + K1) % K1;
                    long idx = ix + (long)K1 * (iy + (long)K2 * iz);
                    A[idx] += q * W[0][i] * W[1][j] * W[2][k];
                    B[idx] += q * (dW[0][i] * W[1][j] * W[2][k] * w[3 * m] + W[0][i] * dW[1][j] * W[2][k] * w[3 * m + 1] +
                                   W[0][i] * W[1][j] * dW[2][k] * w[3 * m + 2]);
                }
            }
        }
    }
    fft3d(A, K1, K2, K3, -1);
    fft3d(B, K1, K2, K3, -1);
    for (int k = 0; k < K3; ++k)
        for (int j = 0; j < K2; ++j)
            for (int i = 0; i < K1; ++i) {
                long idx = i + (long)K1 * (j + (long)K2 * k);
                double g = psi[idx] * bm[0][i] * bm[1][j] * bm[2][k];
                A[idx] *= g;
                B[idx] *= g;
            }
    fft3d(A, K1, K2, K3, +1);
    fft3d(B, K1, K2, K3, +1);
    const double c = ORC_EPS / (ORC_PI * V);
    for (int m = 0; m < n; ++m) {
        const double q = s * p->q[m < nel ? 0 : 1];
        ORC_WEIGHTS(m)
        double h[3] = {0.0, 0.0, 0.0};
        const double *wm = w + 3 * m;
        for (int k = 0; k < P; ++k) {
            int iz = ((base[2] + k) % K3 + K3) % K3;
            for (int j = 0; j < P; ++j) {
                int iy = ((base[1] + j) % K2 + K2) % K2;
                for (int i = 0; i < P; ++i) {
                    int ix = ((base[0] + i) % K1 + K1) % K1;
                    long idx = ix + (long)K1 * (iy + (long)K2 * iz);
                    const double ph = creal(A[idx]), dph = creal(B[idx]);
                    const double gx = dW[0][i] * W[1][j] * W[2][k], gy = W[0][i] * dW[1][j] * W[2][k],
                                 gz = W[0][i] * W[1][j] * dW[2][k];
                    const double hxx = d2W[0][i] * W[1][j] * W[2][k], hyy = W[0][i] * d2W[1][j] * W[2][k],
                                 hzz = W[0][i] * W[1][j] * d2W[2][k];
                    const double hxy = dW[0][i] * dW[1][j] * W[2][k], hxz = dW[0][i] * W[1][j] * dW[2][k],
                                 hyz = W[0][i] * dW[1][j] * dW[2][k];
                    h[0] += (hxx * wm[0] + hxy * wm[1] + hxz * wm[2]) * ph + gx * dph;
                    h[1] += (hxy * wm[0] + hyy * wm[1] + hyz * wm[2]) * ph + gy * dph;
                    h[2] += (hxz * wm[0] + hyz * wm[1] + hzz * wm[2]) * ph + gz * dph;
                }
            }
        }
        for (int d = 0; d < 3; ++d) hw[3 * m + d] += c * q * h[d];
    }
#undef ORC_WEIGHTS
    for (int d = 0; d < 3; ++d) free(bm[d]);
    free(A);
    free(B);
}

/* Plain Ewald part: hw += H_k w.  E = C sum_m theta |S|^2, C = eps/(2 pi V),
 * S = sum_j q_j e^{i ph_j}, ph_j = 2 pi m.x_j, dS = sum_j q_j (2 pi i m.w_j) e^{i ph_j}:
 *   (H w)_i = -(2 eps/V) q_i sum_m theta m [Im(conj(dS) e^{i ph_i}) + 2 pi (m.w_i) Re(conj(S) e^{i ph_i})] */
static void ewald_hvp(const orc_params *p, int nel, int nion, const double *x, int nmax2, const double *w,
                      double *hw) {
    const int n = nel + nion;
    const double V = p->box[0] * p->box[1] * p->box[2];
    const double s = p->charge_scale;
    const int nm = (int)floor(sqrt((double)nmax2)), side = 2 * nm + 1;
    for (int t = 0; t < side * side * side; ++t) {
        int n1 = t % side - nm, n2 = (t / side) % side - nm, n3 = t / (side * side) - nm;
        int nn = n1 * n1 + n2 * n2 + n3 * n3;
        if (nn == 0 || nn > nmax2) continue;
        double m[3] = {n1 / p->box[0], n2 / p->box[1], n3 / p->box[2]};
        double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
        double th = exp(-m2 * ORC_PI * ORC_PI / (p->a * p->a)) / m2;
        double sr = 0.0, si = 0.0, dr = 0.0, di = 0.0;
        for (int j = 0; j < n; ++j) {
            double q = s * p->q[j < nel ? 0 : 1];
            double ph = 2.0 * ORC_PI * (m[0] * x[3 * j] + m[1] * x[3 * j + 1] + m[2] * x[3 * j + 2]);
            double mw = 2.0 * ORC_PI * (m[0] * w[3 * j] + m[1] * w[3 * j + 1] + m[2] * w[3 * j + 2]);
            sr += q * cos(ph);
            si += q * sin(ph);
            dr += -q * mw * sin(ph);   /* i mw e^{i ph} = mw (-sin + i cos) */
            di += q * mw * cos(ph);
        }
        for (int i = 0; i < n; ++i) {
            double q = s * p->q[i < nel ? 0 : 1];
            double ph = 2.0 * ORC_PI * (m[0] * x[3 * i] + m[1] * x[3 * i + 1] + m[2] * x[3 * i + 2]);
            double mw = 2.0 * ORC_PI * (m[0] * w[3 * i] + m[1] * w[3 * i + 1] + m[2] * w[3 * i + 2]);
            double cs = cos(ph), sn = sin(ph);
            double im_d = dr * sn - di * cs;   /* Im(conj(dS) e^{i ph}) */
            double re_s = sr * cs + si * sn;   /* Re(conj(S) e^{i ph}) */
            double coef = -2.0 * ORC_EPS / V * q * th * (im_d + mw * re_s);
            for (int k = 0; k < 3; ++k) hw[3 * i + k] += coef * m[k];
        }
    }
}

void orc_adjoint_energy(const orc_params *p, int nel, int nion, const double *x, double *dEdl, int nthreads) {
    real_adjoint(p, nel, nion, x, NULL, NULL, dEdl, NULL, nthreads);
}

void orc_hvp(const orc_params *p, int nel, int nion, const double *x, const double *psi, int reciprocal, int nmax2,
             const double *w, double *hw, double *dFdl_w, int nthreads) {
    const int n = nel + nion;
    memset(hw, 0, sizeof(double) * 3 * (size_t)n);
    real_adjoint(p, nel, nion, x, w, hw, NULL, dFdl_w, nthreads);
    if (reciprocal == 1) spme_hvp(p, nel, nion, x, psi, w, hw);
    else if (reciprocal == 2) ewald_hvp(p, nel, nion, x, nmax2, w, hw);
}

static void project_mean(int n, double *g) {
    orc_remove_rigidmtn(n, g);   /* the same projection as the force (force.f90:986-1004) */
}

/* J = (1/K) sum_{k=1..K} (mv2el_k + mv2ion_k)/(3N) over K NOTEMP steps of
 * orc_md_step from (x0, v0) with f_0 = F(x_0), and dJ/dlambda by the discrete
 * adjoint of that map.  Checkpoints (x_k, v_k) every M steps; each segment is
 * recomputed forward and swept in reverse:
 *   vb += 2 m v_k/(3NK);  g = fb + a vb;  xb -= H(x_k) P g;  lb += dF/dl(x_k) . P g
 *   vb += dt xb;  fb = a vb                     (a = dt/(2m), P = mean removal)
 * and finally lb += dF/dl(x_0) . P fb. */
int orc_reverse_md(const orc_params *p, int nel, int nion, const double *x0, const double *v0, const double *psi,
                   int reciprocal, int nmax2, double dt, int K, int M, double *J, double *dJdl, int nthreads) {
    const int n = nel + nion;
    const size_t sz = 3 * (size_t)n;
    if (K <= 0 || M <= 0) return -1;
    const int nck = (K + M - 1) / M;
    double *ck = (double *)malloc(sizeof(double) * 2 * sz * nck);
    double *seg = (double *)malloc(sizeof(double) * 2 * sz * (M + 1));
    double *x = (double *)malloc(sizeof(double) * sz), *v = (double *)malloc(sizeof(double) * sz),
           *f = (double *)malloc(sizeof(double) * sz);
    double *xb = (double *)calloc(sz, sizeof(double)), *vb = (double *)calloc(sz, sizeof(double)),
           *fb = (double *)calloc(sz, sizeof(double)), *g = (double *)malloc(sizeof(double) * sz),
           *hw = (double *)malloc(sizeof(double) * sz);
    double ur, um, e[5], jsum = 0.0, lb = 0.0, d;
    memcpy(x, x0, sizeof(double) * sz);
    memcpy(v, v0, sizeof(double) * sz);
    orc_force_total(p, nel, nion, x, psi, reciprocal, nmax2, f, &ur, &um, NULL, nthreads);
    for (int k = 0; k < K; ++k) {
        if (k % M == 0) {
            memcpy(ck + 2 * sz * (k / M), x, sizeof(double) * sz);
            memcpy(ck + 2 * sz * (k / M) + sz, v, sizeof(double) * sz);
        }
        orc_md_step(p, ORC_NOTEMP, 0, nel, nion, dt, x, v, f, psi, 0.0, reciprocal, nmax2, e, NULL, NULL, nthreads);
        jsum += e[3] + e[4];
    }
    *J = jsum / (3.0 * n * K);
    for (int s = nck - 1; s >= 0; --s) {
        const int k0 = s * M, k1 = (k0 + M < K) ? k0 + M : K;
        memcpy(x, ck + 2 * sz * s, sizeof(double) * sz);
        memcpy(v, ck + 2 * sz * s + sz, sizeof(double) * sz);
        orc_force_total(p, nel, nion, x, psi, reciprocal, nmax2, f, &ur, &um, NULL, nthreads);
        for (int k = k0 + 1; k <= k1; ++k) {
            orc_md_step(p, ORC_NOTEMP, 0, nel, nion, dt, x, v, f, psi, 0.0, reciprocal, nmax2, e, NULL, NULL, nthreads);
            memcpy(seg + 2 * sz * (k - k0), x, sizeof(double) * sz);
            memcpy(seg + 2 * sz * (k - k0) + sz, v, sizeof(double) * sz);
        }
        for (int k = k1; k > k0; --k) {
            const double *xk = seg + 2 * sz * (k - k0), *vk = xk + sz;
            for (int i = 0; i < n; ++i) {
                const double m = p->xm[i < nel ? 0 : 1], a = 0.5 * dt / m, cj = 2.0 * m / (3.0 * n * K);
                for (int c = 0; c < 3; ++c) {
                    vb[3 * i + c] += cj * vk[3 * i + c];
                    g[3 * i + c] = fb[3 * i + c] + a * vb[3 * i + c];
                }
            }
            project_mean(n, g);
            orc_hvp(p, nel, nion, xk, psi, reciprocal, nmax2, g, hw, &d, nthreads);
            lb += d;
            for (int i = 0; i < n; ++i) {
                const double a = 0.5 * dt / p->xm[i < nel ? 0 : 1];
                for (int c = 0; c < 3; ++c) {
                    xb[3 * i + c] -= hw[3 * i + c];
                    vb[3 * i + c] += dt * xb[3 * i + c];
                    fb[3 * i + c] = a * vb[3 * i + c];
                }
            }
        }
    }
    memcpy(g, fb, sizeof(double) * sz);
    project_mean(n, g);
    real_adjoint(p, nel, nion, x0, g, NULL, NULL, &d, nthreads);
    lb += d;
    *dJdl = lb;
    free(ck); free(seg); free(x); free(v); free(f); free(xb); free(vb); free(fb); free(g); free(hw);
    return 0;
}

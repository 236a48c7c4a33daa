/*
 * FP64 CPU oracle: exact spherical-harmonic synthesis / adjoint synthesis at
 * arbitrary points -- TEST INFRASTRUCTURE ONLY (never linked into the product).
 *
 * C restatement of oracle/oracle.py:synth_points / adjoint_synth_points, i.e.
 * of the semantics of ducc0.sht.synthesis_general / adjoint_synthesis_general
 * as called by the reference (cunusht/deflection/CPU_nufft_transformer.py:
 * 645-652) and of the GPU nusht2d2 / nusht2d1 pair
 * (cunusht/deflection/GPU_nufft_transformer.py:386-484), evaluated by direct
 * summation (no nuFFT, no approximation).
 *
 * Conventions: orthonormal Condon-Shortley harmonics; spin s>0 uses
 * s_a_lm = -(G_lm + i C_lm), Q + iU = sum_lm s_a_lm sY_lm (HEALPix / ducc0).
 * alm arrays are complex128 interleaved (re, im), healpy m-major layout.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define FOURPI 12.566370614359172953850573533118

static long nalm_of(int lmax) { return ((long)(lmax + 1) * (lmax + 2)) / 2; }
static long idx_of(int lmax, int l, int m) { return (long)m * (2 * lmax + 1 - m) / 2 + l; }

typedef struct {
    int lmax, spin;
    double *al, *ga, *be; /* per (l,m) in alm layout */
    double *lg0;          /* per m: log2 of the start normalisation */
} coeffs_t;

static void build_coeffs(coeffs_t *c, int lmax, int s) {
    long n = nalm_of(lmax);
    c->lmax = lmax;
    c->spin = s;
    c->al = (double *)calloc(n, sizeof(double));
    c->ga = (double *)calloc(n, sizeof(double));
    c->be = (double *)calloc(n, sizeof(double));
    c->lg0 = (double *)calloc(lmax + 1, sizeof(double));
    for (int m = 0; m <= lmax; ++m) {
        int l0 = m > s ? m : s;
        double v = log((2.0 * l0 + 1) / FOURPI) + lgamma(2.0 * l0 + 1) - lgamma(m + s + 1.0)
                   - lgamma(fabs((double)(m - s)) + 1.0);
        c->lg0[m] = 0.5 * v / log(2.0);
        for (int l = l0; l < lmax; ++l) {
            double lp = l + 1.0;
            double den = sqrt((lp * lp - (double)m * m) * (lp * lp - (double)s * s));
            long i = idx_of(lmax, l, m);
            c->al[i] = lp * sqrt((2.0 * l + 1) * (2.0 * l + 3)) / den;
            c->ga[i] = l > 0 ? c->al[i] * ((double)m * s / (l * lp)) : 0.0;
            c->be[i] = l > 0 ? (lp / l) * sqrt(((double)l * l - (double)m * m) * ((double)l * l - (double)s * s)) / den
                                   * sqrt((2.0 * l + 3) / (2.0 * l - 1))
                             : 0.0;
        }
    }
}

static void free_coeffs(coeffs_t *c) {
    free(c->al); free(c->ga); free(c->be); free(c->lg0);
}

/* sLambda_lm(theta) for l = l0..lmax written into lam[l] (zeros below l0). */
static void slambda_col(const coeffs_t *c, int m, double theta, double *lam) {
    int lmax = c->lmax, s = c->spin;
    int l0 = m > s ? m : s;
    for (int l = 0; l <= lmax; ++l) lam[l] = 0.0;
    if (l0 > lmax) return;
    double sh = sin(0.5 * theta), ch = cos(0.5 * theta), x = cos(theta);
    double lg = c->lg0[m];
    if (m + s > 0) {
        if (sh == 0.0) return;
        lg += (m + s) * log2(sh);
    }
    if (m != s) {
        if (ch == 0.0) return;
        lg += fabs((double)(m - s)) * log2(ch);
    }
    double e = floor(lg);
    double cur = exp2(lg - e) * ((m & 1) ? -1.0 : 1.0), prev = 0.0;
    double fac = ldexp(1.0, (int)fmax(e, -3000.0));
    lam[l0] = cur * fac;
    const double BIG = ldexp(1.0, 200), SMALL = ldexp(1.0, -200);
    for (int l = l0; l < lmax; ++l) {
        long i = idx_of(lmax, l, m);
        double nxt = (c->al[i] * x + c->ga[i]) * cur - c->be[i] * prev;
        prev = cur;
        cur = nxt;
        if (fabs(cur) > BIG) {
            cur *= SMALL;
            prev *= SMALL;
            e += 200.0;
            fac = ldexp(1.0, (int)fmax(e, -3000.0));
        }
        lam[l + 1] = cur * fac;
    }
}

/* out: spin 0 -> npts values; spin>0 -> 2*npts (Q block then U block). */
int oracle_synth(int lmax, int spin, const double *G, const double *C, long npts,
                 const double *theta, const double *phi, double *out, int nthreads) {
    coeffs_t cf;
    build_coeffs(&cf, lmax, spin);
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
    {
        double *lp = (double *)malloc(sizeof(double) * (lmax + 1));
        double *lm = (double *)malloc(sizeof(double) * (lmax + 1));
#pragma omp for schedule(dynamic, 16)
        for (long j = 0; j < npts; ++j) {
            double th = theta[j], ph = phi[j];
            double zr = 0.0, zi = 0.0;
            for (int m = 0; m <= lmax; ++m) {
                long b = idx_of(lmax, m, m);
                double cm = cos(m * ph), sm = sin(m * ph);
                slambda_col(&cf, m, th, lp);
                if (spin == 0) {
                    double hr = 0.0, hi = 0.0;
                    for (int l = m; l <= lmax; ++l) {
                        hr += G[2 * (b + l - m)] * lp[l];
                        hi += G[2 * (b + l - m) + 1] * lp[l];
                    }
                    double re = hr * cm - hi * sm;
                    zr += (m == 0) ? hr : 2.0 * re;
                } else {
                    double hr = 0.0, hi = 0.0;
                    for (int l = m; l <= lmax; ++l) {
                        double gr = G[2 * (b + l - m)], gi = G[2 * (b + l - m) + 1];
                        double cr = C ? C[2 * (b + l - m)] : 0.0, ci = C ? C[2 * (b + l - m) + 1] : 0.0;
                        /* A = G + iC */
                        hr -= (gr - ci) * lp[l];
                        hi -= (gi + cr) * lp[l];
                    }
                    zr += hr * cm - hi * sm;
                    zi += hr * sm + hi * cm;
                    if (m > 0) {
                        slambda_col(&cf, m, M_PI - th, lm);
                        double sgs = (spin & 1) ? -1.0 : 1.0;
                        double kr = 0.0, ki = 0.0;
                        for (int l = m; l <= lmax; ++l) {
                            double gr = G[2 * (b + l - m)], gi = G[2 * (b + l - m) + 1];
                            double cr = C ? C[2 * (b + l - m)] : 0.0, ci = C ? C[2 * (b + l - m) + 1] : 0.0;
                            /* B = conj(G) + i conj(C) = (gr + ci) + i(cr - gi) */
                            double par = ((l + m) & 1) ? -1.0 : 1.0;
                            kr += (gr + ci) * par * lm[l];
                            ki += (cr - gi) * par * lm[l];
                        }
                        kr *= -sgs;
                        ki *= -sgs;
                        /* times e^{-i m phi} */
                        zr += kr * cm + ki * sm;
                        zi += ki * cm - kr * sm;
                    }
                }
            }
            if (spin == 0) out[j] = zr;
            else { out[j] = zr; out[npts + j] = zi; }
        }
        free(lp);
        free(lm);
    }
    free_coeffs(&cf);
    return 0;
}

/* values: spin 0 -> npts; spin>0 -> 2*npts (Q block then U block).
 * G (and C when spin>0, may be NULL) receive the adjoint alm. */
int oracle_adjoint(int lmax, int spin, const double *values, long npts, const double *theta,
                   const double *phi, double *G, double *C, int nthreads) {
    coeffs_t cf;
    build_coeffs(&cf, lmax, spin);
    long n = nalm_of(lmax);
    memset(G, 0, sizeof(double) * 2 * n);
    if (C) memset(C, 0, sizeof(double) * 2 * n);
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
    {
        double *lp = (double *)malloc(sizeof(double) * (lmax + 1));
        double *lm = (double *)malloc(sizeof(double) * (lmax + 1));
        double *acc = (double *)malloc(sizeof(double) * 4 * (lmax + 1));
#pragma omp for schedule(dynamic, 1)
        for (int m = 0; m <= lmax; ++m) {
            long b = idx_of(lmax, m, m);
            memset(acc, 0, sizeof(double) * 4 * (lmax + 1));
            for (long j = 0; j < npts; ++j) {
                double ph = phi[j];
                double cm = cos(m * ph), sm = sin(m * ph);
                slambda_col(&cf, m, theta[j], lp);
                if (spin == 0) {
                    double v = values[j];
                    for (int l = m; l <= lmax; ++l) {
                        acc[4 * l] += lp[l] * v * cm;
                        acc[4 * l + 1] -= lp[l] * v * sm;
                    }
                } else {
                    double qr = values[j], qi = values[npts + j];
                    /* h'_m = z e^{-i m phi} */
                    double hr = qr * cm + qi * sm, hi = qi * cm - qr * sm;
                    /* conj(h'_{-m}) = conj(z e^{+i m phi}) */
                    double kr = qr * cm - qi * sm, ki = -(qi * cm + qr * sm);
                    if (m > 0) slambda_col(&cf, m, M_PI - theta[j], lm);
                    for (int l = m; l <= lmax; ++l) {
                        acc[4 * l] += lp[l] * hr;
                        acc[4 * l + 1] += lp[l] * hi;
                        if (m > 0) {
                            double par = ((l + m) & 1) ? -1.0 : 1.0;
                            acc[4 * l + 2] += par * lm[l] * kr;
                            acc[4 * l + 3] += par * lm[l] * ki;
                        }
                    }
                }
            }
            for (int l = m; l <= lmax; ++l) {
                long i = b + l - m;
                if (spin == 0) {
                    G[2 * i] = acc[4 * l];
                    G[2 * i + 1] = (m == 0) ? 0.0 : acc[4 * l + 1];
                } else if (m == 0) {
                    G[2 * i] = -acc[4 * l];
                    if (C) C[2 * i] = -acc[4 * l + 1];
                } else {
                    double sgs = (spin & 1) ? -1.0 : 1.0;
                    double pr = acc[4 * l], pi_ = acc[4 * l + 1];
                    double qr = sgs * acc[4 * l + 2], qi = sgs * acc[4 * l + 3];
                    G[2 * i] = -0.5 * (pr + qr);
                    G[2 * i + 1] = -0.5 * (pi_ + qi);
                    if (C) { /* (i/2)(p - q) */
                        C[2 * i] = -0.5 * (pi_ - qi);
                        C[2 * i + 1] = 0.5 * (pr - qr);
                    }
                }
            }
        }
        free(lp);
        free(lm);
        free(acc);
    }
    free_coeffs(&cf);
    return 0;
}

/*
 * FP64 CPU restatement of the reference's lensing algorithm -- TEST AND CPU
 * TIMING-BASELINE INFRASTRUCTURE ONLY (never linked into the product).
 *
 * The reference's CPU backend (cunusht/deflection/CPU_nufft_transformer.py,
 * ducc0 synthesis_general as called at :645-652, get_deflected_angles at
 * :118-131, the exp(i s gamma) rotation :154-160) and its GPU pipeline
 * (GPU_nufft_transformer.py: dlm2pointing :64-104, nusht2d2 :386-435 =
 * Legendre synthesis on CC rings :257-260, doubling :315-317, fft2 :274-278,
 * type-2 nuFFT :292-298) compute a lensed map as
 *   1. spin-1 synthesis of sqrt(l(l+1)) dlm_scaled on the GL rings (Legendre
 *      recursion per m, then per ring a transform over m),
 *   2. the pointing rotation per pixel (pointing.cu:210-213) and gamma,
 *   3. spin-s Legendre synthesis on Clenshaw-Curtis rings of the 2 pi theta
 *      torus, doubling, 2D FFT, kernel deconvolution, zero padding to the
 *      oversampled torus, inverse FFT,
 *   4. type-2 interpolation with the exponential-of-semicircle kernel at the
 *      deflected points, and the exp(i s gamma) rotation.
 * This file does the same in FP64 on the host cores (OpenMP over m, columns,
 * rows, rings and points): radix-2 FFTs, Bluestein's chirp-z transform for
 * the ring length, the normalised Wigner-d recursion with an exponent kept
 * apart, the ES kernel psi(z) = exp(beta (sqrt(1 - z^2) - 1)) with the same
 * width / shape rule as the product (w = ceil(log10(10/eps)) + 1,
 * beta = 2.30 w) and its Fourier transform by Gauss-Legendre quadrature.
 * It is the "reference CPU path" timed as the CPU baseline (ducc0 is not
 * available) and a full-map cross-check of the GPU path; the exact checker is
 * direct.c.
 *
 * Conventions as direct.c: orthonormal Condon-Shortley harmonics, spin s > 0
 * s_a_lm = -(G_lm + i C_lm), Q + iU = sum s_a_lm sY_lm; healpy m-major alm.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

typedef double complex cplx;

#define PI_L 3.14159265358979323846264338327950288L
#define TWOPI 6.283185307179586476925286766559
#define FOURPI 12.566370614359172953850573533118

static long nalm_of(int lmax) { return ((long)(lmax + 1) * (lmax + 2)) / 2; }
static long idx_of(int lmax, int l, int m) { return (long)m * (2 * lmax + 1 - m) / 2 + l; }
static int next_pow2(long n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

/* ------------------------------------------------------------------ FFT */
typedef struct {
    int n;
    cplx *tw; /* e^{-2 pi i k / n}, k < n/2 */
    int *rev;
} fft_t;

static void fft_init(fft_t *f, int n) {
    f->n = n;
    f->tw = (cplx *)malloc(sizeof(cplx) * (n / 2 > 0 ? n / 2 : 1));
    for (int k = 0; k < n / 2; ++k) {
        long double a = -2.0L * PI_L * (long double)k / (long double)n;
        f->tw[k] = (double)cosl(a) + I * (double)sinl(a);
    }
    f->rev = (int *)malloc(sizeof(int) * n);
    int lg = 0;
    while ((1 << lg) < n) ++lg;
    for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < lg; ++b)
            if (i & (1 << b)) r |= 1 << (lg - 1 - b);
        f->rev[i] = r;
    }
}

static void fft_free(fft_t *f) {
    free(f->tw);
    free(f->rev);
}

/* in place; dir = -1: X_k = sum x_n e^{-2 pi i nk/N}; dir = +1: unnormalised inverse */
static void fft_run(const fft_t *f, cplx *a, int dir) {
    const int n = f->n;
    for (int i = 0; i < n; ++i) {
        const int r = f->rev[i];
        if (i < r) {
            cplx t = a[i];
            a[i] = a[r];
            a[r] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < half; ++k) {
                cplx w = f->tw[k * step];
                if (dir > 0) w = conj(w);
                const cplx u = a[i + k], v = a[i + k + half] * w;
                a[i + k] = u + v;
                a[i + k + half] = u - v;
            }
        }
    }
}

/* ------------------------------------------------------------------ Legendre */
typedef struct {
    double *al, *ga, *be; /* per (l, m) in alm layout */
    double *lg0;          /* per m: log2 of the start normalisation */
} coef_t;

static void coef_build(coef_t *c, int lmax, int s) {
    const long n = nalm_of(lmax);
    c->al = (double *)calloc(n, sizeof(double));
    c->ga = (double *)calloc(n, sizeof(double));
    c->be = (double *)calloc(n, sizeof(double));
    c->lg0 = (double *)calloc(lmax + 1, sizeof(double));
    for (int m = 0; m <= lmax; ++m) {
        const int l0 = m > s ? m : s;
        const double v = log((2.0 * l0 + 1) / FOURPI) + lgamma(2.0 * l0 + 1) - lgamma(m + s + 1.0) -
                         lgamma(fabs((double)(m - s)) + 1.0);
        c->lg0[m] = 0.5 * v / log(2.0);
        for (int l = l0; l < lmax; ++l) {
            const double lp = l + 1.0, dm = m, ds = s, dl = l;
            const double den = sqrt((lp * lp - dm * dm) * (lp * lp - ds * ds));
            const long i = idx_of(lmax, l, m);
            c->al[i] = lp * sqrt((2.0 * dl + 1) * (2.0 * dl + 3)) / den;
            if (l > 0) {
                c->ga[i] = c->al[i] * (dm * ds / (dl * lp));
                c->be[i] = (lp / dl) * sqrt((dl * dl - dm * dm) * (dl * dl - ds * ds)) / den *
                           sqrt((2.0 * dl + 3) / (2.0 * dl - 1));
            }
        }
    }
}

static void coef_free(coef_t *c) {
    free(c->al);
    free(c->ga);
    free(c->be);
    free(c->lg0);
}

/* start value (-1)^m 2^lg0 sin^{m+s}(t/2) cos^{|m-s|}(t/2) as mantissa x 2^e, e <= 0 a multiple of 512 */
static void rec_start(double lg0, int m, int s, double sh, double ch, double *cur, double *prev, int *e) {
    double lg = lg0;
    int zero = 0;
    *prev = 0.0;
    if (m + s > 0) {
        if (sh <= 0.0) zero = 1;
        else lg += (double)(m + s) * log2(sh);
    }
    if (m != s) {
        if (ch <= 0.0) zero = 1;
        else lg += (double)abs(m - s) * log2(ch);
    }
    if (zero) {
        *cur = 0.0;
        *e = 0;
        return;
    }
    int k = 0;
    if (lg < -400.0) k = (int)ceil((-400.0 - lg) / 512.0);
    *e = -512 * k;
    *cur = exp2(lg + 512.0 * (double)k);
    if (m & 1) *cur = -*cur;
}

#define PB 64 /* ring pairs per inner block: independent recursions overlap */

typedef struct {
    int npairs;
    double *x, *sh, *ch;
    int *rn, *rs;
} pairs_t;

/* H[c * ld + ring], c = m (spin 0) or m + lmax (spin s, m in [-lmax, lmax]);
 * spin 0 uses one recursion per pair and the parity (-1)^{l+m}. */
static void leg_synth(int L, int spin, const coef_t *cf, const cplx *G, const cplx *C, const double *lfac,
                      const pairs_t *pr, cplx *H, long ld) {
#pragma omp parallel
    {
        cplx *A = (cplx *)malloc(sizeof(cplx) * (L + 1));
        cplx *B = (cplx *)malloc(sizeof(cplx) * (L + 1));
        double cN[PB], pN[PB], cS[PB], pS[PB];
        int eN[PB], eS[PB];
        cplx a1[PB], a2[PB], a3[PB], a4[PB];
#pragma omp for schedule(dynamic, 1)
        for (int m = 0; m <= L; ++m) {
            const int l0 = m > spin ? m : spin;
            const long b = idx_of(L, m, m) - m;
            for (int l = l0; l <= L; ++l) {
                const double f = lfac ? lfac[l] : 1.0;
                const cplx g = G[b + l], c = C ? C[b + l] : 0.0;
                if (spin == 0) {
                    A[l] = f * g;
                } else {
                    A[l] = f * (g + I * c);                                      /* G + iC */
                    const double par = ((l + m) & 1) ? -f : f;
                    B[l] = par * (conj(g) + I * conj(c));                        /* (conj G + i conj C)(-1)^{l+m} */
                }
            }
            for (int p0 = 0; p0 < pr->npairs; p0 += PB) {
                const int nb = pr->npairs - p0 < PB ? pr->npairs - p0 : PB;
                for (int q = 0; q < nb; ++q) {
                    const int p = p0 + q;
                    rec_start(cf->lg0[m], m, spin, pr->sh[p], pr->ch[p], &cN[q], &pN[q], &eN[q]);
                    if (spin) rec_start(cf->lg0[m], m, spin, pr->ch[p], pr->sh[p], &cS[q], &pS[q], &eS[q]);
                    a1[q] = a2[q] = a3[q] = a4[q] = 0.0;
                }
                for (int l = l0; l <= L; ++l) {
                    const double al = cf->al[b + l], ga = cf->ga[b + l], be = cf->be[b + l];
                    if (spin == 0) {
                        const cplx a = A[l];
                        const int odd = (l + m) & 1;
                        for (int q = 0; q < nb; ++q) {
                            const double x = pr->x[p0 + q];
                            if (eN[q] == 0) {
                                if (odd) a2[q] += a * cN[q];
                                else a1[q] += a * cN[q];
                            }
                            const double nx = al * x * cN[q] - be * pN[q];
                            pN[q] = cN[q];
                            cN[q] = nx;
                            if (eN[q] < 0 && fabs(cN[q]) > 0x1p200) {
                                cN[q] *= 0x1p-512;
                                pN[q] *= 0x1p-512;
                                eN[q] += 512;
                            }
                        }
                    } else {
                        const cplx Av = A[l], Bv = B[l];
                        for (int q = 0; q < nb; ++q) {
                            const double x = pr->x[p0 + q];
                            if (eN[q] == 0) {
                                a1[q] += Av * cN[q]; /* h+ at north ring */
                                a4[q] += Bv * cN[q]; /* h- at south ring */
                            }
                            if (eS[q] == 0) {
                                a2[q] += Av * cS[q]; /* h+ at south ring */
                                a3[q] += Bv * cS[q]; /* h- at north ring */
                            }
                            const double nN = (al * x + ga) * cN[q] - be * pN[q];
                            const double nS = (-al * x + ga) * cS[q] - be * pS[q];
                            pN[q] = cN[q];
                            cN[q] = nN;
                            pS[q] = cS[q];
                            cS[q] = nS;
                            if (eN[q] < 0 && fabs(cN[q]) > 0x1p200) {
                                cN[q] *= 0x1p-512;
                                pN[q] *= 0x1p-512;
                                eN[q] += 512;
                            }
                            if (eS[q] < 0 && fabs(cS[q]) > 0x1p200) {
                                cS[q] *= 0x1p-512;
                                pS[q] *= 0x1p-512;
                                eS[q] += 512;
                            }
                        }
                    }
                }
                for (int q = 0; q < nb; ++q) {
                    const int p = p0 + q, n = pr->rn[p], s = pr->rs[p];
                    if (spin == 0) {
                        H[(long)m * ld + n] = a1[q] + a2[q];
                        if (s != n) H[(long)m * ld + s] = a1[q] - a2[q];
                    } else {
                        const double sgs = (spin & 1) ? -1.0 : 1.0;
                        H[(long)(L + m) * ld + n] = -a1[q];
                        if (s != n) H[(long)(L + m) * ld + s] = -a2[q];
                        if (m > 0) {
                            H[(long)(L - m) * ld + n] = -sgs * a3[q];
                            if (s != n) H[(long)(L - m) * ld + s] = -sgs * a4[q];
                        }
                    }
                }
            }
        }
        free(A);
        free(B);
    }
}

/* ------------------------------------------------------------------ ES kernel */
static void gauss_legendre(int n, double *x, double *w) {
    for (int i = 0; i < n; ++i) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double dz = p1 / pp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

static void es_params(double eps, int *w, double *beta) {
    int ww = (int)ceil(-log10(eps / 10.0) - 1e-9) + 1;
    if (ww < 2) ww = 2;
    if (ww > 16) ww = 16;
    double bon = 2.30;
    if (ww == 2) bon = 2.20;
    else if (ww == 3) bon = 2.26;
    else if (ww == 4) bon = 2.38;
    *w = ww;
    *beta = bon * ww;
}

/* int_{-w/2}^{w/2} psi(2t/w) cos(xi t) dt */
static double es_ft(double xi, int w, double beta, const double *z, const double *wz, int nq) {
    double s = 0.0;
    for (int i = 0; i < nq; ++i) {
        const double q = 1.0 - z[i] * z[i];
        s += wz[i] * exp(beta * (sqrt(q) - 1.0)) * cos(xi * 0.5 * w * z[i]);
    }
    return 0.5 * w * s;
}

static double es_kernel(double zz, double beta) {
    const double q = 1.0 - zz * zz;
    return q > 0.0 ? exp(beta * (sqrt(q) - 1.0)) : 0.0;
}

/* ------------------------------------------------------------------ plan */
typedef struct {
    int lmax, max_spin, nring, nphi, w, Nt, Np, ncc, Ntf, Npf, n_lo, nrows, Mb;
    long npix, nalm;
    double beta;
    double *theta, *phi0, *sth, *cth;
    pairs_t gl, cc;
    coef_t cf[3];
    double *lfac, *Dth, *Dph;
    fft_t f_nt, f_ntf, f_npf, f_mb;
    cplx *chirp, *bker;
    cplx *Hgl, *H, *F, *U;
    double *glmap, *ptg, *gam;
} fc_plan;

static void pairs_alloc(pairs_t *p, int n) {
    p->npairs = n;
    p->x = (double *)malloc(sizeof(double) * n);
    p->sh = (double *)malloc(sizeof(double) * n);
    p->ch = (double *)malloc(sizeof(double) * n);
    p->rn = (int *)malloc(sizeof(int) * n);
    p->rs = (int *)malloc(sizeof(int) * n);
}

static void pairs_free(pairs_t *p) {
    free(p->x);
    free(p->sh);
    free(p->ch);
    free(p->rn);
    free(p->rs);
}

/* GL-type geometry: nring rings (ascending theta, north/south symmetric), nphi
 * pixels each, ring r at offset r * nphi, longitudes phi0[r] + 2 pi j / nphi. */
void *fc_plan_create(int lmax, int max_spin, int nring, const double *theta, const double *phi0, int nphi,
                     double eps) {
    fc_plan *P = (fc_plan *)calloc(1, sizeof(fc_plan));
    P->lmax = lmax;
    P->max_spin = max_spin;
    P->nring = nring;
    P->nphi = nphi;
    P->npix = (long)nring * nphi;
    P->nalm = nalm_of(lmax);
    P->theta = (double *)malloc(sizeof(double) * nring);
    P->phi0 = (double *)malloc(sizeof(double) * nring);
    P->sth = (double *)malloc(sizeof(double) * nring);
    P->cth = (double *)malloc(sizeof(double) * nring);
    for (int r = 0; r < nring; ++r) {
        P->theta[r] = theta[r];
        P->phi0[r] = phi0[r];
        P->sth[r] = sin(theta[r]);
        P->cth[r] = cos(theta[r]);
    }
    pairs_alloc(&P->gl, (nring + 1) / 2);
    for (int p = 0; p < P->gl.npairs; ++p) {
        const double t = theta[p];
        P->gl.x[p] = cos(t);
        P->gl.sh[p] = sin(0.5 * t);
        P->gl.ch[p] = cos(0.5 * t);
        P->gl.rn[p] = p;
        P->gl.rs[p] = nring - 1 - p;
    }
    P->Nt = next_pow2(2L * lmax + 2);
    if (P->Nt < 32) P->Nt = 32;
    P->Np = P->Nt;
    P->ncc = P->Nt / 2 + 1;
    P->Ntf = 2 * P->Nt;
    P->Npf = 2 * P->Np;
    es_params(eps, &P->w, &P->beta);
    const int hw = (P->w + 1) / 2;
    P->n_lo = -hw - 1;
    P->nrows = (P->Ntf / 2 + hw + 1) - P->n_lo + 1;
    pairs_alloc(&P->cc, P->Nt / 4 + 1);
    for (int k = 0; k <= P->Nt / 4; ++k) {
        const double t = TWOPI * k / P->Nt;
        P->cc.x[k] = cos(t);
        P->cc.sh[k] = sin(0.5 * t);
        P->cc.ch[k] = cos(0.5 * t);
        P->cc.rn[k] = k;
        P->cc.rs[k] = P->Nt / 2 - k;
    }
    for (int s = 0; s <= 2; ++s) coef_build(&P->cf[s], lmax, s);
    P->lfac = (double *)malloc(sizeof(double) * (lmax + 1));
    for (int l = 0; l <= lmax; ++l) P->lfac[l] = sqrt((double)l * (l + 1.0));
    {
        const int nq = 400;
        double *z = (double *)malloc(sizeof(double) * nq), *wz = (double *)malloc(sizeof(double) * nq);
        gauss_legendre(nq, z, wz);
        P->Dth = (double *)calloc(P->Nt, sizeof(double));
        P->Dph = (double *)calloc(2 * lmax + 1, sizeof(double));
        for (int k = -P->Nt / 2 + 1; k < P->Nt / 2; ++k)
            P->Dth[(k + P->Nt) % P->Nt] = 1.0 / (P->Nt * es_ft(TWOPI * k / P->Ntf, P->w, P->beta, z, wz, nq));
        for (int m = -lmax; m <= lmax; ++m)
            P->Dph[m + lmax] = 1.0 / es_ft(TWOPI * m / P->Npf, P->w, P->beta, z, wz, nq);
        free(z);
        free(wz);
    }
    fft_init(&P->f_nt, P->Nt);
    fft_init(&P->f_ntf, P->Ntf);
    fft_init(&P->f_npf, P->Npf);
    /* Bluestein for the ring length */
    P->Mb = next_pow2(2L * nphi - 1);
    fft_init(&P->f_mb, P->Mb);
    P->chirp = (cplx *)malloc(sizeof(cplx) * nphi);
    P->bker = (cplx *)calloc(P->Mb, sizeof(cplx));
    for (int q = 0; q < nphi; ++q) {
        const long qq = ((long)q * q) % (2L * nphi);
        const long double a = PI_L * (long double)qq / (long double)nphi;
        P->chirp[q] = (double)cosl(a) + I * (double)sinl(a);
    }
    for (int k = 0; k < nphi; ++k) {
        const cplx bb = conj(P->chirp[k]) / P->Mb;
        P->bker[k] = bb;
        if (k > 0) P->bker[P->Mb - k] = bb;
    }
    fft_run(&P->f_mb, P->bker, -1);
    const long ncols = max_spin ? 2L * lmax + 1 : lmax + 1;
    P->Hgl = (cplx *)malloc(sizeof(cplx) * (2L * lmax + 1) * nring);
    P->H = (cplx *)malloc(sizeof(cplx) * ncols * P->ncc);
    P->F = (cplx *)malloc(sizeof(cplx) * ncols * P->nrows);
    P->U = (cplx *)malloc(sizeof(cplx) * (long)P->nrows * P->Npf);
    P->glmap = (double *)malloc(sizeof(double) * 2 * P->npix);
    P->ptg = (double *)malloc(sizeof(double) * 2 * P->npix);
    P->gam = (double *)malloc(sizeof(double) * P->npix);
    return P;
}

void fc_plan_destroy(void *vp) {
    fc_plan *P = (fc_plan *)vp;
    if (!P) return;
    free(P->theta);
    free(P->phi0);
    free(P->sth);
    free(P->cth);
    pairs_free(&P->gl);
    pairs_free(&P->cc);
    for (int s = 0; s <= 2; ++s) coef_free(&P->cf[s]);
    free(P->lfac);
    free(P->Dth);
    free(P->Dph);
    fft_free(&P->f_nt);
    fft_free(&P->f_ntf);
    fft_free(&P->f_npf);
    fft_free(&P->f_mb);
    free(P->chirp);
    free(P->bker);
    free(P->Hgl);
    free(P->H);
    free(P->F);
    free(P->U);
    free(P->glmap);
    free(P->ptg);
    free(P->gam);
    free(P);
}

long fc_plan_npix(void *vp) { return ((fc_plan *)vp)->npix; }

/* ------------------------------------------------------------------ stages */
/* spin-s ring transform z_p = sum_m h_m e^{i m (phi0 + 2 pi p / N)} by Bluestein */
static void ring_synth(fc_plan *P, int spin, const cplx *Hgl, double *out0, double *out1) {
    const int L = P->lmax, N = P->nphi, M = P->Mb, nring = P->nring;
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * M);
#pragma omp for schedule(static)
        for (int r = 0; r < nring; ++r) {
            memset(buf, 0, sizeof(cplx) * M);
            const double ph0 = P->phi0[r];
            if (spin == 0) {
                for (int m = 0; m <= L; ++m) {
                    cplx h = Hgl[(long)m * nring + r];
                    if (m == 0) {
                        buf[0] = creal(h);
                        continue;
                    }
                    if (ph0 != 0.0) h *= cexp(I * (m * ph0));
                    buf[m] = h * P->chirp[m];
                    buf[N - m] = conj(h) * P->chirp[N - m];
                }
            } else {
                for (int c = 0; c < 2 * L + 1; ++c) {
                    const int m = c - L;
                    cplx h = Hgl[(long)c * nring + r];
                    if (ph0 != 0.0) h *= cexp(I * (m * ph0));
                    const int q = ((m % N) + N) % N;
                    buf[q] = h * P->chirp[q];
                }
            }
            fft_run(&P->f_mb, buf, -1);
            for (int i = 0; i < M; ++i) buf[i] *= P->bker[i];
            fft_run(&P->f_mb, buf, +1);
            const long o = (long)r * N;
            for (int p = 0; p < N; ++p) {
                const cplx z = buf[p] * P->chirp[p];
                out0[o + p] = creal(z);
                if (spin) out1[o + p] = cimag(z);
            }
        }
        free(buf);
    }
}

/* deflected angles (pointing.cu:210-213, phi' wrapped only when >= 2 pi) and
 * gamma (CPU_nufft_transformer.py:158-160) */
static void pointing(fc_plan *P, const double *dth, const double *dph, double *oth, double *oph, double *ogam) {
    const int N = P->nphi;
#pragma omp parallel for schedule(static)
    for (long j = 0; j < P->npix; ++j) {
        const int r = (int)(j / N);
        const double st = P->sth[r], ct = P->cth[r];
        const double phi = P->phi0[r] + (double)(j - (long)r * N) * (TWOPI / N);
        const double t = dth[j], p = dph[j];
        const double d2 = t * t + p * p;
        double sinaoa, cosa;
        if (d2 > 1e-6) {
            const double a = sqrt(d2);
            sinaoa = sin(a) / a;
            cosa = cos(a);
        } else {
            sinaoa = 1.0 - d2 / 6.0 * (1.0 - d2 / 20.0 * (1.0 - d2 / 42.0 * (1.0 - d2 / 72.0)));
            cosa = 1.0 - d2 / 2.0 * (1.0 - d2 / 12.0 * (1.0 - d2 / 30.0 * (1.0 - d2 / 56.0)));
        }
        const double nx = st * cosa + ct * t * sinaoa;
        const double ny = -p * sinaoa;
        const double nz = ct * cosa - st * t * sinaoa;
        oth[j] = atan2(sqrt(nx * nx + ny * ny), nz);
        double php = phi - atan2(ny, nx);
        if (php >= TWOPI) php -= TWOPI;
        oph[j] = php;
        if (ogam) {
            const double x2 = d2 * sinaoa * (ct / st) + t * cosa;
            ogam[j] = (d2 > 0.0) ? atan2(p * x2 - t * p, t * x2 + p * p) : 0.0;
        }
    }
}

/* theta pass: extend each CC column to the torus, FFT, deconvolve, pad, inverse FFT */
static void theta_pass(fc_plan *P, int spin) {
    const int L = P->lmax, Nt = P->Nt, Ntf = P->Ntf, half = Nt / 2;
    const int ncols = spin ? 2 * L + 1 : L + 1, mofs = spin ? L : 0;
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * Nt);
        cplx *pad = (cplx *)malloc(sizeof(cplx) * Ntf);
#pragma omp for schedule(static)
        for (int c = 0; c < ncols; ++c) {
            const int m = c - mofs;
            const double sgn = ((abs(m) + spin) & 1) ? -1.0 : 1.0;
            const cplx *col = P->H + (long)c * P->ncc;
            for (int k = 0; k < Nt; ++k) buf[k] = k <= half ? col[k] : sgn * col[Nt - k];
            fft_run(&P->f_nt, buf, -1);
            const double dm = P->Dph[m + L];
            memset(pad, 0, sizeof(cplx) * Ntf);
            for (int i = 0; i < half; ++i) pad[i] = buf[i] * (P->Dth[i] * dm);
            for (int i = 0; i < half - 1; ++i) pad[Ntf - 1 - i] = buf[Nt - 1 - i] * (P->Dth[Nt - 1 - i] * dm);
            fft_run(&P->f_ntf, pad, +1);
            for (int r = 0; r < P->nrows; ++r) {
                const int n = ((r + P->n_lo) % Ntf + Ntf) % Ntf;
                P->F[(long)r * ncols + c] = pad[n];
            }
        }
        free(buf);
        free(pad);
    }
}

/* phi pass: modes -> oversampled longitudes; spin 0 rows are real (h_{-m} = conj h_m) */
static void phi_pass(fc_plan *P, int spin) {
    const int L = P->lmax, Npf = P->Npf;
    const int ncols = spin ? 2 * L + 1 : L + 1;
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * Npf);
#pragma omp for schedule(static)
        for (int r = 0; r < P->nrows; ++r) {
            memset(buf, 0, sizeof(cplx) * Npf);
            const cplx *row = P->F + (long)r * ncols;
            if (spin) {
                for (int c = 0; c < ncols; ++c) buf[((c - L) % Npf + Npf) % Npf] = row[c];
            } else {
                buf[0] = creal(row[0]);
                for (int m = 1; m < ncols; ++m) {
                    buf[m] = row[m];
                    buf[Npf - m] = conj(row[m]);
                }
            }
            fft_run(&P->f_npf, buf, +1);
            memcpy(P->U + (long)r * Npf, buf, sizeof(cplx) * Npf);
        }
        free(buf);
    }
}

/* type-2 interpolation at (theta', phi') with the exp(i s gamma) rotation */
static void interp(fc_plan *P, int spin, const double *th, const double *ph, const double *gam, double *out0,
                   double *out1) {
    const int w = P->w, Ntf = P->Ntf, Npf = P->Npf, nrows = P->nrows;
    const double beta = P->beta, s2 = 2.0 / w, hw = 0.5 * w;
#pragma omp parallel for schedule(static)
    for (long j = 0; j < P->npix; ++j) {
        double t = th[j] * ((double)Ntf / TWOPI);
        if (t < -1.0) t = -1.0;
        if (t > 0.5 * Ntf + 1.0) t = 0.5 * Ntf + 1.0;
        double p = ph[j] * ((double)Npf / TWOPI);
        p -= floor(p / (double)Npf) * (double)Npf;
        const int n0 = (int)ceil(t - hw), p0 = (int)ceil(p - hw);
        const double ft = (double)n0 - t, fp = (double)p0 - p;
        int r0 = n0 - P->n_lo;
        if (r0 < 0) r0 = 0;
        if (r0 > nrows - w) r0 = nrows - w;
        double kt[16], kp[16];
        int cols[16];
        for (int a = 0; a < w; ++a) {
            kt[a] = es_kernel((ft + a) * s2, beta);
            kp[a] = es_kernel((fp + a) * s2, beta);
            int c = p0 + a;
            c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
            cols[a] = c;
        }
        cplx acc = 0.0;
        for (int a = 0; a < w; ++a) {
            const cplx *row = P->U + (long)(r0 + a) * Npf;
            cplx rr = 0.0;
            for (int b2 = 0; b2 < w; ++b2) rr += kp[b2] * row[cols[b2]];
            acc += kt[a] * rr;
        }
        if (spin) {
            if (gam) acc *= cexp(I * (spin * gam[j]));
            out0[j] = creal(acc);
            out1[j] = cimag(acc);
        } else {
            out0[j] = creal(acc);
        }
    }
}

/* Lensed map: gclm (ncomp, nalm) complex interleaved, dlm_scaled (nalm)
 * [+ dclm_scaled for curl, may be NULL] -> out (npix) spin 0 or (2, npix)
 * (Q, U) spin s.  nthreads <= 0: all cores. */
int fc_lensing(void *vp, int spin, int ncomp, const double *gclm, const double *dlm, const double *dclm,
               double *out, int nthreads) {
    fc_plan *P = (fc_plan *)vp;
    if (spin > P->max_spin || spin < 0) return 1;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const int L = P->lmax;
    const long npix = P->npix;
    leg_synth(L, 1, &P->cf[1], (const cplx *)dlm, (const cplx *)dclm, P->lfac, &P->gl, P->Hgl, P->nring);
    ring_synth(P, 1, P->Hgl, P->glmap, P->glmap + npix);
    pointing(P, P->glmap, P->glmap + npix, P->ptg, P->ptg + npix, spin ? P->gam : NULL);
    const cplx *G = (const cplx *)gclm;
    const cplx *C = (spin && ncomp > 1) ? G + P->nalm : NULL;
    leg_synth(L, spin, &P->cf[spin], G, C, NULL, &P->cc, P->H, P->ncc);
    theta_pass(P, spin);
    phi_pass(P, spin);
    interp(P, spin, P->ptg, P->ptg + npix, spin ? P->gam : NULL, out, spin ? out + npix : NULL);
    return 0;
}

/* pointing of the last fc_lensing call: (2, npix) theta', phi' */
void fc_last_pointing(void *vp, double *ptg) {
    fc_plan *P = (fc_plan *)vp;
    memcpy(ptg, P->ptg, sizeof(double) * 2 * P->npix);
}

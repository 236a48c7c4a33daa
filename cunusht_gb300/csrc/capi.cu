// C ABI of the library (include/cunusht_gb300.h): plans and entry points.
#include <stdarg.h>
#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cunusht {

static thread_local std::string g_err;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
}
void clear_error() { g_err.clear(); }

static int next_pow2(long long n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

// Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on P_n.
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(PI * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int j = 2; j <= n; ++j) {
                double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int j = 2; j <= n; ++j) {
            double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
            p0 = p1;
            p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// ES kernel parameters for oversampling 2: beta = 2.30 width as in the FINUFFT
// rule behind cuFINUFFT's upsampfac 2, but one tap wider than its
// width = ceil(log10(10/eps)), which measures 1.5e-7 relative L2 for
// full-band white spectra at eps = 1e-7; the extra tap keeps results within eps.
static void es_params(double eps, int &w, double &beta) {
    w = (int)std::ceil(-std::log10(eps / 10.0) - 1e-9) + 1;
    w = std::max(2, std::min(16, w));
    double bon = 2.30;
    if (w == 2) bon = 2.20;
    else if (w == 3) bon = 2.26;
    else if (w == 4) bon = 2.38;
    beta = bon * w;
}

// Fourier transform of the kernel in fine-grid units:
// Phi(xi) = int_{-w/2}^{w/2} psi(2 t / w) cos(xi t) dt.
struct EsFT {
    std::vector<double> z, wz;
    int w;
    double beta;
    EsFT(int w_, double beta_) : w(w_), beta(beta_) { gauss_legendre(400, z, wz); }
    double operator()(double xi) const {
        double s = 0.0;
        for (size_t i = 0; i < z.size(); ++i) {
            const double q = 1.0 - z[i] * z[i];
            const double psi = std::exp(beta * (std::sqrt(q) - 1.0));
            s += wz[i] * psi * std::cos(xi * 0.5 * w * z[i]);
        }
        return 0.5 * w * s;
    }
};

template <typename T> static int dalloc(cunusht_plan_s *P, T **p, size_t n) {
    *p = nullptr;
    if (n == 0) return CUNUSHT_OK;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        set_error("cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
        *p = nullptr;
        return CUNUSHT_ERR_ALLOC;
    }
    P->ws_bytes += n * sizeof(T);
    return CUNUSHT_OK;
}

int plan_alloc(cunusht_plan_s *P, void **p, size_t bytes) {
    char *c = nullptr;
    RC_TRY(dalloc(P, &c, bytes));
    *p = c;
    return CUNUSHT_OK;
}

template <typename T> static int upload(cunusht_plan_s *P, T **p, const std::vector<T> &h) {
    RC_TRY(dalloc(P, p, h.size()));
    if (!h.empty()) CU_TRY(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return CUNUSHT_OK;
}

static void free_plan(cunusht_plan_s *P) {
    if (!P) return;
    void *ptrs[] = {P->d_ring_sc, P->d_ring_theta, P->d_ring_phi0, P->d_ring_nph, P->d_ring_ofs, P->d_gl_x, P->d_gl_sh,
                    P->d_gl_ch, P->d_gl_rn, P->d_gl_rs, P->d_cc_x, P->d_cc_sh, P->d_cc_ch, P->d_cc_rn,
                    P->d_cc_rs, P->d_Dth, P->d_Dph, P->d_coef[0], P->d_coef[1], P->d_coef[2], P->d_lg0[0],
                    P->d_lg0[1], P->d_lg0[2], P->d_lfac, P->d_coef_df[0], P->d_coef_df[1], P->d_coef_df[2], P->d_tw64, P->d_tw32, P->d_twdf, P->d_chirp_df, P->d_bker_df, P->d_chirp, P->d_bker,
                    P->d_H, P->d_F, P->d_U, P->d_Hgl, P->d_ring, P->d_glmap, P->d_alm, P->d_vjp, P->d_lfac_g, P->d_ring_cls, P->d_cls_N, P->d_cls_Mb, P->d_cls_SP,
                    P->d_cls_coff, P->d_cls_boff, P->d_Hb, P->d_Fb, P->d_Ub,  // d_Hglb, d_glmapb alias d_Hb, d_Fb
                    P->d_ptgb, P->d_gamb, P->d_status, P->d_tc_woff[0], P->d_tc_woff[1], P->d_tc_woff[2],
                    P->d_tc_rec, P->d_mr_pos, P->d_mr_tw64, P->d_mr_twdf};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (P->d_bin) cudaFree(P->d_bin);
    if (P->d_ufix) cudaFree(P->d_ufix);
    if (P->d_vmax) cudaFree(P->d_vmax);
    for (int g = 0; g < 2; ++g)
        for (int s = 0; s < 3; ++s) {
            if (P->d_tc_stv[g][s]) cudaFree(P->d_tc_stv[g][s]);
            if (P->d_tc_ste[g][s]) cudaFree(P->d_tc_ste[g][s]);
        }
    for (auto &e : P->evt_pool) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    delete P;
}

static double lg0_of(int m, int s) {
    const int l0 = std::max(m, s);
    const double v = std::log((2.0 * l0 + 1.0) / (4.0 * PI)) + std::lgamma(2.0 * l0 + 1.0) -
                     std::lgamma(m + s + 1.0) - std::lgamma(std::fabs((double)(m - s)) + 1.0);
    return 0.5 * v / std::log(2.0);
}

// In-place forward DFT X_k = sum_n x_n e^{-2 pi i nk/n} (n a power of two):
// iterative radix-2 Cooley-Tukey in long double, plan set-up only.
static void host_fft_forward(std::vector<double2> &a) {
    const size_t n = a.size();
    std::vector<std::complex<long double>> x(n);
    for (size_t i = 0; i < n; ++i) x[i] = {a[i].x, a[i].y};
    for (size_t i = 1, j = 0; i < n; ++i) {  // bit reversal
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    const long double pi = 3.14159265358979323846264338327950288L;
    for (size_t len = 2; len <= n; len <<= 1) {
        for (size_t k = 0; k < len / 2; ++k) {
            const long double ang = -2.0L * pi * (long double)k / (long double)len;
            const std::complex<long double> w(std::cos(ang), std::sin(ang));
            for (size_t i = 0; i < n; i += len) {
                const std::complex<long double> u = x[i + k], v = x[i + k + len / 2] * w;
                x[i + k] = u + v;
                x[i + k + len / 2] = u - v;
            }
        }
    }
    for (size_t i = 0; i < n; ++i) a[i] = make_double2((double)x[i].real(), (double)x[i].imag());
}

static int build_plan(cunusht_plan_s *P, int lmax, double eps, int precision, int max_spin, int nring,
                      const double *rth, const double *rph0, const int64_t *rnph, const int64_t *rofs) {
    ARG_CHECK(lmax >= 1 && lmax <= 16383, "lmax must be in [1, 16383], got %d", lmax);
    ARG_CHECK(eps >= 1e-14 && eps < 1.0, "epsilon must be in [1e-14, 1), got %g", eps);
    ARG_CHECK(max_spin >= 0 && max_spin <= 2, "max_spin must be 0, 1 or 2, got %d", max_spin);
    ARG_CHECK(nring >= 1 && rth && rph0 && rnph && rofs, "pointing geometry arrays missing (nring=%d)", nring);
    ARG_CHECK(precision >= 0 && precision <= 2, "precision must be 0 (auto), 1 (fp64) or 2 (mixed)");
    P->lmax = lmax;
    P->eps = eps;
    P->max_spin = max_spin;
    P->nalm = (long long)(lmax + 1) * (lmax + 2) / 2;
    P->nalm_tab = P->nalm;
    P->mmax = lmax;
    P->prec = precision == CUNUSHT_PREC_AUTO ? (eps > 1e-6 ? CUNUSHT_PREC_MIXED : CUNUSHT_PREC_FP64) : precision;
    P->grid_fp32 = (P->prec != CUNUSHT_PREC_FP64) && eps > 1e-6;
    P->fwd_u32 = (P->prec == CUNUSHT_PREC_MIXED) && !P->grid_fp32;
    P->fft_df = P->fwd_u32;
    // the ring transforms stay double-float at every eps: in FP64 they were the
    // largest FP64-pipe stage of the eps > 1e-6 plans (GB300 issues FP64 at
    // 1/80 of the FP32 rate)
    P->ring_df = P->prec == CUNUSHT_PREC_MIXED;

    // ---- pointing geometry, sorted by first pixel (Geom, geometry.py:47-52)
    std::vector<int> order(nring);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return rofs[a] < rofs[b]; });
    P->nring = nring;
    P->h_theta.resize(nring);
    P->h_phi0.resize(nring);
    P->h_nph.resize(nring);
    P->h_ofs.resize(nring);
    long long npix = 0;
    for (int i = 0; i < nring; ++i) {
        const int o = order[i];
        ARG_CHECK(rnph[o] >= 1, "ring %d has %lld pixels", o, (long long)rnph[o]);
        ARG_CHECK(rth[o] >= 0.0 && rth[o] <= PI, "ring %d colatitude %g outside [0, pi]", o, rth[o]);
        P->h_theta[i] = rth[o];
        P->h_phi0[i] = rph0[o];
        P->h_nph[i] = rnph[o];
        P->h_ofs[i] = rofs[o];
        npix += rnph[o];
    }
    for (int i = 0; i + 1 < nring; ++i)
        ARG_CHECK(P->h_ofs[i] + P->h_nph[i] <= P->h_ofs[i + 1], "rings overlap (ring starts/counts inconsistent)");
    P->npix = npix;
    const long long npix_span = P->h_ofs[nring - 1] + P->h_nph[nring - 1];
    ARG_CHECK(npix_span == npix && P->h_ofs[0] == 0, "ring pixels must tile [0, npix) contiguously");
    // rings may have different pixel counts (HEALPix, thinned grids), fewer than
    // 2 lmax + 1 included (the ring transforms fold the aliased modes)
    P->nph_uniform = (int)P->h_nph[0];
    for (int i = 1; i < nring; ++i)
        if (P->h_nph[i] != P->h_nph[0]) P->nph_uniform = 0;

    // ring pairs (theta, pi - theta)
    {
        std::vector<int> idx(nring);
        std::iota(idx.begin(), idx.end(), 0);
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return P->h_theta[a] < P->h_theta[b]; });
        std::vector<double> x, sh, ch;
        std::vector<int> rn, rs;
        for (int i = 0, j = nring - 1; i <= j; ++i, --j) {
            const double tn = P->h_theta[idx[i]], ts = P->h_theta[idx[j]];
            if (std::fabs(tn + ts - PI) > 1e-9) {
                set_error("pointing geometry is not north/south symmetric (ring %g vs %g)", tn, ts);
                return CUNUSHT_ERR_UNSUPPORTED;
            }
            x.push_back(std::cos(tn));
            sh.push_back(std::sin(0.5 * tn));
            ch.push_back(std::cos(0.5 * tn));
            rn.push_back(idx[i]);
            rs.push_back(idx[j]);
        }
        P->gl_npairs = (int)x.size();
        for (int k = 0; k < P->gl_npairs; ++k)
            if (sh[k] == 0.0) P->gl_pole = k, P->gl_pole_ring[0] = rn[k], P->gl_pole_ring[1] = rs[k];
        RC_TRY(upload(P, &P->d_gl_x, x));
        RC_TRY(upload(P, &P->d_gl_sh, sh));
        RC_TRY(upload(P, &P->d_gl_ch, ch));
        RC_TRY(upload(P, &P->d_gl_rn, rn));
        RC_TRY(upload(P, &P->d_gl_rs, rs));
    }
    RC_TRY(upload(P, &P->d_ring_theta, P->h_theta));
    RC_TRY(upload(P, &P->d_ring_phi0, P->h_phi0));
    RC_TRY(upload(P, &P->d_ring_nph, P->h_nph));
    RC_TRY(upload(P, &P->d_ring_ofs, P->h_ofs));
    {
        std::vector<float4> sc(nring);
        for (int i = 0; i < nring; ++i) {
            const dfl s_ = df_from_host(std::sin(P->h_theta[i])), c_ = df_from_host(std::cos(P->h_theta[i]));
            sc[i] = make_float4(s_.h, s_.l, c_.h, c_.l);
        }
        RC_TRY(upload(P, &P->d_ring_sc, sc));
    }

    // ---- torus and fine grid
    P->Nt = std::max(32, next_pow2(2LL * lmax + 2));
    P->Np = std::max(32, next_pow2(2LL * lmax + 2));
    P->ncc = P->Nt / 2 + 1;
    P->Ntf = 2 * P->Nt;
    P->Npf = 2 * P->Np;
    es_params(eps, P->w, P->beta);
    const int hw = (P->w + 1) / 2;
    P->n_lo = -hw - 1;
    const int n_hi = P->Ntf / 2 + hw + 1;
    P->nrows = n_hi - P->n_lo + 1;
    {
        // transforms longer than 16 x FFT_TPB points run as two half-length
        // transforms split by output parity (a half-size shared buffer)
        const int emax = 16 * FFT_TPB;
        P->sp_theta = P->Ntf > emax ? 2 : 1;
        P->sp_phi = P->Npf > emax ? 2 : 1;
        const int nb = std::max(P->Ntf / P->sp_theta, P->Npf / P->sp_phi);
        if (nb > emax) {
            set_error("lmax %d needs %d-point fine-grid transforms; at most lmax 4095 is supported", lmax, nb);
            return CUNUSHT_ERR_UNSUPPORTED;
        }
    }
    // CC ring pairs: ring k at theta = 2 pi k / Nt, k = 0 .. Nt/2; pair (k, Nt/2 - k)
    {
        std::vector<double> x, sh, ch;
        std::vector<int> rn, rs;
        for (int k = 0; k <= P->Nt / 4; ++k) {
            const double t = TWOPI * k / P->Nt;
            x.push_back(std::cos(t));
            sh.push_back(std::sin(0.5 * t));
            ch.push_back(std::cos(0.5 * t));
            rn.push_back(k);
            rs.push_back(P->Nt / 2 - k);
        }
        P->cc_npairs = (int)x.size();
        for (int k = 0; k < P->cc_npairs; ++k)
            if (sh[k] == 0.0) P->cc_pole = k, P->cc_pole_ring[0] = rn[k], P->cc_pole_ring[1] = rs[k];
        RC_TRY(upload(P, &P->d_cc_x, x));
        RC_TRY(upload(P, &P->d_cc_sh, sh));
        RC_TRY(upload(P, &P->d_cc_ch, ch));
        RC_TRY(upload(P, &P->d_cc_rn, rn));
        RC_TRY(upload(P, &P->d_cc_rs, rs));
    }
    // deconvolution
    {
        EsFT ft(P->w, P->beta);
        std::vector<double> dth(P->Nt, 0.0), dph(2 * lmax + 1, 0.0);
        for (int k = -P->Nt / 2 + 1; k < P->Nt / 2; ++k)
            dth[(k + P->Nt) % P->Nt] = 1.0 / (P->Nt * ft(TWOPI * k / P->Ntf));
        for (int m = -lmax; m <= lmax; ++m) dph[m + lmax] = 1.0 / ft(TWOPI * m / P->Npf);
        RC_TRY(upload(P, &P->d_Dth, dth));
        RC_TRY(upload(P, &P->d_Dph, dph));
    }
    // recursion tables
    for (int s = 0; s <= 2; ++s) {
        RC_TRY(dalloc(P, &P->d_coef[s], 3 * (size_t)P->nalm_tab));
        std::vector<double> lg(lmax + 1);
        for (int m = 0; m <= lmax; ++m) lg[m] = lg0_of(m, s);
        RC_TRY(upload(P, &P->d_lg0[s], lg));
    }
    RC_TRY(build_coef_tables(P, 0));
    if (P->prec == CUNUSHT_PREC_MIXED) {
        for (int s = 0; s <= 2; ++s) RC_TRY(dalloc(P, &P->d_coef_df[s], 3 * (size_t)P->nalm_tab));
        RC_TRY(build_coef_tables_df(P, 0));
    }
    RC_TRY(dalloc(P, &P->d_status, 1));
    CU_TRY(cudaMemset(P->d_status, 0, sizeof(int)));
    if (P->prec == CUNUSHT_PREC_MIXED) RC_TRY(tc_plan_init(P));
    {
        std::vector<double> lf(lmax + 1);
        for (int l = 0; l <= lmax; ++l) lf[l] = std::sqrt((double)l * (l + 1.0));
        RC_TRY(upload(P, &P->d_lfac, lf));
        for (int l = 0; l <= lmax; ++l) lf[l] = l >= 1 ? std::sqrt((l - 1.0) * (l + 2.0)) : 0.0;
        RC_TRY(upload(P, &P->d_lfac_g, lf));
    }
    // Bluestein data for the ring transforms, one set per distinct ring length
    std::vector<int> cls_N, cls_Mb, cls_SP;
    std::vector<long long> cls_coff, cls_boff;
    {
        std::map<long long, int> cls_of;
        std::vector<int> rcls(nring);
        long long csum = 0, bsum = 0;
        P->Mb = 0;
        P->sp_ring = 1;
        P->ring_buf = 0;
        for (int i = 0; i < nring; ++i) {
            const long long N = P->h_nph[i];
            auto it = cls_of.find(N);
            if (it == cls_of.end()) {
                const int Mb = next_pow2(2LL * N - 1);
                const int SP = Mb > 16 * FFT_TPB ? 2 : 1;
                if (Mb / SP > 16 * FFT_TPB) {
                    set_error("ring length %lld needs a Bluestein FFT of %d points; at most 8192 pixels per ring "
                              "are supported", N, Mb);
                    return CUNUSHT_ERR_UNSUPPORTED;
                }
                it = cls_of.emplace(N, (int)cls_N.size()).first;
                cls_N.push_back((int)N);
                cls_Mb.push_back(Mb);
                cls_SP.push_back(SP);
                cls_coff.push_back(csum);
                cls_boff.push_back(bsum);
                csum += N;
                bsum += Mb;
                P->Mb = std::max(P->Mb, Mb);
                P->sp_ring = std::max(P->sp_ring, SP);
                P->ring_buf = std::max(P->ring_buf, Mb / SP);
            }
            rcls[i] = it->second;
        }
        P->ncls = (int)cls_N.size();
        P->nchirp = csum;
        P->nbker = bsum;
        std::vector<double2> chirp(csum), bk(bsum, make_double2(0.0, 0.0));
        for (int c = 0; c < P->ncls; ++c) {
            const int N = cls_N[c], Mb = cls_Mb[c];
            double2 *ch = chirp.data() + cls_coff[c], *bkc = bk.data() + cls_boff[c];
            for (int q = 0; q < N; ++q) {
                const long long qq = ((long long)q * q) % (2LL * N);
                const double a = PI * (double)qq / N;
                ch[q] = make_double2(std::cos(a), std::sin(a));
            }
            const double inv = 1.0 / Mb;
            for (int k = 0; k < N; ++k) {
                const double2 b = make_double2(ch[k].x * inv, -ch[k].y * inv);
                bkc[k] = b;
                if (k > 0) bkc[Mb - k] = b;
            }
        }
        RC_TRY(upload(P, &P->d_chirp, chirp));
        RC_TRY(upload(P, &P->d_bker, bk));
        if (P->ncls > 1) {
            RC_TRY(upload(P, &P->d_ring_cls, rcls));
            RC_TRY(upload(P, &P->d_cls_N, cls_N));
            RC_TRY(upload(P, &P->d_cls_Mb, cls_Mb));
            RC_TRY(upload(P, &P->d_cls_SP, cls_SP));
            RC_TRY(upload(P, &P->d_cls_coff, cls_coff));
            RC_TRY(upload(P, &P->d_cls_boff, cls_boff));
        }
    }
    RC_TRY(ring_mr_init(P));
    // twiddles
    {
        P->TW = std::max(std::max(P->Ntf, P->Npf), P->Mb);
        std::vector<double2> tw(P->TW);
        std::vector<float2> tw32(P->TW);
        for (int t = 0; t < P->TW; ++t) {
            const long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)P->TW;
            tw[t] = make_double2((double)std::cos(a), (double)std::sin(a));
            tw32[t] = make_float2((float)tw[t].x, (float)tw[t].y);
        }
        RC_TRY(upload(P, &P->d_tw64, tw));
        RC_TRY(upload(P, &P->d_tw32, tw32));
    }
    // kernel spectra, per class
    for (int c = 0; c < P->ncls; ++c) {
        double2 *b = P->d_bker + cls_boff[c];
        const int Mb = cls_Mb[c];
        if (cls_SP[c] == 1) {
            RC_TRY(fft_global_f64(b, Mb, -1, P->d_tw64, P->TW, 0));
        } else {
            // too long for one shared-memory transform: the kernel spectrum on the host
            std::vector<double2> bk(Mb);
            CU_TRY(cudaMemcpy(bk.data(), b, Mb * sizeof(double2), cudaMemcpyDeviceToHost));
            host_fft_forward(bk);
            CU_TRY(cudaMemcpy(b, bk.data(), Mb * sizeof(double2), cudaMemcpyHostToDevice));
        }
    }
    if (P->fft_df || P->ring_df) {
        char *t = nullptr, *c = nullptr, *b = nullptr;
        RC_TRY(dalloc(P, &t, 16 * (size_t)P->TW));
        RC_TRY(dalloc(P, &c, 16 * (size_t)P->nchirp));
        RC_TRY(dalloc(P, &b, 16 * (size_t)P->nbker));
        P->d_twdf = t;
        P->d_chirp_df = c;
        P->d_bker_df = b;
        RC_TRY(split_c128_to_df(P->d_tw64, P->TW, P->d_twdf, 0));
        RC_TRY(split_c128_to_df(P->d_chirp, P->nchirp, P->d_chirp_df, 0));
        RC_TRY(split_c128_to_df(P->d_bker, P->nbker, P->d_bker_df, 0));
    }
    // workspace
    {
        const long long ncols = max_spin ? 2LL * lmax + 1 : lmax + 1;
        const size_t gsz = P->grid_fp32 ? sizeof(float2) : sizeof(double2);
        const size_t usz = (P->grid_fp32 ? sizeof(float) : sizeof(double)) * (max_spin ? 2 : 1);
        RC_TRY(dalloc(P, &P->d_H, (size_t)ncols * P->ncc));
        char *f = nullptr, *u = nullptr;
        RC_TRY(dalloc(P, &f, gsz * (size_t)ncols * P->nrows));
        P->d_F = f;
        RC_TRY(dalloc(P, &u, usz * (size_t)P->nrows * P->Npf));
        P->d_U = u;
        P->u_bytes = usz * (size_t)P->nrows * P->Npf;
        if (P->sp_theta == 2 && (size_t)ncols * P->Nt * gsz > usz * (size_t)P->nrows * P->Npf) {
            set_error("internal: split theta adjoint scratch does not fit the fine-grid workspace");
            return CUNUSHT_ERR_UNSUPPORTED;
        }
        RC_TRY(dalloc(P, &P->d_Hgl, (size_t)(2 * lmax + 1) * nring));
        RC_TRY(dalloc(P, &P->d_glmap, 2 * (size_t)npix));
        RC_TRY(dalloc(P, &P->d_alm, 2 * (size_t)P->nalm));
        RC_TRY(dalloc(P, &P->d_vjp, 4 * (size_t)npix));
    }
    CU_TRY(cudaStreamSynchronize(0));
    CU_TRY(cudaGetLastError());
    return CUNUSHT_OK;
}

static int check_plan(const cunusht_plan_s *P) {
    ARG_CHECK(P != nullptr, "plan is NULL");
    return CUNUSHT_OK;
}

static int check_spin(const cunusht_plan_s *P, int spin, int ncomp) {
    ARG_CHECK(spin >= 0 && spin <= P->max_spin, "spin %d outside [0, max_spin=%d] of the plan", spin,
              P->max_spin);
    if (spin == 0) ARG_CHECK(ncomp == 1, "spin 0 takes ncomp = 1, got %d", ncomp);
    else ARG_CHECK(ncomp == 1 || ncomp == 2, "spin %d takes ncomp 1 (gradient only) or 2, got %d", spin, ncomp);
    return CUNUSHT_OK;
}


// Brackets one stage launch with CUDA events when profiling is on.
struct StageScope {
    cunusht_plan_s *P;
    int stage;
    cudaStream_t st;
    int slot = -1;
    StageScope(cunusht_plan_s *P_, int stage_, cudaStream_t st_) : P(P_), stage(stage_), st(st_) {
        if (!P->profiling) return;
        if (P->evt_used >= (int)P->evt_pool.size()) flush_events(P);
        if (P->evt_used >= (int)P->evt_pool.size()) return;
        slot = P->evt_used++;
        P->evt_pool[slot].stage = stage;
        cudaEventRecord(P->evt_pool[slot].a, st);
    }
    ~StageScope() {
        if (slot >= 0) cudaEventRecord(P->evt_pool[slot].b, st);
    }
    static void flush_events(cunusht_plan_s *P) {
        for (int i = 0; i < P->evt_used; ++i) {
            auto &e = P->evt_pool[i];
            float ms = 0.f;
            if (cudaEventSynchronize(e.b) == cudaSuccess && cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
                P->stage_ms[e.stage] += ms;
                P->stage_cnt[e.stage] += 1;
            }
        }
        P->evt_used = 0;
    }
};

}  // namespace cunusht

using namespace cunusht;

extern "C" {

const char *cunusht_last_error(void) { return g_err.c_str(); }

int cunusht_version(void) { return 100; }

int cunusht_plan_create(cunusht_plan_t **plan, int lmax, double epsilon, int precision, int max_spin, int nring,
                        const double *ring_theta, const double *ring_phi0, const int64_t *ring_nph,
                        const int64_t *ring_ofs) {
    clear_error();
    if (!plan) {
        set_error("plan output pointer is NULL");
        return CUNUSHT_ERR_ARG;
    }
    *plan = nullptr;
    cunusht_plan_s *P = new cunusht_plan_s();
    int rc = build_plan(P, lmax, epsilon, precision, max_spin, nring, ring_theta, ring_phi0, ring_nph, ring_ofs);
    if (rc != CUNUSHT_OK) {
        std::string keep = g_err;
        free_plan(P);
        g_err = keep;
        return rc;
    }
    *plan = P;
    return CUNUSHT_OK;
}

int cunusht_plan_destroy(cunusht_plan_t *plan) {
    clear_error();
    free_plan(plan);
    return CUNUSHT_OK;
}

int cunusht_plan_info(const cunusht_plan_t *P, int64_t *info, int ninfo) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(info != nullptr, "info array is NULL");
    const int64_t v[10] = {P->npix, P->Nt, P->Np, P->Ntf, P->Npf, P->w, P->nrows, (int64_t)P->ws_bytes,
                           P->prec, P->nalm};
    int n = std::min(ninfo, 10);
    for (int i = 0; i < n; ++i) info[i] = v[i];
    return n;
}

int cunusht_plan_set_mmax(cunusht_plan_t *P, int mmax) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(mmax >= 0 && mmax <= P->lmax, "mmax must be in [0, lmax = %d], got %d", P->lmax, mmax);
    P->mmax = mmax;
    P->nalm = (long long)(mmax + 1) * (mmax + 2) / 2 + (long long)(mmax + 1) * (P->lmax - mmax);
    return CUNUSHT_OK;
}

int cunusht_plan_force_split(cunusht_plan_t *P, int force) {
    clear_error();
    RC_TRY(check_plan(P));
    const int emax = 16 * FFT_TPB;
    P->sp_theta = (force || P->Ntf > emax) ? 2 : 1;
    P->sp_phi = (force || P->Npf > emax) ? 2 : 1;
    P->sp_ring = (force || P->Mb > emax) ? 2 : 1;
    P->ring_bluestein = force != 0;
    return CUNUSHT_OK;
}

int cunusht_plan_set_ring_transform(cunusht_plan_t *P, int method) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(method == 0 || method == 1, "ring transform method must be 0 (mixed radix where possible) or 1 "
              "(Bluestein), got %d", method);
    P->ring_bluestein = method == 1;
    return CUNUSHT_OK;
}

int cunusht_plan_ring_transform(const cunusht_plan_t *P) {
    if (!P) return -1;
    return ring_mr_available(P) ? 0 : 1;
}

int cunusht_plan_set_start_states(cunusht_plan_t *P, int grid, int spin, int enable) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(P->prec == CUNUSHT_PREC_MIXED, "start states belong to mixed-precision plans");
    ARG_CHECK(grid == 0 || grid == 1, "grid must be 0 (Gauss-Legendre pointing rings) or 1 (Clenshaw-Curtis), got %d",
              grid);
    const int smax = grid ? P->max_spin : std::max(P->max_spin, 1);
    ARG_CHECK(spin >= 0 && spin <= smax, "spin %d outside [0, %d] for this grid", spin, smax);
    return tc_start_states(P, grid, spin, enable != 0);
}

int cunusht_plan_set_tensor_cores(cunusht_plan_t *P, int enable) {
    clear_error();
    RC_TRY(check_plan(P));
    P->use_tc = enable != 0;
    return CUNUSHT_OK;
}

int cunusht_plan_device_status(cunusht_plan_t *P, int *status) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(status != nullptr, "status must not be NULL");
    CU_TRY(cudaDeviceSynchronize());
    int h = 0;
    CU_TRY(cudaMemcpy(&h, P->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    CU_TRY(cudaMemset(P->d_status, 0, sizeof(int)));
    *status = h;
    return CUNUSHT_OK;
}

int cunusht_tc_selftest(int n, int reps, int mode, double *maxerr, int *timeout) {
    clear_error();
    ARG_CHECK(maxerr != nullptr && timeout != nullptr, "maxerr and timeout must not be NULL");
    ARG_CHECK(n == 16 || n == 32 || n == 64, "n must be 16, 32 or 64, got %d", n);
    ARG_CHECK(reps >= 1 && reps <= 16, "reps must be in [1, 16], got %d", reps);
    ARG_CHECK(mode >= 0 && mode <= 6, "mode must be in [0, 6], got %d", mode);
    return tc_selftest(n, reps, mode, maxerr, timeout);
}

int cunusht_plan_set_profiling(cunusht_plan_t *P, int enable) {
    clear_error();
    RC_TRY(check_plan(P));
    if (enable && P->evt_pool.empty()) {
        P->evt_pool.resize(4096);
        for (auto &e : P->evt_pool) {
            CU_TRY(cudaEventCreate(&e.a));
            CU_TRY(cudaEventCreate(&e.b));
        }
    }
    P->profiling = enable != 0;
    return CUNUSHT_OK;
}

int cunusht_plan_stage_times(cunusht_plan_t *P, double *ms, int64_t *count, int nstage) {
    clear_error();
    RC_TRY(check_plan(P));
    StageScope::flush_events(P);
    for (int i = 0; i < CUNUSHT_NSTAGE; ++i) {
        if (i < nstage) {
            if (ms) ms[i] = P->stage_ms[i];
            if (count) count[i] = P->stage_cnt[i];
        }
        P->stage_ms[i] = 0.0;
        P->stage_cnt[i] = 0;
    }
    return CUNUSHT_OK;
}

static size_t f_elem(const cunusht_plan_s *P) { return P->grid_fp32 ? sizeof(float2) : 16; }
static size_t adj_scalar(const cunusht_plan_s *P) { return P->grid_fp32 ? sizeof(float) : sizeof(double); }

// workspace of the spreading options for max(batch capacity, 1) requests
static int spread_alloc(cunusht_plan_s *P) {
    if (P->d_bin || P->d_ufix) CU_TRY(cudaDeviceSynchronize());  // queued work may still use them
    if (P->d_bin) {
        cudaFree(P->d_bin);
        P->d_bin = nullptr;
    }
    if (P->d_ufix) {
        cudaFree(P->d_ufix);
        P->ws_bytes -= P->ufix_bytes;
        P->d_ufix = nullptr;
        P->ufix_bytes = 0;
    }
    const int nreq = P->batch_cap > 1 ? P->batch_cap : 1;
    if (P->spread_method == 1) RC_TRY(dalloc(P, &P->d_bin, (size_t)nreq * bin_workspace_ints(P, P->bin_npts)));
    if (P->spread_det) {
        const size_t n = (size_t)nreq * (P->max_spin ? 2 : 1) * P->nrows * P->Npf;
        RC_TRY(dalloc(P, &P->d_ufix, n));
        P->ufix_bytes = n * sizeof(unsigned long long);
        if (!P->d_vmax) RC_TRY(dalloc(P, &P->d_vmax, 64));
    }
    P->spread_nreq = nreq;
    return CUNUSHT_OK;
}

int cunusht_plan_set_spreading(cunusht_plan_t *P, int method, int deterministic, int64_t max_points) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(method == 0 || method == 1, "method must be 0 (warp strips) or 1 (bin-sorted), got %d", method);
    ARG_CHECK(deterministic == 0 || deterministic == 1, "deterministic must be 0 or 1");
    ARG_CHECK(max_points >= 0 && max_points < (1LL << 31), "max_points must be in [0, 2^31)");
    P->spread_method = method;
    P->spread_det = deterministic;
    P->bin_npts = max_points > 0 ? max_points : P->npix;
    return spread_alloc(P);
}

int cunusht_plan_reserve_batch(cunusht_plan_t *P, int max_batch) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(max_batch >= 1 && max_batch <= 64, "max_batch must be in [1, 64], got %d", max_batch);
    if (max_batch <= P->batch_cap) return CUNUSHT_OK;
    void *old[] = {P->d_Hb, P->d_Fb, P->d_Ub, P->d_ptgb, P->d_gamb};  // d_Hglb, d_glmapb are aliases
    CU_TRY(cudaDeviceSynchronize());
    for (void *q : old)
        if (q) cudaFree(q);
    P->d_Hb = nullptr;
    P->d_Fb = P->d_Ub = nullptr;
    P->ub_bytes = 0;
    P->d_Hglb = nullptr;
    P->d_glmapb = P->d_ptgb = P->d_gamb = nullptr;
    P->batch_cap = 0;
    const int L = P->lmax;
    const size_t B = max_batch;
    const size_t ncols = P->max_spin ? 2 * (size_t)L + 1 : (size_t)L + 1;
    char *f = nullptr, *u = nullptr;
    // The pointing's GL columns and maps are dead before the synthesis (adjoint)
    // writes the CC columns and the theta-pass rows, so they share memory:
    // d_Hglb lives in d_Hb and d_glmapb in d_Fb (lensing: Hglb, glmapb in the
    // pointing stages, then Hb, Fb; delensing: the pointing stages first, then
    // Fb from the phi adjoint on and Hb from the theta adjoint on).
    const size_t hb = std::max(ncols * P->ncc, (2 * (size_t)L + 1) * P->nring);      // double2 per request
    const size_t fb = std::max(f_elem(P) * ncols * P->nrows, 2 * sizeof(double) * (size_t)P->npix);  // bytes
    RC_TRY(dalloc(P, &P->d_Hb, B * hb));
    RC_TRY(dalloc(P, &f, B * fb));
    // sized for the adjoint (FP64 grid unless eps > 1e-6); the forward's FP32
    // grid uses the first half of each request's slot
    RC_TRY(dalloc(P, &u, B * adj_scalar(P) * (P->max_spin ? 2 : 1) * (size_t)P->nrows * P->Npf));
    P->d_Fb = f;
    P->d_Ub = u;
    P->ub_bytes = B * adj_scalar(P) * (P->max_spin ? 2 : 1) * (size_t)P->nrows * P->Npf;
    P->d_Hglb = P->d_Hb;
    P->d_glmapb = reinterpret_cast<double *>(f);
    RC_TRY(dalloc(P, &P->d_ptgb, B * 2 * (size_t)P->npix));
    RC_TRY(dalloc(P, &P->d_gamb, B * (size_t)P->npix));
    if (P->prec == CUNUSHT_PREC_MIXED) RC_TRY(tc_reserve(P, max_batch));
    P->batch_cap = max_batch;
    if (P->spread_method == 1 || P->spread_det) RC_TRY(spread_alloc(P));
    return CUNUSHT_OK;
}

int cunusht_lensing_batch(cunusht_plan_t *P, int nreq, int spin, int ncomp, const void *gclm,
                          const void *dlm_scaled, const void *dclm_scaled, double *ptg, double *gamma, void *out,
                          int out_dtype, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    RC_TRY(check_spin(P, spin, ncomp));
    ARG_CHECK(nreq >= 1, "nreq must be >= 1");
    ARG_CHECK(nreq <= P->batch_cap, "nreq %d exceeds the reserved batch capacity %d (cunusht_plan_reserve_batch)",
              nreq, P->batch_cap);
    ARG_CHECK(gclm && dlm_scaled && out, "NULL array argument");
    ARG_CHECK(out_dtype == CUNUSHT_F64 || out_dtype == CUNUSHT_F32, "bad out dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const int L = P->lmax;
    const long long npix = P->npix, nalm = P->nalm;
    const long long ncols = spin ? 2LL * L + 1 : (long long)L + 1;
    const long long hgl_s = (2LL * L + 1) * P->nring;
    double *ptg_b = ptg ? ptg : P->d_ptgb;
    double *gam_b = gamma ? gamma : (spin ? P->d_gamb : nullptr);
    // pointing of every request
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_LEG, st);
        RC_TRY(leg_synth_batch(P, nreq, 1, (const double2 *)dlm_scaled, (const double2 *)dclm_scaled, nalm, true,
                               false, P->d_Hglb, hgl_s, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_RING, st);
        RC_TRY(ring_synth_batch(P, nreq, 1, P->d_Hglb, hgl_s, P->d_glmapb, P->d_glmapb + npix, 2 * npix, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_ROT, st);
        RC_TRY(pointing_batch(P, nreq, P->d_glmapb, 2 * npix, ptg_b, 2 * npix, gam_b, st));
    }
    // synthesis at the deflected points
    const double2 *G = (const double2 *)gclm;
    const long long fs = (long long)P->nrows * ncols;
    const long long us = (long long)P->nrows * P->Npf;
    {
        StageScope sc(P, CUNUSHT_STAGE_LEG_SYNTH, st);
        RC_TRY(leg_synth_batch(P, nreq, spin, G, ncomp > 1 ? G + nalm : nullptr, ncomp * nalm, false, true, P->d_Hb,
                               ncols * P->ncc, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_THETA_FWD, st);
        RC_TRY(theta_fwd_batch(P, nreq, spin, P->d_Hb, ncols * P->ncc, P->d_Fb, fs, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_PHI_FWD, st);
        RC_TRY(phi_fwd_batch(P, nreq, spin, P->d_Fb, fs, P->d_Ub, us, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_INTERP, st);
        RC_TRY(nufft_interp_batch(P, nreq, spin, P->d_Ub, (spin ? 2 : 1) * us, ptg_b, 2 * npix, npix, 1, gam_b, out,
                                  (spin ? 2 : 1) * npix, out_dtype, st));
    }
    return CUNUSHT_OK;
}

int cunusht_delensing_batch(cunusht_plan_t *P, int nreq, int spin, int ncomp, const void *lenmap, int map_dtype,
                            const void *dlm_scaled, const void *dclm_scaled, double *ptg, double *gamma,
                            void *alm_out, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    RC_TRY(check_spin(P, spin, ncomp));
    ARG_CHECK(nreq >= 1, "nreq must be >= 1");
    ARG_CHECK(nreq <= P->batch_cap, "nreq %d exceeds the reserved batch capacity %d (cunusht_plan_reserve_batch)",
              nreq, P->batch_cap);
    ARG_CHECK(lenmap && dlm_scaled && alm_out, "NULL array argument");
    ARG_CHECK(map_dtype == CUNUSHT_F64 || map_dtype == CUNUSHT_F32, "bad map dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const int L = P->lmax;
    const long long npix = P->npix, nalm = P->nalm;
    const long long ncols = spin ? 2LL * L + 1 : (long long)L + 1;
    const long long hgl_s = (2LL * L + 1) * P->nring;
    double *ptg_b = ptg ? ptg : P->d_ptgb;
    double *gam_b = gamma ? gamma : (spin ? P->d_gamb : nullptr);
    // pointing of every request (shared recursion on the mixed path)
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_LEG, st);
        RC_TRY(leg_synth_batch(P, nreq, 1, (const double2 *)dlm_scaled, (const double2 *)dclm_scaled, nalm, true,
                               false, P->d_Hglb, hgl_s, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_RING, st);
        RC_TRY(ring_synth_batch(P, nreq, 1, P->d_Hglb, hgl_s, P->d_glmapb, P->d_glmapb + npix, 2 * npix, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_ROT, st);
        RC_TRY(pointing_batch(P, nreq, P->d_glmapb, 2 * npix, ptg_b, 2 * npix, gam_b, st));
    }
    // adjoint nuFFT and adjoint SHT at the deflected points
    const long long us = (spin ? 2LL : 1LL) * P->nrows * P->Npf;  // grid scalars per request
    const long long fs = (long long)P->nrows * ncols;
    {
        StageScope sc(P, CUNUSHT_STAGE_SPREAD, st);
        RC_TRY(nufft_spread_batch(P, nreq, spin, P->d_Ub, us, ptg_b, 2 * npix, npix, 1, gam_b, lenmap,
                                  (spin ? 2 : 1) * npix, map_dtype, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_PHI_ADJ, st);
        RC_TRY(phi_adj_batch(P, nreq, spin, P->d_Ub, us, P->d_Fb, fs, st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_THETA_ADJ, st);
        RC_TRY(theta_adj_batch(P, nreq, spin, P->d_Fb, fs, P->d_Hb, ncols * P->ncc, P->d_Ub,
                               us * (long long)adj_scalar(P), st));
    }
    {
        StageScope sc(P, CUNUSHT_STAGE_LEG_ADJ, st);
        double2 *G = (double2 *)alm_out;
        // the fine grids are free once the theta pass is done: the tensor-core
        // adjoint keeps its fixed-point sums there
        RC_TRY(leg_adjoint_batch(P, nreq, spin, ncomp, P->d_Hb, ncols * P->ncc, false, true, G, G + nalm,
                                 ncomp * nalm, st, P->d_Ub, P->ub_bytes));
    }
    return CUNUSHT_OK;
}

int cunusht_nusht2d2(cunusht_plan_t *P, int spin, int ncomp, const void *alm, int alm_dtype, const double *loc,
                     int64_t npts, int loc_layout, const double *gamma, void *out, int out_dtype, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    RC_TRY(check_spin(P, spin, ncomp));
    ARG_CHECK(alm && out && (loc || npts == 0), "NULL array argument");
    ARG_CHECK(npts >= 0, "npts must be >= 0");
    ARG_CHECK(loc_layout == 0 || loc_layout == 1, "loc_layout must be 0 or 1");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    ARG_CHECK(out_dtype == CUNUSHT_F64 || out_dtype == CUNUSHT_F32, "bad out dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const double2 *G, *C = nullptr;
    if (alm_dtype == CUNUSHT_F64) {
        G = (const double2 *)alm;
        if (ncomp > 1) C = G + P->nalm;
    } else {
        RC_TRY(convert_alm(alm, alm_dtype, ncomp * P->nalm, P->d_alm, st));
        G = P->d_alm;
        if (ncomp > 1) C = P->d_alm + P->nalm;
    }
    { StageScope sc(P, CUNUSHT_STAGE_LEG_SYNTH, st); RC_TRY(leg_synth(P, spin, G, C, false, true, P->d_H, st)); }
    { StageScope sc(P, CUNUSHT_STAGE_THETA_FWD, st); RC_TRY(theta_fwd(P, spin, P->d_H, P->d_F, st)); }
    { StageScope sc(P, CUNUSHT_STAGE_PHI_FWD, st); RC_TRY(phi_fwd(P, spin, P->d_F, P->d_U, st)); }
    { StageScope sc(P, CUNUSHT_STAGE_INTERP, st); RC_TRY(nufft_interp(P, spin, loc, npts, loc_layout, spin ? gamma : nullptr, out, out_dtype, st)); }
    return CUNUSHT_OK;
}

int cunusht_nusht2d1(cunusht_plan_t *P, int spin, int ncomp, const void *map, int map_dtype, const double *loc,
                     int64_t npts, int loc_layout, const double *gamma, void *alm_out, int alm_dtype,
                     void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    RC_TRY(check_spin(P, spin, ncomp));
    ARG_CHECK(alm_out && (map || npts == 0) && (loc || npts == 0), "NULL array argument");
    ARG_CHECK(npts >= 0, "npts must be >= 0");
    ARG_CHECK(loc_layout == 0 || loc_layout == 1, "loc_layout must be 0 or 1");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    ARG_CHECK(map_dtype == CUNUSHT_F64 || map_dtype == CUNUSHT_F32, "bad map dtype");
    cudaStream_t st = (cudaStream_t)stream;
    { StageScope sc(P, CUNUSHT_STAGE_SPREAD, st); RC_TRY(nufft_spread(P, spin, loc, npts, loc_layout, spin ? gamma : nullptr, map, map_dtype, st)); }
    { StageScope sc(P, CUNUSHT_STAGE_PHI_ADJ, st); RC_TRY(phi_adj(P, spin, P->d_U, P->d_F, st)); }
    { StageScope sc(P, CUNUSHT_STAGE_THETA_ADJ, st); RC_TRY(theta_adj(P, spin, P->d_F, P->d_H, st)); }
    double2 *G = alm_dtype == CUNUSHT_F64 ? (double2 *)alm_out : P->d_alm;
    double2 *C = G + P->nalm;
    { StageScope sc(P, CUNUSHT_STAGE_LEG_ADJ, st); RC_TRY(leg_adjoint(P, spin, ncomp, P->d_H, false, true, G, C, st, P->d_U, P->u_bytes)); }
    if (alm_dtype != CUNUSHT_F64) RC_TRY(store_alm(P->d_alm, ncomp * P->nalm, alm_dtype, alm_out, st));
    return CUNUSHT_OK;
}

int cunusht_dlm2pointing(cunusht_plan_t *P, const void *dlm, const void *dclm, int alm_dtype, double *ptg,
                         double *gamma, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(dlm && ptg, "NULL array argument");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const double2 *G = (const double2 *)dlm, *C = (const double2 *)dclm;
    if (alm_dtype != CUNUSHT_F64) {
        RC_TRY(convert_alm(dlm, alm_dtype, P->nalm, P->d_alm, st));
        G = P->d_alm;
        if (dclm) {
            RC_TRY(convert_alm(dclm, alm_dtype, P->nalm, P->d_alm + P->nalm, st));
            C = P->d_alm + P->nalm;
        }
    }
    { StageScope sc(P, CUNUSHT_STAGE_PTG_LEG, st); RC_TRY(leg_synth(P, 1, G, C, true, false, P->d_Hgl, st)); }
    { StageScope sc(P, CUNUSHT_STAGE_PTG_RING, st); RC_TRY(ring_synth(P, 1, P->d_Hgl, P->d_glmap, P->d_glmap + P->npix, st)); }
    {
        StageScope sc(P, CUNUSHT_STAGE_PTG_ROT, st);
        if (P->prec == CUNUSHT_PREC_MIXED)
            RC_TRY(pointing_mixed_launch(P->nring, P->nph_uniform, P->d_ring_theta, P->d_ring_sc, P->d_ring_phi0,
                                         P->d_ring_nph,
                                         P->d_ring_ofs, P->npix, P->d_glmap, P->d_glmap + P->npix, ptg,
                                         ptg + P->npix, gamma, st));
        else
            RC_TRY(pointing_launch(P->nring, P->d_ring_theta, P->d_ring_phi0, P->d_ring_nph, P->d_ring_ofs,
                                   P->npix, P->d_glmap, P->d_glmap + P->npix, ptg, ptg + P->npix, gamma, st));
    }
    return CUNUSHT_OK;
}

int cunusht_dlm2A(cunusht_plan_t *P, const void *dlm, const void *dclm, int alm_dtype, double *A, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(dlm && A, "NULL array argument");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const double2 *G = (const double2 *)dlm, *C = (const double2 *)dclm;
    if (alm_dtype != CUNUSHT_F64) {
        RC_TRY(convert_alm(dlm, alm_dtype, P->nalm, P->d_alm, st));
        G = P->d_alm;
        if (dclm) {
            RC_TRY(convert_alm(dclm, alm_dtype, P->nalm, P->d_alm + P->nalm, st));
            C = P->d_alm + P->nalm;
        }
    }
    const long long npix = P->npix;
    double *d1 = P->d_vjp, *d2 = P->d_vjp + npix, *g1 = P->d_vjp + 2 * npix, *g2 = P->d_vjp + 3 * npix;
    double *kp = P->d_glmap, *wp = dclm ? P->d_glmap + npix : nullptr;
    // deflection (spin 1 of dlm, dclm)
    RC_TRY(leg_synth_batch_fl(P, 1, 1, G, C, 0, nullptr, false, P->d_Hgl, 0, st));
    RC_TRY(ring_synth(P, 1, P->d_Hgl, d1, d2, st));
    // convergence: spin 0 of sqrt(l(l+1)) dlm (x 1/2 in the determinant kernel)
    RC_TRY(leg_synth_batch_fl(P, 1, 0, G, nullptr, 0, P->d_lfac, false, P->d_Hgl, 0, st));
    RC_TRY(ring_synth(P, 0, P->d_Hgl, kp, nullptr, st));
    // shear: spin 2 of sqrt((l-1)(l+2)) (dlm, dclm) (x -1/2)
    RC_TRY(leg_synth_batch_fl(P, 1, 2, G, C, 0, P->d_lfac_g, false, P->d_Hgl, 0, st));
    RC_TRY(ring_synth(P, 2, P->d_Hgl, g1, g2, st));
    if (dclm) {  // rotation: spin 0 of sqrt(l(l+1)) dclm (x 1/2)
        RC_TRY(leg_synth_batch_fl(P, 1, 0, C, nullptr, 0, P->d_lfac, false, P->d_Hgl, 0, st));
        RC_TRY(ring_synth(P, 0, P->d_Hgl, wp, nullptr, st));
    }
    return magnification_det(npix, kp, g1, g2, d1, d2, wp, A, st);
}

int cunusht_synth_points(cunusht_plan_t *P, int spin, int ncomp, const void *alm, int alm_dtype, const double *loc,
                         int64_t npts, int loc_layout, const double *gamma, double *out, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(spin >= 0 && spin <= 2, "spin must be 0, 1 or 2, got %d", spin);
    if (spin == 0) ARG_CHECK(ncomp == 1, "spin 0 takes ncomp = 1, got %d", ncomp);
    else ARG_CHECK(ncomp == 1 || ncomp == 2, "spin %d takes ncomp 1 or 2, got %d", spin, ncomp);
    ARG_CHECK(alm && out && (loc || npts == 0), "NULL array argument");
    ARG_CHECK(npts >= 0 && npts < (int64_t)1 << 31, "npts must be in [0, 2^31)");
    ARG_CHECK(loc_layout == 0 || loc_layout == 1, "loc_layout must be 0 or 1");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const double2 *G = (const double2 *)alm;
    if (alm_dtype != CUNUSHT_F64) {
        RC_TRY(convert_alm(alm, alm_dtype, ncomp * P->nalm, P->d_alm, st));
        G = P->d_alm;
    }
    const double2 *C = (spin > 0 && ncomp > 1) ? G + P->nalm : nullptr;
    return synth_points(P, spin, G, C, npts, loc, loc_layout, spin ? gamma : nullptr, out, st);
}

int cunusht_lensing_vjp_dlm(cunusht_plan_t *P, int spin, const void *gclm, int alm_dtype, const void *dlm_scaled,
                            int dlm_dtype, const double *grad_map, void *grad_dlm, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(gclm && dlm_scaled && grad_map && grad_dlm, "NULL array argument");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    ARG_CHECK(dlm_dtype == CUNUSHT_F64 || dlm_dtype == CUNUSHT_F32, "bad dlm dtype");
    if (spin != 0) {
        set_error("lensing VJP with respect to the deflection is implemented for spin 0 only");
        return CUNUSHT_ERR_UNSUPPORTED;
    }
    cudaStream_t st = (cudaStream_t)stream;
    double *ptg = P->d_vjp, *gd = P->d_vjp + 2 * P->npix;
    // deflection (kept in d_glmap) and deflected angles
    const double2 *D = (const double2 *)dlm_scaled;
    if (dlm_dtype != CUNUSHT_F64) {
        RC_TRY(convert_alm(dlm_scaled, dlm_dtype, P->nalm, P->d_alm + P->nalm, st));
        D = P->d_alm + P->nalm;
    }
    RC_TRY(leg_synth(P, 1, D, nullptr, true, false, P->d_Hgl, st));
    RC_TRY(ring_synth(P, 1, P->d_Hgl, P->d_glmap, P->d_glmap + P->npix, st));
    RC_TRY(pointing_launch(P->nring, P->d_ring_theta, P->d_ring_phi0, P->d_ring_nph, P->d_ring_ofs, P->npix,
                           P->d_glmap, P->d_glmap + P->npix, ptg, ptg + P->npix, nullptr, st));
    // fine grid of the unlensed field
    const double2 *G = (const double2 *)gclm;
    if (alm_dtype != CUNUSHT_F64) {
        RC_TRY(convert_alm(gclm, alm_dtype, P->nalm, P->d_alm, st));
        G = P->d_alm;
    }
    RC_TRY(leg_synth(P, 0, G, nullptr, false, true, P->d_H, st));
    RC_TRY(theta_fwd(P, 0, P->d_H, P->d_F, st));
    RC_TRY(phi_fwd(P, 0, P->d_F, P->d_U, st));
    // per-pixel pull-back, then the adjoint spin-1 synthesis (scaled by sqrt(l(l+1)))
    RC_TRY(lens_vjp_launch(P, ptg, grad_map, gd, st));
    RC_TRY(ring_adjoint(P, 1, gd, gd + P->npix, P->d_Hgl, st));
    RC_TRY(leg_adjoint(P, 1, 1, P->d_Hgl, true, false, (double2 *)grad_dlm, nullptr, st, P->d_U, P->u_bytes));
    return CUNUSHT_OK;
}

int cunusht_synthesis(cunusht_plan_t *P, int spin, int ncomp, const void *alm, int alm_dtype, double *map,
                      void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(spin >= 0 && spin <= 2, "spin must be 0, 1 or 2");
    if (spin == 0) ARG_CHECK(ncomp == 1, "spin 0 takes ncomp = 1");
    else ARG_CHECK(ncomp == 1 || ncomp == 2, "spin > 0 takes ncomp 1 or 2");
    ARG_CHECK(alm && map, "NULL array argument");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    cudaStream_t st = (cudaStream_t)stream;
    const double2 *G = (const double2 *)alm, *C = nullptr;
    if (alm_dtype != CUNUSHT_F64) {
        RC_TRY(convert_alm(alm, alm_dtype, ncomp * P->nalm, P->d_alm, st));
        G = P->d_alm;
    }
    if (ncomp > 1) C = G + P->nalm;
    RC_TRY(leg_synth(P, spin, G, C, false, false, P->d_Hgl, st));
    RC_TRY(ring_synth(P, spin, P->d_Hgl, map, spin ? map + P->npix : nullptr, st));
    return CUNUSHT_OK;
}

int cunusht_adjoint_synthesis(cunusht_plan_t *P, int spin, int ncomp, const double *map, void *alm_out,
                              int alm_dtype, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(spin >= 0 && spin <= 2, "spin must be 0, 1 or 2");
    if (spin == 0) ARG_CHECK(ncomp == 1, "spin 0 takes ncomp = 1");
    else ARG_CHECK(ncomp == 1 || ncomp == 2, "spin > 0 takes ncomp 1 or 2");
    ARG_CHECK(alm_out && map, "NULL array argument");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    cudaStream_t st = (cudaStream_t)stream;
    RC_TRY(ring_adjoint(P, spin, map, spin ? map + P->npix : nullptr, P->d_Hgl, st));
    double2 *G = alm_dtype == CUNUSHT_F64 ? (double2 *)alm_out : P->d_alm;
    RC_TRY(leg_adjoint(P, spin, ncomp, P->d_Hgl, false, false, G, G + P->nalm, st, P->d_U, P->u_bytes));
    if (alm_dtype != CUNUSHT_F64) RC_TRY(store_alm(P->d_alm, ncomp * P->nalm, alm_dtype, alm_out, st));
    return CUNUSHT_OK;
}

int cunusht_analysis(cunusht_plan_t *P, int spin, int ncomp, const double *map, const double *ring_weight,
                     void *alm_out, int alm_dtype, void *stream) {
    clear_error();
    RC_TRY(check_plan(P));
    ARG_CHECK(spin >= 0 && spin <= 2, "spin must be 0, 1 or 2");
    if (spin == 0) ARG_CHECK(ncomp == 1, "spin 0 takes ncomp = 1");
    else ARG_CHECK(ncomp == 1 || ncomp == 2, "spin > 0 takes ncomp 1 or 2");
    ARG_CHECK(alm_out && map && ring_weight, "NULL array argument");
    ARG_CHECK(alm_dtype == CUNUSHT_F64 || alm_dtype == CUNUSHT_F32, "bad alm dtype");
    cudaStream_t st = (cudaStream_t)stream;
    RC_TRY(ring_adjoint(P, spin, map, spin ? map + P->npix : nullptr, P->d_Hgl, st, ring_weight));
    double2 *G = alm_dtype == CUNUSHT_F64 ? (double2 *)alm_out : P->d_alm;
    RC_TRY(leg_adjoint(P, spin, ncomp, P->d_Hgl, false, false, G, G + P->nalm, st, P->d_U, P->u_bytes));
    if (alm_dtype != CUNUSHT_F64) RC_TRY(store_alm(P->d_alm, ncomp * P->nalm, alm_dtype, alm_out, st));
    return CUNUSHT_OK;
}

int cunusht_pointing(int nring, const double *ring_theta, const double *ring_phi0, const int64_t *ring_nph,
                     const int64_t *ring_ofs, int64_t npix, const double *s1t, const double *s1p, double *ot,
                     double *op, double *og, void *stream) {
    clear_error();
    ARG_CHECK(nring >= 1 && ring_theta && ring_phi0 && ring_nph && ring_ofs, "ring tables missing");
    ARG_CHECK(s1t && s1p && ot && op, "NULL array argument");
    ARG_CHECK(npix >= 0, "npix must be >= 0");
    return pointing_launch(nring, ring_theta, ring_phi0, (const long long *)ring_nph, (const long long *)ring_ofs,
                           npix, s1t, s1p, ot, op, og, (cudaStream_t)stream);
}

int cunusht_doubling(const void *cc_map, int64_t ntheta, int64_t nphi, int layout, int spin, int dtype, void *out,
                     void *stream) {
    clear_error();
    ARG_CHECK(cc_map && out, "NULL array argument");
    ARG_CHECK(ntheta >= 2 && nphi >= 2 && nphi % 2 == 0, "need ntheta >= 2 and even nphi >= 2");
    ARG_CHECK(layout == 0 || layout == 1, "layout must be 0 (ring-major) or 1 (theta-contiguous)");
    ARG_CHECK(dtype == CUNUSHT_F64 || dtype == CUNUSHT_F32, "bad dtype");
    return doubling_launch(cc_map, ntheta, nphi, layout, spin, dtype, out, (cudaStream_t)stream);
}

int cunusht_adjoint_doubling(const void *dmap, int64_t ntheta, int64_t nphi, int spin, int dtype, void *out,
                             void *stream) {
    clear_error();
    ARG_CHECK(dmap && out, "NULL array argument");
    ARG_CHECK(ntheta >= 2 && nphi >= 2 && nphi % 2 == 0, "need ntheta >= 2 and even nphi >= 2");
    ARG_CHECK(dtype == CUNUSHT_F64 || dtype == CUNUSHT_F32, "bad dtype");
    return adjoint_doubling_launch(dmap, ntheta, nphi, spin, dtype, out, (cudaStream_t)stream);
}

}  // extern "C"

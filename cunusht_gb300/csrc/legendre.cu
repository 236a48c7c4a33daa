// Legendre stage of the spin-s spherical harmonic transform on iso-latitude
// ring sets, FP64 (plain path).
//
// Replaces the SHTns calls of the reference: ``synth`` on the Clenshaw-Curtis
// grid (cunusht/sht/GPU_sht_transformer.py:56-62), ``analys(map*iw)`` as the
// adjoint (:65-73) and ``synth_grad`` on the Gauss-Legendre grid (:88-97).
//
// Per order m and ring theta the kernels evaluate
//     h_m(theta)  = sum_l a_lm  sLambda_lm(theta)             (synthesis)
//     a'_lm       = sum_rings   sLambda_lm(theta_r) h'_m(r)    (adjoint)
// with the normalised Wigner-d three-term recursion in l
//     sLambda_{l+1} = (alpha_l x + gamma_l) sLambda_l - beta_l sLambda_{l-1},
// started at l0 = max(m, s) from the closed form
//     sLambda_{l0,m} = (-1)^m 2^{lg0[m]} sin^{m+s}(theta/2) cos^{|m-s|}(theta/2),
// which is regular at both poles.  The start is kept as mantissa x 2^e with
// e a non-positive multiple of 512 so that sin^m never underflows; values are
// accumulated only once e has climbed back to 0 (before that they are below
// 2^-312 and cannot contribute).
//
// Rings come in pairs (theta, pi - theta): spin 0 uses the parity
// Lambda_lm(pi - theta) = (-1)^{l+m} Lambda_lm(theta) (one recursion per pair);
// spin s > 0 runs the recursion at both rings and gets the (-s) functions from
// -sLambda_lm(theta) = (-1)^{l+m} sLambda_lm(pi - theta).
//
// Output layout: H[c][ring], c = m (spin 0) or c = m + lmax (spin s, m in
// [-lmax, lmax]), rings contiguous (ldH = ring count).
#include "common.cuh"
#include "df.cuh"
#include "kernels.cuh"

namespace cunusht {

__device__ __forceinline__ void rec_start(double lg0, int m, int s, double sh, double ch,
                                          double &cur, double &prev, int &e) {
    prev = 0.0;
    double lg = lg0;
    bool zero = false;
    if (m + s > 0) {
        if (sh <= 0.0) zero = true;
        else lg += (double)(m + s) * log2(sh);
    }
    if (m != s) {
        if (ch <= 0.0) zero = true;
        else lg += (double)abs(m - s) * log2(ch);
    }
    if (zero) {
        cur = 0.0;
        e = 0;
        return;
    }
    int k = 0;
    if (lg < -400.0) k = (int)ceil((-400.0 - lg) / 512.0);
    e = -512 * k;
    cur = exp2(lg + 512.0 * (double)k);
    if (m & 1) cur = -cur;
}

#define REC_RESCALE(cur, prev, e)                                                        \
    if ((e) < 0 && fabs(cur) > 0x1p200) {                                               \
        (cur) *= 0x1p-512;                                                               \
        (prev) *= 0x1p-512;                                                              \
        (e) += 512;                                                                      \
    }

// ---------------------------------------------------------------- tables
__global__ void k_build_coef(int L, int s, double *__restrict__ coef, long long nalm) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nalm) return;
    int lo = 0, hi = L;
    while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        if (almidx(L, mid, mid) <= idx) lo = mid;
        else hi = mid - 1;
    }
    const int m = lo;
    const int l = m + (int)(idx - almidx(L, m, m));
    const int l0 = max(m, s);
    double al = 0.0, ga = 0.0, be = 0.0;
    if (l >= l0 && l < L) {
        const double lp = l + 1.0, dm = m, ds = s, dl = l;
        const double den = sqrt((lp * lp - dm * dm) * (lp * lp - ds * ds));
        al = lp * sqrt((2.0 * dl + 1.0) * (2.0 * dl + 3.0)) / den;
        if (l > 0) {
            ga = al * (dm * ds / (dl * lp));
            be = (lp / dl) * sqrt((dl * dl - dm * dm) * (dl * dl - ds * ds)) / den *
                 sqrt((2.0 * dl + 3.0) / (2.0 * dl - 1.0));
        }
    }
    coef[idx] = al;
    coef[nalm + idx] = ga;
    coef[2 * nalm + idx] = be;
}

int build_coef_tables(cunusht_plan_s *P, cudaStream_t st) {
    for (int s = 0; s <= 2; ++s) {
        int nb = (int)((P->nalm_tab + 255) / 256);
        k_build_coef<<<nb, 256, 0, st>>>(P->lmax, s, P->d_coef[s], P->nalm_tab);
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int build_coef_tables_spin(const cunusht_plan_s *P, int spin, double *coef, cudaStream_t st) {
    const int nb = (int)((P->nalm_tab + 255) / 256);
    k_build_coef<<<nb, 256, 0, st>>>(P->lmax, spin, coef, P->nalm_tab);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// ---------------------------------------------------------------- synthesis, spin 0
constexpr int LEG_TPB = 128;
constexpr int LEG_CH = 128;

__global__ void __launch_bounds__(LEG_TPB)
    k_leg_synth_s0(int L, const double2 *__restrict__ alm, const double *__restrict__ lfac,
                   const double *__restrict__ coef, long long nalm, const double *__restrict__ lg0,
                   int npairs, const double *__restrict__ px, const double *__restrict__ psh,
                   const double *__restrict__ pch, const int *__restrict__ prn,
                   const int *__restrict__ prs, double2 *__restrict__ H, int ldH) {
    __shared__ double s_al[LEG_CH], s_be[LEG_CH];
    __shared__ double2 s_a[LEG_CH];
    const int m = blockIdx.y;
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
    }
    double cur, prev;
    int e;
    rec_start(lg0[m], m, 0, sh, ch, cur, prev, e);
    double Er = 0.0, Ei = 0.0, Or = 0.0, Oi = 0.0;
    const double *al = coef, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;  // (l, m) at b + l
    for (int lb = m; lb <= L; lb += LEG_CH) {
        const int cnt = min(LEG_CH, L - lb + 1);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += LEG_TPB) {
            const long long ix = b + lb + i;
            s_al[i] = al[ix];
            s_be[i] = be[ix];
            double2 a = alm[ix];
            const double f = lfac ? lfac[lb + i] : 1.0;
            s_a[i] = make_double2(a.x * f, a.y * f);
        }
        __syncthreads();
        for (int i = 0; i < cnt; ++i) {
            if (e == 0) {
                const double2 a = s_a[i];
                if ((lb + i + m) & 1) {
                    Or = fma(a.x, cur, Or);
                    Oi = fma(a.y, cur, Oi);
                } else {
                    Er = fma(a.x, cur, Er);
                    Ei = fma(a.y, cur, Ei);
                }
            }
            const double nxt = fma(s_al[i] * x, cur, -s_be[i] * prev);
            prev = cur;
            cur = nxt;
            REC_RESCALE(cur, prev, e);
        }
    }
    if (act) {
        const int n = prn[p], s = prs[p];
        H[(long long)m * ldH + n] = make_double2(Er + Or, Ei + Oi);
        if (s != n) H[(long long)m * ldH + s] = make_double2(Er - Or, Ei - Oi);
    }
}

// ---------------------------------------------------------------- synthesis, spin s > 0
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_synth_spin(int L, int spin, const double2 *__restrict__ G, const double2 *__restrict__ C,
                     const double *__restrict__ lfac, const double *__restrict__ coef,
                     long long nalm, const double *__restrict__ lg0, int npairs,
                     const double *__restrict__ px, const double *__restrict__ psh,
                     const double *__restrict__ pch, const int *__restrict__ prn,
                     const int *__restrict__ prs, double2 *__restrict__ H, int ldH) {
    __shared__ double s_al[LEG_CH], s_ga[LEG_CH], s_be[LEG_CH];
    __shared__ double2 s_A[LEG_CH], s_B[LEG_CH];
    const int m = blockIdx.y;
    const int l0 = max(m, spin);
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
    }
    double cN, pN, cS, pS;
    int eN, eS;
    rec_start(lg0[m], m, spin, sh, ch, cN, pN, eN);  // ring theta
    rec_start(lg0[m], m, spin, ch, sh, cS, pS, eS);  // ring pi - theta
    double2 hpn = make_double2(0, 0), hps = hpn, hmn = hpn, hms = hpn;
    const double *al = coef, *ga = coef + nalm, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    for (int lb = l0; lb <= L; lb += LEG_CH) {
        const int cnt = min(LEG_CH, L - lb + 1);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += LEG_TPB) {
            const int l = lb + i;
            const long long ix = b + l;
            s_al[i] = al[ix];
            s_ga[i] = ga[ix];
            s_be[i] = be[ix];
            const double f = lfac ? lfac[l] : 1.0;
            const double2 g = G[ix];
            const double2 c = C ? C[ix] : make_double2(0.0, 0.0);
            // A = G + iC ; B = (conj G + i conj C) (-1)^{l+m}
            s_A[i] = make_double2(f * (g.x - c.y), f * (g.y + c.x));
            const double par = ((l + m) & 1) ? -f : f;
            s_B[i] = make_double2(par * (g.x + c.y), par * (c.x - g.y));
        }
        __syncthreads();
        for (int i = 0; i < cnt; ++i) {
            const double2 A = s_A[i], B = s_B[i];
            if (eN == 0) {
                hpn.x = fma(A.x, cN, hpn.x);
                hpn.y = fma(A.y, cN, hpn.y);
                hms.x = fma(B.x, cN, hms.x);
                hms.y = fma(B.y, cN, hms.y);
            }
            if (eS == 0) {
                hps.x = fma(A.x, cS, hps.x);
                hps.y = fma(A.y, cS, hps.y);
                hmn.x = fma(B.x, cS, hmn.x);
                hmn.y = fma(B.y, cS, hmn.y);
            }
            const double a_ = s_al[i], g_ = s_ga[i], b_ = s_be[i];
            const double nN = fma(fma(a_, x, g_), cN, -b_ * pN);
            const double nS = fma(fma(a_, -x, g_), cS, -b_ * pS);
            pN = cN;
            cN = nN;
            pS = cS;
            cS = nS;
            REC_RESCALE(cN, pN, eN);
            REC_RESCALE(cS, pS, eS);
        }
    }
    if (act) {
        const int n = prn[p], s = prs[p];
        const double sgs = (spin & 1) ? -1.0 : 1.0;
        H[(long long)(L + m) * ldH + n] = make_double2(-hpn.x, -hpn.y);
        if (s != n) H[(long long)(L + m) * ldH + s] = make_double2(-hps.x, -hps.y);
        if (m > 0) {
            H[(long long)(L - m) * ldH + n] = make_double2(-sgs * hmn.x, -sgs * hmn.y);
            if (s != n) H[(long long)(L - m) * ldH + s] = make_double2(-sgs * hms.x, -sgs * hms.y);
        }
    }
}

// ---------------------------------------------------------------- mixed precision synthesis
// Same recursion and accumulation pattern as the FP64 kernels, with the
// recursion in double-float (FP32 hi/lo, ~48 bits) and each product a_lm * lam
// formed from the hi/lo parts, rounded once to FP32 and added with Kahan
// compensation.  The start mantissa is kept in FP32 range with an exponent in
// steps of 96 (values below 2^-56 are not accumulated).
__global__ void k_split_coef(const double *__restrict__ c, long long n, float2 *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = c[i];
    const float h = (float)v;
    out[i] = make_float2(h, (float)(v - (double)h));
}

int build_coef_tables_df(cunusht_plan_s *P, cudaStream_t st) {
    for (int s = 0; s <= 2; ++s) {
        const long long n = 3 * P->nalm_tab;
        k_split_coef<<<(int)((n + 255) / 256), 256, 0, st>>>(P->d_coef[s], n, P->d_coef_df[s]);
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

// NB requests per launch share the recursion: request r reads its alm at
// alm + r * astride and writes its columns at H + r * hstride.
template <int NB>
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_synth_s0_df(int L, const double2 *__restrict__ alm, long long astride, const double *__restrict__ lfac,
                      const float2 *__restrict__ coef, long long nalm, const double *__restrict__ lg0,
                      int npairs, const double *__restrict__ px, const double *__restrict__ psh,
                      const double *__restrict__ pch, const int *__restrict__ prn,
                      const int *__restrict__ prs, double2 *__restrict__ H, long long hstride, int ldH) {
    __shared__ float2 s_al[LEG_CH], s_be[LEG_CH];
    __shared__ float4 s_a[NB][LEG_CH];
    const int m = blockIdx.y;
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
    }
    const dfl xd = df_from(x);
    dfl cur, prev;
    int e;
    rec_start_df(lg0[m], m, 0, sh, ch, cur, prev, e);
    kahan Er[NB], Ei[NB], Or[NB], Oi[NB];
    const float2 *al = coef, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    for (int lb = m; lb <= L; lb += LEG_CH) {
        const int cnt = min(LEG_CH, L - lb + 1);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += LEG_TPB) {
            const long long ix = b + lb + i;
            s_al[i] = al[ix];
            s_be[i] = be[ix];
            const double f = lfac ? lfac[lb + i] : 1.0;
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                const double2 a = alm[r * astride + ix];
                const dfl re = df_from(a.x * f), im = df_from(a.y * f);
                s_a[r][i] = make_float4(re.h, re.l, im.h, im.l);
            }
        }
        __syncthreads();
        for (int i = 0; i < cnt; ++i) {
            if (e == 0) {
                const bool odd = (lb + i + m) & 1;
#pragma unroll
                for (int r = 0; r < NB; ++r) {
                    const float4 a = s_a[r][i];
                    const float pr = df_prod(a.x, a.y, cur), pi = df_prod(a.z, a.w, cur);
                    if (odd) {
                        Or[r].add(pr);
                        Oi[r].add(pi);
                    } else {
                        Er[r].add(pr);
                        Ei[r].add(pi);
                    }
                }
            }
            const float2 a2 = s_al[i], b2 = s_be[i];
            const dfl t = df_mul_u(dfl{a2.x, a2.y}, xd);
            const dfl nxt = df_mul_sub(t, cur, dfl{b2.x, b2.y}, prev);
            prev = cur;
            cur = nxt;
            REC_RESCALE_DF(cur, prev, e);
        }
    }
    if (act) {
        const int n = prn[p], s = prs[p];
#pragma unroll
        for (int r = 0; r < NB; ++r) {
            double2 *Hr = H + r * hstride;
            const double er = Er[r].value(), ei = Ei[r].value(), orr = Or[r].value(), oi = Oi[r].value();
            Hr[(long long)m * ldH + n] = make_double2(er + orr, ei + oi);
            if (s != n) Hr[(long long)m * ldH + s] = make_double2(er - orr, ei - oi);
        }
    }
}

template <int NB>
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_synth_spin_df(int L, int spin, const double2 *__restrict__ G, const double2 *__restrict__ C,
                        long long astride, const double *__restrict__ lfac, const float2 *__restrict__ coef,
                        long long nalm, const double *__restrict__ lg0, int npairs, const double *__restrict__ px,
                        const double *__restrict__ psh, const double *__restrict__ pch,
                        const int *__restrict__ prn, const int *__restrict__ prs, double2 *__restrict__ H,
                        long long hstride, int ldH) {
    __shared__ float2 s_al[LEG_CH], s_ga[LEG_CH], s_be[LEG_CH];
    __shared__ float4 s_A[NB][LEG_CH], s_B[NB][LEG_CH];
    const int m = blockIdx.y;
    const int l0 = max(m, spin);
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
    }
    const dfl xN = df_from(x), xS = df_from(-x);
    dfl cN, pN, cS, pS;
    int eN, eS;
    rec_start_df(lg0[m], m, spin, sh, ch, cN, pN, eN);
    rec_start_df(lg0[m], m, spin, ch, sh, cS, pS, eS);
    kahan hpn_r[NB], hpn_i[NB], hps_r[NB], hps_i[NB], hmn_r[NB], hmn_i[NB], hms_r[NB], hms_i[NB];
    const float2 *al = coef, *ga = coef + nalm, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    for (int lb = l0; lb <= L; lb += LEG_CH) {
        const int cnt = min(LEG_CH, L - lb + 1);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += LEG_TPB) {
            const int l = lb + i;
            const long long ix = b + l;
            s_al[i] = al[ix];
            s_ga[i] = ga[ix];
            s_be[i] = be[ix];
            const double f = lfac ? lfac[l] : 1.0;
            const double par = ((l + m) & 1) ? -f : f;
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                const double2 g = G[r * astride + ix];
                const double2 c = C ? C[r * astride + ix] : make_double2(0.0, 0.0);
                const dfl ar = df_from(f * (g.x - c.y)), ai = df_from(f * (g.y + c.x));
                const dfl br = df_from(par * (g.x + c.y)), bi = df_from(par * (c.x - g.y));
                s_A[r][i] = make_float4(ar.h, ar.l, ai.h, ai.l);
                s_B[r][i] = make_float4(br.h, br.l, bi.h, bi.l);
            }
        }
        __syncthreads();
        for (int i = 0; i < cnt; ++i) {
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                const float4 A = s_A[r][i], B = s_B[r][i];
                if (eN == 0) {
                    hpn_r[r].add(df_prod(A.x, A.y, cN));
                    hpn_i[r].add(df_prod(A.z, A.w, cN));
                    hms_r[r].add(df_prod(B.x, B.y, cN));
                    hms_i[r].add(df_prod(B.z, B.w, cN));
                }
                if (eS == 0) {
                    hps_r[r].add(df_prod(A.x, A.y, cS));
                    hps_i[r].add(df_prod(A.z, A.w, cS));
                    hmn_r[r].add(df_prod(B.x, B.y, cS));
                    hmn_i[r].add(df_prod(B.z, B.w, cS));
                }
            }
            const float2 a2 = s_al[i], g2 = s_ga[i], b2 = s_be[i];
            const dfl ad{a2.x, a2.y}, gd{g2.x, g2.y}, bd{b2.x, b2.y};
            const dfl tN = df_fma_u(ad, xN, gd);
            const dfl tS = df_fma_u(ad, xS, gd);
            const dfl nN = df_mul_sub(tN, cN, bd, pN);
            const dfl nS = df_mul_sub(tS, cS, bd, pS);
            pN = cN;
            cN = nN;
            pS = cS;
            cS = nS;
            REC_RESCALE_DF(cN, pN, eN);
            REC_RESCALE_DF(cS, pS, eS);
        }
    }
    if (act) {
        const int n = prn[p], s = prs[p];
        const double sgs = (spin & 1) ? -1.0 : 1.0;
#pragma unroll
        for (int r = 0; r < NB; ++r) {
            double2 *Hr = H + r * hstride;
            Hr[(long long)(L + m) * ldH + n] = make_double2(-hpn_r[r].value(), -hpn_i[r].value());
            if (s != n) Hr[(long long)(L + m) * ldH + s] = make_double2(-hps_r[r].value(), -hps_i[r].value());
            if (m > 0) {
                Hr[(long long)(L - m) * ldH + n] = make_double2(-sgs * hmn_r[r].value(), -sgs * hmn_i[r].value());
                if (s != n)
                    Hr[(long long)(L - m) * ldH + s] = make_double2(-sgs * hms_r[r].value(), -sgs * hms_i[r].value());
            }
        }
    }
}

// ---------------------------------------------------------------- adjoint helpers
// Sum v[16] over the 32 lanes of a warp; afterwards lane k holds the total of
// index ((k >> 1) & 15) in v[0] (lanes 2j and 2j+1 hold the same value).
__device__ __forceinline__ void warp_reduce_scatter16(double v[16]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const bool up = lane & 16;
        const double send = up ? v[i] : v[i + 8];
        const double keep = up ? v[i + 8] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool up = lane & 8;
        const double send = up ? v[i] : v[i + 4];
        const double keep = up ? v[i + 4] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const bool up = lane & 4;
        const double send = up ? v[i] : v[i + 2];
        const double keep = up ? v[i + 2] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    {
        const bool up = lane & 2;
        const double send = up ? v[0] : v[1];
        const double keep = up ? v[1] : v[0];
        v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}
// index held by lane after the reduce-scatter: bits (lane>>1) reversed order
// of the halving steps: step 16 -> bit 3 of index, step 8 -> bit 2, 4 -> 1, 2 -> 0
__device__ __forceinline__ int rs16_index(int lane) {
    return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

// ---------------------------------------------------------------- adjoint, spin 0
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_adj_s0(int L, const double2 *__restrict__ H, int ldH, const double *__restrict__ lfac,
                 const double *__restrict__ coef, long long nalm, const double *__restrict__ lg0,
                 int npairs, const double *__restrict__ px, const double *__restrict__ psh,
                 const double *__restrict__ pch, const int *__restrict__ prn,
                 const int *__restrict__ prs, double *__restrict__ alm /* interleaved */) {
    constexpr int NW = LEG_TPB / 32;
    __shared__ double red[NW][16];
    const int m = blockIdx.y;
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    double2 Ep = make_double2(0, 0), Op = Ep;
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
        const int n = prn[p], s = prs[p];
        const double2 hn = H[(long long)m * ldH + n];
        if (s != n) {
            const double2 hs = H[(long long)m * ldH + s];
            Ep = make_double2(hn.x + hs.x, hn.y + hs.y);
            Op = make_double2(hn.x - hs.x, hn.y - hs.y);
        } else {
            Ep = hn;
            Op = hn;
        }
    }
    double cur, prev;
    int e;
    rec_start(lg0[m], m, 0, sh, ch, cur, prev, e);
    if (!act) {
        cur = 0.0;
        e = 0;
    }
    const double *al = coef, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int lb = m; lb <= L; lb += 8) {
        double v[16];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int l = lb + i;
            const double lam = (e == 0 && l <= L) ? cur : 0.0;
            const double2 src = ((l + m) & 1) ? Op : Ep;
            v[2 * i] = lam * src.x;
            v[2 * i + 1] = lam * src.y;
            if (l < L) {
                const double nxt = fma(__ldg(al + b + l) * x, cur, -__ldg(be + b + l) * prev);
                prev = cur;
                cur = nxt;
                REC_RESCALE(cur, prev, e);
            }
        }
        warp_reduce_scatter16(v);
        if (!(lane & 1)) red[wid][rs16_index(lane)] = v[0];
        __syncthreads();
        if (threadIdx.x < 16) {
            double t = 0.0;
#pragma unroll
            for (int w = 0; w < NW; ++w) t += red[w][threadIdx.x];
            const int l = lb + (threadIdx.x >> 1);
            if (l <= L) {
                const double f = lfac ? lfac[l] : 1.0;
                atomicAdd(alm + 2 * (b + l) + (threadIdx.x & 1), t * f);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- adjoint, spin s > 0
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_adj_spin(int L, int spin, int ncomp, const double2 *__restrict__ H, int ldH,
                   const double *__restrict__ lfac, const double *__restrict__ coef,
                   long long nalm, const double *__restrict__ lg0, int npairs,
                   const double *__restrict__ px, const double *__restrict__ psh,
                   const double *__restrict__ pch, const int *__restrict__ prn,
                   const int *__restrict__ prs, double *__restrict__ Gout,
                   double *__restrict__ Cout) {
    constexpr int NW = LEG_TPB / 32;
    __shared__ double red[NW][16];
    __shared__ double tot[16];
    const int m = blockIdx.y;
    const int l0 = max(m, spin);
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    double2 hpn = make_double2(0, 0), hps = hpn, hmn = hpn, hms = hpn;
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
        const int n = prn[p], s = prs[p];
        hpn = H[(long long)(L + m) * ldH + n];
        hmn = H[(long long)(L - m) * ldH + n];
        if (s != n) {
            hps = H[(long long)(L + m) * ldH + s];
            hms = H[(long long)(L - m) * ldH + s];
        }
    }
    double cN, pN, cS, pS;
    int eN, eS;
    rec_start(lg0[m], m, spin, sh, ch, cN, pN, eN);
    rec_start(lg0[m], m, spin, ch, sh, cS, pS, eS);
    if (!act) {
        cN = cS = 0.0;
        eN = eS = 0;
    }
    const double *al = coef, *ga = coef + nalm, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double sgs = (spin & 1) ? -1.0 : 1.0;
    for (int lb = l0; lb <= L; lb += 4) {
        double v[16];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int l = lb + i;
            const double lN = (eN == 0 && l <= L) ? cN : 0.0;
            const double lS = (eS == 0 && l <= L) ? cS : 0.0;
            const double par = ((l + m) & 1) ? -1.0 : 1.0;
            // P = lN hpn + lS hps ; Q = par (lS conj(hmn) + lN conj(hms))
            v[4 * i + 0] = fma(lN, hpn.x, lS * hps.x);
            v[4 * i + 1] = fma(lN, hpn.y, lS * hps.y);
            v[4 * i + 2] = par * fma(lS, hmn.x, lN * hms.x);
            v[4 * i + 3] = -par * fma(lS, hmn.y, lN * hms.y);
            if (l < L) {
                const double a_ = __ldg(al + b + l), g_ = __ldg(ga + b + l), b_ = __ldg(be + b + l);
                const double nN = fma(fma(a_, x, g_), cN, -b_ * pN);
                const double nS = fma(fma(a_, -x, g_), cS, -b_ * pS);
                pN = cN;
                cN = nN;
                pS = cS;
                cS = nS;
                REC_RESCALE(cN, pN, eN);
                REC_RESCALE(cS, pS, eS);
            }
        }
        warp_reduce_scatter16(v);
        if (!(lane & 1)) red[wid][rs16_index(lane)] = v[0];
        __syncthreads();
        if (threadIdx.x < 16) {
            double t = 0.0;
#pragma unroll
            for (int w = 0; w < NW; ++w) t += red[w][threadIdx.x];
            tot[threadIdx.x] = t;
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            const int l = lb + threadIdx.x;
            if (l <= L) {
                const double f = lfac ? lfac[l] : 1.0;
                const double Pr = tot[4 * threadIdx.x], Pi = tot[4 * threadIdx.x + 1];
                const double Qr = sgs * tot[4 * threadIdx.x + 2], Qi = sgs * tot[4 * threadIdx.x + 3];
                atomicAdd(Gout + 2 * (b + l), -0.5 * f * (Pr + Qr));
                atomicAdd(Gout + 2 * (b + l) + 1, -0.5 * f * (Pi + Qi));
                if (ncomp > 1) {
                    atomicAdd(Cout + 2 * (b + l), -0.5 * f * (Pi - Qi));
                    atomicAdd(Cout + 2 * (b + l) + 1, 0.5 * f * (Pr - Qr));
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- mixed precision adjoint
// The adjoint recursion runs in double-float as in the synthesis kernels; each
// product lambda * h' is formed as a double-float (h' split into FP32 hi/lo)
// and the sums over rings -- across the lanes of a warp, then across warps --
// are double-float additions, converted to FP64 once per (l, m) and block for
// the atomic accumulation.  No FP64 arithmetic in the inner loop.

// The adjoint sums keep (value, error) pairs unnormalised (df_add_u): the same
// ~2^-48 of the operands as normalised double-floats (renormalising adds no
// accuracy), a product of 4 FP32 operations instead of 7.
__device__ __forceinline__ dfl prod_pair(dfl lam, float hh, float hl) { return df_mul_u(lam, dfl{hh, hl}); }

__device__ __forceinline__ dfl shfl_xor_df(dfl v, int mask) {
    return dfl{__shfl_xor_sync(0xffffffffu, v.h, mask), __shfl_xor_sync(0xffffffffu, v.l, mask)};
}

// warp_reduce_scatter16 in double-float: same lane -> index mapping (rs16_index)
__device__ __forceinline__ void warp_reduce_scatter16_df(dfl v[16]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const bool up = lane & 16;
        const dfl send = up ? v[i] : v[i + 8];
        const dfl keep = up ? v[i + 8] : v[i];
        v[i] = df_add_u(keep, shfl_xor_df(send, 16));
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool up = lane & 8;
        const dfl send = up ? v[i] : v[i + 4];
        const dfl keep = up ? v[i + 4] : v[i];
        v[i] = df_add_u(keep, shfl_xor_df(send, 8));
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const bool up = lane & 4;
        const dfl send = up ? v[i] : v[i + 2];
        const dfl keep = up ? v[i + 2] : v[i];
        v[i] = df_add_u(keep, shfl_xor_df(send, 4));
    }
    {
        const bool up = lane & 2;
        const dfl send = up ? v[0] : v[1];
        const dfl keep = up ? v[1] : v[0];
        v[0] = df_add_u(keep, shfl_xor_df(send, 2));
    }
    v[0] = df_add_u(v[0], shfl_xor_df(v[0], 1));
}

// lam * (hh + hl) as a normalised double-float (the lam.l * hl term dropped)
__device__ __forceinline__ dfl df_prod_split(dfl lam, float hh, float hl) {
    const dfl p = df_mul_u(lam, dfl{hh, hl});
    return df_fast(p.h, p.l);
}

struct split2 {
    float xh, xl, yh, yl;
};

__device__ __forceinline__ split2 split_c(double2 v) {
    split2 r;
    r.xh = (float)v.x;
    r.xl = (float)(v.x - (double)r.xh);
    r.yh = (float)v.y;
    r.yl = (float)(v.y - (double)r.yh);
    return r;
}

// NB requests share the recursion: request r reads its columns at
// H + r * hstride and accumulates into its alm at alm + 2 r astride.
template <int NB>
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_adj_s0_df(int L, const double2 *__restrict__ H, long long hstride, int ldH,
                    const double *__restrict__ lfac, const float2 *__restrict__ coef, long long nalm,
                    const double *__restrict__ lg0, int npairs, const double *__restrict__ px,
                    const double *__restrict__ psh, const double *__restrict__ pch, const int *__restrict__ prn,
                    const int *__restrict__ prs, double *__restrict__ alm /* interleaved */, long long astride) {
    constexpr int NW = LEG_TPB / 32;
    __shared__ dfl red[NB][NW][16];
    const int m = blockIdx.y;
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    split2 E[NB], O[NB];
#pragma unroll
    for (int r = 0; r < NB; ++r) {
        double2 Ep = make_double2(0, 0), Op = Ep;
        if (act) {
            const double2 *Hr = H + r * hstride;
            const int n = prn[p], s = prs[p];
            const double2 hn = Hr[(long long)m * ldH + n];
            if (s != n) {
                const double2 hs = Hr[(long long)m * ldH + s];
                Ep = make_double2(hn.x + hs.x, hn.y + hs.y);
                Op = make_double2(hn.x - hs.x, hn.y - hs.y);
            } else {
                Ep = hn;
                Op = hn;
            }
        }
        E[r] = split_c(Ep);
        O[r] = split_c(Op);
    }
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
    }
    const dfl xd = df_from(x);
    dfl cur, prev;
    int e;
    rec_start_df(lg0[m], m, 0, sh, ch, cur, prev, e);
    if (!act) {
        cur.h = cur.l = 0.f;
        e = 0;
    }
    const float2 *al = coef, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const dfl zero{0.f, 0.f};
    for (int lb = m; lb <= L; lb += 8) {
        dfl lam[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int l = lb + i;
            lam[i] = (e == 0 && l <= L) ? cur : zero;
            if (l < L) {
                const float2 a2 = __ldg(al + b + l), b2 = __ldg(be + b + l);
                const dfl t = df_mul_u(dfl{a2.x, a2.y}, xd);
                const dfl nxt = df_mul_sub(t, cur, dfl{b2.x, b2.y}, prev);
                prev = cur;
                cur = nxt;
                REC_RESCALE_DF(cur, prev, e);
            }
        }
#pragma unroll
        for (int r = 0; r < NB; ++r) {
            dfl v[16];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const split2 &src = ((lb + i + m) & 1) ? O[r] : E[r];
                v[2 * i] = df_prod_split(lam[i], src.xh, src.xl);
                v[2 * i + 1] = df_prod_split(lam[i], src.yh, src.yl);
            }
            warp_reduce_scatter16_df(v);
            if (!(lane & 1)) red[r][wid][rs16_index(lane)] = v[0];
        }
        __syncthreads();
        if (threadIdx.x < 16 * NB) {
            const int r = threadIdx.x >> 4, q = threadIdx.x & 15;
            dfl t = red[r][0][q];
#pragma unroll
            for (int w2 = 1; w2 < NW; ++w2) t = df_add(t, red[r][w2][q]);
            const int l = lb + (q >> 1);
            if (l <= L) {
                const double f = lfac ? lfac[l] : 1.0;
                atomicAdd(alm + 2 * (r * astride + b + l) + (q & 1), df_to(t) * f);
            }
        }
        __syncthreads();
    }
}

template <int NB>
__global__ void __launch_bounds__(LEG_TPB)
    k_leg_adj_spin_df(int L, int spin, int ncomp, const double2 *__restrict__ H, long long hstride, int ldH,
                      const double *__restrict__ lfac, const float2 *__restrict__ coef,
                      long long nalm, const double *__restrict__ lg0, int npairs,
                      const double *__restrict__ px, const double *__restrict__ psh,
                      const double *__restrict__ pch, const int *__restrict__ prn,
                      const int *__restrict__ prs, double *__restrict__ Gout,
                      double *__restrict__ Cout, long long astride) {
    constexpr int NW = LEG_TPB / 32;
    __shared__ dfl red[NB][NW][16];
    __shared__ double tot[NB][16];
    const int m = blockIdx.y;
    const int l0 = max(m, spin);
    const int p = blockIdx.x * LEG_TPB + threadIdx.x;
    const bool act = p < npairs;
    double x = 0.0, sh = 0.0, ch = 1.0;
    split2 PN[NB], PS[NB], MN[NB], MS[NB];
#pragma unroll
    for (int r = 0; r < NB; ++r) {
        double2 hpn = make_double2(0, 0), hps = hpn, hmn = hpn, hms = hpn;
        if (act) {
            const double2 *Hr = H + r * hstride;
            const int n = prn[p], s = prs[p];
            hpn = Hr[(long long)(L + m) * ldH + n];
            hmn = Hr[(long long)(L - m) * ldH + n];
            if (s != n) {
                hps = Hr[(long long)(L + m) * ldH + s];
                hms = Hr[(long long)(L - m) * ldH + s];
            }
        }
        PN[r] = split_c(hpn);
        PS[r] = split_c(hps);
        MN[r] = split_c(hmn);
        MS[r] = split_c(hms);
    }
    if (act) {
        x = px[p];
        sh = psh[p];
        ch = pch[p];
    }
    const dfl xN = df_from(x), xS = df_from(-x);
    dfl cN, pN, cS, pS;
    int eN, eS;
    rec_start_df(lg0[m], m, spin, sh, ch, cN, pN, eN);
    rec_start_df(lg0[m], m, spin, ch, sh, cS, pS, eS);
    if (!act) {
        cN.h = cN.l = cS.h = cS.l = 0.f;
        eN = eS = 0;
    }
    const float2 *al = coef, *ga = coef + nalm, *be = coef + 2 * nalm;
    const long long b = almidx(L, m, m) - m;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double sgs = (spin & 1) ? -1.0 : 1.0;
    const dfl zero{0.f, 0.f};
    for (int lb = l0; lb <= L; lb += 4) {
        dfl lN[4], lS[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int l = lb + i;
            lN[i] = (eN == 0 && l <= L) ? cN : zero;
            lS[i] = (eS == 0 && l <= L) ? cS : zero;
            if (l < L) {
                const float2 a2 = __ldg(al + b + l), g2 = __ldg(ga + b + l), b2 = __ldg(be + b + l);
                const dfl ad{a2.x, a2.y}, gd{g2.x, g2.y}, bd{b2.x, b2.y};
                const dfl tN = df_fma_u(ad, xN, gd);
                const dfl tS = df_fma_u(ad, xS, gd);
                const dfl nN = df_mul_sub(tN, cN, bd, pN);
                const dfl nS = df_mul_sub(tS, cS, bd, pS);
                pN = cN;
                cN = nN;
                pS = cS;
                cS = nS;
                REC_RESCALE_DF(cN, pN, eN);
                REC_RESCALE_DF(cS, pS, eS);
            }
        }
#pragma unroll
        for (int r = 0; r < NB; ++r) {
            dfl v[16];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                // P = lN hpn + lS hps ; Q = par (lS conj(hmn) + lN conj(hms))
                v[4 * i + 0] = df_add_u(prod_pair(lN[i], PN[r].xh, PN[r].xl), prod_pair(lS[i], PS[r].xh, PS[r].xl));
                v[4 * i + 1] = df_add_u(prod_pair(lN[i], PN[r].yh, PN[r].yl), prod_pair(lS[i], PS[r].yh, PS[r].yl));
                const dfl qr = df_add_u(prod_pair(lS[i], MN[r].xh, MN[r].xl), prod_pair(lN[i], MS[r].xh, MS[r].xl));
                const dfl qi = df_add_u(prod_pair(lS[i], MN[r].yh, MN[r].yl), prod_pair(lN[i], MS[r].yh, MS[r].yl));
                const bool odd = (lb + i + m) & 1;
                v[4 * i + 2] = odd ? df_neg(qr) : qr;
                v[4 * i + 3] = odd ? qi : df_neg(qi);
            }
            warp_reduce_scatter16_df(v);
            if (!(lane & 1)) red[r][wid][rs16_index(lane)] = v[0];
        }
        __syncthreads();
        if (threadIdx.x < 16 * NB) {
            const int r = threadIdx.x >> 4, q = threadIdx.x & 15;
            dfl t = red[r][0][q];
#pragma unroll
            for (int w2 = 1; w2 < NW; ++w2) t = df_add(t, red[r][w2][q]);
            tot[r][q] = df_to(t);
        }
        __syncthreads();
        if (threadIdx.x < 4 * NB) {
            const int r = threadIdx.x >> 2, i = threadIdx.x & 3;
            const int l = lb + i;
            if (l <= L) {
                const double f = lfac ? lfac[l] : 1.0;
                const double Pr = tot[r][4 * i], Pi = tot[r][4 * i + 1];
                const double Qr = sgs * tot[r][4 * i + 2], Qi = sgs * tot[r][4 * i + 3];
                double *Gr = Gout + 2 * r * astride, *Cr = Cout ? Cout + 2 * r * astride : nullptr;
                atomicAdd(Gr + 2 * (b + l), -0.5 * f * (Pr + Qr));
                atomicAdd(Gr + 2 * (b + l) + 1, -0.5 * f * (Pi + Qi));
                if (ncomp > 1) {
                    atomicAdd(Cr + 2 * (b + l), -0.5 * f * (Pi - Qi));
                    atomicAdd(Cr + 2 * (b + l) + 1, 0.5 * f * (Pr - Qr));
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- exact synthesis at points
// Direct FP64 spin-s synthesis at arbitrary (theta, phi): one block per
// point, threads over m, the recursion in l run at theta (and at pi - theta
// for the negative-m functions, spin > 0), block reduction of the phased
// sums.  O(lmax^2) per point: the on-device spot check of the remapping
// (the reference's gclm2lenpixs, CPU_nufft_transformer.py:531-558, which
// synthesises on one 2-pixel ring per point).  Conventions as the transforms:
// spin 0 real, spin s Q + iU = -sum (G + iC) sY_lm, optional exp(i s gamma).
constexpr int SP_PTS_TPB = 128;

__global__ void __launch_bounds__(SP_PTS_TPB)
    k_synth_points(int L, int mmax, int spin, const double2 *__restrict__ G, const double2 *__restrict__ C,
                   const double *__restrict__ coef, long long nalm, const double *__restrict__ lg0,
                   const double *__restrict__ loc, long long npts, int layout, const double *__restrict__ gamma,
                   double *__restrict__ out) {
    __shared__ double2 red[SP_PTS_TPB];
    const long long j = blockIdx.x;
    double th, ph;
    if (layout == 0) {
        th = loc[2 * j];
        ph = loc[2 * j + 1];
    } else {
        th = loc[j];
        ph = loc[npts + j];
    }
    double st, ct, sh, ch;
    sincos(th, &st, &ct);
    sincos(0.5 * th, &sh, &ch);
    const double *al = coef, *ga = coef + nalm, *be = coef + 2 * nalm;
    double zr = 0.0, zi = 0.0;
    for (int m = threadIdx.x; m <= mmax; m += blockDim.x) {
        const int l0 = max(m, spin);
        const long long b = almidx(L, m, m) - m;
        double cN, pN, cS = 0.0, pS = 0.0;
        int eN, eS = 0;
        rec_start(lg0[m], m, spin, sh, ch, cN, pN, eN);
        if (spin) rec_start(lg0[m], m, spin, ch, sh, cS, pS, eS);
        double2 hp = make_double2(0, 0), hm = hp;
        for (int l = l0; l <= L; ++l) {
            const double2 g = G[b + l];
            if (spin == 0) {
                if (eN == 0) {
                    hp.x = fma(g.x, cN, hp.x);
                    hp.y = fma(g.y, cN, hp.y);
                }
            } else {
                const double2 c = C ? C[b + l] : make_double2(0.0, 0.0);
                if (eN == 0) {  // (G + iC) lambda(theta)
                    hp.x = fma(g.x - c.y, cN, hp.x);
                    hp.y = fma(g.y + c.x, cN, hp.y);
                }
                if (eS == 0) {  // (conj G + i conj C) (-1)^{l+m} lambda(pi - theta)
                    const double par = ((l + m) & 1) ? -cS : cS;
                    hm.x = fma(g.x + c.y, par, hm.x);
                    hm.y = fma(c.x - g.y, par, hm.y);
                }
            }
            if (l < L) {
                const double a_ = al[b + l], g_ = ga[b + l], b_ = be[b + l];
                const double nN = fma(fma(a_, ct, g_), cN, -b_ * pN);
                pN = cN;
                cN = nN;
                REC_RESCALE(cN, pN, eN);
                if (spin) {
                    const double nS = fma(fma(a_, -ct, g_), cS, -b_ * pS);
                    pS = cS;
                    cS = nS;
                    REC_RESCALE(cS, pS, eS);
                }
            }
        }
        double sn, cs;
        sincos((double)m * ph, &sn, &cs);
        if (spin == 0) {
            zr += (m == 0) ? hp.x : 2.0 * (hp.x * cs - hp.y * sn);
        } else {
            // -hp e^{i m phi} - (-1)^s hm e^{-i m phi} (m > 0)
            zr -= hp.x * cs - hp.y * sn;
            zi -= hp.x * sn + hp.y * cs;
            if (m > 0) {
                const double sg = (spin & 1) ? -1.0 : 1.0;
                zr -= sg * (hm.x * cs + hm.y * sn);
                zi -= sg * (hm.y * cs - hm.x * sn);
            }
        }
    }
    red[threadIdx.x] = make_double2(zr, zi);
    __syncthreads();
    for (int o = SP_PTS_TPB / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            red[threadIdx.x].x += red[threadIdx.x + o].x;
            red[threadIdx.x].y += red[threadIdx.x + o].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double vr = red[0].x, vi = red[0].y;
        if (spin == 0) {
            out[j] = vr;
        } else {
            if (gamma) {
                double s, c;
                sincos(spin * gamma[j], &s, &c);
                const double t = vr * c - vi * s;
                vi = vr * s + vi * c;
                vr = t;
            }
            out[j] = vr;
            out[npts + j] = vi;
        }
    }
}

int synth_points(const cunusht_plan_s *P, int spin, const double2 *G, const double2 *C, long long npts,
                 const double *loc, int layout, const double *gamma, double *out, cudaStream_t st) {
    if (npts == 0) return CUNUSHT_OK;
    k_synth_points<<<(unsigned)npts, SP_PTS_TPB, 0, st>>>(P->lmax, P->mmax, spin, G, C, P->d_coef[spin], P->nalm_tab,
                                                         P->d_lg0[spin], loc, npts, layout, gamma, out);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// ---------------------------------------------------------------- host launchers
struct RingPairs {
    int npairs;
    const double *x, *sh, *ch;
    const int *rn, *rs;
    int ld;
    int pole = -1;  // pair (theta = 0, pi), or -1
    int pole_rn = 0, pole_rs = 0;  // its ring indices
    const float4 *const *stv = nullptr;  // tensor-core recursion starts per spin (or NULL)
    const short2 *const *ste = nullptr;
};

static RingPairs pairs_of(const cunusht_plan_s *P, bool cc) {
    if (cc)
        return {P->cc_npairs, P->d_cc_x, P->d_cc_sh, P->d_cc_ch, P->d_cc_rn, P->d_cc_rs, P->ncc,
                P->cc_pole, P->cc_pole_ring[0], P->cc_pole_ring[1], P->d_tc_stv[1], P->d_tc_ste[1]};
    return {P->gl_npairs, P->d_gl_x, P->d_gl_sh, P->d_gl_ch, P->d_gl_rn, P->d_gl_rs, P->nring,
            P->gl_pole, P->gl_pole_ring[0], P->gl_pole_ring[1], P->d_tc_stv[0], P->d_tc_ste[0]};
}

template <int NB>
static void launch_synth_df(const cunusht_plan_s *P, const RingPairs &R, dim3 grid, int spin, const double2 *G,
                            const double2 *C, long long astride, const double *lf, double2 *H, long long hstride,
                            cudaStream_t st) {
    const int L = P->lmax;
    if (spin == 0)
        k_leg_synth_s0_df<NB><<<grid, LEG_TPB, 0, st>>>(L, G, astride, lf, P->d_coef_df[0], P->nalm_tab, P->d_lg0[0],
                                                        R.npairs, R.x, R.sh, R.ch, R.rn, R.rs, H, hstride, R.ld);
    else
        k_leg_synth_spin_df<NB><<<grid, LEG_TPB, 0, st>>>(L, spin, G, C, astride, lf, P->d_coef_df[spin], P->nalm_tab,
                                                          P->d_lg0[spin], R.npairs, R.x, R.sh, R.ch, R.rn, R.rs, H,
                                                          hstride, R.ld);
}

int leg_synth_spin_df_pairs(const cunusht_plan_s *P, int nb, int npairs, const double *x, const double *sh,
                            const double *ch, const int *rn, const int *rs, int ld, int spin, const double2 *G,
                            const double2 *C, long long astride, const double *lf, double2 *H, long long hstride,
                            cudaStream_t st) {
    const RingPairs R{npairs, x, sh, ch, rn, rs, ld};
    const dim3 grid((npairs + LEG_TPB - 1) / LEG_TPB, P->mmax + 1);
    if (nb == 4) launch_synth_df<4>(P, R, grid, spin, G, C, astride, lf, H, hstride, st);
    else if (nb == 2) launch_synth_df<2>(P, R, grid, spin, G, C, astride, lf, H, hstride, st);
    else launch_synth_df<1>(P, R, grid, spin, G, C, astride, lf, H, hstride, st);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// nreq requests (alm at G + r * astride, columns at H + r * hstride); the
// mixed-precision kernels process several requests per launch with one shared
// recursion (tensor cores: up to eight, CUDA cores: up to four), the FP64
// kernels one request per launch.
int leg_synth_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *G, const double2 *C,
                    long long astride, bool use_lfac, bool cc, double2 *H, long long hstride, cudaStream_t st) {
    return leg_synth_batch_fl(P, nreq, spin, G, C, astride, use_lfac ? P->d_lfac : nullptr, cc, H, hstride, st);
}

// as leg_synth_batch with the alm multiplied by an arbitrary per-l factor fl (NULL: 1)
int leg_synth_batch_fl(const cunusht_plan_s *P, int nreq, int spin, const double2 *G, const double2 *C,
                       long long astride, const double *lf, bool cc, double2 *H, long long hstride, cudaStream_t st) {
    const RingPairs R = pairs_of(P, cc);
    const int L = P->lmax;
    if (P->mmax < L) {  // alm up to mmax only: the columns of larger |m| are zero
        const size_t ncols = spin ? 2 * (size_t)L + 1 : (size_t)L + 1;
        for (int r = 0; r < nreq; ++r)
            CU_TRY(cudaMemsetAsync(H + r * hstride, 0, sizeof(double2) * ncols * R.ld, st));
    }
    dim3 grid((R.npairs + LEG_TPB - 1) / LEG_TPB, P->mmax + 1);
    if (P->prec == CUNUSHT_PREC_MIXED && P->d_coef_df[spin]) {
        for (int r0 = 0; r0 < nreq;) {
            const int left = nreq - r0;
            const double2 *Gr = G + r0 * astride, *Cr = C ? C + r0 * astride : nullptr;
            double2 *Hr = H + r0 * hstride;
            if (P->use_tc) {
                // as many requests per launch as the window records were reserved for
                const int cap = left < P->tc_rec_nb ? left : P->tc_rec_nb;
                const int nb = cap >= 8 ? 8 : cap >= 4 ? 4 : cap >= 2 ? 2 : 1;
                RC_TRY(leg_synth_spin_tc(P, nb, R.npairs, R.x, R.sh, R.ch, R.rn, R.rs, R.ld, R.pole, R.pole_rn,
                                         R.pole_rs, R.stv ? R.stv[spin] : nullptr, R.ste ? R.ste[spin] : nullptr,
                                         spin, Gr, Cr, astride, lf, Hr, hstride, st));
                r0 += nb;
                continue;
            }
            if (left >= 4) {
                launch_synth_df<4>(P, R, grid, spin, Gr, Cr, astride, lf, Hr, hstride, st);
                r0 += 4;
            } else if (left >= 2) {
                launch_synth_df<2>(P, R, grid, spin, Gr, Cr, astride, lf, Hr, hstride, st);
                r0 += 2;
            } else {
                launch_synth_df<1>(P, R, grid, spin, Gr, Cr, astride, lf, Hr, hstride, st);
                r0 += 1;
            }
            CU_LAUNCH_CHECK();
        }
        return CUNUSHT_OK;
    }
    for (int r = 0; r < nreq; ++r) {
        const double2 *Gr = G + r * astride, *Cr = C ? C + r * astride : nullptr;
        double2 *Hr = H + r * hstride;
        if (spin == 0) {
            k_leg_synth_s0<<<grid, LEG_TPB, 0, st>>>(L, Gr, lf, P->d_coef[0], P->nalm_tab, P->d_lg0[0], R.npairs, R.x,
                                                     R.sh, R.ch, R.rn, R.rs, Hr, R.ld);
        } else {
            k_leg_synth_spin<<<grid, LEG_TPB, 0, st>>>(L, spin, Gr, Cr, lf, P->d_coef[spin], P->nalm_tab,
                                                       P->d_lg0[spin], R.npairs, R.x, R.sh, R.ch, R.rn, R.rs, Hr,
                                                       R.ld);
        }
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int leg_synth(const cunusht_plan_s *P, int spin, const double2 *G, const double2 *C,
              bool use_lfac, bool cc, double2 *H, cudaStream_t st) {
    return leg_synth_batch(P, 1, spin, G, C, 0, use_lfac, cc, H, 0, st);
}

// Adjoint of the pole ring pair (theta = 0, pi) for spin s >= 1: every
// function vanishes at theta = 0 and at pi all but m = s, with
// sLambda_ls(pi) = (-1)^l sqrt((2l + 1) / (4 pi)), so the pair adds, for
// m = s only, the terms k_leg_adj_spin_df forms from its S ring (P = lambda
// h(+m, pi), Q = par lambda conj(h(-m, 0))), in FP64; block row r = request r.
__global__ void k_pole_pair_adj_spin(int L, int spin, int ncomp, int mmax, const double2 *__restrict__ H,
                                     long long hstride, int ldH, const double *__restrict__ lfac, int rn, int rs,
                                     double *__restrict__ Gout, double *__restrict__ Cout, long long astride) {
    if (spin > mmax) return;
    const int r = blockIdx.y;
    const double2 *Hr = H + r * hstride;
    const double2 hps = Hr[(long long)(L + spin) * ldH + rs], hmn = Hr[(long long)(L - spin) * ldH + rn];
    const double sgs = (spin & 1) ? -1.0 : 1.0;
    const long long b = almidx(L, spin, spin) - spin;
    double *Gr = Gout + 2 * r * astride, *Cr = Cout ? Cout + 2 * r * astride : nullptr;
    for (int l = spin + blockIdx.x * blockDim.x + threadIdx.x; l <= L; l += gridDim.x * blockDim.x) {
        const double lam = ((l & 1) ? -1.0 : 1.0) * sqrt((2.0 * l + 1.0) / (4.0 * PI));
        const double f = lfac ? lfac[l] : 1.0;
        const bool odd = (l + spin) & 1;
        const double Pr = lam * hps.x, Pi = lam * hps.y, qr = lam * hmn.x, qi = lam * hmn.y;
        const double Qr = sgs * (odd ? -qr : qr), Qi = sgs * (odd ? qi : -qi);
        atomicAdd(Gr + 2 * (b + l), -0.5 * f * (Pr + Qr));
        atomicAdd(Gr + 2 * (b + l) + 1, -0.5 * f * (Pi + Qi));
        if (ncomp > 1) {
            atomicAdd(Cr + 2 * (b + l), -0.5 * f * (Pi - Qi));
            atomicAdd(Cr + 2 * (b + l) + 1, 0.5 * f * (Pr - Qr));
        }
    }
}

template <int NB>
static void launch_adj_df(const cunusht_plan_s *P, const RingPairs &R, dim3 grid, int spin, int ncomp,
                          const double2 *H, long long hstride, const double *lf, double2 *G, double2 *C,
                          long long astride, cudaStream_t st) {
    const int L = P->lmax;
    if (spin == 0)
        k_leg_adj_s0_df<NB><<<grid, LEG_TPB, 0, st>>>(L, H, hstride, R.ld, lf, P->d_coef_df[0], P->nalm_tab,
                                                      P->d_lg0[0], R.npairs, R.x, R.sh, R.ch, R.rn, R.rs,
                                                      (double *)G, astride);
    else
        k_leg_adj_spin_df<NB><<<grid, LEG_TPB, 0, st>>>(L, spin, ncomp, H, hstride, R.ld, lf, P->d_coef_df[spin],
                                                        P->nalm_tab, P->d_lg0[spin], R.npairs, R.x, R.sh, R.ch, R.rn,
                                                        R.rs, (double *)G, (double *)C, astride);
}

// the pole pair (theta = 0, pi) of a spin s >= 1 adjoint, added to the alm
int leg_adj_pole_pair_spin(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                           int ld, const double *lf, int rn, int rs, double2 *G, double2 *C, long long astride,
                           cudaStream_t st) {
    const int L = P->lmax;
    k_pole_pair_adj_spin<<<dim3((L - spin + 256) / 256, nreq), 256, 0, st>>>(
        L, spin, ncomp, P->mmax, H, hstride, ld, lf, rn, rs, (double *)G, (spin > 0 && ncomp > 1) ? (double *)C : nullptr,
        astride);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// npairs ring pairs of a grid through the double-float CUDA-core adjoint,
// added to the alm (up to four requests share a recursion)
int leg_adj_df_pairs(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                     int ld, int npairs, const double *x, const double *sh, const double *ch, const int *rn,
                     const int *rs, const double *lf, double2 *G, double2 *C, long long astride, cudaStream_t st) {
    const RingPairs R{npairs, x, sh, ch, rn, rs, ld};
    const dim3 grid((npairs + LEG_TPB - 1) / LEG_TPB, P->mmax + 1);
    for (int r0 = 0; r0 < nreq;) {
        const int left = nreq - r0;
        const double2 *Hr = H + r0 * hstride;
        double2 *Gr = G + r0 * astride, *Cr = (spin > 0 && ncomp > 1) ? C + r0 * astride : nullptr;
        const int nb = left >= 4 ? 4 : left >= 2 ? 2 : 1;
        if (nb == 4) launch_adj_df<4>(P, R, grid, spin, ncomp, Hr, hstride, lf, Gr, Cr, astride, st);
        else if (nb == 2) launch_adj_df<2>(P, R, grid, spin, ncomp, Hr, hstride, lf, Gr, Cr, astride, st);
        else launch_adj_df<1>(P, R, grid, spin, ncomp, Hr, hstride, lf, Gr, Cr, astride, st);
        CU_LAUNCH_CHECK();
        r0 += nb;
    }
    return CUNUSHT_OK;
}

// nreq requests: columns at H + r * hstride, alm written at G + r * astride
// (and C + r * astride).  Mixed precision: on the tensor cores when the plan
// uses them and scratch (the caller's free workspace, scratch_bytes) holds the
// fixed-point sums, else double-float CUDA-core kernels sharing one recursion
// between up to four requests; the FP64 kernels run one request per launch.
int leg_adjoint_batch(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                      bool use_lfac, bool cc, double2 *G, double2 *C, long long astride, cudaStream_t st,
                      void *scratch, size_t scratch_bytes) {
    const RingPairs R = pairs_of(P, cc);
    const int L = P->lmax;
    if (P->prec == CUNUSHT_PREC_MIXED && P->use_tc && P->d_coef_df[spin] && scratch &&
        scratch_bytes >= adj_tc_scratch_bytes(P, nreq)) {
        return leg_adjoint_tc(P, nreq, spin, ncomp, H, hstride, R.ld, R.npairs, R.x, R.sh, R.ch, R.rn, R.rs, R.pole,
                              R.pole_rn, R.pole_rs, R.stv ? R.stv[spin] : nullptr, R.ste ? R.ste[spin] : nullptr,
                              use_lfac ? P->d_lfac : nullptr, G, C, astride, scratch, st);
    }
    for (int r = 0; r < nreq; ++r) {
        CU_TRY(cudaMemsetAsync(G + r * astride, 0, sizeof(double2) * P->nalm, st));
        if (spin > 0 && ncomp > 1) CU_TRY(cudaMemsetAsync(C + r * astride, 0, sizeof(double2) * P->nalm, st));
    }
    dim3 grid((R.npairs + LEG_TPB - 1) / LEG_TPB, P->mmax + 1);
    const double *lf = use_lfac ? P->d_lfac : nullptr;
    if (P->prec == CUNUSHT_PREC_MIXED && P->d_coef_df[spin]) {
        RingPairs Rm = R;
        if (spin > 0 && R.pole == 0 && R.npairs > 1) {
            // the pole pair in closed form; the other 2^k pairs fill whole blocks
            k_pole_pair_adj_spin<<<dim3((L - spin + 256) / 256, nreq), 256, 0, st>>>(
                L, spin, ncomp, P->mmax, H, hstride, R.ld, lf, R.pole_rn, R.pole_rs, (double *)G,
                (spin > 0 && ncomp > 1) ? (double *)C : nullptr, astride);
            CU_LAUNCH_CHECK();
            ++Rm.x, ++Rm.sh, ++Rm.ch, ++Rm.rn, ++Rm.rs;
            --Rm.npairs;
            grid.x = (Rm.npairs + LEG_TPB - 1) / LEG_TPB;
        }
        for (int r0 = 0; r0 < nreq;) {
            const int left = nreq - r0;
            const double2 *Hr = H + r0 * hstride;
            double2 *Gr = G + r0 * astride, *Cr = (spin > 0 && ncomp > 1) ? C + r0 * astride : nullptr;
            if (left >= 4) {
                launch_adj_df<4>(P, Rm, grid, spin, ncomp, Hr, hstride, lf, Gr, Cr, astride, st);
                r0 += 4;
            } else if (left >= 2) {
                launch_adj_df<2>(P, Rm, grid, spin, ncomp, Hr, hstride, lf, Gr, Cr, astride, st);
                r0 += 2;
            } else {
                launch_adj_df<1>(P, Rm, grid, spin, ncomp, Hr, hstride, lf, Gr, Cr, astride, st);
                r0 += 1;
            }
            CU_LAUNCH_CHECK();
        }
        return CUNUSHT_OK;
    }
    for (int r = 0; r < nreq; ++r) {
        const double2 *Hr = H + r * hstride;
        double2 *Gr = G + r * astride, *Cr = (spin > 0 && ncomp > 1) ? C + r * astride : nullptr;
        if (spin == 0) {
            k_leg_adj_s0<<<grid, LEG_TPB, 0, st>>>(L, Hr, R.ld, lf, P->d_coef[0], P->nalm_tab, P->d_lg0[0], R.npairs,
                                                   R.x, R.sh, R.ch, R.rn, R.rs, (double *)Gr);
        } else {
            k_leg_adj_spin<<<grid, LEG_TPB, 0, st>>>(L, spin, ncomp, Hr, R.ld, lf, P->d_coef[spin], P->nalm_tab,
                                                     P->d_lg0[spin], R.npairs, R.x, R.sh, R.ch, R.rn, R.rs,
                                                     (double *)Gr, (double *)Cr);
        }
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int leg_adjoint(const cunusht_plan_s *P, int spin, int ncomp, const double2 *H, bool use_lfac,
                bool cc, double2 *G, double2 *C, cudaStream_t st, void *scratch, size_t scratch_bytes) {
    return leg_adjoint_batch(P, 1, spin, ncomp, H, 0, use_lfac, cc, G, C, 0, st, scratch, scratch_bytes);
}

}  // namespace cunusht

// Ring transforms of the pointing geometry by a mixed-radix FFT of the ring
// length itself, for rings of one length N <= 8192 whose prime factors are at
// most 13: the 4095-pixel Gauss-Legendre rings of lmax 2047 (3^2 5 7 13), the
// power-of-two rings of the default geometries.  The Bluestein form
// (fft.cu k_ring_synth) runs two transforms of the next power of two >= 2N - 1
// per ring; this one runs one transform of N points in about a quarter of the
// arithmetic.  Other ring lengths keep Bluestein.  This is the transform SHTns
// performs inside synth_grad (cunusht/sht/GPU_sht_transformer.py:95), on the
// ring lengths its FFT library handles natively.
//
// Algorithm: in-place decimation in frequency (Gentleman-Sande) over the
// radices R_1 .. R_k (N = prod R_i, the largest radix last so that its stage
// has no twiddles).  A stage of sub-transform length Ls and radix R, S = Ls/R,
// takes every block of Ls points and j < S through
//     Y_q = sum_r y_r e^{2 pi i r q / R},  y_r = x[j + r S],
//     x[j + q S] = Y_q e^{2 pi i j q / Ls},
// in place (a butterfly owns its R positions, one barrier per stage).  The
// result X_k sits at pos(k) = sum_i q_i N / (R_1 .. R_i) with q_i the i-th
// mixed-radix digit of k (least significant first); the output loop reads it
// there.  Odd radices use the symmetric form
//     Y_q, Y_{R-q} = y_0 + sum_r s_r cos(2 pi r q / R)  +-  i sum_r d_r sin(2 pi r q / R),
//     s_r = y_r + y_{R-r},  d_r = y_r - y_{R-r},  r, q = 1 .. (R-1)/2,
// (R-1)^2 real multiply-adds instead of 2 (R-1)^2; radices 2 and 4 are
// written out.  The twiddles e^{2 pi i t / N} come from a table of N entries
// (FP64 or double-float), read through L1; the constants of each stage's
// radix are staged in shared memory.
#include "common.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace cunusht {

constexpr int MR_TPB = 256;  // threads per ring block

// ------------------------------------------------------------ plan set-up
// Radices of N (each in {2, 3, 4, 5, 7, 9, 11, 13}, ascending, so the
// largest stage comes last); empty when N has another prime factor.
static std::vector<int> mr_radices(int N) {
    std::vector<int> r;
    int n = N;
    int c2 = 0, c3 = 0;
    while (n % 2 == 0) n /= 2, ++c2;
    while (n % 3 == 0) n /= 3, ++c3;
    for (int i = 0; i < c2 / 2; ++i) r.push_back(4);
    if (c2 & 1) r.push_back(2);
    for (int i = 0; i < c3 / 2; ++i) r.push_back(9);
    if (c3 & 1) r.push_back(3);
    for (int p : {5, 7, 11, 13})
        while (n % p == 0) n /= p, r.push_back(p);
    if (n != 1) return {};
    std::sort(r.begin(), r.end());
    return r;
}

int ring_mr_init(cunusht_plan_s *P) {
    P->mr_nst = 0;
    const int N = P->nph_uniform;
    if (P->ncls > 1 || N < 2 || N > MR_NMAX) return CUNUSHT_OK;
    const std::vector<int> rad = mr_radices(N);
    if (rad.empty() || (int)rad.size() > MR_MAXST) return CUNUSHT_OK;
    int Ls = N, cst = 0;
    for (size_t i = 0; i < rad.size(); ++i) {
        P->mr_R[i] = rad[i];
        P->mr_Ls[i] = Ls;
        P->mr_coff[i] = cst;
        cst += rad[i];
        Ls /= rad[i];
    }
    // output positions: X_k at sum_i q_i N / (R_1 .. R_i)
    std::vector<int> pos(N);
    for (int k = 0; k < N; ++k) {
        long long p = 0, kk = k, span = N;
        for (int r : rad) {
            span /= r;
            p += (kk % r) * span;
            kk /= r;
        }
        pos[k] = (int)p;
    }
    std::vector<double2> tw(N);
    std::vector<dcplx> twd(N);
    for (int t = 0; t < N; ++t) {
        const long double a = 2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)N;
        const long double c = std::cos(a), s = std::sin(a);
        tw[t] = make_double2((double)c, (double)s);
        twd[t].x.h = (float)c;
        twd[t].x.l = (float)(c - (long double)twd[t].x.h);
        twd[t].y.h = (float)s;
        twd[t].y.l = (float)(s - (long double)twd[t].y.h);
    }
    RC_TRY(plan_alloc(P, (void **)&P->d_mr_pos, sizeof(int) * (size_t)N));
    RC_TRY(plan_alloc(P, (void **)&P->d_mr_tw64, sizeof(double2) * (size_t)N));
    RC_TRY(plan_alloc(P, (void **)&P->d_mr_twdf, sizeof(dcplx) * (size_t)N));
    CU_TRY(cudaMemcpy(P->d_mr_pos, pos.data(), sizeof(int) * (size_t)N, cudaMemcpyHostToDevice));
    CU_TRY(cudaMemcpy(P->d_mr_tw64, tw.data(), sizeof(double2) * (size_t)N, cudaMemcpyHostToDevice));
    CU_TRY(cudaMemcpy(P->d_mr_twdf, twd.data(), sizeof(dcplx) * (size_t)N, cudaMemcpyHostToDevice));
    P->mr_nst = (int)rad.size();
    return CUNUSHT_OK;
}

// ------------------------------------------------------------ butterflies
struct MrStages {
    int n;                // stages
    int R[MR_MAXST];      // radix
    int Ls[MR_MAXST];     // sub-transform length
    int coff[MR_MAXST];   // offset of the stage's radix constants in shared memory
};

// i * v
template <typename C> __device__ __forceinline__ C mr_i(C v) {
    C r;
    r.x = -v.y;
    r.y = v.x;
    return r;
}

// One butterfly of a stage: y_r = x[r S], Y = DFT_R(y) with the kernel
// e^{+2 pi i / R} (K[m] = e^{2 pi i m / R}), x[q S] = Y_q w_q with the
// twiddles w_q = tw[t q] (t = 0: none).  The inputs stay in registers while
// the outputs are written, and each output pair is twiddled and stored as
// soon as it is formed, which keeps the live set of the odd radices at the R
// inputs plus a few temporaries.
template <typename T, int R>
__device__ __forceinline__ void mr_butterfly(cplx<T> *x, int S, int t, const cplx<T> *__restrict__ K,
                                             const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    C y[R];
#pragma unroll
    for (int r = 0; r < R; ++r) y[r] = x[r * S];
    auto put = [&](int q, C v) { x[q * S] = t ? cmul(v, tw[t * q]) : v; };
    if constexpr (R == 2) {
        x[0] = cadd(y[0], y[1]);
        put(1, csub(y[0], y[1]));
    } else if constexpr (R == 4) {
        const C a = cadd(y[0], y[2]), b = csub(y[0], y[2]), c = cadd(y[1], y[3]), d = mr_i(csub(y[1], y[3]));
        x[0] = cadd(a, c);
        put(2, csub(a, c));
        put(1, cadd(b, d));
        put(3, csub(b, d));
    } else {
        constexpr int H = (R - 1) / 2;
        // y[r] <- s_r = y_r + y_{R-r}, y[R-r] <- d_r = y_r - y_{R-r}
        C sum = y[0];
#pragma unroll
        for (int r = 1; r <= H; ++r) {
            const C a = y[r], b = y[R - r];
            y[r] = cadd(a, b);
            y[R - r] = csub(a, b);
            sum = cadd(sum, y[r]);
        }
        x[0] = sum;
#pragma unroll
        for (int q = 1; q <= H; ++q) {
            C A = y[0], B;
            B.x = cvt<T>(0.0);
            B.y = cvt<T>(0.0);
#pragma unroll
            for (int r = 1; r <= H; ++r) {
                const C k = K[(r * q) % R];
                A = cadd(A, cscale(y[r], k.x));
                B = cadd(B, cscale(y[R - r], k.y));
            }
            const C iB = mr_i(B);
            put(q, cadd(A, iB));
            put(R - q, csub(A, iB));
            // one output pair at a time: keeps the twiddle loads of later
            // pairs out of the live set
            asm volatile("" ::: "memory");
        }
    }
}

template <typename T, int R>
__device__ __forceinline__ void mr_stage(cplx<T> *buf, int N, int Ls, const cplx<T> *__restrict__ K,
                                         const cplx<T> *__restrict__ tw) {
    const int S = Ls / R, nb = N / R, f = N / Ls;  // e^{2 pi i j q / Ls} = tw[f j q]
    for (int bf = threadIdx.x; bf < nb; bf += blockDim.x) {
        const int b = bf / S, j = bf - b * S;
        mr_butterfly<T, R>(buf + b * Ls + j, S, f * j, K, tw);
    }
    __syncthreads();
}

template <typename T>
__device__ __forceinline__ void mr_fft(cplx<T> *buf, int N, const MrStages &st, const cplx<T> *K,
                                       const cplx<T> *__restrict__ tw) {
    for (int i = 0; i < st.n; ++i) {
        const cplx<T> *Ki = K + st.coff[i];
        switch (st.R[i]) {
            case 2: mr_stage<T, 2>(buf, N, st.Ls[i], Ki, tw); break;
            case 3: mr_stage<T, 3>(buf, N, st.Ls[i], Ki, tw); break;
            case 4: mr_stage<T, 4>(buf, N, st.Ls[i], Ki, tw); break;
            case 5: mr_stage<T, 5>(buf, N, st.Ls[i], Ki, tw); break;
            case 7: mr_stage<T, 7>(buf, N, st.Ls[i], Ki, tw); break;
            case 9: mr_stage<T, 9>(buf, N, st.Ls[i], Ki, tw); break;
            case 11: mr_stage<T, 11>(buf, N, st.Ls[i], Ki, tw); break;
            default: mr_stage<T, 13>(buf, N, st.Ls[i], Ki, tw); break;
        }
    }
}

// z_p = sum_m h_m e^{i m (phi0 + 2 pi p / N)}, p < N, one ring per block
// (blockIdx.x) and request (blockIdx.y); the same bins, phases and output as
// k_ring_synth: spin 0 takes h_{-m} = conj h_m from the m >= 0 columns and
// writes the real part, spin s writes both parts.
template <typename T>
__global__ void __launch_bounds__(MR_TPB, 2)
    k_ring_synth_mr(const double2 *__restrict__ Hgl, int nring, int L, int spin, int N,
                    const double *__restrict__ phi0, const long long *__restrict__ ofs, MrStages st,
                    const cplx<T> *__restrict__ tw, const int *__restrict__ pos, double *__restrict__ out0,
                    double *__restrict__ out1, long long hbs, long long obs) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *K = reinterpret_cast<C *>(smem_raw);  // radix constants of every stage
    C *buf = K + MR_KMAX;
    const int ring = blockIdx.x;
    Hgl += blockIdx.y * hbs;
    out0 += blockIdx.y * obs;
    if (out1) out1 += blockIdx.y * obs;
    for (int i = 0; i < st.n; ++i)
        for (int m = threadIdx.x; m < st.R[i]; m += blockDim.x) K[st.coff[i] + m] = tw[m * (N / st.R[i])];
    const double ph0 = phi0[ring];
    for (int qi = threadIdx.x; qi < N; qi += blockDim.x) {
        // bin qi gathers every m = qi (mod N); with N >= 2L + 1 (no aliasing) one term.
        // Double-float sums for the mixed path: no FP64 arithmetic unless phi0 != 0
        T ax = cvt<T>(0.0), ay = cvt<T>(0.0);
        for (int m = qi - N * ((qi + L) / N); m <= L; m += N) {
            double2 h;
            if (spin == 0) {
                const double2 hm = Hgl[(long long)(m < 0 ? -m : m) * nring + ring];
                h = m == 0 ? make_double2(hm.x, 0.0) : (m > 0 ? hm : make_double2(hm.x, -hm.y));
            } else {
                h = Hgl[(long long)(m + L) * nring + ring];
            }
            if (ph0 != 0.0 && m != 0) {
                double sn, cs;
                sincos(m * ph0, &sn, &cs);
                h = cmul(h, make_double2(cs, sn));
            }
            ax = ax + cvt<T>(h.x);
            ay = ay + cvt<T>(h.y);
        }
        buf[qi] = mk<T>(ax, ay);
    }
    __syncthreads();
    mr_fft<T>(buf, N, st, K, tw);
    const long long o = ofs[ring];
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        const C z = buf[pos[p]];
        out0[o + p] = to_d(z.x);
        if (spin != 0) out1[o + p] = to_d(z.y);
    }
}

bool ring_mr_available(const cunusht_plan_s *P) { return P->mr_nst > 0 && !P->ring_bluestein; }

int ring_synth_mr_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *Hgl, long long hbs, double *out0,
                        double *out1, long long obs, cudaStream_t st) {
    MrStages s;
    s.n = P->mr_nst;
    for (int i = 0; i < MR_MAXST; ++i) {
        s.R[i] = i < s.n ? P->mr_R[i] : 1;
        s.Ls[i] = i < s.n ? P->mr_Ls[i] : 1;
        s.coff[i] = i < s.n ? P->mr_coff[i] : 0;
    }
    const int N = P->nph_uniform;
    const dim3 grid(P->nring, nreq);
    if (P->ring_df) {
        const size_t sm = sizeof(dcplx) * ((size_t)MR_KMAX + N);
        if (sm > 48 * 1024)
            CU_TRY(cudaFuncSetAttribute(k_ring_synth_mr<dfl>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_ring_synth_mr<dfl><<<grid, MR_TPB, sm, st>>>(Hgl, P->nring, P->lmax, spin, N, P->d_ring_phi0,
                                                      P->d_ring_ofs, s, (const dcplx *)P->d_mr_twdf, P->d_mr_pos,
                                                      out0, out1, hbs, obs);
    } else {
        const size_t sm = sizeof(double2) * ((size_t)MR_KMAX + N);
        if (sm > 48 * 1024)
            CU_TRY(cudaFuncSetAttribute(k_ring_synth_mr<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sm));
        k_ring_synth_mr<double><<<grid, MR_TPB, sm, st>>>(Hgl, P->nring, P->lmax, spin, N, P->d_ring_phi0,
                                                         P->d_ring_ofs, s, P->d_mr_tw64, P->d_mr_pos, out0, out1,
                                                         hbs, obs);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

}  // namespace cunusht

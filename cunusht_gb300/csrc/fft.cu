// FFT stages of the nuSHT pipeline: shared-memory Stockham FFTs (radix 2/4/8/16
// butterflies in registers, twiddles from a table), used by
//   * the theta pass: per phi-mode column, extend the CC rings to the 2 pi theta
//     torus (the reference's doubling, doubling.cu:180-201), FFT, multiply by the
//     nuFFT kernel deconvolution, zero-pad to the oversampled length, inverse
//     FFT -- together the reference's fft2 (GPU_nufft_transformer.py:274-278)
//     and the deconvolve/pad/fine-FFT half of cuFINUFFT type 2 (:292-298);
//     its adjoint is the type-1 half, ifft2 and the adjoint doubling (:475-480);
//   * the phi pass: per fine-grid row, Fourier modes m -> longitudes;
//   * the ring transform on the pointing geometry via Bluestein's chirp-z
//     algorithm (any ring length, e.g. 4095 = 3^2*5*7*13 or the prime 8191),
//     which SHTns performs inside synth_grad (GPU_sht_transformer.py:95).
#include <type_traits>

#include "common.cuh"
#include "kernels.cuh"

namespace cunusht {

// ------------------------------------------------------------ register DFTs
template <typename C> __device__ __forceinline__ void dft2(C &a, C &b) {
    C t = a;
    a = cadd(a, b);
    b = csub(t, b);
}

template <typename C> __device__ __forceinline__ void dft4(C &v0, C &v1, C &v2, C &v3, int dir) {
    C a = cadd(v0, v2), b = csub(v0, v2), c = cadd(v1, v3), d = cmul_idir(csub(v1, v3), dir);
    v0 = cadd(a, c);
    v2 = csub(a, c);
    v1 = cadd(b, d);
    v3 = csub(b, d);
}

template <typename T> __device__ __forceinline__ void dft8(cplx<T> *v, int dir) {
    using C = cplx<T>;
    dft4(v[0], v[2], v[4], v[6], dir);
    dft4(v[1], v[3], v[5], v[7], dir);
    const T r = cvt<T>(0.70710678118654752440084436210485);
    C o1 = v[3], o2 = v[5], o3 = v[7];
    // w^1 = (1 + dir i)/sqrt2, w^2 = dir i, w^3 = (-1 + dir i)/sqrt2
    C t1 = mk<T>(r * (o1.x - dir * o1.y), r * (o1.y + dir * o1.x));
    C t2 = cmul_idir(o2, dir);
    C t3 = mk<T>(r * (-o3.x - dir * o3.y), r * (-o3.y + dir * o3.x));
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, t1);
    v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2);
    v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3);
    v[7] = csub(e3, t3);
}

template <typename T> __device__ __forceinline__ void dft16(cplx<T> *v, int dir) {
    using C = cplx<T>;
    C e[8], o[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        e[i] = v[2 * i];
        o[i] = v[2 * i + 1];
    }
    dft8<T>(e, dir);
    dft8<T>(o, dir);
    const T cs[8] = {cvt<T>(1.0),
                     cvt<T>(0.92387953251128675612818318939679),
                     cvt<T>(0.70710678118654752440084436210485),
                     cvt<T>(0.38268343236508977172845998403040),
                     cvt<T>(0.0),
                     cvt<T>(-0.38268343236508977172845998403040),
                     cvt<T>(-0.70710678118654752440084436210485),
                     cvt<T>(-0.92387953251128675612818318939679)};
    const T sn[8] = {cvt<T>(0.0),
                     cvt<T>(0.38268343236508977172845998403040),
                     cvt<T>(0.70710678118654752440084436210485),
                     cvt<T>(0.92387953251128675612818318939679),
                     cvt<T>(1.0),
                     cvt<T>(0.92387953251128675612818318939679),
                     cvt<T>(0.70710678118654752440084436210485),
                     cvt<T>(0.38268343236508977172845998403040)};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        C w = mk<T>(cs[q], dir * sn[q]);
        C t = cmul(o[q], w);
        v[q] = cadd(e[q], t);
        v[q + 8] = csub(e[q], t);
    }
}

template <typename T, int RAD> __device__ __forceinline__ void dftR(cplx<T> *v, int dir) {
    if constexpr (RAD == 2) dft2(v[0], v[1]);
    else if constexpr (RAD == 4) dft4(v[0], v[1], v[2], v[3], dir);
    else if constexpr (RAD == 8) dft8<T>(v, dir);
    else dft16<T>(v, dir);
}

// One Stockham pass (Govindaraju et al. 2008 formulation), in place in shared
// memory.  Each of the nthr = N / E active threads owns exactly E elements
// (NB butterflies of R points, E = NB R, all compile-time), so the butterfly
// data stays in registers: loads, barrier, twiddle + R-point DFT, stores,
// barrier.
template <typename T, int R, int NB>
__device__ __forceinline__ void fft_pass_e(cplx<T> *buf, int N, int Ns, int dir,
                                           const cplx<T> *__restrict__ tw, int twstride, int nthr) {
    using C = cplx<T>;
    const int nb = N / R;  // == nthr * NB
    const bool act = (int)threadIdx.x < nthr;
    C v[NB][R];
    if (act) {
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            const int j = threadIdx.x + c * nthr;
#pragma unroll
            for (int r = 0; r < R; ++r) v[c][r] = buf[j + r * nb];
        }
    }
    __syncthreads();
    if (act) {
        const int tstep = (N / (Ns * R)) * twstride;
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            const int j = threadIdx.x + c * nthr;
            const int k = j & (Ns - 1);
            if (Ns > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    C w = tw[r * k * tstep];
                    if (dir > 0) w.y = -w.y;
                    v[c][r] = cmul(v[c][r], w);
                }
            }
            dftR<T, R>(v[c], dir);
            const int idxD = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) buf[idxD + r * Ns] = v[c][r];
            // one butterfly at a time: keeps the twiddle loads and DFT
            // temporaries of the other butterflies out of the live set
            asm volatile("" ::: "memory");
        }
    }
    __syncthreads();
}

// Whole transform with E elements per thread; radices up to min(E, RMAX) with
// RMAX = 16 for float and 8 for double / double-float (register budget).
template <typename T, int E, int LMAX = (std::is_same<T, float>::value ? 4 : 3)>
__device__ __forceinline__ void fft_smem_e(cplx<T> *buf, int N, int dir, const cplx<T> *__restrict__ tw, int TW) {
    constexpr int LE = (E >= 16) ? 4 : (E >= 8) ? 3 : (E >= 4) ? 2 : 1;
    constexpr int LR = LE < LMAX ? LE : LMAX;
    const int nthr = N / E;
    const int twstride = TW / N;
    int rem = __ffs(N) - 1;
    int Ns = 1;
    while (rem > 0) {
        const int r = rem < LR ? rem : LR;
        if (r == 4) {
            if constexpr (LR >= 4) fft_pass_e<T, 16, E / 16>(buf, N, Ns, dir, tw, twstride, nthr);
        } else if (r == 3) {
            if constexpr (LR >= 3) fft_pass_e<T, 8, E / 8>(buf, N, Ns, dir, tw, twstride, nthr);
        } else if (r == 2) {
            if constexpr (LR >= 2) fft_pass_e<T, 4, E / 4>(buf, N, Ns, dir, tw, twstride, nthr);
        } else {
            fft_pass_e<T, 2, E / 2>(buf, N, Ns, dir, tw, twstride, nthr);
        }
        Ns <<= r;
        rem -= r;
    }
}

// In-place FFT of length N (power of two, 2 <= N <= 16 blockDim; 32 blockDim
// for float) in shared memory.  dir = -1: X_k = sum_n x_n e^{-2 pi i nk/N};
// dir = +1: the unnormalised inverse.  tw[t] = e^{-2 pi i t / TW}, N | TW.
template <typename T>
__device__ void fft_smem(cplx<T> *buf, int N, int dir, const cplx<T> *__restrict__ tw, int TW) {
    const int B = blockDim.x;
    if (N > 16 * B) {
        if constexpr (std::is_same<T, float>::value) fft_smem_e<T, 32, 3>(buf, N, dir, tw, TW);
    } else if (N > 8 * B) {
        // 16 elements per thread: radix <= 8 for float, <= 4 for double and
        // double-float keeps the pass within the 128-register budget of a
        // 512-thread block
        if constexpr (std::is_same<T, float>::value) fft_smem_e<T, 16, 3>(buf, N, dir, tw, TW);
        else fft_smem_e<T, 16, 2>(buf, N, dir, tw, TW);
    } else if (N > 4 * B) {
        fft_smem_e<T, 8, 3>(buf, N, dir, tw, TW);
    } else if (N > 2 * B) {
        fft_smem_e<T, 4>(buf, N, dir, tw, TW);
    } else {
        fft_smem_e<T, 2>(buf, N, dir, tw, TW);
    }
}

size_t fft_smem_bytes(int N, bool f32) { return (size_t)N * (f32 ? sizeof(float2) : sizeof(double2)); }

template <typename T> __device__ __forceinline__ cplx<T> czero() { return mk<T>(cvt<T>(0.0), cvt<T>(0.0)); }

__device__ __forceinline__ int wrapi(int n, int N) {
    n %= N;
    return n < 0 ? n + N : n;
}

// ------------------------------------------------------------ theta pass
template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_theta_fwd(const double2 *__restrict__ H, int ldH, int Nt, int Ntf, int spin, int mofs, int L,
                const double *__restrict__ Dth, const double *__restrict__ Dph,
                cplx<T> *__restrict__ F, int ncols, int n_lo, int nrows,
                const cplx<T> *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int c = blockIdx.x;
    const int m = c - mofs;
    const double sgn = ((abs(m) + spin) & 1) ? -1.0 : 1.0;
    const double2 *col = H + (long long)c * ldH;
    const int half = Nt / 2;
    for (int k = threadIdx.x; k < Nt; k += blockDim.x) {
        const bool lo = k <= half;
        const double2 v = lo ? col[k] : col[Nt - k];
        const double s = lo ? 1.0 : sgn;
        buf[k] = mk<T>(cvt<T>(v.x * s), cvt<T>(v.y * s));
    }
    __syncthreads();
    fft_smem<T>(buf, Nt, -1, tw, TW);
    const double dm = Dph[m + L];
    for (int i = threadIdx.x; i < half - 1; i += blockDim.x) {
        const int src = Nt - 1 - i;  // kappa = -(i+1)
        buf[Ntf - 1 - i] = cscale(buf[src], cvt<T>(Dth[src] * dm));
    }
    for (int i = threadIdx.x; i < half; i += blockDim.x) buf[i] = cscale(buf[i], cvt<T>(Dth[i] * dm));
    __syncthreads();
    for (int i = half + threadIdx.x; i <= Ntf - half; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    fft_smem<T>(buf, Ntf, +1, tw, TW);
    for (int r = threadIdx.x; r < nrows; r += blockDim.x)
        F[(long long)r * ncols + c] = buf[wrapi(r + n_lo, Ntf)];
}

template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_theta_adj(const cplx<T> *__restrict__ F, int ncols, int n_lo, int nrows, int Nt, int Ntf,
                int spin, int mofs, int L, const double *__restrict__ Dth,
                const double *__restrict__ Dph, double2 *__restrict__ H, int ldH,
                const cplx<T> *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int c = blockIdx.x;
    const int m = c - mofs;
    const T sgn = cvt<T>(((abs(m) + spin) & 1) ? -1.0 : 1.0);
    for (int i = threadIdx.x; i < Ntf; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    for (int r = threadIdx.x; r < nrows; r += blockDim.x)
        buf[wrapi(r + n_lo, Ntf)] = F[(long long)r * ncols + c];
    __syncthreads();
    fft_smem<T>(buf, Ntf, -1, tw, TW);
    const int half = Nt / 2;
    const double dm = Dph[m + L];
    for (int i = threadIdx.x; i < half - 1; i += blockDim.x) {
        const int dst = Nt - 1 - i;  // kappa = -(i+1)
        buf[dst] = cscale(buf[Ntf - 1 - i], cvt<T>(Dth[dst] * dm));
    }
    for (int i = threadIdx.x; i < half; i += blockDim.x) buf[i] = cscale(buf[i], cvt<T>(Dth[i] * dm));
    if (threadIdx.x == 0) buf[half] = czero<T>();
    __syncthreads();
    fft_smem<T>(buf, Nt, +1, tw, TW);
    double2 *col = H + (long long)c * ldH;
    for (int k = threadIdx.x; k <= half; k += blockDim.x) {
        cplx<T> v = buf[k];
        if (k > 0 && k < half) v = cadd(v, cscale(buf[Nt - k], sgn));
        col[k] = make_double2(to_d(v.x), to_d(v.y));
    }
}

// ------------------------------------------------------------ phi pass
// spin 0: two real rows per block packed as one complex transform
template <typename T, typename TU>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_fwd_s0(const cplx<T> *__restrict__ F, int ncols, int nrows, int Npf, TU *__restrict__ U,
                 const cplx<T> *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int r1 = 2 * blockIdx.x, r2 = r1 + 1;
    const bool has2 = r2 < nrows;
    for (int i = threadIdx.x; i < Npf; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    for (int m = threadIdx.x; m < ncols; m += blockDim.x) {
        const cplx<T> a = F[(long long)r1 * ncols + m];
        const cplx<T> b = has2 ? F[(long long)r2 * ncols + m] : czero<T>();
        if (m == 0) {
            buf[0] = mk<T>(a.x, b.x);
        } else {
            buf[m] = mk<T>(a.x - b.y, a.y + b.x);
            buf[Npf - m] = mk<T>(a.x + b.y, b.x - a.y);
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Npf, +1, tw, TW);
    TU *u1 = U + (long long)r1 * Npf;
    TU *u2 = U + (long long)r2 * Npf;
    for (int p = threadIdx.x; p < Npf; p += blockDim.x) {
        const cplx<T> z = buf[p];
        u1[p] = to_t<TU>(z.x);
        if (has2) u2[p] = to_t<TU>(z.y);
    }
}

template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_adj_s0(const T *__restrict__ U, int nrows, int Npf, cplx<T> *__restrict__ F, int ncols,
                 const cplx<T> *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int r1 = 2 * blockIdx.x, r2 = r1 + 1;
    const bool has2 = r2 < nrows;
    const T *u1 = U + (long long)r1 * Npf;
    const T *u2 = U + (long long)r2 * Npf;
    for (int p = threadIdx.x; p < Npf; p += blockDim.x) buf[p] = mk<T>(u1[p], has2 ? u2[p] : cvt<T>(0.0));
    __syncthreads();
    fft_smem<T>(buf, Npf, -1, tw, TW);
    for (int m = threadIdx.x; m < ncols; m += blockDim.x) {
        const cplx<T> zm = buf[m];
        const cplx<T> zn = buf[m == 0 ? 0 : Npf - m];
        // U1 = (zm + conj zn)/2 ; U2 = (zm - conj zn)/(2i)
        F[(long long)r1 * ncols + m] = mk<T>(cvt<T>(0.5) * (zm.x + zn.x), cvt<T>(0.5) * (zm.y - zn.y));
        if (has2) F[(long long)r2 * ncols + m] = mk<T>(cvt<T>(0.5) * (zm.y + zn.y), cvt<T>(-0.5) * (zm.x - zn.x));
    }
}

// spin s: one complex row per block, columns c = m + L for m in [-L, L]
template <typename T, typename TU>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_fwd_spin(const cplx<T> *__restrict__ F, int L, int Npf, cplx<TU> *__restrict__ U,
                   const cplx<T> *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int r = blockIdx.x;
    const int ncols = 2 * L + 1;
    for (int i = threadIdx.x; i < Npf; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) buf[wrapi(c - L, Npf)] = F[(long long)r * ncols + c];
    __syncthreads();
    fft_smem<T>(buf, Npf, +1, tw, TW);
    for (int p = threadIdx.x; p < Npf; p += blockDim.x) U[(long long)r * Npf + p] = ccast<TU>(buf[p]);
}

template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_adj_spin(const cplx<T> *__restrict__ U, int L, int Npf, cplx<T> *__restrict__ F,
                   const cplx<T> *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int r = blockIdx.x;
    const int ncols = 2 * L + 1;
    for (int p = threadIdx.x; p < Npf; p += blockDim.x) buf[p] = U[(long long)r * Npf + p];
    __syncthreads();
    fft_smem<T>(buf, Npf, -1, tw, TW);
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) F[(long long)r * ncols + c] = buf[wrapi(c - L, Npf)];
}

// ------------------------------------------------------------ ring transform (Bluestein)
// z_p = sum_m h_m e^{i m (phi0 + 2 pi p / N)}, p < N, for one ring per block.
// spin 0: real output from m in [0, L] (h_{-m} = conj h_m); spin s: complex.
// T = double (plain path) or dfl (mixed path); tables are given in T.
template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_ring_synth(const double2 *__restrict__ Hgl, int nring, int L, int spin,
                 const double *__restrict__ phi0, const long long *__restrict__ ofs, int N, int Mb,
                 const cplx<T> *__restrict__ chirp, const cplx<T> *__restrict__ bker,
                 double *__restrict__ out0, double *__restrict__ out1,
                 const cplx<T> *__restrict__ tw, int TW) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *buf = reinterpret_cast<C *>(smem_raw);
    const int ring = blockIdx.x;
    const double ph0 = phi0[ring];
    for (int i = threadIdx.x; i < Mb; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    if (spin == 0) {
        for (int m = threadIdx.x; m <= L; m += blockDim.x) {
            double2 h = Hgl[(long long)m * nring + ring];
            if (m == 0) {
                buf[0] = mk<T>(cvt<T>(h.x), cvt<T>(0.0));
            } else {
                if (ph0 != 0.0) {
                    double sn, cs;
                    sincos(m * ph0, &sn, &cs);
                    h = cmul(h, make_double2(cs, sn));
                }
                const C hc = mk<T>(cvt<T>(h.x), cvt<T>(h.y));
                buf[m] = cmul(hc, chirp[m]);
                buf[N - m] = cmul(cconj(hc), chirp[N - m]);
            }
        }
    } else {
        for (int cidx = threadIdx.x; cidx < 2 * L + 1; cidx += blockDim.x) {
            const int m = cidx - L;
            double2 h = Hgl[(long long)cidx * nring + ring];
            if (ph0 != 0.0) {
                double sn, cs;
                sincos(m * ph0, &sn, &cs);
                h = cmul(h, make_double2(cs, sn));
            }
            const int q = wrapi(m, N);
            buf[q] = cmul(mk<T>(cvt<T>(h.x), cvt<T>(h.y)), chirp[q]);
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Mb, -1, tw, TW);
    for (int i = threadIdx.x; i < Mb; i += blockDim.x) buf[i] = cmul(buf[i], bker[i]);
    __syncthreads();
    fft_smem<T>(buf, Mb, +1, tw, TW);
    const long long o = ofs[ring];
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        const C z = cmul(buf[p], chirp[p]);
        out0[o + p] = to_d(z.x);
        if (spin != 0) out1[o + p] = to_d(z.y);
    }
}

// split FP64 complex tables into double-float ones (plan set-up)
__global__ void k_split_c128(const double2 *__restrict__ in, long long n, dcplx *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dcplx r;
    r.x = df_from(in[i].x);
    r.y = df_from(in[i].y);
    out[i] = r;
}

int split_c128_to_df(const double2 *in, long long n, void *out, cudaStream_t st) {
    if (n == 0) return CUNUSHT_OK;
    k_split_c128<<<(int)((n + 255) / 256), 256, 0, st>>>(in, n, (dcplx *)out);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// h'_m = e^{-i m phi0} sum_p z'_p e^{-2 pi i m p / N} (adjoint of k_ring_synth)
__global__ void __launch_bounds__(FFT_TPB)
    k_ring_adj(const double *__restrict__ in0, const double *__restrict__ in1, int nring, int L,
               int spin, const double *__restrict__ phi0, const long long *__restrict__ ofs, int N,
               int Mb, const double2 *__restrict__ chirp, const double2 *__restrict__ bker,
               double2 *__restrict__ Hgl, const double2 *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *buf = reinterpret_cast<double2 *>(smem_raw);
    const int ring = blockIdx.x;
    const double ph0 = phi0[ring];
    const long long o = ofs[ring];
    for (int i = threadIdx.x; i < Mb; i += blockDim.x) buf[i] = make_double2(0, 0);
    __syncthreads();
    // Bluestein on conj(z'): c_p = conj(z'_p)
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        const double2 z = make_double2(in0[o + p], spin ? -in1[o + p] : 0.0);
        buf[p] = cmul(z, chirp[p]);
    }
    __syncthreads();
    fft_smem<double>(buf, Mb, -1, tw, TW);
    for (int i = threadIdx.x; i < Mb; i += blockDim.x) buf[i] = cmul(buf[i], bker[i]);
    __syncthreads();
    fft_smem<double>(buf, Mb, +1, tw, TW);
    if (spin == 0) {
        for (int m = threadIdx.x; m <= L; m += blockDim.x) {
            const double2 y = cconj(cmul(buf[m], chirp[m]));  // sum_p z' e^{-2 pi i m p/N}
            double s, c;
            sincos(m * ph0, &s, &c);
            Hgl[(long long)m * nring + ring] = cmul(y, make_double2(c, -s));
        }
    } else {
        for (int cidx = threadIdx.x; cidx < 2 * L + 1; cidx += blockDim.x) {
            const int m = cidx - L;
            const int q = wrapi(m, N);
            const double2 y = cconj(cmul(buf[q], chirp[q]));
            double s, c;
            sincos(m * ph0, &s, &c);
            Hgl[(long long)cidx * nring + ring] = cmul(y, make_double2(c, -s));
        }
    }
}

// ------------------------------------------------------------ whole-array FFT (setup only)
__global__ void __launch_bounds__(FFT_TPB)
    k_fft_global(double2 *data, int N, int dir, const double2 *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *buf = reinterpret_cast<double2 *>(smem_raw);
    for (int i = threadIdx.x; i < N; i += blockDim.x) buf[i] = data[i];
    __syncthreads();
    fft_smem<double>(buf, N, dir, tw, TW);
    for (int i = threadIdx.x; i < N; i += blockDim.x) data[i] = buf[i];
}

// ------------------------------------------------------------ host launchers
template <typename K> static int set_smem(K kernel, size_t bytes) {
    if (bytes > 48 * 1024) CU_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return CUNUSHT_OK;
}

int fft_global_f64(double2 *data, int N, int dir, const double2 *tw, int TW, cudaStream_t st) {
    size_t sm = fft_smem_bytes(N, false);
    RC_TRY(set_smem(k_fft_global, sm));
    k_fft_global<<<1, FFT_TPB, sm, st>>>(data, N, dir, tw, TW);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int theta_fwd(const cunusht_plan_s *P, int spin, const double2 *H, void *F, cudaStream_t st) {
    const int L = P->lmax;
    const int ncols = spin ? 2 * L + 1 : L + 1;
    const int mofs = spin ? L : 0;
    size_t sm = fft_smem_bytes(P->Ntf, P->grid_fp32);
    if (P->grid_fp32) {
        RC_TRY(set_smem(k_theta_fwd<float>, sm));
        k_theta_fwd<float><<<ncols, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                       (float2 *)F, ncols, P->n_lo, P->nrows, P->d_tw32, P->TW);
    } else if (P->fft_df) {
        RC_TRY(set_smem(k_theta_fwd<dfl>, sm));
        k_theta_fwd<dfl><<<ncols, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                     (dcplx *)F, ncols, P->n_lo, P->nrows, (const dcplx *)P->d_twdf,
                                                     P->TW);
    } else {
        RC_TRY(set_smem(k_theta_fwd<double>, sm));
        k_theta_fwd<double><<<ncols, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                        (double2 *)F, ncols, P->n_lo, P->nrows, P->d_tw64, P->TW);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int theta_adj(const cunusht_plan_s *P, int spin, const void *F, double2 *H, cudaStream_t st) {
    const int L = P->lmax;
    const int ncols = spin ? 2 * L + 1 : L + 1;
    const int mofs = spin ? L : 0;
    size_t sm = fft_smem_bytes(P->Ntf, P->grid_fp32);
    if (P->grid_fp32) {
        RC_TRY(set_smem(k_theta_adj<float>, sm));
        k_theta_adj<float><<<ncols, FFT_TPB, sm, st>>>((const float2 *)F, ncols, P->n_lo, P->nrows, P->Nt, P->Ntf, spin,
                                                       mofs, L, P->d_Dth, P->d_Dph, H, P->ncc, P->d_tw32, P->TW);
    } else {
        RC_TRY(set_smem(k_theta_adj<double>, sm));
        k_theta_adj<double><<<ncols, FFT_TPB, sm, st>>>((const double2 *)F, ncols, P->n_lo, P->nrows, P->Nt, P->Ntf,
                                                        spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc, P->d_tw64, P->TW);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int phi_fwd(const cunusht_plan_s *P, int spin, const void *F, void *U, cudaStream_t st) {
    const int L = P->lmax;
    size_t sm = fft_smem_bytes(P->Npf, P->grid_fp32);
    if (spin == 0) {
        const int nb = (P->nrows + 1) / 2;
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_phi_fwd_s0<float, float>, sm));
            k_phi_fwd_s0<float, float><<<nb, FFT_TPB, sm, st>>>((const float2 *)F, L + 1, P->nrows, P->Npf,
                                                                (float *)U, P->d_tw32, P->TW);
        } else if (P->fft_df) {
            RC_TRY(set_smem(k_phi_fwd_s0<dfl, float>, sm));
            k_phi_fwd_s0<dfl, float><<<nb, FFT_TPB, sm, st>>>((const dcplx *)F, L + 1, P->nrows, P->Npf,
                                                              (float *)U, (const dcplx *)P->d_twdf, P->TW);
        } else if (P->fwd_u32) {
            RC_TRY(set_smem(k_phi_fwd_s0<double, float>, sm));
            k_phi_fwd_s0<double, float><<<nb, FFT_TPB, sm, st>>>((const double2 *)F, L + 1, P->nrows, P->Npf,
                                                                 (float *)U, P->d_tw64, P->TW);
        } else {
            RC_TRY(set_smem(k_phi_fwd_s0<double, double>, sm));
            k_phi_fwd_s0<double, double><<<nb, FFT_TPB, sm, st>>>((const double2 *)F, L + 1, P->nrows, P->Npf,
                                                                  (double *)U, P->d_tw64, P->TW);
        }
    } else {
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_phi_fwd_spin<float, float>, sm));
            k_phi_fwd_spin<float, float><<<P->nrows, FFT_TPB, sm, st>>>((const float2 *)F, L, P->Npf,
                                                                        (float2 *)U, P->d_tw32, P->TW);
        } else if (P->fft_df) {
            RC_TRY(set_smem(k_phi_fwd_spin<dfl, float>, sm));
            k_phi_fwd_spin<dfl, float><<<P->nrows, FFT_TPB, sm, st>>>((const dcplx *)F, L, P->Npf, (float2 *)U,
                                                                      (const dcplx *)P->d_twdf, P->TW);
        } else if (P->fwd_u32) {
            RC_TRY(set_smem(k_phi_fwd_spin<double, float>, sm));
            k_phi_fwd_spin<double, float><<<P->nrows, FFT_TPB, sm, st>>>((const double2 *)F, L, P->Npf,
                                                                         (float2 *)U, P->d_tw64, P->TW);
        } else {
            RC_TRY(set_smem(k_phi_fwd_spin<double, double>, sm));
            k_phi_fwd_spin<double, double><<<P->nrows, FFT_TPB, sm, st>>>((const double2 *)F, L, P->Npf,
                                                                          (double2 *)U, P->d_tw64, P->TW);
        }
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int phi_adj(const cunusht_plan_s *P, int spin, const void *U, void *F, cudaStream_t st) {
    const int L = P->lmax;
    size_t sm = fft_smem_bytes(P->Npf, P->grid_fp32);
    if (spin == 0) {
        const int nb = (P->nrows + 1) / 2;
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_phi_adj_s0<float>, sm));
            k_phi_adj_s0<float><<<nb, FFT_TPB, sm, st>>>((const float *)U, P->nrows, P->Npf, (float2 *)F, L + 1,
                                                         P->d_tw32, P->TW);
        } else {
            RC_TRY(set_smem(k_phi_adj_s0<double>, sm));
            k_phi_adj_s0<double><<<nb, FFT_TPB, sm, st>>>((const double *)U, P->nrows, P->Npf, (double2 *)F, L + 1,
                                                          P->d_tw64, P->TW);
        }
    } else {
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_phi_adj_spin<float>, sm));
            k_phi_adj_spin<float><<<P->nrows, FFT_TPB, sm, st>>>((const float2 *)U, L, P->Npf, (float2 *)F,
                                                                 P->d_tw32, P->TW);
        } else {
            RC_TRY(set_smem(k_phi_adj_spin<double>, sm));
            k_phi_adj_spin<double><<<P->nrows, FFT_TPB, sm, st>>>((const double2 *)U, L, P->Npf, (double2 *)F,
                                                                  P->d_tw64, P->TW);
        }
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int ring_synth(const cunusht_plan_s *P, int spin, const double2 *Hgl, double *out0, double *out1,
               cudaStream_t st) {
    size_t sm = fft_smem_bytes(P->Mb, false);
    if (P->fft_df && P->d_chirp_df) {
        RC_TRY(set_smem(k_ring_synth<dfl>, sm));
        k_ring_synth<dfl><<<P->nring, FFT_TPB, sm, st>>>(Hgl, P->nring, P->lmax, spin, P->d_ring_phi0,
                                                         P->d_ring_ofs, P->nph_uniform, P->Mb,
                                                         (const dcplx *)P->d_chirp_df, (const dcplx *)P->d_bker_df,
                                                         out0, out1, (const dcplx *)P->d_twdf, P->TW);
    } else {
        RC_TRY(set_smem(k_ring_synth<double>, sm));
        k_ring_synth<double><<<P->nring, FFT_TPB, sm, st>>>(Hgl, P->nring, P->lmax, spin, P->d_ring_phi0,
                                                            P->d_ring_ofs, P->nph_uniform, P->Mb, P->d_chirp,
                                                            P->d_bker, out0, out1, P->d_tw64, P->TW);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int ring_adjoint(const cunusht_plan_s *P, int spin, const double *in0, const double *in1,
                 double2 *Hgl, cudaStream_t st) {
    size_t sm = fft_smem_bytes(P->Mb, false);
    RC_TRY(set_smem(k_ring_adj, sm));
    k_ring_adj<<<P->nring, FFT_TPB, sm, st>>>(in0, in1, P->nring, P->lmax, spin, P->d_ring_phi0, P->d_ring_ofs,
                                              P->nph_uniform, P->Mb, P->d_chirp, P->d_bker, Hgl, P->d_tw64,
                                              P->TW);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

}  // namespace cunusht

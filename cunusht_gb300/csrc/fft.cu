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
// Position of entry u of the quarter table in shared memory: the low bits
// (one 128-byte row of 8 double / double-float or 16 float entries) XORed with
// every higher group of as many bits, so that reads at any power-of-two
// stride (the twiddles of one pass, k consecutive) fall in distinct banks.
// Entries stay within their aligned group: the table takes M/4 + 16 slots.
template <typename T> __device__ __forceinline__ int tw_swz(int u) {
    if constexpr (sizeof(cplx<T>) == 16) return u ^ (((u >> 3) ^ (u >> 6) ^ (u >> 9) ^ (u >> 12)) & 7);
    else return u ^ (((u >> 4) ^ (u >> 8) ^ (u >> 12)) & 15);
}

// e^{-2 pi i t / M} for 0 <= t < M from the quarter table S[u] = e^{-2 pi i u / M},
// u <= M/4, held in shared memory: t = q M/4 + u gives (-i)^q S[u]; lq = log2(M/4)
template <typename T>
__device__ __forceinline__ cplx<T> tw_quarter(const cplx<T> *S, int t, int lq) {
    const int q = t >> lq, u = t & ((1 << lq) - 1);
    const cplx<T> w = S[tw_swz<T>(u)];
    T x = (q & 1) ? w.y : w.x;
    T y = (q & 1) ? w.x : w.y;
    if (q & 2) x = -x;
    if (q == 1 || q == 2) y = -y;
    return mk<T>(x, y);
}

template <typename T, int R, int NB>
__device__ __forceinline__ void fft_pass_e(cplx<T> *buf, int N, int Ns, int dir,
                                           const cplx<T> *__restrict__ stw, int M, int nthr) {
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
        const int tstep = M / (Ns * R);
        const int lq = __ffs(M) - 3;  // log2(M / 4), M a power of two
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            const int j = threadIdx.x + c * nthr;
            const int k = j & (Ns - 1);
            if (Ns > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    C w = tw_quarter<T>(stw, r * k * tstep, lq);
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
// l0 > 0: the first passes, of 2^l0 points in all, are already done (buf
// holds the output of a radix-2^l0 pass with Ns = 1).
template <typename T, int E, int LMAX = (std::is_same<T, float>::value ? 4 : 3)>
__device__ __forceinline__ void fft_smem_e(cplx<T> *buf, int N, int dir, const cplx<T> *__restrict__ stw, int M,
                                           int l0 = 0) {
    constexpr int LE = (E >= 16) ? 4 : (E >= 8) ? 3 : (E >= 4) ? 2 : 1;
    constexpr int LR = LE < LMAX ? LE : LMAX;
    const int nthr = N / E;
    int rem = __ffs(N) - 1 - l0;
    int Ns = 1 << l0;
    while (rem > 0) {
        const int r = rem < LR ? rem : LR;
        if (r == 4) {
            if constexpr (LR >= 4) fft_pass_e<T, 16, E / 16>(buf, N, Ns, dir, stw, M, nthr);
        } else if (r == 3) {
            if constexpr (LR >= 3) fft_pass_e<T, 8, E / 8>(buf, N, Ns, dir, stw, M, nthr);
        } else if (r == 2) {
            if constexpr (LR >= 2) fft_pass_e<T, 4, E / 4>(buf, N, Ns, dir, stw, M, nthr);
        } else {
            fft_pass_e<T, 2, E / 2>(buf, N, Ns, dir, stw, M, nthr);
        }
        Ns <<= r;
        rem -= r;
    }
}

// In-place FFT of length N (power of two, 2 <= N <= 16 blockDim) in shared
// memory.  dir = -1: X_k = sum_n x_n e^{-2 pi i nk/N}; dir = +1: the
// unnormalised inverse.  stw: the quarter twiddle table of length M >= N in
// shared memory (load_twiddles).  Longer transforms are split by output parity
// in the callers (sp_* of the plan).
template <typename T>
__device__ __forceinline__ void fft_smem(cplx<T> *buf, int N, int dir, const cplx<T> *__restrict__ stw, int M,
                                         int l0 = 0) {
    const int B = blockDim.x;
    if (N > 8 * B) {
        // 16 elements per thread: radix <= 8 for float, <= 4 for double and
        // double-float keeps the pass within the 128-register budget of a
        // 512-thread block
        if constexpr (std::is_same<T, float>::value) fft_smem_e<T, 16, 3>(buf, N, dir, stw, M, l0);
        else fft_smem_e<T, 16, 2>(buf, N, dir, stw, M, l0);
    } else if (N > 4 * B) {
        fft_smem_e<T, 8, 3>(buf, N, dir, stw, M, l0);
    } else if (N > 2 * B) {
        fft_smem_e<T, 4>(buf, N, dir, stw, M, l0);
    } else {
        fft_smem_e<T, 2>(buf, N, dir, stw, M, l0);
    }
}

// First radix-4 Stockham pass (Ns = 1) of a transform of N >= 4 points whose
// inputs x[j + N/4] and x[j + N/2] are zero for every j < N/4 (a zero-padded
// spectrum: modes |k| < N/4 at [0, N/4) and (3N/4, N)).  Butterfly j takes
// v0 = x[j], v3 = x[j + 3N/4] and stores its four outputs at 4j .. 4j + 3,
// which is what fft_pass_e<T, 4> writes for it; the transform then continues
// with fft_smem(..., l0 = 2).  Half the pass's additions, and the zero middle
// of the input is neither stored nor read.
template <typename T>
__device__ __forceinline__ void r4_first_pruned(cplx<T> *buf, int j, cplx<T> v0, cplx<T> v3, int dir) {
    const cplx<T> t = cmul_idir(v3, dir);
    buf[4 * j] = cadd(v0, v3);
    buf[4 * j + 1] = csub(v0, t);
    buf[4 * j + 2] = csub(v0, v3);
    buf[4 * j + 3] = cadd(v0, t);
}

// Shared memory of a transform kernel with an N-element buffer: the buffer
// plus its quarter twiddle table (N/4 + 1 entries, swizzled over N/4 + 16
// slots).  The twiddles are read in every butterfly; from global memory they
// were L2-latency loads (the data buffer leaves little L1), the first stall
// reason of these kernels.
size_t fft_smem_bytes(int N, bool f32) { return (size_t)(N + N / 4 + 16) * (f32 ? sizeof(float2) : sizeof(double2)); }

// S[u] = e^{-2 pi i u / M} for u <= M/4 from the plan's table tw[t] =
// e^{-2 pi i t / TW} (M | TW), placed after the M-element data buffer.  The
// first transform pass reads it only after a block barrier.
template <typename T>
__device__ __forceinline__ cplx<T> *load_twiddles(cplx<T> *buf, int M, const cplx<T> *__restrict__ tw, int TW) {
    cplx<T> *S = buf + M;
    const int st = TW / M;
    for (int u = threadIdx.x; u <= M / 4; u += blockDim.x) S[tw_swz<T>(u)] = tw[u * st];
    return S;
}

template <typename T> __device__ __forceinline__ cplx<T> czero() { return mk<T>(cvt<T>(0.0), cvt<T>(0.0)); }

// e^{dirsign 2 pi i k / TW'} from the table, tstep = TW / TW' (TW' | TW,
// |k| < TW'), dirsign = +-1
template <typename T>
__device__ __forceinline__ cplx<T> twk(const cplx<T> *__restrict__ tw, int k, int tstep, int dirsign) {
    cplx<T> w = tw[(k < 0 ? -k : k) * tstep];
    if ((k < 0) != (dirsign > 0)) w.y = -w.y;
    return w;
}

// a * b in the transform's type; double-float from the split factors (no FP64 product)
template <typename T> __device__ __forceinline__ T scale_of(double a, double b) { return cvt<T>(a * b); }
template <> __device__ __forceinline__ dfl scale_of<dfl>(double a, double b) { return df_mul(df_from(a), df_from(b)); }

__device__ __forceinline__ int wrapi(int n, int N) {
    n %= N;
    return n < 0 ? n + N : n;
}
// n mod N for N a power of two (also for negative n, two's complement)
__device__ __forceinline__ int wrap2(int n, int N) { return n & (N - 1); }

// ------------------------------------------------------------ theta pass
// SP = 2 (long columns): the 2 Nt-point inverse is done as two Nt-point
// inverses, one per output parity q = blockIdx.z: y_{2j+q} = sum_k X_k
// e^{i pi k q / Nt} e^{2 pi i k j / Nt} (X band-limited to |k| < Nt/2), each
// block repeating the forward Nt-point transform.  (A loop over q inside the
// block would put the inlined transforms in a loop, which ptxas compiles to a
// 32-register spilling kernel.)
template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_theta_fwd(const double2 *__restrict__ H, int ldH, int Nt, int Ntf, int spin, int mofs, int L,
                const double *__restrict__ Dth, const double *__restrict__ Dph,
                cplx<T> *__restrict__ F, int ncols, int n_lo, int nrows,
                const cplx<T> *__restrict__ tw, int TW, long long hbs, long long fbs, int SP) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int MTW = Ntf / SP;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    H += blockIdx.y * hbs;  // request of a batch
    F += blockIdx.y * fbs;
    const int q = blockIdx.z;
    const int c = blockIdx.x;
    const int m = c - mofs;
    const double sgn = ((abs(m) + spin) & 1) ? -1.0 : 1.0;
    const double2 *col = H + (long long)c * ldH;
    const int half = Nt / 2;
    const double dm = Dph[m + L];
    for (int k = threadIdx.x; k < Nt; k += blockDim.x) {
        const bool lo = k <= half;
        const double2 v = lo ? col[k] : col[Nt - k];
        const double s = lo ? 1.0 : sgn;
        buf[k] = mk<T>(cvt<T>(v.x * s), cvt<T>(v.y * s));
    }
    __syncthreads();
    fft_smem<T>(buf, Nt, -1, stw, MTW);
    if (SP == 1) {
        for (int i = threadIdx.x; i < half - 1; i += blockDim.x) {
            const int src = Nt - 1 - i;  // kappa = -(i+1)
            buf[Ntf - 1 - i] = cscale(buf[src], scale_of<T>(Dth[src], dm));
        }
        for (int i = threadIdx.x; i < half; i += blockDim.x) buf[i] = cscale(buf[i], scale_of<T>(Dth[i], dm));
        __syncthreads();
        for (int i = half + threadIdx.x; i <= Ntf - half; i += blockDim.x) buf[i] = czero<T>();
    } else {
        const int tstep = TW / Ntf;
        for (int i = threadIdx.x; i < Nt; i += blockDim.x) {
            // Dth[half] = 0 drops the Nyquist term
            cplx<T> v = cscale(buf[i], scale_of<T>(Dth[i], dm));
            if (q) v = cmul(v, twk<T>(tw, i < half ? i : i - Nt, tstep, +1));
            buf[i] = v;
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Ntf / SP, +1, stw, MTW);
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        const int n = wrap2(r + n_lo, Ntf);
        if (SP == 1) F[(long long)r * ncols + c] = buf[n];
        else if ((n & 1) == q) F[(long long)r * ncols + c] = buf[n >> 1];
    }
}

// Theta pass of two columns at once (transforms unsplit, SP = 1): the torus
// extensions of columns c1 = 2b and c2 = 2b + 1 have opposite symmetry
// (x_{-k} = s x_k with s = (-1)^(|m| + spin), and consecutive m alternate), so
// one complex transform of z = x1 + i x2 carries both:
//     X1_j = (Z_j + s1 Z_{-j}) / 2,   X2_j = (Z_j - s1 Z_{-j}) / (2i).
// The deconvolved spectra recombine as W = Y1 + i Y2, whose inverse
// w = y1 + i y2 separates the same way (the outputs keep the symmetry of their
// columns).  Half the transforms of k_theta_fwd; the separation adds an
// absolute error of the transform's rounding times the partner column.
template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_theta_fwd2(const double2 *__restrict__ H, int ldH, int Nt, int Ntf, int spin, int mofs, int L,
                 const double *__restrict__ Dth, const double *__restrict__ Dph, cplx<T> *__restrict__ F, int ncols,
                 int n_lo, int nrows, const cplx<T> *__restrict__ tw, int TW, long long hbs, long long fbs) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *buf = reinterpret_cast<C *>(smem_raw);
    const C *stw = load_twiddles<T>(buf, Ntf, tw, TW);
    H += blockIdx.y * hbs;  // request of a batch
    F += blockIdx.y * fbs;
    const int c1 = 2 * blockIdx.x, c2 = c1 + 1;
    const bool two = c2 < ncols;
    const int m1 = c1 - mofs;
    const double s1 = ((abs(m1) + spin) & 1) ? -1.0 : 1.0, s2 = -s1;
    const double2 *col1 = H + (long long)c1 * ldH, *col2 = H + (long long)c2 * ldH;
    const int half = Nt / 2;
    const double dm1 = Dph[m1 + L], dm2 = two ? Dph[m1 + 1 + L] : 0.0;
    for (int k = threadIdx.x; k < Nt; k += blockDim.x) {
        const bool lo = k <= half;
        const int kk = lo ? k : Nt - k;
        double2 v1 = col1[kk], v2 = two ? col2[kk] : make_double2(0.0, 0.0);
        if constexpr (std::is_same<T, dfl>::value) {
            // split first, combine in double-float: no FP64 arithmetic (s2 = -s1)
            dfl ax = df_from(v1.x), ay = df_from(v1.y), bx = df_from(v2.x), by = df_from(v2.y);
            if (!lo) {
                if (s1 < 0.0) ax = df_neg(ax), ay = df_neg(ay);
                else bx = df_neg(bx), by = df_neg(by);
            }
            buf[k] = mk<T>(df_add(ax, df_neg(by)), df_add(ay, bx));  // x1 + i x2
        } else {
            if (!lo) {
                v1 = make_double2(s1 * v1.x, s1 * v1.y);
                v2 = make_double2(s2 * v2.x, s2 * v2.y);
            }
            buf[k] = mk<T>(cvt<T>(v1.x - v2.y), cvt<T>(v1.y + v2.x));  // x1 + i x2
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Nt, -1, stw, Ntf);
    // separate, deconvolve, recombine; thread j owns the frequencies +-j
    // (reads j and Nt - j, writes j and Ntf - j: no other thread touches them);
    // the Nyquist term is dropped (Dth[half] = 0)
    const T hf = cvt<T>(0.5), ts1 = cvt<T>(s1), ts2 = cvt<T>(s2);
    for (int j = threadIdx.x; j < half; j += blockDim.x) {
        const int jn = j ? Nt - j : 0;
        const C zp = buf[j], zn = cscale(buf[jn], ts1);
        const C x1 = cscale(cadd(zp, zn), hf);
        const C d = cscale(csub(zp, zn), hf);
        const C x2 = mk<T>(d.y, -d.x);  // d / i
        const C y1 = cscale(x1, scale_of<T>(Dth[j], dm1)), y2 = cscale(x2, scale_of<T>(Dth[j], dm2));
        buf[j] = mk<T>(y1.x - y2.y, y1.y + y2.x);  // y1 + i y2
        if (j) {
            const C y1n = cscale(y1, ts1), y2n = cscale(y2, ts2);  // Y_{-j} = s Y_j (D even)
            buf[Ntf - j] = mk<T>(y1n.x - y2n.y, y1n.y + y2n.x);
        }
    }
    __syncthreads();
    // the inverse's input is zero in [half, Ntf - half] (Ntf / 4 = half): its
    // first radix-4 pass reads only x[j] and x[j + 3 Ntf / 4] (zero for j = 0),
    // up to four butterflies per thread (Ntf <= 16 blockDim)
    {
        C a[4], b[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int j = threadIdx.x + c * blockDim.x;
            if (j < half) {
                a[c] = buf[j];
                b[c] = j ? buf[j + 3 * half] : czero<T>();
            }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int j = threadIdx.x + c * blockDim.x;
            if (j < half) r4_first_pruned<T>(buf, j, a[c], b[c], +1);
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Ntf, +1, stw, Ntf, 2);
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        const int n = wrap2(r + n_lo, Ntf);
        const C wp = buf[n], wn = cscale(buf[wrap2(-n, Ntf)], ts1);
        F[(long long)r * ncols + c1] = cscale(cadd(wp, wn), hf);
        if (two) {
            const C d = cscale(csub(wp, wn), hf);
            F[(long long)r * ncols + c2] = mk<T>(d.y, -d.x);
        }
    }
}

// SP = 2: Z_k = E_k + e^{-i pi k / Nt} O_k with E / O the Nt-point transforms
// of the even / odd fine rows: launched for q = 1 (odd rows, phase applied,
// written to the scratch S, Nt values per column), then q = 0 (even rows plus
// S, deconvolution, inverse transform to the CC column).
template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_theta_adj(const cplx<T> *__restrict__ F, int ncols, int n_lo, int nrows, int Nt, int Ntf,
                int spin, int mofs, int L, const double *__restrict__ Dth,
                const double *__restrict__ Dph, double2 *__restrict__ H, int ldH,
                const cplx<T> *__restrict__ tw, int TW, int SP, int q, cplx<T> *__restrict__ S, long long fbs,
                long long hbs, long long sbs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int MTW = Ntf / SP;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    F += blockIdx.y * fbs;  // request of a batch
    H += blockIdx.y * hbs;
    S += blockIdx.y * sbs;
    const int c = blockIdx.x;
    const int m = c - mofs;
    const T sgn = cvt<T>(((abs(m) + spin) & 1) ? -1.0 : 1.0);
    const int half = Nt / 2;
    const double dm = Dph[m + L];
    const int Nb = Ntf / SP;  // forward transform length
    for (int i = threadIdx.x; i < Nb; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        const int n = wrap2(r + n_lo, Ntf);
        if (SP == 1) buf[n] = F[(long long)r * ncols + c];
        else if ((n & 1) == q) buf[n >> 1] = F[(long long)r * ncols + c];
    }
    __syncthreads();
    fft_smem<T>(buf, Nb, -1, stw, MTW);
    if (SP == 1) {
        for (int i = threadIdx.x; i < half - 1; i += blockDim.x) {
            const int dst = Nt - 1 - i;  // kappa = -(i+1)
            buf[dst] = cscale(buf[Ntf - 1 - i], scale_of<T>(Dth[dst], dm));
        }
        for (int i = threadIdx.x; i < half; i += blockDim.x) buf[i] = cscale(buf[i], scale_of<T>(Dth[i], dm));
        if (threadIdx.x == 0) buf[half] = czero<T>();
    } else {
        const int tstep = TW / Ntf;
        cplx<T> *sc = S + (long long)c * Nt;
        if (q) {
            for (int i = threadIdx.x; i < Nt; i += blockDim.x)
                sc[i] = cmul(buf[i], twk<T>(tw, i < half ? i : i - Nt, tstep, -1));
            return;
        }
        for (int i = threadIdx.x; i < Nt; i += blockDim.x)
            buf[i] = cscale(cadd(buf[i], sc[i]), scale_of<T>(Dth[i], dm));  // Dth[half] = 0
    }
    __syncthreads();
    fft_smem<T>(buf, Nt, +1, stw, MTW);
    double2 *col = H + (long long)c * ldH;
    for (int k = threadIdx.x; k <= half; k += blockDim.x) {
        cplx<T> v = buf[k];
        if (k > 0 && k < half) v = cadd(v, cscale(buf[Nt - k], sgn));
        col[k] = make_double2(to_d(v.x), to_d(v.y));
    }
}

// ------------------------------------------------------------ phi pass
// SP = 2 (long rows): U_{2j+q} = sum_m X_m e^{i pi m q / Np} e^{2 pi i m j / Np},
// Np = Npf / 2 >= 2L + 2 (no aliasing): one half-length inverse per parity,
// q = blockIdx.z in the forward kernels; the adjoint kernels are launched for
// q = 1 (writes F) and then q = 0 (adds to F).
// spin 0: two real rows per block packed as one complex transform
// PRUNE (SP = 1, Nb / 4 > L): first radix-4 pass done as the rows are read,
// as in k_phi_fwd_spin
template <typename T, typename TU, bool PRUNE = false>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_fwd_s0(const cplx<T> *__restrict__ F, int ncols, int nrows, int Npf, TU *__restrict__ U,
                 const cplx<T> *__restrict__ tw, int TW, long long fbs, long long ubs, int SP) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int MTW = Npf / SP;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    F += blockIdx.y * fbs;
    U += blockIdx.y * ubs;
    const int q = blockIdx.z;
    const int r1 = 2 * blockIdx.x, r2 = r1 + 1;
    const bool has2 = r2 < nrows;
    const int Nb = Npf / SP;
    const int tstep = TW / Npf;
    if constexpr (PRUNE) {
        // x[j] = a_j + i b_j (j <= L), x[j + 3 Nb / 4] = conj a_m + i conj b_m
        // at m = Nb / 4 - j (m <= L); x[0] = (Re a_0, Re b_0)
        const cplx<T> *f1 = F + (long long)r1 * ncols, *f2 = F + (long long)r2 * ncols;
        const int nb = Nb / 4;
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            cplx<T> v0 = czero<T>(), v3 = czero<T>();
            if (j < ncols) {
                const cplx<T> a = f1[j], b = has2 ? f2[j] : czero<T>();
                v0 = j ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x, b.x);
            }
            const int m = nb - j;
            if (m < ncols) {
                const cplx<T> a = f1[m], b = has2 ? f2[m] : czero<T>();
                v3 = mk<T>(a.x + b.y, b.x - a.y);
            }
            r4_first_pruned<T>(buf, j, v0, v3, +1);
        }
        __syncthreads();
        fft_smem<T>(buf, Nb, +1, stw, MTW, 2);
        TU *u1 = U + (long long)r1 * Npf;
        TU *u2 = U + (long long)r2 * Npf;
        for (int j = threadIdx.x; j < Nb; j += blockDim.x) {
            const cplx<T> z = buf[j];
            u1[j] = to_t<TU>(z.x);
            if (has2) u2[j] = to_t<TU>(z.y);
        }
        return;
    }
    for (int i = threadIdx.x; i < Nb; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    for (int m = threadIdx.x; m < ncols; m += blockDim.x) {
        const cplx<T> a = F[(long long)r1 * ncols + m];
        const cplx<T> b = has2 ? F[(long long)r2 * ncols + m] : czero<T>();
        if (m == 0) {
            buf[0] = mk<T>(a.x, b.x);
        } else {
            cplx<T> pp = mk<T>(a.x - b.y, a.y + b.x);  // a + i b at +m
            cplx<T> pn = mk<T>(a.x + b.y, b.x - a.y);  // conj a + i conj b at -m
            if (q) {
                pp = cmul(pp, twk<T>(tw, m, tstep, +1));
                pn = cmul(pn, twk<T>(tw, -m, tstep, +1));
            }
            buf[m] = pp;
            buf[Nb - m] = pn;
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Nb, +1, stw, MTW);
    TU *u1 = U + (long long)r1 * Npf;
    TU *u2 = U + (long long)r2 * Npf;
    for (int j = threadIdx.x; j < Nb; j += blockDim.x) {
        const cplx<T> z = buf[j];
        const int p = SP * j + q;
        u1[p] = to_t<TU>(z.x);
        if (has2) u2[p] = to_t<TU>(z.y);
    }
}

// TU: the grid's scalar type (double for the double-float transforms of the
// mixed plan, whose spread accumulates in FP64)
template <typename T, typename TU = T>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_adj_s0(const TU *__restrict__ U, int nrows, int Npf, cplx<T> *__restrict__ F, int ncols,
                 const cplx<T> *__restrict__ tw, int TW, int SP, int q, long long ubs, long long fbs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int MTW = Npf / SP;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    U += blockIdx.y * ubs;
    F += blockIdx.y * fbs;
    const int r1 = 2 * blockIdx.x, r2 = r1 + 1;
    const bool has2 = r2 < nrows;
    const TU *u1 = U + (long long)r1 * Npf;
    const TU *u2 = U + (long long)r2 * Npf;
    const int Nb = Npf / SP;
    const int tstep = TW / Npf;
    for (int j = threadIdx.x; j < Nb; j += blockDim.x) {
        const int p = SP * j + q;
        buf[j] = mk<T>(cvt<T>(to_d(u1[p])), cvt<T>(has2 ? to_d(u2[p]) : 0.0));
    }
    __syncthreads();
    fft_smem<T>(buf, Nb, -1, stw, MTW);
    for (int m = threadIdx.x; m < ncols; m += blockDim.x) {
        cplx<T> zm = buf[m];
        cplx<T> zn = buf[m == 0 ? 0 : Nb - m];
        if (q) {  // odd samples: Z_m gets e^{-i pi m / Np} O_m
            zm = cmul(zm, twk<T>(tw, m, tstep, -1));
            zn = cmul(zn, twk<T>(tw, -m, tstep, -1));
        }
        // U1 = (zm + conj zn)/2 ; U2 = (zm - conj zn)/(2i)
        cplx<T> f1 = mk<T>(cvt<T>(0.5) * (zm.x + zn.x), cvt<T>(0.5) * (zm.y - zn.y));
        cplx<T> f2 = mk<T>(cvt<T>(0.5) * (zm.y + zn.y), cvt<T>(-0.5) * (zm.x - zn.x));
        if (SP == 2 && q == 0) {
            f1 = cadd(f1, F[(long long)r1 * ncols + m]);
            if (has2) f2 = cadd(f2, F[(long long)r2 * ncols + m]);
        }
        F[(long long)r1 * ncols + m] = f1;
        if (has2) F[(long long)r2 * ncols + m] = f2;
    }
}

// spin s: one complex row per block, columns c = m + L for m in [-L, L].
// PRUNE (SP = 1, where Nb / 4 > L): the modes fill at most [0, Nb/4) and
// (3 Nb / 4, Nb), so the first radix-4 pass is done as the row is read
// (r4_first_pruned) and the zero middle of the row is never written.
template <typename T, typename TU, bool PRUNE = false>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_fwd_spin(const cplx<T> *__restrict__ F, int L, int Npf, cplx<TU> *__restrict__ U,
                   const cplx<T> *__restrict__ tw, int TW, long long fbs, long long ubs, int SP) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int MTW = Npf / SP;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    F += blockIdx.y * fbs;
    U += blockIdx.y * ubs;
    const int q = blockIdx.z;
    const int r = blockIdx.x;
    const int ncols = 2 * L + 1;
    const int Nb = Npf / SP;
    const int tstep = TW / Npf;
    if constexpr (PRUNE) {
        const cplx<T> *row = F + (long long)r * ncols + L;  // mode m at row[m]
        const int nb = Nb / 4;
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            const cplx<T> v0 = j <= L ? row[j] : czero<T>();
            const int m3 = j - nb;  // the mode at x[j + 3 Nb / 4]
            const cplx<T> v3 = m3 >= -L ? row[m3] : czero<T>();
            r4_first_pruned<T>(buf, j, v0, v3, +1);
        }
        __syncthreads();
        fft_smem<T>(buf, Nb, +1, stw, MTW, 2);
        for (int j = threadIdx.x; j < Nb; j += blockDim.x) U[(long long)r * Npf + j] = ccast<TU>(buf[j]);
        return;
    }
    // modes m in [-L, L] land in [0, L] and [Nb - L, Nb); only the gap between is zeroed
    for (int i = L + 1 + threadIdx.x; i < Nb - L; i += blockDim.x) buf[i] = czero<T>();
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
        cplx<T> v = F[(long long)r * ncols + c];
        if (q) v = cmul(v, twk<T>(tw, c - L, tstep, +1));
        buf[wrap2(c - L, Nb)] = v;
    }
    __syncthreads();
    fft_smem<T>(buf, Nb, +1, stw, MTW);
    for (int j = threadIdx.x; j < Nb; j += blockDim.x) U[(long long)r * Npf + SP * j + q] = ccast<TU>(buf[j]);
}

template <typename T, typename TU = T>
__global__ void __launch_bounds__(FFT_TPB)
    k_phi_adj_spin(const cplx<TU> *__restrict__ U, int L, int Npf, cplx<T> *__restrict__ F,
                   const cplx<T> *__restrict__ tw, int TW, int SP, int q, long long ubs, long long fbs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(smem_raw);
    const int MTW = Npf / SP;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    U += blockIdx.y * ubs;
    F += blockIdx.y * fbs;
    const int r = blockIdx.x;
    const int ncols = 2 * L + 1;
    const int Nb = Npf / SP;
    const int tstep = TW / Npf;
    for (int j = threadIdx.x; j < Nb; j += blockDim.x) {
        const cplx<TU> u = U[(long long)r * Npf + SP * j + q];
        buf[j] = mk<T>(cvt<T>(to_d(u.x)), cvt<T>(to_d(u.y)));
    }
    __syncthreads();
    fft_smem<T>(buf, Nb, -1, stw, MTW);
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
        cplx<T> v = buf[wrap2(c - L, Nb)];
        if (q) v = cmul(v, twk<T>(tw, c - L, tstep, -1));
        else if (SP == 2) v = cadd(v, F[(long long)r * ncols + c]);
        F[(long long)r * ncols + c] = v;
    }
}

// ------------------------------------------------------------ ring transform (Bluestein)
// z_p = sum_m h_m e^{i m (phi0 + 2 pi p / N)}, p < N, for one ring per block.
// spin 0: real output from m in [0, L] (h_{-m} = conj h_m); spin s: complex.
// T = double (plain path) or dfl (mixed path); tables are given in T.
// Rings may have different lengths N (HEALPix, thinned grids): each ring uses
// the tables of its length class (RingCls).  Rings shorter than 2L + 1 alias
// the modes: bin q of the length-N transform gathers every m = q (mod N).
// SP = 2 (Mb > 16 x FFT_TPB): the Mb-point circular convolution is done in a
// buffer of Mb/2 >= N points, one launch per frequency parity q (1, then 0):
// the chirped input x (length N) gives X_{2k+q} = FFT_{Mb/2}(x_j w^{jq})_k,
// w = e^{-2 pi i / Mb}, and the convolution at p < N is the sum over q of
// w^{-pq} IFFT_{Mb/2}(X_{2k+q} B_{2k+q})_p, accumulated in the output (rings
// with SP = 1 do all their work in the q = 0 launch).
__device__ __forceinline__ void ring_class(const RingCls &rc, int ring, int &N, int &Mb, int &SP, long long &co,
                                           long long &bo) {
    if (rc.rcls) {
        const int c = rc.rcls[ring];
        N = rc.N[c];
        Mb = rc.Mb[c];
        SP = rc.SP[c];
        co = rc.coff[c];
        bo = rc.boff[c];
    } else {
        N = rc.N0;
        Mb = rc.Mb0;
        SP = rc.SP0;
        co = bo = 0;
    }
}

template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_ring_synth(const double2 *__restrict__ Hgl, int nring, int L, int spin,
                 const double *__restrict__ phi0, const long long *__restrict__ ofs, RingCls rc,
                 const cplx<T> *__restrict__ chirp_all, const cplx<T> *__restrict__ bker_all,
                 double *__restrict__ out0, double *__restrict__ out1,
                 const cplx<T> *__restrict__ tw, int TW, long long hbs, long long obs, int q) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *buf = reinterpret_cast<C *>(smem_raw);
    const int MTW = rc.Hmax;  // length of the quarter twiddle table
    const cplx<T> *stw = load_twiddles<T>(buf, MTW, tw, TW);
    const int ring = blockIdx.x;
    int N, Mb, SP;
    long long co, bo;
    ring_class(rc, ring, N, Mb, SP, co, bo);
    if (q >= SP) return;  // odd-parity launch: split rings only
    Hgl += blockIdx.y * hbs;
    out0 += blockIdx.y * obs;
    if (out1) out1 += blockIdx.y * obs;
    const C *chirp = chirp_all + co, *bker = bker_all + bo;
    const double ph0 = phi0[ring];
    const int Hb = Mb / SP;
    const int tstep = TW / Mb;
    const long long o = ofs[ring];
    for (int i = threadIdx.x; i < Hb; i += blockDim.x) buf[i] = czero<T>();
    __syncthreads();
    // bin qi gathers h_m e^{i m phi0} over m = qi (mod N), m in [-L, L]
    for (int qi = threadIdx.x; qi < N; qi += blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
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
            acc.x += h.x;
            acc.y += h.y;
        }
        C v = cmul(mk<T>(cvt<T>(acc.x), cvt<T>(acc.y)), chirp[qi]);
        if (q) v = cmul(v, twk<T>(tw, qi, tstep, -1));
        buf[qi] = v;
    }
    __syncthreads();
    fft_smem<T>(buf, Hb, -1, stw, MTW);
    for (int i = threadIdx.x; i < Hb; i += blockDim.x) buf[i] = cmul(buf[i], bker[SP * i + q]);
    __syncthreads();
    fft_smem<T>(buf, Hb, +1, stw, MTW);
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        C y = buf[p];
        if (q) y = cmul(y, twk<T>(tw, p, tstep, +1));
        const C z = cmul(y, chirp[p]);
        double z0 = to_d(z.x), z1 = to_d(z.y);
        if (SP == 2 && q == 0) {
            z0 += out0[o + p];
            if (spin != 0) z1 += out1[o + p];
        }
        out0[o + p] = z0;
        if (spin != 0) out1[o + p] = z1;
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

// h'_m = e^{-i m phi0} sum_p z'_p e^{-2 pi i m p / N} (adjoint of k_ring_synth;
// a mode reads its bin m mod N, so rings shorter than 2L + 1 alias as in the
// synthesis); SP = 2 as in k_ring_synth, the two parity launches summed into Hgl.
// wring (may be NULL): per-ring quadrature weight multiplied into h' (the
// weighted adjoint = analysis, SHTns analys)
__global__ void __launch_bounds__(FFT_TPB)
    k_ring_adj(const double *__restrict__ in0, const double *__restrict__ in1, int nring, int L,
               int spin, const double *__restrict__ phi0, const long long *__restrict__ ofs, RingCls rc,
               const double2 *__restrict__ chirp_all, const double2 *__restrict__ bker_all,
               double2 *__restrict__ Hgl, const double2 *__restrict__ tw, int TW, int q,
               const double *__restrict__ wring) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *buf = reinterpret_cast<double2 *>(smem_raw);
    const int MTW = rc.Hmax;  // length of the quarter twiddle table
    const cplx<double> *stw = load_twiddles<double>(buf, MTW, tw, TW);
    const int ring = blockIdx.x;
    int N, Mb, SP;
    long long co, bo;
    ring_class(rc, ring, N, Mb, SP, co, bo);
    if (q >= SP) return;
    const double2 *chirp = chirp_all + co, *bker = bker_all + bo;
    const double ph0 = phi0[ring];
    const long long o = ofs[ring];
    const int Hb = Mb / SP;
    const int tstep = TW / Mb;
    for (int i = threadIdx.x; i < Hb; i += blockDim.x) buf[i] = make_double2(0, 0);
    __syncthreads();
    // Bluestein on conj(z'): c_p = conj(z'_p)
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        const double2 z = make_double2(in0[o + p], spin ? -in1[o + p] : 0.0);
        double2 v = cmul(z, chirp[p]);
        if (q) v = cmul(v, twk<double>(tw, p, tstep, -1));
        buf[p] = v;
    }
    __syncthreads();
    fft_smem<double>(buf, Hb, -1, stw, MTW);
    for (int i = threadIdx.x; i < Hb; i += blockDim.x) buf[i] = cmul(buf[i], bker[SP * i + q]);
    __syncthreads();
    fft_smem<double>(buf, Hb, +1, stw, MTW);
    const int nc = spin == 0 ? L + 1 : 2 * L + 1;
    for (int cidx = threadIdx.x; cidx < nc; cidx += blockDim.x) {
        const int m = spin == 0 ? cidx : cidx - L;
        const int qi = wrapi(m, N);
        double2 y = buf[qi];
        if (q) y = cmul(y, twk<double>(tw, qi, tstep, +1));
        y = cconj(cmul(y, chirp[qi]));  // sum_p z' e^{-2 pi i m p/N}
        double s, c;
        sincos(m * ph0, &s, &c);
        double2 h = cmul(y, make_double2(c, -s));
        if (wring) {
            const double w = wring[ring];
            h = make_double2(h.x * w, h.y * w);
        }
        if (SP == 2 && q == 0) {
            const double2 prev = Hgl[(long long)cidx * nring + ring];
            h = make_double2(h.x + prev.x, h.y + prev.y);
        }
        Hgl[(long long)cidx * nring + ring] = h;
    }
}

// ------------------------------------------------------------ whole-array FFT (setup only)
__global__ void __launch_bounds__(FFT_TPB)
    k_fft_global(double2 *data, int N, int dir, const double2 *__restrict__ tw, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *buf = reinterpret_cast<double2 *>(smem_raw);
    const int MTW = N;  // length of the quarter twiddle table
    const cplx<double> *stw = load_twiddles<double>(buf, MTW, tw, TW);
    for (int i = threadIdx.x; i < N; i += blockDim.x) buf[i] = data[i];
    __syncthreads();
    fft_smem<double>(buf, N, dir, stw, MTW);
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

int theta_fwd_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *H, long long hbs, void *F,
                    long long fbs, cudaStream_t st) {
    const int L = P->lmax;
    const int ncols = spin ? 2 * L + 1 : L + 1;
    const int mofs = spin ? L : 0;
    size_t sm = fft_smem_bytes(P->Ntf / P->sp_theta, P->grid_fp32);
    dim3 grid(ncols, nreq, P->sp_theta);
    if (P->sp_theta == 1) {  // two columns per block
        const dim3 g2((ncols + 1) / 2, nreq);
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_theta_fwd2<float>, sm));
            k_theta_fwd2<float><<<g2, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                         (float2 *)F, ncols, P->n_lo, P->nrows, P->d_tw32, P->TW, hbs,
                                                         fbs);
        } else if (P->fft_df) {
            RC_TRY(set_smem(k_theta_fwd2<dfl>, sm));
            k_theta_fwd2<dfl><<<g2, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                       (dcplx *)F, ncols, P->n_lo, P->nrows, (const dcplx *)P->d_twdf,
                                                       P->TW, hbs, fbs);
        } else {
            RC_TRY(set_smem(k_theta_fwd2<double>, sm));
            k_theta_fwd2<double><<<g2, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth,
                                                          P->d_Dph, (double2 *)F, ncols, P->n_lo, P->nrows,
                                                          P->d_tw64, P->TW, hbs, fbs);
        }
        CU_LAUNCH_CHECK();
        return CUNUSHT_OK;
    }
    if (P->grid_fp32) {
        RC_TRY(set_smem(k_theta_fwd<float>, sm));
        k_theta_fwd<float><<<grid, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                      (float2 *)F, ncols, P->n_lo, P->nrows, P->d_tw32, P->TW, hbs,
                                                      fbs, P->sp_theta);
    } else if (P->fft_df) {
        RC_TRY(set_smem(k_theta_fwd<dfl>, sm));
        k_theta_fwd<dfl><<<grid, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                    (dcplx *)F, ncols, P->n_lo, P->nrows, (const dcplx *)P->d_twdf,
                                                    P->TW, hbs, fbs, P->sp_theta);
    } else {
        RC_TRY(set_smem(k_theta_fwd<double>, sm));
        k_theta_fwd<double><<<grid, FFT_TPB, sm, st>>>(H, P->ncc, P->Nt, P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph,
                                                       (double2 *)F, ncols, P->n_lo, P->nrows, P->d_tw64, P->TW, hbs,
                                                       fbs, P->sp_theta);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int theta_fwd(const cunusht_plan_s *P, int spin, const double2 *H, void *F, cudaStream_t st) {
    return theta_fwd_batch(P, 1, spin, H, 0, F, 0, st);
}

// nreq requests: F + r fbs, H + r hbs (elements); the split transform's
// scratch is the request's fine-grid workspace U + r ubs (consumed by the phi
// pass adjoint before this pass runs)
// Adjoint theta pass of two columns at once (SP = 1).  Every step between the
// fine-grid column and the fold (transforms, band limit, even deconvolution)
// commutes with the reflection n -> -n, and the fold keeps only the part of
// symmetry s = (-1)^(|m| + spin): each input column is first projected onto
// it, g_s = (g + s g_{-n}) / 2, after which columns c1 = 2b, c2 = 2b + 1 (of
// opposite s) share the transforms as in k_theta_fwd2.  The fold of the
// s-symmetric result is 2 y_k inside and y_k at the pole rings k = 0, Nt/2;
// there an odd column's opposite-symmetry part is dropped, which meets the
// Legendre adjoint's zero weight at the poles for those columns.
template <typename T>
__global__ void __launch_bounds__(FFT_TPB)
    k_theta_adj2(const cplx<T> *__restrict__ F, int ncols, int n_lo, int nrows, int Nt, int Ntf, int spin, int mofs,
                 int L, const double *__restrict__ Dth, const double *__restrict__ Dph, double2 *__restrict__ H,
                 int ldH, const cplx<T> *__restrict__ tw, int TW, long long fbs, long long hbs) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *buf = reinterpret_cast<C *>(smem_raw);
    const C *stw = load_twiddles<T>(buf, Ntf, tw, TW);
    F += blockIdx.y * fbs;  // request of a batch
    H += blockIdx.y * hbs;
    const int c1 = 2 * blockIdx.x, c2 = c1 + 1;
    const bool two = c2 < ncols;
    const int m1 = c1 - mofs;
    const double s1 = ((abs(m1) + spin) & 1) ? -1.0 : 1.0, s2 = -s1;
    const int half = Nt / 2;
    const double dm1 = Dph[m1 + L], dm2 = two ? Dph[m1 + 1 + L] : 0.0;
    const T hf = cvt<T>(0.5), ts1 = cvt<T>(s1), ts2 = cvt<T>(s2);
    // z_n = g1s_n + i g2s_n for the pair (n, -n); rows outside the stored band are zero
    auto row = [&](int n, int c) -> C {
        const int r = wrap2(n - n_lo, Ntf);
        return r < nrows ? F[(long long)r * ncols + c] : czero<T>();
    };
    for (int n = threadIdx.x; n <= Ntf / 2; n += blockDim.x) {
        const int nn = wrap2(-n, Ntf);
        const C a1 = row(n, c1), b1 = row(nn, c1);
        const C a2 = two ? row(n, c2) : czero<T>(), b2 = two ? row(nn, c2) : czero<T>();
        const C p1 = cscale(cadd(a1, cscale(b1, ts1)), hf), p2 = cscale(cadd(a2, cscale(b2, ts2)), hf);
        buf[n] = mk<T>(p1.x - p2.y, p1.y + p2.x);
        if (nn != n) {
            const C q1 = cscale(p1, ts1), q2 = cscale(p2, ts2);
            buf[nn] = mk<T>(q1.x - q2.y, q1.y + q2.x);
        }
    }
    __syncthreads();
    fft_smem<T>(buf, Ntf, -1, stw, Ntf);
    // separate, deconvolve, recombine into the Nt-point band; thread j owns +-j
    // (reads j and Ntf - j, writes j and Nt - j); the Nyquist term is zero
    for (int j = threadIdx.x; j < half; j += blockDim.x) {
        const int jn = j ? Ntf - j : 0;
        const C zp = buf[j], zn = cscale(buf[jn], ts1);
        const C x1 = cscale(cadd(zp, zn), hf);
        const C d = cscale(csub(zp, zn), hf);
        const C x2 = mk<T>(d.y, -d.x);
        const C y1 = cscale(x1, scale_of<T>(Dth[j], dm1)), y2 = cscale(x2, scale_of<T>(Dth[j], dm2));
        buf[j] = mk<T>(y1.x - y2.y, y1.y + y2.x);
        if (j) {
            const C y1n = cscale(y1, ts1), y2n = cscale(y2, ts2);
            buf[Nt - j] = mk<T>(y1n.x - y2n.y, y1n.y + y2n.x);
        }
    }
    if (threadIdx.x == 0) buf[half] = czero<T>();
    __syncthreads();
    fft_smem<T>(buf, Nt, +1, stw, Ntf);
    double2 *col1 = H + (long long)c1 * ldH, *col2 = H + (long long)c2 * ldH;
    for (int k = threadIdx.x; k <= half; k += blockDim.x) {
        const C wp = buf[k], wn = cscale(buf[k ? Nt - k : 0], ts1);
        const bool pole = k == 0 || k == half;
        const T f = pole ? hf : cvt<T>(1.0);  // 2 y_k inside, y_k at the poles
        const C v1 = cscale(cadd(wp, wn), f);
        col1[k] = make_double2(to_d(v1.x), to_d(v1.y));
        if (two) {
            const C d = cscale(csub(wp, wn), f);
            col2[k] = make_double2(to_d(d.y), to_d(-d.x));
        }
    }
}

int theta_adj_batch(const cunusht_plan_s *P, int nreq, int spin, const void *F, long long fbs, double2 *H,
                    long long hbs, void *U, long long ubs_bytes, cudaStream_t st) {
    const int L = P->lmax;
    const int ncols = spin ? 2 * L + 1 : L + 1;
    const int mofs = spin ? L : 0;
    const int SP = P->sp_theta;
    size_t sm = fft_smem_bytes(P->Ntf / SP, P->grid_fp32);
    dim3 grid(ncols, nreq);
    if (SP == 1) {  // two columns per block
        const dim3 g2((ncols + 1) / 2, nreq);
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_theta_adj2<float>, sm));
            k_theta_adj2<float><<<g2, FFT_TPB, sm, st>>>((const float2 *)F, ncols, P->n_lo, P->nrows, P->Nt, P->Ntf,
                                                         spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc, P->d_tw32,
                                                         P->TW, fbs, hbs);
        } else if (P->fft_df) {
            RC_TRY(set_smem(k_theta_adj2<dfl>, sm));
            k_theta_adj2<dfl><<<g2, FFT_TPB, sm, st>>>((const dcplx *)F, ncols, P->n_lo, P->nrows, P->Nt, P->Ntf,
                                                       spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc,
                                                       (const dcplx *)P->d_twdf, P->TW, fbs, hbs);
        } else {
            RC_TRY(set_smem(k_theta_adj2<double>, sm));
            k_theta_adj2<double><<<g2, FFT_TPB, sm, st>>>((const double2 *)F, ncols, P->n_lo, P->nrows, P->Nt,
                                                          P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc,
                                                          P->d_tw64, P->TW, fbs, hbs);
        }
        CU_LAUNCH_CHECK();
        return CUNUSHT_OK;
    }
    for (int q = SP - 1; q >= 0; --q) {
        if (P->grid_fp32) {
            RC_TRY(set_smem(k_theta_adj<float>, sm));
            k_theta_adj<float><<<grid, FFT_TPB, sm, st>>>((const float2 *)F, ncols, P->n_lo, P->nrows, P->Nt, P->Ntf,
                                                          spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc, P->d_tw32,
                                                          P->TW, SP, q, (float2 *)U, fbs, hbs,
                                                          ubs_bytes / (long long)sizeof(float2));
        } else if (P->fft_df) {
            RC_TRY(set_smem(k_theta_adj<dfl>, sm));
            k_theta_adj<dfl><<<grid, FFT_TPB, sm, st>>>((const dcplx *)F, ncols, P->n_lo, P->nrows, P->Nt, P->Ntf,
                                                        spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc,
                                                        (const dcplx *)P->d_twdf, P->TW, SP, q, (dcplx *)U, fbs, hbs,
                                                        ubs_bytes / (long long)sizeof(dcplx));
        } else {
            RC_TRY(set_smem(k_theta_adj<double>, sm));
            k_theta_adj<double><<<grid, FFT_TPB, sm, st>>>((const double2 *)F, ncols, P->n_lo, P->nrows, P->Nt,
                                                           P->Ntf, spin, mofs, L, P->d_Dth, P->d_Dph, H, P->ncc,
                                                           P->d_tw64, P->TW, SP, q, (double2 *)U, fbs, hbs,
                                                           ubs_bytes / (long long)sizeof(double2));
        }
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int theta_adj(const cunusht_plan_s *P, int spin, const void *F, double2 *H, cudaStream_t st) {
    return theta_adj_batch(P, 1, spin, F, 0, H, 0, P->d_U, 0, st);
}

// spin-0 phi pass of nreq requests (two real rows per transform); unsplit
// rows (SP = 1, Npf >= 4 (L + 1)) take the pruned first pass
template <typename T, typename TU>
static int phi_fwd_s0_launch(const cunusht_plan_s *P, int nreq, const void *F, long long fbs, void *U, long long ubs,
                             const cplx<T> *tw, size_t sm, cudaStream_t st) {
    const int L = P->lmax, SP = P->sp_phi;
    const dim3 grid((P->nrows + 1) / 2, nreq, SP);
    if (SP == 1 && P->Npf / 4 > L) {
        RC_TRY(set_smem(k_phi_fwd_s0<T, TU, true>, sm));
        k_phi_fwd_s0<T, TU, true><<<grid, FFT_TPB, sm, st>>>((const cplx<T> *)F, L + 1, P->nrows, P->Npf, (TU *)U, tw,
                                                              P->TW, fbs, ubs, SP);
    } else {
        RC_TRY(set_smem(k_phi_fwd_s0<T, TU, false>, sm));
        k_phi_fwd_s0<T, TU, false><<<grid, FFT_TPB, sm, st>>>((const cplx<T> *)F, L + 1, P->nrows, P->Npf, (TU *)U,
                                                               tw, P->TW, fbs, ubs, SP);
    }
    return CUNUSHT_OK;
}

// spin phi pass of nreq requests; unsplit rows (SP = 1, Npf >= 4 (L + 1))
// take the pruned first pass
template <typename T, typename TU>
static int phi_fwd_spin_launch(const cunusht_plan_s *P, int nreq, const void *F, long long fbs, void *U, long long ubs,
                               const cplx<T> *tw, size_t sm, cudaStream_t st) {
    const int L = P->lmax, SP = P->sp_phi;
    const dim3 grid(P->nrows, nreq, SP);
    if (SP == 1 && P->Npf / 4 > L) {
        RC_TRY(set_smem(k_phi_fwd_spin<T, TU, true>, sm));
        k_phi_fwd_spin<T, TU, true><<<grid, FFT_TPB, sm, st>>>((const cplx<T> *)F, L, P->Npf, (cplx<TU> *)U, tw,
                                                                P->TW, fbs, ubs, SP);
    } else {
        RC_TRY(set_smem(k_phi_fwd_spin<T, TU, false>, sm));
        k_phi_fwd_spin<T, TU, false><<<grid, FFT_TPB, sm, st>>>((const cplx<T> *)F, L, P->Npf, (cplx<TU> *)U, tw,
                                                                 P->TW, fbs, ubs, SP);
    }
    return CUNUSHT_OK;
}

int phi_fwd_batch(const cunusht_plan_s *P, int nreq, int spin, const void *F, long long fbs, void *U, long long ubs,
                  cudaStream_t st) {
    const int L = P->lmax;
    size_t sm = fft_smem_bytes(P->Npf / P->sp_phi, P->grid_fp32);
    const int SP = P->sp_phi;
    if (spin == 0) {
        if (P->grid_fp32) {
            RC_TRY((phi_fwd_s0_launch<float, float>(P, nreq, F, fbs, U, ubs, P->d_tw32, sm, st)));
        } else if (P->fft_df) {
            RC_TRY((phi_fwd_s0_launch<dfl, float>(P, nreq, F, fbs, U, ubs, (const dcplx *)P->d_twdf, sm, st)));
        } else if (P->fwd_u32) {
            RC_TRY((phi_fwd_s0_launch<double, float>(P, nreq, F, fbs, U, ubs, P->d_tw64, sm, st)));
        } else {
            RC_TRY((phi_fwd_s0_launch<double, double>(P, nreq, F, fbs, U, ubs, P->d_tw64, sm, st)));
        }
    } else {
        if (P->grid_fp32) {
            RC_TRY((phi_fwd_spin_launch<float, float>(P, nreq, F, fbs, U, ubs, P->d_tw32, sm, st)));
        } else if (P->fft_df) {
            RC_TRY((phi_fwd_spin_launch<dfl, float>(P, nreq, F, fbs, U, ubs, (const dcplx *)P->d_twdf, sm, st)));
        } else if (P->fwd_u32) {
            RC_TRY((phi_fwd_spin_launch<double, float>(P, nreq, F, fbs, U, ubs, P->d_tw64, sm, st)));
        } else {
            RC_TRY((phi_fwd_spin_launch<double, double>(P, nreq, F, fbs, U, ubs, P->d_tw64, sm, st)));
        }
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int phi_fwd(const cunusht_plan_s *P, int spin, const void *F, void *U, cudaStream_t st) {
    return phi_fwd_batch(P, 1, spin, F, 0, U, 0, st);
}

// nreq requests: U + r ubs (scalars), F + r fbs (complex elements)
int phi_adj_batch(const cunusht_plan_s *P, int nreq, int spin, const void *U, long long ubs, void *F, long long fbs,
                  cudaStream_t st) {
    const int L = P->lmax;
    size_t sm = fft_smem_bytes(P->Npf / P->sp_phi, P->grid_fp32);
    const int SP = P->sp_phi;
    for (int q = SP - 1; q >= 0; --q) {
        if (spin == 0) {
            const dim3 grid((P->nrows + 1) / 2, nreq);
            if (P->grid_fp32) {
                RC_TRY(set_smem(k_phi_adj_s0<float>, sm));
                k_phi_adj_s0<float><<<grid, FFT_TPB, sm, st>>>((const float *)U, P->nrows, P->Npf, (float2 *)F, L + 1,
                                                               P->d_tw32, P->TW, SP, q, ubs, fbs);
            } else if (P->fft_df) {  // FP64 grid, double-float transforms
                RC_TRY(set_smem(k_phi_adj_s0<dfl, double>, sm));
                k_phi_adj_s0<dfl, double><<<grid, FFT_TPB, sm, st>>>((const double *)U, P->nrows, P->Npf, (dcplx *)F,
                                                                     L + 1, (const dcplx *)P->d_twdf, P->TW, SP, q,
                                                                     ubs, fbs);
            } else {
                RC_TRY(set_smem(k_phi_adj_s0<double>, sm));
                k_phi_adj_s0<double><<<grid, FFT_TPB, sm, st>>>((const double *)U, P->nrows, P->Npf, (double2 *)F,
                                                                L + 1, P->d_tw64, P->TW, SP, q, ubs, fbs);
            }
        } else {
            const dim3 grid(P->nrows, nreq);
            if (P->grid_fp32) {
                RC_TRY(set_smem(k_phi_adj_spin<float>, sm));
                k_phi_adj_spin<float><<<grid, FFT_TPB, sm, st>>>((const float2 *)U, L, P->Npf, (float2 *)F,
                                                                 P->d_tw32, P->TW, SP, q, ubs / 2, fbs);
            } else if (P->fft_df) {
                RC_TRY(set_smem(k_phi_adj_spin<dfl, double>, sm));
                k_phi_adj_spin<dfl, double><<<grid, FFT_TPB, sm, st>>>((const double2 *)U, L, P->Npf, (dcplx *)F,
                                                                       (const dcplx *)P->d_twdf, P->TW, SP, q,
                                                                       ubs / 2, fbs);
            } else {
                RC_TRY(set_smem(k_phi_adj_spin<double>, sm));
                k_phi_adj_spin<double><<<grid, FFT_TPB, sm, st>>>((const double2 *)U, L, P->Npf, (double2 *)F,
                                                                  P->d_tw64, P->TW, SP, q, ubs / 2, fbs);
            }
        }
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int phi_adj(const cunusht_plan_s *P, int spin, const void *U, void *F, cudaStream_t st) {
    return phi_adj_batch(P, 1, spin, U, 0, F, 0, st);
}

// shared-memory buffer (complex elements) of the ring transforms: the largest
// Mb / SP over the ring-length classes
static int ring_buffer_len(const cunusht_plan_s *P) { return P->ncls > 1 ? P->ring_buf : P->Mb / P->sp_ring; }

int ring_synth_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *Hgl, long long hbs, double *out0,
                     double *out1, long long obs, cudaStream_t st) {
    if (ring_mr_available(P)) return ring_synth_mr_batch(P, nreq, spin, Hgl, hbs, out0, out1, obs, st);
    size_t sm = fft_smem_bytes(ring_buffer_len(P), false);
    dim3 grid(P->nring, nreq);
    const RingCls rc = ring_cls_of(P);
    for (int q = P->sp_ring - 1; q >= 0; --q) {
        if (P->ring_df && P->d_chirp_df) {
            RC_TRY(set_smem(k_ring_synth<dfl>, sm));
            k_ring_synth<dfl><<<grid, FFT_TPB, sm, st>>>(Hgl, P->nring, P->lmax, spin, P->d_ring_phi0, P->d_ring_ofs,
                                                         rc, (const dcplx *)P->d_chirp_df,
                                                         (const dcplx *)P->d_bker_df, out0, out1,
                                                         (const dcplx *)P->d_twdf, P->TW, hbs, obs, q);
        } else {
            RC_TRY(set_smem(k_ring_synth<double>, sm));
            k_ring_synth<double><<<grid, FFT_TPB, sm, st>>>(Hgl, P->nring, P->lmax, spin, P->d_ring_phi0,
                                                            P->d_ring_ofs, rc, P->d_chirp, P->d_bker, out0, out1,
                                                            P->d_tw64, P->TW, hbs, obs, q);
        }
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int ring_synth(const cunusht_plan_s *P, int spin, const double2 *Hgl, double *out0, double *out1,
               cudaStream_t st) {
    return ring_synth_batch(P, 1, spin, Hgl, 0, out0, out1, 0, st);
}

int ring_adjoint(const cunusht_plan_s *P, int spin, const double *in0, const double *in1,
                 double2 *Hgl, cudaStream_t st, const double *wring) {
    size_t sm = fft_smem_bytes(ring_buffer_len(P), false);
    RC_TRY(set_smem(k_ring_adj, sm));
    const RingCls rc = ring_cls_of(P);
    for (int q = P->sp_ring - 1; q >= 0; --q) {
        k_ring_adj<<<P->nring, FFT_TPB, sm, st>>>(in0, in1, P->nring, P->lmax, spin, P->d_ring_phi0, P->d_ring_ofs,
                                                  rc, P->d_chirp, P->d_bker, Hgl, P->d_tw64, P->TW, q, wring);
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

}  // namespace cunusht

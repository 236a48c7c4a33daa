// Non-uniform interpolation (type 2) and spreading (type 1) on the oversampled
// 2 pi torus with the "exponential of semicircle" kernel
//     psi(z) = exp(beta (sqrt(1 - z^2) - 1)),  |z| <= 1,  z = 2 (x - n) / w,
// which replaces the cuFINUFFT execute calls of the reference
// (cunusht/deflection/GPU_nufft_transformer.py:292-310; plan :242-246 with
// isign +1 for type 2 and -1 for type 1, FFT mode ordering).  The deconvolution
// by the kernel's Fourier transform is applied in the theta pass (fft.cu).
//
// Fine-grid layout: rows n in [n_lo, n_lo + nrows) of the theta torus (row
// r = n - n_lo), each row Npf longitudes; real (spin 0) or complex (spin s).
// Points are read in the caller's order; for lensing they are the deflected
// pixels in ring order, so neighbouring threads touch neighbouring columns.
#include <type_traits>

#include "common.cuh"
#include "df.cuh"
#include "kernels.cuh"
#include "nufft_pts.cuh"

namespace cunusht {

template <typename T, int W = MAXW>
__device__ __forceinline__ void weights(const PointCoords &pc, int w, T beta, T *kt, T *kp) {
    const T s = (T)2 / (T)w;
#pragma unroll
    for (int a = 0; a < W; ++a) {
        if (W < MAXW || a < w) {  // exact trip count when the width is a template argument
            kt[a] = es_kernel<T>(((T)pc.ft + (T)a) * s, beta);
            kp[a] = es_kernel<T>(((T)pc.fp + (T)a) * s, beta);
        }
    }
}

// f(std::integral_constant<int, w>) for a runtime kernel width 2 <= w <= MAXW:
// kernels whose tap loops take the width as a template argument run exactly
// w x w taps instead of MAXW-wide predicated loops
template <int W0 = 2, typename F> static void with_width(int w, F &&f) {
    if constexpr (W0 <= MAXW) {
        if (w == W0) f(std::integral_constant<int, W0>{});
        else with_width<W0 + 1>(w, f);
    }
}

// ------------------------------------------------------------ interp (type 2)
template <typename T, bool CPLX, int W>
__global__ void __launch_bounds__(NU_TPB)
    k_interp(const T *__restrict__ U, int nrows, int Npf, int Ntf, int n_lo, int w, T beta,
             const double *__restrict__ loc, long long npts, int layout,
             const double *__restrict__ gamma, int spin, void *__restrict__ out, int out_f32, long long ubs,
             long long lbs, long long obs) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npts) return;
    U += blockIdx.y * ubs;  // request of a batch (strides in elements)
    loc += blockIdx.y * lbs;
    if (gamma) gamma += blockIdx.y * npts;
    out = out_f32 ? (void *)((float *)out + blockIdx.y * obs) : (void *)((double *)out + blockIdx.y * obs);
    double th, ph;
    load_point(loc, j, npts, layout, th, ph);
    const PointCoords pc = point_coords(th, ph, Ntf, Npf, n_lo, nrows, W);
    T kt[W], kp[W];
    weights<T, W>(pc, W, beta, kt, kp);
    int cols[W];
#pragma unroll
    for (int b = 0; b < W; ++b) {
        int c = pc.p0 + b;
        c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
        cols[b] = c;
    }
    T ar = 0, ai = 0;
#pragma unroll
    for (int a = 0; a < W; ++a) {
        const long long rowoff = (long long)(pc.r0 + a) * Npf;
        T rr = 0, ri = 0;
        if constexpr (CPLX) {
            const cplx<T> *row = reinterpret_cast<const cplx<T> *>(U) + rowoff;
#pragma unroll
            for (int b = 0; b < W; ++b) {
                const cplx<T> v = row[cols[b]];
                rr = fma(kp[b], v.x, rr);
                ri = fma(kp[b], v.y, ri);
            }
        } else {
            const T *row = U + rowoff;
#pragma unroll
            for (int b = 0; b < W; ++b) rr = fma(kp[b], row[cols[b]], rr);
        }
        ar = fma(kt[a], rr, ar);
        if constexpr (CPLX) ai = fma(kt[a], ri, ai);
    }
    if constexpr (CPLX) {
        double zr = ar, zi = ai;
        if (gamma) {
            double s, c;
            sincos(spin * gamma[j], &s, &c);
            const double tr = zr * c - zi * s;
            zi = zr * s + zi * c;
            zr = tr;
        }
        if (out_f32) {
            ((float *)out)[j] = (float)zr;
            ((float *)out)[npts + j] = (float)zi;
        } else {
            ((double *)out)[j] = zr;
            ((double *)out)[npts + j] = zi;
        }
    } else {
        if (out_f32) ((float *)out)[j] = (float)ar;
        else ((double *)out)[j] = (double)ar;
    }
}

// ------------------------------------------------------------ warp-strip spreading (type 1)
// Each warp spreads 32 consecutive points (for lensing: neighbouring pixels of
// one ring, whose w x w footprints overlap) into a private shared-memory strip
// covering their joint footprint.  All lanes step through the taps (a, b) in
// lockstep, so two lanes touch the same strip cell only when their points
// share the first-tap cell; such lanes are serialised by rank
// (__match_any_sync), and the strip needs no atomics.  The strip is then added
// to U with global atomics, one per touched cell instead of one per tap.
// Warps whose footprint does not fit the strip (a ring boundary, scattered
// points) add their taps to U directly.
constexpr int SPW_WARPS = 4;  // warps per block

template <typename T, bool CPLX, int W>
__global__ void __launch_bounds__(SPW_WARPS * 32)
    k_spread_warp(T *__restrict__ U, int nrows, int Npf, int Ntf, int n_lo, int w, T beta,
                  const double *__restrict__ loc, long long npts, int layout, const double *__restrict__ gamma,
                  int spin, const void *__restrict__ in, int in_f32, int SR, int SC, long long ubs, long long lbs,
                  long long ibs, unsigned long long *__restrict__ Ufix, const float *__restrict__ vmax, int lgn) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NC = CPLX ? 2 : 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T *strip = reinterpret_cast<T *>(smem_raw) + (size_t)wid * SR * SC * NC;
    // deterministic plans add to the int64 fixed-point grid instead (exact, order-free)
    const int E = Ufix ? fix_exp(vmax[blockIdx.y], lgn) : 0;
    if (Ufix) Ufix += blockIdx.y * ubs;
    U += blockIdx.y * ubs;  // request of a batch
    loc += blockIdx.y * lbs;
    if (gamma) gamma += blockIdx.y * npts;
    in = in_f32 ? (const void *)((const float *)in + blockIdx.y * ibs) : (const void *)((const double *)in + blockIdx.y * ibs);
    const long long j = ((long long)blockIdx.x * SPW_WARPS + wid) * 32 + lane;
    const bool act = j < npts;
    const unsigned amask = __ballot_sync(0xffffffffu, act);
    if (amask == 0) return;
    PointCoords pc{0, 0, 0.0, 0.0};
    double vr = 0.0, vi = 0.0;
    if (act) {
        double th, ph;
        load_point(loc, j, npts, layout, th, ph);
        pc = point_coords(th, ph, Ntf, Npf, n_lo, nrows, W);
        if (in_f32) {
            vr = ((const float *)in)[j];
            if (CPLX) vi = ((const float *)in)[npts + j];
        } else {
            vr = ((const double *)in)[j];
            if (CPLX) vi = ((const double *)in)[npts + j];
        }
        if (CPLX && gamma) {
            double s, c;
            sincos(spin * gamma[j], &s, &c);  // multiply by e^{-i spin gamma}
            const double t2 = vr * c + vi * s;
            vi = vi * c - vr * s;
            vr = t2;
        }
    }
    T kt[W], kp[W];
    weights<T, W>(pc, W, beta, kt, kp);
    // joint footprint of the warp's points
    const int big = 1 << 30;
    const int rmin = __reduce_min_sync(0xffffffffu, act ? pc.r0 : big);
    const int rmax = __reduce_max_sync(0xffffffffu, act ? pc.r0 : -big);
    const int pmin = __reduce_min_sync(0xffffffffu, act ? pc.p0 : big);
    const int pmax = __reduce_max_sync(0xffffffffu, act ? pc.p0 : -big);
    const int nr = rmax - rmin + W, ncl = pmax - pmin + W;
    if (nr > SR || ncl > SC) {
        // footprint too wide for the strip: direct global atomics
        if (!act) return;
#pragma unroll 1
        for (int a = 0; a < W; ++a) {
            const long long rowoff = (long long)(pc.r0 + a) * Npf;
            const T fr = kt[a] * (T)vr, fi = kt[a] * (T)vi;
#pragma unroll
            for (int b = 0; b < W; ++b) {
                int c = pc.p0 + b;
                c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
                if (Ufix) {
                    unsigned long long *fc = Ufix + (rowoff + c) * NC;
                    atomicAdd(fc, (unsigned long long)to_fix(kp[b] * fr, E));
                    if constexpr (CPLX) atomicAdd(fc + 1, (unsigned long long)to_fix(kp[b] * fi, E));
                    continue;
                }
                T *cell = U + (rowoff + c) * NC;
                atomicAdd(cell, kp[b] * fr);
                if constexpr (CPLX) atomicAdd(cell + 1, kp[b] * fi);
            }
        }
        return;
    }
    for (int i = lane; i < nr * ncl * NC; i += 32) strip[i] = (T)0;
    __syncwarp();
    // lanes with the same first-tap cell go in separate rounds
    const int key = act ? (pc.r0 - rmin) * SC + (pc.p0 - pmin) : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int myrank = __popc(peers & ((1u << lane) - 1u));
    const int nround = __reduce_max_sync(0xffffffffu, act ? myrank : 0) + 1;
    const int base = (pc.r0 - rmin) * ncl + (pc.p0 - pmin);
    for (int rd = 0; rd < nround; ++rd) {
        const bool go = act && myrank == rd;
#pragma unroll 1
        for (int a = 0; a < W; ++a) {
            const T fr = kt[a] * (T)vr, fi = kt[a] * (T)vi;
            T *row = strip + (size_t)(base + a * ncl) * NC;
#pragma unroll
            for (int b = 0; b < W; ++b) {
                if (go) {
                    row[b * NC] += kp[b] * fr;
                    if constexpr (CPLX) row[b * NC + 1] += kp[b] * fi;
                }
                // footprints of neighbouring points overlap: order every
                // step's read-modify-write before the next step's
                __syncwarp();
            }
        }
    }
    __syncwarp();
    for (int i = lane; i < nr * ncl; i += 32) {
        const int lr = i / ncl, lc = i - lr * ncl;
        int c = pmin + lc;
        c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
        const long long ci = ((long long)(rmin + lr) * Npf + c) * NC;
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            const T v = strip[i * NC + q];
            if (v == (T)0) continue;
            if (Ufix) atomicAdd(Ufix + ci + q, (unsigned long long)to_fix(v, E));
            else atomicAdd(U + ci + q, v);
        }
    }
}

template <typename T, bool CPLX>
static int launch_spread_warp(const cunusht_plan_s *P, int nreq, T *U, long long ubs, const double *loc, long long lbs,
                              long long npts, int layout, const double *gamma, int spin, const void *in,
                              long long ibs, int f32i, cudaStream_t st) {
    int lgn = 0;
    while ((1LL << lgn) < npts + 1) ++lgn;
    // strip: the footprint of 32 neighbouring ring pixels at about 2 fine
    // cells per pixel, plus row jitter from the deflection
    const int SR = P->w + 4, SC = 80 + P->w;
    const size_t sm = (size_t)SPW_WARPS * SR * SC * (CPLX ? 2 : 1) * sizeof(T);
    const long long nwarps = (npts + 31) / 32;
    const unsigned nb = (unsigned)((nwarps + SPW_WARPS - 1) / SPW_WARPS);
    cudaError_t e = cudaSuccess;
    with_width(P->w, [&](auto WC) {
        constexpr int W = decltype(WC)::value;
        if (sm > 48 * 1024)
            e = cudaFuncSetAttribute(k_spread_warp<T, CPLX, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e == cudaSuccess)
            k_spread_warp<T, CPLX, W><<<dim3(nb, nreq), SPW_WARPS * 32, sm, st>>>(
                U, P->nrows, P->Npf, P->Ntf, P->n_lo, W, (T)P->beta, loc, npts, layout, gamma, spin, in, f32i, SR, SC,
                ubs, lbs, ibs, P->spread_det ? P->d_ufix : nullptr, P->d_vmax, lgn);
    });
    CU_TRY(e);
    return CUNUSHT_OK;
}

// Exact float -> double conversion on the integer pipe (GB300's FP64 pipe
// runs conversions at the FP64 rate): sign, exponent rebias 127 -> 1023,
// mantissa shifted into the top of the 52-bit field.  FP32 denormals
// (|x| < 2^-126) are flushed to zero; infinities / NaN are not expected.
__device__ __forceinline__ double f2d_exact_int(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex == 0) return 0.0;
    const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) |
                                    ((unsigned long long)(ex + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

// Mixed-precision variant: kernel weights in FP32 from the FP64 tap offset
// split into hi + lo floats (as k_interp_mixed), FP32 products, global
// accumulation in the grid's type TG.  FP64 grid (eps <= 1e-6):
// Kahan-compensated FP32 strip sums, each added as two exact FP64 atomics.
// FP32 grid (eps > 1e-6): plain FP32 strip sums (half the shared memory, so
// twice the resident blocks) and one FP32 atomic per strip cell.  The FP64 variant is bound by its FP64 exponentials and
// products (GB300 runs FP64 at about 1/80 of the FP32 rate).
template <typename TG, bool CPLX, int W>
__global__ void __launch_bounds__(SPW_WARPS * 32)
    k_spread_warp_mixed(TG *__restrict__ U, int nrows, int Npf, int Ntf, int n_lo, int w, float beta,
                        const double *__restrict__ loc, long long npts, int layout, const double *__restrict__ gamma,
                        int spin, const void *__restrict__ in, int in_f32, int SR, int SC, long long ubs,
                        long long lbs, long long ibs, unsigned long long *__restrict__ Ufix,
                        const float *__restrict__ vmax, int lgn) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NC = CPLX ? 2 : 1;
    constexpr bool KAHAN = std::is_same<TG, double>::value;
    using SE = typename std::conditional<KAHAN, float2, float>::type;  // (sum, compensation) or sum
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    SE *strip = reinterpret_cast<SE *>(smem_raw) + (size_t)wid * SR * SC * NC;
    const int E = Ufix ? fix_exp(vmax[blockIdx.y], lgn) : 0;
    if (Ufix) Ufix += blockIdx.y * ubs;
    U += blockIdx.y * ubs;  // request of a batch
    loc += blockIdx.y * lbs;
    if (gamma) gamma += blockIdx.y * npts;
    in = in_f32 ? (const void *)((const float *)in + blockIdx.y * ibs) : (const void *)((const double *)in + blockIdx.y * ibs);
    const long long j = ((long long)blockIdx.x * SPW_WARPS + wid) * 32 + lane;
    const bool act = j < npts;
    const unsigned amask = __ballot_sync(0xffffffffu, act);
    if (amask == 0) return;
    // coordinates, values and the rotation in double-float: no FP64 instruction
    // on this path (GB300 issues FP64 at 1/64 of the FP32 rate)
    PointCoordsDf pc{0, 0, dfl{0.f, 0.f}, dfl{0.f, 0.f}};
    dfl vr{0.f, 0.f}, vi{0.f, 0.f};
    if (act) {
        double th, ph;
        load_point(loc, j, npts, layout, th, ph);
        pc = point_coords_df(th, ph, Ntf, Npf, n_lo, nrows, W);
        if (in_f32) {
            vr = dfl{((const float *)in)[j], 0.f};
            if (CPLX) vi = dfl{((const float *)in)[npts + j], 0.f};
        } else {
            vr = df_from(((const double *)in)[j]);
            if (CPLX) vi = df_from(((const double *)in)[npts + j]);
        }
        if (CPLX && gamma) {
            // multiply by e^{-i spin gamma}; 1 - cos from 2 sin^2(x/2) keeps
            // the FP32 error of the small correction terms relative to the angle
            const float x = (float)spin * df_from(gamma[j]).h;
            const float sh = sinf(0.5f * x);
            const float d = 2.f * sh * sh;
            const float sn = sinf(x);
            const float cr = fmaf(vr.h, d, -vi.h * sn), ci = fmaf(vi.h, d, vr.h * sn);
            vr = df_add(vr, dfl{-cr, 0.f});
            vi = df_add(vi, dfl{-ci, 0.f});
        }
    }
    float kt[W], kp[W];
    {
        const float sc = 2.f / (float)W;
        const float fth = pc.ft.h, ftl = pc.ft.l;
        const float fph = pc.fp.h, fpl = pc.fp.l;
#pragma unroll
        for (int a = 0; a < W; ++a) {
            kt[a] = es_kernel_acc((((float)a + fth) + ftl) * sc, beta);
            kp[a] = es_kernel_acc((((float)a + fph) + fpl) * sc, beta);
        }
    }
    const int big = 1 << 30;
    const int rmin = __reduce_min_sync(0xffffffffu, act ? pc.r0 : big);
    const int rmax = __reduce_max_sync(0xffffffffu, act ? pc.r0 : -big);
    const int pmin = __reduce_min_sync(0xffffffffu, act ? pc.p0 : big);
    const int pmax = __reduce_max_sync(0xffffffffu, act ? pc.p0 : -big);
    const int nr = rmax - rmin + W, ncl = pmax - pmin + W;
    const float vrh = vr.h, vrl = vr.l;
    const float vih = vi.h, vil = vi.l;
    if (nr > SR || ncl > SC) {
        if (!act) return;
        // footprint wider than the strip (scattered points): FP64 products and
        // atomics (FP32 ones into an FP32 grid)
        const double vrd = df_to(vr), vid = df_to(vi);
#pragma unroll 1
        for (int a = 0; a < W; ++a) {
            const long long rowoff = (long long)(pc.r0 + a) * Npf;
#pragma unroll
            for (int b = 0; b < W; ++b) {
                int c = pc.p0 + b;
                c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
                const double kw = (double)kt[a] * (double)kp[b];
                if (Ufix) {
                    unsigned long long *fc = Ufix + (rowoff + c) * NC;
                    atomicAdd(fc, (unsigned long long)to_fix(kw * vrd, E));
                    if constexpr (CPLX) atomicAdd(fc + 1, (unsigned long long)to_fix(kw * vid, E));
                    continue;
                }
                TG *cell = U + (rowoff + c) * NC;
                if constexpr (std::is_same<TG, double>::value) {
                    atomicAdd(cell, kw * vrd);
                    if constexpr (CPLX) atomicAdd(cell + 1, kw * vid);
                } else {
                    const float kf = kt[a] * kp[b];
                    atomicAdd(cell, kf * (vrh + vrl));
                    if constexpr (CPLX) atomicAdd(cell + 1, kf * (vih + vil));
                }
            }
        }
        return;
    }
    for (int i = lane; i < nr * ncl * NC; i += 32) strip[i] = SE{};
    __syncwarp();
    const int key = act ? (pc.r0 - rmin) * SC + (pc.p0 - pmin) : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int myrank = __popc(peers & ((1u << lane) - 1u));
    const int nround = __reduce_max_sync(0xffffffffu, act ? myrank : 0) + 1;
    const int base = (pc.r0 - rmin) * ncl + (pc.p0 - pmin);
    for (int rd = 0; rd < nround; ++rd) {
        const bool go = act && myrank == rd;
#pragma unroll 1
        for (int a = 0; a < W; ++a) {
            // row factor kt[a] * value as a double-float (FP32 TwoProduct on
            // the split value): each tap product then carries one FP32 rounding
            const float frh = kt[a] * vrh, frl = fmaf(kt[a], vrh, -frh) + kt[a] * vrl;
            const float fih = kt[a] * vih, fil = fmaf(kt[a], vih, -fih) + kt[a] * vil;
            SE *row = strip + (size_t)(base + a * ncl) * NC;
            if constexpr (!KAHAN) {
#pragma unroll
                for (int b = 0; b < W; ++b) {
                    if (go) {
                        row[b * NC] += kp[b] * (frh + frl);
                        if constexpr (CPLX) row[b * NC + 1] += kp[b] * (fih + fil);
                    }
                    __syncwarp();
                }
            } else {
#pragma unroll
                for (int b = 0; b < W; ++b) {
                    if (go) {
                        // Kahan: sum = x, comp = c; value = x - c
                        float2 t = row[b * NC];
                        float y = fmaf(kp[b], frh, kp[b] * frl) - t.y;
                        float s2 = t.x + y;
                        row[b * NC] = make_float2(s2, (s2 - t.x) - y);
                        if constexpr (CPLX) {
                            t = row[b * NC + 1];
                            y = fmaf(kp[b], fih, kp[b] * fil) - t.y;
                            s2 = t.x + y;
                            row[b * NC + 1] = make_float2(s2, (s2 - t.x) - y);
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    __syncwarp();
    for (int i = lane; i < nr * ncl; i += 32) {
        const int lr = i / ncl, lc = i - lr * ncl;
        int c = pmin + lc;
        c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
        const long long ci = ((long long)(rmin + lr) * Npf + c) * NC;
        TG *cell = U + ci;
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            // Kahan value x - c as two exact FP64 atomic adds (the additions
            // happen in L2, the conversions on the integer pipe), or as one
            // FP32 atomic add of x - c into an FP32 grid
            if constexpr (KAHAN) {
                const float2 v = strip[i * NC + q];
                if (Ufix) {
                    if (v.x != 0.f || v.y != 0.f)
                        atomicAdd(Ufix + ci + q, (unsigned long long)(to_fix(v.x, E) - to_fix(v.y, E)));
                    continue;
                }
                if (v.x != 0.f) atomicAdd(cell + q, f2d_exact_int(v.x));
                if (v.y != 0.f) atomicAdd(cell + q, -f2d_exact_int(v.y));
            } else {
                const float v = strip[i * NC + q];
                if (v == 0.f) continue;
                if (Ufix) atomicAdd(Ufix + ci + q, (unsigned long long)to_fix(v, E));
                else atomicAdd(cell + q, v);
            }
        }
    }
}

template <typename TG, bool CPLX>
static int launch_spread_warp_mixed(const cunusht_plan_s *P, int nreq, TG *U, long long ubs, const double *loc,
                                    long long lbs, long long npts, int layout, const double *gamma, int spin,
                                    const void *in, long long ibs, int f32i, cudaStream_t st) {
    int lgn = 0;
    while ((1LL << lgn) < npts + 1) ++lgn;
    const int SR = P->w + 4, SC = 80 + P->w;
    const size_t sm = (size_t)SPW_WARPS * SR * SC * (CPLX ? 2 : 1) * (std::is_same<TG, double>::value ? 8 : 4);
    const long long nwarps = (npts + 31) / 32;
    const unsigned nb = (unsigned)((nwarps + SPW_WARPS - 1) / SPW_WARPS);
    cudaError_t e = cudaSuccess;
    with_width(P->w, [&](auto WC) {
        constexpr int W = decltype(WC)::value;
        if (sm > 48 * 1024)
            e = cudaFuncSetAttribute(k_spread_warp_mixed<TG, CPLX, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm);
        if (e == cudaSuccess)
            k_spread_warp_mixed<TG, CPLX, W><<<dim3(nb, nreq), SPW_WARPS * 32, sm, st>>>(
                U, P->nrows, P->Npf, P->Ntf, P->n_lo, W, (float)P->beta, loc, npts, layout, gamma, spin, in, f32i, SR,
                SC, ubs, lbs, ibs, P->spread_det ? P->d_ufix : nullptr, P->d_vmax, lgn);
    });
    CU_TRY(e);
    return CUNUSHT_OK;
}

// ------------------------------------------------------------ interp, mixed precision
// FP32 fine grid of a mixed plan (from the double-float FFTs at eps <= 1e-6,
// the FP32 ones above), FP32 kernel weights from the cancellation-free
// exponent  beta (sqrt(1 - z^2) - 1) = -beta z^2 / (1 + sqrt(1 - z^2)),
// Kahan-compensated FP32 sums, and the exp(i s gamma) rotation applied in
// double-float from d = 1 - cos(x) = 2 sin^2(x/2) and sin(x) evaluated in FP32
// (errors relative to the small angle, not to 1).

// Five 256-thread blocks per SM for kernel widths up to 9 (48 registers, an
// 8-byte spill at width 9): the kernel waits on its tap loads, and 40 warps
// per SM hide more of that latency than the 32 of four blocks.
template <bool CPLX, int W>
__global__ void __launch_bounds__(NU_TPB, W <= 9 ? 5 : 4)
    k_interp_mixed(const float *__restrict__ U, int nrows, int Npf, int Ntf, int n_lo, int w, float beta,
                   const double *__restrict__ loc, long long npts, int layout, const double *__restrict__ gamma,
                   int spin, void *__restrict__ out, int out_f32, long long ubs, long long lbs, long long obs) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npts) return;
    U += blockIdx.y * ubs;  // request of a batch (strides in elements)
    loc += blockIdx.y * lbs;
    if (gamma) gamma += blockIdx.y * npts;
    out = out_f32 ? (void *)((float *)out + blockIdx.y * obs) : (void *)((double *)out + blockIdx.y * obs);
    double th, ph;
    load_point(loc, j, npts, layout, th, ph);
    const PointCoordsDf pc = point_coords_df(th, ph, Ntf, Npf, n_lo, nrows, W);
    // tap offsets (n0 + a - t) from the double-float offset: (a + ft_h) is
    // exact in FP32, so each tap argument carries only its own final rounding
    // (a single FP32 rounding of ft would shift every tap of the point by up
    // to 2.4e-7 grid cells, a coherent position error).  The theta weights are
    // evaluated row by row and the columns wrap only for points whose taps
    // cross phi = 0 (a separate path), which keeps the live registers low.
    const float sc = 2.f / (float)W;
    const float fth = pc.ft.h, ftl = pc.ft.l;
    const float fph = pc.fp.h, fpl = pc.fp.l;
    float kp[W];
#pragma unroll
    for (int b = 0; b < W; ++b) kp[b] = es_kernel_acc((((float)b + fph) + fpl) * sc, beta);
    kahan zr, zi;
    auto rows = [&](auto wrap) {
#pragma unroll
        for (int a = 0; a < W; ++a) {
            const float kta = es_kernel_acc((((float)a + fth) + ftl) * sc, beta);
            const long long rowoff = (long long)(pc.r0 + a) * Npf;
            kahan rr;
            [[maybe_unused]] kahan ri;
#pragma unroll
            for (int b = 0; b < W; ++b) {
                int c = pc.p0 + b;
                if constexpr (decltype(wrap)::value) c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
                if constexpr (CPLX) {
                    const float2 v = reinterpret_cast<const float2 *>(U)[rowoff + c];
                    rr.add(kp[b] * v.x);
                    ri.add(kp[b] * v.y);
                } else {
                    rr.add(kp[b] * U[rowoff + c]);
                }
            }
            // row sums carry their compensation into the outer sum
            zr.add(kta * rr.s);
            zr.add(-kta * rr.c);
            if constexpr (CPLX) {
                zi.add(kta * ri.s);
                zi.add(-kta * ri.c);
            }
        }
    };
    // complex grid away from phi = 0: each row's taps come as NQ aligned
    // 16-byte loads (two taps each) from the even column pa <= p0, with the
    // weights shifted by p0 - pa and zero on the extra tap(s): about half the
    // load instructions of one 8-byte load per tap (Npf is even, so every
    // row of every request starts 16-byte aligned)
    constexpr int NQ = (W + 2) / 2;
    const int pa = pc.p0 & ~1;
    if (CPLX && pc.p0 >= 0 && pa + 2 * NQ <= Npf) {
        const bool odd = pc.p0 & 1;
        float kq[2 * NQ];
#pragma unroll
        for (int i = 0; i < 2 * NQ; ++i) {
            const float ke = i < W ? kp[i] : 0.f, ko = (i >= 1 && i - 1 < W) ? kp[i - 1] : 0.f;
            kq[i] = odd ? ko : ke;
        }
#pragma unroll
        for (int a = 0; a < W; ++a) {
            const float kta = es_kernel_acc((((float)a + fth) + ftl) * sc, beta);
            const float4 *row = reinterpret_cast<const float4 *>(U + 2 * ((long long)(pc.r0 + a) * Npf + pa));
            kahan rr, ri;
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const float4 v = row[q];
                rr.add(kq[2 * q] * v.x);
                ri.add(kq[2 * q] * v.y);
                rr.add(kq[2 * q + 1] * v.z);
                ri.add(kq[2 * q + 1] * v.w);
            }
            zr.add(kta * rr.s);
            zr.add(-kta * rr.c);
            zi.add(kta * ri.s);
            zi.add(-kta * ri.c);
        }
    } else if (pc.p0 >= 0 && pc.p0 + W <= Npf) {
        rows(std::false_type{});
    } else {
        rows(std::true_type{});
    }
    // the compensated sums as double-floats (value s - c); no FP64 instruction below
    if constexpr (CPLX) {
        dfl vr = df_fast(zr.s, -zr.c), vi = df_fast(zi.s, -zi.c);
        if (gamma) {
            // (vr + i vi) e^{i x}: 1 - cos x = 2 sin^2(x / 2) keeps the FP32
            // error of the small correction terms relative to the angle
            const float x = (float)spin * df_from(gamma[j]).h;
            const float sh = sinf(0.5f * x);
            const float d = 2.f * sh * sh;  // 1 - cos x
            const float s = sinf(x);
            const float cr = fmaf(vi.h, s, vr.h * d), ci = fmaf(vr.h, -s, vi.h * d);
            vr = df_add(vr, dfl{-cr, 0.f});
            vi = df_add(vi, dfl{-ci, 0.f});
        }
        if (out_f32) {
            ((float *)out)[j] = vr.h + vr.l;
            ((float *)out)[npts + j] = vi.h + vi.l;
        } else {
            ((double *)out)[j] = df_to(vr);
            ((double *)out)[npts + j] = df_to(vi);
        }
    } else {
        const dfl v = df_fast(zr.s, -zr.c);
        if (out_f32) ((float *)out)[j] = v.h + v.l;
        else ((double *)out)[j] = df_to(v);
    }
}

int nufft_interp_batch(const cunusht_plan_s *P, int nreq, int spin, const void *U, long long ubs, const double *loc,
                       long long lbs, long long npts, int layout, const double *gamma, void *out, long long obs,
                       int out_dtype, cudaStream_t st) {
    if (npts == 0 || nreq == 0) return CUNUSHT_OK;
    dim3 grid((unsigned)((npts + NU_TPB - 1) / NU_TPB), nreq);
    const int f32o = out_dtype == CUNUSHT_F32;
    with_width(P->w, [&](auto WC) {
        constexpr int W = decltype(WC)::value;
        if (P->fwd_u32 || P->grid_fp32) {  // FP32 grid of a mixed plan
            if (spin == 0)
                k_interp_mixed<false, W><<<grid, NU_TPB, 0, st>>>((const float *)U, P->nrows, P->Npf, P->Ntf, P->n_lo,
                                                                  W, (float)P->beta, loc, npts, layout, gamma, spin,
                                                                  out, f32o, ubs, lbs, obs);
            else
                k_interp_mixed<true, W><<<grid, NU_TPB, 0, st>>>((const float *)U, P->nrows, P->Npf, P->Ntf, P->n_lo,
                                                                 W, (float)P->beta, loc, npts, layout, gamma, spin,
                                                                 out, f32o, ubs, lbs, obs);
        } else {
            if (spin == 0)
                k_interp<double, false, W><<<grid, NU_TPB, 0, st>>>((const double *)U, P->nrows, P->Npf, P->Ntf,
                                                                    P->n_lo, W, P->beta, loc, npts, layout, gamma,
                                                                    spin, out, f32o, ubs, lbs, obs);
            else
                k_interp<double, true, W><<<grid, NU_TPB, 0, st>>>((const double *)U, P->nrows, P->Npf, P->Ntf,
                                                                   P->n_lo, W, P->beta, loc, npts, layout, gamma,
                                                                   spin, out, f32o, ubs, lbs, obs);
        }
    });
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int nufft_interp(const cunusht_plan_s *P, int spin, const double *loc, long long npts, int layout,
                 const double *gamma, void *out, int out_dtype, cudaStream_t st) {
    return nufft_interp_batch(P, 1, spin, P->d_U, 0, loc, 0, npts, layout, gamma, out, 0, out_dtype, st);
}

// nreq requests: grid U + r ubs (scalars of the grid type, zeroed here),
// points loc + r lbs, values in + r ibs (elements), gamma + r npts
int nufft_spread_batch(const cunusht_plan_s *P, int nreq, int spin, void *U, long long ubs, const double *loc,
                       long long lbs, long long npts, int layout, const double *gamma, const void *in, long long ibs,
                       int in_dtype, cudaStream_t st) {
    const size_t scal = P->grid_fp32 ? 4 : 8;
    const size_t cell = scal * (spin ? 2 : 1);
    for (int r = 0; r < nreq; ++r)
        CU_TRY(cudaMemsetAsync((char *)U + r * ubs * scal, 0, cell * (size_t)P->nrows * P->Npf, st));
    if (npts == 0) return CUNUSHT_OK;
    const int f32i = in_dtype == CUNUSHT_F32;
    // the plan's spreading options: bin-sorted path, fixed-point accumulation
    int done = 0;
    RC_TRY(spread_options_begin(P, nreq, spin, U, ubs, loc, lbs, npts, layout, gamma, in, ibs, in_dtype, &done, st));
    if (done) return spread_options_end(P, nreq, spin, U, ubs, npts, st);
    if (P->grid_fp32) {  // FP32 grid (eps > 1e-6), always a mixed plan
        if (spin == 0) RC_TRY((launch_spread_warp_mixed<float, false>(P, nreq, (float *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, st)));
        else RC_TRY((launch_spread_warp_mixed<float, true>(P, nreq, (float *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, st)));
    } else if (P->prec == CUNUSHT_PREC_MIXED) {
        if (spin == 0) RC_TRY((launch_spread_warp_mixed<double, false>(P, nreq, (double *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, st)));
        else RC_TRY((launch_spread_warp_mixed<double, true>(P, nreq, (double *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, st)));
    } else {
        if (spin == 0) RC_TRY((launch_spread_warp<double, false>(P, nreq, (double *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, st)));
        else RC_TRY((launch_spread_warp<double, true>(P, nreq, (double *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, st)));
    }
    CU_LAUNCH_CHECK();
    return spread_options_end(P, nreq, spin, U, ubs, npts, st);
}

int nufft_spread(const cunusht_plan_s *P, int spin, const double *loc, long long npts, int layout,
                 const double *gamma, const void *in, int in_dtype, cudaStream_t st) {
    return nufft_spread_batch(P, 1, spin, P->d_U, 0, loc, 0, npts, layout, gamma, in, 0, in_dtype, st);
}

// ------------------------------------------------------------ pointing
// Deflected angles per pixel, cunusht/c/pointing.cu:210-222 (one thread per
// pixel instead of one per ring); the rotation angle gamma of
// CPU_nufft_transformer.py:160 is computed as a single atan2 of the angle
// difference (equal modulo 2 pi).
__global__ void __launch_bounds__(256)
    k_pointing(int nring, const double *__restrict__ rth, const double *__restrict__ rph0,
               const long long *__restrict__ rnph, const long long *__restrict__ rofs, long long npix,
               const double *__restrict__ dth, const double *__restrict__ dph,
               double *__restrict__ oth, double *__restrict__ oph, double *__restrict__ ogam, long long dbs,
               long long pbs) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npix) return;
    dth += blockIdx.y * dbs;  // request of a batch
    dph += blockIdx.y * dbs;
    oth += blockIdx.y * pbs;
    oph += blockIdx.y * pbs;
    if (ogam) ogam += blockIdx.y * npix;
    int lo = 0, hi = nring - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (rofs[mid] <= j) lo = mid;
        else hi = mid - 1;
    }
    const int ring = lo;
    const double theta = rth[ring];
    const long long nph = rnph[ring];
    const double phi = rph0[ring] + (double)(j - rofs[ring]) * (TWOPI / (double)nph);
    const double t = dth[j], p = dph[j];
    const double d2 = t * t + p * p;
    double sinaoa, cosa;
    if (d2 > 1e-6) {
        const double a = sqrt(d2);
        double sa;
        sincos(a, &sa, &cosa);
        sinaoa = sa / a;
    } else {
        // sin(a)/a and cos(a) series, error < a^10/10!
        sinaoa = 1.0 - d2 / 6.0 * (1.0 - d2 / 20.0 * (1.0 - d2 / 42.0 * (1.0 - d2 / 72.0)));
        cosa = 1.0 - d2 / 2.0 * (1.0 - d2 / 12.0 * (1.0 - d2 / 30.0 * (1.0 - d2 / 56.0)));
    }
    double st, ct;
    sincos(theta, &st, &ct);
    const double nx = st * cosa + ct * t * sinaoa;
    const double ny = -p * sinaoa;
    const double nz = ct * cosa - st * t * sinaoa;
    oth[j] = atan2(sqrt(nx * nx + ny * ny), nz);
    double php = phi - atan2(ny, nx);
    if (php >= TWOPI) php -= TWOPI;
    oph[j] = php;
    if (ogam) {
        // gamma = atan2(p, t) - atan2(p, d sin d cot(theta) + t cos d)
        //       = atan2(p * x2 - t * p, t * x2 + p * p),  x2 = d^2 (sin d / d) cot + t cos d
        const double x2 = d2 * sinaoa * (ct / st) + t * cosa;
        ogam[j] = (d2 > 0.0) ? atan2(p * x2 - t * p, t * x2 + p * p) : 0.0;
    }
}

// Mixed-precision pointing: the same rotation as k_pointing, written as small
// increments evaluated in double-float (FP32 hi/lo) and added to the ring
// angles in FP64:
//   phi'   = phi + atan(d_p S / nx),  nx = st C + ct d_t S
//   theta' = theta + asin( ct num / (rho + st C) + st^2 d_t S ),
//   num = rho^2 - st^2 C^2 = 2 st ct C d_t S + (ct^2 d_t^2 + d_p^2) S^2
// (sin(theta' - theta) = rho ct - nz st), S = sin(a)/a = 1 + s1,
// C = cos a = 1 + c1 with the small s1, c1 from their series in FP32;
// asin / atan of the small increments by x + (x^3/6 + 3x^5/40) and
// x - x^3/3 + x^5/5 with the correction in FP32 (FP64 atan2 / asin for the
// few near-pole pixels where the increment is not small).
// gamma = atan2(d_p (x2 - d_t), d_t x2 + d_p^2), x2 - d_t = a^2 S cot + d_t c1,
// in FP32 (it only enters through exp(i s gamma)).
__device__ __forceinline__ dfl df_div(dfl a, dfl b) {
    const float q0 = a.h / b.h;
    // r = a - q0 b
    const float p = q0 * b.h;
    const float pe = fmaf(q0, b.h, -p);
    float r = (a.h - p) - pe;
    r = fmaf(-q0, b.l, r) + a.l;
    return df_fast(q0, r / b.h);
}

__device__ __forceinline__ dfl df_sqrt(dfl a) {
    if (a.h <= 0.f) return dfl{0.f, 0.f};
    const float r0 = sqrtf(a.h);
    const float e = fmaf(-r0, r0, a.h) + a.l;
    return df_fast(r0, e / (2.f * r0));
}

// the large-angle branches of k_pointing_mixed in FP64, out of line so that
// the common (series) path carries no predicated FP64 instruction
static __device__ __noinline__ dfl df_asin_fp64(dfl s) { return df_from(asin(fmin(fmax(df_to(s), -1.0), 1.0))); }
static __device__ __noinline__ dfl df_atan2_fp64(dfl y, dfl x) { return df_from(atan2(df_to(y), df_to(x))); }

__global__ void __launch_bounds__(256)
    k_pointing_mixed(int nring, int nph_uniform, const double *__restrict__ rth,
                     const float4 *__restrict__ rsc, const double *__restrict__ rph0,
                     const long long *__restrict__ rnph, const long long *__restrict__ rofs, long long npix,
                     const double *__restrict__ dth, const double *__restrict__ dph, double *__restrict__ oth,
                     double *__restrict__ oph, double *__restrict__ ogam, long long dbs, long long pbs) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npix) return;
    dth += blockIdx.y * dbs;  // request of a batch
    dph += blockIdx.y * dbs;
    oth += blockIdx.y * pbs;
    oph += blockIdx.y * pbs;
    if (ogam) ogam += blockIdx.y * npix;
    int ring;
    if (nph_uniform > 0) {
        // 32-bit division when it fits (64-bit division is a long software sequence)
        ring = j < 0x7FFFFFFFLL ? (int)((unsigned)j / (unsigned)nph_uniform) : (int)(j / nph_uniform);
    } else {
        int lo = 0, hi = nring - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (rofs[mid] <= j) lo = mid;
            else hi = mid - 1;
        }
        ring = lo;
    }
    // ring angles and the pixel's longitude as double-floats (no FP64 division)
    const dfl twopi{0x1.921fb6p+2f, -0x1.777a5cp-23f};  // 2 pi
    const dfl theta = df_from(rth[ring]);
    const float nph = (float)(int)rnph[ring];  // 32-bit integer conversions
    const dfl phi =
        df_add(df_from(rph0[ring]), df_mul(dfl{(float)(int)(j - rofs[ring]), 0.f}, df_div(twopi, dfl{nph, 0.f})));
    const double t64 = dth[j], p64 = dph[j];
    const dfl t = df_from(t64), p = df_from(p64);
    const float d2 = t.h * t.h + p.h * p.h;
    float s1, c1;
    if (d2 < 1e-3f) {
        s1 = -d2 / 6.f * (1.f - d2 / 20.f * (1.f - d2 / 42.f));
        c1 = -0.5f * d2 * (1.f - d2 / 12.f * (1.f - d2 / 30.f * (1.f - d2 / 56.f)));
    } else {
        const float a = sqrtf(d2);
        const float sh = sinf(0.5f * a);
        s1 = sinf(a) / a - 1.f;
        c1 = -2.f * sh * sh;
    }
    const dfl S{1.f, s1}, C{1.f, c1};
    const float4 sc = rsc[ring];
    const dfl st{sc.x, sc.y}, ct{sc.z, sc.w};
    const dfl tS = df_mul(t, S);
    const dfl stC = df_mul(st, C);
    const dfl nx = df_add(stC, df_mul(ct, tS));
    const dfl pS = df_mul(p, S);
    const dfl rho = df_sqrt(df_add(df_mul(nx, nx), df_mul(pS, pS)));
    const dfl ctt = df_mul(ct, t), two_st_ct_C = df_scale(df_mul(df_mul(st, ct), C), 2.f);
    const dfl num = df_add(df_mul(two_st_ct_C, tS), df_mul(df_add(df_mul(ctt, ctt), df_mul(p, p)), df_mul(S, S)));
    const dfl sdt = df_add(df_mul(ct, df_div(num, df_add(rho, stC))), df_mul(df_mul(st, st), tS));
    // series branches in double-float (deflections of a few arcmin); FP64 asin /
    // atan2 only for large angles
    dfl dtheta;
    if (fabsf(sdt.h) < 0.02f) {
        const float x = sdt.h, x2 = x * x;
        dtheta = df_add(sdt, dfl{x * x2 * (1.f / 6.f + 0.075f * x2), 0.f});
    } else {
        dtheta = df_asin_fp64(sdt);
    }
    oth[j] = df_to(df_add(theta, dtheta));
    dfl dphi;
    const dfl q = nx.h > 0.f ? df_div(pS, nx) : dfl{1e30f, 0.f};
    if (fabsf(q.h) < 0.02f) {
        const float x = q.h, x2 = x * x;
        dphi = df_add(q, dfl{x * x2 * (-1.f / 3.f + 0.2f * x2), 0.f});
    } else {
        dphi = df_atan2_fp64(pS, nx);
    }
    dfl php = df_add(phi, dphi);
    if (php.h > twopi.h || (php.h == twopi.h && php.l >= twopi.l)) php = df_add(php, df_neg(twopi));
    oph[j] = df_to(php);
    if (ogam) {
        const float x2m = d2 * (1.f + s1) * (sc.z / sc.x) + t.h * c1;  // x2 - d_t
        const float x2 = t.h + x2m;
        ogam[j] = d2 > 0.f ? df_to(dfl{atan2f(p.h * x2m, t.h * x2 + p.h * p.h), 0.f}) : 0.0;
    }
}

// ------------------------------------------------------------ lensing VJP (spin 0)
// Vector-Jacobian product of lenmap_j = f(theta'_j, phi'_j) with respect to
// the deflection d_j = (d_theta, d_phi) of every pixel:
//   dL/dd_i = g_j [ f_theta(n') e'_theta . dn'/dd_i + f_phi(n') / sin(theta') e'_phi . dn'/dd_i ],
//   n' = C n + S (d_theta e_theta + d_phi e_phi),  C = cos a, S = sin(a)/a,
//   dn'/dd_i = -S d_i n + K d_i (d_theta e_theta + d_phi e_phi) + S e_i,  K = (C - S)/a^2,
// (the pointing rotation of pointing.cu:210-213 as a vector formula).  The
// derivatives f_theta, f_phi of the unlensed field at the deflected points
// are interpolated from the same fine grid with the derivative of the same
// ES kernel, so this is the exact derivative of the implemented forward map.
template <typename TU>
__global__ void __launch_bounds__(256)
    k_lens_vjp_s0(const TU *__restrict__ U, int nrows, int Npf, int Ntf, int n_lo, int w, double beta,
                  int nring, const double *__restrict__ rth, const double *__restrict__ rph0,
                  const long long *__restrict__ rnph, const long long *__restrict__ rofs, long long npix,
                  const double *__restrict__ dth, const double *__restrict__ dph,
                  const double *__restrict__ ptg, const double *__restrict__ grad, double *__restrict__ gd) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npix) return;
    int lo = 0, hi = nring - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (rofs[mid] <= j) lo = mid;
        else hi = mid - 1;
    }
    const int ring = lo;
    const double theta = rth[ring];
    const double phi = rph0[ring] + (double)(j - rofs[ring]) * (TWOPI / (double)rnph[ring]);
    const double tp = ptg[j], pp = ptg[npix + j];
    const PointCoords pc = point_coords(tp, pp, Ntf, Npf, n_lo, nrows, w);
    double kt[MAXW], dkt[MAXW], kp[MAXW], dkp[MAXW];
    const double sc = 2.0 / w;
    const double dzt = -sc * Ntf / TWOPI, dzp = -sc * Npf / TWOPI;  // dz / dtheta, dz / dphi
#pragma unroll
    for (int a = 0; a < MAXW; ++a) {
        if (a < w) {
            const double zt = (pc.ft + a) * sc, zp = (pc.fp + a) * sc;
            const double qt = 1.0 - zt * zt, qp = 1.0 - zp * zp;
            const double rt = qt > 0.0 ? sqrt(qt) : 0.0, rp = qp > 0.0 ? sqrt(qp) : 0.0;
            kt[a] = qt > 0.0 ? exp(beta * (rt - 1.0)) : 0.0;
            kp[a] = qp > 0.0 ? exp(beta * (rp - 1.0)) : 0.0;
            dkt[a] = qt > 1e-24 ? kt[a] * (-beta * zt / rt) * dzt : 0.0;
            dkp[a] = qp > 1e-24 ? kp[a] * (-beta * zp / rp) * dzp : 0.0;
        }
    }
    double ft = 0.0, fp = 0.0;
    for (int a = 0; a < w; ++a) {
        const TU *row = U + (long long)(pc.r0 + a) * Npf;
        double r0 = 0.0, r1 = 0.0;
#pragma unroll
        for (int b = 0; b < MAXW; ++b) {
            if (b < w) {
                int c = pc.p0 + b;
                c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
                const double v = (double)row[c];
                r0 = fma(kp[b], v, r0);
                r1 = fma(dkp[b], v, r1);
            }
        }
        ft = fma(dkt[a], r0, ft);
        fp = fma(kt[a], r1, fp);
    }
    const double g = grad[j];
    const double Gt = g * ft, Gp = g * fp;
    const double t = dth[j], p = dph[j];
    const double a2 = t * t + p * p;
    double S, C, K;
    if (a2 < 1e-3) {
        S = 1.0 - a2 / 6.0 * (1.0 - a2 / 20.0 * (1.0 - a2 / 42.0 * (1.0 - a2 / 72.0)));
        C = 1.0 - a2 / 2.0 * (1.0 - a2 / 12.0 * (1.0 - a2 / 30.0 * (1.0 - a2 / 56.0)));
        K = -1.0 / 3.0 + a2 / 30.0 - a2 * a2 / 840.0 + a2 * a2 * a2 / 45360.0;
    } else {
        const double a = sqrt(a2);
        double sa;
        sincos(a, &sa, &C);
        S = sa / a;
        K = (C - S) / a2;
    }
    double st, ct, sp, cp;
    sincos(theta, &st, &ct);
    sincos(phi, &sp, &cp);
    const double n[3] = {st * cp, st * sp, ct};
    const double et[3] = {ct * cp, ct * sp, -st};
    const double ep[3] = {-sp, cp, 0.0};
    double stq, ctq, spq, cpq;
    sincos(tp, &stq, &ctq);
    sincos(pp, &spq, &cpq);
    const double etq[3] = {ctq * cpq, ctq * spq, -stq};
    const double epq[3] = {-spq, cpq, 0.0};
    const double gpq = Gp / fmax(stq, 1e-300);
    double dt_t = 0.0, dt_p = 0.0, dp_t = 0.0, dp_p = 0.0;  // e'_theta . dn'/dd_t, ...
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double dv = t * et[i] + p * ep[i];
        const double dnt = -S * t * n[i] + K * t * dv + S * et[i];
        const double dnp = -S * p * n[i] + K * p * dv + S * ep[i];
        dt_t += etq[i] * dnt;
        dp_t += epq[i] * dnt;
        dt_p += etq[i] * dnp;
        dp_p += epq[i] * dnp;
    }
    gd[j] = Gt * dt_t + gpq * dp_t;
    gd[npix + j] = Gt * dt_p + gpq * dp_p;
}

int lens_vjp_launch(const cunusht_plan_s *P, const double *ptg, const double *grad, double *gd, cudaStream_t st) {
    const int nb = (int)((P->npix + 255) / 256);
    if (P->fwd_u32 || P->grid_fp32)
        k_lens_vjp_s0<float><<<nb, 256, 0, st>>>((const float *)P->d_U, P->nrows, P->Npf, P->Ntf, P->n_lo, P->w,
                                                 P->beta, P->nring, P->d_ring_theta, P->d_ring_phi0, P->d_ring_nph,
                                                 P->d_ring_ofs, P->npix, P->d_glmap, P->d_glmap + P->npix, ptg, grad,
                                                 gd);
    else
        k_lens_vjp_s0<double><<<nb, 256, 0, st>>>((const double *)P->d_U, P->nrows, P->Npf, P->Ntf, P->n_lo, P->w,
                                                  P->beta, P->nring, P->d_ring_theta, P->d_ring_phi0, P->d_ring_nph,
                                                  P->d_ring_ofs, P->npix, P->d_glmap, P->d_glmap + P->npix, ptg,
                                                  grad, gd);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int pointing_batch(const cunusht_plan_s *P, int nreq, const double *d, long long dbs, double *ptg, long long pbs,
                   double *gamma, cudaStream_t st) {
    if (P->npix == 0 || nreq == 0) return CUNUSHT_OK;
    dim3 grid((unsigned)((P->npix + 255) / 256), nreq);
    if (P->prec == CUNUSHT_PREC_MIXED)
        k_pointing_mixed<<<grid, 256, 0, st>>>(P->nring, P->nph_uniform, P->d_ring_theta, P->d_ring_sc, P->d_ring_phi0,
                                               P->d_ring_nph, P->d_ring_ofs, P->npix, d, d + P->npix, ptg,
                                               ptg + P->npix, gamma, dbs, pbs);
    else
        k_pointing<<<grid, 256, 0, st>>>(P->nring, P->d_ring_theta, P->d_ring_phi0, P->d_ring_nph, P->d_ring_ofs,
                                         P->npix, d, d + P->npix, ptg, ptg + P->npix, gamma, dbs, pbs);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int pointing_mixed_launch(int nring, int nph_uniform, const double *rth, const float4 *rsc, const double *rph0,
                          const long long *rnph, const long long *rofs, long long npix, const double *dth,
                          const double *dph, double *out_th, double *out_ph, double *out_gamma, cudaStream_t st) {
    if (npix == 0) return CUNUSHT_OK;
    const int nb = (int)((npix + 255) / 256);
    k_pointing_mixed<<<nb, 256, 0, st>>>(nring, nph_uniform, rth, rsc, rph0, rnph, rofs, npix, dth, dph, out_th,
                                         out_ph, out_gamma, 0, 0);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int pointing_launch(int nring, const double *rth, const double *rph0, const long long *rnph,
                    const long long *rofs, long long npix, const double *dth, const double *dph,
                    double *out_th, double *out_ph, double *out_gamma, cudaStream_t st) {
    if (npix == 0) return CUNUSHT_OK;
    const int nb = (int)((npix + 255) / 256);
    k_pointing<<<nb, 256, 0, st>>>(nring, rth, rph0, rnph, rofs, npix, dth, dph, out_th, out_ph, out_gamma, 0, 0);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// ------------------------------------------------------------ magnification matrix
// Determinant of the magnification matrix from the convergence kappa, shear
// (g1, g2), rotation w and deflection (d1, d2) maps (helper_GPU.py:145-161):
//   A = f0 ((1 - k)^2 - g1^2 - g2^2 + w^2)
//     + f1 (1 - k - ((d1^2 - d2^2) g1 + 2 d1 d2 g2) / d^2),
// f0 = sin d / d, f1 = cos d - f0.  Inputs are the unscaled syntheses:
// k = kp / 2, (g1, g2) = -(g1p, g2p) / 2, w = wp / 2 (wp may be NULL).  For
// small d the series of f0 and f1 replace the cancelling differences; at
// d = 0 the f1 term is 0 (the reference divides 0 by 0 there).
__global__ void k_magnification(long long npix, const double *__restrict__ kp, const double *__restrict__ g1p,
                                const double *__restrict__ g2p, const double *__restrict__ d1,
                                const double *__restrict__ d2, const double *__restrict__ wp,
                                double *__restrict__ A) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npix) return;
    const double k = 0.5 * kp[j], g1 = -0.5 * g1p[j], g2 = -0.5 * g2p[j], w = wp ? 0.5 * wp[j] : 0.0;
    const double a = d1[j], b = d2[j];
    const double dd = a * a + b * b;
    double f0, f1;
    if (dd > 1e-4) {
        const double d = sqrt(dd);
        double sn, cs;
        sincos(d, &sn, &cs);
        f0 = sn / d;
        f1 = cs - f0;
    } else {
        f0 = 1.0 - dd / 6.0 * (1.0 - dd / 20.0 * (1.0 - dd / 42.0 * (1.0 - dd / 72.0)));
        f1 = -dd / 3.0 * (1.0 - dd / 10.0 * (1.0 - dd / 28.0 * (1.0 - dd / 54.0)));
    }
    double r = f0 * ((1.0 - k) * (1.0 - k) - g1 * g1 - g2 * g2 + w * w);
    if (dd > 0.0) r += f1 * (1.0 - k - ((a * a - b * b) * g1 + 2.0 * a * b * g2) / dd);
    A[j] = r;
}

int magnification_det(long long npix, const double *k, const double *g1, const double *g2, const double *d1,
                      const double *d2, const double *w, double *A, cudaStream_t st) {
    if (npix == 0) return CUNUSHT_OK;
    k_magnification<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(npix, k, g1, g2, d1, d2, w, A);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// ------------------------------------------------------------ doubling
// The reference's doubling (doubling.cu:137-220): the CC map (nt rings x np
// longitudes, theta from 0 to pi) extended to the 2 pi theta torus (2 nt - 2
// rings): ring k >= nt is ring 2 nt - 2 - k shifted by pi in longitude,
// times (-1)^spin.  One CTA row per output row (blockIdx.y), threads along the
// contiguous axis -- no index division -- with 16-byte accesses (2 doubles /
// 4 floats per thread) when the rows and the pi shift stay 16-byte aligned.
// layout 0: ring-major in / out [ring][np]; layout 1: theta-contiguous
// in [np][nt] -> out [np][2 nt - 2].
// V consecutive elements as one access (16 bytes when V > 1; the caller
// guarantees the alignment)
template <typename T, int V> struct vecT;
template <> struct vecT<double, 1> { using t = double; };
template <> struct vecT<float, 1> { using t = float; };
template <> struct vecT<double, 2> { using t = double2; };
template <> struct vecT<float, 4> { using t = float4; };

template <typename T, int V> __device__ __forceinline__ void ldv(const T *p, T (&v)[V]) {
    const typename vecT<T, V>::t w = *reinterpret_cast<const typename vecT<T, V>::t *>(p);
    static_assert(sizeof(w) == V * sizeof(T), "vector size");
    memcpy(v, &w, sizeof(w));
}

template <typename T, int V> __device__ __forceinline__ void stv(T *p, const T (&v)[V]) {
    typename vecT<T, V>::t w;
    memcpy(&w, v, sizeof(w));
    *reinterpret_cast<typename vecT<T, V>::t *>(p) = w;
}

template <typename T, int V>
__global__ void __launch_bounds__(256)
    k_doubling(const T *__restrict__ in, long long nt, long long np, int layout, T sg, T *__restrict__ out) {
    const long long dt = 2 * nt - 2;
    const long long h = np / 2;
    if (layout == 0) {
        // one CTA row per input ring j: read once, write torus rings j and
        // 2 nt - 2 - j (the latter shifted by pi, times sg)
        for (long long j = blockIdx.y; j < nt; j += gridDim.y) {
            const long long c0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * V;
            if (c0 >= np) continue;
            T v[V];
            ldv<T, V>(in + j * np + c0, v);
            stv<T, V>(out + j * np + c0, v);
            if (j > 0 && j < nt - 1) {
#pragma unroll
                for (int e = 0; e < V; ++e) v[e] *= sg;
                const long long cm = c0 < h ? c0 + h : c0 - h;  // a V-group never straddles h (h % V == 0)
                stv<T, V>(out + (dt - j) * np + cm, v);
            }
        }
    } else {
        // theta-contiguous: one CTA row per longitude i of the output
        for (long long i = blockIdx.y; i < np; i += gridDim.y) {
            const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
            if (k >= dt) continue;
            const long long im = i < h ? i + h : i - h;
            out[i * dt + k] = k < nt ? in[i * nt + k] : sg * in[im * nt + (dt - k)];
        }
    }
}

template <typename T, int V>
__global__ void __launch_bounds__(256)
    k_adjoint_doubling(const T *__restrict__ in, long long nt, long long np, T sg, T *__restrict__ out) {
    const long long h = np / 2;
    for (long long k = blockIdx.y; k < nt; k += gridDim.y) {
        const long long c0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * V;
        if (c0 >= np) continue;
        T v[V];
        ldv<T, V>(in + k * np + c0, v);
        if (k > 0 && k < nt - 1) {
            const long long km = 2 * nt - 2 - k;
            const long long im = c0 < h ? c0 + h : c0 - h;
            T u[V];
            ldv<T, V>(in + km * np + im, u);
#pragma unroll
            for (int e = 0; e < V; ++e) v[e] += sg * u[e];
        }
        stv<T, V>(out + k * np + c0, v);
    }
}

template <typename T, int V>
static void doubling_go(const void *in, long long nt, long long np, int layout, T sg, void *out, cudaStream_t st) {
    const long long nrow = layout == 1 ? np : nt, ncol = layout == 1 ? 2 * nt - 2 : np;
    const dim3 grid((unsigned)((ncol / V + 255) / 256), (unsigned)std::min<long long>(nrow, 65535));
    k_doubling<T, V><<<grid, 256, 0, st>>>((const T *)in, nt, np, layout, sg, (T *)out);
}

template <typename T, int V>
static void adjoint_doubling_go(const void *in, long long nt, long long np, T sg, void *out, cudaStream_t st) {
    const dim3 grid((unsigned)((np / V + 255) / 256), (unsigned)std::min<long long>(nt, 65535));
    k_adjoint_doubling<T, V><<<grid, 256, 0, st>>>((const T *)in, nt, np, sg, (T *)out);
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

int doubling_launch(const void *in, long long nt, long long np, int layout, int spin, int dtype, void *out,
                    cudaStream_t st) {
    if ((2 * nt - 2) * np <= 0) return CUNUSHT_OK;
    const bool f32 = dtype == CUNUSHT_F32;
    const int V = f32 ? 4 : 2;  // 16 bytes
    // vector path: ring-major rows of np elements, pi shift h = np / 2, all multiples of V
    const bool vec = layout == 0 && np % V == 0 && (np / 2) % V == 0 && aligned16(in) && aligned16(out);
    // (layout 1 runs one element per thread)
    if (f32) {
        if (vec) doubling_go<float, 4>(in, nt, np, layout, (spin & 1) ? -1.f : 1.f, out, st);
        else doubling_go<float, 1>(in, nt, np, layout, (spin & 1) ? -1.f : 1.f, out, st);
    } else {
        if (vec) doubling_go<double, 2>(in, nt, np, layout, (spin & 1) ? -1.0 : 1.0, out, st);
        else doubling_go<double, 1>(in, nt, np, layout, (spin & 1) ? -1.0 : 1.0, out, st);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

int adjoint_doubling_launch(const void *in, long long nt, long long np, int spin, int dtype, void *out,
                            cudaStream_t st) {
    if (nt * np <= 0) return CUNUSHT_OK;
    const bool f32 = dtype == CUNUSHT_F32;
    const int V = f32 ? 4 : 2;
    const bool vec = np % V == 0 && (np / 2) % V == 0 && aligned16(in) && aligned16(out);
    if (f32) {
        if (vec) adjoint_doubling_go<float, 4>(in, nt, np, (spin & 1) ? -1.f : 1.f, out, st);
        else adjoint_doubling_go<float, 1>(in, nt, np, (spin & 1) ? -1.f : 1.f, out, st);
    } else {
        if (vec) adjoint_doubling_go<double, 2>(in, nt, np, (spin & 1) ? -1.0 : 1.0, out, st);
        else adjoint_doubling_go<double, 1>(in, nt, np, (spin & 1) ? -1.0 : 1.0, out, st);
    }
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// ------------------------------------------------------------ alm dtype conversion
__global__ void k_c64_to_c128(const float2 *__restrict__ in, long long n, double2 *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_double2(in[i].x, in[i].y);
}
__global__ void k_c128_to_c64(const double2 *__restrict__ in, long long n, float2 *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

int convert_alm(const void *in, int dtype, long long n, double2 *out, cudaStream_t st) {
    if (dtype == CUNUSHT_F64) {
        CU_TRY(cudaMemcpyAsync(out, in, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    } else {
        k_c64_to_c128<<<(int)((n + 255) / 256), 256, 0, st>>>((const float2 *)in, n, out);
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

int store_alm(const double2 *in, long long n, int dtype, void *out, cudaStream_t st) {
    if (dtype == CUNUSHT_F64) {
        CU_TRY(cudaMemcpyAsync(out, in, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    } else {
        k_c128_to_c64<<<(int)((n + 255) / 256), 256, 0, st>>>(in, n, (float2 *)out);
        CU_LAUNCH_CHECK();
    }
    return CUNUSHT_OK;
}

}  // namespace cunusht

// Spreading options of the type-1 nuFFT (nusht2d1 / delensing), the choices
// cuFINUFFT's gpu_method / gpu_sort make in the reference's plan
// (cunusht/deflection/GPU_nufft_transformer.py:242-246: method 2 = shared-memory
// spreading of sorted points):
//
// * Bin-sorted spreading, for points in any order.  The fine grid is cut into
//   bins of BIN x BIN cells; every point goes to the bin of its first tap cell
//   (k_bin_count), the bin sizes are scanned (k_bin_scan) and the point indices
//   scattered into bin order (k_bin_scatter).  One block per bin then adds its
//   points' w x w footprints to a shared-memory tile of (BIN + w - 1)^2 cells
//   and the tile to the grid: one global atomic per touched cell instead of one
//   per tap.  (The warp-strip kernels of nufft.cu need neighbouring points in
//   neighbouring threads, as the ring-ordered lensing pointing has them.)
// * Deterministic accumulation, with either path: the grid sums are formed in
//   int64 fixed point, unit 2^E per request with E from the request's largest
//   |value| and the point count, so that no sum can overflow; integer addition
//   is exact, so the result does not depend on the order in which the atomics
//   land.  A last pass converts to the grid's type.  The deterministic bin
//   tiles are int64 fixed point as well.
#include <type_traits>

#include "common.cuh"
#include "kernels.cuh"
#include "nufft_pts.cuh"

namespace cunusht {

constexpr int BIN = 32;       // fine cells per bin side
constexpr int BIN_TPB = 128;  // threads per bin block

// largest |value| of each request (blockIdx.y), float bits maxed into vmax
__global__ void k_spread_vmax(const void *__restrict__ in, int in_f32, long long n, long long ibs,
                              float *__restrict__ vmax) {
    const int r = blockIdx.y;
    float mx = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        mx = fmaxf(mx, in_f32 ? fabsf(((const float *)in)[r * ibs + i]) : fabsf((float)((const double *)in)[r * ibs + i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int *>(vmax + r), __float_as_int(mx * 1.000001f));
}

template <typename T>
__global__ void k_fix_to_grid(const unsigned long long *__restrict__ Ufix, T *__restrict__ U, long long n, long long ubs,
                              const float *__restrict__ vmax, int lgn) {
    const int r = blockIdx.y;
    const int E = fix_exp(vmax[r], lgn);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long v = (long long)Ufix[r * ubs + i];
        if constexpr (std::is_same<T, float>::value) U[r * ubs + i] = ldexpf(__ll2float_rn(v), E);
        else U[r * ubs + i] = ldexp((double)v, E);
    }
}

// bin of every point (the bin of its first tap cell) and the bin sizes
__global__ void k_bin_count(int nrows, int Npf, int Ntf, int n_lo, int w, const double *__restrict__ loc, long long npts,
                            int layout, long long lbs, int nbc, int nbins, int *__restrict__ bin_of,
                            int *__restrict__ cnt) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npts) return;
    const int r = blockIdx.y;
    double th, ph;
    load_point(loc + r * lbs, j, npts, layout, th, ph);
    const PointCoords pc = point_coords(th, ph, Ntf, Npf, n_lo, nrows, w);
    int c = pc.p0;
    c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
    const int b = (pc.r0 / BIN) * nbc + c / BIN;
    bin_of[r * npts + j] = b;
    atomicAdd(cnt + (long long)r * (nbins + 1) + b, 1);
}

// exclusive scan of the bin sizes (in place, entry nbins = total) and a copy
// as the scatter cursor; one block per request
__global__ void __launch_bounds__(1024) k_bin_scan(int *__restrict__ cnt, int nbins, int *__restrict__ cursor) {
    __shared__ int s_w[32];
    __shared__ int s_carry;
    int *c = cnt + (long long)blockIdx.x * (nbins + 1);
    int *cur = cursor + (long long)blockIdx.x * (nbins + 1);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < nbins; base += 1024) {
        const int i = base + tid;
        const int v = i < nbins ? c[i] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int t = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            s_w[lane] = t;  // inclusive over warps
        }
        __syncthreads();
        const int carry = s_carry;
        const int excl = carry + (wid ? s_w[wid - 1] : 0) + x - v;
        if (i < nbins) {
            c[i] = excl;
            cur[i] = excl;
        }
        __syncthreads();
        if (tid == 0) s_carry = carry + s_w[31];
        __syncthreads();
    }
    if (tid == 0) c[nbins] = s_carry;
}

__global__ void k_bin_scatter(const int *__restrict__ bin_of, long long npts, int nbins, int *__restrict__ cursor,
                              int *__restrict__ perm) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npts) return;
    const int r = blockIdx.y;
    const int pos = atomicAdd(cursor + (long long)r * (nbins + 1) + bin_of[r * npts + j], 1);
    perm[r * npts + pos] = (int)j;
}

// A point's value (rotated by exp(-i spin gamma) for spin s), its bin-relative
// first cell and its tap weights.  SPLIT: FP32 weights from the FP64 tap
// offset split into hi + lo floats (the mixed-precision FP64 grid, as
// k_spread_warp_mixed); else weights in the grid's type T (as k_spread_warp).
template <typename T, bool CPLX, bool SPLIT>
__device__ __forceinline__ void bin_point(const double *loc, long long j, long long npts, int layout,
                                          const double *gamma, int spin, const void *in, int in_f32, int nrows,
                                          int Npf, int Ntf, int n_lo, int w, double beta, int br, int bc, int &lr,
                                          int &lc, T &vr, T &vi, T *kt, T *kp) {
    double th, ph;
    load_point(loc, j, npts, layout, th, ph);
    const PointCoords pc = point_coords(th, ph, Ntf, Npf, n_lo, nrows, w);
    int c = pc.p0;
    c = c < 0 ? c + Npf : (c >= Npf ? c - Npf : c);
    lr = pc.r0 - br * BIN;
    lc = c - bc * BIN;
    double xr = in_f32 ? ((const float *)in)[j] : ((const double *)in)[j], xi = 0.0;
    if (CPLX) {
        xi = in_f32 ? ((const float *)in)[npts + j] : ((const double *)in)[npts + j];
        if (gamma) {
            double s, co;
            sincos(spin * gamma[j], &s, &co);  // multiply by e^{-i spin gamma}
            const double t2 = xr * co + xi * s;
            xi = xi * co - xr * s;
            xr = t2;
        }
    }
    vr = (T)xr;
    vi = (T)xi;
    if (SPLIT) {
        const float sc = 2.f / (float)w;
        const float fth = (float)pc.ft, ftl = (float)(pc.ft - (double)fth);
        const float fph = (float)pc.fp, fpl = (float)(pc.fp - (double)fph);
        for (int a = 0; a < w; ++a) {
            kt[a] = (T)es_kernel_acc((((float)a + fth) + ftl) * sc, (float)beta);
            kp[a] = (T)es_kernel_acc((((float)a + fph) + fpl) * sc, (float)beta);
        }
    } else {
        const T s = (T)2 / (T)w;
        for (int a = 0; a < w; ++a) {
            kt[a] = es_kernel<T>(((T)pc.ft + (T)a) * s, (T)beta);
            kp[a] = es_kernel<T>(((T)pc.fp + (T)a) * s, (T)beta);
        }
    }
}

// One block per (bin, request); threads take points and add their taps to a
// shared-memory tile, which then goes to the grid with one global atomic per
// touched cell.  DET: the tile holds int64 fixed point (per-tap rounding to the
// request's unit 2^E, far below the grid type's rounding) and goes to the
// fixed-point grid Ufix: integer sums, so the order in which points reach the
// bin (atomic scatter cursors) and the tile does not matter.  Else the tile
// holds the grid type T and goes to U.
template <typename T, bool CPLX, bool DET, bool SPLIT>
__global__ void __launch_bounds__(BIN_TPB)
    k_spread_bins(T *__restrict__ U, unsigned long long *__restrict__ Ufix, int nrows, int Npf, int Ntf, int n_lo,
                  int w, double beta, const double *__restrict__ loc, long long npts, int layout,
                  const double *__restrict__ gamma, int spin, const void *__restrict__ in, int in_f32,
                  const int *__restrict__ off, const int *__restrict__ perm, int nbc, int nbins, long long ubs,
                  long long lbs, long long ibs, const float *__restrict__ vmax, int lgn) {
    using A = typename std::conditional<DET, unsigned long long, T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NC = CPLX ? 2 : 1;
    const int r = blockIdx.y, bin = blockIdx.x, tid = threadIdx.x;
    off += (long long)r * (nbins + 1);
    const int k0 = off[bin], k1 = off[bin + 1];
    if (k0 == k1) return;
    perm += r * npts;
    loc += r * lbs;
    if (gamma) gamma += r * npts;
    in = in_f32 ? (const void *)((const float *)in + r * ibs) : (const void *)((const double *)in + r * ibs);
    const int PT = BIN + w - 1;  // tile side
    A *tile = reinterpret_cast<A *>(smem_raw);
    for (int i = tid; i < PT * PT * NC; i += BIN_TPB) tile[i] = (A)0;
    const int br = bin / nbc, bc = bin - (bin / nbc) * nbc;
    const int E = DET ? fix_exp(vmax[r], lgn) : 0;
    __syncthreads();
    for (int k = k0 + tid; k < k1; k += BIN_TPB) {
        int lr, lc;
        T vr, vi, kt[MAXW], kp[MAXW];
        bin_point<T, CPLX, SPLIT>(loc, perm[k], npts, layout, gamma, spin, in, in_f32, nrows, Npf, Ntf, n_lo, w, beta,
                                  br, bc, lr, lc, vr, vi, kt, kp);
        for (int a = 0; a < w; ++a) {
            const T fr = kt[a] * vr, fi = kt[a] * vi;
            A *row = tile + (size_t)((lr + a) * PT + lc) * NC;
            for (int b = 0; b < w; ++b) {
                if constexpr (DET) {
                    atomicAdd(row + b * NC, (unsigned long long)to_fix(kp[b] * fr, E));
                    if constexpr (CPLX) atomicAdd(row + b * NC + 1, (unsigned long long)to_fix(kp[b] * fi, E));
                } else {
                    atomicAdd(row + b * NC, kp[b] * fr);
                    if constexpr (CPLX) atomicAdd(row + b * NC + 1, kp[b] * fi);
                }
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < PT * PT; i += BIN_TPB) {
        const int lr = i / PT, lc = i - (i / PT) * PT;
        const int row = br * BIN + lr;
        if (row >= nrows) continue;
        const int col = (bc * BIN + lc) % Npf;
        const long long cell = ((long long)row * Npf + col) * NC;
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            const A v = tile[i * NC + q];
            if (v == (A)0) continue;
            if constexpr (DET) atomicAdd(Ufix + r * ubs + cell + q, v);
            else atomicAdd(U + r * ubs + cell + q, v);
        }
    }
}

static int ceil_log2(long long n) {
    int lg = 0;
    while ((1LL << lg) < n) ++lg;
    return lg;
}

size_t bin_workspace_ints(const cunusht_plan_s *P, long long npts) {
    const long long nbins = (long long)((P->nrows + BIN - 1) / BIN) * ((P->Npf + BIN - 1) / BIN);
    return (size_t)(2 * npts + 2 * (nbins + 1));
}

template <typename T, bool CPLX, bool DET, bool SPLIT>
static int launch_bins(const cunusht_plan_s *P, int nreq, T *U, long long ubs, const double *loc, long long lbs,
                       long long npts, int layout, const double *gamma, int spin, const void *in, long long ibs,
                       int f32i, const int *off, const int *perm, int nbc, int nbins, int lgn, cudaStream_t st) {
    const int PT = BIN + P->w - 1;
    const size_t sm = (size_t)PT * PT * (CPLX ? 2 : 1) * (DET ? sizeof(unsigned long long) : sizeof(T));
    auto kern = k_spread_bins<T, CPLX, DET, SPLIT>;
    if (sm > 48 * 1024) CU_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<dim3(nbins, nreq), BIN_TPB, sm, st>>>(U, P->d_ufix, P->nrows, P->Npf, P->Ntf, P->n_lo, P->w, P->beta, loc,
                                                 npts, layout, gamma, spin, in, f32i, off, perm, nbc, nbins, ubs, lbs,
                                                 ibs, P->d_vmax, lgn);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

// The spreading options of the plan around the warp-strip kernels: fixed-point
// set-up and conversion (deterministic), and the bin-sorted path.  U (zeroed
// by the caller) holds nreq grids of ubs scalars; returns 1 in *done when the
// bin path spread the points, 0 when the warp-strip kernels still have to run
// (they then write the fixed-point grid when the plan is deterministic).
int spread_options_begin(const cunusht_plan_s *P, int nreq, int spin, void *U, long long ubs, const double *loc,
                         long long lbs, long long npts, int layout, const double *gamma, const void *in,
                         long long ibs, int in_dtype, int *done, cudaStream_t st) {
    *done = 0;
    const bool det = P->spread_det;
    const int lgn = ceil_log2(npts + 1);
    const int NC = spin ? 2 : 1;
    const int f32i = in_dtype == CUNUSHT_F32;
    if (det) {
        const size_t span = ((size_t)(nreq - 1) * ubs + (size_t)NC * P->nrows * P->Npf) * sizeof(unsigned long long);
        if (!P->d_ufix || span > P->ufix_bytes || !P->d_vmax || nreq > 64) {
            set_error("deterministic spreading workspace too small for %d requests", nreq);
            return CUNUSHT_ERR_ARG;
        }
        CU_TRY(cudaMemsetAsync(P->d_ufix, 0, span, st));
        CU_TRY(cudaMemsetAsync(P->d_vmax, 0, sizeof(float) * 64, st));
        k_spread_vmax<<<dim3(256, nreq), 256, 0, st>>>(in, f32i, npts * NC, ibs, P->d_vmax);
        CU_LAUNCH_CHECK();
    }
    const bool bins = P->spread_method == 1 && npts <= P->bin_npts && nreq <= P->spread_nreq && npts < (1LL << 31);
    if (!bins) return CUNUSHT_OK;
    const int nbc = (P->Npf + BIN - 1) / BIN;
    const int nbins = ((P->nrows + BIN - 1) / BIN) * nbc;
    int *bin_of = P->d_bin, *perm = bin_of + (size_t)nreq * npts;
    int *cnt = perm + (size_t)nreq * npts, *cursor = cnt + (size_t)nreq * (nbins + 1);
    CU_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)nreq * (nbins + 1), st));
    const dim3 gp((unsigned)((npts + 255) / 256), nreq);
    k_bin_count<<<gp, 256, 0, st>>>(P->nrows, P->Npf, P->Ntf, P->n_lo, P->w, loc, npts, layout, lbs, nbc, nbins, bin_of,
                                    cnt);
    CU_LAUNCH_CHECK();
    k_bin_scan<<<nreq, 1024, 0, st>>>(cnt, nbins, cursor);
    CU_LAUNCH_CHECK();
    k_bin_scatter<<<gp, 256, 0, st>>>(bin_of, npts, nbins, cursor, perm);
    CU_LAUNCH_CHECK();
    const int *off = cnt;
    auto go = [&](auto tag, auto cplx, auto detc, auto split) {
        using T = decltype(tag);
        return launch_bins<T, decltype(cplx)::value, decltype(detc)::value, decltype(split)::value>(
            P, nreq, (T *)U, ubs, loc, lbs, npts, layout, gamma, spin, in, ibs, f32i, off, perm, nbc, nbins, lgn, st);
    };
    using TT = std::true_type;
    using FF = std::false_type;
    int rc;
    const bool split = !P->grid_fp32 && P->prec == CUNUSHT_PREC_MIXED;
    if (P->grid_fp32) {
        if (spin) rc = det ? go(0.f, TT{}, TT{}, FF{}) : go(0.f, TT{}, FF{}, FF{});
        else rc = det ? go(0.f, FF{}, TT{}, FF{}) : go(0.f, FF{}, FF{}, FF{});
    } else if (split) {
        if (spin) rc = det ? go(0.0, TT{}, TT{}, TT{}) : go(0.0, TT{}, FF{}, TT{});
        else rc = det ? go(0.0, FF{}, TT{}, TT{}) : go(0.0, FF{}, FF{}, TT{});
    } else {
        if (spin) rc = det ? go(0.0, TT{}, TT{}, FF{}) : go(0.0, TT{}, FF{}, FF{});
        else rc = det ? go(0.0, FF{}, TT{}, FF{}) : go(0.0, FF{}, FF{}, FF{});
    }
    RC_TRY(rc);
    *done = 1;
    return CUNUSHT_OK;
}

// deterministic: the fixed-point sums -> the grid's type
int spread_options_end(const cunusht_plan_s *P, int nreq, int spin, void *U, long long ubs, long long npts,
                       cudaStream_t st) {
    if (!P->spread_det) return CUNUSHT_OK;
    const long long n = (long long)(spin ? 2 : 1) * P->nrows * P->Npf;
    const int lgn = ceil_log2(npts + 1);
    if (P->grid_fp32)
        k_fix_to_grid<float><<<dim3(1024, nreq), 256, 0, st>>>(P->d_ufix, (float *)U, n, ubs, P->d_vmax, lgn);
    else
        k_fix_to_grid<double><<<dim3(1024, nreq), 256, 0, st>>>(P->d_ufix, (double *)U, n, ubs, P->d_vmax, lgn);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

}  // namespace cunusht

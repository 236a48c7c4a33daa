// Shared definitions of the cunusht_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <vector>
#include <string>

#include "../../include/cunusht_gb300.h"
#include "df.cuh"

namespace cunusht {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
void clear_error();

#define CU_TRY(expr)                                                                     \
    do {                                                                                 \
        cudaError_t _e = (expr);                                                         \
        if (_e != cudaSuccess) {                                                         \
            ::cunusht::set_error("%s:%d: %s -> %s", __FILE__, __LINE__, #expr,           \
                                 cudaGetErrorString(_e));                                \
            return CUNUSHT_ERR_CUDA;                                                     \
        }                                                                                \
    } while (0)

#define CU_LAUNCH_CHECK()                                                                \
    do {                                                                                 \
        cudaError_t _e = cudaGetLastError();                                             \
        if (_e != cudaSuccess) {                                                         \
            ::cunusht::set_error("%s:%d: kernel launch -> %s", __FILE__, __LINE__,       \
                                 cudaGetErrorString(_e));                                \
            return CUNUSHT_ERR_CUDA;                                                     \
        }                                                                                \
    } while (0)

#define ARG_CHECK(cond, ...)                                                             \
    do {                                                                                 \
        if (!(cond)) {                                                                   \
            ::cunusht::set_error(__VA_ARGS__);                                           \
            return CUNUSHT_ERR_ARG;                                                      \
        }                                                                                \
    } while (0)

#define RC_TRY(expr)                                                                     \
    do {                                                                                 \
        int _rc = (expr);                                                                \
        if (_rc != CUNUSHT_OK) return _rc;                                               \
    } while (0)

// ---------------------------------------------------------------- complex
template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<dfl> { using type = dcplx; };

// scalar conversions used by code templated on float / double / dfl
template <typename T> __device__ __forceinline__ T cvt(double x) { return (T)x; }
template <> __device__ __forceinline__ dfl cvt<dfl>(double x) { return df_from(x); }
__device__ __forceinline__ double to_d(float x) { return (double)x; }
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(dfl x) { return df_to(x); }  // integer pipe, bit-exact
template <typename To> __device__ __forceinline__ To to_t(float x) { return (To)x; }
template <typename To> __device__ __forceinline__ To to_t(double x) { return (To)x; }
template <typename To> __device__ __forceinline__ To to_t(dfl x);
template <> __device__ __forceinline__ float to_t<float>(dfl x) { return x.h + x.l; }
template <> __device__ __forceinline__ double to_t<double>(dfl x) { return df_to(x); }
template <typename T> using cplx = typename cplx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T re, T im) {
    cplx<T> r;
    r.x = re;
    r.y = im;
    return r;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) {
    C r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) {
    C r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    return r;
}
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// Complex double-float product: each real part a b +- c d from the two
// unnormalised products (df_mul_u) and one full TwoSum of their leading parts,
// left unnormalised like every double-float addition of the butterflies
// (32 FP32 operations instead of the 44 of four renormalised products and
// two additions).
__device__ __forceinline__ dfl df_dot2_u(dfl a, dfl b, dfl c, dfl d) {  // a b + c d
    const dfl p = df_mul_u(a, b), q = df_mul_u(c, d);
    const float s = p.h + q.h;
    const float bb = s - p.h;
    const float t = (p.h - (s - bb)) + (q.h - bb);
    return dfl{s, (p.l + q.l) + t};
}
__device__ __forceinline__ dcplx cmul(dcplx a, dcplx b) {
    dcplx r;
    r.x = df_dot2_u(a.x, b.x, df_neg(a.y), b.y);
    r.y = df_dot2_u(a.x, b.y, a.y, b.x);
    return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) {
    C r;
    r.x = a.x;
    r.y = -a.y;
    return r;
}
template <typename C, typename S> __host__ __device__ __forceinline__ C cscale(C a, S s) {
    C r;
    r.x = a.x * s;
    r.y = a.y * s;
    return r;
}
// multiply by i*dir (dir = +1 or -1)
template <typename C> __host__ __device__ __forceinline__ C cmul_idir(C a, int dir) {
    C r;
    r.x = -dir * a.y;
    r.y = dir * a.x;
    return r;
}
template <typename To, typename From> __device__ __forceinline__ cplx<To> ccast(From a) {
    cplx<To> r;
    r.x = to_t<To>(a.x);
    r.y = to_t<To>(a.y);
    return r;
}

__host__ __device__ __forceinline__ long long almidx(int lmax, int l, int m) {
    return (long long)m * (2 * lmax + 1 - m) / 2 + l;
}

constexpr double PI = 3.141592653589793238462643383279502884;
constexpr double TWOPI = 6.283185307179586476925286766559005768;

}  // namespace cunusht

// ---------------------------------------------------------------- plan
// mixed-radix ring transforms: longest ring, most stages, radix constants
constexpr int MR_NMAX = 8192;
constexpr int MR_MAXST = 16;
constexpr int MR_KMAX = 128;

struct cunusht_plan_s {
    int lmax = 0;
    int max_spin = 0;
    int prec = CUNUSHT_PREC_FP64;  // resolved precision
    bool grid_fp32 = false;        // FFT + nuFFT grids in FP32
    bool fwd_u32 = false;          // forward fine grid stored FP32 (FFTs FP64), mixed-precision interp
    bool fft_df = false;           // forward FFTs (theta, phi, ring) in double-float
    bool ring_df = false;          // dlm2pointing's ring transforms in double-float (every mixed plan)
    double eps = 1e-7;
    long long nalm = 0;      // alm count of the arrays the calls take: m <= mmax (healpy m-major layout)
    long long nalm_tab = 0;  // size of the recursion tables: every (l, m <= lmax), same index as the alm
    int mmax = 0;            // largest m of the alm arrays (cunusht_plan_set_mmax), <= lmax

    // pointing (output) geometry
    int nring = 0;
    long long npix = 0;
    int nph_uniform = 0;  // all rings have this many pixels (0 if not uniform)
    std::vector<double> h_theta, h_phi0;
    std::vector<long long> h_nph, h_ofs;
    double *d_ring_theta = nullptr, *d_ring_phi0 = nullptr;
    long long *d_ring_nph = nullptr, *d_ring_ofs = nullptr;
    float4 *d_ring_sc = nullptr;  // (sin theta, cos theta) per ring as hi/lo FP32 pairs
    // ring pairs (theta, pi - theta) of the pointing geometry
    int gl_npairs = 0;
    double *d_gl_x = nullptr, *d_gl_sh = nullptr, *d_gl_ch = nullptr;
    int *d_gl_rn = nullptr, *d_gl_rs = nullptr;

    // doubled Clenshaw-Curtis torus and fine (oversampled) nuFFT grid
    int Nt = 0, Np = 0, ncc = 0;   // torus theta / phi lengths, CC rings = Nt/2+1
    int Ntf = 0, Npf = 0;          // fine grid lengths
    // parity split of the long transforms: 2 when a transform of more than
    // 16 x FFT_TPB points is done as two half-length transforms (even / odd
    // outputs) in a buffer of half the size, else 1
    int sp_theta = 1, sp_phi = 1, sp_ring = 1;
    int w = 0;                     // ES kernel width
    double beta = 0.0;
    int n_lo = 0, nrows = 0;       // fine rows stored: n in [n_lo, n_lo + nrows)
    int cc_npairs = 0;
    int cc_pole = -1, gl_pole = -1;  // index of the pair (theta = 0, pi) in each pair set, or -1
    int cc_pole_ring[2] = {0, 0}, gl_pole_ring[2] = {0, 0};  // its ring indices (theta = 0, theta = pi)
    double *d_cc_x = nullptr, *d_cc_sh = nullptr, *d_cc_ch = nullptr;
    int *d_cc_rn = nullptr, *d_cc_rs = nullptr;
    double *d_Dth = nullptr;  // [Nt] deconvolution * 1/Nt, index kappa mod Nt
    double *d_Dph = nullptr;  // [2L+1] deconvolution, index m+L

    // Legendre recursion tables, per spin s = 0,1,2: alpha, gamma, beta (alm layout)
    double *d_coef[3] = {nullptr, nullptr, nullptr};
    double *d_lg0[3] = {nullptr, nullptr, nullptr};  // per m: log2 start normalisation
    double *d_lfac = nullptr;                        // sqrt(l(l+1)), l = 0..L
    float2 *d_coef_df[3] = {nullptr, nullptr, nullptr};  // the same tables as (hi, lo) FP32 pairs
    bool use_tc = true;       // mixed precision: Legendre synthesis (every spin) on the tensor cores
    int *d_status = nullptr;  // device status word: bit 0 = a bounded wait of a tensor-core kernel ran out
    // tensor-core synthesis: per spin 1, 2 the first window record of each m (m = 0..lmax+1),
    // and the record buffer (alm digit planes and scales per (m, l-window), written per call)
    int *d_tc_woff[3] = {nullptr, nullptr, nullptr};
    unsigned char *d_tc_rec = nullptr;
    size_t tc_rec_bytes = 0;
    size_t tc_nrec = 0;  // window records per call (the larger of spin 1 and 2)
    int tc_rec_nb = 0;   // requests per launch the record buffer holds (1 at creation, up to 8 by reserve_batch)
    // recursion starts of the tensor-core synthesis per [grid: 0 GL, 1 CC][spin]: for every
    // (m, side, pair) the start value (hi, lo) and its exponent / 96, built at plan creation
    // (NULL: the kernel evaluates the start itself)
    float4 *d_tc_stv[2][3] = {};
    short2 *d_tc_ste[2][3] = {};

    // FFT twiddles e^{-2 pi i t / TW}
    int TW = 0;
    double2 *d_tw64 = nullptr;
    float2 *d_tw32 = nullptr;
    void *d_twdf = nullptr;      // double-float twiddles (dcplx)
    void *d_chirp_df = nullptr;  // double-float Bluestein tables (dcplx)
    void *d_bker_df = nullptr;

    // Bluestein data for the ring (phi) transform of the pointing geometry
    int Mb = 0;                  // largest Bluestein length over the ring-length classes
    double2 *d_chirp = nullptr;  // per class [N] e^{i pi q^2 / N}, concatenated
    double2 *d_bker = nullptr;   // per class [Mb] FFT_Mb(conj chirp, circular) / Mb, concatenated
    // ring-length classes (rings of equal pixel count share Bluestein tables);
    // ncls <= 1: one class, described by nph_uniform / Mb / sp_ring
    int ncls = 0;
    int ring_buf = 0;  // largest Mb / SP over the classes (shared-memory buffer of the ring transforms)
    long long nchirp = 0, nbker = 0;
    int *d_ring_cls = nullptr, *d_cls_N = nullptr, *d_cls_Mb = nullptr, *d_cls_SP = nullptr;
    long long *d_cls_coff = nullptr, *d_cls_boff = nullptr;
    // mixed-radix ring transform (ring_mr.cu) of uniform rings whose length
    // factors into radices <= 13: stages (radix, sub-transform length, offset
    // of the radix constants), output positions and e^{+2 pi i t / N} tables
    int mr_nst = 0;
    int mr_R[MR_MAXST] = {}, mr_Ls[MR_MAXST] = {}, mr_coff[MR_MAXST] = {};
    int *d_mr_pos = nullptr;
    double2 *d_mr_tw64 = nullptr;
    void *d_mr_twdf = nullptr;  // dcplx
    bool ring_bluestein = false;  // cunusht_plan_set_ring_transform(plan, 1): Bluestein for every ring length

    // workspace
    double2 *d_H = nullptr;    // Legendre columns on the CC rings  [ncols][ncc]
    void *d_F = nullptr;       // theta-pass output                 [nrows][ncols]
    void *d_U = nullptr;       // fine grid                          [nrows][Npf](x2)
    size_t u_bytes = 0;        // its size (free scratch of the adjoint Legendre stage)
    double2 *d_Hgl = nullptr;  // Legendre columns on pointing rings [ncols][nring]
    double2 *d_ring = nullptr; // Bluestein buffers (unused: in smem)
    double *d_glmap = nullptr; // spin-1 maps on pointing grid       [2][npix]
    double2 *d_alm = nullptr;  // alm staging (dtype conversion)     [2][nalm]
    double *d_vjp = nullptr;   // lensing VJP scratch: pointing + deflection gradient [4][npix]
    double *d_lfac_g = nullptr; // sqrt((l - 1)(l + 2)): deflection -> shear (spin-raising) factor [lmax + 1]
    // batched-solve workspace (cunusht_plan_reserve_batch), per request:
    int batch_cap = 0;
    double2 *d_Hb = nullptr;    // [cap][ncols][ncc]
    void *d_Fb = nullptr;       // [cap][nrows][ncols]
    void *d_Ub = nullptr;       // [cap][nrows][Npf] (x2 for spin)
    size_t ub_bytes = 0;        // its size
    double2 *d_Hglb = nullptr;  // [cap][2L+1][nring]
    double *d_glmapb = nullptr; // [cap][2][npix]
    double *d_ptgb = nullptr;   // [cap][2][npix]
    double *d_gamb = nullptr;   // [cap][npix]
    // spreading options (cunusht_plan_set_spreading): 0 warp strips, 1 bin-sorted
    int spread_method = 0;
    int spread_det = 0;          // int64 fixed-point accumulation
    int spread_nreq = 0;         // requests the option workspace holds
    long long bin_npts = 0;      // points per request the bin workspace holds
    int *d_bin = nullptr;        // [nreq][npts] bins | [nreq][npts] order | [nreq][nbins + 1] x 2 counts
    unsigned long long *d_ufix = nullptr;  // [nreq][grid scalars] fixed-point grid
    size_t ufix_bytes = 0;
    float *d_vmax = nullptr;     // [64] largest |value| per request
    size_t ws_bytes = 0;

    // per-stage CUDA-event timing (cunusht_plan_set_profiling)
    bool profiling = false;
    struct StageEvt {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<StageEvt> evt_pool;  // created once, reused
    int evt_used = 0;
    double stage_ms[CUNUSHT_NSTAGE] = {0};
    long long stage_cnt[CUNUSHT_NSTAGE] = {0};
};

// Ring-length class of a ring for the Bluestein ring transforms: per-ring
// class index and per-class length N, Bluestein length Mb, parity split SP and
// offsets of the class's chirp / kernel tables (rcls == NULL: every ring has
// N0, Mb0, SP0 and the tables start at 0).
struct RingCls {
    const int *rcls = nullptr, *N = nullptr, *Mb = nullptr, *SP = nullptr;
    const long long *coff = nullptr, *boff = nullptr;
    int N0 = 0, Mb0 = 0, SP0 = 1;
    int Hmax = 0;  // largest Mb / SP over the rings (shared buffer and twiddle-table length)
};

inline RingCls ring_cls_of(const cunusht_plan_s *P) {
    RingCls rc;
    if (P->ncls > 1) {
        rc.rcls = P->d_ring_cls;
        rc.N = P->d_cls_N;
        rc.Mb = P->d_cls_Mb;
        rc.SP = P->d_cls_SP;
        rc.coff = P->d_cls_coff;
        rc.boff = P->d_cls_boff;
        rc.Hmax = P->ring_buf;
    } else {
        rc.N0 = P->nph_uniform;
        rc.Mb0 = P->Mb;
        rc.SP0 = P->sp_ring;
        rc.Hmax = P->Mb / P->sp_ring;
    }
    return rc;
}

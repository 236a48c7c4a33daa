// Point coordinates and exponential-of-semicircle kernel values on the
// oversampled theta / phi torus, shared by the interpolation and spreading
// kernels (nufft.cu, spread_bins.cu).
#pragma once
#include "common.cuh"
#include "df.cuh"

namespace cunusht {

constexpr int NU_TPB = 256;
constexpr int MAXW = 16;

template <typename T> __device__ __forceinline__ T es_kernel(T z, T beta) {
    const T q = (T)1 - z * z;
    return q > (T)0 ? exp(beta * (sqrt(q) - (T)1)) : (T)0;
}

struct PointCoords {
    int r0;  // first fine row (relative to n_lo)
    int p0;  // first fine column (may be negative / >= Npf: wrap)
    double ft, fp;  // (n0 - t), (p0 - p): offsets of the first tap
};

__device__ __forceinline__ PointCoords point_coords(double th, double ph, int Ntf, int Npf, int n_lo,
                                                    int nrows, int w) {
    PointCoords pc;
    // non-finite or far out-of-range coordinates are clamped so every index
    // below stays inside the grid (the result for such points is garbage-in)
    if (!isfinite(th)) th = 0.0;
    if (!isfinite(ph) || fabs(ph) > 1e12) ph = 0.0;
    double t = th * ((double)Ntf / TWOPI);
    t = fmin(fmax(t, -1.0), 0.5 * Ntf + 1.0);
    double p = ph * ((double)Npf / TWOPI);
    p -= floor(p / (double)Npf) * (double)Npf;
    p = fmin(fmax(p, 0.0), (double)Npf);
    const double hw = 0.5 * w;
    const int n0 = (int)ceil(t - hw);
    const int p0 = (int)ceil(p - hw);
    pc.ft = (double)n0 - t;
    pc.fp = (double)p0 - p;
    int r0 = n0 - n_lo;
    r0 = r0 < 0 ? 0 : (r0 > nrows - w ? nrows - w : r0);  // stays in bounds for any input
    pc.r0 = r0;
    pc.p0 = p0;
    return pc;
}

// The same coordinates in double-float arithmetic, for the mixed-precision
// kernels: no FP64 instruction (GB300 issues FP64 at 1/64 of the FP32 rate,
// and point_coords' FP64 products, division, rounding and clamps made the
// interpolation kernel FP64-pipe bound).  theta and phi become double-floats
// on the integer pipe (df_from), are scaled by Ntf / 2 pi and Npf / 2 pi
// (1 / 2 pi as a double-float constant, Ntf and Npf powers of two), and the
// first taps and offsets follow as in point_coords: ceil of a normalised
// double-float is ceilf(h) unless h is an integer and l > 0, and the offsets
// n0 - t, p0 - p are formed exactly (|n0 - t.h| <= w / 2 + 1 is a multiple of
// ulp(t.h)) and renormalised.  Positions carry about 2^-47 of the grid size
// (6e-11 cells at 8192) instead of 2^-53.
struct PointCoordsDf {
    int r0;      // first fine row (relative to n_lo), clamped into the grid
    int p0;      // first fine column (may be negative / >= Npf: wrap)
    dfl ft, fp;  // (n0 - t), (p0 - p)
};

__device__ __forceinline__ float df_ceil(dfl x) {
    const float c = ceilf(x.h);
    return (c == x.h && x.l > 0.f) ? c + 1.f : c;
}

__device__ __forceinline__ PointCoordsDf point_coords_df(double th, double ph, int Ntf, int Npf, int n_lo,
                                                         int nrows, int w) {
    const dfl inv2pi{0x1.45f306p-3f, 0x1.b93910p-28f};  // 1 / 2 pi
    dfl a = df_from(th), b = df_from(ph);
    // non-finite or far out-of-range coordinates are clamped so every index
    // below stays inside the grid (the result for such points is garbage-in)
    if (!isfinite(a.h) || !isfinite(a.l)) a = dfl{0.f, 0.f};
    if (!isfinite(b.h) || !isfinite(b.l) || fabsf(b.h) > 1e12f) b = dfl{0.f, 0.f};
    dfl t = df_scale(df_mul(a, inv2pi), (float)Ntf);
    const float thi = 0.5f * (float)Ntf + 1.f;
    if (t.h < -1.f) t = dfl{-1.f, 0.f};
    else if (t.h > thi) t = dfl{thi, 0.f};
    dfl p = df_scale(df_mul(b, inv2pi), (float)Npf);
    const float k = floorf(p.h / (float)Npf);  // Npf a power of two: exact quotient
    p = df_add(p, dfl{-k * (float)Npf, 0.f});
    if (p.h < 0.f) p = df_add(p, dfl{(float)Npf, 0.f});  // p.h an integer multiple of Npf with p.l < 0
    if (p.h < 0.f) p = dfl{0.f, 0.f};
    else if (p.h > (float)Npf) p = dfl{(float)Npf, 0.f};
    const float hw = 0.5f * (float)w;
    const float n0 = df_ceil(df_add(t, dfl{-hw, 0.f}));
    const float q0 = df_ceil(df_add(p, dfl{-hw, 0.f}));
    PointCoordsDf pc;
    pc.ft = df_fast(n0 - t.h, -t.l);  // |n0 - t.h| >= w / 2 - 1 > |t.l|
    pc.fp = df_fast(q0 - p.h, -p.l);
    int r0 = (int)n0 - n_lo;
    r0 = r0 < 0 ? 0 : (r0 > nrows - w ? nrows - w : r0);  // stays in bounds for any input
    pc.r0 = r0;
    pc.p0 = (int)q0;
    return pc;
}

__device__ __forceinline__ void load_point(const double *loc, long long j, long long npts, int layout,
                                           double &th, double &ph) {
    if (layout == 0) {
        th = loc[2 * j];
        ph = loc[2 * j + 1];
    } else {
        th = loc[j];
        ph = loc[npts + j];
    }
}

// FP32 kernel value from the cancellation-free exponent
// beta (sqrt(1 - z^2) - 1) = -beta z^2 / (1 + sqrt(1 - z^2))
__device__ __forceinline__ float es_kernel_acc(float z, float beta) {
    const float q = 1.f - z * z;
    if (q <= 0.f) return 0.f;
    const float r = sqrtf(q);
    return expf(-beta * (z * z) / (1.f + r));
}

// Fixed-point accumulation of the deterministic spreading: every cell sum is
// at most npts x (the largest rotated value, below 2 vmax) < 2^(E + 61), with
// lgn = ceil(log2(npts + 1)); values are added as round(v 2^-E) in int64.
__device__ __forceinline__ int fix_exp(float vmax, int lgn) {
    int ev = 0;
    if (vmax > 0.f) frexpf(2.f * vmax, &ev);
    return ev + lgn - 61;
}
__device__ __forceinline__ long long to_fix(float v, int E) { return __float2ll_rn(ldexpf(v, -E)); }
__device__ __forceinline__ long long to_fix(double v, int E) { return __double2ll_rn(ldexp(v, -E)); }

}  // namespace cunusht

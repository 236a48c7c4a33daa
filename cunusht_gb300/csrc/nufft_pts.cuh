// Point coordinates and exponential-of-semicircle kernel values on the
// oversampled theta / phi torus, shared by the interpolation and spreading
// kernels (nufft.cu, spread_bins.cu).
#pragma once
#include "common.cuh"

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

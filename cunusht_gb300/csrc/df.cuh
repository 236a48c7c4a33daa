// Double-float ("df") arithmetic: a value is hi + lo with two FP32 numbers,
// about 48 significant bits.  Error-free transformations (Knuth TwoSum,
// FMA-based TwoProduct; Dekker 1971) on the FP32 pipe, which on GB300 runs
// about 80 times the FP64 instruction rate.  Only additions, subtractions and
// explicit fmaf are used, so FMA contraction cannot change the error terms.
#pragma once
#include <cuda_runtime.h>

namespace cunusht {

struct dfl {
    float h, l;
};

// Conversions between FP64 and double-float.  GB300 issues FP64 arithmetic
// and FP64 conversions (DADD, F2F.F64) at about 1.6 lanes per SM and clock,
// 1/80 of FP32 (measured), so the FP64 forms ((float)x, x - (double)hi,
// (double)h + (double)l: 4 and 3 FP64-pipe instructions) made the conversions
// at stage boundaries an FP64-pipe bottleneck (the interpolation kernel ran
// its FP64 pipe at 85 %).  df_from splits on the integer pipe: hi = x rounded
// to nearest even in 24 bits, lo = the exact 29-bit remainder converted by
// I2F.F32 (integer and FMA pipes); bit for bit what the FP64 form gives.
// df_to builds the exact doubles of h and l from their bits and adds them
// with one DADD (the same correctly rounded sum).  Operands outside the
// ranges handled (|x| >= 2^127 or < 2^-74, subnormal or non-finite floats)
// take the FP64 forms through a call, so the common path carries no
// predicated FP64 instructions.
static __device__ __noinline__ dfl df_from_fp64(double x) {
    dfl r;
    r.h = (float)x;
    r.l = (float)(x - (double)r.h);
    return r;
}
static __device__ __noinline__ double df_to_fp64(float h, float l) { return (double)h + (double)l; }

__device__ __forceinline__ bool df_split_i(double x, float &hi, float &lo) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned uh = (unsigned)(u >> 32);
    const unsigned sgn = uh >> 31;
    if ((u << 1) == 0) {  // +-0
        hi = __uint_as_float(sgn << 31);
        lo = 0.f;
        return true;
    }
    const int E = (int)((uh >> 20) & 0x7FF) - 1023;
    if (E < -74 || E > 126) return false;
    const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    unsigned mh = (unsigned)(m >> 29);
    const unsigned rem = (unsigned)u & 0x1FFFFFFFu;
    if (rem > 0x10000000u || (rem == 0x10000000u && (mh & 1u))) mh += 1u;
    const int r = (int)rem - ((int)(mh - (unsigned)(m >> 29)) << 29);  // m - mh 2^29, |r| <= 2^28
    // hi = mh 2^(E - 23): the implicit bit of mh (or its carry to 2^24) lands in the exponent field
    hi = __uint_as_float((sgn << 31) + ((unsigned)(E + 126) << 23) + mh);
    // lo = r 2^(E - 52), r rounded to 24 bits by the conversion, 2^(E - 52) a normal float
    lo = __int2float_rn(sgn ? -r : r) * __uint_as_float((unsigned)(E - 52 + 127) << 23);
    return true;
}

// the exact double of a normal float or zero from its bits
__device__ __forceinline__ bool df_f2d_i(float f, double &d) {
    const unsigned u = __float_as_uint(f), a = u & 0x7FFFFFFFu;
    if (a == 0u) {
        d = __hiloint2double((int)u, 0);
        return true;
    }
    if (a - 0x00800000u >= 0x7F000000u) return false;  // subnormal, inf, nan
    d = __hiloint2double((int)(((a >> 3) + 0x38000000u) | (u & 0x80000000u)), (int)(u << 29));
    return true;
}

__device__ __forceinline__ dfl df_from(double x) {
    dfl r;
    if (!df_split_i(x, r.h, r.l)) r = df_from_fp64(x);
    return r;
}

__device__ __forceinline__ double df_to(dfl a) {
    double h, l;
    if (!df_f2d_i(a.h, h) || !df_f2d_i(a.l, l)) return df_to_fp64(a.h, a.l);
    return h + l;
}

// hi/lo renormalisation, |a| >= |b| assumed (Fast2Sum)
__device__ __forceinline__ dfl df_fast(float a, float b) {
    dfl r;
    r.h = a + b;
    r.l = b - (r.h - a);
    return r;
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_fast(p, e);
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    float e = (a.h - (s - bb)) + (b.h - bb);
    e += a.l + b.l;
    return df_fast(s, e);
}

__device__ __forceinline__ dfl df_scale(dfl a, float s) {
    dfl r;
    r.h = a.h * s;
    r.l = a.l * s;
    return r;
}

// Kahan-compensated FP32 sum: value = s - c
struct kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float p) {
        const float y = p - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return df_to(dfl{s, -c}); }
};

// Compensated FP32 sum with the exact error of every addition (Knuth's
// TwoSum) collected in c: value = s + c, error O(u^2) of the addends (Ogita,
// Rump and Oishi 2005, Sum2).  Kahan's form above rounds the corrected addend
// and so keeps a relative error u per addend.
struct sum2 {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        const float bb = t - s;
        c += (s - (t - bb)) + (x - bb);
        s = t;
    }
    __device__ __forceinline__ double value() const { return df_to(dfl{s, c}); }
    __device__ __forceinline__ dfl df() const { return dfl{s, c}; }
};

// a * lam with both operands as df, rounded once to FP32
__device__ __forceinline__ float df_prod(float ah, float al, dfl lam) {
    return fmaf(ah, lam.h, fmaf(al, lam.h, ah * lam.l));
}

// a + b as an unnormalised (value, error) pair: TwoSum of the leading terms,
// the error terms added.  The same accuracy as df_add relative to the
// operands (renormalising adds none) in 8 FP32 operations and 5 dependent
// steps instead of 11 and 8; products (df_mul) accept such pairs.
__device__ __forceinline__ dfl df_add_u(dfl a, dfl b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float t = (a.h - (s - bb)) + (b.h - bb);
    return dfl{s, (a.l + b.l) + t};
}

// Three-term recursion steps.  The factor t = a x + g of a step is rebuilt
// from exact inputs every step, so it may stay an unnormalised pair (h, l):
// a product with it drops only the l * l term.  The step's result must be
// renormalised: an unnormalised low part propagates through the recursion
// like the value itself (the high parts then follow an FP32 recursion of
// their own), grows to about 2^-8 of the value over 2000 steps, and its own
// FP32 rounding enters the result (4e-6 at lmax 2047 against 1e-11).

// a * x as an unnormalised pair: 4 operations instead of 7
__device__ __forceinline__ dfl df_mul_u(dfl a, dfl x) {
    const float p = a.h * x.h;
    float e = fmaf(a.h, x.h, -p);
    e = fmaf(a.h, x.l, e);
    e = fmaf(a.l, x.h, e);
    return dfl{p, e};
}

// a * x + g as an unnormalised pair: 12 operations instead of 18 (df_mul, df_add)
__device__ __forceinline__ dfl df_fma_u(dfl a, dfl x, dfl g) { return df_add_u(df_mul_u(a, x), g); }

// t * x - b * y, renormalised (t may be unnormalised)
__device__ __forceinline__ dfl df_mul_sub(dfl t, dfl x, dfl b, dfl y) {
    const dfl p1 = df_mul_u(t, x), p2 = df_mul_u(b, y);
    const float s = p1.h - p2.h;
    const float bb = s - p1.h;
    const float err = (p1.h - (s - bb)) + (-p2.h - bb);
    return df_fast(s, err + (p1.l - p2.l));
}

// operators so that templated complex code (FFT butterflies) runs on dfl;
// additions leave unnormalised pairs (df_add_u), products renormalise
__host__ __device__ __forceinline__ dfl df_neg(dfl a) {
    dfl r;
    r.h = -a.h;
    r.l = -a.l;
    return r;
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) { return df_add_u(a, b); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return df_add_u(a, df_neg(b)); }
__device__ __forceinline__ dfl operator-(dfl a) { return df_neg(a); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) { return df_mul(a, b); }
// scale by +-1 (FFT direction) or a power of two: exact
__device__ __forceinline__ dfl operator*(int s, dfl a) { return df_scale(a, (float)s); }

// complex double-float, same 16-byte footprint as double2
struct dcplx {
    dfl x, y;
};

// host-side split of a double into hi + lo floats
inline dfl df_from_host(double x) {
    dfl r;
    r.h = (float)x;
    r.l = (float)(x - (double)r.h);
    return r;
}

// Start of the double-float Wigner-d recursion at l0 = max(m, s):
// (-1)^m 2^lg0 sh^(m+s) ch^|m-s| as an FP32-range mantissa (cur) times 2^e,
// e a non-positive multiple of 96; prev = 0.  Values below 2^-40 start with
// e < 0 and are not accumulated until REC_RESCALE_DF has brought e to 0.
__device__ __forceinline__ void rec_start_df(double lg0, int m, int s, double sh, double ch, dfl &cur,
                                             dfl &prev, int &e) {
    prev.h = prev.l = 0.f;
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
        cur.h = cur.l = 0.f;
        e = 0;
        return;
    }
    int k = 0;
    if (lg < -40.0) k = (int)ceil((-40.0 - lg) / 96.0);
    e = -96 * k;
    double v = exp2(lg + 96.0 * (double)k);
    if (m & 1) v = -v;
    cur = df_from(v);
}

#define REC_RESCALE_DF(cur, prev, e)                                                     \
    if ((e) < 0 && fabsf((cur).h) > 0x1p40f) {                                          \
        (cur) = df_scale((cur), 0x1p-96f);                                               \
        (prev) = df_scale((prev), 0x1p-96f);                                             \
        (e) += 96;                                                                       \
    }

}  // namespace cunusht

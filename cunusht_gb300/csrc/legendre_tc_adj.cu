// Adjoint Legendre transform on the tensor cores (tcgen05), mixed-precision
// path: the contraction of nusht2d1's adjoint synthesis (the reference's SHTns
// analys of map * iw, cunusht/sht/GPU_sht_transformer.py:65-73, called from
// GPU_nufft_transformer.py:265-269 and :483).
//
// For one order m and the columns X of the rings (per request four reals:
// spin s: (h+m re, h+m im, h-m' re, h-m' im) with the -m column taken from the
// mirror ring; spin 0: the even / odd sums (E re, E im, O re, O im) of a ring
// pair), the adjoint is
//     D(l, col) = sum_ring lambda_l(theta_ring) X(ring, col),
// a product over RINGS.  Both factors are split into integer digits as in the
// synthesis (legendre_tc.cu):
//     lambda = 2^El 2^-7 sum_i d_i 2^-8i,   X = 2^Ea 2^-7 sum_j t_j 2^-8j,
// |d_i|, |t_j| <= 128 (exact in bf16), El per chunk of 16 l from the bound
// sqrt((2l+1)/(4 pi)), Ea per block and column from the block's largest |X|.
// Per chunk of 16 l and lambda digit i one tensor-memory accumulator holds
//     D_i[(j, col)][l] = sum_ring t_j(ring, col) d_i(ring, l)
// (M = 128 rows (digit j, column), N = (digit i, l) = 4 x 16, K = the block's
// 256 rings in 16 K-steps of one MMA each): integer products below 2^14
// summed 256 times stay below 2^22, so the FP32 accumulation is exact.  Both
// operands are stored MN-major: the A tile (map digits, fixed for the block)
// and the B tile (lambda digits of 16 l) are written by each ring thread as
// 16-byte rows of 8 consecutive values, as in the synthesis.
//
// Block: one order m and 256 rings (spin s: 128 ring pairs, both sides; spin
// 0: 256 ring pairs, the theta side only), 8 ring warps (one ring per
// thread, double-float recursion, digit split, B rows), 1 MMA warp (16 MMAs
// of 128 x 64 x 16 per chunk) and 4 epilogue warps (one TMEM lane
// quarter each).  Two B buffers (full / empty mbarriers) and four
// tensor-memory chunk buffers (full / empty) let the three roles run apart.
// The epilogue folds the digit sums of a row, hi = v_0 (exact) and lo =
// sum_{i>0} v_i 2^-8i (FP32, rounding 2^-32 of the row), combines the four
// digit rows j of a column through shared memory, and adds the block's part of
// D(l, col) to an int64 fixed-point accumulator (exact integer atomics, unit
// 2^U(l, request) from a bound on |D|).  A finish kernel turns the sums into
// alm (the same combinations as the double-float CUDA-core kernel,
// legendre.cu k_leg_adj_*_df).  Every wait is bounded; on a timeout the block
// sets bit 0 of the plan's status word and returns.
#include "common.cuh"
#include "df.cuh"
#include "kernels.cuh"
#include "tcgen05.cuh"

namespace cunusht {

constexpr int TCA_R = 256;                      // rings per block (K)
constexpr int TCA_KC = 16;                      // l per chunk (N)
constexpr int TCA_NTB = 4;                      // tensor-memory chunk buffers
constexpr int TCA_RW = TCA_R / 32;              // ring warps
constexpr int TCA_MMA = TCA_RW;                 // the MMA warp
constexpr int TCA_EPI0 = TCA_RW + 1;            // first of the four epilogue warps
constexpr int TCA_THREADS = (TCA_RW + 5) * 32;  // 416
constexpr int TCA_A_LBO = 16 * 128;             // A: [K-core 32][M-core 16][8 K-rows][16 B]
constexpr int TCA_A_SBO = 128;
constexpr int TCA_ABYTES = (TCA_R / 8) * TCA_A_LBO;    // 64 KB
// B of a chunk: N = (lambda digit i, l) = 4 x 16, [K-core 32][N-core 8 = (i, l half)][8 K-rows][16 B],
// so that one MMA of N = 64 per K-step forms all four digit sums
constexpr int TCA_B_SBO = 128;                  // N-core stride
constexpr int TCA_B_LBO = 8 * TCA_B_SBO;        // K-core stride
constexpr int TCA_BBUF = (TCA_R / 8) * TCA_B_LBO;      // 32 KB per chunk
constexpr int TCA_XBYTES = TCA_KC * 128 * 8;           // exchange [l][row] float2
constexpr int TCA_OFF_B = TCA_ABYTES;
constexpr int TCA_OFF_X = TCA_OFF_B + 2 * TCA_BBUF;
constexpr int TCA_OFF_BAR = TCA_OFF_X + TCA_XBYTES;    // bfull[2] bempty[2] tfull[4] tempty[4]
constexpr int TCA_OFF_MISC = TCA_OFF_BAR + 12 * 8;     // tmem base, bad flag, Ea[32], maxima[8][32]
constexpr int TCA_BYTES = TCA_OFF_MISC + 16 + 32 * 4 + TCA_RW * 32 * 4;
constexpr int TCA_TCOLS = TCA_NTB * 64;
constexpr int TCA_MIN_TAIL = 32;                // fewer leftover pairs go to the CUDA-core kernel

struct TcAdjArgs {
    int spin = 0;
    const double2 *H = nullptr;
    long long hstride = 0;
    int ld = 0;
    int ntc = 0;         // ring pairs on the tensor cores
    int npairs_all = 0;  // ring pairs of the grid (fixed-point bound)
    int st_ld = 0;       // row stride of the start tables
    const double *x = nullptr, *sh = nullptr, *ch = nullptr;
    const int *rn = nullptr, *rs = nullptr;
    const float4 *stv = nullptr;
    const short2 *ste = nullptr;
    float *hm = nullptr;
    unsigned long long *acc = nullptr;
};

// Exponent U of the fixed-point unit 2^U of D(l, .) for a request whose
// columns are bounded by hm: |D| <= 2 npairs |lambda_l| 2 hm with |lambda_l|
// <= sqrt((2l+1)/(4 pi)) (spin 0: E, O <= 2 hm over npairs pairs; spin s: 2
// npairs rings of |X| <= hm), below 2^(U + 61).  FP32 and deterministic: the
// block kernels and the finish kernel evaluate it identically.
__device__ __forceinline__ int adj_unit_exp(int npairs, int l, float hm) {
    int e = 0;
    frexpf(4.f * (float)npairs * sqrtf((2.f * l + 1.f) * 0.0795774715459476679f) * hm, &e);
    return e - 61;
}

// exponent El of the chunk [lb, lhi]: 2^El > sqrt((2 lhi + 1) / (4 pi)) >= |lambda_l|
__device__ __forceinline__ int adj_chunk_el(int lhi) {
    int e = 0;
    frexpf(sqrtf((2.f * lhi + 1.f) * 0.0795774715459476679f), &e);
    return e;
}

// largest |re|, |im| of the columns [c0, c1] x rings [0, nring) of each request
// (blockIdx.y), as float bits, atomically maxed into hm[request]
__global__ void k_adj_hmax(const double2 *__restrict__ H, long long hstride, int ldH, int c0, int c1, int nring,
                           float *__restrict__ hm) {
    const double2 *Hr = H + blockIdx.y * hstride;
    const long long n = (long long)(c1 - c0 + 1) * nring;
    float mx = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long c = c0 + i / nring, ring = i % nring;
        const double2 v = Hr[c * ldH + ring];
        mx = fmaxf(mx, fmaxf(fabsf(df_from(v.x).h), fabsf(df_from(v.y).h)));  // no FP64 conversion
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    // float rounding may shave an ulp off the largest |value|: a 2^-20 margin
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int *>(hm + blockIdx.y), __float_as_int(mx * 1.000001f));
}

template <int NB, bool S0>
__global__ void __launch_bounds__(TCA_THREADS, 1)
    k_leg_adj_tc(int L, int spin, const double2 *__restrict__ H, long long hstride, int ldH,
                 const float2 *__restrict__ coef, long long nalm, const double *__restrict__ lg0, int npairs,
                 const double *__restrict__ px, const double *__restrict__ psh, const double *__restrict__ pch,
                 const int *__restrict__ prn, const int *__restrict__ prs, const float4 *__restrict__ stv,
                 const short2 *__restrict__ ste, int st_ld, const float *__restrict__ hm, int npairs_all,
                 unsigned long long *__restrict__ acc, int *status) {
    constexpr int NO = 4 * NB;       // columns per ring
    constexpr int NROW = 4 * NO;     // used rows (digit j, column) of the 128
    static_assert(NROW <= 128, "at most 8 requests per launch");
    static_assert(TCA_BYTES <= 227 * 1024, "dynamic shared memory of one block");
    static_assert(TCA_OFF_BAR % 8 == 0 && TCA_OFF_B % 1024 == 0 && TCA_BBUF % 1024 == 0, "layout alignment");
    extern __shared__ __align__(1024) unsigned char sm[];
    uint32_t *s_tm = reinterpret_cast<uint32_t *>(sm + TCA_OFF_MISC);
    volatile int *s_bad = reinterpret_cast<volatile int *>(sm + TCA_OFF_MISC + 4);
    int *s_c0 = reinterpret_cast<int *>(sm + TCA_OFF_MISC + 8);
    int *s_ea = reinterpret_cast<int *>(sm + TCA_OFF_MISC + 16);
    float *s_mx = reinterpret_cast<float *>(sm + TCA_OFF_MISC + 16 + 32 * 4);  // [ring warp][col]
    const uint32_t sbase = smem_u32(sm);
    const uint32_t bfull0 = sbase + TCA_OFF_BAR, bempty0 = bfull0 + 16, tfull0 = bfull0 + 32, tempty0 = bfull0 + 64;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m = blockIdx.y;
    const int l0 = max(m, spin);
    const long long b = almidx(L, m, m) - m;  // (l, m) at b + l

    if (warp == TCA_MMA) tmem_alloc(sbase + TCA_OFF_MISC, TCA_TCOLS);
    if (tid == 0) {
        mbar_init(bfull0, TCA_RW);
        mbar_init(bfull0 + 8, TCA_RW);
        mbar_init(bempty0, 1);
        mbar_init(bempty0 + 8, 1);
        for (int k = 0; k < TCA_NTB; ++k) {
            mbar_init(tfull0 + 8 * k, 1);
            mbar_init(tempty0 + 8 * k, 4);
        }
        *s_bad = 0;
        *s_c0 = TC_NEVER;
        mbar_init_fence();
    }
    // A rows >= NROW stay zero
    for (int i = tid; i < TCA_ABYTES / 16; i += TCA_THREADS)
        reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0u, 0u, 0u, 0u);

    // ---------------- ring data: this thread's ring and its columns
    const bool ring_thread = warp < TCA_RW;
    const int side = S0 ? 0 : tid / (TCA_R / 2);  // 0: ring theta, 1: ring pi - theta
    const int p = S0 ? blockIdx.x * TCA_R + tid : blockIdx.x * (TCA_R / 2) + (tid & (TCA_R / 2 - 1));
    const bool act = ring_thread && p < npairs;
    // this ring's recursion state at its first accumulated chunk c_me (the plan's
    // table, legendre_tc.cu k_tc_starts), or the start at l0 (c_me = 0)
    dfl cur{0.f, 0.f}, prev{0.f, 0.f};
    int e = 0, c_me = TC_NEVER;
    if (act) {
        if (stv) {
            const size_t ix = ((size_t)m * 2 + side) * st_ld + p;
            const float4 v = stv[ix];
            const short2 ec = ste[ix];
            cur = dfl{v.x, v.y};
            prev = dfl{v.z, v.w};
            e = 96 * (int)ec.x;
            c_me = ec.y;
        } else {
            const double sh = psh[p], ch = pch[p];
            if (side) rec_start_df(lg0[m], m, spin, ch, sh, cur, prev, e);
            else rec_start_df(lg0[m], m, spin, sh, ch, cur, prev, e);
            c_me = 0;
        }
    }
    // column col = 4 r + c of request r (see the file comment)
    // columns as double-floats (split on the integer pipe, sums in FP32 pairs: no
    // FP64 arithmetic)
    auto column = [&](int r, int c) -> dfl {
        const dfl z{0.f, 0.f};
        if (!act) return z;
        const double2 *Hr = H + r * hstride;
        const int n = prn[p], s = prs[p];
        if (S0) {
            // E = h(theta) + h(pi - theta), O = h(theta) - h(pi - theta); a self-paired
            // ring gives E = O = h
            const double2 hn = Hr[(long long)m * ldH + n];
            const dfl a = df_from((c & 1) ? hn.y : hn.x);
            if (s == n) return a;
            const double2 hs = Hr[(long long)m * ldH + s];
            const dfl bs = df_from((c & 1) ? hs.y : hs.x);
            return df_add(a, c < 2 ? bs : df_neg(bs));
        }
        // side 0: (h(+m) at n, h(-m) at s); side 1: (h(+m) at s, h(-m) at n); the S
        // ring of a self-paired ring carries nothing
        const int rp = side ? s : n, rm = side ? n : s;
        if (c < 2) {
            if (side && s == n) return z;
            const double2 v = Hr[(long long)(L + m) * ldH + rp];
            return df_from(c == 0 ? v.x : v.y);
        }
        if (!side && s == n) return z;
        const double2 v = Hr[(long long)(L - m) * ldH + rm];
        return df_from(c == 2 ? v.x : v.y);
    };
    const int c_warp = __reduce_min_sync(0xffffffffu, c_me);  // this warp's first chunk
    if (ring_thread) {
#pragma unroll
        for (int col = 0; col < NO; ++col) {
            float a = fabsf(column(col >> 2, col & 3).h);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
            if (lane == 0) s_mx[warp * 32 + col] = a;
        }
    }
    __syncthreads();  // s_c0 initialised
    if (ring_thread && lane == 0 && c_warp < TC_NEVER) atomicMin(s_c0, c_warp);
    if (tid < NO) {
        float cm = 0.f;
        for (int w = 0; w < TCA_RW; ++w) cm = fmaxf(cm, s_mx[w * 32 + tid]);
        int ex = 0;
        if (cm > 0.f) frexpf(cm * 1.000001f, &ex);  // 2^ex > max |X| despite the float rounding
        s_ea[tid] = min(max(ex, -80), 100);
    }
    __syncthreads();
    if (ring_thread) {
        // map digits t_j of every column into A (MN-major: row (j, col) = j NO + col, K = ring)
        unsigned char *aK = sm + (tid >> 3) * TCA_A_LBO + (tid & 7) * 16;
#pragma unroll 4
        for (int col = 0; col < NO; ++col) {
            const dfl x = column(col >> 2, col & 3);
            float t[4];
            digits4s(x.h, x.l, pow2f(7 - s_ea[col]), t);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int row = j * NO + col;
                *reinterpret_cast<unsigned short *>(aK + (row >> 3) * TCA_A_SBO + (row & 7) * 2) =
                    (unsigned short)(__float_as_uint(t[j]) >> 16);
            }
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *s_tm;
    // the block starts at the first chunk in which any of its rings accumulates
    // (earlier chunks would add zero digit products); none when no ring ever does
    const int nchk = l0 <= L ? (L - l0 + 1 + TCA_KC - 1) / TCA_KC : 0;
    const int cb = *s_c0;
    const int lstart = cb < nchk ? l0 + TCA_KC * cb : L + 1;

    if (warp == TCA_MMA) {
        // ---------------- MMA warp
        constexpr uint32_t IDESC = idesc_bf16_f32(128, 4 * TCA_KC) | (1u << 15) | (1u << 16);  // A, B MN-major
        int gc = 0;
        bool ok = true;
        for (int lb = lstart; lb <= L; lb += TCA_KC, ++gc) {
            const int buf = gc & 1, tb = gc % TCA_NTB;
            bool got = !*s_bad && mbar_wait(bfull0 + 8 * buf, (gc >> 1) & 1);
            if (got && gc >= TCA_NTB) got = mbar_wait(tempty0 + 8 * tb, ((gc / TCA_NTB) - 1) & 1);
            if (!__all_sync(0xffffffffu, got)) {
                *s_bad = 1;
                ok = false;
                break;
            }
            if (lane == 0) {
                tc_fence_after();
                const uint32_t bb = sbase + TCA_OFF_B + buf * TCA_BBUF;
#pragma unroll 4
                for (int ks = 0; ks < TCA_R / 16; ++ks)  // columns i 16 + l: the sums of lambda digit i
                    tc_mma(tbase + tb * 64, sdesc(sbase + 2 * ks * TCA_A_LBO, TCA_A_LBO, TCA_A_SBO),
                           sdesc(bb + 2 * ks * TCA_B_LBO, TCA_B_LBO, TCA_B_SBO), IDESC, ks > 0 ? 1u : 0u);
                tc_commit(bempty0 + 8 * buf);
                tc_commit(tfull0 + 8 * tb);
            }
            __syncwarp();
        }
        if (!ok && gc > 0) mbar_wait(bempty0 + 8 * ((gc - 1) & 1), ((gc - 1) >> 1) & 1);
        __syncwarp();
    } else if (warp >= TCA_EPI0) {
        // ---------------- epilogue warps: TMEM lane quarter q = warp % 4, row 32 q + lane
        const int q = warp & 3, row = 32 * q + lane, eid = tid - TCA_EPI0 * 32;
        float2 *X = reinterpret_cast<float2 *>(sm + TCA_OFF_X);
        float hmr[NB];
#pragma unroll
        for (int r = 0; r < NB; ++r) hmr[r] = hm[r];
        int gc = 0;
        for (int lb = lstart; lb <= L; lb += TCA_KC, ++gc) {
            const int tb = gc % TCA_NTB;
            const bool got = !*s_bad && mbar_wait(tfull0 + 8 * tb, (gc / TCA_NTB) & 1);
            if (bar_or_n(2, 128, !__all_sync(0xffffffffu, got))) {
                *s_bad = 1;
                break;
            }
            tc_fence_after();
            float v0[16], v1[16], v2[16], v3[16];
            const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + tb * 64;
            tmem_ld16(ta, v0);
            tmem_ld16(ta + 16, v1);
            tmem_ld16(ta + 32, v2);
            tmem_ld16(ta + 48, v3);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty0 + 8 * tb);
            if (row < NROW) {
#pragma unroll
                for (int l = 0; l < TCA_KC; ++l)
                    X[l * 128 + row] =
                        make_float2(v0[l], fmaf(fmaf(v3[l], 0x1p-8f, v2[l]), 0x1p-8f, v1[l]) * 0x1p-8f);
            }
            bar_sync_n(2, 128);
            const int El = adj_chunk_el(min(lb + TCA_KC - 1, L));
#pragma unroll
            for (int k = 0; k < (NO * TCA_KC + 127) / 128; ++k) {
                const int o = eid + 128 * k;  // output (column, l) = (o % NO, o / NO)
                const int col = o % NO, li = o / NO, l = lb + li;
                if (o < NO * TCA_KC && l <= L) {
                    const float2 x0 = X[li * 128 + col], x1 = X[li * 128 + NO + col];
                    const float2 x2 = X[li * 128 + 2 * NO + col], x3 = X[li * 128 + 3 * NO + col];
                    // D / 2^(El + Ea - 14) = x0.x + lo, x0.x an exact integer below 2^22
                    const float lo = x0.y + 0x1p-8f * ((x1.x + x1.y) + 0x1p-8f * ((x2.x + x2.y) +
                                                                                   0x1p-8f * (x3.x + x3.y)));
                    const float li_ = truncf(lo);
                    const long long n30 = ((long long)((int)x0.x + (int)li_) << 30) +
                                          (long long)__float2int_rn((lo - li_) * 0x1p30f);
                    const int r = col >> 2, c = col & 3;
                    const int sh = El + s_ea[col] - 44 - adj_unit_exp(npairs_all, l, hmr[r]);
                    const long long nv = sh >= 0 ? (n30 << sh) : (sh > -63 ? (n30 >> (-sh)) : (n30 < 0 ? -1 : 0));
                    atomicAdd(acc + ((long long)r * nalm + b + l) * 4 + c, (unsigned long long)nv);
                }
            }
            bar_sync_n(2, 128);  // X is rewritten by the next chunk
        }
    } else {
        // ---------------- ring warps
        const double x = act ? px[p] : 0.0;
        const dfl xd = df_from(side ? -x : x);
        const float2 *al = coef, *ga = coef + nalm, *be = coef + 2 * nalm;
        const uint32_t boff = (tid >> 3) * TCA_B_LBO + (tid & 7) * 16;
        int gc = 0, bad = 0;
        for (int lb = lstart; lb <= L; lb += TCA_KC, ++gc) {
            const int buf = gc & 1;
            if (gc >= 2) bad |= !mbar_wait(bempty0 + 8 * buf, ((gc - 2) >> 1) & 1);
            bad = __any_sync(0xffffffffu, bad | *s_bad);
            if (bad) break;
            const float lsc = pow2f(7 - adj_chunk_el(min(lb + TCA_KC - 1, L)));
            unsigned char *sB = sm + TCA_OFF_B + buf * TCA_BBUF + boff;
            // before its first chunk a ring holds its table state and writes zero digits
            const bool live = (lb - l0) / TCA_KC >= c_me;
            if (live) {
                // two halves of 8 l; the exponent check runs once per half (a step grows the
                // mantissa by less than 2^8.5: eight steps from below 2^40 stay inside FP32)
#pragma unroll
                for (int lh = 0; lh < 2; ++lh) {
                    uint32_t pk[4][4];
                    const float scg = (act && e == 0) ? lsc : 0.f;
#pragma unroll
                    for (int j2 = 0; j2 < 4; ++j2) {
                        float d0[4], d1[4];
                        auto step = [&](int l, float(&d)[4]) {
                            digits4s(cur.h, cur.l, l <= L ? scg : 0.f, d);
                            float2 a2 = make_float2(0.f, 0.f), g2 = a2, b2 = a2;
                            if (l < L) {
                                a2 = __ldg(al + b + l);
                                g2 = __ldg(ga + b + l);
                                b2 = __ldg(be + b + l);
                            }
                            const dfl t = df_fma_u(dfl{a2.x, a2.y}, xd, dfl{g2.x, g2.y});
                            const dfl nxt = df_mul_sub(t, cur, dfl{b2.x, b2.y}, prev);
                            prev = cur;
                            cur = nxt;
                        };
                        const int l = lb + 8 * lh + 2 * j2;
                        step(l, d0);
                        step(l + 1, d1);
#pragma unroll
                        for (int k = 0; k < 4; ++k) pk[k][j2] = pack_bf16(d0[k], d1[k]);
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)  // digit k of lambda -> N-core (k, lh)
                        *reinterpret_cast<uint4 *>(sB + (2 * k + lh) * TCA_B_SBO) =
                            make_uint4(pk[k][0], pk[k][1], pk[k][2], pk[k][3]);
                    REC_RESCALE_DF(cur, prev, e);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    *reinterpret_cast<uint4 *>(sB + k * TCA_B_SBO) = make_uint4(0u, 0u, 0u, 0u);
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(bfull0 + 8 * buf);
        }
        if (bad) *s_bad = 1;
    }
    tc_fence_before();
    __syncthreads();
    if (tid == 0 && *s_bad && status) atomicOr(status, 1);
    if (warp == TCA_MMA) {
        tc_fence_after();
        tmem_dealloc(tbase, TCA_TCOLS);
    }
}

// v 2^e2 as a double, on the integer pipe (GB300 runs integer-to-FP64
// conversions at the FP64 rate): the leading-zero count normalises |v|, the
// top 53 bits round to nearest even, and e2 goes into the exponent field.
// Requires |v| < 2^63 and a result in the normal range.
__device__ __forceinline__ double i64_ldexp(long long v, int e2) {
    if (v == 0) return 0.0;
    const unsigned long long sgn = v < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long u = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll((long long)u);
    const unsigned long long m = u << lz;  // leading one at bit 63
    unsigned long long mant = m >> 11;      // 53 bits, leading one at bit 52
    const unsigned long long rem = m & 0x7FFull;
    mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
    int ex = 63 - lz + e2;
    if (mant >> 53) {  // rounding carried into bit 53
        mant >>= 1;
        ++ex;
    }
    return __longlong_as_double((long long)(sgn | ((unsigned long long)(ex + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// D(l, col) from the fixed-point sums -> alm, the combinations of the
// double-float kernels (legendre.cu k_leg_adj_s0_df / k_leg_adj_spin_df):
// spin 0: a = f (E or O by the parity of l + m); spin s: P = (D0, D1),
// Q = sgn (D2, -D3) for even l + m and sgn (-D2, D3) for odd (sgn = -1 for
// odd s), G = -f (P + Q) / 2 and C = f (-(P im - Q im), P re - Q re) / 2.
// The sums and differences are exact in int64 (|D| < 2^61), so each output
// takes one conversion (i64_ldexp) and, with a per-l factor f, one product.
// Every alm of the orders m <= mmax is written (=); the pole pair and the
// leftover ring pairs are added afterwards.
__global__ void k_leg_adj_tc_finish(int L, int spin, int ncomp, const unsigned long long *__restrict__ acc,
                                    long long nalm_tab, const float *__restrict__ hm, int npairs_all,
                                    const double *__restrict__ lfac, double *__restrict__ G, double *__restrict__ C,
                                    long long astride) {
    const int m = blockIdx.y, r = blockIdx.z;
    const int l = m + blockIdx.x * blockDim.x + threadIdx.x;
    if (l > L) return;
    const long long ix = almidx(L, m, m) - m + l;
    const unsigned long long *a = acc + ((long long)r * nalm_tab + ix) * 4;
    const long long d0 = (long long)a[0], d1 = (long long)a[1], d2 = (long long)a[2], d3 = (long long)a[3];
    const int U = adj_unit_exp(npairs_all, l, hm[r]);
    const bool odd = (l + m) & 1;
    double *Gr = G + 2 * r * astride;
    double f0, f1;
    if (spin == 0) {
        f0 = i64_ldexp(odd ? d2 : d0, U);
        f1 = i64_ldexp(odd ? d3 : d1, U);
    } else {
        const bool neg = (spin & 1) != 0;
        long long qr = odd ? -d2 : d2, qi = odd ? d3 : -d3;
        if (neg) qr = -qr, qi = -qi;
        f0 = i64_ldexp(-(d0 + qr), U - 1);
        f1 = i64_ldexp(-(d1 + qi), U - 1);
        if (ncomp > 1) {
            double c0 = i64_ldexp(-(d1 - qi), U - 1), c1 = i64_ldexp(d0 - qr, U - 1);
            if (lfac) c0 *= lfac[l], c1 *= lfac[l];
            double *Cr = C + 2 * r * astride;
            Cr[2 * ix] = c0;
            Cr[2 * ix + 1] = c1;
        }
    }
    if (lfac) f0 *= lfac[l], f1 *= lfac[l];
    Gr[2 * ix] = f0;
    Gr[2 * ix + 1] = f1;
}

// The pole pair of a spin-0 adjoint: lambda_lm(0) = delta_m0 sqrt((2l+1)/(4 pi))
// and lambda_lm(pi) = (-1)^l lambda_lm(0), so only m = 0 receives
// f sqrt((2l+1)/(4 pi)) (h(0, theta=0) + (-1)^l h(0, theta=pi)); block row r =
// request r, added to the finished alm.
__global__ void k_pole_pair_adj_s0(int L, const double2 *__restrict__ H, long long hstride, const double *__restrict__ lfac,
                                   int rn, int rs, double *__restrict__ G, long long astride) {
    const int r = blockIdx.y;
    const double2 hn = H[r * hstride + rn], hs = H[r * hstride + rs];
    double *Gr = G + 2 * r * astride;
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l <= L; l += gridDim.x * blockDim.x) {
        const double lam = sqrt((2.0 * l + 1.0) / (4.0 * PI)) * (lfac ? lfac[l] : 1.0);
        const double sg = (l & 1) ? -1.0 : 1.0;
        Gr[2 * l] += lam * (hn.x + sg * hs.x);  // (l, 0) at index l, one writer per l
        Gr[2 * l + 1] += lam * (hn.y + sg * hs.y);
    }
}

template <int NB, bool S0>
static int launch_adj_tc_nb(const cunusht_plan_s *P, const TcAdjArgs &A, int r0, cudaStream_t st) {
    CU_TRY(cudaFuncSetAttribute(k_leg_adj_tc<NB, S0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TCA_BYTES));
    constexpr int PER = S0 ? TCA_R : TCA_R / 2;
    const dim3 grid((A.ntc + PER - 1) / PER, P->mmax + 1);
    k_leg_adj_tc<NB, S0><<<grid, TCA_THREADS, TCA_BYTES, st>>>(
        P->lmax, A.spin, A.H + r0 * A.hstride, A.hstride, A.ld, P->d_coef_df[A.spin], P->nalm_tab, P->d_lg0[A.spin],
        A.ntc, A.x, A.sh, A.ch, A.rn, A.rs, A.stv, A.ste, A.st_ld, A.hm + r0, A.npairs_all,
        A.acc + (long long)r0 * P->nalm_tab * 4, P->d_status);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

size_t adj_tc_scratch_bytes(const cunusht_plan_s *P, int nreq) {
    return 256 + (size_t)nreq * P->nalm_tab * 4 * sizeof(unsigned long long);
}

// Tensor-core adjoint of nreq requests (columns at H + r hstride; alm at G +
// r astride, C + r astride): fixed-point sums in scratch (adj_tc_scratch_bytes),
// launches of up to 8 requests sharing the recursion, then the finish kernel,
// the pole pair and the leftover pairs (double-float CUDA cores).
int leg_adjoint_tc(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                   int ld, int npairs, const double *x, const double *sh, const double *ch, const int *rn,
                   const int *rs, int pole, int pole_rn, int pole_rs, const float4 *stv, const short2 *ste,
                   const double *lf, double2 *G, double2 *C, long long astride, void *scratch, cudaStream_t st) {
    const int L = P->lmax;
    TcAdjArgs A;
    A.spin = spin;
    A.H = H;
    A.hstride = hstride;
    A.ld = ld;
    A.hm = reinterpret_cast<float *>(scratch);
    A.acc = reinterpret_cast<unsigned long long *>(static_cast<char *>(scratch) + 256);
    A.npairs_all = npairs;
    A.st_ld = npairs;
    CU_TRY(cudaMemsetAsync(scratch, 0, adj_tc_scratch_bytes(P, nreq), st));
    {
        const int c0 = spin ? L - P->mmax : 0, c1 = spin ? L + P->mmax : P->mmax;
        k_adj_hmax<<<dim3(256, nreq), 256, 0, st>>>(H, hstride, ld, c0, c1, ld, A.hm);
        CU_LAUNCH_CHECK();
    }
    const bool has_pole = pole == 0 && npairs > 1;
    if (has_pole) {
        ++x, ++sh, ++ch, ++rn, ++rs;
        if (stv) ++stv, ++ste;
        --npairs;
    }
    const int per = spin == 0 ? TCA_R : TCA_R / 2, tail = npairs % per;
    A.ntc = (npairs > per && tail < TCA_MIN_TAIL) ? npairs - tail : npairs;
    A.x = x, A.sh = sh, A.ch = ch, A.rn = rn, A.rs = rs, A.stv = stv, A.ste = ste;
    for (int r0 = 0; r0 < nreq;) {
        const int left = nreq - r0;
        const int nb = left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        if (spin == 0) {
            if (nb == 8) RC_TRY((launch_adj_tc_nb<8, true>(P, A, r0, st)));
            else if (nb == 4) RC_TRY((launch_adj_tc_nb<4, true>(P, A, r0, st)));
            else if (nb == 2) RC_TRY((launch_adj_tc_nb<2, true>(P, A, r0, st)));
            else RC_TRY((launch_adj_tc_nb<1, true>(P, A, r0, st)));
        } else {
            if (nb == 8) RC_TRY((launch_adj_tc_nb<8, false>(P, A, r0, st)));
            else if (nb == 4) RC_TRY((launch_adj_tc_nb<4, false>(P, A, r0, st)));
            else if (nb == 2) RC_TRY((launch_adj_tc_nb<2, false>(P, A, r0, st)));
            else RC_TRY((launch_adj_tc_nb<1, false>(P, A, r0, st)));
        }
        r0 += nb;
    }
    k_leg_adj_tc_finish<<<dim3((L + 1 + 255) / 256, P->mmax + 1, nreq), 256, 0, st>>>(
        L, spin, ncomp, A.acc, P->nalm_tab, A.hm, A.npairs_all, lf, (double *)G,
        (spin > 0 && ncomp > 1) ? (double *)C : nullptr, astride);
    CU_LAUNCH_CHECK();
    if (has_pole) {
        if (spin == 0) {
            k_pole_pair_adj_s0<<<dim3((L + 256) / 256, nreq), 256, 0, st>>>(L, H, hstride, lf, pole_rn, pole_rs,
                                                                            (double *)G, astride);
            CU_LAUNCH_CHECK();
        } else {
            RC_TRY(leg_adj_pole_pair_spin(P, nreq, spin, ncomp, H, hstride, ld, lf, pole_rn, pole_rs, G, C, astride,
                                          st));
        }
    }
    if (A.ntc < npairs)
        RC_TRY(leg_adj_df_pairs(P, nreq, spin, ncomp, H, hstride, ld, npairs - A.ntc, x + A.ntc, sh + A.ntc,
                                ch + A.ntc, rn + A.ntc, rs + A.ntc, lf, G, C, astride, st));
    return CUNUSHT_OK;
}

}  // namespace cunusht

// Legendre synthesis on the tensor cores (tcgen05), mixed-precision path.
//
// For one order m the synthesis is a product of two matrices,
//     h(ring, col) = sum_l lambda_l(theta_ring) a(l, col),
// rings x l times l x cols, with cols = (A re, A im, B re, B im) per request
// (the spin-s combinations of the reference's SHTns synthesis,
// cunusht/sht/GPU_sht_transformer.py:56-62 and :88-97; A = G - iC pairs with
// +s at theta, B with -s, whose values at pi - theta are the +s functions at
// theta).  The recursion in l stays on the CUDA cores in double-float
// (legendre.cu); the contraction goes to the tensor cores exactly:
//
//   lambda = 2^El 2^-7 (d0 + d1 2^-8 + d2 2^-16 + d3 2^-24),  |d_i| <= 128
//   a      = 2^Ea 2^-7 (t0 + t1 2^-8 + t2 2^-16 + t3 2^-24),  |t_j| <= 128
//
// with integer digits (exact in bf16), El fixed per l-window from the bound
// |lambda_l| <= sqrt((2l+1)/(4 pi)) and Ea per window and column from the
// largest |a|.  Digit products of equal weight g = i + j are summed by one
// bf16 MMA (the K axis holds (digit i, l), the N axis (weight g, column) with
// B'[(g, col)][(i, l)] = t_{g-i}(l, col)).  Weights g = 0..4 are kept (13 of
// the 16 digit pairs: the low digits span the whole +-128, so dropping g = 4
// would cost 2^-27 of a typical product; g >= 5 is below 2^-40).  The
// products are integers below 2^14 and a 128-l window sums at most 4 x 128 of
// them per weight, so the FP32 accumulation in tensor memory is exact.  Per
// window the weights 4..1 of each output are folded by Horner in FP32 and,
// with weight 0, scaled by powers of two and added to compensated FP32
// accumulators that keep the exact error of every addition (sum2).  The
// truncation of the digit strings (2^-32 of the bounds) dominates the error:
// the products are more accurate than the double-float CUDA-core kernels,
// which round every product to FP32.
//
// Block: one order m and 256 ring pairs as four 128-row MMA tiles (544
// threads) for launches of up to 4 requests, 192 ring pairs as three tiles
// (416 threads) for 8 requests, whose 160 tensor-memory columns per tile fit
// 512 three times.  Each ring thread holds one ring (the first half of them the
// rings theta, the second half pi - theta); per chunk of 16 l it writes its
// four digit rows (two 16-byte K-cores per digit) into the A tile, and the
// ring threads together write the B' digits.  The last warp issues tiles x 4
// K-steps of M=128, N=5 x 4 NB (rounded up to 16), K=16 MMAs.  Two A/B'
// buffers alternate; an mbarrier per buffer (tcgen05.commit) tells when the
// MMAs reading it are done.  Every wait is bounded: on a timeout the block
// records it in the plan's status word, waits once more (bounded) for its
// MMAs, frees its tensor memory and returns.  Recursion starts come from the
// plan's table (k_tc_starts) when it has one.
#include "common.cuh"
#include "df.cuh"
#include "kernels.cuh"
#include "tcgen05.cuh"

#include <algorithm>
#include <type_traits>
#include <vector>

namespace cunusht {

// ---------------------------------------------------------------- self test
// A 128 x n x 32 product of integer matrices (|entries| <= 128) accumulated
// reps times (reps <= 16: sums below 2^24) through the same descriptors and
// tensor-memory path as the Legendre kernel; writes the largest
// |D - reps A B| to out[0] and 1 to out[1] on a barrier timeout.  mode 0:
// entries of both signs; 1: entries in [64, 128] (sums near 2^23); 2: one
// product of 2^14 per output among products of at most 4 (small addends
// against a large partial sum).
__device__ __forceinline__ int st_a(int r, int k, int mode) {
    if (mode == 1) return 64 + ((r * 37 + k * 11 + 5) * 73) % 65;
    if (mode == 2) return k == 0 ? 128 : (r + k) % 5 - 2;
    return ((r * 37 + k * 11 + 5) * 73) % 257 - 128;
}
__device__ __forceinline__ int st_b(int n, int k, int mode) {
    if (mode == 1) return 64 + ((n * 53 + k * 29 + 3) * 97) % 65;
    if (mode == 2) return k == 0 ? 128 : (n + 2 * k) % 5 - 2;
    return ((n * 53 + k * 29 + 3) * 97) % 257 - 128;
}

// mode 3 issues no product and gives the completion wait a limit of 64 polls:
// nothing arrives on the barrier, the wait runs out and the kernel takes its
// timeout path (status out[1] = 1, tensor memory released, no read-back) with
// no copy or MMA in flight.
__global__ void __launch_bounds__(128) k_tc_selftest(int nn, int reps, int mode, float *out) {
    __shared__ __align__(1024) unsigned char sA[128 * 64];
    __shared__ __align__(1024) unsigned char sB[64 * 64];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(smem_u32(&tmem_base), 64);
    if (tid == 0) {
        mbar_init(smem_u32(&bar), 1);
        mbar_init_fence();
    }
    // row r: four K-cores (8 bf16 each) at (r>>3)*512 + c*128 + (r&7)*16
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t q[4];
#pragma unroll
        for (int h = 0; h < 4; ++h)
            q[h] = pack_bf16((float)st_a(tid, 8 * c + 2 * h, mode), (float)st_a(tid, 8 * c + 2 * h + 1, mode));
        *reinterpret_cast<uint4 *>(sA + (tid >> 3) * 512 + c * 128 + (tid & 7) * 16) = make_uint4(q[0], q[1], q[2], q[3]);
        if (tid < nn) {
#pragma unroll
            for (int h = 0; h < 4; ++h)
                q[h] = pack_bf16((float)st_b(tid, 8 * c + 2 * h, mode), (float)st_b(tid, 8 * c + 2 * h + 1, mode));
            *reinterpret_cast<uint4 *>(sB + (tid >> 3) * 512 + c * 128 + (tid & 7) * 16) =
                make_uint4(q[0], q[1], q[2], q[3]);
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = tmem_base;
    if (tid == 0 && mode != 3) {
        const uint32_t id = idesc_bf16_f32(128, nn);
        for (int rep = 0; rep < reps; ++rep)
#pragma unroll
            for (int k = 0; k < 2; ++k)
                tc_mma(tb, sdesc(smem_u32(sA) + k * 256, 128, 512), sdesc(smem_u32(sB) + k * 256, 128, 512), id,
                       (rep > 0 || k > 0) ? 1u : 0u);
        tc_commit(smem_u32(&bar));
    }
    const bool ok = mbar_wait(smem_u32(&bar), 0, mode == 3 ? 64 : MBAR_SPIN_LIMIT);
    const int bad = __syncthreads_or(!ok);
    tc_fence_after();
    float err = 0.f;
    if (!bad) {
        for (int c0 = 0; c0 < nn; c0 += 16) {
            float v[16];
            tmem_ld16(tb + ((uint32_t)(warp * 32) << 16) + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                int ref = 0;
                for (int k = 0; k < 32; ++k) ref += st_a(tid, k, mode) * st_b(c0 + i, k, mode);
                err = fmaxf(err, fabsf(v[i] - (float)(reps * ref)));  // |reps ref| < 2^24: exact in FP32
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tb, 64);
    }
    atomicMax(reinterpret_cast<int *>(out), __float_as_int(err));  // err >= 0: int order = float order
    if (bad && tid == 0) out[1] = 1.f;
}

// Operands stored MN-major (the transpose bits 15 / 16 of the instruction
// descriptor): no-swizzle core matrices of 8 K-rows x 16 bytes (8 elements
// along M or N), SBO = byte distance between core matrices adjacent along
// M / N, LBO = along K.  A (128 x 32) and B (nn x 32) hold the integer
// entries of k_tc_selftest; amn / bmn choose the layout of each operand
// (K-major as in k_tc_selftest otherwise).  Both buffers are sized so that a
// reading of the descriptor with LBO and SBO exchanged still stays inside
// them (A 48 KB, B 16 KB of dynamic shared memory).
constexpr int TST_ABYTES = 48 * 1024, TST_BBYTES = 16 * 1024;
__global__ void __launch_bounds__(128) k_tc_selftest_mn(int nn, int amn, int bmn, float *out) {
    extern __shared__ __align__(1024) unsigned char dsm[];
    unsigned char *sA = dsm, *sB = dsm + TST_ABYTES;
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(smem_u32(&tmem_base), 64);
    if (tid == 0) {
        mbar_init(smem_u32(&bar), 1);
        mbar_init_fence();
    }
    for (int i = tid; i < (TST_ABYTES + TST_BBYTES) / 16; i += 128)
        reinterpret_cast<uint4 *>(dsm)[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    // element (r, k) of A and (n, k) of B, one 2-byte store each
    const int a_lbo = amn ? 16 * 128 : 128, a_sbo = amn ? 128 : 512;
    const int b_lbo = bmn ? (nn / 8) * 128 : 128, b_sbo = bmn ? 128 : 512;
    for (int k = 0; k < 32; ++k) {
        const float av = (float)st_a(tid, k, 0);
        const int ao = amn ? (k >> 3) * a_lbo + (tid >> 3) * a_sbo + (k & 7) * 16 + (tid & 7) * 2
                           : (tid >> 3) * a_sbo + (k >> 3) * a_lbo + (tid & 7) * 16 + (k & 7) * 2;
        *reinterpret_cast<unsigned short *>(sA + ao) = (unsigned short)(__float_as_uint(av) >> 16);
        if (tid < nn) {
            const float bv = (float)st_b(tid, k, 0);
            const int bo = bmn ? (k >> 3) * b_lbo + (tid >> 3) * b_sbo + (k & 7) * 16 + (tid & 7) * 2
                               : (tid >> 3) * b_sbo + (k >> 3) * b_lbo + (tid & 7) * 16 + (k & 7) * 2;
            *reinterpret_cast<unsigned short *>(sB + bo) = (unsigned short)(__float_as_uint(bv) >> 16);
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = tmem_base;
    if (tid == 0) {
        const uint32_t id = idesc_bf16_f32(128, nn) | (amn ? (1u << 15) : 0u) | (bmn ? (1u << 16) : 0u);
#pragma unroll
        for (int k = 0; k < 2; ++k)  // K-step k: K-cores 2k, 2k + 1
            tc_mma(tb, sdesc(smem_u32(sA) + 2 * k * a_lbo, a_lbo, a_sbo),
                   sdesc(smem_u32(sB) + 2 * k * b_lbo, b_lbo, b_sbo), id, k > 0 ? 1u : 0u);
        tc_commit(smem_u32(&bar));
    }
    const bool ok = mbar_wait(smem_u32(&bar), 0);
    const int bad = __syncthreads_or(!ok);
    tc_fence_after();
    float err = 0.f;
    if (!bad) {
        for (int c0 = 0; c0 < nn; c0 += 16) {
            float v[16];
            tmem_ld16(tb + ((uint32_t)(warp * 32) << 16) + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                int ref = 0;
                for (int k = 0; k < 32; ++k) ref += st_a(tid, k, 0) * st_b(c0 + i, k, 0);
                err = fmaxf(err, fabsf(v[i] - (float)ref));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tb, 64);
    }
    atomicMax(reinterpret_cast<int *>(out), __float_as_int(err));
    if (bad && tid == 0) out[1] = 1.f;
}

int tc_selftest(int nn, int reps, int mode, double *maxerr, int *timeout) {
    if ((nn != 16 && nn != 32 && nn != 64) || reps < 1 || reps > 16 || mode < 0 || mode > 6) return CUNUSHT_ERR_ARG;
    float *d = nullptr;
    CU_TRY(cudaMalloc(&d, 2 * sizeof(float)));
    CU_TRY(cudaMemset(d, 0, 2 * sizeof(float)));
    if (mode >= 4) {
        // 4: A and B MN-major; 5: A MN-major, B K-major; 6: A K-major, B MN-major
        const int amn = mode != 6, bmn = mode != 5;
        const int bytes = TST_ABYTES + TST_BBYTES;
        cudaError_t ea = cudaFuncSetAttribute(k_tc_selftest_mn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (ea == cudaSuccess) k_tc_selftest_mn<<<1, 128, bytes>>>(nn, amn, bmn, d);
        else cudaFree(d), d = nullptr;
        CU_TRY(ea);
    } else {
        k_tc_selftest<<<1, 128>>>(nn, reps, mode, d);
    }
    cudaError_t e = cudaGetLastError();
    float h[2] = {0.f, 0.f};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    CU_TRY(e);
    *maxerr = h[0];
    *timeout = h[1] != 0.f;
    return CUNUSHT_OK;
}

// ---------------------------------------------------------------- spin-s synthesis
constexpr int TCL_W = 128;     // l window accumulated in tensor memory
constexpr int TCL_KC = 16;     // l per chunk: K = 4 digits x 16 l = 4 MMA K-steps
constexpr int TCL_TILE = 128 * 128;       // A tile: 128 rows x 8 K-cores x 16 bytes
constexpr int TCL_SBO = 1024;             // 8-row group stride (8 rows x 8 K-cores x 16 bytes)
constexpr int TCL_TPS = TCL_W + 8;        // digit-plane row stride in elements (272 bytes: 16-byte aligned, fewer bank conflicts)
constexpr int TCL_MIN_TAIL = 32;          // fewer leftover ring pairs than this go to the CUDA-core kernel

// Launches of NB <= 4 requests run blocks of four 128-ring tiles (256 ring
// pairs); NB = 8 needs 5 x 32 = 160 tensor-memory columns per tile and runs
// blocks of three tiles (192 ring pairs, 480 of the 512 columns; a tile may
// hold rings of both sides).
template <int NB>
struct TclLayout {
    static constexpr int NT = NB >= 8 ? 3 : 4;           // 128-row MMA tiles per block
    static constexpr int T = 128 * NT;                   // ring threads (one ring each)
    static constexpr int BLOCK = T + 32;                 // + the MMA warp
    static constexpr int ABUF = NT * TCL_TILE;           // A buffer: NT tiles
    static constexpr int NO = 4 * NB;                    // outputs per ring
    static constexpr int NG = 5;                         // digit-product weights g = 0..4
    static constexpr int NN = (NG * NO + 15) / 16 * 16;  // MMA N: weights x outputs, padded to 16
    static constexpr int NCOLS = NT * NN <= 32    ? 32
                                 : NT * NN <= 64  ? 64
                                 : NT * NN <= 128 ? 128
                                 : NT * NN <= 256 ? 256
                                                  : 512;
    // window record (written by k_tc_records, one per (m, l-window)):
    static constexpr int RSC = 4 * NO * TCL_TPS * 2;        // bf16 digit planes [4][NO][TPS], then
    static constexpr int RLS = RSC + NG * NO * 4;           // float epilogue scales [NG][NO], then
    static constexpr int RCO = (RLS + 4 + 15) / 16 * 16;    // float lambda digit scale, then
    static constexpr int RBE = RCO + (TCL_W + 1) * 16;      // float4 (alpha, gamma) [W + 1] and
    static constexpr int RSZ = (RBE + (TCL_W + 1) * 8 + 15) / 16 * 16;  // float2 beta [W + 1] (zero past the window)
    static constexpr int BBUF = NN * 128;                // B' buffer: NN rows x 8 K-cores x 16 bytes
    static constexpr int OFF_B = 2 * ABUF;
    static constexpr int OFF_R = OFF_B + 2 * BBUF;       // two window records (current, next)
    static constexpr int OFF_BAR = OFF_R + 2 * RSZ;      // full[2], empty[2], record[2]
    static constexpr int OFF_TM = OFF_BAR + 48;          // tensor-memory base, give-up flag
    static constexpr int BYTES = OFF_TM + 16;
};

// B' digit pairs (g, i) with 0 <= g - i <= 3, g < 5, in order:
// (0,0) (1,0) (1,1) (2,0) (2,1) (2,2) (3,0) .. (3,3) (4,1) (4,2) (4,3)
__device__ __forceinline__ void tcl_pair(int pr, int &g, int &di) {
    if (pr == 0) g = 0, di = 0;
    else if (pr < 3) g = 1, di = pr - 1;
    else if (pr < 6) g = 2, di = pr - 3;
    else if (pr < 10) g = 3, di = pr - 6;
    else g = 4, di = pr - 9;
}

// Window records: one block of TCL_W threads per (l-window k, order m), thread
// i for l = wb + i.  The NO alm combinations of the NB requests (A = G - iC
// pairs with +s, B with -s, times the per-l factor) as double-float, the
// column exponents Ea (2^Ea > max over the window), their digit planes, the
// epilogue scales 2^(El + Ea - 14 - 8g) and the lambda digit scale
// 2^(7 - El).  All FP64 work of the tensor-core synthesis happens here, in
// parallel over every window, rather than between the ring warps' chunks.
//
// Spin 0 (S0): one recursion per ring pair at theta serves both rings, since
// lambda_lm(pi - theta) = (-1)^(l+m) lambda_lm(theta); the four columns of a
// request are the alm split by the parity of l + m, (E re, E im, O re, O im),
// and the rings receive E + O (theta) and E - O (pi - theta).
template <int NB, bool S0>
__global__ void __launch_bounds__(TCL_W)
    k_tc_records(int L, int spin, const double2 *__restrict__ G, const double2 *__restrict__ C, long long astride,
                 const double *__restrict__ lfac, const float2 *__restrict__ coef, long long nalm,
                 const int *__restrict__ woff, unsigned char *__restrict__ rec) {
    using LY = TclLayout<NB>;
    constexpr int NO = LY::NO, NG = LY::NG;
    __shared__ float s_mx[TCL_W / 32][NO];
    __shared__ int s_ea[NO];
    const int m = blockIdx.y, k = blockIdx.x;
    if (k >= woff[m + 1] - woff[m]) return;
    const int wb = max(m, spin) + k * TCL_W, cnt = min(TCL_W, L - wb + 1);
    unsigned char *R = rec + (size_t)(woff[m] + k) * LY::RSZ;
    const int i = threadIdx.x, lane = i & 31, warp = i >> 5;
    {
        // recursion coefficients (double-float) of the window, zero past its end
        float4 *ag = reinterpret_cast<float4 *>(R + LY::RCO);
        float2 *bt = reinterpret_cast<float2 *>(R + LY::RBE);
        const long long b = almidx(L, m, m) - m;
        for (int j = i; j < TCL_W + 1; j += TCL_W) {
            float4 a4 = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 b2 = make_float2(0.f, 0.f);
            if (j < cnt) {
                const float2 a2 = coef[b + wb + j], g2 = coef[nalm + b + wb + j];
                a4 = make_float4(a2.x, a2.y, g2.x, g2.y);
                b2 = coef[2 * nalm + b + wb + j];
            }
            ag[j] = a4;
            bt[j] = b2;
        }
    }
    dfl v[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) v[o] = dfl{0.f, 0.f};
    if (i < cnt) {
        // the combinations in double-float from the split inputs: no FP64
        // arithmetic (GB300 issues FP64 at 1/64 of the FP32 rate); 2^-47 of
        // each value, far below the 2^-32 digit truncation
        const int l = wb + i;
        const long long ix = almidx(L, m, m) - m + l;
        const dfl f = lfac ? df_from(lfac[l]) : dfl{1.f, 0.f};
        const dfl par = ((l + m) & 1) ? df_neg(f) : f;
        const dfl z{0.f, 0.f};
#pragma unroll
        for (int r = 0; r < NB; ++r) {
            const double2 g = G[r * astride + ix];
            const dfl gx = df_from(g.x), gy = df_from(g.y);
            if (S0) {
                const bool odd = (l + m) & 1;
                const dfl ex = df_mul(f, gx), ey = df_mul(f, gy);
                v[4 * r + 0] = odd ? z : ex;
                v[4 * r + 1] = odd ? z : ey;
                v[4 * r + 2] = odd ? ex : z;
                v[4 * r + 3] = odd ? ey : z;
                continue;
            }
            const double2 c = C ? C[r * astride + ix] : make_double2(0.0, 0.0);
            const dfl cx = df_from(c.x), cy = df_from(c.y);
            v[4 * r + 0] = df_mul(f, df_add(gx, df_neg(cy)));
            v[4 * r + 1] = df_mul(f, df_add(gy, cx));
            v[4 * r + 2] = df_mul(par, df_add(gx, cy));
            v[4 * r + 3] = df_mul(par, df_add(cx, df_neg(gy)));
        }
    }
#pragma unroll
    for (int o = 0; o < NO; ++o) {
        float mx = fabsf(v[o].h);
#pragma unroll
        for (int sft = 16; sft > 0; sft >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, sft));
        if (lane == 0) s_mx[warp][o] = mx;
    }
    // lambda exponent: 2^El > sqrt((2 lhi + 1) / (4 pi)) >= |lambda_l| for l <= lhi;
    // in FP32: (2 lhi + 1) / (4 pi) is at least 1 / (2 lhi + 1) (relative) away
    // from every power of two, far beyond the FP32 rounding
    int El;
    frexpf(sqrtf((2.f * (wb + cnt - 1) + 1.f) * 0.0795774715459476679f), &El);
    __syncthreads();
    if (i < NO) {
        float cm = 0.f;
#pragma unroll
        for (int w = 0; w < TCL_W / 32; ++w) cm = fmaxf(cm, s_mx[w][i]);
        // column exponent 2^Ea > max |a|, clamped so that the digit scale stays a
        // normal power of two (columns below 2^-80 contribute digits 0)
        int ex = 0;
        if (cm > 0.f) frexpf(cm, &ex);
        ex = min(max(ex, -80), 100);
        s_ea[i] = ex;
        float *sc = reinterpret_cast<float *>(R + LY::RSC);
#pragma unroll
        for (int g = 0; g < NG; ++g) sc[g * NO + i] = pow2f_or0(El + ex - 14 - 8 * g);
    }
    if (i == 0) *reinterpret_cast<float *>(R + LY::RLS) = pow2f(7 - El);
    __syncthreads();
    unsigned short *tp = reinterpret_cast<unsigned short *>(R);
#pragma unroll
    for (int o = 0; o < NO; ++o) {
        float d[4];
        digits4s(v[o].h, v[o].l, pow2f(7 - s_ea[o]), d);
#pragma unroll
        for (int j = 0; j < 4; ++j) tp[(j * NO + o) * TCL_TPS + i] = (unsigned short)(__float_as_uint(d[j]) >> 16);
    }
}

// Roles: the ring warps (LY::T threads) hold one ring each and write the
// digit tiles (lambda into A, the window's alm digits into B'); the last warp
// issues the MMAs.  Per chunk each ring warp waits until the MMAs that last
// read the buffer are done (empty barrier, tcgen05.commit), writes its rows,
// and arrives on the buffer's full barrier (one arrival per warp); the MMA
// warp waits for all the arrivals.  The ring warps thus run up to a chunk
// apart instead of meeting at a block barrier every chunk.  The window
// records arrive by bulk copy, the next one prefetched while the current
// window runs; block-wide steps use barrier 1 over the ring warps only.
//
// S0 (spin 0): every ring thread holds one ring PAIR at theta (no second
// side), so a block covers T pairs instead of T / 2, and the columns (E, O)
// give theta E + O and pi - theta E - O.
template <int NB, bool S0>
__global__ void __launch_bounds__(TclLayout<NB>::BLOCK, 1)
    k_leg_synth_spin_tc(int L, int spin, const unsigned char *__restrict__ rec, const int *__restrict__ woff,
                        const double *__restrict__ lg0, int npairs,
                        const double *__restrict__ px, const double *__restrict__ psh,
                        const double *__restrict__ pch, const int *__restrict__ prn, const int *__restrict__ prs,
                        const float4 *__restrict__ stv, const short2 *__restrict__ ste, int st_ld,
                        double2 *__restrict__ H, long long hstride, int ldH, int *status) {
    using LY = TclLayout<NB>;
    constexpr int NO = LY::NO, NN = LY::NN, NG = LY::NG, T = LY::T, NT = LY::NT;
    constexpr int NCOPY = 13 * 2 * NO;  // B' K-cores per chunk
    static_assert(NT * NN <= 512, "tensor memory holds 512 columns");
    static_assert(LY::BYTES <= 227 * 1024, "dynamic shared memory of one block");
    static_assert(LY::OFF_R % 16 == 0 && LY::RSZ % 16 == 0, "bulk copies start and end on 16 bytes");
    static_assert(LY::OFF_B % 1024 == 0 && LY::BBUF % 1024 == 0, "MMA operand tiles on 8-row groups");
    static_assert(LY::OFF_BAR % 8 == 0, "mbarriers are 8-byte words");
    extern __shared__ __align__(1024) unsigned char sm[];
    uint32_t *s_tm = reinterpret_cast<uint32_t *>(sm + LY::OFF_TM);
    volatile int *s_bad = reinterpret_cast<volatile int *>(sm + LY::OFF_TM + 4);
    const uint32_t sbase = smem_u32(sm);
    const uint32_t full0 = sbase + LY::OFF_BAR, empty0 = full0 + 16, rbar0 = full0 + 32;  // [2] each

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m = blockIdx.y;
    const int l0 = max(m, spin);
    const unsigned char *recm = rec + (size_t)woff[m] * LY::RSZ;  // this order's window records

    int *s_c0 = reinterpret_cast<int *>(sm + LY::OFF_TM + 8);
    if (warp == T / 32) tmem_alloc(sbase + LY::OFF_TM, LY::NCOLS);
    if (tid == 0) {
        mbar_init(full0, T / 32);
        mbar_init(full0 + 8, T / 32);
        mbar_init(empty0, 1);
        mbar_init(empty0 + 8, 1);
        mbar_init(rbar0, 1);
        mbar_init(rbar0 + 8, 1);
        *s_bad = 0;
        *s_c0 = TC_NEVER;
        mbar_init_fence();
    }
    // B' positions with g - i outside [0, 3] and the padding rows stay zero for the whole kernel
    for (int i = tid; i < 2 * LY::BBUF / 16; i += LY::BLOCK)
        reinterpret_cast<uint4 *>(sm + LY::OFF_B)[i] = make_uint4(0u, 0u, 0u, 0u);

    // ring threads: this ring's recursion state at its first accumulated chunk c_me
    // (the plan's table), or the start at l0 (c_me = 0)
    const bool ring_thread = warp < T / 32;
    const int side = S0 ? 0 : tid / (T / 2);  // 0: ring theta, 1: ring pi - theta
    const int p = S0 ? blockIdx.x * T + tid : blockIdx.x * (T / 2) + tid % (T / 2);
    const bool act = ring_thread && p < npairs;
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
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *s_tm;
    {
        const int cm = __reduce_min_sync(0xffffffffu, c_me);
        if (lane == 0 && ring_thread && cm < TC_NEVER) atomicMin(s_c0, cm);
    }
    __syncthreads();
    // the block starts at the first chunk in which any of its rings accumulates:
    // window kw0, chunk cs0 of it; nothing to do when no ring ever does
    const int nchk = l0 <= L ? (L - l0 + 1 + TCL_KC - 1) / TCL_KC : 0;
    const int cb = *s_c0;
    const bool work = cb < nchk;
    constexpr int CPW = TCL_W / TCL_KC;  // chunks per window
    const int kw0 = work ? cb / CPW : 0, cs0 = cb - kw0 * CPW;
    if (tid == 0 && work) bulk_g2s(sbase + LY::OFF_R, recm + (size_t)kw0 * LY::RSZ, LY::RSZ, rbar0);

    if (warp == T / 32) {
        // ---------------- MMA warp: the whole warp follows the chunk sequence (its
        // outcome kept warp-uniform), lane 0 issues
        constexpr uint32_t IDESC = idesc_bf16_f32(128, NN);
        int gc = 0;
        bool ok = true;
        for (int kw = kw0; work && l0 + kw * TCL_W <= L && ok; ++kw) {
            const int wb = l0 + kw * TCL_W;
            const int nch = (min(TCL_W, L - wb + 1) + TCL_KC - 1) / TCL_KC;
            const int cs = kw == kw0 ? cs0 : 0;
            for (int c = cs; c < nch; ++c, ++gc) {
                const int buf = gc & 1;
                const bool got = !*s_bad && mbar_wait(full0 + 8 * buf, (gc >> 1) & 1);
                if (!__all_sync(0xffffffffu, got)) {
                    *s_bad = 1;
                    ok = false;
                    break;
                }
                if (lane == 0) {
                    tc_fence_after();
                    const uint32_t aa = sbase + buf * LY::ABUF, ba = sbase + LY::OFF_B + buf * LY::BBUF;
#pragma unroll
                    for (int t = 0; t < NT; ++t)
#pragma unroll
                        for (int k = 0; k < 4; ++k)  // K-step k: digit k of lambda, 16 l
                            tc_mma(tbase + t * NN, sdesc(aa + t * TCL_TILE + k * 256, 128, TCL_SBO),
                                   sdesc(ba + k * 256, 128, TCL_SBO), IDESC, (c > cs || k > 0) ? 1u : 0u);
                    tc_commit(empty0 + 8 * buf);
                }
                __syncwarp();
            }
        }
        if (!ok && gc > 0) mbar_wait(empty0 + 8 * ((gc - 1) & 1), ((gc - 1) >> 1) & 1);
        __syncwarp();
    } else {
        // ---------------- ring warps
        const int tile = tid >> 7, row = tid & 127;
        const double x = act ? px[p] : 0.0;
        const dfl xd = df_from(side ? -x : x);
        sum2 acc[NO];
        const uint32_t t_lane = tbase + ((uint32_t)((warp & 3) * 32) << 16) + tile * NN;  // this thread's row
        const uint32_t a_row = (uint32_t)tile * TCL_TILE + (row >> 3) * TCL_SBO + (row & 7) * 16;
        int gc = 0, kw = kw0, kl = 0;  // kl: windows processed (record buffer and barrier phase)
        int bad = 0;

        for (; work && l0 + kw * TCL_W <= L; ++kw, ++kl) {
            const int wb = l0 + kw * TCL_W;
            const int cnt = min(TCL_W, L - wb + 1);
            // prefetch the next window's record into the other buffer (its readers
            // finished at the previous window's closing barrier)
            if (tid == 0 && wb + TCL_W <= L) {
                fence_async_smem();
                bulk_g2s(sbase + LY::OFF_R + ((kl + 1) & 1) * LY::RSZ, recm + (size_t)(kw + 1) * LY::RSZ, LY::RSZ,
                         rbar0 + 8 * ((kl + 1) & 1));
            }
            bad |= !mbar_wait(rbar0 + 8 * (kl & 1), (kl >> 1) & 1);  // this window's record has landed
            const unsigned char *Rw = sm + LY::OFF_R + (kl & 1) * LY::RSZ;
            const unsigned short *s_tp = reinterpret_cast<const unsigned short *>(Rw);
            const float *s_sc = reinterpret_cast<const float *>(Rw + LY::RSC);
            const float lsc = *reinterpret_cast<const float *>(Rw + LY::RLS);
            // recursion coefficients, zero past the window so that the steps beyond lmax stay finite
            const float4 *s_ag = reinterpret_cast<const float4 *>(Rw + LY::RCO);
            const float2 *s_be = reinterpret_cast<const float2 *>(Rw + LY::RBE);

            const int nch = (cnt + TCL_KC - 1) / TCL_KC;
            for (int c = kw == kw0 ? cs0 : 0; c < nch; ++c, ++gc) {
                const int buf = gc & 1;
                // before its first chunk a ring holds its table state and writes zero digits
                const bool live = kw * CPW + c >= c_me;
                if (gc >= 2) bad |= !mbar_wait(empty0 + 8 * buf, ((gc - 2) >> 1) & 1);
                unsigned char *sA = sm + buf * LY::ABUF;
                unsigned char *sB = sm + LY::OFF_B + buf * LY::BBUF;
                // B' of this chunk: row n = g NO + o, K-core (digit i, 8 l) = t_{g-i} of
                // output o; one 16-byte copy from the record's digit planes per (pair
                // (g, i), l half, o), spread over the ring threads
#pragma unroll
                for (int q0 = 0; q0 < NCOPY; q0 += T) {
                    const int q = q0 + tid;
                    if (q < NCOPY) {
                        const int pr = q / (2 * NO), rem = q - pr * 2 * NO;
                        const int lh = rem / NO, o = rem - lh * NO;
                        int g, di;
                        tcl_pair(pr, g, di);
                        const int n = g * NO + o;
                        const uint4 v = *reinterpret_cast<const uint4 *>(s_tp + ((g - di) * NO + o) * TCL_TPS +
                                                                         c * TCL_KC + 8 * lh);
                        *reinterpret_cast<uint4 *>(sB + (n >> 3) * TCL_SBO + (2 * di + lh) * 128 + (n & 7) * 16) = v;
                    }
                }
                // lambda digits for 16 l in two halves of 8, each stored as four 16-byte K-cores.
                // The exponent check runs once per half: a step grows the mantissa by at
                // most (alpha + beta) < 2^8.5 (alpha_m ~ sqrt(2m) <= 181 for lmax <= 16383),
                // so from below 2^40 eight steps stay below 2^108, inside the FP32
                // range, and e (hence the digit mask) stays fixed within the half.
                float4 agn = s_ag[c * TCL_KC];  // coefficients of the next step, loaded one step ahead
                float2 ben = s_be[c * TCL_KC];
                if (live) {
#pragma unroll
                    for (int lh = 0; lh < 2; ++lh) {
                        uint32_t pk[4][4];
                        const float scg = (act && e == 0) ? lsc : 0.f;
#pragma unroll
                        for (int j2 = 0; j2 < 4; ++j2) {
                            float d0[4], d1[4];
                            // digits of lambda_l (zero unless accumulated), then one recursion step l -> l + 1
                            auto step = [&](int i, float(&d)[4]) {
                                digits4s(cur.h, cur.l, i < cnt ? scg : 0.f, d);
                                const float4 ag = agn;
                                const float2 b2 = ben;
                                agn = s_ag[i + 1];
                                ben = s_be[i + 1];
                                const dfl t = df_fma_u(dfl{ag.x, ag.y}, xd, dfl{ag.z, ag.w});
                                const dfl nxt = df_mul_sub(t, cur, dfl{b2.x, b2.y}, prev);
                                prev = cur;
                                cur = nxt;
                            };
                            const int i0 = c * TCL_KC + 8 * lh + 2 * j2;
                            step(i0, d0);
                            step(i0 + 1, d1);
#pragma unroll
                            for (int k = 0; k < 4; ++k) pk[k][j2] = pack_bf16(d0[k], d1[k]);
                        }
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            *reinterpret_cast<uint4 *>(sA + a_row + (2 * k + lh) * 128) =
                                make_uint4(pk[k][0], pk[k][1], pk[k][2], pk[k][3]);
                        REC_RESCALE_DF(cur, prev, e);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        *reinterpret_cast<uint4 *>(sA + a_row + k * 128) = make_uint4(0u, 0u, 0u, 0u);
                }
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(full0 + 8 * buf);
            }
            // window epilogue: the exact weight sums -> compensated accumulators
            bad |= !mbar_wait(empty0 + 8 * ((gc - 1) & 1), ((gc - 1) >> 1) & 1);
            bad = __any_sync(0xffffffffu, bad);  // warp-uniform: the loads below are warp-collective
            tc_fence_after();
            if (!bad) {
                // Column n = g NO + o holds the exact sum of weight 2^-8g (an integer
                // below 2^24).  Weights 4..1 are folded by Horner in FP32: its rounding,
                // 2^-24 of a value that carries weight 2^-8, is about 2^-32 of the
                // window's sum, below the digit truncation of lambda and a.  Weight 0
                // and the fold then enter the compensated accumulator.  Outputs go in
                // groups of OG (one 8-column load per weight, starting on a multiple of
                // 8) so that the fold, the loaded sums and the accumulators fit the
                // register budget.
                static_assert(NO % 4 == 0, "outputs per ring");
                constexpr int OG = NO % 8 == 0 ? 8 : 4;
#pragma unroll
                for (int o0 = 0; o0 < NO; o0 += OG) {
                    float hr[OG];
#pragma unroll
                    for (int g = NG - 1; g >= 0; --g) {
                        const int col = g * NO + o0, sub = col & 7;  // sub + OG <= 8
                        float dv[8];
                        tmem_ld8(t_lane + (col - sub), dv);
#pragma unroll
                        for (int i = 0; i < OG; ++i) {
                            if (g == NG - 1) hr[i] = dv[sub + i];
                            else if (g > 0) hr[i] = fmaf(hr[i], 0x1p-8f, dv[sub + i]);
                            else {
                                acc[o0 + i].add(dv[sub + i] * s_sc[o0 + i]);
                                acc[o0 + i].add(hr[i] * s_sc[NO + o0 + i]);
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            // all ring warps are done with the window's tables; any wait that ran out ends the block
            bad = bar_or_1(T, bad | *s_bad);
            if (bad) break;
        }

        if (bad) {
            *s_bad = 1;
            if (tid == 0) {
                if (status) atomicOr(status, 1);
                // the record copy of the window after the last one entered may still be in flight
                if (l0 + (kw + 1) * TCL_W <= L) mbar_wait(rbar0 + 8 * ((kl + 1) & 1), ((kl + 1) >> 1) & 1);
            }
        } else if (act && S0) {
            const int n = prn[p], s = prs[p];
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                // E + O, E - O in double-float, one integer-pipe conversion each (no FP64 arithmetic)
                double2 *Hr = H + r * hstride;
                const dfl er = acc[4 * r].df(), ei = acc[4 * r + 1].df();
                const dfl orr = acc[4 * r + 2].df(), oi = acc[4 * r + 3].df();
                Hr[(long long)m * ldH + n] = make_double2(df_to(df_add(er, orr)), df_to(df_add(ei, oi)));
                if (s != n)
                    Hr[(long long)m * ldH + s] =
                        make_double2(df_to(df_add(er, df_neg(orr))), df_to(df_add(ei, df_neg(oi))));
            }
        } else if (act) {
            const int n = prn[p], s = prs[p];
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                // signs applied to the pairs before the conversion (no FP64 products)
                double2 *Hr = H + r * hstride;
                const double2 A = make_double2(df_to(df_neg(acc[4 * r].df())), df_to(df_neg(acc[4 * r + 1].df())));
                const dfl b2 = acc[4 * r + 2].df(), b3 = acc[4 * r + 3].df();
                const double2 B = (spin & 1) ? make_double2(df_to(b2), df_to(b3))
                                             : make_double2(df_to(df_neg(b2)), df_to(df_neg(b3)));
                if (side == 0) {
                    Hr[(long long)(L + m) * ldH + n] = A;
                    if (m > 0 && s != n) Hr[(long long)(L - m) * ldH + s] = B;
                } else {
                    if (s != n) Hr[(long long)(L + m) * ldH + s] = A;
                    if (m > 0) Hr[(long long)(L - m) * ldH + n] = B;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == T / 32) {
        tc_fence_after();
        tmem_dealloc(tbase, LY::NCOLS);
    }
}

template <int NB, bool S0>
static int launch_synth_tc_nb(const cunusht_plan_s *P, int npairs, const double *x, const double *sh,
                              const double *ch, const int *rn, const int *rs, const float4 *stv, const short2 *ste,
                              int st_ld, int ld, int spin, const double2 *G,
                              const double2 *C, long long astride, const double *lf, double2 *H, long long hstride,
                              cudaStream_t st) {
    using LY = TclLayout<NB>;
    const int L = P->lmax;
    if (P->tc_rec_nb < NB) {
        set_error("tensor-core records hold %d requests per launch, %d asked (cunusht_plan_reserve_batch)",
                  P->tc_rec_nb, NB);
        return CUNUSHT_ERR_ARG;
    }
    const dim3 rgrid((L - spin + 1 + TCL_W - 1) / TCL_W, P->mmax + 1);  // m <= spin has the most windows
    k_tc_records<NB, S0><<<rgrid, TCL_W, 0, st>>>(L, spin, G, C, astride, lf, P->d_coef_df[spin], P->nalm_tab,
                                                  P->d_tc_woff[spin], P->d_tc_rec);
    CU_LAUNCH_CHECK();
    CU_TRY(cudaFuncSetAttribute(k_leg_synth_spin_tc<NB, S0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                LY::BYTES));
    constexpr int PER = S0 ? LY::T : LY::T / 2;  // ring pairs per block
    dim3 grid((npairs + PER - 1) / PER, P->mmax + 1);
    k_leg_synth_spin_tc<NB, S0><<<grid, LY::BLOCK, LY::BYTES, st>>>(L, spin, P->d_tc_rec, P->d_tc_woff[spin],
                                                                P->d_lg0[spin], npairs, x, sh, ch, rn, rs, stv, ste,
                                                                st_ld, H, hstride, ld, P->d_status);
    CU_LAUNCH_CHECK();
    return CUNUSHT_OK;
}

static size_t tcl_record_bytes(int nb) {
    return nb >= 8   ? TclLayout<8>::RSZ
           : nb >= 4 ? TclLayout<4>::RSZ
           : nb >= 2 ? TclLayout<2>::RSZ
                     : TclLayout<1>::RSZ;
}

// record buffer for launches of up to nb requests (1, 2, 4 or 8); grows only
int tc_reserve(cunusht_plan_s *P, int nb) {
    nb = nb >= 8 ? 8 : nb >= 4 ? 4 : nb >= 2 ? 2 : 1;
    if (nb <= P->tc_rec_nb || P->tc_nrec == 0) return CUNUSHT_OK;
    const size_t bytes = P->tc_nrec * tcl_record_bytes(nb);
    if (P->d_tc_rec) {
        CU_TRY(cudaDeviceSynchronize());  // the old buffer may still be read by queued work
        cudaFree(P->d_tc_rec);
        P->ws_bytes -= P->tc_rec_bytes;
        P->d_tc_rec = nullptr;
        P->tc_rec_bytes = 0;
        P->tc_rec_nb = 0;
    }
    const cudaError_t e = cudaMalloc(&P->d_tc_rec, bytes);
    if (e != cudaSuccess) {
        P->d_tc_rec = nullptr;
        set_error("cudaMalloc of %zu bytes (tensor-core window records) failed: %s", bytes, cudaGetErrorString(e));
        return CUNUSHT_ERR_ALLOC;
    }
    P->tc_rec_bytes = bytes;
    P->ws_bytes += bytes;
    P->tc_rec_nb = nb;
    return CUNUSHT_OK;
}

// Recursion start states of every (m, side, pair) of one grid and spin, built
// once per plan.  A ring whose functions are still below the accumulated range
// (the evanescent region sin(theta) < m / l, where lambda_lm decays like
// exp(-l ...) towards the pole) contributes zero digits to every chunk before
// the one where its exponent e reaches 0.  The table holds, per ring, that
// first chunk c0 (16 l from l0 = max(m, s)) and the recursion state (cur,
// prev, e) at its start, obtained by running the kernels' own double-float
// steps (same coefficients, same operations, the exponent check after every 8
// l) from rec_start_df.  The kernels start each ring there and each block at
// the smallest c0 of its rings, so chunks in which no ring of a block
// accumulates are neither recursed nor multiplied (about a fifth of the
// (l, m, ring) volume at lmax 2047), with the same digits for the chunks that
// are.  A ring whose start is exactly zero (a pole) gets c0 = 32767 (never).
// Entry ((m * 2 + side) * npairs + p): v = (cur.h, cur.l, prev.h, prev.l),
// ec = (e / 96, c0); e is 0 or -96 at a ring's first chunk.
__device__ __forceinline__ void tc_rec_step(dfl &cur, dfl &prev, dfl xd, const float2 *__restrict__ coef,
                                            long long nalm, long long ix) {
    const float2 a2 = coef[ix], g2 = coef[nalm + ix], b2 = coef[2 * nalm + ix];
    const dfl t = df_fma_u(dfl{a2.x, a2.y}, xd, dfl{g2.x, g2.y});
    const dfl nxt = df_mul_sub(t, cur, dfl{b2.x, b2.y}, prev);
    prev = cur;
    cur = nxt;
}

__global__ void k_tc_starts(int L, int spin, const double *__restrict__ lg0, int npairs, const double *__restrict__ x,
                            const double *__restrict__ sh, const double *__restrict__ ch,
                            const float2 *__restrict__ coef, long long nalm, float4 *__restrict__ v,
                            short2 *__restrict__ ec) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2LL * npairs * (L + 1)) return;
    const int p = (int)(i % npairs);
    const long long ms = i / npairs;
    const int side = (int)(ms & 1), m = (int)(ms >> 1);
    const int l0 = max(m, spin);
    dfl cur, prev;
    int e;
    if (side) rec_start_df(lg0[m], m, spin, ch[p], sh[p], cur, prev, e);
    else rec_start_df(lg0[m], m, spin, sh[p], ch[p], cur, prev, e);
    const dfl xd = df_from(side ? -x[p] : x[p]);
    const long long b = almidx(L, m, m) - m;  // (l, m) at b + l
    const int nchk = l0 <= L ? (L - l0 + 1 + TCL_KC - 1) / TCL_KC : 0;
    int c = 0;
    for (; c < nchk && e != 0; ++c) {
        // the chunk's first half accumulates only if e is 0 at its start; its
        // second half if the check after the first 8 steps brings e to 0
        const dfl c0 = cur, p0 = prev;
        const int e0 = e, lb = l0 + TCL_KC * c;
        for (int j = 0; j < 8; ++j)
            if (lb + j <= L) tc_rec_step(cur, prev, xd, coef, nalm, b + lb + j);
        REC_RESCALE_DF(cur, prev, e);
        if (e == 0) {
            cur = c0, prev = p0, e = e0;
            break;
        }
        for (int j = 8; j < TCL_KC; ++j)
            if (lb + j <= L) tc_rec_step(cur, prev, xd, coef, nalm, b + lb + j);
        REC_RESCALE_DF(cur, prev, e);
    }
    const bool never = c >= nchk || (cur.h == 0.f && prev.h == 0.f);
    v[i] = make_float4(cur.h, cur.l, prev.h, prev.l);
    ec[i] = make_short2((short)(e / 96), never ? TC_NEVER : (short)c);
}

// Build (enable) or release the start states of one grid (0 GL, 1 CC) and
// spin; without them the tensor-core kernels start every ring at l0 from
// rec_start_df (no chunk is skipped).  Synchronises the device.
int tc_start_states(cunusht_plan_s *P, int g, int s, bool enable) {
    const int L = P->lmax;
    const int np = g ? P->cc_npairs : P->gl_npairs;
    const size_t n = 2 * (size_t)np * (L + 1);
    const size_t bytes = n * (sizeof(float4) + sizeof(short2));
    CU_TRY(cudaDeviceSynchronize());  // earlier work may still read the tables
    if (!enable) {
        if (P->d_tc_stv[g][s]) {
            cudaFree(P->d_tc_stv[g][s]);
            cudaFree(P->d_tc_ste[g][s]);
            P->d_tc_stv[g][s] = nullptr;
            P->d_tc_ste[g][s] = nullptr;
            P->ws_bytes -= bytes;
        }
        return CUNUSHT_OK;
    }
    if (P->d_tc_stv[g][s] || np == 0 || s > L) return CUNUSHT_OK;
    const double *x = g ? P->d_cc_x : P->d_gl_x;
    const double *sh = g ? P->d_cc_sh : P->d_gl_sh, *ch = g ? P->d_cc_ch : P->d_gl_ch;
    CU_TRY(cudaMalloc(&P->d_tc_stv[g][s], n * sizeof(float4)));
    const cudaError_t e = cudaMalloc(&P->d_tc_ste[g][s], n * sizeof(short2));
    if (e != cudaSuccess) {
        cudaFree(P->d_tc_stv[g][s]);
        P->d_tc_stv[g][s] = nullptr;
        P->d_tc_ste[g][s] = nullptr;
        CU_TRY(e);
    }
    P->ws_bytes += bytes;
    k_tc_starts<<<(unsigned)((n + 255) / 256), 256>>>(L, s, P->d_lg0[s], np, x, sh, ch, P->d_coef_df[s],
                                                     P->nalm_tab, P->d_tc_stv[g][s], P->d_tc_ste[g][s]);
    CU_LAUNCH_CHECK();
    CU_TRY(cudaDeviceSynchronize());  // the tables are read from any stream
    return CUNUSHT_OK;
}

int tc_plan_init(cunusht_plan_s *P) {
    const int L = P->lmax;
    // start tables: GL spin 1 (the pointing's synthesis) and spins 0 up to max_spin on both grids
    for (int g = 0; g < 2; ++g) {
        const int smax = g ? P->max_spin : std::max(P->max_spin, 1);
        for (int s = 0; s <= smax && s <= L; ++s) RC_TRY(tc_start_states(P, g, s, true));
    }
    size_t nrec = 0;
    for (int s = 0; s <= 2 && s <= L; ++s) {
        std::vector<int> wo(L + 2, 0);
        for (int m = 0; m <= L; ++m) wo[m + 1] = wo[m] + (L - std::max(m, s) + 1 + TCL_W - 1) / TCL_W;
        CU_TRY(cudaMalloc(&P->d_tc_woff[s], wo.size() * sizeof(int)));
        CU_TRY(cudaMemcpy(P->d_tc_woff[s], wo.data(), wo.size() * sizeof(int), cudaMemcpyHostToDevice));
        P->ws_bytes += wo.size() * sizeof(int);
        nrec = std::max(nrec, (size_t)wo[L + 1]);
    }
    P->tc_nrec = nrec;
    return tc_reserve(P, 1);  // single requests; cunusht_plan_reserve_batch grows it
}

// The pole pair (theta = 0, pi) of a spin s >= 1 synthesis: every function
// vanishes at theta = 0, and at theta = pi all but m = s, where
// sLambda_ls(pi) = (-1)^l sqrt((2l + 1) / (4 pi)).  The ring values are then
// one FP64 sum over l per request and component, and zeros; block r handles
// request r.  Same outputs and signs as the pair in k_leg_synth_spin_tc.
constexpr int POLE_TPB = 256;
__global__ void __launch_bounds__(POLE_TPB)
    k_pole_pair_spin(int L, int spin, int mmax, const double2 *__restrict__ G, const double2 *__restrict__ C,
                     long long astride, const double *__restrict__ lfac, int rn, int rs, double2 *__restrict__ H,
                     long long hstride, int ldH) {
    __shared__ double s_red[4][POLE_TPB / 32];
    const int r = blockIdx.x, tid = threadIdx.x;
    double2 *Hr = H + r * hstride;
    const double2 z = make_double2(0.0, 0.0);
    for (int m = tid; m <= mmax; m += POLE_TPB) {
        Hr[(long long)(L + m) * ldH + rn] = z;
        if (m != spin) Hr[(long long)(L + m) * ldH + rs] = z;
        if (m > 0) {
            Hr[(long long)(L - m) * ldH + rs] = z;
            if (m != spin) Hr[(long long)(L - m) * ldH + rn] = z;
        }
    }
    if (spin > mmax) return;
    const double2 *Gr = G + r * astride, *Cr = C ? C + r * astride : nullptr;
    const long long b = almidx(L, spin, spin) - spin;
    double a_re = 0.0, a_im = 0.0, b_re = 0.0, b_im = 0.0;
    for (int l = spin + tid; l <= L; l += POLE_TPB) {
        const double lam = ((l & 1) ? -1.0 : 1.0) * sqrt((2.0 * l + 1.0) / (4.0 * PI));
        const double f = lfac ? lfac[l] : 1.0;
        const double par = ((l + spin) & 1) ? -f : f;
        const double2 g = Gr[b + l];
        const double2 c = Cr ? Cr[b + l] : z;
        a_re += f * (g.x - c.y) * lam;
        a_im += f * (g.y + c.x) * lam;
        b_re += par * (g.x + c.y) * lam;
        b_im += par * (c.x - g.y) * lam;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a_re += __shfl_xor_sync(0xffffffffu, a_re, o);
        a_im += __shfl_xor_sync(0xffffffffu, a_im, o);
        b_re += __shfl_xor_sync(0xffffffffu, b_re, o);
        b_im += __shfl_xor_sync(0xffffffffu, b_im, o);
    }
    if ((tid & 31) == 0) {
        s_red[0][tid >> 5] = a_re;
        s_red[1][tid >> 5] = a_im;
        s_red[2][tid >> 5] = b_re;
        s_red[3][tid >> 5] = b_im;
    }
    __syncthreads();
    if (tid == 0) {
        double t[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < 4; ++k)
            for (int w = 0; w < POLE_TPB / 32; ++w) t[k] += s_red[k][w];
        const double sgs = (spin & 1) ? -1.0 : 1.0;
        Hr[(long long)(L + spin) * ldH + rs] = make_double2(-t[0], -t[1]);
        Hr[(long long)(L - spin) * ldH + rn] = make_double2(-sgs * t[2], -sgs * t[3]);
    }
}

// The pole pair of a spin-0 synthesis: lambda_lm(0) = delta_m0 sqrt((2l+1)/(4 pi))
// and lambda_lm(pi) = (-1)^l lambda_lm(0), so both rings get zeros for m > 0
// and one FP64 sum over l for m = 0; block r handles request r.
__global__ void __launch_bounds__(POLE_TPB)
    k_pole_pair_s0(int L, int mmax, const double2 *__restrict__ G, long long astride,
                   const double *__restrict__ lfac, int rn, int rs, double2 *__restrict__ H, long long hstride,
                   int ldH) {
    __shared__ double s_red[4][POLE_TPB / 32];
    const int r = blockIdx.x, tid = threadIdx.x;
    double2 *Hr = H + r * hstride;
    for (int m = 1 + tid; m <= mmax; m += POLE_TPB) {
        Hr[(long long)m * ldH + rn] = make_double2(0.0, 0.0);
        Hr[(long long)m * ldH + rs] = make_double2(0.0, 0.0);
    }
    const double2 *Gr = G + r * astride;  // m = 0: (l, 0) at index l
    double n_re = 0.0, n_im = 0.0, s_re = 0.0, s_im = 0.0;
    for (int l = tid; l <= L; l += POLE_TPB) {
        const double lam = sqrt((2.0 * l + 1.0) / (4.0 * PI)) * (lfac ? lfac[l] : 1.0);
        const double2 a = Gr[l];
        const double sg = (l & 1) ? -lam : lam;
        n_re += a.x * lam;
        n_im += a.y * lam;
        s_re += a.x * sg;
        s_im += a.y * sg;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_re += __shfl_xor_sync(0xffffffffu, n_re, o);
        n_im += __shfl_xor_sync(0xffffffffu, n_im, o);
        s_re += __shfl_xor_sync(0xffffffffu, s_re, o);
        s_im += __shfl_xor_sync(0xffffffffu, s_im, o);
    }
    if ((tid & 31) == 0) {
        s_red[0][tid >> 5] = n_re;
        s_red[1][tid >> 5] = n_im;
        s_red[2][tid >> 5] = s_re;
        s_red[3][tid >> 5] = s_im;
    }
    __syncthreads();
    if (tid == 0) {
        double t[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < 4; ++k)
            for (int w = 0; w < POLE_TPB / 32; ++w) t[k] += s_red[k][w];
        Hr[rn] = make_double2(t[0], t[1]);
        Hr[rs] = make_double2(t[2], t[3]);
    }
}

// Ring pairs in full blocks (256 pairs, 128 for NB = 8; spin 0: 512 and 256) on the tensor cores; a
// tail of fewer than TCL_MIN_TAIL pairs after at least one full block goes to
// the double-float CUDA-core kernel instead of a nearly empty block per order m.
int leg_synth_spin_tc(const cunusht_plan_s *P, int nb, int npairs, const double *x, const double *sh,
                      const double *ch, const int *rn, const int *rs, int ld, int pole, int pole_rn, int pole_rs,
                      const float4 *stv, const short2 *ste, int spin, const double2 *G, const double2 *C,
                      long long astride, const double *lf, double2 *H, long long hstride, cudaStream_t st) {
    const int st_ld = npairs;  // row stride of the start table: all pairs of the grid
    if (pole == 0 && npairs > 1) {
        // the pole pair in closed form; the tensor cores take the other pairs
        // (a Clenshaw-Curtis grid of 2^k + 1 rings then fills whole blocks)
        if (spin == 0)
            k_pole_pair_s0<<<nb, POLE_TPB, 0, st>>>(P->lmax, P->mmax, G, astride, lf, pole_rn, pole_rs, H, hstride,
                                                    ld);
        else
            k_pole_pair_spin<<<nb, POLE_TPB, 0, st>>>(P->lmax, spin, P->mmax, G, C, astride, lf, pole_rn, pole_rs,
                                                      H, hstride, ld);
        CU_LAUNCH_CHECK();
        ++x, ++sh, ++ch, ++rn, ++rs;
        if (stv) ++stv, ++ste;
        --npairs;
    }
    const int per = (nb == 8 ? TclLayout<8>::T : TclLayout<4>::T) / (spin == 0 ? 1 : 2), tail = npairs % per;
    const int ntc = (npairs > per && tail < TCL_MIN_TAIL) ? npairs - tail : npairs;
    auto launch = [&](auto nbc) {
        constexpr int NBV = decltype(nbc)::value;
        if (spin == 0)
            return launch_synth_tc_nb<NBV, true>(P, ntc, x, sh, ch, rn, rs, stv, ste, st_ld, ld, spin, G, nullptr,
                                                 astride, lf, H, hstride, st);
        return launch_synth_tc_nb<NBV, false>(P, ntc, x, sh, ch, rn, rs, stv, ste, st_ld, ld, spin, G, C, astride,
                                              lf, H, hstride, st);
    };
    if (nb == 8) RC_TRY(launch(std::integral_constant<int, 8>{}));
    else if (nb == 4) RC_TRY(launch(std::integral_constant<int, 4>{}));
    else if (nb == 2) RC_TRY(launch(std::integral_constant<int, 2>{}));
    else RC_TRY(launch(std::integral_constant<int, 1>{}));
    // the CUDA-core kernels take at most four requests per launch
    for (int r0 = 0; ntc < npairs && r0 < nb; r0 += 4)
        RC_TRY(leg_synth_spin_df_pairs(P, std::min(4, nb - r0), npairs - ntc, x + ntc, sh + ntc, ch + ntc, rn + ntc,
                                       rs + ntc, ld, spin, G + r0 * astride, C ? C + r0 * astride : nullptr, astride,
                                       lf, H + r0 * hstride, hstride, st));
    return CUNUSHT_OK;
}

}  // namespace cunusht

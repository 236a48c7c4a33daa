// Spin-s synthesis on a small ring geometry that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool (the pool owns all device memory and forbids raw
// allocations next to it), latency-critical pipelines that forbid allocation
// after start-up because cudaMalloc can synchronise the device, and plugin
// hosts that hand a plugin no allocator at all.  cunusht_synthesis_noalloc
// serves them: the caller passes the alm and the output map, and every
// intermediate table and buffer lives in one file-scope __device__ array of
// CUNUSHT_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// until the process exits.  It runs the same kernels as cunusht_synthesis.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cunusht {

static __device__ __align__(256) unsigned char g_noalloc_scratch[CUNUSHT_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device.  In host code the symbol
// name is only a host-side stand-in, never a device address, so it is looked
// up with cudaGetSymbolAddress once per device, with that device current.
// The cached address outlives nothing but the process's CUDA context: after a
// cudaDeviceReset the module is loaded again and the cached address would be
// stale, so a device reset between calls is not supported.
static std::mutex g_scratch_mu;
static void *g_scratch_ptr[256] = {};

static int scratch_address(void **out) {
    int dev = 0;
    CU_TRY(cudaGetDevice(&dev));
    ARG_CHECK(dev >= 0 && dev < 256, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("cudaGetSymbolAddress of the no-alloc scratch failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            return CUNUSHT_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return CUNUSHT_OK;
}

// Bump layout of the scratch array (256-byte aligned pieces).
struct ScratchLayout {
    size_t off = 0;
    template <typename T> size_t take(size_t n) {
        const size_t at = off;
        off += ((n * sizeof(T) + 255) / 256) * 256;
        return at;
    }
};

// Ring tables of one call, passed BY VALUE as a kernel parameter (under the
// classic 4 KB parameter limit), so that the call copies nothing from host
// memory: no pageable transfer that could block the host.  Ring pairs
// (theta, pi - theta) are sorted on the host; everything else is computed on
// the device into the scratch array.
struct NoallocRings {
    double theta_n[(CUNUSHT_NOALLOC_MAX_NRING + 1) / 2];  // north ring of each pair
    short rn[(CUNUSHT_NOALLOC_MAX_NRING + 1) / 2];        // ring index, north / south member
    short rs[(CUNUSHT_NOALLOC_MAX_NRING + 1) / 2];
    double phi0[CUNUSHT_NOALLOC_MAX_NRING];
    int npairs, nring, nphi, lmax, spin, Mb;
};
static_assert(sizeof(NoallocRings) <= 4000, "no-alloc ring tables must fit a 4 KB kernel parameter");

struct NoallocTables {
    double *lg, *px, *psh, *pch, *phi0;
    int *prn, *prs;
    long long *nph, *ofs;
    double2 *chirp, *bk, *tw;
};

// One thread per table entry over the concatenated index ranges:
// pairs | rings | m = 0..lmax | chirp (nphi) | Bluestein kernel (Mb) | twiddles (Mb)
__global__ void k_noalloc_tables(const NoallocRings R, NoallocTables T) {
    const long long n_pairs = R.npairs, n_rings = R.nring, n_m = R.lmax + 1, n_ch = R.nphi, n_bk = R.Mb;
    const long long total = n_pairs + n_rings + n_m + n_ch + 2 * n_bk;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        long long k = i;
        if (k < n_pairs) {
            const double t = R.theta_n[k];
            T.px[k] = cos(t);
            T.psh[k] = sin(0.5 * t);
            T.pch[k] = cos(0.5 * t);
            T.prn[k] = R.rn[k];
            T.prs[k] = R.rs[k];
            continue;
        }
        k -= n_pairs;
        if (k < n_rings) {
            T.phi0[k] = R.phi0[k];
            T.nph[k] = R.nphi;
            T.ofs[k] = k * (long long)R.nphi;
            continue;
        }
        k -= n_rings;
        if (k < n_m) {  // log2 of the recursion start's normalisation (as the plan's lg0 table)
            const int m = (int)k, s = R.spin, l0 = m > s ? m : s;
            const double v = log((2.0 * l0 + 1.0) / (4.0 * PI)) + lgamma(2.0 * l0 + 1.0) - lgamma(m + s + 1.0) -
                             lgamma(fabs((double)(m - s)) + 1.0);
            T.lg[m] = 0.5 * v / log(2.0);
            continue;
        }
        k -= n_m;
        if (k < n_ch) {  // chirp_q = exp(i pi q^2 / nphi), q^2 reduced mod 2 nphi
            const long long qq = (k * k) % (2LL * R.nphi);
            double sn, cs;
            sincospi((double)qq / R.nphi, &sn, &cs);
            T.chirp[k] = make_double2(cs, sn);
            continue;
        }
        k -= n_ch;
        if (k < n_bk) {  // conj(chirp) / Mb at k and Mb - k (k < nphi), zero between
            long long q = -1;
            if (k < R.nphi) q = k;
            else if (k > R.Mb - R.nphi) q = R.Mb - k;
            double2 b = make_double2(0.0, 0.0);
            if (q >= 0) {
                const long long qq = (q * q) % (2LL * R.nphi);
                double sn, cs;
                sincospi((double)qq / R.nphi, &sn, &cs);
                b = make_double2(cs / R.Mb, -sn / R.Mb);
            }
            T.bk[k] = b;
            continue;
        }
        k -= n_bk;
        {  // twiddles exp(-2 pi i t / Mb)
            double sn, cs;
            sincospi(-2.0 * (double)k / R.Mb, &sn, &cs);
            T.tw[k] = make_double2(cs, sn);
        }
    }
}

}  // namespace cunusht

using namespace cunusht;

extern "C" int cunusht_synthesis_noalloc(int lmax, int spin, int ncomp, const void *alm, int nring,
                                         const double *ring_theta, const double *ring_phi0, int nphi,
                                         double *map, void *stream) {
    clear_error();
    ARG_CHECK(lmax >= 1 && lmax <= CUNUSHT_NOALLOC_MAX_LMAX,
              "no-alloc synthesis: lmax %d outside [1, %d] (the scratch array holds at most lmax %d)", lmax,
              CUNUSHT_NOALLOC_MAX_LMAX, CUNUSHT_NOALLOC_MAX_LMAX);
    ARG_CHECK(nring >= 1 && nring <= CUNUSHT_NOALLOC_MAX_NRING,
              "no-alloc synthesis: nring %d outside [1, %d]", nring, CUNUSHT_NOALLOC_MAX_NRING);
    ARG_CHECK(nphi >= 2 * lmax + 1 && nphi <= CUNUSHT_NOALLOC_MAX_NPHI,
              "no-alloc synthesis: nphi %d outside [2 lmax + 1 = %d, %d]", nphi, 2 * lmax + 1,
              CUNUSHT_NOALLOC_MAX_NPHI);
    ARG_CHECK(spin >= 0 && spin <= 2, "no-alloc synthesis: spin must be 0, 1 or 2");
    if (spin == 0) ARG_CHECK(ncomp == 1, "spin 0 takes ncomp = 1");
    else ARG_CHECK(ncomp == 1 || ncomp == 2, "spin > 0 takes ncomp 1 or 2");
    ARG_CHECK(alm && map && ring_theta && ring_phi0, "NULL array argument");
    cudaStream_t st = (cudaStream_t)stream;

    // ring pairs (theta, pi - theta) sorted on the host; the device builds the rest
    cunusht_plan_s P;  // host-side view; all device pointers point into the scratch array
    P.lmax = lmax;
    P.nalm = (long long)(lmax + 1) * (lmax + 2) / 2;
    P.nalm_tab = P.nalm;
    P.mmax = lmax;
    P.nring = nring;
    P.npix = (long long)nring * nphi;
    P.nph_uniform = nphi;
    std::vector<int> idx(nring);
    for (int i = 0; i < nring; ++i) {
        ARG_CHECK(ring_theta[i] >= 0.0 && ring_theta[i] <= PI, "ring %d colatitude outside [0, pi]", i);
        idx[i] = i;
    }
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return ring_theta[a] < ring_theta[b]; });
    NoallocRings R;
    int np = 0;
    for (int i = 0, j = nring - 1; i <= j; ++i, --j) {
        const double tn = ring_theta[idx[i]], ts = ring_theta[idx[j]];
        ARG_CHECK(std::fabs(tn + ts - PI) <= 1e-9, "no-alloc synthesis: rings must be north/south symmetric");
        R.theta_n[np] = tn;
        R.rn[np] = (short)idx[i];
        R.rs[np] = (short)idx[j];
        ++np;
    }
    for (int i = 0; i < nring; ++i) R.phi0[i] = ring_phi0[i];
    P.gl_npairs = np;
    int Mb = 1;
    while (Mb < 2 * nphi - 1) Mb <<= 1;
    P.Mb = Mb;
    P.TW = Mb;
    R.npairs = np;
    R.nring = nring;
    R.nphi = nphi;
    R.lmax = lmax;
    R.spin = spin;
    R.Mb = Mb;

    // scratch layout (the limits above keep it below CUNUSHT_NOALLOC_SCRATCH_BYTES)
    ScratchLayout Lo;
    const size_t o_coef = Lo.take<double>(3 * (size_t)P.nalm);
    const size_t o_lg = Lo.take<double>(lmax + 1);
    const size_t o_px = Lo.take<double>(np), o_psh = Lo.take<double>(np);
    const size_t o_pch = Lo.take<double>(np);
    const size_t o_prn = Lo.take<int>(np), o_prs = Lo.take<int>(np);
    const size_t o_phi0 = Lo.take<double>(nring);
    const size_t o_nph = Lo.take<long long>(nring), o_ofs = Lo.take<long long>(nring);
    const size_t o_chirp = Lo.take<double2>(nphi), o_bk = Lo.take<double2>(Mb);
    const size_t o_tw = Lo.take<double2>(Mb);
    const size_t o_H = Lo.take<double2>((size_t)(2 * lmax + 1) * nring);
    if (Lo.off > CUNUSHT_NOALLOC_SCRATCH_BYTES) {
        set_error("no-alloc synthesis needs %zu bytes of scratch, above the %u-byte array", Lo.off,
                  (unsigned)CUNUSHT_NOALLOC_SCRATCH_BYTES);
        return CUNUSHT_ERR_UNSUPPORTED;
    }
    void *base = nullptr;
    RC_TRY(scratch_address(&base));
    char *b = (char *)base;
    P.d_coef[spin] = (double *)(b + o_coef);
    P.d_lg0[spin] = (double *)(b + o_lg);
    P.d_gl_x = (double *)(b + o_px);
    P.d_gl_sh = (double *)(b + o_psh);
    P.d_gl_ch = (double *)(b + o_pch);
    P.d_gl_rn = (int *)(b + o_prn);
    P.d_gl_rs = (int *)(b + o_prs);
    P.d_ring_phi0 = (double *)(b + o_phi0);
    P.d_ring_nph = (long long *)(b + o_nph);
    P.d_ring_ofs = (long long *)(b + o_ofs);
    P.d_chirp = (double2 *)(b + o_chirp);
    P.d_bker = (double2 *)(b + o_bk);
    P.d_tw64 = (double2 *)(b + o_tw);
    double2 *H = (double2 *)(b + o_H);
    NoallocTables Tb{P.d_lg0[spin], P.d_gl_x, P.d_gl_sh, P.d_gl_ch, P.d_ring_phi0, P.d_gl_rn, P.d_gl_rs,
                     P.d_ring_nph, P.d_ring_ofs, P.d_chirp, P.d_bker, P.d_tw64};
    k_noalloc_tables<<<64, 256, 0, st>>>(R, Tb);
    CU_LAUNCH_CHECK();

    // every scratch piece read below is fully rewritten by this call
    RC_TRY(build_coef_tables_spin(&P, spin, P.d_coef[spin], st));
    RC_TRY(fft_global_f64(P.d_bker, Mb, -1, P.d_tw64, P.TW, st));
    const double2 *G = (const double2 *)alm;
    const double2 *C = ncomp > 1 ? G + P.nalm : nullptr;
    RC_TRY(leg_synth(&P, spin, G, C, false, false, H, st));
    RC_TRY(ring_synth(&P, spin, H, map, spin ? map + P.npix : nullptr, st));
    return CUNUSHT_OK;
}

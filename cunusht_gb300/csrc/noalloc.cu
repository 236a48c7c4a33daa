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

static double lg0_start(int m, int s) {
    const int l0 = m > s ? m : s;
    const double v = std::log((2.0 * l0 + 1.0) / (4.0 * PI)) + std::lgamma(2.0 * l0 + 1.0) -
                     std::lgamma(m + s + 1.0) - std::lgamma(std::fabs((double)(m - s)) + 1.0);
    return 0.5 * v / std::log(2.0);
}

template <typename T>
static int put(void *base, size_t off, const std::vector<T> &h, cudaStream_t st) {
    if (h.empty()) return CUNUSHT_OK;
    CU_TRY(cudaMemcpyAsync((char *)base + off, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return CUNUSHT_OK;
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

    // host tables: ring pairs (theta, pi - theta), start normalisations, Bluestein chirp
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
    std::vector<double> px, psh, pch;
    std::vector<int> prn, prs;
    for (int i = 0, j = nring - 1; i <= j; ++i, --j) {
        const double tn = ring_theta[idx[i]], ts = ring_theta[idx[j]];
        ARG_CHECK(std::fabs(tn + ts - PI) <= 1e-9, "no-alloc synthesis: rings must be north/south symmetric");
        px.push_back(std::cos(tn));
        psh.push_back(std::sin(0.5 * tn));
        pch.push_back(std::cos(0.5 * tn));
        prn.push_back(idx[i]);
        prs.push_back(idx[j]);
    }
    P.gl_npairs = (int)px.size();
    std::vector<double> lg(lmax + 1), phi0(ring_phi0, ring_phi0 + nring);
    for (int m = 0; m <= lmax; ++m) lg[m] = lg0_start(m, spin);
    std::vector<long long> nph(nring, nphi), ofs(nring);
    for (int i = 0; i < nring; ++i) ofs[i] = (long long)i * nphi;
    int Mb = 1;
    while (Mb < 2 * nphi - 1) Mb <<= 1;
    P.Mb = Mb;
    P.TW = Mb;
    std::vector<double2> chirp(nphi), bk(Mb, make_double2(0.0, 0.0)), tw(Mb);
    for (int q = 0; q < nphi; ++q) {
        const long long qq = ((long long)q * q) % (2LL * nphi);
        const double a = PI * (double)qq / nphi;
        chirp[q] = make_double2(std::cos(a), std::sin(a));
    }
    for (int k = 0; k < nphi; ++k) {
        const double2 b = make_double2(chirp[k].x / Mb, -chirp[k].y / Mb);
        bk[k] = b;
        if (k > 0) bk[Mb - k] = b;
    }
    for (int t = 0; t < Mb; ++t) {
        const long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)Mb;
        tw[t] = make_double2((double)std::cos(a), (double)std::sin(a));
    }

    // scratch layout (the limits above keep it below CUNUSHT_NOALLOC_SCRATCH_BYTES)
    ScratchLayout Lo;
    const size_t o_coef = Lo.take<double>(3 * (size_t)P.nalm);
    const size_t o_lg = Lo.take<double>(lg.size());
    const size_t o_px = Lo.take<double>(px.size()), o_psh = Lo.take<double>(psh.size());
    const size_t o_pch = Lo.take<double>(pch.size());
    const size_t o_prn = Lo.take<int>(prn.size()), o_prs = Lo.take<int>(prs.size());
    const size_t o_phi0 = Lo.take<double>(phi0.size());
    const size_t o_nph = Lo.take<long long>(nph.size()), o_ofs = Lo.take<long long>(ofs.size());
    const size_t o_chirp = Lo.take<double2>(chirp.size()), o_bk = Lo.take<double2>(bk.size());
    const size_t o_tw = Lo.take<double2>(tw.size());
    const size_t o_H = Lo.take<double2>((size_t)(2 * lmax + 1) * nring);
    if (Lo.off > CUNUSHT_NOALLOC_SCRATCH_BYTES) {
        set_error("no-alloc synthesis needs %zu bytes of scratch, above the %u-byte array", Lo.off,
                  (unsigned)CUNUSHT_NOALLOC_SCRATCH_BYTES);
        return CUNUSHT_ERR_UNSUPPORTED;
    }
    void *base = nullptr;
    RC_TRY(scratch_address(&base));
    char *b = (char *)base;
    RC_TRY(put(base, o_lg, lg, st));
    RC_TRY(put(base, o_px, px, st));
    RC_TRY(put(base, o_psh, psh, st));
    RC_TRY(put(base, o_pch, pch, st));
    RC_TRY(put(base, o_prn, prn, st));
    RC_TRY(put(base, o_prs, prs, st));
    RC_TRY(put(base, o_phi0, phi0, st));
    RC_TRY(put(base, o_nph, nph, st));
    RC_TRY(put(base, o_ofs, ofs, st));
    RC_TRY(put(base, o_chirp, chirp, st));
    RC_TRY(put(base, o_bk, bk, st));
    RC_TRY(put(base, o_tw, tw, st));
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

    // every scratch piece read below is fully rewritten by this call
    RC_TRY(build_coef_tables_spin(&P, spin, P.d_coef[spin], st));
    RC_TRY(fft_global_f64(P.d_bker, Mb, -1, P.d_tw64, P.TW, st));
    const double2 *G = (const double2 *)alm;
    const double2 *C = ncomp > 1 ? G + P.nalm : nullptr;
    RC_TRY(leg_synth(&P, spin, G, C, false, false, H, st));
    RC_TRY(ring_synth(&P, spin, H, map, spin ? map + P.npix : nullptr, st));
    return CUNUSHT_OK;
}

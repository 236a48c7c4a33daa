/*
 * cunusht_gb300 -- C ABI of the GB300 (sm_103a) non-uniform spherical harmonic
 * transform / CMB lensing engine.
 *
 * Every entry point returns an int status (CUNUSHT_OK == 0) and never
 * synchronises the device implicitly: work is enqueued on the caller's
 * ``stream`` (a cudaStream_t passed as void*, NULL = legacy default stream).
 * All array arguments are DEVICE pointers unless stated otherwise.  A failed
 * call leaves a human-readable message in cunusht_last_error().
 *
 * Conventions (same as the reference, Sebastian-Belkner/cunuSHT):
 *   alm      healpy m-major layout, idx(l,m) = m(2 lmax+1-m)/2 + l
 *            (cunusht/utils.py:58); complex128 or complex64 interleaved.
 *            A spin-s (s>0) field is ncomp consecutive alm arrays (G[, C]),
 *            i.e. E[, B] for s = 2; s_a_lm = -(G_lm + i C_lm).
 *   loc      points; layout 0 = (npts, 2) rows of (theta, phi) as nusht2d2's
 *            ``loc`` (GPU_nufft_transformer.py:386), layout 1 = (2, npts)
 *            planar (theta block then phi block) as ``ptg``
 *            (GPU_nufft_transformer.py:344-351).
 *   maps     spin 0: npts reals.  spin s>0: (2, npts) planar (Q block, U block).
 *   dtype    CUNUSHT_F64 (float64 / complex128) or CUNUSHT_F32 (float32 /
 *            complex64).
 */
#ifndef CUNUSHT_GB300_H
#define CUNUSHT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUNUSHT_OK 0
#define CUNUSHT_ERR_ARG 1         /* bad argument (sizes, layout, spin ...) */
#define CUNUSHT_ERR_CUDA 2        /* a CUDA runtime call or kernel launch failed */
#define CUNUSHT_ERR_ALLOC 3       /* device allocation failed */
#define CUNUSHT_ERR_UNSUPPORTED 4 /* valid request outside what this build supports */

#define CUNUSHT_F64 0
#define CUNUSHT_F32 1

#define CUNUSHT_PREC_AUTO 0  /* eps > 1e-6 -> FP32 FFT/nuFFT, else FP64 */
#define CUNUSHT_PREC_FP64 1  /* plain FP64 everywhere */
#define CUNUSHT_PREC_MIXED 2 /* split-precision Legendre + FP32/FP64 rest */

typedef struct cunusht_plan_s cunusht_plan_t;

/* Last error message of the calling thread ("" when none). */
const char *cunusht_last_error(void);

/* ABI version (major*10000 + minor*100 + patch). */
int cunusht_version(void);

/*
 * Plan = the transformer state of GPU_cufinufft_transformer.__init__ /
 * plan (cunusht/deflection/GPU_nufft_transformer.py:108-173, :227-246):
 * band limit, accuracy, the pointing (output) ring geometry, the doubled
 * Clenshaw-Curtis torus, nuFFT kernel and all device workspace.  All
 * device memory of the plan is allocated here, none per call.
 *   ring_*   host arrays of the pointing geometry (Geom, geometry.py:29-57):
 *            colatitude, first longitude, pixels per ring, first pixel.
 *   max_spin largest spin the plan will be asked for (0, 1 or 2).
 */
int cunusht_plan_create(cunusht_plan_t **plan, int lmax, double epsilon, int precision,
                        int max_spin, int nring, const double *ring_theta,
                        const double *ring_phi0, const int64_t *ring_nph,
                        const int64_t *ring_ofs);
int cunusht_plan_destroy(cunusht_plan_t *plan);

/*
 * Per-stage timing.  When enabled, every stage launch of this plan is
 * bracketed by CUDA events recorded on the caller's stream (no extra
 * synchronisation); cunusht_plan_stage_times waits for the recorded events,
 * returns per stage the summed milliseconds and launch counts since the last
 * query, and resets them.  Replaces the reference's timing_decorator /
 * execmode='timing' (cunusht/helper_GPU.py:10-51), which synchronised the
 * device around every stage.
 */
#define CUNUSHT_STAGE_LEG_SYNTH 0    /* Legendre synthesis, CC rings      */
#define CUNUSHT_STAGE_THETA_FWD 1    /* theta pass (FFT, deconv, pad, iFFT) */
#define CUNUSHT_STAGE_PHI_FWD 2      /* phi pass to the fine grid          */
#define CUNUSHT_STAGE_INTERP 3       /* nuFFT interpolation (type 2)       */
#define CUNUSHT_STAGE_SPREAD 4       /* nuFFT spreading (type 1)           */
#define CUNUSHT_STAGE_PHI_ADJ 5      /* adjoint phi pass                   */
#define CUNUSHT_STAGE_THETA_ADJ 6    /* adjoint theta pass                 */
#define CUNUSHT_STAGE_LEG_ADJ 7      /* Legendre adjoint, CC rings         */
#define CUNUSHT_STAGE_PTG_LEG 8      /* spin-1 Legendre on pointing rings  */
#define CUNUSHT_STAGE_PTG_RING 9     /* ring (phi) transform, pointing     */
#define CUNUSHT_STAGE_PTG_ROT 10     /* pointing rotation                  */
#define CUNUSHT_NSTAGE 11
int cunusht_plan_set_profiling(cunusht_plan_t *plan, int enable);
int cunusht_plan_stage_times(cunusht_plan_t *plan, double *ms, int64_t *count, int nstage);

/*
 * Largest m of the alm arrays the plan's calls take and return (healpy
 * m-major layout truncated at mmax, nalm = (mmax+1)(mmax+2)/2 +
 * (mmax+1)(lmax-mmax)); default lmax.  One value for every alm argument of
 * the plan (gclm, dlm_scaled, outputs).  The reference's GPU transformer
 * requires mmax == lmax (GPU_nufft_transformer.py:389-390); its CPU paths and
 * geometries take mmax <= lmax.
 */
int cunusht_plan_set_mmax(cunusht_plan_t *plan, int mmax);

/*
 * Transforms longer than 8192 points (theta / phi passes above lmax 2047,
 * Bluestein ring transforms above 4096 pixels per ring) run as two
 * half-length transforms split by output parity.  force = 1 selects that
 * split form for every transform of the plan, so that it can be checked
 * against the direct form at small sizes (the ring transforms then run
 * Bluestein, the form that has a split); force = 0 restores the automatic
 * choice.  No reference counterpart (the reference delegates its FFTs to
 * cuFFT / cuFINUFFT).
 */
int cunusht_plan_force_split(cunusht_plan_t *plan, int force);

/*
 * Ring transform of the pointing geometry (the phi FFT inside SHTns
 * synth_grad, GPU_sht_transformer.py:95).  method 0 (default): rings of one
 * length N <= 8192 whose prime factors are at most 13 (e.g. the 4095-pixel
 * Gauss-Legendre rings of lmax 2047, power-of-two rings) run a mixed-radix
 * FFT of N points; every other geometry runs Bluestein.  method 1: Bluestein
 * for every ring length (for comparisons).  cunusht_plan_ring_transform
 * returns 0 when the plan's rings run the mixed-radix form, 1 for Bluestein.
 */
int cunusht_plan_set_ring_transform(cunusht_plan_t *plan, int method);
int cunusht_plan_ring_transform(const cunusht_plan_t *plan);

/*
 * Recursion start states of the tensor-core Legendre kernels (mixed plans):
 * per ring, its first 16-l chunk outside the evanescent region and the
 * recursion state there, so that chunks in which no ring of a block
 * accumulates are skipped.  Built by cunusht_plan_create for the Gauss-Legendre
 * grid (grid 0: spins 0 .. max(max_spin, 1)) and the Clenshaw-Curtis grid
 * (grid 1: spins 0 .. max_spin), 84 MB each at lmax 2047.  enable = 0
 * releases one table: its kernels then start every ring at l = max(m, s)
 * (the same result, no chunk skipped); enable = 1 builds it again
 * (allocates).  Synchronises the device.  No reference counterpart.
 */
int cunusht_plan_set_start_states(cunusht_plan_t *plan, int grid, int spin, int enable);

/*
 * Mixed precision: the Legendre synthesis (CC synthesis of spin 0 / 1 / 2
 * maps, the deflection synthesis of dlm2pointing, the ring synthesis of the
 * SHT-only mode) runs on the tensor cores (exact integer-digit bf16 products
 * accumulated in tensor memory, enable = 1, the default) or on the CUDA
 * cores in double-float (enable = 0).
 * Both replace the SHTns synthesis of the reference
 * (cunusht/sht/GPU_sht_transformer.py:56-62, :88-97); the switch exists so
 * that the two can be checked against each other.
 */
int cunusht_plan_set_tensor_cores(cunusht_plan_t *plan, int enable);

/*
 * Spreading of the type-1 nuFFT (nusht2d1, lenmap2gclm, the delensing batch),
 * the options cuFINUFFT's gpu_method / gpu_sort set in the reference's plan
 * (GPU_nufft_transformer.py:242-246):
 *   method 0  warp strips (default): neighbouring points in neighbouring
 *             threads share shared-memory strips -- the ring-ordered pointing
 *             of a lensing solve; scattered points fall back to global atomics;
 *   method 1  bin-sorted: points counted into 32 x 32-cell bins of the fine
 *             grid, scattered into bin order, one block per bin accumulating
 *             a shared-memory tile -- points in any order (up to max_points per
 *             request, 0 = the plan's pixel count; more points use method 0);
 *   deterministic 1: the grid sums are accumulated in int64 fixed point (exact,
 *             so independent of the order of the atomics) and converted after;
 *             the same inputs then give bit-identical grids run after run,
 *             alone or batched.
 * Allocates the option's workspace (grown by cunusht_plan_reserve_batch).
 */
int cunusht_plan_set_spreading(cunusht_plan_t *plan, int method, int deterministic, int64_t max_points);

/*
 * Device status word of the plan, read after the plan's work so far has
 * finished (device-wide synchronisation) and then cleared: 0 = fine; bit 0 =
 * a bounded wait inside a tensor-core kernel ran out (the kernel gave up,
 * its outputs are not valid).  No reference counterpart.
 */
int cunusht_plan_device_status(cunusht_plan_t *plan, int *status);

/*
 * Tensor-core self test: a 128 x n x 32 product of integer matrices
 * (n = 16, 32 or 64, entries |.| <= 128) accumulated reps times (1..16, sums
 * below 2^24) through the descriptors, tensor-memory accumulation and
 * read-back path of the tensor-core Legendre kernel, on the current device.
 * mode 0: entries of both signs; 1: entries in [64, 128]; 2: one large
 * product per output among small ones; 3: no product is issued and the
 * completion wait is limited to 64 polls, so it runs out on purpose (the
 * kernel's timeout path: status set, tensor memory released, nothing read;
 * the context stays usable); 4, 5, 6: one 128 x n x 32 product (reps unused)
 * with A and B, A only, or B only stored MN-major (transposed operands, the
 * layout of the tensor-core adjoint).  *maxerr = largest |result - exact| (0 when the
 * accumulation is exact), *timeout = 1 if the completion wait ran out.  No
 * reference counterpart.
 */
int cunusht_tc_selftest(int n, int reps, int mode, double *maxerr, int *timeout);

/* Plan sizes: info[0]=npix, [1]=torus theta length, [2]=torus phi length,
 * [3]=fine grid theta length, [4]=fine grid phi length, [5]=kernel width,
 * [6]=fine rows stored, [7]=workspace bytes, [8]=precision in use,
 * [9]=nalm.  Returns the number of entries written. */
int cunusht_plan_info(const cunusht_plan_t *plan, int64_t *info, int ninfo);

/*
 * nusht2d2: alm -> values at arbitrary points (type-2 direction).
 * Replaces GPU_cufinufft_transformer.nusht2d2
 * (cunusht/deflection/GPU_nufft_transformer.py:386-435: SHTns CC synthesis,
 * doubling, cuFFT fft2, cuFINUFFT type 2).  gamma (may be NULL) is the
 * polarisation rotation angle per point; when given and spin>0 the output is
 * multiplied by exp(i spin gamma) (CPU_nufft_transformer.py:356-368).
 */
int cunusht_nusht2d2(cunusht_plan_t *plan, int spin, int ncomp, const void *alm, int alm_dtype,
                     const double *loc, int64_t npts, int loc_layout, const double *gamma,
                     void *out, int out_dtype, void *stream);

/*
 * nusht2d1: values at arbitrary points -> alm, the exact adjoint of
 * cunusht_nusht2d2 (real map inner product, alm inner product with m>0
 * counted twice).  Replaces GPU_cufinufft_transformer.nusht2d1
 * (GPU_nufft_transformer.py:439-484: cuFINUFFT type 1, ifft2, adjoint
 * doubling, SHTns analysis of map*iw).  gamma (may be NULL) applies
 * exp(-i spin gamma) first.
 */
int cunusht_nusht2d1(cunusht_plan_t *plan, int spin, int ncomp, const void *map, int map_dtype,
                     const double *loc, int64_t npts, int loc_layout, const double *gamma,
                     void *alm_out, int alm_dtype, void *stream);

/*
 * Served form: nreq lensing solves (dlm2pointing + nusht2d2 with the
 * exp(i spin gamma) rotation, i.e. GPU_cufinufft_transformer.gclm2lenmap,
 * GPU_nufft_transformer.py:487-578) of one lmax / spin / accuracy in one
 * pass of batched launches.  The mixed-precision Legendre kernels share one
 * recursion between the requests of a launch: up to eight on the tensor cores
 * (as many as cunusht_plan_reserve_batch reserved window records for: 1, 2, 4
 * or 8), up to four on the CUDA cores.  Arrays are contiguous per request:
 * gclm (nreq, ncomp, nalm) complex128, dlm_scaled / dclm_scaled (nreq, nalm)
 * complex128 (dclm may be NULL), out (nreq, spin ? 2 : 1, npix); ptg
 * (nreq, 2, npix) and gamma (nreq, npix) receive the pointing when not NULL.
 * cunusht_plan_reserve_batch allocates the per-request workspace once
 * (nreq <= max_batch); the batched call itself allocates nothing.
 */
int cunusht_plan_reserve_batch(cunusht_plan_t *plan, int max_batch);
int cunusht_lensing_batch(cunusht_plan_t *plan, int nreq, int spin, int ncomp, const void *gclm,
                          const void *dlm_scaled, const void *dclm_scaled, double *ptg, double *gamma,
                          void *out, int out_dtype, void *stream);

/*
 * Served form of the adjoint: nreq delensing solves (dlm2pointing + nusht2d1
 * with the exp(-i spin gamma) rotation, i.e. GPU_cufinufft_transformer.
 * lenmap2gclm, GPU_nufft_transformer.py:581-673) of one lmax / spin /
 * accuracy in one batched pass; the mixed-precision Legendre kernels share one
 * recursion between up to four requests.  lenmap (nreq, spin ? 2 : 1, npix)
 * float64 / float32; dlm_scaled / dclm_scaled (nreq, nalm) complex128 (dclm
 * may be NULL); alm_out (nreq, ncomp, nalm) complex128; ptg (nreq, 2, npix)
 * and gamma (nreq, npix) receive the pointing when not NULL.  Needs
 * cunusht_plan_reserve_batch(plan, >= nreq).  No reference counterpart as a
 * batch.
 */
int cunusht_delensing_batch(cunusht_plan_t *plan, int nreq, int spin, int ncomp, const void *lenmap, int map_dtype,
                            const void *dlm_scaled, const void *dclm_scaled, double *ptg, double *gamma,
                            void *alm_out, void *stream);

/*
 * dlm2pointing: deflected angles of every pixel of the plan geometry.
 * Replaces GPU_cufinufft_transformer.dlm2pointing / deflection.dlm2pointing
 * (GPU_nufft_transformer.py:64-104, :344-351: SHTns synth_grad on the GL
 * grid + compute_pointing_1Dto1D_lowmem, pointing.cu:197-255).
 *   dlm_scaled   complex alm of the lensing potential (dlm / sqrt(l(l+1)))
 *   dclm_scaled  curl potential (may be NULL)
 *   ptg          out (2, npix) planar: theta' block then phi' block
 *   gamma        out npix rotation angle (may be NULL), CPU_nufft_transformer.py:158-160
 */
int cunusht_dlm2pointing(cunusht_plan_t *plan, const void *dlm_scaled, const void *dclm_scaled,
                         int alm_dtype, double *ptg, double *gamma, void *stream);

/*
 * Continuous-batching lensing server (the served form's host scheduler; the
 * reference has no serving layer).  Requests of any lmax (GL grid, nphi
 * pixels per ring, 0 = 2 lmax + 1), spin and accuracy are queued per bucket;
 * each bucket gets slots (plan + batch workspace + stream) when its measured
 * device memory fits the HBM budget; cunusht_server_poll() retires finished
 * launches and launches queued requests on idle slots, batching up to the
 * bucket's requests-per-launch through cunusht_lensing_batch /
 * cunusht_delensing_batch replayed as CUDA graphs.
 *   direction 0 (gclm2lenmap): input gclm (spin ? 2 : 1, nalm) complex128,
 *     output (spin ? 2 : 1, npix) float64;
 *   direction 1 (lenmap2gclm): input lensed map (spin ? 2 : 1, npix) float64,
 *     output (spin ? 2 : 1, nalm) complex128;
 *   dlm_scaled (nalm) complex128.  All device pointers, owned by the caller
 *   and valid until the request id is returned by cunusht_server_poll; inputs
 *   are read after the work already queued on producer_stream.
 * One host thread drives a server.  Default policy: lmax >= 4095: 1 request
 * per launch, 1 slot; >= 2047: 4, 2; else 8, 2 (cunusht_server_set_policy).
 * cunusht_server_stats: [launches, completed, bytes in use, buckets, slots,
 * refused admissions, evicted buckets].  A bucket that does not fit releases
 * idle buckets (empty queue, nothing in flight), least recently used first
 * and only as many as it needs once its size is known, or none, and waits.
 * cunusht_server_prewarm: admits the bucket (lmax, spin, eps, nphi) ahead of
 * traffic and captures the graphs of both directions and every batch size up
 * to its requests per launch on each of its slots (one eager run and one
 * capture each, on zeroed inputs), so that no launch of the served stream
 * pays for a capture; *admitted = 0 when the bucket does not fit the budget.
 * Returns after the device has finished the warm-up work.
 */
typedef struct cunusht_server_s cunusht_server_t;
int cunusht_server_create(cunusht_server_t **server, double hbm_budget_bytes, int precision);
int cunusht_server_set_policy(cunusht_server_t *server, int lmax, int requests_per_launch, int slots);
int cunusht_server_submit(cunusht_server_t *server, int direction, int lmax, int spin, double eps, int nphi,
                          const void *input, const void *dlm_scaled, void *output, void *producer_stream,
                          int64_t *request_id);
int cunusht_server_poll(cunusht_server_t *server, int64_t *done_ids, int max_ids, int *ndone, int *pending);
int cunusht_server_stats(cunusht_server_t *server, double *stats, int n);
int cunusht_server_prewarm(cunusht_server_t *server, int lmax, int spin, double eps, int nphi, int *admitted);
int cunusht_server_destroy(cunusht_server_t *server);

/*
 * Determinant of the magnification matrix of a deflection field on the plan's
 * pointing geometry (helper_GPU.py:113-161 dlm2A): A (npix, float64) from the
 * gradient deflection alm dlm = sqrt(l(l+1)) phi_lm (NOT dlm_scaled) and the
 * optional curl dclm (may be NULL), via spin-0 convergence, spin-2 shear,
 * spin-1 deflection (and spin-0 rotation) syntheses.  Used to weight lensed
 * maps for inverse lensing (GPU_nufft_transformer.py:586).
 */
int cunusht_dlm2A(cunusht_plan_t *plan, const void *dlm, const void *dclm, int alm_dtype, double *A,
                  void *stream);

/*
 * Exact spin-s synthesis at arbitrary points by direct FP64 summation,
 * O(lmax^2) per point (one block per point): the remapped field at selected
 * pixels, gclm2lenpixs (CPU_nufft_transformer.py:531-558), as an on-device
 * spot check of nusht2d2.  alm (ncomp, nalm); loc as cunusht_nusht2d2; out
 * (npts) spin 0 or (2, npts) Q, U with the optional exp(i spin gamma) rotation.
 */
int cunusht_synth_points(cunusht_plan_t *plan, int spin, int ncomp, const void *alm, int alm_dtype,
                         const double *loc, int64_t npts, int loc_layout, const double *gamma, double *out,
                         void *stream);

/*
 * Vector-Jacobian product of the spin-0 lensing map with respect to the
 * scaled lensing potential: for lenmap = gclm2lenmap(gclm, dlm_scaled) and a
 * map gradient g = dL/dlenmap (npix float64), returns grad_dlm (complex128,
 * nalm) = sqrt(l(l+1)) x spin-1 adjoint synthesis of J^T (g grad f), with f the
 * unlensed field and J the Jacobian of the pointing rotation
 * (pointing.cu:210-213).  Same alm inner-product convention as
 * cunusht_nusht2d1 (m > 0 counted twice).  Backward of the differentiable
 * gclm2lenmap; the reference has no gradient path.  Spin 0 only.
 */
int cunusht_lensing_vjp_dlm(cunusht_plan_t *plan, int spin, const void *gclm, int alm_dtype,
                            const void *dlm_scaled, int dlm_dtype, const double *grad_map,
                            void *grad_dlm, void *stream);

/*
 * Spin-s synthesis / adjoint synthesis on the plan's ring geometry (SHT-only
 * mode; GPU_cufinufft_transformer.synthesis / adjoint_synthesis,
 * GPU_nufft_transformer.py:356-383).  maps as above (npix or 2 x npix, FP64).
 * The adjoint has no quadrature weights (adjoint, not analysis).
 */
int cunusht_synthesis(cunusht_plan_t *plan, int spin, int ncomp, const void *alm, int alm_dtype,
                      double *map, void *stream);
int cunusht_adjoint_synthesis(cunusht_plan_t *plan, int spin, int ncomp, const double *map,
                              void *alm_out, int alm_dtype, void *stream);

/*
 * Analysis on the plan's ring geometry: the adjoint synthesis of the map
 * weighted per ring by ring_weight (DEVICE array, nring entries: the
 * quadrature weight of one pixel of that ring, e.g. Gauss-Legendre weight x
 * 2 pi / nphi), so that on a Gauss-Legendre grid with nring >= lmax + 1 and
 * nphi >= 2 lmax + 1 it inverts cunusht_synthesis exactly.  Replaces the
 * SHTns analys of the reference's SHT-only mode (GPU_SHTns_transformer.
 * analysis / adjoint_synthesis_cupy / map2alm, GPU_sht_transformer.py:65-73,
 * :99-127; with iw = 1 / w the weighted adjoint of GPU_nufft_transformer.py:
 * 265-269 is cunusht_adjoint_synthesis).  Maps as cunusht_adjoint_synthesis.
 */
int cunusht_analysis(cunusht_plan_t *plan, int spin, int ncomp, const double *map, const double *ring_weight,
                     void *alm_out, int alm_dtype, void *stream);

/*
 * Raw pointing rotation/*
 * Raw pointing rotation (compute_pointing_1Dto1D_lowmem, pointing.cu:197-226):
 * per pixel of a ring geometry, deflected (theta', phi') from the spin-1
 * deflection maps (d_theta, d_phi) in ring-major pixel order; gamma optional.
 * Ring tables are DEVICE arrays here (as the reference binding takes them).
 */
int cunusht_pointing(int nring, const double *ring_theta, const double *ring_phi0,
                     const int64_t *ring_nph, const int64_t *ring_ofs, int64_t npix,
                     const double *spin1_theta, const double *spin1_phi, double *out_theta,
                     double *out_phi, double *out_gamma, void *stream);

/*
 * Map doubling to the 2 pi theta torus and its adjoint.
 * cunusht_doubling replaces CUdoubling_contig_1D (layout 1, theta-contiguous
 * (nphi, ntheta) in, (nphi, 2 ntheta - 2) out; doubling.cu:180-220) and
 * CUdoubling_1D (layout 0, ring-major (ntheta, nphi) in, (2 ntheta - 2, nphi)
 * out; doubling.cu:137-178).  cunusht_adjoint_doubling replaces
 * CUadjoint_doubling_1D (ring-major (2 ntheta - 2, nphi) in, (ntheta, nphi)
 * out; doubling.cu:53-92).  spin odd negates the mirrored half
 * (CPU_nufft_transformer.py:284-318).  nphi must be even.
 */
int cunusht_doubling(const void *cc_map, int64_t ntheta, int64_t nphi, int layout, int spin,
                     int dtype, void *out, void *stream);
int cunusht_adjoint_doubling(const void *dmap, int64_t ntheta, int64_t nphi, int spin, int dtype,
                             void *out, void *stream);

/*
 * Spin-s synthesis on a small ring geometry that allocates no device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- code running inside another framework's memory pool, which
 * owns all device memory, latency-critical pipelines that forbid allocation
 * after start-up (cudaMalloc can synchronise the device), and plugin hosts
 * that give a plugin no allocator.  The caller passes the alm (complex128,
 * device, ncomp x nalm) and the output map (device, npix or 2 x npix float64,
 * ring i at pixels [i nphi, (i + 1) nphi)); ring colatitudes and first
 * longitudes are host arrays and the rings must be north/south symmetric;
 * they are read on the host and reach the device as a kernel parameter, so
 * the call makes no host-to-device copy and does not block the host.
 * Every intermediate lives in one file-scope device array of
 * CUNUSHT_NOALLOC_SCRATCH_BYTES that each GPU loading the library holds until
 * the process exits; sizes beyond the CUNUSHT_NOALLOC_MAX_* limits are
 * rejected with CUNUSHT_ERR_ARG.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current; make
 * that first call before any stream capture.  The address is kept per device
 * for the life of the process: a cudaDeviceReset between calls is not
 * supported.  All calls share the one array, so calls that overlap on the GPU
 * (different streams or host threads) race.  Same math as cunusht_synthesis;
 * nothing is allocated and nothing freed.
 */
#define CUNUSHT_NOALLOC_SCRATCH_BYTES (4u * 1024u * 1024u)
#define CUNUSHT_NOALLOC_MAX_LMAX 255
#define CUNUSHT_NOALLOC_MAX_NRING 256
#define CUNUSHT_NOALLOC_MAX_NPHI 1024
int cunusht_synthesis_noalloc(int lmax, int spin, int ncomp, const void *alm, int nring,
                              const double *ring_theta, const double *ring_phi0, int nphi,
                              double *map, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CUNUSHT_GB300_H */

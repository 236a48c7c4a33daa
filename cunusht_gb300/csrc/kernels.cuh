// Host-side launchers shared between the translation units of the library.
#pragma once
#include "common.cuh"

namespace cunusht {

constexpr int FFT_TPB = 512;

// capi.cu: device allocation counted in the plan's workspace bytes
int plan_alloc(cunusht_plan_s *P, void **p, size_t bytes);

// ring_mr.cu: mixed-radix ring transforms of uniform rings
int ring_mr_init(cunusht_plan_s *P);
bool ring_mr_available(const cunusht_plan_s *P);
int ring_synth_mr_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *Hgl, long long hbs, double *out0,
                        double *out1, long long obs, cudaStream_t st);

// capi.cu: Gauss-Legendre nodes x (descending cos theta) and weights, Newton iteration
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w);

// legendre.cu
int build_coef_tables(cunusht_plan_s *P, cudaStream_t st);
int build_coef_tables_df(cunusht_plan_s *P, cudaStream_t st);
int build_coef_tables_spin(const cunusht_plan_s *P, int spin, double *coef, cudaStream_t st);
int leg_synth(const cunusht_plan_s *P, int spin, const double2 *G, const double2 *C,
              bool use_lfac, bool cc, double2 *H, cudaStream_t st);
int leg_synth_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *G, const double2 *C,
                    long long astride, bool use_lfac, bool cc, double2 *H, long long hstride, cudaStream_t st);
int leg_synth_batch_fl(const cunusht_plan_s *P, int nreq, int spin, const double2 *G, const double2 *C,
                       long long astride, const double *fl, bool cc, double2 *H, long long hstride, cudaStream_t st);
int synth_points(const cunusht_plan_s *P, int spin, const double2 *G, const double2 *C, long long npts,
                 const double *loc, int layout, const double *gamma, double *out, cudaStream_t st);
// scratch (may be NULL): free device workspace of scratch_bytes; the tensor-core
// adjoint keeps its fixed-point sums there (adj_tc_scratch_bytes), else the
// CUDA-core kernels run
int leg_adjoint(const cunusht_plan_s *P, int spin, int ncomp, const double2 *H, bool use_lfac,
                bool cc, double2 *G, double2 *C, cudaStream_t st, void *scratch = nullptr, size_t scratch_bytes = 0);
int leg_adjoint_batch(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                      bool use_lfac, bool cc, double2 *G, double2 *C, long long astride, cudaStream_t st,
                      void *scratch = nullptr, size_t scratch_bytes = 0);
int leg_adj_pole_pair_spin(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                           int ld, const double *lf, int rn, int rs, double2 *G, double2 *C, long long astride,
                           cudaStream_t st);
int leg_adj_df_pairs(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                     int ld, int npairs, const double *x, const double *sh, const double *ch, const int *rn,
                     const int *rs, const double *lf, double2 *G, double2 *C, long long astride, cudaStream_t st);
// legendre_tc_adj.cu: tensor-core adjoint (mixed precision, every spin)
size_t adj_tc_scratch_bytes(const cunusht_plan_s *P, int nreq);
int leg_adjoint_tc(const cunusht_plan_s *P, int nreq, int spin, int ncomp, const double2 *H, long long hstride,
                   int ld, int npairs, const double *x, const double *sh, const double *ch, const int *rn,
                   const int *rs, int pole, int pole_rn, int pole_rs, const float4 *stv, const short2 *ste,
                   const double *lf, double2 *G, double2 *C, long long astride, void *scratch, cudaStream_t st);

// first chunk of a ring that never reaches the accumulated range (start tables, k_tc_starts)
constexpr short TC_NEVER = 32767;
// legendre_tc.cu: tensor-core synthesis (mixed precision, every spin), nb in {1, 2, 4, 8};
// stv / ste: the plan's recursion-start table of the grid and spin (row stride npairs), or NULL
int leg_synth_spin_tc(const cunusht_plan_s *P, int nb, int npairs, const double *x, const double *sh,
                      const double *ch, const int *rn, const int *rs, int ld, int pole, int pole_rn, int pole_rs,
                      const float4 *stv, const short2 *ste, int spin, const double2 *G,
                      const double2 *C, long long astride, const double *lf, double2 *H, long long hstride,
                      cudaStream_t st);
int tc_selftest(int nn, int reps, int mode, double *maxerr, int *timeout);
int tc_plan_init(cunusht_plan_s *P);  // window tables and record buffer of a mixed-precision plan
int tc_start_states(cunusht_plan_s *P, int grid, int spin, bool enable);  // build / release one start-state table
int tc_reserve(cunusht_plan_s *P, int nb);  // record buffer for launches of up to nb requests
// legendre.cu: double-float CUDA-core synthesis (spin > 0) of npairs ring pairs given by their tables
int leg_synth_spin_df_pairs(const cunusht_plan_s *P, int nb, int npairs, const double *x, const double *sh,
                            const double *ch, const int *rn, const int *rs, int ld, int spin, const double2 *G,
                            const double2 *C, long long astride, const double *lf, double2 *H, long long hstride,
                            cudaStream_t st);

// fft.cu
int theta_fwd(const cunusht_plan_s *P, int spin, const double2 *H, void *F, cudaStream_t st);
int theta_adj(const cunusht_plan_s *P, int spin, const void *F, double2 *H, cudaStream_t st);
int phi_fwd(const cunusht_plan_s *P, int spin, const void *F, void *U, cudaStream_t st);
int phi_adj(const cunusht_plan_s *P, int spin, const void *U, void *F, cudaStream_t st);
int phi_adj_batch(const cunusht_plan_s *P, int nreq, int spin, const void *U, long long ubs, void *F, long long fbs,
                  cudaStream_t st);
int theta_adj_batch(const cunusht_plan_s *P, int nreq, int spin, const void *F, long long fbs, double2 *H,
                    long long hbs, void *U, long long ubs_bytes, cudaStream_t st);
int ring_synth(const cunusht_plan_s *P, int spin, const double2 *Hgl, double *out0, double *out1,
               cudaStream_t st);
int theta_fwd_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *H, long long hbs, void *F,
                    long long fbs, cudaStream_t st);
int phi_fwd_batch(const cunusht_plan_s *P, int nreq, int spin, const void *F, long long fbs, void *U, long long ubs,
                  cudaStream_t st);
int ring_synth_batch(const cunusht_plan_s *P, int nreq, int spin, const double2 *Hgl, long long hbs, double *out0,
                     double *out1, long long obs, cudaStream_t st);
int ring_adjoint(const cunusht_plan_s *P, int spin, const double *in0, const double *in1,
                 double2 *Hgl, cudaStream_t st, const double *wring = nullptr);
int split_c128_to_df(const double2 *in, long long n, void *out, cudaStream_t st);
int fft_global_f64(double2 *data, int N, int dir, const double2 *tw, int TW, cudaStream_t st);
size_t fft_smem_bytes(int N, bool f32);

// nufft.cu
int nufft_interp(const cunusht_plan_s *P, int spin, const double *loc, long long npts,
                 int layout, const double *gamma, void *out, int out_dtype, cudaStream_t st);
int nufft_interp_batch(const cunusht_plan_s *P, int nreq, int spin, const void *U, long long ubs, const double *loc,
                       long long lbs, long long npts, int layout, const double *gamma, void *out, long long obs,
                       int out_dtype, cudaStream_t st);
int magnification_det(long long npix, const double *k, const double *g1, const double *g2, const double *d1,
                      const double *d2, const double *w, double *A, cudaStream_t st);
int pointing_batch(const cunusht_plan_s *P, int nreq, const double *d, long long dbs, double *ptg, long long pbs,
                   double *gamma, cudaStream_t st);
// spread_bins.cu: the plan's spreading options (bin-sorted path, deterministic
// fixed-point accumulation) around the warp-strip kernels of nufft_spread_batch
size_t bin_workspace_ints(const cunusht_plan_s *P, long long npts);
int spread_options_begin(const cunusht_plan_s *P, int nreq, int spin, void *U, long long ubs, const double *loc,
                         long long lbs, long long npts, int layout, const double *gamma, const void *in,
                         long long ibs, int in_dtype, int *done, cudaStream_t st);
int spread_options_end(const cunusht_plan_s *P, int nreq, int spin, void *U, long long ubs, long long npts,
                       cudaStream_t st);
int nufft_spread_batch(const cunusht_plan_s *P, int nreq, int spin, void *U, long long ubs, const double *loc,
                       long long lbs, long long npts, int layout, const double *gamma, const void *in, long long ibs,
                       int in_dtype, cudaStream_t st);
int nufft_spread(const cunusht_plan_s *P, int spin, const double *loc, long long npts,
                 int layout, const double *gamma, const void *in, int in_dtype,
                 cudaStream_t st);

// pointing.cu
int pointing_launch(int nring, const double *rth, const double *rph0, const long long *rnph,
                    const long long *rofs, long long npix, const double *dth, const double *dph,
                    double *out_th, double *out_ph, double *out_gamma, cudaStream_t st);
int pointing_mixed_launch(int nring, int nph_uniform, const double *rth, const float4 *rsc, const double *rph0,
                          const long long *rnph, const long long *rofs, long long npix, const double *dth,
                          const double *dph, double *out_th, double *out_ph, double *out_gamma, cudaStream_t st);
int lens_vjp_launch(const cunusht_plan_s *P, const double *ptg, const double *grad, double *gd, cudaStream_t st);
int doubling_launch(const void *in, long long ntheta, long long nphi, int layout, int spin,
                    int dtype, void *out, cudaStream_t st);
int adjoint_doubling_launch(const void *in, long long ntheta, long long nphi, int spin, int dtype,
                            void *out, cudaStream_t st);
int convert_alm(const void *in, int dtype, long long n, double2 *out, cudaStream_t st);
int store_alm(const double2 *in, long long n, int dtype, void *out, cudaStream_t st);

}  // namespace cunusht

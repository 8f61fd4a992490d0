// Device-side view of a context (passed by value to kernels) and kernel launchers.
#pragma once
#include "afq_common.cuh"

struct afq_ctx_dev {
  int norb, nchol, nw, n_exp_terms;
  double dt;
  int nslab;         // walker slabs: 1 restricted, 2 unrestricted
  int kslab[2];      // stored slab widths
  int nocc_slab[2];  // occupied columns used per slab (== kslab here)
  int kmax;          // max(kslab)
  int restricted_square;  // RHF trial with restricted walkers: overlap = det^2
  int nspin_g;       // Green blocks per walker: 1 (RHF: G or G_up+G_dn), 2 (UHF)
  int gocc[2];
  int ktot;          // (gocc0 + (nspin_g==2 ? gocc1 : 0)) * norb
  int energy_mode;   // 0 RHF restricted, 1 RHF two-slab, 2 UHF
  double h0, h0_prop_re, h0_prop_im;
  const double* trial[2];     // [norb, nocc_s]
  const double* exp_h1[2];    // [norb, norb] per slab
  const double* rot_chol[2];  // [nchol, gocc_s, norb]
  const double* rot_h1[2];    // [gocc_s, norb]
  const double2* mf;          // [nchol]
};

namespace afq {
// dynamic shared memory of the FP64 Green's-function / overlap kernel (k_green_overlap)
inline size_t green_f64_smem(int norb, int kmax) {
  return (size_t)norb * kmax * 16 + (size_t)kmax * 2 * kmax * 16 + (size_t)norb * kmax * 8;
}
// 0 when `smem` bytes fit the current device's opt-in shared-memory limit; otherwise the
// error text names `what` and the limit, and the return is -2
int check_smem_optin(size_t smem, const char* what);
template <typename WT>
int launch_green(const afq_ctx_dev& c, const void* wu, const void* wd, double2* green,
                 double2* ovl, bool write_green, cudaStream_t st);
int launch_gemm_cr(bool b_kn, int M, int N, int K, const double2* A, long lda, const double* B,
                   long ldb, double2* C, long ldc, double2 alpha, cudaStream_t st);
int launch_field_shifts(const afq_ctx_dev& c, const double* fields, const double2* fb,
                        double2* xt, double2* shift, double2* fbt, cudaStream_t st);
template <typename WT>
int launch_taylor_f64(const afq_ctx_dev& c, int w0, int nwc, const double2* vhs, void* wu, void* wd,
                      cudaStream_t st);
// shift / fbt: per-walker partial sums [nw][ntiles] (summed here)
// status (may be NULL): a device guard word folded into scalars[AFQ_S_STATUS]
int launch_weights(const afq_ctx_dev& c, const double2* shift, const double2* fbt, int ntiles,
                   const double2* ovl_new, double2* ovl, double* weights, double* scalars,
                   cudaStream_t st, const int* status = nullptr);
int launch_energy_f64(const afq_ctx_dev& c, int nchunks, int gchunk, const double2* green,
                      double2* epart, double2* energy, cudaStream_t st);
// rdiag (optional, [nslab][nw] complex): prod(diag R) per walker slab
template <typename WT>
int launch_qr(const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st, double2* rdiag = nullptr);
template <typename WT>
int launch_sr(const afq_ctx_dev& c, const double* zeta, double* weights, double* cum, int32_t* idx,
              void* wu, void* wd, void* wcopy, cudaStream_t st);
int launch_block_stats(const afq_ctx_dev& c, const double2* energy, const double* weights,
                       double* scalars, double* be, double* bw, cudaStream_t st);
int launch_phaseless_begin(double* scalars, cudaStream_t st);
int launch_clamped_energies(const afq_ctx_dev& c, const double2* energy, const double* scalars,
                            double* out, cudaStream_t st);
int launch_cs_outlier(double* w1, double* w2, const double* e1, const double* e2, int nw,
                      double z_thresh, double* sums, cudaStream_t st);
int launch_phaseless_end(int nblk, double denom, const double* be, const double* bw,
                         double* scalars, double* energy, cudaStream_t st);
int launch_driver_update(const afq_ctx_dev& c, const double* weights, const double* energy,
                         double* scalars, double* wsum, cudaStream_t st);
// free projection (afq_free.cu)
int launch_free_prep(const afq_ctx_dev& c, const double* fields, double ene0, double2* xt, double2* consts,
                     cudaStream_t st);
int launch_free_scale(const afq_ctx_dev& c, const double2* consts, void* wu, void* wd, cudaStream_t st);
int launch_free_finish(int nw, const double2* rdiag, double2* norms, double2* ovl, cudaStream_t st);
int launch_free_block_stats(int nw, const double2* energy, const double2* ovl, double2* be, double2* bw,
                            cudaStream_t st);
// CPMC, Hubbard on-site U (afq_cpmc.cu); mode 0: overlaps and Green's functions, 1: one step,
// 2: continuous fields, 3: one step with the nearest-neighbour interaction
int launch_cpmc(int norb, int n_up, int n_dn, int nw, double dt, double u, const double* exp_up,
                const double* exp_dn, const double* trial_up, const double* trial_dn, double* w_up, double* w_dn,
                double* weights, double* overlaps, double* greens, double* scalars, const double* gauss, int mode,
                cudaStream_t st, double u1 = 0.0, const int32_t* neighbors = nullptr, int npairs = 0,
                const double* uniforms = nullptr);
int launch_fill_normal(double* out, int64_t n, uint64_t seed, uint64_t offset, cudaStream_t st);
int launch_fill_uniform(double* out, int64_t n, uint64_t seed, uint64_t offset, cudaStream_t st);
}  // namespace afq

// Reverse-mode (adjoint) buffers and launchers of the FP64 phaseless block.
#pragma once
#include "afq_kernels.cuh"

namespace afq {

struct AdjointBufs {
  double2* wb[2];      // walker cotangent at the current point of the backward sweep
  double2* wb2[2];     // second walker cotangent (outputs of the Taylor, QR and SR adjoints)
  double* wbar;        // weight cotangent [nw]
  double2* lbar;       // pending log-overlap cotangent at the current point [nw]
  double2* lbar2;      // log-overlap cotangent at the start of the current step [nw]
  double2* gpend;      // pending G cotangent at the current point [nw][ktot]
  double2* gene;       // G cotangent of the local energy [nw][ktot]
  double2* fbb;        // force-bias cotangent [nw][nchol]
  double2* xtb;        // shifted-field cotangent [nw][nchol]
  double2* shb;        // [nw]
  double2* fbtb;       // [nw]
  double2* vbar;       // vhs cotangent [nw_chunk][norb^2]
  double2* tay;        // Taylor scratch [nw_chunk][2 M + 2][norb * (k0 + k1)], M = n_exp_terms - 1
  double* ebar;        // local-energy cotangent [nw]
  double* scal;        // [0]: cotangent of the population-control shift
  double* beb;         // block-energy cotangents [n blocks]
  double* bwb;         // block-weight cotangents [n blocks]
  double* gexp[2];     // outputs: d energy / d exp_h1 per slab [norb^2]
  double* grot[2];     // outputs: d energy / d rot_h1 per Green block [gocc * norb]
  // orbital rotation (NULL: not requested): d energy / d trial per Green block [norb][gocc]
  // and d energy / d rot_chol in the concatenated layout [nchol][ktot]
  double* gtrial[2];
  double* grc;
  // Cholesky-vector gradients (NULL: not requested): d energy / d chol [nchol][norb^2] (the
  // vhs contraction), d energy / d mf_shifts [nchol] complex (field shifts) and
  // d energy / d h0_prop (complex; from the weights, accumulated in scal[1])
  double* gchol;
  double2* gmf;
};

int a_launch_end(int nblk, const double* be, const double* bw, const AdjointBufs& a, cudaStream_t st);
int a_launch_block_stats(const afq_ctx_dev& c, const AdjointBufs& a, int blk, const double2* energy,
                         const double* weights, const double* scalars, const double* be, cudaStream_t st);
int a_launch_energy(const afq_ctx_dev& c, const AdjointBufs& a, const double2* green, cudaStream_t st);
// gt (may be NULL): the trial cotangents, accumulated (gtrial of AdjointBufs)
int a_launch_green(const afq_ctx_dev& c, const void* wu, const void* wd, const double2* ga, const double2* gb,
                   const double2* lbar, double2* wbu, double2* wbd, cudaStream_t st,
                   double* const* gt = nullptr);
// rot_chol cotangent of the force bias: grc += alpha Re(fb-bar^H G) (G of the step's start)
int a_launch_rc_fb(const afq_ctx_dev& c, const AdjointBufs& a, const double2* green, double alpha,
                   cudaStream_t st);
// rot_chol cotangent of the local energy at a measurement (G of the QR'd walkers)
int a_launch_rc_energy(const afq_ctx_dev& c, const AdjointBufs& a, const double2* green, cudaStream_t st);
int a_launch_qr(const afq_ctx_dev& c, const void* wold_u, const void* wold_d, const void* q_u, const void* q_d,
                const double2* qb_u, const double2* qb_d, double2* ob_u, double2* ob_d, cudaStream_t st);
int a_launch_weights(const afq_ctx_dev& c, const AdjointBufs& a, const double2* shift, const double2* fbt,
                     const double2* ovl_new, const double2* ovl, const double* w_start, const double* w_post,
                     const double* scalars, cudaStream_t st);
int a_launch_taylor(const afq_ctx_dev& c, const AdjointBufs& a, int w0, int nwc, const double2* vhs,
                    const void* wu, const void* wd, cudaStream_t st);
int a_launch_field(const afq_ctx_dev& c, const AdjointBufs& a, const double2* xt, cudaStream_t st);
int a_launch_sr(const afq_ctx_dev& c, const AdjointBufs& a, const int32_t* idx, cudaStream_t st);
// chol-bar[g][pq] += sqrt(dt) Re(i sum_w xt[w][g] conj(vhs-bar[w][pq])) over a walker chunk
int a_launch_chol_grad(const afq_ctx_dev& c, const AdjointBufs& a, int nwc, const double2* xt, cudaStream_t st);

}  // namespace afq

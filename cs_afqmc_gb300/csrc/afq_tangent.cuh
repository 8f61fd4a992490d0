// Tangent (forward-mode derivative) buffers and launchers of the FP64 phaseless block.
#pragma once
#include "afq_kernels.cuh"

namespace afq {

struct TangentBufs {
  double2* dw[2];      // walker tangents, layout of the walker slabs
  double2* wold[2];    // walkers before a QR (value); scratch of the SR gather
  double2* dgreen;     // [nw][ktot]
  double2* dfb;        // [nw][nchol]
  double2* dxt;        // [nw][nchol]
  double2* dshift;     // [nw]
  double2* dfbt;       // [nw]
  double2* dvhs;       // [nw_chunk][norb^2]
  double2* dlo;        // d log overlap [nw]
  double2* dlo_new;    // [nw]
  double* dweights;    // [nw]
  double* dscalars;    // [AFQ_NSCALARS]
  double2* dene;       // [nw]
  double2* dpart;      // [nw][e_chunks][5]
  double* dsum;        // [1]
  double* dbe;         // [n blocks]
  double* dbw;         // [n blocks]
  const double* dexp[2];  // d exp_h1 / d lambda per slab
  const double* drot[2];  // d rot_h1 / d lambda per Green block
  // orbital rotation (NULL: trial fixed): d trial / d lambda per slab [norb][nocc_s] and
  // d rot_chol / d lambda per Green block (layout of rot_chol) and concatenated [nchol][ktot]
  const double* dtrial[2];
  const double* drc[2];
  const double* drccat;
};

int t_launch_green(const afq_ctx_dev& c, const TangentBufs& t, const void* wu, const void* wd,
                   double2* green, double2* dgreen, double2* ovl, double2* dlog, cudaStream_t st);
int t_launch_field_shifts(const afq_ctx_dev& c, const double* fields, const double2* fb, const double2* dfb,
                          double2* xt, double2* dxt, double2* shift, double2* dshift, double2* fbt, double2* dfbt,
                          cudaStream_t st);
int t_launch_taylor(const afq_ctx_dev& c, const TangentBufs& t, int w0, int nwc, const double2* vhs,
                    const double2* dvhs, void* wu, void* wd, cudaStream_t st);
int t_launch_weights(const afq_ctx_dev& c, const TangentBufs& t, const double2* shift, const double2* fbt,
                     const double2* ovl_new, double2* ovl, double* weights, double* scalars, cudaStream_t st);
int t_launch_qr(const afq_ctx_dev& c, const TangentBufs& t, const void* wu, const void* wd, cudaStream_t st);
int t_launch_energy(const afq_ctx_dev& c, const TangentBufs& t, int nchunks, int gchunk, const double2* green,
                    cudaStream_t st);
// y += x, complex, n elements
int t_launch_add(long n, const double2* x, double2* y, cudaStream_t st);
int t_launch_block_stats(const afq_ctx_dev& c, const TangentBufs& t, const double2* energy, const double* weights,
                         const double* scalars, const double* be, double* dbe, double* dbw, cudaStream_t st);
int t_launch_sr_pre(const afq_ctx_dev& c, const TangentBufs& t, cudaStream_t st);
int t_launch_sr_post(const afq_ctx_dev& c, const TangentBufs& t, const int32_t* idx, cudaStream_t st);
int t_launch_end(int nblk, const double* be, const double* bw, const TangentBufs& t, double* energy,
                 double* denergy, cudaStream_t st);

}  // namespace afq

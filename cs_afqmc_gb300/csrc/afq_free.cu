// Free-projection AFQMC on FP64 unrestricted walkers (propagation.py:436-490; the sampler's
// free block, sampling.py:95-124, 344-360): no force bias and no phaseless constraint.
// The step reuses the FP64 vhs GEMM, Taylor kernel, Householder QR and overlap kernel of the
// phaseless path; these kernels add the mean-field constants, the QR norm bookkeeping and
// the block sums of the complex local energies.

#include <math.h>

#include "afq_common.cuh"
#include "afq_kernels.cuh"
#include "afq_prof.cuh"

namespace afq {

static int free_err(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    afq_set_error("%s: %s", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

// Per walker: S = sum_g x_g mf_g; for each spin s with n_s electrons the constant
// exp(-sqrt(dt) S / (2 n_s)) exp(dt (h0_prop + ene0) / (2 n_s)) (mf_shifts_fp and h0_prop_fp
// of propagation.py:473-486); the unshifted fields as the complex vhs operand.
__global__ void k_free_prep(int nw, int nchol, double sqdt, double dt, double h0p, int n0, int n1,
                            const double* __restrict__ fields, const double2* __restrict__ mf,
                            double2* __restrict__ xt, double2* __restrict__ consts) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  double sx = 0.0, sy = 0.0;
  for (int g = threadIdx.x; g < nchol; g += blockDim.x) {
    const double x = fields[(size_t)w * nchol + g];
    xt[(size_t)w * nchol + g] = c2(x, 0.0);
    sx += x * mf[g].x;
    sy += x * mf[g].y;
  }
  sx = block_sum(sx, red);
  sy = block_sum(sy, red);
  if (threadIdx.x == 0)
    for (int s = 0; s < 2; ++s) {
      const double inv = 1.0 / (2.0 * (s == 0 ? n0 : n1));
      consts[(size_t)s * nw + w] = cexp_(c2(-sqdt * sx * inv + dt * h0p * inv, -sqdt * sy * inv));
    }
}

// each walker slab times its spin's constant (propagation.py:455-457)
__global__ void k_free_scale(const afq_ctx_dev c, const double2* __restrict__ consts, double2* __restrict__ wu,
                             double2* __restrict__ wd) {
  const int w = blockIdx.x, s = blockIdx.y;
  const size_t n = (size_t)c.norb * c.kslab[s];
  double2* W = (s == 0 ? wu : wd) + (size_t)w * n;
  const double2 a = consts[(size_t)s * c.nw + w];
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) W[i] = cmul(W[i], a);
}

// norms *= prod(diag R_up) prod(diag R_dn); overlaps *= norms (propagation.py:458-461)
__global__ void k_free_finish(int nw, const double2* __restrict__ rdiag, double2* __restrict__ norms,
                              double2* __restrict__ ovl) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const double2 nrm = cmul(norms[w], cmul(rdiag[w], rdiag[nw + w]));
  norms[w] = nrm;
  ovl[w] = cmul(ovl[w], nrm);
}

// block_energy = sum_w E_w O_w / sum_w O_w, block_weight = sum_w O_w (sampling.py:118-123)
__global__ void k_free_block_stats(int nw, const double2* __restrict__ energy, const double2* __restrict__ ovl,
                                   double2* __restrict__ be, double2* __restrict__ bw) {
  __shared__ double red[32];
  double ax = 0, ay = 0, ox = 0, oy = 0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    const double2 p = cmul(energy[w], ovl[w]);
    ax += p.x;
    ay += p.y;
    ox += ovl[w].x;
    oy += ovl[w].y;
  }
  ax = block_sum(ax, red);
  ay = block_sum(ay, red);
  ox = block_sum(ox, red);
  oy = block_sum(oy, red);
  if (threadIdx.x == 0) {
    *be = cdiv(c2(ax, ay), c2(ox, oy));
    *bw = c2(ox, oy);
  }
}

int launch_free_prep(const afq_ctx_dev& c, const double* fields, double ene0, double2* xt, double2* consts,
                     cudaStream_t st) {
  {
    ProfScope _ps(K_FIELD, st);
    k_free_prep<<<c.nw, 256, 0, st>>>(c.nw, c.nchol, sqrt(c.dt), c.dt, c.h0_prop_re + ene0, c.nocc_slab[0],
                                      c.nocc_slab[1], fields, c.mf, xt, consts);
  }
  return free_err("free_prep");
}

int launch_free_scale(const afq_ctx_dev& c, const double2* consts, void* wu, void* wd, cudaStream_t st) {
  {
    ProfScope _ps(K_WEIGHTS, st);
    k_free_scale<<<dim3(c.nw, 2), 256, 0, st>>>(c, consts, static_cast<double2*>(wu), static_cast<double2*>(wd));
  }
  return free_err("free_scale");
}

int launch_free_finish(int nw, const double2* rdiag, double2* norms, double2* ovl, cudaStream_t st) {
  {
    ProfScope _ps(K_WEIGHTS, st);
    k_free_finish<<<(nw + 127) / 128, 128, 0, st>>>(nw, rdiag, norms, ovl);
  }
  return free_err("free_finish");
}

int launch_free_block_stats(int nw, const double2* energy, const double2* ovl, double2* be, double2* bw,
                            cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_free_block_stats<<<1, 1024, 0, st>>>(nw, energy, ovl, be, bw);
  }
  return free_err("free_block_stats");
}

}  // namespace afq

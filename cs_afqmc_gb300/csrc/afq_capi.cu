// C ABI of the AFQMC hot path: context creation, workspace layout and the stream-ordered
// orchestration of the kernels (one propagation step, QR, SR, measurements, and the
// sampler's block loop). See include/afqmc_gb300.h for the contract of each entry point.

#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "afq_common.cuh"
#include "afq_adjoint.cuh"
#include "afq_kernels.cuh"
#include "afq_tangent.cuh"
#include "afq_tc.cuh"

static thread_local char g_err[512] = "";

void afq_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

struct afq_ctx {
  afq_dims d;
  afq_hamiltonian h;
  afq_ctx_dev dev;
  int nw_chunk;
  int e_chunks, e_gchunk;
  size_t welem;  // bytes per walker element (16 complex128, 8 complex64)
  // workspace views
  char* ws;
  size_t ws_bytes;
  double2* green;
  double2* fb;
  double2* xt;
  double2* shift;
  double2* fbt;
  double2* vhs;
  double2* ovl_new;
  double2* ene;
  double2* epart;
  double* rccat;
  void* wcopy;
  int32_t* sr_idx;
  double* cum;
  double2* free_scr;  // free projection: spin constants and QR norm factors [4][nw]
  afq::TcState tc;  // tensor-core (mixed precision) operands and plans
  // Inside afq_propagate_phaseless only (mixed path): 1 when the operand buffers already
  // hold G, its operands and the walker operand of the current walkers, else 0.
  int gstate;
};

namespace {

struct Layout {
  size_t off = 0;
  size_t take(size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  }
};

struct Sizes {
  size_t green, fb, xt, shift, fbt, vhs, ovl_new, ene, epart, rccat, wcopy, sr_idx, cum, free_scr, tc, total;
};

int derive(const afq_dims* d, afq_ctx_dev* c, int* nw_chunk, int* e_chunks, int* e_gchunk,
           size_t* welem) {
  if (!d) { afq_set_error("dims is NULL"); return -1; }
  if (d->norb < 1 || d->n_up < 1 || d->n_dn < 0 || d->nchol < 1 || d->n_walkers < 1) {
    afq_set_error("bad sizes norb=%d n_up=%d n_dn=%d nchol=%d n_walkers=%d", d->norb, d->n_up,
                  d->n_dn, d->nchol, d->n_walkers);
    return -1;
  }
  if (d->n_up > d->norb || d->n_dn > d->norb) { afq_set_error("more electrons than orbitals"); return -1; }
  if (d->precision != AFQ_PREC_FP64 && d->precision != AFQ_PREC_MIXED) {
    afq_set_error("unknown precision %d", d->precision); return -1;
  }
  if (d->walker_type != AFQ_WALKERS_RESTRICTED && d->walker_type != AFQ_WALKERS_UNRESTRICTED) {
    afq_set_error("unknown walker_type %d", d->walker_type); return -1;
  }
  if (d->trial_type != AFQ_TRIAL_RHF && d->trial_type != AFQ_TRIAL_UHF) {
    afq_set_error("unknown trial_type %d", d->trial_type); return -1;
  }
  if (d->trial_type == AFQ_TRIAL_RHF && d->n_up != d->n_dn) {
    afq_set_error("RHF requires equal number of up and down electrons"); return -1;
  }
  if (d->walker_type == AFQ_WALKERS_RESTRICTED && d->trial_type != AFQ_TRIAL_RHF) {
    afq_set_error("restricted walkers are supported with the RHF trial only"); return -1;
  }
  if (d->walker_type == AFQ_WALKERS_UNRESTRICTED && d->n_dn < 1) {
    afq_set_error("unrestricted walkers need n_dn >= 1"); return -1;
  }
  if (d->n_exp_terms < 1 || d->n_exp_terms > 32) { afq_set_error("n_exp_terms out of range"); return -1; }
  if (!(d->dt > 0.0)) { afq_set_error("dt must be positive"); return -1; }
  int nb = d->n_batch < 1 ? 1 : d->n_batch;
  if (d->n_walkers % nb != 0) { afq_set_error("n_batch must divide n_walkers"); return -1; }
  memset(c, 0, sizeof(*c));
  c->norb = d->norb;
  c->nchol = d->nchol;
  c->nw = d->n_walkers;
  c->n_exp_terms = d->n_exp_terms;
  c->dt = d->dt;
  if (d->walker_type == AFQ_WALKERS_RESTRICTED) {
    c->nslab = 1;
    c->kslab[0] = c->nocc_slab[0] = d->n_up;
    c->restricted_square = 1;
  } else {
    c->nslab = 2;
    c->kslab[0] = c->nocc_slab[0] = d->n_up;
    c->kslab[1] = c->nocc_slab[1] = d->n_dn;
  }
  c->kmax = c->kslab[0] > c->kslab[1] ? c->kslab[0] : c->kslab[1];
  if (d->trial_type == AFQ_TRIAL_RHF) {
    c->nspin_g = 1;
    c->gocc[0] = d->n_up;
    c->ktot = d->n_up * d->norb;
    c->energy_mode = (c->nslab == 1) ? 0 : 1;
  } else {
    c->nspin_g = 2;
    c->gocc[0] = d->n_up;
    c->gocc[1] = d->n_dn;
    c->ktot = (d->n_up + d->n_dn) * d->norb;
    c->energy_mode = 2;
  }
  // kernel resource limits
  if (c->kmax > 64) { afq_set_error("at most 64 electrons per spin are supported"); return -1; }
  if ((size_t)d->norb * c->kmax > 7000) { afq_set_error("norb * nocc too large (<= 7000)"); return -1; }
  *nw_chunk = d->n_walkers / nb;
  *e_gchunk = 16;
  *e_chunks = (d->nchol + *e_gchunk - 1) / *e_gchunk;
  *welem = d->precision == AFQ_PREC_FP64 ? 16 : 8;
  return 0;
}

Sizes sizes_for(const afq_dims* d, const afq_ctx_dev& c, int nw_chunk, int e_chunks, size_t welem,
                Layout* L) {
  Sizes s;
  const size_t nw = c.nw, C16 = sizeof(double2);
  s.green = L->take(nw * c.ktot * C16);
  s.fb = L->take(nw * c.nchol * C16);
  s.xt = L->take(nw * c.nchol * C16);
  s.shift = L->take(nw * C16);
  s.fbt = L->take(nw * C16);
  s.vhs = L->take(d->precision == AFQ_PREC_FP64 ? (size_t)nw_chunk * c.norb * c.norb * C16 : 256);
  s.ovl_new = L->take(nw * C16);
  s.ene = L->take(nw * C16);
  s.epart = L->take(nw * e_chunks * 5 * C16);
  s.rccat = L->take(c.nspin_g == 2 ? (size_t)c.nchol * c.ktot * sizeof(double) : 256);
  s.wcopy = L->take(nw * c.norb * (c.kslab[0] + c.kslab[1]) * welem);
  s.sr_idx = L->take(nw * sizeof(int32_t));
  s.cum = L->take(nw * sizeof(double));
  s.free_scr = L->take(4 * nw * C16);
  s.tc = L->take(d->precision == AFQ_PREC_MIXED ? afq::tc_workspace_bytes(c, nw_chunk, d->mixed_config)
                                                : 256);
  s.total = L->off;
  return s;
}

inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

#define CHECK(x)            \
  do {                      \
    int _e = (x);           \
    if (_e) return _e;      \
  } while (0)

bool is_fp64(const afq_ctx* c) { return c->d.precision == AFQ_PREC_FP64; }

// Green's function + overlap. FP64: G into c->green. Mixed: the 16-bit operands of the
// force-bias, energy and exp_h1 contractions (wg) and/or the overlap.
// chain (mixed path, inside afq_propagate_phaseless): the walkers are propagated next, so
// the same launch also forms G and the operands; c->gstate records that for the next step.
int green(afq_ctx* c, const void* wu, const void* wd, double2* g, double2* ovl, bool wg, cudaStream_t st,
          bool chain = false) {
  if (is_fp64(c)) return afq::launch_green<double>(c->dev, wu, wd, g, ovl, wg, st);
  CHECK(afq::tc_green(c->tc, c->dev, wu, wd, ovl, wg, st, chain));
  c->gstate = chain ? 1 : 0;
  return 0;
}

int force_bias_from_green(afq_ctx* c, double2* out, cudaStream_t st) {
  const afq_ctx_dev& d = c->dev;
  double2 alpha = c2(d.energy_mode == 0 ? 2.0 : 1.0, 0.0);
  const double* B = d.nspin_g == 2 ? c->rccat : d.rot_chol[0];
  if (!is_fp64(c)) return afq::tc_force_bias(c->tc, d, out, st);
  return afq::launch_gemm_cr(false, d.nw, d.nchol, d.ktot, c->green, d.ktot, B, d.ktot, out, d.nchol,
                             alpha, st);
}

int energy_from_green(afq_ctx* c, double2* out, cudaStream_t st) {
  if (!is_fp64(c)) return afq::tc_energy(c->tc, c->dev, out, st);
  return afq::launch_energy_f64(c->dev, c->e_chunks, c->e_gchunk, c->green, c->epart, out, st);
}

int check_walkers(const afq_ctx* c, const void* wu, const void* wd) {
  if (!wu) { afq_set_error("walkers_up is NULL"); return -1; }
  if (c->dev.nslab == 2 && !wd) { afq_set_error("unrestricted walkers need walkers_dn"); return -1; }
  return 0;
}

int check_state(const afq_ctx* c, const afq_walker_state* s) {
  if (!s) { afq_set_error("state is NULL"); return -1; }
  CHECK(check_walkers(c, s->walkers_up, s->walkers_dn));
  if (!s->weights || !s->overlaps || !s->scalars) { afq_set_error("state has NULL arrays"); return -1; }
  return 0;
}

// chain: a step inside afq_propagate_phaseless, where the Green's-function work of the
// previous overlap evaluation on the same walkers (c->gstate) is reused.
// next_g (with chain): the next operation propagates the same walkers again, so the overlap
// evaluation after the step also forms G and the operands (not before a QR).
int propagate_impl(afq_ctx* c, afq_walker_state* s, const double* fields, cudaStream_t st,
                   bool chain = false, bool next_g = true) {
  const afq_ctx_dev& d = c->dev;
  if (!is_fp64(c)) {
    // mixed: operands -> fused force bias / field shifts -> exp_h1, vhs + Taylor, exp_h1
    if (!(chain && c->gstate == 1)) CHECK(afq::tc_green(c->tc, d, s->walkers_up, s->walkers_dn, nullptr, true, st));
    CHECK(afq::tc_field_shifts(c->tc, d, fields, st));
    CHECK(afq::tc_propagate_walkers(c->tc, d, s->walkers_up, s->walkers_dn, st));
    CHECK(green(c, s->walkers_up, s->walkers_dn, nullptr, c->ovl_new, false, st, chain && next_g));
    return afq::tc_weights(c->tc, d, c->ovl_new, reinterpret_cast<double2*>(s->overlaps), s->weights,
                           s->scalars, st);
  }
  CHECK(green(c, s->walkers_up, s->walkers_dn, c->green, nullptr, true, st));
  CHECK(force_bias_from_green(c, c->fb, st));
  CHECK(afq::launch_field_shifts(d, fields, c->fb, c->xt, c->shift, c->fbt, st));
  const int nb = d.nw / c->nw_chunk;
  for (int b = 0; b < nb; ++b) {
    const int w0 = b * c->nw_chunk;
    double sq = sqrt(d.dt);
    CHECK(afq::launch_gemm_cr(true, c->nw_chunk, d.norb * d.norb, d.nchol, c->xt + (size_t)w0 * d.nchol,
                              d.nchol, c->h.chol, (long)d.norb * d.norb, c->vhs, (long)d.norb * d.norb,
                              c2(0.0, sq), st));
    CHECK(afq::launch_taylor_f64<double>(d, w0, c->nw_chunk, c->vhs, s->walkers_up, s->walkers_dn, st));
  }
  CHECK(green(c, s->walkers_up, s->walkers_dn, nullptr, c->ovl_new, false, st));
  return afq::launch_weights(d, c->shift, c->fbt, 1, c->ovl_new, reinterpret_cast<double2*>(s->overlaps),
                             s->weights, s->scalars, st);
}

int qr_impl(afq_ctx* c, afq_walker_state* s, cudaStream_t st) {
  if (is_fp64(c)) return afq::launch_qr<double>(c->dev, s->walkers_up, s->walkers_dn, st);
  return afq::tc_orthonormalize(c->tc, c->dev, s->walkers_up, s->walkers_dn, st);
}

int sr_impl(afq_ctx* c, afq_walker_state* s, const double* zeta, int32_t* indices, cudaStream_t st) {
  if (is_fp64(c))
    CHECK(afq::launch_sr<double>(c->dev, zeta, s->weights, c->cum, c->sr_idx, s->walkers_up,
                                 s->walkers_dn, c->wcopy, st));
  else
    CHECK(afq::launch_sr<float>(c->dev, zeta, s->weights, c->cum, c->sr_idx, s->walkers_up,
                                s->walkers_dn, c->wcopy, st));
  if (indices) {
    cudaError_t e = cudaMemcpyAsync(indices, c->sr_idx, sizeof(int32_t) * c->dev.nw,
                                    cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) { afq_set_error("sr index copy: %s", cudaGetErrorString(e)); return (int)e; }
  }
  return 0;
}

// One free-projection step (propagation.py:436-462), FP64 unrestricted walkers.
int free_step(afq_ctx* c, afq_walker_state* s, const double* fields, double ene0, double2* norms, double2* normed,
              cudaStream_t st) {
  const afq_ctx_dev& d = c->dev;
  double2* consts = c->free_scr;
  double2* rdiag = c->free_scr + 2 * (size_t)d.nw;
  double2* ovl = reinterpret_cast<double2*>(s->overlaps);
  CHECK(afq::launch_free_prep(d, fields, ene0, c->xt, consts, st));
  const int nb = d.nw / c->nw_chunk;
  const long nn = (long)d.norb * d.norb;
  for (int b = 0; b < nb; ++b) {
    const int w0 = b * c->nw_chunk;
    CHECK(afq::launch_gemm_cr(true, c->nw_chunk, d.norb * d.norb, d.nchol, c->xt + (size_t)w0 * d.nchol, d.nchol,
                              c->h.chol, nn, c->vhs, nn, c2(0.0, sqrt(d.dt)), st));
    CHECK(afq::launch_taylor_f64<double>(d, w0, c->nw_chunk, c->vhs, s->walkers_up, s->walkers_dn, st));
  }
  CHECK(afq::launch_free_scale(d, consts, s->walkers_up, s->walkers_dn, st));
  CHECK(afq::launch_qr<double>(d, s->walkers_up, s->walkers_dn, st, rdiag));
  CHECK(green(c, s->walkers_up, s->walkers_dn, nullptr, ovl, false, st));
  CHECK(afq::launch_free_finish(d.nw, rdiag, norms, ovl, st));
  // normed overlaps: the walkers through the QR once more, on a copy
  const size_t e0 = (size_t)d.nw * d.norb * d.kslab[0], e1 = (size_t)d.nw * d.norb * d.kslab[1];
  double2* cu = static_cast<double2*>(c->wcopy);
  double2* cd = cu + e0;
  cudaError_t e = cudaMemcpyAsync(cu, s->walkers_up, e0 * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cd, s->walkers_dn, e1 * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) { afq_set_error("walker copy: %s", cudaGetErrorString(e)); return (int)e; }
  CHECK(afq::launch_qr<double>(d, cu, cd, st));
  return green(c, cu, cd, nullptr, normed, false, st);
}

int check_free(const afq_ctx* c) {
  if (!is_fp64(c) || c->dev.nslab != 2) {
    afq_set_error("free projection needs an FP64 context with unrestricted walkers");
    return -1;
  }
  return 0;
}

// Tangent workspace of afq_propagate_phaseless_jvp, carved like the main workspace.
struct TSizes {
  size_t dw[2], wold[2], dgreen, dfb, dxt, dshift, dfbt, dvhs, dlo, dlo_new, dweights, dscalars, dene, dpart,
      dsum, drccat, total;
};

TSizes tangent_sizes(const afq_ctx_dev& c, int nw_chunk, int e_chunks, Layout* L) {
  TSizes s;
  const size_t nw = c.nw, C16 = sizeof(double2);
  for (int k = 0; k < 2; ++k) {  // kslab[1] is 0 for restricted walkers
    s.dw[k] = L->take(nw * c.norb * c.kslab[k] * C16);
    s.wold[k] = L->take(nw * c.norb * c.kslab[k] * C16);
  }
  s.dgreen = L->take(nw * c.ktot * C16);
  s.dfb = L->take(nw * c.nchol * C16);
  s.dxt = L->take(nw * c.nchol * C16);
  s.dshift = L->take(nw * C16);
  s.dfbt = L->take(nw * C16);
  s.dvhs = L->take((size_t)nw_chunk * c.norb * c.norb * C16);
  s.dlo = L->take(nw * C16);
  s.dlo_new = L->take(nw * C16);
  s.dweights = L->take(nw * sizeof(double));
  s.dscalars = L->take(AFQ_NSCALARS * sizeof(double));
  s.dene = L->take(nw * C16);
  s.dpart = L->take(nw * e_chunks * 5 * C16);
  s.dsum = L->take(sizeof(double));
  s.drccat = L->take(c.nspin_g == 2 ? (size_t)c.nchol * c.ktot * sizeof(double) : 256);
  s.total = L->off;
  return s;
}

// One phaseless step with tangents (propagate_impl's FP64 branch, each stage followed by
// its tangent).
int propagate_jvp(afq_ctx* c, afq_walker_state* s, const afq::TangentBufs& t, const double* fields,
                  cudaStream_t st) {
  const afq_ctx_dev& d = c->dev;
  CHECK(afq::t_launch_green(d, t, s->walkers_up, s->walkers_dn, c->green, t.dgreen, c->ovl_new, t.dlo_new, st));
  CHECK(force_bias_from_green(c, c->fb, st));
  {
    const double2 alpha = c2(d.energy_mode == 0 ? 2.0 : 1.0, 0.0);
    const double* B = d.nspin_g == 2 ? c->rccat : d.rot_chol[0];
    CHECK(afq::launch_gemm_cr(false, d.nw, d.nchol, d.ktot, t.dgreen, d.ktot, B, d.ktot, t.dfb, d.nchol, alpha,
                              st));
    if (t.drccat) {  // orbital rotation: + alpha G dRC^T (t.dxt as scratch, rewritten below)
      CHECK(afq::launch_gemm_cr(false, d.nw, d.nchol, d.ktot, c->green, d.ktot, t.drccat, d.ktot, t.dxt, d.nchol,
                                alpha, st));
      CHECK(afq::t_launch_add((long)d.nw * d.nchol, t.dxt, t.dfb, st));
    }
  }
  CHECK(afq::t_launch_field_shifts(d, fields, c->fb, t.dfb, c->xt, t.dxt, c->shift, t.dshift, c->fbt, t.dfbt, st));
  const int nb = d.nw / c->nw_chunk;
  const long nn = (long)d.norb * d.norb;
  const double2 isq = c2(0.0, sqrt(d.dt));
  for (int b = 0; b < nb; ++b) {
    const int w0 = b * c->nw_chunk;
    CHECK(afq::launch_gemm_cr(true, c->nw_chunk, d.norb * d.norb, d.nchol, c->xt + (size_t)w0 * d.nchol, d.nchol,
                              c->h.chol, nn, c->vhs, nn, isq, st));
    CHECK(afq::launch_gemm_cr(true, c->nw_chunk, d.norb * d.norb, d.nchol, t.dxt + (size_t)w0 * d.nchol, d.nchol,
                              c->h.chol, nn, t.dvhs, nn, isq, st));
    CHECK(afq::t_launch_taylor(d, t, w0, c->nw_chunk, c->vhs, t.dvhs, s->walkers_up, s->walkers_dn, st));
  }
  CHECK(afq::t_launch_green(d, t, s->walkers_up, s->walkers_dn, nullptr, nullptr, c->ovl_new, t.dlo_new, st));
  return afq::t_launch_weights(d, t, c->shift, c->fbt, c->ovl_new, reinterpret_cast<double2*>(s->overlaps),
                               s->weights, s->scalars, st);
}

int copy_d2d(void* dst, const void* src, size_t bytes, cudaStream_t st, const char* what) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) { afq_set_error("%s: %s", what, cudaGetErrorString(e)); return (int)e; }
  return 0;
}

// Workspace of afq_propagate_phaseless_vjp: the recorded forward sweep (snapshots of the
// walker state before every step, after the last step of an energy block and after its QR;
// shifted fields and shift terms of every step; local energies of every block; SR indices)
// followed by the backward sweep's cotangents.
struct AdjSizes {
  size_t snap_w, snap_wt, snap_ov, snap_sc, t_xt, t_sh, t_fbt, t_ene, t_idx;
  size_t wb, wb2, wbar, lbar, lbar2, gpend, gene, fbb, xtb, shb, fbtb, vbar, tay, ebar, scal, beb, bwb, total;
  size_t wslab;  // walker elements of one snapshot, both slabs
  int nblk, nsteps, nsnap;
};

AdjSizes adjoint_sizes(const afq_ctx_dev& c, int nw_chunk, int n_prop, int n_ene, int n_sr, Layout* L) {
  AdjSizes s;
  const size_t nw = c.nw, C16 = sizeof(double2), nk = (size_t)c.norb * (c.kslab[0] + c.kslab[1]);
  s.nblk = n_ene * n_sr;
  s.nsteps = s.nblk * n_prop;
  s.nsnap = s.nblk * (n_prop + 2);
  s.wslab = nw * nk;
  s.snap_w = L->take((size_t)s.nsnap * s.wslab * C16);
  s.snap_wt = L->take((size_t)s.nsnap * nw * sizeof(double));
  s.snap_ov = L->take((size_t)s.nsnap * nw * C16);
  s.snap_sc = L->take((size_t)s.nsnap * AFQ_NSCALARS * sizeof(double));
  s.t_xt = L->take((size_t)s.nsteps * nw * c.nchol * C16);
  s.t_sh = L->take((size_t)s.nsteps * nw * C16);
  s.t_fbt = L->take((size_t)s.nsteps * nw * C16);
  s.t_ene = L->take((size_t)s.nblk * nw * C16);
  s.t_idx = L->take((size_t)n_sr * nw * sizeof(int32_t));
  s.wb = L->take(s.wslab * C16);
  s.wb2 = L->take(s.wslab * C16);
  s.wbar = L->take(nw * sizeof(double));
  s.lbar = L->take(nw * C16);
  s.lbar2 = L->take(nw * C16);
  s.gpend = L->take(nw * c.ktot * C16);
  s.gene = L->take(nw * c.ktot * C16);
  s.fbb = L->take(nw * c.nchol * C16);
  s.xtb = L->take(nw * c.nchol * C16);
  s.shb = L->take(nw * C16);
  s.fbtb = L->take(nw * C16);
  s.vbar = L->take((size_t)nw_chunk * c.norb * c.norb * C16);
  s.tay = L->take((size_t)nw_chunk * (2 * (c.n_exp_terms - 1) + 2) * nk * C16);
  s.ebar = L->take(nw * sizeof(double));
  s.scal = L->take(8 * sizeof(double));
  s.beb = L->take((size_t)s.nblk * sizeof(double));
  s.bwb = L->take((size_t)s.nblk * sizeof(double));
  s.total = L->off;
  return s;
}

// Views of the recorded forward sweep. Snapshot i = blk * (n_prop + 2) + j: j < n_prop
// before step j, j == n_prop after the last step (before the QR), j == n_prop + 1 after
// the QR and the overlap evaluation.
struct Tape {
  char* base;
  AdjSizes s;
  const afq_ctx_dev* d;
  double2* w(int i, int slab) const {
    return reinterpret_cast<double2*>(base + s.snap_w) + (size_t)i * s.wslab +
           (slab ? (size_t)d->nw * d->norb * d->kslab[0] : 0);
  }
  double* wt(int i) const { return reinterpret_cast<double*>(base + s.snap_wt) + (size_t)i * d->nw; }
  double2* ov(int i) const { return reinterpret_cast<double2*>(base + s.snap_ov) + (size_t)i * d->nw; }
  double* sc(int i) const { return reinterpret_cast<double*>(base + s.snap_sc) + (size_t)i * AFQ_NSCALARS; }
  double2* xt(int step) const {
    return reinterpret_cast<double2*>(base + s.t_xt) + (size_t)step * d->nw * d->nchol;
  }
  double2* sh(int step) const { return reinterpret_cast<double2*>(base + s.t_sh) + (size_t)step * d->nw; }
  double2* fbt(int step) const { return reinterpret_cast<double2*>(base + s.t_fbt) + (size_t)step * d->nw; }
  double2* ene(int blk) const { return reinterpret_cast<double2*>(base + s.t_ene) + (size_t)blk * d->nw; }
  int32_t* idx(int sr) const { return reinterpret_cast<int32_t*>(base + s.t_idx) + (size_t)sr * d->nw; }
};

int snapshot(const Tape& t, int i, const afq_walker_state* st_, cudaStream_t st) {
  const afq_ctx_dev& d = *t.d;
  const size_t e0 = (size_t)d.nw * d.norb * d.kslab[0], e1 = (size_t)d.nw * d.norb * d.kslab[1];
  CHECK(copy_d2d(t.w(i, 0), st_->walkers_up, e0 * sizeof(double2), st, "walker snapshot"));
  if (d.nslab == 2) CHECK(copy_d2d(t.w(i, 1), st_->walkers_dn, e1 * sizeof(double2), st, "walker snapshot"));
  CHECK(copy_d2d(t.wt(i), st_->weights, d.nw * sizeof(double), st, "weight snapshot"));
  CHECK(copy_d2d(t.ov(i), st_->overlaps, d.nw * sizeof(double2), st, "overlap snapshot"));
  return copy_d2d(t.sc(i), st_->scalars, AFQ_NSCALARS * sizeof(double), st, "scalar snapshot");
}

int zero(void* p, size_t bytes, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(p, 0, bytes, st);
  if (e != cudaSuccess) { afq_set_error("memset: %s", cudaGetErrorString(e)); return (int)e; }
  return 0;
}

void swap_slabs(double2* a[2], double2* b[2]) {
  for (int k = 0; k < 2; ++k) {
    double2* t = a[k];
    a[k] = b[k];
    b[k] = t;
  }
}

}  // namespace

extern "C" {

int afq_abi_version(void) { return AFQ_ABI_VERSION; }

const char* afq_last_error(void) { return g_err; }

size_t afq_workspace_size(const afq_dims* dims) {
  afq_ctx_dev c;
  int nwc, ec, eg;
  size_t we;
  if (derive(dims, &c, &nwc, &ec, &eg, &we)) return 0;
  Layout L;
  return sizes_for(dims, c, nwc, ec, we, &L).total;
}

int afq_ctx_create(const afq_dims* dims, const afq_hamiltonian* ham, void* workspace,
                   size_t workspace_bytes, void* stream, afq_ctx** out) {
  if (!out) { afq_set_error("out is NULL"); return -1; }
  *out = nullptr;
  afq_ctx_dev dev;
  int nwc, ec, eg;
  size_t we;
  CHECK(derive(dims, &dev, &nwc, &ec, &eg, &we));
  if (!ham) { afq_set_error("hamiltonian is NULL"); return -1; }
  const bool uhf = dims->trial_type == AFQ_TRIAL_UHF;
  const bool unres = dims->walker_type == AFQ_WALKERS_UNRESTRICTED;
  if (!ham->trial_up || !ham->chol || !ham->rot_chol_up || !ham->rot_h1_up || !ham->exp_h1_up ||
      !ham->mf_shifts || (uhf && (!ham->trial_dn || !ham->rot_chol_dn || !ham->rot_h1_dn)) ||
      (unres && !ham->exp_h1_dn)) {
    afq_set_error("hamiltonian has NULL arrays");
    return -1;
  }
  Layout L;
  Sizes sz = sizes_for(dims, dev, nwc, ec, we, &L);
  if (!workspace || workspace_bytes < sz.total) {
    afq_set_error("workspace too small: need %zu bytes, got %zu", sz.total, workspace_bytes);
    return -1;
  }
  if (reinterpret_cast<uintptr_t>(workspace) & 255) { afq_set_error("workspace must be 256-byte aligned"); return -1; }
  afq_ctx* c = new (std::nothrow) afq_ctx();
  if (!c) { afq_set_error("out of host memory"); return -1; }
  c->d = *dims;
  if (c->d.n_batch < 1) c->d.n_batch = 1;
  c->h = *ham;
  c->nw_chunk = nwc;
  c->e_chunks = ec;
  c->e_gchunk = eg;
  c->welem = we;
  dev.h0 = ham->h0;
  dev.h0_prop_re = ham->h0_prop_re;
  dev.h0_prop_im = ham->h0_prop_im;
  dev.trial[0] = ham->trial_up;
  dev.trial[1] = uhf ? ham->trial_dn : ham->trial_up;
  dev.exp_h1[0] = ham->exp_h1_up;
  dev.exp_h1[1] = unres ? ham->exp_h1_dn : ham->exp_h1_up;
  dev.rot_chol[0] = ham->rot_chol_up;
  dev.rot_chol[1] = uhf ? ham->rot_chol_dn : ham->rot_chol_up;
  dev.rot_h1[0] = ham->rot_h1_up;
  dev.rot_h1[1] = uhf ? ham->rot_h1_dn : ham->rot_h1_up;
  dev.mf = reinterpret_cast<const double2*>(ham->mf_shifts);
  c->dev = dev;
  char* ws = static_cast<char*>(workspace);
  c->ws = ws;
  c->ws_bytes = workspace_bytes;
  c->green = reinterpret_cast<double2*>(ws + sz.green);
  c->fb = reinterpret_cast<double2*>(ws + sz.fb);
  c->xt = reinterpret_cast<double2*>(ws + sz.xt);
  c->shift = reinterpret_cast<double2*>(ws + sz.shift);
  c->fbt = reinterpret_cast<double2*>(ws + sz.fbt);
  c->vhs = reinterpret_cast<double2*>(ws + sz.vhs);
  c->ovl_new = reinterpret_cast<double2*>(ws + sz.ovl_new);
  c->ene = reinterpret_cast<double2*>(ws + sz.ene);
  c->epart = reinterpret_cast<double2*>(ws + sz.epart);
  c->rccat = reinterpret_cast<double*>(ws + sz.rccat);
  c->wcopy = ws + sz.wcopy;
  c->sr_idx = reinterpret_cast<int32_t*>(ws + sz.sr_idx);
  c->cum = reinterpret_cast<double*>(ws + sz.cum);
  c->free_scr = reinterpret_cast<double2*>(ws + sz.free_scr);
  cudaStream_t st = S(stream);
  if (uhf) {
    // rccat[g] = [rot_chol_up[g] | rot_chol_dn[g]]
    const size_t a = (size_t)dims->n_up * dims->norb, b = (size_t)dims->n_dn * dims->norb;
    cudaError_t e = cudaMemcpy2DAsync(c->rccat, dev.ktot * sizeof(double), ham->rot_chol_up, a * sizeof(double),
                                      a * sizeof(double), dims->nchol, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(c->rccat + a, dev.ktot * sizeof(double), ham->rot_chol_dn, b * sizeof(double),
                            b * sizeof(double), dims->nchol, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
      afq_set_error("rot_chol concat: %s", cudaGetErrorString(e));
      delete c;
      return (int)e;
    }
  }
  if (dims->precision == AFQ_PREC_MIXED) {
    int e = afq::tc_init(&c->tc, c->dev, *ham, c->rccat, nwc, dims->mixed_config, ws + sz.tc, st);
    if (e) {
      delete c;
      return e;
    }
  }
  *out = c;
  return 0;
}

void afq_ctx_destroy(afq_ctx* ctx) { delete ctx; }

int afq_calc_overlap(afq_ctx* ctx, const void* walkers_up, const void* walkers_dn, double* overlaps,
                     void* stream) {
  if (!ctx || !overlaps) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_walkers(ctx, walkers_up, walkers_dn));
  return green(ctx, walkers_up, walkers_dn, nullptr, reinterpret_cast<double2*>(overlaps), false, S(stream));
}

int afq_calc_force_bias(afq_ctx* ctx, const void* walkers_up, const void* walkers_dn,
                        double* force_bias, void* stream) {
  if (!ctx || !force_bias) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_walkers(ctx, walkers_up, walkers_dn));
  CHECK(green(ctx, walkers_up, walkers_dn, ctx->green, nullptr, true, S(stream)));
  return force_bias_from_green(ctx, reinterpret_cast<double2*>(force_bias), S(stream));
}

int afq_calc_energy(afq_ctx* ctx, const void* walkers_up, const void* walkers_dn, double* energies,
                    void* stream) {
  if (!ctx || !energies) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_walkers(ctx, walkers_up, walkers_dn));
  CHECK(green(ctx, walkers_up, walkers_dn, ctx->green, nullptr, true, S(stream)));
  return energy_from_green(ctx, reinterpret_cast<double2*>(energies), S(stream));
}

int afq_propagate(afq_ctx* ctx, afq_walker_state* state, const double* fields, void* stream) {
  if (!ctx || !fields) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_state(ctx, state));
  return propagate_impl(ctx, state, fields, S(stream));
}

int afq_orthonormalize_walkers(afq_ctx* ctx, afq_walker_state* state, void* stream) {
  if (!ctx) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_state(ctx, state));
  return qr_impl(ctx, state, S(stream));
}

int afq_stochastic_reconfiguration(afq_ctx* ctx, afq_walker_state* state, const double* zeta,
                                   int32_t* indices, void* stream) {
  if (!ctx || !zeta) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_state(ctx, state));
  return sr_impl(ctx, state, zeta, indices, S(stream));
}

int afq_propagate_phaseless(afq_ctx* ctx, afq_walker_state* state, const double* fields,
                            const double* zetas, int32_t n_prop_steps, int32_t n_ene_blocks,
                            int32_t n_sr_blocks, double* block_energy, double* block_weight,
                            double* energy, void* stream) {
  if (!ctx || !fields || !zetas || !block_energy || !block_weight || !energy) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (n_prop_steps < 1 || n_ene_blocks < 1 || n_sr_blocks < 1) {
    afq_set_error("block counts must be >= 1");
    return -1;
  }
  CHECK(check_state(ctx, state));
  cudaStream_t st = S(stream);
  const afq_ctx_dev& d = ctx->dev;
  double2* ovl = reinterpret_cast<double2*>(state->overlaps);
  ctx->gstate = 0;
  CHECK(green(ctx, state->walkers_up, state->walkers_dn, nullptr, ovl, false, st, true));
  CHECK(afq::launch_phaseless_begin(state->scalars, st));
  const size_t step_elems = (size_t)d.nw * d.nchol;
  int blk = 0;
  for (int sr = 0; sr < n_sr_blocks; ++sr) {
    for (int eb = 0; eb < n_ene_blocks; ++eb, ++blk) {
      for (int p = 0; p < n_prop_steps; ++p) {
        const double* f = fields + ((size_t)blk * n_prop_steps + p) * step_elems;
        CHECK(propagate_impl(ctx, state, f, st, true, p + 1 < n_prop_steps));
      }
      ctx->gstate = 0;
      CHECK(qr_impl(ctx, state, st));
      CHECK(green(ctx, state->walkers_up, state->walkers_dn, ctx->green, ovl, true, st, true));
      CHECK(energy_from_green(ctx, ctx->ene, st));
      CHECK(afq::launch_block_stats(d, ctx->ene, state->weights, state->scalars, block_energy + blk,
                                    block_weight + blk, st));
    }
    ctx->gstate = 0;
    CHECK(sr_impl(ctx, state, zetas + sr, nullptr, st));
    CHECK(green(ctx, state->walkers_up, state->walkers_dn, nullptr, ovl, false, st, true));
  }
  ctx->gstate = 0;
  return afq::launch_phaseless_end(blk, (double)n_sr_blocks * n_ene_blocks * d.nw, block_energy,
                                   block_weight, state->scalars, energy, st);
}

size_t afq_tangent_workspace_size(const afq_dims* dims) {
  afq_ctx_dev c;
  int nwc, ec, eg;
  size_t we;
  if (derive(dims, &c, &nwc, &ec, &eg, &we)) return 0;
  Layout L;
  return tangent_sizes(c, nwc, ec, &L).total;
}

int afq_propagate_phaseless_jvp(afq_ctx* ctx, afq_walker_state* state, const double* dexp_h1_up,
                                const double* dexp_h1_dn, const double* drot_h1_up, const double* drot_h1_dn,
                                void* tangent_workspace, size_t tangent_workspace_bytes, const double* fields,
                                const double* zetas, int32_t n_prop_steps, int32_t n_ene_blocks,
                                int32_t n_sr_blocks, int32_t flags, double* block_energy, double* block_weight,
                                double* dblock_energy, double* dblock_weight, double* energy, double* denergy,
                                void* stream) {
  afq_jvp_inputs in;
  memset(&in, 0, sizeof(in));
  in.dexp_h1_up = dexp_h1_up;
  in.dexp_h1_dn = dexp_h1_dn;
  in.drot_h1_up = drot_h1_up;
  in.drot_h1_dn = drot_h1_dn;
  return afq_propagate_phaseless_jvp_ex(ctx, state, &in, tangent_workspace, tangent_workspace_bytes, fields, zetas,
                                        n_prop_steps, n_ene_blocks, n_sr_blocks, flags, block_energy, block_weight,
                                        dblock_energy, dblock_weight, energy, denergy, stream);
}

int afq_propagate_phaseless_jvp_ex(afq_ctx* ctx, afq_walker_state* state, const afq_jvp_inputs* in,
                                   void* tangent_workspace, size_t tangent_workspace_bytes, const double* fields,
                                   const double* zetas, int32_t n_prop_steps, int32_t n_ene_blocks,
                                   int32_t n_sr_blocks, int32_t flags, double* block_energy, double* block_weight,
                                   double* dblock_energy, double* dblock_weight, double* energy, double* denergy,
                                   void* stream) {
  if (!in) { afq_set_error("NULL argument"); return -1; }
  const double *dexp_h1_up = in->dexp_h1_up, *dexp_h1_dn = in->dexp_h1_dn, *drot_h1_up = in->drot_h1_up,
               *drot_h1_dn = in->drot_h1_dn;
  const bool do_sr = !(flags & AFQ_JVP_NO_SR);
  if (!ctx || !fields || (do_sr && !zetas) || !block_energy || !block_weight || !dblock_energy || !dblock_weight || !energy ||
      !denergy || !dexp_h1_up || !drot_h1_up) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (!is_fp64(ctx)) { afq_set_error("the derivative path needs an FP64 context"); return -1; }
  if (n_prop_steps < 1 || n_ene_blocks < 1 || n_sr_blocks < 1 || (!do_sr && n_sr_blocks != 1)) {
    afq_set_error("block counts must be >= 1 (n_sr_blocks == 1 without SR)");
    return -1;
  }
  if (flags & ~AFQ_JVP_NO_SR) { afq_set_error("unknown flags 0x%x", (unsigned)flags); return -1; }
  CHECK(check_state(ctx, state));
  const afq_ctx_dev& d = ctx->dev;
  if (d.nslab == 2 && !dexp_h1_dn) { afq_set_error("unrestricted walkers need dexp_h1_dn"); return -1; }
  if (d.nspin_g == 2 && !drot_h1_dn) { afq_set_error("the UHF trial needs drot_h1_dn"); return -1; }
  const bool rot = in->dtrial_up || in->drot_chol_up;
  if (rot && (!in->dtrial_up || !in->drot_chol_up ||
              (d.nspin_g == 2 && (!in->dtrial_dn || !in->drot_chol_dn)))) {
    afq_set_error("orbital rotation needs dtrial and drot_chol for every spin of the trial");
    return -1;
  }
  Layout L;
  const TSizes ts = tangent_sizes(d, ctx->nw_chunk, ctx->e_chunks, &L);
  if (!tangent_workspace || tangent_workspace_bytes < ts.total) {
    afq_set_error("tangent workspace too small: need %zu bytes, got %zu", ts.total, tangent_workspace_bytes);
    return -1;
  }
  if (reinterpret_cast<uintptr_t>(tangent_workspace) & 255) {
    afq_set_error("tangent workspace must be 256-byte aligned");
    return -1;
  }
  char* tw = static_cast<char*>(tangent_workspace);
  afq::TangentBufs t;
  for (int k = 0; k < 2; ++k) {
    t.dw[k] = reinterpret_cast<double2*>(tw + ts.dw[k]);
    t.wold[k] = reinterpret_cast<double2*>(tw + ts.wold[k]);
  }
  t.dgreen = reinterpret_cast<double2*>(tw + ts.dgreen);
  t.dfb = reinterpret_cast<double2*>(tw + ts.dfb);
  t.dxt = reinterpret_cast<double2*>(tw + ts.dxt);
  t.dshift = reinterpret_cast<double2*>(tw + ts.dshift);
  t.dfbt = reinterpret_cast<double2*>(tw + ts.dfbt);
  t.dvhs = reinterpret_cast<double2*>(tw + ts.dvhs);
  t.dlo = reinterpret_cast<double2*>(tw + ts.dlo);
  t.dlo_new = reinterpret_cast<double2*>(tw + ts.dlo_new);
  t.dweights = reinterpret_cast<double*>(tw + ts.dweights);
  t.dscalars = reinterpret_cast<double*>(tw + ts.dscalars);
  t.dene = reinterpret_cast<double2*>(tw + ts.dene);
  t.dpart = reinterpret_cast<double2*>(tw + ts.dpart);
  t.dsum = reinterpret_cast<double*>(tw + ts.dsum);
  t.dbe = dblock_energy;
  t.dbw = dblock_weight;
  t.dexp[0] = dexp_h1_up;
  t.dexp[1] = d.nslab == 2 ? dexp_h1_dn : dexp_h1_up;
  t.drot[0] = drot_h1_up;
  t.drot[1] = d.nspin_g == 2 ? drot_h1_dn : drot_h1_up;
  // the RHF trial serves both walker slabs: one trial tangent for both
  t.dtrial[0] = rot ? in->dtrial_up : nullptr;
  t.dtrial[1] = rot ? (d.nspin_g == 2 ? in->dtrial_dn : in->dtrial_up) : nullptr;
  t.drc[0] = rot ? in->drot_chol_up : nullptr;
  t.drc[1] = rot && d.nspin_g == 2 ? in->drot_chol_dn : nullptr;
  t.drccat = nullptr;
  cudaStream_t st = S(stream);
  // walker, weight, overlap and shift tangents start at zero (driver.py:190-200)
  {
    cudaError_t e = cudaMemsetAsync(tangent_workspace, 0, ts.total, st);
    if (e != cudaSuccess) { afq_set_error("tangent workspace clear: %s", cudaGetErrorString(e)); return (int)e; }
  }
  if (rot && d.nspin_g == 2) {  // [drot_chol_up[g] | drot_chol_dn[g]], the layout of rccat
    double* cat = reinterpret_cast<double*>(tw + ts.drccat);
    const size_t a = (size_t)d.gocc[0] * d.norb, b = (size_t)d.gocc[1] * d.norb;
    cudaError_t e = cudaMemcpy2DAsync(cat, d.ktot * sizeof(double), in->drot_chol_up, a * sizeof(double),
                                      a * sizeof(double), d.nchol, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(cat + a, d.ktot * sizeof(double), in->drot_chol_dn, b * sizeof(double),
                            b * sizeof(double), d.nchol, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) { afq_set_error("drot_chol concat: %s", cudaGetErrorString(e)); return (int)e; }
    t.drccat = cat;
  } else if (rot) {
    t.drccat = in->drot_chol_up;
  }
  double2* ovl = reinterpret_cast<double2*>(state->overlaps);
  const size_t welems[2] = {(size_t)d.nw * d.norb * d.kslab[0], (size_t)d.nw * d.norb * d.kslab[1]};
  void* wslab[2] = {state->walkers_up, state->walkers_dn};
  ctx->gstate = 0;
  CHECK(afq::t_launch_green(d, t, state->walkers_up, state->walkers_dn, nullptr, nullptr, ovl, t.dlo, st));
  CHECK(afq::launch_phaseless_begin(state->scalars, st));
  const size_t step_elems = (size_t)d.nw * d.nchol;
  int blk = 0;
  for (int sr = 0; sr < n_sr_blocks; ++sr) {
    for (int eb = 0; eb < n_ene_blocks; ++eb, ++blk) {
      for (int p = 0; p < n_prop_steps; ++p) {
        const double* f = fields + ((size_t)blk * n_prop_steps + p) * step_elems;
        CHECK(propagate_jvp(ctx, state, t, f, st));
      }
      for (int k = 0; k < d.nslab; ++k)
        CHECK(copy_d2d(t.wold[k], wslab[k], welems[k] * sizeof(double2), st, "walker copy before QR"));
      CHECK(qr_impl(ctx, state, st));
      CHECK(afq::t_launch_qr(d, t, state->walkers_up, state->walkers_dn, st));
      CHECK(afq::t_launch_green(d, t, state->walkers_up, state->walkers_dn, ctx->green, t.dgreen, ovl, t.dlo, st));
      CHECK(energy_from_green(ctx, ctx->ene, st));
      CHECK(afq::t_launch_energy(d, t, ctx->e_chunks, ctx->e_gchunk, ctx->green, st));
      CHECK(afq::launch_block_stats(d, ctx->ene, state->weights, state->scalars, block_energy + blk,
                                    block_weight + blk, st));
      CHECK(afq::t_launch_block_stats(d, t, ctx->ene, state->weights, state->scalars, block_energy + blk,
                                      dblock_energy + blk, dblock_weight + blk, st));
    }
    if (!do_sr) continue;
    CHECK(afq::t_launch_sr_pre(d, t, st));
    CHECK(sr_impl(ctx, state, zetas + sr, nullptr, st));
    CHECK(afq::t_launch_sr_post(d, t, ctx->sr_idx, st));
    CHECK(afq::t_launch_green(d, t, state->walkers_up, state->walkers_dn, nullptr, nullptr, ovl, t.dlo, st));
  }
  CHECK(afq::launch_phaseless_end(blk, (double)n_sr_blocks * n_ene_blocks * d.nw, block_energy, block_weight,
                                  state->scalars, energy, st));
  return afq::t_launch_end(blk, block_energy, block_weight, t, nullptr, denergy, st);
}

size_t afq_vjp_workspace_size(const afq_dims* dims, int32_t n_prop_steps, int32_t n_ene_blocks,
                              int32_t n_sr_blocks) {
  afq_ctx_dev c;
  int nwc, ec, eg;
  size_t we;
  if (n_prop_steps < 1 || n_ene_blocks < 1 || n_sr_blocks < 1) return 0;
  if (derive(dims, &c, &nwc, &ec, &eg, &we)) return 0;
  Layout L;
  return adjoint_sizes(c, nwc, n_prop_steps, n_ene_blocks, n_sr_blocks, &L).total;
}

int afq_propagate_phaseless_vjp(afq_ctx* ctx, afq_walker_state* state, void* vjp_workspace,
                                size_t vjp_workspace_bytes, const double* fields, const double* zetas,
                                int32_t n_prop_steps, int32_t n_ene_blocks, int32_t n_sr_blocks,
                                int32_t flags, double* block_energy, double* block_weight,
                                double* energy, double* gexp_h1_up, double* gexp_h1_dn,
                                double* grot_h1_up, double* grot_h1_dn, void* stream) {
  afq_vjp_outputs out;
  memset(&out, 0, sizeof(out));
  out.gexp_h1_up = gexp_h1_up;
  out.gexp_h1_dn = gexp_h1_dn;
  out.grot_h1_up = grot_h1_up;
  out.grot_h1_dn = grot_h1_dn;
  return afq_propagate_phaseless_vjp_ex(ctx, state, vjp_workspace, vjp_workspace_bytes, fields, zetas, n_prop_steps,
                                        n_ene_blocks, n_sr_blocks, flags, block_energy, block_weight, energy, &out,
                                        stream);
}

int afq_propagate_phaseless_vjp_ex(afq_ctx* ctx, afq_walker_state* state, void* vjp_workspace,
                                   size_t vjp_workspace_bytes, const double* fields, const double* zetas,
                                   int32_t n_prop_steps, int32_t n_ene_blocks, int32_t n_sr_blocks, int32_t flags,
                                   double* block_energy, double* block_weight, double* energy,
                                   const afq_vjp_outputs* out, void* stream) {
  if (!out) { afq_set_error("NULL argument"); return -1; }
  double *gexp_h1_up = out->gexp_h1_up, *gexp_h1_dn = out->gexp_h1_dn, *grot_h1_up = out->grot_h1_up,
         *grot_h1_dn = out->grot_h1_dn;
  const bool do_sr = !(flags & AFQ_JVP_NO_SR);
  if (!ctx || !fields || (do_sr && !zetas) || !block_energy || !block_weight || !energy || !gexp_h1_up ||
      !grot_h1_up) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (!is_fp64(ctx)) { afq_set_error("the derivative path needs an FP64 context"); return -1; }
  if (n_prop_steps < 1 || n_ene_blocks < 1 || n_sr_blocks < 1 || (!do_sr && n_sr_blocks != 1)) {
    afq_set_error("block counts must be >= 1 (n_sr_blocks == 1 without SR)");
    return -1;
  }
  if (flags & ~AFQ_JVP_NO_SR) { afq_set_error("unknown flags 0x%x", (unsigned)flags); return -1; }
  CHECK(check_state(ctx, state));
  const afq_ctx_dev& d = ctx->dev;
  if (d.nslab == 2 && !gexp_h1_dn) { afq_set_error("unrestricted walkers need gexp_h1_dn"); return -1; }
  if (d.nspin_g == 2 && !grot_h1_dn) { afq_set_error("the UHF trial needs grot_h1_dn"); return -1; }
  const bool rot = out->gtrial_up || out->grot_chol;
  if (rot && (!out->gtrial_up || !out->grot_chol || (d.nspin_g == 2 && !out->gtrial_dn))) {
    afq_set_error("orbital-rotation gradients need gtrial for every spin of the trial and grot_chol");
    return -1;
  }
  const int P = n_prop_steps, NE = n_ene_blocks;
  Layout L;
  const AdjSizes as = adjoint_sizes(d, ctx->nw_chunk, P, NE, n_sr_blocks, &L);
  if (!vjp_workspace || vjp_workspace_bytes < as.total) {
    afq_set_error("vjp workspace too small: need %zu bytes, got %zu", as.total, vjp_workspace_bytes);
    return -1;
  }
  if (reinterpret_cast<uintptr_t>(vjp_workspace) & 255) {
    afq_set_error("vjp workspace must be 256-byte aligned");
    return -1;
  }
  char* base = static_cast<char*>(vjp_workspace);
  const Tape tp{base, as, &d};
  afq::AdjointBufs a;
  const size_t e0 = (size_t)d.nw * d.norb * d.kslab[0];
  a.wb[0] = reinterpret_cast<double2*>(base + as.wb);
  a.wb[1] = a.wb[0] + e0;
  a.wb2[0] = reinterpret_cast<double2*>(base + as.wb2);
  a.wb2[1] = a.wb2[0] + e0;
  a.wbar = reinterpret_cast<double*>(base + as.wbar);
  a.lbar = reinterpret_cast<double2*>(base + as.lbar);
  a.lbar2 = reinterpret_cast<double2*>(base + as.lbar2);
  a.gpend = reinterpret_cast<double2*>(base + as.gpend);
  a.gene = reinterpret_cast<double2*>(base + as.gene);
  a.fbb = reinterpret_cast<double2*>(base + as.fbb);
  a.xtb = reinterpret_cast<double2*>(base + as.xtb);
  a.shb = reinterpret_cast<double2*>(base + as.shb);
  a.fbtb = reinterpret_cast<double2*>(base + as.fbtb);
  a.vbar = reinterpret_cast<double2*>(base + as.vbar);
  a.tay = reinterpret_cast<double2*>(base + as.tay);
  a.ebar = reinterpret_cast<double*>(base + as.ebar);
  a.scal = reinterpret_cast<double*>(base + as.scal);
  a.beb = reinterpret_cast<double*>(base + as.beb);
  a.bwb = reinterpret_cast<double*>(base + as.bwb);
  a.gexp[0] = gexp_h1_up;
  a.gexp[1] = d.nslab == 2 ? gexp_h1_dn : nullptr;
  a.grot[0] = grot_h1_up;
  a.grot[1] = d.nspin_g == 2 ? grot_h1_dn : nullptr;
  a.gtrial[0] = rot ? out->gtrial_up : nullptr;
  a.gtrial[1] = rot && d.nspin_g == 2 ? out->gtrial_dn : nullptr;
  a.grc = rot ? out->grot_chol : nullptr;
  double* const* gt = rot ? a.gtrial : nullptr;
  const bool cg = out->gchol != nullptr;
  if (cg && (!out->gmf_shifts || !out->gh0_prop)) {
    afq_set_error("Cholesky-vector gradients need gchol, gmf_shifts and gh0_prop");
    return -1;
  }
  a.gchol = cg ? out->gchol : nullptr;
  a.gmf = cg ? reinterpret_cast<double2*>(out->gmf_shifts) : nullptr;
  cudaStream_t st = S(stream);
  double2* ovl = reinterpret_cast<double2*>(state->overlaps);
  const size_t step_elems = (size_t)d.nw * d.nchol;

  // forward sweep: afq_propagate_phaseless's FP64 path, recording the state
  ctx->gstate = 0;
  CHECK(green(ctx, state->walkers_up, state->walkers_dn, nullptr, ovl, false, st));
  CHECK(afq::launch_phaseless_begin(state->scalars, st));
  int blk = 0;
  for (int sr = 0; sr < n_sr_blocks; ++sr) {
    for (int eb = 0; eb < NE; ++eb, ++blk) {
      for (int p = 0; p < P; ++p) {
        const int step = blk * P + p;
        CHECK(snapshot(tp, blk * (P + 2) + p, state, st));
        CHECK(propagate_impl(ctx, state, fields + (size_t)step * step_elems, st));
        CHECK(copy_d2d(tp.xt(step), ctx->xt, step_elems * sizeof(double2), st, "shifted-field record"));
        CHECK(copy_d2d(tp.sh(step), ctx->shift, d.nw * sizeof(double2), st, "shift record"));
        CHECK(copy_d2d(tp.fbt(step), ctx->fbt, d.nw * sizeof(double2), st, "fbt record"));
      }
      CHECK(snapshot(tp, blk * (P + 2) + P, state, st));
      CHECK(qr_impl(ctx, state, st));
      CHECK(green(ctx, state->walkers_up, state->walkers_dn, ctx->green, ovl, true, st));
      CHECK(snapshot(tp, blk * (P + 2) + P + 1, state, st));
      CHECK(energy_from_green(ctx, ctx->ene, st));
      CHECK(copy_d2d(tp.ene(blk), ctx->ene, d.nw * sizeof(double2), st, "local-energy record"));
      CHECK(afq::launch_block_stats(d, ctx->ene, state->weights, state->scalars, block_energy + blk,
                                    block_weight + blk, st));
    }
    if (!do_sr) continue;
    CHECK(sr_impl(ctx, state, zetas + sr, tp.idx(sr), st));
    CHECK(green(ctx, state->walkers_up, state->walkers_dn, nullptr, ovl, false, st));
  }
  CHECK(afq::launch_phaseless_end(blk, (double)n_sr_blocks * NE * d.nw, block_energy, block_weight,
                                  state->scalars, energy, st));

  // backward sweep, from the sampler total to the start of the first block
  CHECK(zero(base + as.wb, as.wslab * sizeof(double2), st));
  CHECK(zero(a.wbar, d.nw * sizeof(double), st));
  CHECK(zero(a.lbar, d.nw * sizeof(double2), st));
  CHECK(zero(a.scal, 8 * sizeof(double), st));
  CHECK(zero(gexp_h1_up, (size_t)d.norb * d.norb * sizeof(double), st));
  if (d.nslab == 2) CHECK(zero(gexp_h1_dn, (size_t)d.norb * d.norb * sizeof(double), st));
  CHECK(zero(grot_h1_up, (size_t)d.gocc[0] * d.norb * sizeof(double), st));
  if (d.nspin_g == 2) CHECK(zero(grot_h1_dn, (size_t)d.gocc[1] * d.norb * sizeof(double), st));
  if (rot) {
    for (int b = 0; b < d.nspin_g; ++b)
      CHECK(zero(a.gtrial[b], (size_t)d.norb * d.gocc[b] * sizeof(double), st));
    CHECK(zero(a.grc, (size_t)d.nchol * d.ktot * sizeof(double), st));
  }
  if (cg) {
    CHECK(zero(a.gchol, (size_t)d.nchol * d.norb * d.norb * sizeof(double), st));
    CHECK(zero(a.gmf, (size_t)d.nchol * sizeof(double2), st));
  }
  CHECK(afq::a_launch_end(blk, block_energy, block_weight, a, st));
  const int nwc = ctx->nw_chunk, nb = d.nw / nwc;
  const long nn = (long)d.norb * d.norb;
  const double sq = sqrt(d.dt);
  const double* brc = d.nspin_g == 2 ? ctx->rccat : d.rot_chol[0];
  const double alpha = d.energy_mode == 0 ? 2.0 : 1.0;
  bool gp = false;  // a.gpend holds the pending G cotangent of the current point
  for (int b = blk - 1; b >= 0; --b) {
    if (do_sr && b + 1 < blk && b % NE == NE - 1) {
      // the SR between blocks b and b + 1: finish the cotangent of its output walkers,
      // then send it back through the gather
      const int s0 = (b + 1) * (P + 2);
      CHECK(afq::a_launch_green(d, tp.w(s0, 0), tp.w(s0, 1), gp ? a.gpend : nullptr, nullptr, a.lbar, a.wb[0],
                                a.wb[1], st, gt));
      CHECK(afq::a_launch_sr(d, a, tp.idx(b / NE), st));
      swap_slabs(a.wb, a.wb2);
      CHECK(zero(a.lbar, d.nw * sizeof(double2), st));
      gp = false;
    }
    const int sq_i = b * (P + 2) + P + 1, sw_i = b * (P + 2) + P;
    CHECK(afq::a_launch_block_stats(d, a, b, tp.ene(b), tp.wt(sq_i), tp.sc(sq_i), block_energy, st));
    CHECK(afq::launch_green<double>(d, tp.w(sq_i, 0), tp.w(sq_i, 1), ctx->green, nullptr, true, st));
    CHECK(afq::a_launch_energy(d, a, ctx->green, st));
    if (rot) CHECK(afq::a_launch_rc_energy(d, a, ctx->green, st));
    CHECK(afq::a_launch_green(d, tp.w(sq_i, 0), tp.w(sq_i, 1), a.gene, gp ? a.gpend : nullptr, a.lbar, a.wb[0],
                              a.wb[1], st, gt));
    CHECK(zero(a.lbar, d.nw * sizeof(double2), st));
    gp = false;
    CHECK(afq::a_launch_qr(d, tp.w(sw_i, 0), tp.w(sw_i, 1), tp.w(sq_i, 0), tp.w(sq_i, 1), a.wb[0], a.wb[1],
                           a.wb2[0], a.wb2[1], st));
    swap_slabs(a.wb, a.wb2);
    for (int p = P - 1; p >= 0; --p) {
      const int post = b * (P + 2) + p + 1, start = b * (P + 2) + p, step = b * P + p;
      CHECK(afq::a_launch_weights(d, a, tp.sh(step), tp.fbt(step), tp.ov(post), tp.ov(start), tp.wt(start),
                                  tp.wt(post), tp.sc(start), st));
      CHECK(afq::a_launch_green(d, tp.w(post, 0), tp.w(post, 1), gp ? a.gpend : nullptr, nullptr, a.lbar, a.wb[0],
                                a.wb[1], st, gt));
      for (int k = 0; k < nb; ++k) {
        const int w0 = k * nwc;
        CHECK(afq::launch_gemm_cr(true, nwc, (int)nn, d.nchol, tp.xt(step) + (size_t)w0 * d.nchol, d.nchol,
                                  ctx->h.chol, nn, ctx->vhs, nn, c2(0.0, sq), st));
        CHECK(afq::a_launch_taylor(d, a, w0, nwc, ctx->vhs, tp.w(start, 0), tp.w(start, 1), st));
        if (cg) CHECK(afq::a_launch_chol_grad(d, a, nwc, tp.xt(step) + (size_t)w0 * d.nchol, st));
        CHECK(afq::launch_gemm_cr(false, nwc, d.nchol, (int)nn, a.vbar, nn, ctx->h.chol, nn,
                                  a.xtb + (size_t)w0 * d.nchol, d.nchol, c2(0.0, -sq), st));
      }
      CHECK(afq::a_launch_field(d, a, tp.xt(step), st));
      if (rot) {  // fb = alpha rot_chol G(W_start): rot_chol-bar += alpha Re(fb-bar^H G)
        CHECK(afq::launch_green<double>(d, tp.w(start, 0), tp.w(start, 1), ctx->green, nullptr, true, st));
        CHECK(afq::a_launch_rc_fb(d, a, ctx->green, alpha, st));
      }
      CHECK(afq::launch_gemm_cr(true, d.nw, d.ktot, d.nchol, a.fbb, d.nchol, brc, d.ktot, a.gpend, d.ktot,
                                c2(alpha, 0.0), st));
      gp = true;
      swap_slabs(a.wb, a.wb2);
      double2* t = a.lbar;
      a.lbar = a.lbar2;
      a.lbar2 = t;
    }
  }
  // the first step's G and the block's initial overlap were evaluated with the trial too
  if (rot)
    CHECK(afq::a_launch_green(d, tp.w(0, 0), tp.w(0, 1), gp ? a.gpend : nullptr, nullptr, a.lbar, a.wb[0], a.wb[1], st,
                              gt));
  if (cg) {  // h0_prop-bar = (scal[1], 0): only its real part enters the weights
    CHECK(zero(out->gh0_prop, 2 * sizeof(double), st));
    CHECK(copy_d2d(out->gh0_prop, a.scal + 1, sizeof(double), st, "h0_prop cotangent"));
  }
  return 0;
}

int afq_propagate_free(afq_ctx* ctx, afq_walker_state* state, const double* fields, double ene0, double* norms,
                       double* normed_overlaps, void* stream) {
  if (!ctx || !fields || !norms || !normed_overlaps) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_state(ctx, state));
  CHECK(check_free(ctx));
  return free_step(ctx, state, fields, ene0, reinterpret_cast<double2*>(norms),
                   reinterpret_cast<double2*>(normed_overlaps), S(stream));
}

int afq_propagate_free_blocks(afq_ctx* ctx, afq_walker_state* state, const double* fields, int32_t n_prop_steps,
                              int32_t n_blocks, double ene0, double* norms, double* normed_overlaps,
                              double* block_energy, double* block_weight, void* stream) {
  if (!ctx || !fields || !norms || !normed_overlaps || !block_energy || !block_weight) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (n_prop_steps < 1 || n_blocks < 1) { afq_set_error("block counts must be >= 1"); return -1; }
  CHECK(check_state(ctx, state));
  CHECK(check_free(ctx));
  cudaStream_t st = S(stream);
  const afq_ctx_dev& d = ctx->dev;
  double2* ovl = reinterpret_cast<double2*>(state->overlaps);
  CHECK(green(ctx, state->walkers_up, state->walkers_dn, nullptr, ovl, false, st));
  const size_t step_elems = (size_t)d.nw * d.nchol;
  for (int b = 0; b < n_blocks; ++b) {
    for (int p = 0; p < n_prop_steps; ++p)
      CHECK(free_step(ctx, state, fields + ((size_t)b * n_prop_steps + p) * step_elems, ene0,
                      reinterpret_cast<double2*>(norms), reinterpret_cast<double2*>(normed_overlaps), st));
    CHECK(green(ctx, state->walkers_up, state->walkers_dn, ctx->green, nullptr, true, st));
    CHECK(energy_from_green(ctx, ctx->ene, st));
    CHECK(afq::launch_free_block_stats(d.nw, ctx->ene, ovl, reinterpret_cast<double2*>(block_energy) + b,
                                       reinterpret_cast<double2*>(block_weight) + b, st));
  }
  return 0;
}

int afq_field_block(afq_ctx* ctx, afq_walker_state* state, const double* fields, int32_t n_prop_steps,
                    double* local_energies, double* block_energy, double* block_weight, void* stream) {
  if (!ctx || !fields || !block_energy || !block_weight) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (n_prop_steps < 1) {
    afq_set_error("n_prop_steps must be >= 1");
    return -1;
  }
  CHECK(check_state(ctx, state));
  cudaStream_t st = S(stream);
  const afq_ctx_dev& d = ctx->dev;
  const size_t step_elems = (size_t)d.nw * d.nchol;
  for (int p = 0; p < n_prop_steps; ++p) CHECK(propagate_impl(ctx, state, fields + p * step_elems, st));
  CHECK(qr_impl(ctx, state, st));
  CHECK(green(ctx, state->walkers_up, state->walkers_dn, ctx->green, reinterpret_cast<double2*>(state->overlaps),
              true, st));
  CHECK(energy_from_green(ctx, ctx->ene, st));
  CHECK(afq::launch_block_stats(d, ctx->ene, state->weights, state->scalars, block_energy, block_weight, st));
  if (local_energies) CHECK(afq::launch_clamped_energies(d, ctx->ene, state->scalars, local_energies, st));
  return 0;
}

int afq_cs_outlier_removal(double* weights1, double* weights2, const double* local_energies1,
                           const double* local_energies2, int32_t n_walkers, double z_thresh, double* sums,
                           void* stream) {
  if (!weights1 || !weights2 || !local_energies1 || !local_energies2 || !sums || n_walkers < 1) {
    afq_set_error("afq_cs_outlier_removal: bad arguments");
    return -1;
  }
  return afq::launch_cs_outlier(weights1, weights2, local_energies1, local_energies2, n_walkers, z_thresh, sums,
                                S(stream));
}

int afq_block_end(afq_ctx* ctx, afq_walker_state* state, const double* energy, const double* zeta,
                  double* block_weight, void* stream) {
  if (!ctx || !energy || !zeta || !block_weight) { afq_set_error("NULL argument"); return -1; }
  CHECK(check_state(ctx, state));
  cudaStream_t st = S(stream);
  CHECK(afq::launch_driver_update(ctx->dev, state->weights, energy, state->scalars, block_weight, st));
  CHECK(qr_impl(ctx, state, st));
  return sr_impl(ctx, state, zeta, nullptr, st);
}

int afq_cpmc_init(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers, const double* trial_up,
                  const double* trial_dn, double* walkers_up, double* walkers_dn, double* overlaps, double* greens,
                  void* stream) {
  if (!trial_up || !trial_dn || !walkers_up || !walkers_dn || !overlaps || !greens) {
    afq_set_error("NULL argument");
    return -1;
  }
  return afq::launch_cpmc(norb, n_up, n_dn, n_walkers, 1.0, 0.0, nullptr, nullptr, trial_up, trial_dn, walkers_up,
                          walkers_dn, nullptr, overlaps, greens, nullptr, nullptr, 0, S(stream));
}

int afq_cpmc_propagate(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers, double dt, double u,
                       const double* exp_h1_up, const double* exp_h1_dn, const double* trial_up,
                       const double* trial_dn, double* walkers_up, double* walkers_dn, double* weights,
                       double* overlaps, double* greens, double* scalars, const double* gaussian, void* stream) {
  if (!exp_h1_up || !exp_h1_dn || !trial_up || !trial_dn || !walkers_up || !walkers_dn || !weights || !overlaps ||
      !greens || !scalars || !gaussian) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (!(dt > 0.0)) { afq_set_error("dt must be positive"); return -1; }
  return afq::launch_cpmc(norb, n_up, n_dn, n_walkers, dt, u, exp_h1_up, exp_h1_dn, trial_up, trial_dn, walkers_up,
                          walkers_dn, weights, overlaps, greens, scalars, gaussian, 1, S(stream));
}

int afq_cpmc_nn_propagate(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers, double dt, double u,
                          double u_1, const int32_t* neighbors, int32_t n_pairs, const double* exp_h1_up,
                          const double* exp_h1_dn, const double* trial_up, const double* trial_dn,
                          double* walkers_up, double* walkers_dn, double* weights, double* overlaps,
                          double* greens, double* scalars, const double* uniforms, void* stream) {
  if (!exp_h1_up || !exp_h1_dn || !trial_up || !trial_dn || !walkers_up || !walkers_dn || !weights || !overlaps ||
      !greens || !scalars || !uniforms || (n_pairs > 0 && !neighbors) || n_pairs < 0) {
    afq_set_error("NULL argument or negative n_pairs");
    return -1;
  }
  if (!(dt > 0.0)) { afq_set_error("dt must be positive"); return -1; }
  return afq::launch_cpmc(norb, n_up, n_dn, n_walkers, dt, u, exp_h1_up, exp_h1_dn, trial_up, trial_dn, walkers_up,
                          walkers_dn, weights, overlaps, greens, scalars, nullptr, 3, S(stream), u_1, neighbors,
                          n_pairs, uniforms);
}

int afq_cpmc_continuous_propagate(int32_t norb, int32_t n_up, int32_t n_dn, int32_t n_walkers, double dt,
                                  double hs_constant, const double* exp_h1_up, const double* exp_h1_dn,
                                  const double* trial_up, const double* trial_dn, double* walkers_up,
                                  double* walkers_dn, double* weights, double* overlaps, double* scalars,
                                  const double* gaussian, void* stream) {
  if (!exp_h1_up || !exp_h1_dn || !trial_up || !trial_dn || !walkers_up || !walkers_dn || !weights || !overlaps ||
      !scalars || !gaussian) {
    afq_set_error("NULL argument");
    return -1;
  }
  if (!(dt > 0.0)) { afq_set_error("dt must be positive"); return -1; }
  return afq::launch_cpmc(norb, n_up, n_dn, n_walkers, dt, hs_constant, exp_h1_up, exp_h1_dn, trial_up, trial_dn,
                          walkers_up, walkers_dn, weights, overlaps, nullptr, scalars, gaussian, 2, S(stream));
}

int afq_fill_normal(double* out, int64_t n, uint64_t seed, uint64_t offset, void* stream) {
  if (!out && n > 0) { afq_set_error("NULL argument"); return -1; }
  return afq::launch_fill_normal(out, n, seed, offset, S(stream));
}

int afq_fill_uniform(double* out, int64_t n, uint64_t seed, uint64_t offset, void* stream) {
  if (!out && n > 0) { afq_set_error("NULL argument"); return -1; }
  return afq::launch_fill_uniform(out, n, seed, offset, S(stream));
}

}  // extern "C"

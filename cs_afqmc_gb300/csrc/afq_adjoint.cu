// Reverse-mode derivative (adjoint) of the FP64 phaseless block with respect to exp_h1 and
// rot_h1: the vjp that the reference's driver takes of sampler.propagate_phaseless_ad*_norot
// in ad_mode "reverse" (driver.py:217-229, sampling.py:266-317). The caller maps the two
// cotangents to d energy / d h1 (the block's one-body density matrix estimate).
//
// Convention: a complex intermediate z carries the cotangent zb = dL/dRe z + i dL/dIm z, so
// that dL = Re sum conj(zb) dz. A complex-linear map y = A x then has xb = A^H yb, and a real
// parameter p of such a map gets pb = Re(...). Every kernel here is the transpose of the
// corresponding tangent kernel of the forward mode, evaluated at the primal values of a
// recorded forward sweep. Clamped quantities (weights set to 0, local energies replaced by
// e_estimate) pass no cotangent, as jnp.where's transpose gives.

#include <math.h>

#include "afq_adjoint.cuh"
#include "afq_common.cuh"
#include "afq_prof.cuh"

namespace afq {

constexpr size_t kASmemMax = 227 * 1024 - 4096;  // opt-in shared memory per CTA, less the static arrays
constexpr int kAMaxPT = 16;                      // Taylor entries per thread: norb * k <= kAMaxPT * 256

static int a_smem(size_t bytes, const char* what) {
  if (bytes > kASmemMax) {
    afq_set_error("adjoint %s kernel: %zu bytes of shared memory needed, %zu available (norb * nocc too large)",
                  what, bytes, kASmemMax);
    return -2;
  }
  return 0;
}

static int a_err(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    afq_set_error("%s: %s", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

// Gauss-Jordan inverse of the o x o matrix in the left half of Aug [o][2o] (right half set
// to the identity by the caller), |re|+|im| partial pivoting as the value kernels use.
// Leaves S^-1 in the right half.
__device__ void gj_inverse(double2* Aug, int o, int* piv_sh, double2* colj) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int j = 0; j < o; ++j) {
    if (tid < 32) {
      double best = -1.0;
      int bi = j;
      for (int r = j + tid; r < o; r += 32) {
        const double2 v = Aug[r * 2 * o + j];
        const double m = fabs(v.x) + fabs(v.y);
        if (m > best) { best = m; bi = r; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) *piv_sh = bi;
    }
    __syncthreads();
    const int pr = *piv_sh;
    if (pr != j)
      for (int e = tid; e < 2 * o; e += nt) {
        const double2 t = Aug[j * 2 * o + e];
        Aug[j * 2 * o + e] = Aug[pr * 2 * o + e];
        Aug[pr * 2 * o + e] = t;
      }
    __syncthreads();
    const double2 inv = cdiv(c2(1.0, 0.0), Aug[j * 2 * o + j]);
    __syncthreads();
    for (int e = tid; e < 2 * o; e += nt) Aug[j * 2 * o + e] = cmul(Aug[j * 2 * o + e], inv);
    for (int r = tid; r < o; r += nt) colj[r] = Aug[r * 2 * o + j];
    __syncthreads();
    for (int e = tid; e < o * 2 * o; e += nt) {
      const int r = e / (2 * o), col = e % (2 * o);
      if (r == j) continue;
      Aug[e] = csub(Aug[e], cmul(colj[r], Aug[j * 2 * o + col]));
    }
    __syncthreads();
  }
}

// ======================================================================================
// Sampler total and block statistics (sampling.py:79-91, 337-341).
// energy = sum E_b w_b / sum w_b: E_b-bar = w_b / sum w, w_b-bar = (E_b - energy) / sum w.
// Block b: E_b = sum e w / sum w over clamped local energies, w_b = sum w, and the shift
// update E_pc <- 0.9 E_pc + 0.1 E_b, transposed with the running shift cotangent scal[0].
// ======================================================================================

__global__ void k_a_end(int nblk, const double* __restrict__ be, const double* __restrict__ bw,
                        double* __restrict__ beb, double* __restrict__ bwb) {
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < nblk; ++i) {
      a += be[i] * bw[i];
      b += bw[i];
    }
    const double e = a / b;
    for (int i = 0; i < nblk; ++i) {
      beb[i] = bw[i] / b;
      bwb[i] = (be[i] - e) / b;
    }
  }
}

__global__ void k_a_block_stats(int nw, double dt, const double2* __restrict__ energy,
                                const double* __restrict__ weights, const double* __restrict__ scalars,
                                const double* __restrict__ be, const double* __restrict__ beb,
                                const double* __restrict__ bwb, double* __restrict__ scal,
                                double* __restrict__ ebar, double* __restrict__ wbar) {
  __shared__ double red[32];
  const double epc = scal[0];
  const double ebt = beb[0] + 0.1 * epc;  // the block energy feeds the total and the shift
  const double e_est = scalars[AFQ_S_E_ESTIMATE], lim = sqrt(2.0 / dt), eb = be[0], wb = bwb[0];
  double sw = 0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) sw += weights[w];
  sw = block_sum(sw, red);
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    const double e = energy[w].x;
    const bool cl = fabs(e - e_est) > lim;
    const double ec = cl ? e_est : e;
    ebar[w] = cl ? 0.0 : ebt * weights[w] / sw;
    wbar[w] += ebt * (ec - eb) / sw + wb;
  }
  if (threadIdx.x == 0) scal[0] = 0.9 * epc;
}

// ======================================================================================
// Local-energy adjoint (wavefunctions.py:529-561, 711-743). With f_g = RC_g G^T and
// c_g = tr f_g, the two-body energy is gamma/2 sum c^2 + kappa/2 sum f_g[i,k] f_g[k,i]
// (RHF restricted: gamma 4, kappa -2; RHF two-slab: 2, -2; UHF: (c_up + c_dn)^2 with
// gamma 1 per spin and kappa -1), so
//   G_s-bar = e-bar (kappa conj(f_s) + gamma conj(c) I) RC_s summed over g,
// plus mult1 e-bar rot_h1 from the one-body term. One CTA per walker, g in sequence.
// ======================================================================================

__global__ void __launch_bounds__(256) k_a_energy(const afq_ctx_dev c, const double2* __restrict__ green,
                                                  const double* __restrict__ ebar, double2* __restrict__ gene) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = blockIdx.x, norb = c.norb, tid = threadIdx.x, nt = blockDim.x, om = c.kmax;
  double2* Gs = reinterpret_cast<double2*>(smem_raw);  // [ktot]
  double2* Gb = Gs + c.ktot;                           // [ktot]
  double2* F = Gb + c.ktot;                            // [2][om*om]
  const double eb = ebar[w];
  double2* out = gene + (size_t)w * c.ktot;
  if (eb == 0.0) {  // clamped or dead walker: no cotangent
    for (int i = tid; i < c.ktot; i += nt) out[i] = c2(0, 0);
    return;
  }
  for (int i = tid; i < c.ktot; i += nt) {
    Gs[i] = green[(size_t)w * c.ktot + i];
    Gb[i] = c2(0, 0);
  }
  __syncthreads();
  const double kappa = c.energy_mode == 2 ? -1.0 : -2.0;
  const double gamma = c.energy_mode == 0 ? 4.0 : (c.energy_mode == 1 ? 2.0 : 1.0);
  for (int g = 0; g < c.nchol; ++g) {
    for (int s = 0; s < c.nspin_g; ++s) {
      const int o = c.gocc[s];
      const double* RC = c.rot_chol[s] + (size_t)g * o * norb;
      const double2* Gsp = Gs + (size_t)s * c.gocc[0] * norb;
      double2* Fs = F + s * om * om;
      for (int e = tid; e < o * o; e += nt) {
        const int i = e / o, k = e % o;
        const double* rr = RC + (size_t)i * norb;
        const double2* gg = Gsp + (size_t)k * norb;
        double2 a = c2(0, 0);
        for (int p = 0; p < norb; ++p) {
          a.x = fma(rr[p], gg[p].x, a.x);
          a.y = fma(rr[p], gg[p].y, a.y);
        }
        Fs[e] = a;
      }
    }
    __syncthreads();
    double2 ct = c2(0, 0);
    for (int s = 0; s < c.nspin_g; ++s)
      for (int i = 0; i < c.gocc[s]; ++i) ct = cadd(ct, F[s * om * om + i * c.gocc[s] + i]);
    const double2 cg = cscale(cconj(ct), gamma);
    for (int s = 0; s < c.nspin_g; ++s) {
      const int o = c.gocc[s];
      const double* RC = c.rot_chol[s] + (size_t)g * o * norb;
      const double2* Fs = F + s * om * om;
      double2* Gbs = Gb + (size_t)s * c.gocc[0] * norb;
      for (int e = tid; e < o * norb; e += nt) {
        const int k = e / norb, p = e % norb;
        double2 a = c2(0, 0);
        for (int i = 0; i < o; ++i) {
          double2 m = cscale(cconj(Fs[k * o + i]), kappa);
          if (i == k) m = cadd(m, cg);
          const double r = RC[(size_t)i * norb + p];
          a.x = fma(m.x, r, a.x);
          a.y = fma(m.y, r, a.y);
        }
        Gbs[e] = cadd(Gbs[e], a);
      }
    }
    __syncthreads();
  }
  const double mult1 = c.energy_mode == 0 ? 2.0 : 1.0;
  for (int i = tid; i < c.ktot; i += nt) {
    const int s = (c.nspin_g == 2 && i >= c.gocc[0] * norb) ? 1 : 0;
    const double r = c.rot_h1[s][i - s * c.gocc[0] * norb];
    out[i] = c2(eb * (Gb[i].x + mult1 * r), eb * Gb[i].y);
  }
}

// rot_h1-bar += mult1 sum_w e-bar_w Re G_w, one thread per element of the Green blocks
__global__ void k_a_rot(const afq_ctx_dev c, const double2* __restrict__ green, const double* __restrict__ ebar,
                        double* gr_up, double* gr_dn) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= c.ktot) return;
  const int s = (c.nspin_g == 2 && e >= c.gocc[0] * c.norb) ? 1 : 0;
  double a = 0;
  for (int w = 0; w < c.nw; ++w) {
    const double eb = ebar[w];
    if (eb != 0.0) a += eb * green[(size_t)w * c.ktot + e].x;
  }
  double* out = s == 0 ? gr_up : gr_dn;
  out[e - s * c.gocc[0] * c.norb] += (c.energy_mode == 0 ? 2.0 : 1.0) * a;
}

// ======================================================================================
// Green's-function and overlap adjoint (wavefunctions.py:478-501, 658-692). Per slab:
// S = C^T W, G^T = W S^-1, log overlap = mult log det S. With B = (G-bar)^T:
//   W-bar += B S^-H + C S^-H (mult l-bar I - W^H B S^-H).
// G-bar = ga + gb (either may be NULL), l-bar may be NULL. One CTA per walker.
// ======================================================================================

__global__ void __launch_bounds__(256) k_a_green(const afq_ctx_dev c, const double2* __restrict__ w_up,
                                                 const double2* __restrict__ w_dn, const double2* __restrict__ ga,
                                                 const double2* __restrict__ gb, const double2* __restrict__ lbar,
                                                 double2* __restrict__ wb_up, double2* __restrict__ wb_dn,
                                                 double* gt_up, double* gt_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wlk = blockIdx.x, norb = c.norb, tid = threadIdx.x, nt = blockDim.x, km = c.kmax;
  double2* Ws = reinterpret_cast<double2*>(smem_raw);  // [norb][km]
  double2* Bs = Ws + (size_t)norb * km;                // [norb][km]
  double2* Xs = Bs + (size_t)norb * km;                // [norb][km]
  double2* Aug = Xs + (size_t)norb * km;               // [km][2 km]
  double2* Ys = Aug + (size_t)km * 2 * km;             // [km][km]
  double2* Zs = Ys + (size_t)km * km;                  // [km][km]
  double* Cs = reinterpret_cast<double*>(Zs + (size_t)km * km);  // [norb][km]
  __shared__ int piv_sh;
  __shared__ double2 colj[64];
  const int mult = (c.nslab == 1 && c.restricted_square) ? 2 : 1;
  const double2 lb = lbar ? cscale(lbar[wlk], (double)mult) : c2(0, 0);
  const bool has_g = ga || gb;
  for (int s = 0; s < c.nslab; ++s) {
    const int ks = c.kslab[s], o = c.nocc_slab[s];
    const double2* W = (s == 0 ? w_up : w_dn) + (size_t)wlk * norb * ks;
    double2* Wb = (s == 0 ? wb_up : wb_dn) + (size_t)wlk * norb * ks;
    const double* C = c.trial[s];
    const size_t gofs = (size_t)wlk * c.ktot + (size_t)((c.nspin_g == 2) ? s : 0) * c.nocc_slab[0] * norb;
    for (int i = tid; i < norb * o; i += nt) {
      const int p = i / o, k = i % o;
      Ws[i] = W[(size_t)p * ks + k];
      Cs[i] = C[(size_t)p * o + k];
      double2 b = c2(0, 0);
      if (ga) b = cadd(b, ga[gofs + (size_t)k * norb + p]);
      if (gb) b = cadd(b, gb[gofs + (size_t)k * norb + p]);
      Bs[i] = b;
    }
    __syncthreads();
    for (int e = tid; e < o * o; e += nt) {
      const int i = e / o, k = e % o;
      double2 a = c2(0, 0);
      for (int p = 0; p < norb; ++p) {
        const double cv = Cs[p * o + i];
        a.x += cv * Ws[p * o + k].x;
        a.y += cv * Ws[p * o + k].y;
      }
      Aug[i * 2 * o + k] = a;
      Aug[i * 2 * o + o + k] = c2(i == k ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    gj_inverse(Aug, o, &piv_sh, colj);
    // X = B S^-H: X[p,j] = sum_i B[p,i] conj(S^-1[j,i])
    for (int e = tid; e < norb * o; e += nt) {
      const int p = e / o, j = e % o;
      double2 a = c2(0, 0);
      if (has_g)
        for (int i = 0; i < o; ++i) a = cadd(a, cmulc(Bs[p * o + i], Aug[j * 2 * o + o + i]));
      Xs[e] = a;
    }
    __syncthreads();
    // Y = mult l-bar I - W^H X
    for (int e = tid; e < o * o; e += nt) {
      const int i = e / o, j = e % o;
      double2 a = c2(0, 0);
      if (has_g)
        for (int p = 0; p < norb; ++p) a = cadd(a, cmulc(Xs[p * o + j], Ws[p * o + i]));
      Ys[e] = csub(i == j ? lb : c2(0, 0), a);
    }
    __syncthreads();
    // Z = S^-H Y: Z[i,j] = sum_k conj(S^-1[k,i]) Y[k,j]
    for (int e = tid; e < o * o; e += nt) {
      const int i = e / o, j = e % o;
      double2 a = c2(0, 0);
      for (int k = 0; k < o; ++k) a = cadd(a, cmulc(Ys[k * o + j], Aug[k * 2 * o + o + i]));
      Zs[e] = a;
    }
    __syncthreads();
    for (int e = tid; e < norb * o; e += nt) {
      const int p = e / o, j = e % o;
      double2 a = Xs[e];
      for (int i = 0; i < o; ++i) {
        const double cv = Cs[p * o + i];
        a.x = fma(cv, Zs[i * o + j].x, a.x);
        a.y = fma(cv, Zs[i * o + j].y, a.y);
      }
      const size_t gi = (size_t)p * ks + j;
      Wb[gi] = cadd(Wb[gi], a);
    }
    // orbital rotation: S = C^T W, so C-bar[p][i] += Re sum_k W[p][k] conj(S-bar[i][k]) with
    // S-bar = Z; the RHF trial serves both slabs
    double* gt = s == 0 ? gt_up : gt_dn;
    if (gt)
      for (int e = tid; e < norb * o; e += nt) {
        const int p = e / o, i = e % o;
        double a = 0.0;
        for (int k = 0; k < o; ++k) a += Ws[p * o + k].x * Zs[i * o + k].x + Ws[p * o + k].y * Zs[i * o + k].y;
        atomicAdd(gt + (size_t)p * o + i, a);
      }
    __syncthreads();
  }
}

// ======================================================================================
// QR adjoint (linalg_utils.py:51-65), the transpose of the tangent dQ = X - Q U(Q^H X),
// X = dW R^-1: with M = Q^H Q-bar and C-bar = triu(M, 1) + triu(M, 1)^H + Re diag(M),
// W-bar = (Q-bar - Q C-bar) R^-H, R = Q^H W. One CTA per (walker, slab).
// ======================================================================================

__global__ void __launch_bounds__(256) k_a_qr(const afq_ctx_dev c, const double2* __restrict__ wold_up,
                                              const double2* __restrict__ wold_dn,
                                              const double2* __restrict__ q_up, const double2* __restrict__ q_dn,
                                              const double2* __restrict__ qb_up, const double2* __restrict__ qb_dn,
                                              double2* __restrict__ ob_up, double2* __restrict__ ob_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wlk = blockIdx.x, s = blockIdx.y;
  const int m = c.norb, k = c.kslab[s], tid = threadIdx.x, nt = blockDim.x;
  double2* Q = reinterpret_cast<double2*>(smem_raw);  // [m][k]
  double2* X = Q + (size_t)m * k;                      // [m][k]
  double2* R = X + (size_t)m * k;                      // [k][k]
  double2* Mm = R + (size_t)k * k;                     // [k][k]
  double2* Cb = Mm + (size_t)k * k;                    // [k][k]
  const size_t off = (size_t)wlk * m * k;
  const double2* Wo = (s == 0 ? wold_up : wold_dn) + off;
  const double2* Qg = (s == 0 ? q_up : q_dn) + off;
  const double2* Qb = (s == 0 ? qb_up : qb_dn) + off;
  double2* Ob = (s == 0 ? ob_up : ob_dn) + off;
  for (int i = tid; i < m * k; i += nt) {
    Q[i] = Qg[i];
    X[i] = Qb[i];
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += nt) {
    const int i = e / k, j = e % k;
    double2 r = c2(0, 0), a = c2(0, 0);
    for (int p = 0; p < m; ++p) {
      r = cadd(r, cmulc(Wo[(size_t)p * k + j], Q[p * k + i]));
      a = cadd(a, cmulc(X[p * k + j], Q[p * k + i]));
    }
    R[e] = r;
    Mm[e] = a;
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += nt) {
    const int i = e / k, j = e % k;
    double2 v;
    if (i < j) v = Mm[e];
    else if (i > j) v = cconj(Mm[j * k + i]);
    else v = c2(Mm[e].x, 0.0);
    Cb[e] = v;
  }
  __syncthreads();
  for (int e = tid; e < m * k; e += nt) {  // X-bar = Q-bar - Q C-bar
    const int p = e / k, j = e % k;
    double2 a = X[e];
    for (int i = 0; i < k; ++i) a = csub(a, cmul(Q[p * k + i], Cb[i * k + j]));
    X[e] = a;
  }
  __syncthreads();
  for (int p = tid; p < m; p += nt) {  // W-bar R^H = X-bar, row by row, last column first
    for (int j = k - 1; j >= 0; --j) {
      double2 a = X[p * k + j];
      for (int l = j + 1; l < k; ++l) a = csub(a, cmulc(X[p * k + l], R[j * k + l]));
      X[p * k + j] = cdiv(a, cconj(R[j * k + j]));
    }
  }
  __syncthreads();
  for (int i = tid; i < m * k; i += nt) Ob[i] = X[i];
}

// ======================================================================================
// Phaseless weights and population control, transposed (propagation.py:133-163). One CTA.
// v = exp(Re arg) Re(u), u = exp(i Im(-sqrt(dt) shift)) O'/O, w' = v w; the shift
// E_pc' = e_estimate - 0.1 log(sum w' / nw) / dt after the step. With v-bar = w w'-bar:
// a = v-bar v, b = -v-bar exp(Re arg) Im(u);
//   shift-bar = -sqrt(dt) (a + i b), fbt-bar = a, E_pc-bar = dt sum a,
//   log O'-bar += a + i b, log O-bar = -(a + i b), w-bar = v w'-bar.
// ======================================================================================

__global__ void k_a_weights(int nw, double dt, double2 h0_prop, const double2* __restrict__ shift,
                            const double2* __restrict__ fbt, const double2* __restrict__ ovl_new,
                            const double2* __restrict__ ovl, const double* __restrict__ w_start,
                            const double* __restrict__ w_post, const double* __restrict__ scalars,
                            double* __restrict__ scal, double* __restrict__ wbar, double2* __restrict__ shb,
                            double2* __restrict__ fbtb, double2* __restrict__ lbar,
                            double2* __restrict__ lbar_start) {
  __shared__ double red[32];
  const double epc_bar = scal[0];
  double sw = 0;
  for (int k = threadIdx.x; k < nw; k += blockDim.x) sw += w_post[k];
  sw = block_sum(sw, red);
  const double pc = -0.1 * epc_bar / (dt * sw);
  const double sqdt = sqrt(dt), pcs = scalars[AFQ_S_POP_CONTROL_SHIFT];
  double sa = 0;
  for (int k = threadIdx.x; k < nw; k += blockDim.x) {
    const double wbp = wbar[k] + pc;
    const double2 ratio = cdiv(ovl_new[k], ovl[k]);
    const double2 sh = shift[k], fb = fbt[k];
    const double re_arg = -sqdt * sh.x + fb.x + dt * (pcs + h0_prop.x);
    double sn, cs;
    sincos(-sqdt * sh.y, &sn, &cs);
    const double ex = exp(re_arg);
    const double v = ex * (cs * ratio.x - sn * ratio.y);
    const bool cl = isnan(v) || v < 1.0e-3 || v > 100.0;
    const double vv = cl ? 0.0 : v;
    const bool cl2 = vv * w_start[k] > 100.0;
    double ws_bar = 0.0, vbar = 0.0;
    if (!cl2) {
      ws_bar = vv * wbp;
      if (!cl) vbar = w_start[k] * wbp;
    }
    double a = 0.0, b = 0.0;
    if (vbar != 0.0) {
      a = vbar * v;
      b = -vbar * ex * (sn * ratio.x + cs * ratio.y);
    }
    shb[k] = c2(-sqdt * a, -sqdt * b);
    fbtb[k] = c2(a, 0.0);
    lbar[k] = cadd(lbar[k], c2(a, b));
    lbar_start[k] = c2(-a, -b);
    wbar[k] = ws_bar;
    sa += dt * a;
  }
  sa = block_sum(sa, red);
  if (threadIdx.x == 0) {
    scal[0] = sa;
    scal[1] += sa;  // arg holds dt (E_pc + Re h0_prop): the same sum is h0_prop's cotangent
  }
}

// ======================================================================================
// Taylor propagator adjoint (propagation.py:67-92). Forward: P_0 = E W, P_m = V P_{m-1},
// acc = sum_m P_m / m!, W' = E acc. Backward from W'-bar: acc-bar = E^T W'-bar,
// P_M-bar = acc-bar / M!, P_m-bar = acc-bar / m! + V^H P_{m+1}-bar, W-bar = E^T P_0-bar.
// The kernel recomputes the chain and leaves P_0..P_{M-1}, P_1-bar..P_M-bar, acc and
// P_0-bar in the scratch (terms 0..M-1, M..2M-1, 2M, 2M+1) for the vhs and exp_h1
// cotangents. One CTA per (walker of the chunk, slab).
// ======================================================================================

__global__ void __launch_bounds__(256) k_a_taylor(const afq_ctx_dev c, int w0, const double2* __restrict__ vhs,
                                                  const double2* __restrict__ wu, const double2* __restrict__ wd,
                                                  const double2* __restrict__ gu, const double2* __restrict__ gd,
                                                  double2* __restrict__ tay, double2* __restrict__ ou,
                                                  double2* __restrict__ od) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wl = blockIdx.x, s = blockIdx.y, wlk = w0 + wl;
  const int norb = c.norb, ks = c.kslab[s], n = norb * ks, tid = threadIdx.x, nt = blockDim.x;
  const int M = c.n_exp_terms - 1, T = 2 * M + 2;
  const size_t nk = (size_t)norb * (c.kslab[0] + c.kslab[1]);
  double2* tw = tay + (size_t)wl * T * nk + (s == 1 ? (size_t)norb * c.kslab[0] : 0);
  double2* A = reinterpret_cast<double2*>(smem_raw);
  double2* B = A + n;
  const double* E = c.exp_h1[s];
  const double2* V = vhs + (size_t)wl * norb * norb;
  const double2* W = (s == 0 ? wu : wd) + (size_t)wlk * n;
  const double2* Gb = (s == 0 ? gu : gd) + (size_t)wlk * n;
  double2* O = (s == 0 ? ou : od) + (size_t)wlk * n;
  for (int i = tid; i < n; i += nt) A[i] = W[i];
  __syncthreads();
  double2 acc[kAMaxPT];
#pragma unroll
  for (int j = 0; j < kAMaxPT; ++j) {
    const int i = tid + j * nt;
    acc[j] = c2(0, 0);
    if (i < n) {
      const int p = i / ks, col = i % ks;
      double2 a = c2(0, 0);
      for (int q = 0; q < norb; ++q) {
        const double e = E[(size_t)p * norb + q];
        const double2 t = A[q * ks + col];
        a.x = fma(e, t.x, a.x);
        a.y = fma(e, t.y, a.y);
      }
      B[i] = a;
      acc[j] = a;
      if (M > 0) tw[i] = a;
    }
  }
  __syncthreads();
  double fact = 1.0;
  double2 *src = B, *dst = A;
  for (int m = 1; m <= M; ++m) {
    fact *= (double)m;
    const double invf = 1.0 / fact;
#pragma unroll
    for (int j = 0; j < kAMaxPT; ++j) {
      const int i = tid + j * nt;
      if (i < n) {
        const int p = i / ks, col = i % ks;
        const double2* Vr = V + (size_t)p * norb;
        double2 a = c2(0, 0);
        for (int q = 0; q < norb; ++q) a = cadd(a, cmul(Vr[q], src[q * ks + col]));
        dst[i] = a;
        acc[j] = cadd(acc[j], cscale(a, invf));
        if (m < M) tw[(size_t)m * nk + i] = a;
      }
    }
    __syncthreads();
    double2* t = src; src = dst; dst = t;
  }
#pragma unroll
  for (int j = 0; j < kAMaxPT; ++j) {
    const int i = tid + j * nt;
    if (i < n) tw[(size_t)(2 * M) * nk + i] = acc[j];
  }
  for (int i = tid; i < n; i += nt) A[i] = Gb[i];
  __syncthreads();
  double2 accb[kAMaxPT];
  const double invfM = 1.0 / fact;  // 1 / M!
#pragma unroll
  for (int j = 0; j < kAMaxPT; ++j) {
    const int i = tid + j * nt;
    accb[j] = c2(0, 0);
    if (i < n) {
      const int p = i / ks, col = i % ks;
      double2 a = c2(0, 0);
      for (int q = 0; q < norb; ++q) {
        const double e = E[(size_t)q * norb + p];
        const double2 t = A[q * ks + col];
        a.x = fma(e, t.x, a.x);
        a.y = fma(e, t.y, a.y);
      }
      accb[j] = a;
      const double2 top = cscale(a, invfM);
      B[i] = top;
      tw[(size_t)(M > 0 ? 2 * M - 1 : 2 * M + 1) * nk + i] = top;
    }
  }
  __syncthreads();
  src = B;
  dst = A;
  double invf = invfM;
  for (int m = M - 1; m >= 0; --m) {
    invf *= (double)(m + 1);  // 1 / m!
#pragma unroll
    for (int j = 0; j < kAMaxPT; ++j) {
      const int i = tid + j * nt;
      if (i < n) {
        const int p = i / ks, col = i % ks;
        double2 a = cscale(accb[j], invf);
        for (int q = 0; q < norb; ++q) a = cadd(a, cmulc(src[q * ks + col], V[(size_t)q * norb + p]));
        dst[i] = a;
        tw[(size_t)(m >= 1 ? M + m - 1 : 2 * M + 1) * nk + i] = a;
      }
    }
    __syncthreads();
    double2* t = src; src = dst; dst = t;
  }
  for (int i = tid; i < n; i += nt) {
    const int p = i / ks, col = i % ks;
    double2 a = c2(0, 0);
    for (int q = 0; q < norb; ++q) {
      const double e = E[(size_t)q * norb + p];
      const double2 t = src[q * ks + col];
      a.x = fma(e, t.x, a.x);
      a.y = fma(e, t.y, a.y);
    }
    O[i] = a;
  }
}

// exp_h1-bar[p][q] += sum_w sum_c Re(W'-bar[p,c] conj(acc[q,c]) + P_0-bar[p,c] conj(W[q,c]))
// over the walkers of the chunk. CTA per (16 x 16 tile, slab), walkers in sequence.
__global__ void __launch_bounds__(256) k_a_exp_grad(const afq_ctx_dev c, int w0, int nwc,
                                                    const double2* __restrict__ gu, const double2* __restrict__ gd,
                                                    const double2* __restrict__ tay, const double2* __restrict__ wu,
                                                    const double2* __restrict__ wd, double* ge_up, double* ge_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = blockIdx.z, norb = c.norb, ks = c.kslab[s], n = norb * ks;
  const int p0 = blockIdx.y * 16, q0 = blockIdx.x * 16, tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int M = c.n_exp_terms - 1, T = 2 * M + 2;
  const size_t nk = (size_t)norb * (c.kslab[0] + c.kslab[1]);
  double2* X1 = reinterpret_cast<double2*>(smem_raw);  // [16][ks]
  double2* Y1 = X1 + 16 * ks;
  double2* X2 = Y1 + 16 * ks;
  double2* Y2 = X2 + 16 * ks;
  double sum = 0;
  for (int wl = 0; wl < nwc; ++wl) {
    const double2* gcot = (s == 0 ? gu : gd) + (size_t)(w0 + wl) * n;
    const double2* wst = (s == 0 ? wu : wd) + (size_t)(w0 + wl) * n;
    const double2* tb = tay + (size_t)wl * T * nk + (s == 1 ? (size_t)norb * c.kslab[0] : 0);
    for (int e = tid; e < 16 * ks; e += 256) {
      const int r = e / ks, col = e % ks;
      const int p = p0 + r, q = q0 + r;
      X1[e] = p < norb ? gcot[(size_t)p * ks + col] : c2(0, 0);
      X2[e] = p < norb ? tb[(size_t)(2 * M + 1) * nk + (size_t)p * ks + col] : c2(0, 0);
      Y1[e] = q < norb ? tb[(size_t)(2 * M) * nk + (size_t)q * ks + col] : c2(0, 0);
      Y2[e] = q < norb ? wst[(size_t)q * ks + col] : c2(0, 0);
    }
    __syncthreads();
    for (int col = 0; col < ks; ++col) {
      const double2 a = X1[ty * ks + col], b = Y1[tx * ks + col];
      const double2 a2 = X2[ty * ks + col], b2 = Y2[tx * ks + col];
      sum += a.x * b.x + a.y * b.y + a2.x * b2.x + a2.y * b2.y;
    }
    __syncthreads();
  }
  const int p = p0 + ty, q = q0 + tx;
  if (p < norb && q < norb) (s == 0 ? ge_up : ge_dn)[(size_t)p * norb + q] += sum;
}

// vhs-bar[w][p][q] = sum_slabs sum_{m=1..M} sum_c P_m-bar[p,c] conj(P_{m-1}[q,c]).
// CTA per (32 x 32 tile, walker of the chunk); c staged through shared memory 16 at a time.
__global__ void __launch_bounds__(256) k_a_vbar(const afq_ctx_dev c, const double2* __restrict__ tay,
                                                double2* __restrict__ vbar) {
  __shared__ double2 Qt[32][17];
  __shared__ double2 Pt[32][17];
  const int wl = blockIdx.z, norb = c.norb, p0 = blockIdx.y * 32, q0 = blockIdx.x * 32;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const int M = c.n_exp_terms - 1, T = 2 * M + 2;
  const size_t nk = (size_t)norb * (c.kslab[0] + c.kslab[1]);
  double2 acc[4] = {c2(0, 0), c2(0, 0), c2(0, 0), c2(0, 0)};
  for (int s = 0; s < c.nslab; ++s) {
    const int ks = c.kslab[s];
    const double2* tb = tay + (size_t)wl * T * nk + (s == 1 ? (size_t)norb * c.kslab[0] : 0);
    for (int m = 1; m <= M; ++m) {
      const double2* Qm = tb + (size_t)(M + m - 1) * nk;
      const double2* Pm = tb + (size_t)(m - 1) * nk;
      for (int c0 = 0; c0 < ks; c0 += 16) {
        for (int e = tid; e < 32 * 16; e += 256) {
          const int r = e >> 4, cc = e & 15, col = c0 + cc;
          Qt[r][cc] = (p0 + r < norb && col < ks) ? Qm[(size_t)(p0 + r) * ks + col] : c2(0, 0);
          Pt[r][cc] = (q0 + r < norb && col < ks) ? Pm[(size_t)(q0 + r) * ks + col] : c2(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int cc = 0; cc < 16; ++cc) {
          const double2 pv = Pt[tx][cc];
#pragma unroll
          for (int r = 0; r < 4; ++r) acc[r] = cadd(acc[r], cmulc(Qt[ty + 8 * r][cc], pv));
        }
        __syncthreads();
      }
    }
  }
  const int q = q0 + tx;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int p = p0 + ty + 8 * r;
    if (p < norb && q < norb) vbar[(size_t)wl * norb * norb + (size_t)p * norb + q] = acc[r];
  }
}

// ======================================================================================
// Field-shift adjoint (propagation.py:121-127): xt = x - s, s = -sqrt(dt)(i fb - mf),
// shift = sum xt mf, fbt = sum (x s - s^2/2). xt-bar += conj(mf) shift-bar,
// s-bar = -xt-bar + conj(x - s) fbt-bar (x - s = xt), fb-bar = i sqrt(dt) s-bar.
// ======================================================================================

// gmf (may be NULL): mf-bar += sqrt(dt) s-bar + conj(xt) shift-bar, summed over walkers
__global__ void k_a_field(int nchol, double sqdt, const double2* __restrict__ xt, const double2* __restrict__ mf,
                          const double2* __restrict__ xtb, const double2* __restrict__ shb,
                          const double2* __restrict__ fbtb, double2* __restrict__ fbb, double2* gmf) {
  const int w = blockIdx.x;
  const double2 sh = shb[w], ft = fbtb[w];
  for (int g = threadIdx.x; g < nchol; g += blockDim.x) {
    const size_t i = (size_t)w * nchol + g;
    const double2 xb = cadd(xtb[i], cmul(cconj(mf[g]), sh));
    const double2 sb = csub(cmul(cconj(xt[i]), ft), xb);
    fbb[i] = c2(-sqdt * sb.y, sqdt * sb.x);
    if (gmf) {
      const double2 m = cadd(cscale(sb, sqdt), cmul(cconj(xt[i]), sh));
      atomicAdd(&gmf[g].x, m.x);
      atomicAdd(&gmf[g].y, m.y);
    }
  }
}

// chol-bar[g][pq] += sqrt(dt) sum_w (xt.x vbar.y - xt.y vbar.x): the transpose of
// vhs = i sqrt(dt) xt chol with respect to chol. CTA per 32 x 64 tile, walkers 8 at a time.
__global__ void __launch_bounds__(256) k_a_chol_grad(int nwc, int nchol, long nn, double sqdt,
                                                     const double2* __restrict__ xt,
                                                     const double2* __restrict__ vbar, double* __restrict__ gchol) {
  __shared__ double2 Xs[8][32];
  __shared__ double2 Vs[8][64];
  const int g0 = blockIdx.y * 32, tid = threadIdx.x, tk = tid & 63, tg = tid >> 6;
  const long k0 = (long)blockIdx.x * 64;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int w0 = 0; w0 < nwc; w0 += 8) {
    for (int e = tid; e < 8 * 32; e += 256) {
      const int wl = e >> 5, gg = e & 31;
      Xs[wl][gg] = (w0 + wl < nwc && g0 + gg < nchol) ? xt[(size_t)(w0 + wl) * nchol + g0 + gg] : c2(0, 0);
    }
    for (int e = tid; e < 8 * 64; e += 256) {
      const int wl = e >> 6, kk = e & 63;
      Vs[wl][kk] = (w0 + wl < nwc && k0 + kk < nn) ? vbar[(size_t)(w0 + wl) * nn + k0 + kk] : c2(0, 0);
    }
    __syncthreads();
#pragma unroll
    for (int wl = 0; wl < 8; ++wl) {
      const double2 v = Vs[wl][tk];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const double2 x = Xs[wl][tg + 4 * r];
        acc[r] += x.x * v.y - x.y * v.x;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int g = g0 + tg + 4 * r;
    const long k = k0 + tk;
    if (g < nchol && k < nn) gchol[(size_t)g * nn + k] += sqdt * acc[r];
  }
}

int a_launch_chol_grad(const afq_ctx_dev& c, const AdjointBufs& a, int nwc, const double2* xt, cudaStream_t st) {
  const long nn = (long)c.norb * c.norb;
  {
    ProfScope _ps(K_VHS, st);
    k_a_chol_grad<<<dim3((unsigned)((nn + 63) / 64), (c.nchol + 31) / 32), 256, 0, st>>>(nwc, c.nchol, nn,
                                                                                         sqrt(c.dt), xt, a.vbar,
                                                                                         a.gchol);
  }
  return a_err("a_chol_grad");
}

// ======================================================================================
// SR adjoint (sr.py:24-47): W_new[i] = W[idx[i]], w_new = sum w / nw. The comb's indices are
// non-decreasing, so the walkers copied from j form one run of i: W-bar[j] = sum over the run.
// ======================================================================================

__global__ void k_a_sr_gather(int elems, int nw, const int32_t* __restrict__ idx, const double2* __restrict__ src,
                              double2* __restrict__ dst) {
  const int j = blockIdx.x;
  int lo = 0, hi = nw;  // first i with idx[i] >= j
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (idx[mid] < j) lo = mid + 1; else hi = mid;
  }
  int lo2 = lo, hi2 = nw;  // first i with idx[i] > j
  while (lo2 < hi2) {
    const int mid = (lo2 + hi2) >> 1;
    if (idx[mid] <= j) lo2 = mid + 1; else hi2 = mid;
  }
  for (int e = threadIdx.x; e < elems; e += blockDim.x) {
    double2 a = c2(0, 0);
    for (int i = lo; i < lo2; ++i) a = cadd(a, src[(size_t)i * elems + e]);
    dst[(size_t)j * elems + e] = a;
  }
}

__global__ void k_a_sr_weights(int nw, double* __restrict__ wbar) {
  __shared__ double red[32];
  double s = 0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) s += wbar[w];
  s = block_sum(s, red);
  for (int w = threadIdx.x; w < nw; w += blockDim.x) wbar[w] = s / (double)nw;
}

// ======================================================================================
// Launchers
// ======================================================================================

int a_launch_end(int nblk, const double* be, const double* bw, const AdjointBufs& a, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_a_end<<<1, 32, 0, st>>>(nblk, be, bw, a.beb, a.bwb);
  }
  return a_err("a_end");
}

int a_launch_block_stats(const afq_ctx_dev& c, const AdjointBufs& a, int blk, const double2* energy,
                         const double* weights, const double* scalars, const double* be, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_a_block_stats<<<1, 1024, 0, st>>>(c.nw, c.dt, energy, weights, scalars, be + blk, a.beb + blk, a.bwb + blk,
                                        a.scal, a.ebar, a.wbar);
  }
  return a_err("a_block_stats");
}

int a_launch_energy(const afq_ctx_dev& c, const AdjointBufs& a, const double2* green, cudaStream_t st) {
  const size_t smem = (2 * (size_t)c.ktot + 2 * (size_t)c.kmax * c.kmax) * sizeof(double2);
  if (int e = a_smem(smem, "energy")) return e;
  cudaFuncSetAttribute(k_a_energy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_ENERGY, st);
    k_a_energy<<<c.nw, 256, smem, st>>>(c, green, a.ebar, a.gene);
  }
  if (int e = a_err("a_energy")) return e;
  {
    ProfScope _ps(K_ENERGY_FIN, st);
    k_a_rot<<<(c.ktot + 255) / 256, 256, 0, st>>>(c, green, a.ebar, a.grot[0], a.grot[1]);
  }
  return a_err("a_rot");
}

int a_launch_green(const afq_ctx_dev& c, const void* wu, const void* wd, const double2* ga, const double2* gb,
                   const double2* lbar, double2* wbu, double2* wbd, cudaStream_t st, double* const* gt) {
  const size_t km = c.kmax;
  const size_t smem = (3 * (size_t)c.norb * km + 4 * km * km) * sizeof(double2) + (size_t)c.norb * km * sizeof(double);
  if (int e = a_smem(smem, "Green")) return e;
  cudaFuncSetAttribute(k_a_green, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_GREEN, st);
    double* gu = gt ? gt[0] : nullptr;
    double* gd = gt ? (c.nspin_g == 2 ? gt[1] : gt[0]) : nullptr;
    k_a_green<<<c.nw, 256, smem, st>>>(c, (const double2*)wu, (const double2*)wd, ga, gb, lbar, wbu, wbd, gu,
                                       c.nslab == 2 ? gd : nullptr);
  }
  return a_err("a_green");
}

// grc[g][k] += alpha Re sum_w conj(fb-bar[w][g]) G[w][k]: the transpose of fb = alpha rot_chol G
// with respect to rot_chol. CTA per 32 x 64 output tile, walkers staged 8 at a time.
__global__ void __launch_bounds__(256) k_a_rc_fb(int nw, int nchol, int ktot, double alpha,
                                                 const double2* __restrict__ fbb, const double2* __restrict__ green,
                                                 double* __restrict__ grc) {
  __shared__ double2 Fs[8][32];
  __shared__ double2 Gs[8][64];
  const int g0 = blockIdx.y * 32, k0 = blockIdx.x * 64, tid = threadIdx.x, tk = tid & 63, tg = tid >> 6;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int w0 = 0; w0 < nw; w0 += 8) {
    for (int e = tid; e < 8 * 32; e += 256) {
      const int wl = e >> 5, gg = e & 31;
      Fs[wl][gg] = (w0 + wl < nw && g0 + gg < nchol) ? fbb[(size_t)(w0 + wl) * nchol + g0 + gg] : c2(0, 0);
    }
    for (int e = tid; e < 8 * 64; e += 256) {
      const int wl = e >> 6, kk = e & 63;
      Gs[wl][kk] = (w0 + wl < nw && k0 + kk < ktot) ? green[(size_t)(w0 + wl) * ktot + k0 + kk] : c2(0, 0);
    }
    __syncthreads();
#pragma unroll
    for (int wl = 0; wl < 8; ++wl) {
      const double2 gv = Gs[wl][tk];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const double2 f = Fs[wl][tg + 4 * r];
        acc[r] += f.x * gv.x + f.y * gv.y;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int g = g0 + tg + 4 * r, k = k0 + tk;
    if (g < nchol && k < ktot) grc[(size_t)g * ktot + k] += alpha * acc[r];
  }
}

// Local-energy part of the rot_chol cotangent: with f_g = RC_g G^T and
// dE / d f_g[i][k] = kappa f_g[k][i] + gamma c delta_ik (as in k_a_energy),
// RC_g-bar[i][p] += sum_w e-bar_w Re sum_k (kappa f_g[k][i] + gamma c delta_ik) G_w[k][p].
// CTA per g, walkers in sequence; the (i, p) entries of both Green blocks are owned by the
// threads (at most kRcPT each).
constexpr int kRcPT = 16;

__global__ void __launch_bounds__(256) k_a_rc_energy(const afq_ctx_dev c, const double2* __restrict__ green,
                                                     const double* __restrict__ ebar, double* __restrict__ grc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int g = blockIdx.x, norb = c.norb, tid = threadIdx.x, nt = blockDim.x, om = c.kmax;
  double2* Gs = reinterpret_cast<double2*>(smem_raw);  // [ktot]
  double2* F = Gs + c.ktot;                            // [2][om*om]
  const double kappa = c.energy_mode == 2 ? -1.0 : -2.0;
  const double gamma = c.energy_mode == 0 ? 4.0 : (c.energy_mode == 1 ? 2.0 : 1.0);
  double acc[kRcPT];
#pragma unroll
  for (int j = 0; j < kRcPT; ++j) acc[j] = 0.0;
  for (int w = 0; w < c.nw; ++w) {
    const double eb = ebar[w];
    if (eb == 0.0) continue;  // uniform over the CTA
    for (int i = tid; i < c.ktot; i += nt) Gs[i] = green[(size_t)w * c.ktot + i];
    __syncthreads();
    for (int s = 0; s < c.nspin_g; ++s) {
      const int o = c.gocc[s];
      const double* RC = c.rot_chol[s] + (size_t)g * o * norb;
      const double2* Gsp = Gs + (size_t)s * c.gocc[0] * norb;
      for (int e = tid; e < o * o; e += nt) {
        const int i = e / o, k = e % o;
        double2 a = c2(0, 0);
        for (int p = 0; p < norb; ++p) {
          a.x = fma(RC[(size_t)i * norb + p], Gsp[(size_t)k * norb + p].x, a.x);
          a.y = fma(RC[(size_t)i * norb + p], Gsp[(size_t)k * norb + p].y, a.y);
        }
        F[s * om * om + e] = a;
      }
    }
    __syncthreads();
    double2 ct = c2(0, 0);
    for (int s = 0; s < c.nspin_g; ++s)
      for (int i = 0; i < c.gocc[s]; ++i) ct = cadd(ct, F[s * om * om + i * c.gocc[s] + i]);
#pragma unroll
    for (int j = 0; j < kRcPT; ++j) {
      const int e = tid + j * nt;
      if (e < c.ktot) {
        const int s = (c.nspin_g == 2 && e >= c.gocc[0] * norb) ? 1 : 0;
        const int o = c.gocc[s], el = e - s * c.gocc[0] * norb, i = el / norb, p = el % norb;
        const double2* Fs = F + s * om * om;
        const double2* Gsp = Gs + (size_t)s * c.gocc[0] * norb;
        double a = 0.0;
        for (int k = 0; k < o; ++k) {
          double2 m = cscale(Fs[k * o + i], kappa);
          if (k == i) m = cadd(m, cscale(ct, gamma));
          a += m.x * Gsp[(size_t)k * norb + p].x - m.y * Gsp[(size_t)k * norb + p].y;
        }
        acc[j] += eb * a;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < kRcPT; ++j) {
    const int e = tid + j * nt;
    if (e < c.ktot) grc[(size_t)g * c.ktot + e] += acc[j];
  }
}

int a_launch_rc_fb(const afq_ctx_dev& c, const AdjointBufs& a, const double2* green, double alpha,
                   cudaStream_t st) {
  {
    ProfScope _ps(K_FB, st);
    k_a_rc_fb<<<dim3((c.ktot + 63) / 64, (c.nchol + 31) / 32), 256, 0, st>>>(c.nw, c.nchol, c.ktot, alpha, a.fbb,
                                                                             green, a.grc);
  }
  return a_err("a_rc_fb");
}

int a_launch_rc_energy(const afq_ctx_dev& c, const AdjointBufs& a, const double2* green, cudaStream_t st) {
  if (c.ktot > kRcPT * 256) {
    afq_set_error("adjoint rot_chol kernel: nocc * norb <= %d", kRcPT * 256);
    return -2;
  }
  const size_t smem = ((size_t)c.ktot + 2 * (size_t)c.kmax * c.kmax) * sizeof(double2);
  if (int e = a_smem(smem, "rot_chol")) return e;
  cudaFuncSetAttribute(k_a_rc_energy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_ENERGY, st);
    k_a_rc_energy<<<c.nchol, 256, smem, st>>>(c, green, a.ebar, a.grc);
  }
  return a_err("a_rc_energy");
}

int a_launch_qr(const afq_ctx_dev& c, const void* wold_u, const void* wold_d, const void* q_u, const void* q_d,
                const double2* qb_u, const double2* qb_d, double2* ob_u, double2* ob_d, cudaStream_t st) {
  const size_t km = c.kmax;
  const size_t smem = (2 * (size_t)c.norb * km + 3 * km * km) * sizeof(double2);
  if (int e = a_smem(smem, "QR")) return e;
  cudaFuncSetAttribute(k_a_qr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_QR, st);
    k_a_qr<<<dim3(c.nw, c.nslab), 256, smem, st>>>(c, (const double2*)wold_u, (const double2*)wold_d,
                                                   (const double2*)q_u, (const double2*)q_d, qb_u, qb_d, ob_u, ob_d);
  }
  return a_err("a_qr");
}

int a_launch_weights(const afq_ctx_dev& c, const AdjointBufs& a, const double2* shift, const double2* fbt,
                     const double2* ovl_new, const double2* ovl, const double* w_start, const double* w_post,
                     const double* scalars, cudaStream_t st) {
  {
    ProfScope _ps(K_WEIGHTS, st);
    k_a_weights<<<1, 1024, 0, st>>>(c.nw, c.dt, c2(c.h0_prop_re, c.h0_prop_im), shift, fbt, ovl_new, ovl, w_start,
                                    w_post, scalars, a.scal, a.wbar, a.shb, a.fbtb, a.lbar, a.lbar2);
  }
  return a_err("a_weights");
}

// Taylor adjoint of walkers [w0, w0 + nwc): a.wb (cotangent after the step) -> a.wb2
// (cotangent before it), exp_h1-bar accumulated, vhs-bar into a.vbar (chunk rows).
int a_launch_taylor(const afq_ctx_dev& c, const AdjointBufs& a, int w0, int nwc, const double2* vhs,
                    const void* wu, const void* wd, cudaStream_t st) {
  const int n = c.norb * c.kmax;
  if (n > kAMaxPT * 256) {
    afq_set_error("adjoint Taylor kernel: norb * nocc <= %d", kAMaxPT * 256);
    return -2;
  }
  const size_t smem = 2 * (size_t)n * sizeof(double2);
  if (int e = a_smem(smem, "Taylor")) return e;
  cudaFuncSetAttribute(k_a_taylor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_TAYLOR, st);
    k_a_taylor<<<dim3(nwc, c.nslab), 256, smem, st>>>(c, w0, vhs, (const double2*)wu, (const double2*)wd, a.wb[0],
                                                      a.wb[1], a.tay, a.wb2[0], a.wb2[1]);
  }
  if (int e = a_err("a_taylor")) return e;
  const size_t esmem = 4 * 16 * (size_t)c.kmax * sizeof(double2);
  cudaFuncSetAttribute(k_a_exp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem);
  const int tiles = (c.norb + 15) / 16;
  {
    ProfScope _ps(K_EXP, st);
    k_a_exp_grad<<<dim3(tiles, tiles, c.nslab), 256, esmem, st>>>(c, w0, nwc, a.wb[0], a.wb[1], a.tay,
                                                                  (const double2*)wu, (const double2*)wd, a.gexp[0],
                                                                  a.gexp[1]);
  }
  if (int e = a_err("a_exp_grad")) return e;
  const int vt = (c.norb + 31) / 32;
  {
    ProfScope _ps(K_TAYLOR, st);
    k_a_vbar<<<dim3(vt, vt, nwc), 256, 0, st>>>(c, a.tay, a.vbar);
  }
  return a_err("a_vbar");
}

int a_launch_field(const afq_ctx_dev& c, const AdjointBufs& a, const double2* xt, cudaStream_t st) {
  {
    ProfScope _ps(K_FIELD, st);
    k_a_field<<<c.nw, 256, 0, st>>>(c.nchol, sqrt(c.dt), xt, c.mf, a.xtb, a.shb, a.fbtb, a.fbb, a.gmf);
  }
  return a_err("a_field");
}

// SR adjoint: a.wb (cotangent after the SR) -> a.wb2, weight cotangents in place
int a_launch_sr(const afq_ctx_dev& c, const AdjointBufs& a, const int32_t* idx, cudaStream_t st) {
  for (int s = 0; s < c.nslab; ++s) {
    ProfScope _ps(K_SR, st);
    k_a_sr_gather<<<c.nw, 256, 0, st>>>(c.norb * c.kslab[s], c.nw, idx, a.wb[s], a.wb2[s]);
  }
  if (int e = a_err("a_sr_gather")) return e;
  {
    ProfScope _ps(K_SR, st);
    k_a_sr_weights<<<1, 1024, 0, st>>>(c.nw, a.wbar);
  }
  return a_err("a_sr_weights");
}

}  // namespace afq

// Forward-mode derivative (tangent) of the FP64 phaseless block with respect to a coupling
// lambda of h1 + lambda D: the jvp that the reference's driver takes of
// sampler.propagate_phaseless_ad (driver.py:207-215, sampling.py:174-196 and its _norot
// variant, trial held fixed). Every quantity x of the FP64 path is carried with its
// tangent dx = dx/dlambda; the only inputs with a tangent are exp_h1 (its Frechet
// derivative) and rot_h1. Walker, weight and overlap tangents start at zero for the block,
// as the driver's jvp seeds them (driver.py:190-200).
//
// Kernels below compute value and tangent together where the value is needed for the
// tangent; plain linear steps (force bias, vhs) reuse the FP64 complex x real GEMM on the
// tangent arrays. Overlaps carry d log(overlap). Clamped quantities (weights set to 0,
// local energies replaced by e_estimate) get a zero tangent, as jnp.where's jvp gives.

#include <math.h>

#include "afq_common.cuh"
#include "afq_kernels.cuh"
#include "afq_prof.cuh"
#include "afq_tangent.cuh"

namespace afq {

constexpr size_t kTSmemMax = 227 * 1024 - 4096;  // opt-in shared memory per CTA, less the static arrays

static int t_smem(size_t bytes, const char* what) {
  if (bytes > kTSmemMax) {
    afq_set_error("tangent %s kernel: %zu bytes of shared memory needed, %zu available (norb * nocc too large)",
                  what, bytes, kTSmemMax);
    return -2;
  }
  return 0;
}

static int t_err(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    afq_set_error("%s: %s", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

// ======================================================================================
// Green's function and overlap with tangents (wavefunctions.py:478-501, 658-692):
// S = C^T W, dS = C^T dW; Gauss-Jordan with partial pivoting gives det S and S^-1;
// d log det S = tr(S^-1 dS); dS^-1 = -S^-1 dS S^-1; G^T = W S^-1,
// dG^T = dW S^-1 + W dS^-1. One CTA per walker.
// ======================================================================================

__global__ void __launch_bounds__(256) k_t_green(const afq_ctx_dev c, const double2* __restrict__ w_up,
                                                 const double2* __restrict__ w_dn,
                                                 const double2* __restrict__ dw_up,
                                                 const double2* __restrict__ dw_dn,
                                                 double2* __restrict__ green, double2* __restrict__ dgreen,
                                                 double2* __restrict__ ovl, double2* __restrict__ dlog_ovl,
                                                 const double* __restrict__ dc_up,
                                                 const double* __restrict__ dc_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wlk = blockIdx.x, norb = c.norb, tid = threadIdx.x, nt = blockDim.x;
  const int km = c.kmax;
  double2* Ws = reinterpret_cast<double2*>(smem_raw);  // [norb][km]
  double2* dWs = Ws + (size_t)norb * km;               // [norb][km]
  double2* Aug = dWs + (size_t)norb * km;              // [km][2 km]
  double2* dS = Aug + (size_t)km * 2 * km;             // [km][km]
  double2* Mb = dS + (size_t)km * km;                  // [km][km]
  double* Cs = reinterpret_cast<double*>(Mb + (size_t)km * km);  // [norb][km]
  __shared__ double red[32];
  __shared__ int piv_sh;
  __shared__ double2 det_sh;
  __shared__ double2 colj[64];

  double2 ov = c2(1.0, 0.0), dl = c2(0.0, 0.0);
  for (int s = 0; s < c.nslab; ++s) {
    const int ks = c.kslab[s], o = c.nocc_slab[s];
    const double2* W = (s == 0 ? w_up : w_dn) + (size_t)wlk * norb * ks;
    const double2* dW = (s == 0 ? dw_up : dw_dn) + (size_t)wlk * norb * ks;
    const double* C = c.trial[s];
    for (int i = tid; i < norb * o; i += nt) {
      const int p = i / o, k = i % o;
      Ws[i] = W[(size_t)p * ks + k];
      dWs[i] = dW[(size_t)p * ks + k];
      Cs[i] = C[(size_t)p * o + k];
    }
    __syncthreads();
    const double* dC = s == 0 ? dc_up : dc_dn;  // orbital rotation: dS += dC^T W
    for (int e = tid; e < o * o; e += nt) {
      const int i = e / o, k = e % o;
      double2 a = c2(0, 0), da = c2(0, 0);
      for (int p = 0; p < norb; ++p) {
        const double cv = Cs[p * o + i];
        a.x += cv * Ws[p * o + k].x;
        a.y += cv * Ws[p * o + k].y;
        da.x += cv * dWs[p * o + k].x;
        da.y += cv * dWs[p * o + k].y;
      }
      if (dC)
        for (int p = 0; p < norb; ++p) {
          const double dv = dC[(size_t)p * o + i];
          da.x += dv * Ws[p * o + k].x;
          da.y += dv * Ws[p * o + k].y;
        }
      Aug[i * 2 * o + k] = a;
      Aug[i * 2 * o + o + k] = c2(i == k ? 1.0 : 0.0, 0.0);
      dS[i * o + k] = da;
    }
    if (tid == 0) det_sh = c2(1.0, 0.0);
    __syncthreads();
    for (int j = 0; j < o; ++j) {  // Gauss-Jordan, |re|+|im| partial pivoting
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
        if (tid == 0) piv_sh = bi;
      }
      __syncthreads();
      const int pr = piv_sh;
      if (pr != j)
        for (int e = tid; e < 2 * o; e += nt) {
          const double2 t = Aug[j * 2 * o + e];
          Aug[j * 2 * o + e] = Aug[pr * 2 * o + e];
          Aug[pr * 2 * o + e] = t;
        }
      __syncthreads();
      const double2 pv = Aug[j * 2 * o + j];
      if (tid == 0) {
        const double2 d = cmul(det_sh, pv);
        det_sh = (pr != j) ? c2(-d.x, -d.y) : d;
      }
      const double2 inv = cdiv(c2(1.0, 0.0), pv);
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
    // d log det = tr(S^-1 dS); Mb = dS S^-1
    double tx = 0, ty = 0;
    for (int e = tid; e < o * o; e += nt) {
      const int k = e / o, i = e % o;
      const double2 p = cmul(Aug[k * 2 * o + o + i], dS[i * o + k]);
      tx += p.x;
      ty += p.y;
    }
    tx = block_sum(tx, red);
    ty = block_sum(ty, red);
    for (int e = tid; e < o * o; e += nt) {
      const int i = e / o, l = e % o;
      double2 a = c2(0, 0);
      for (int k = 0; k < o; ++k) a = cadd(a, cmul(dS[i * o + k], Aug[k * 2 * o + o + l]));
      Mb[e] = a;
    }
    __syncthreads();
    // dS <- dS^-1 = -S^-1 Mb
    for (int e = tid; e < o * o; e += nt) {
      const int k = e / o, l = e % o;
      double2 a = c2(0, 0);
      for (int i = 0; i < o; ++i) a = cadd(a, cmul(Aug[k * 2 * o + o + i], Mb[i * o + l]));
      dS[e] = c2(-a.x, -a.y);
    }
    __syncthreads();
    const int mult = (c.nslab == 1 && c.restricted_square) ? 2 : 1;
    ov = cmul(ov, det_sh);
    if (mult == 2) ov = cmul(ov, det_sh);
    dl = cadd(dl, c2(mult * tx, mult * ty));
    if (green) {
      const int gblk = (c.nspin_g == 2) ? s : 0;
      double2* Gw = green + (size_t)wlk * c.ktot + (size_t)gblk * c.nocc_slab[0] * norb;
      double2* dGw = dgreen + (size_t)wlk * c.ktot + (size_t)gblk * c.nocc_slab[0] * norb;
      for (int e = tid; e < o * norb; e += nt) {
        const int i = e / norb, p = e % norb;
        double2 a = c2(0, 0), da = c2(0, 0);
        for (int k = 0; k < o; ++k) {
          const double2 si = Aug[k * 2 * o + o + i];
          a = cadd(a, cmul(Ws[p * o + k], si));
          da = cadd(da, cadd(cmul(dWs[p * o + k], si), cmul(Ws[p * o + k], dS[k * o + i])));
        }
        if (c.nspin_g == 1 && s == 1) {  // RHF two-slab: G_up + G_dn
          a = cadd(a, Gw[e]);
          da = cadd(da, dGw[e]);
        }
        Gw[e] = a;
        dGw[e] = da;
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    ovl[wlk] = ov;
    dlog_ovl[wlk] = dl;
  }
}

// ======================================================================================
// Field shifts with tangents (propagation.py:121-127): ds = -sqrt(dt) i dfb, dxt = -ds,
// dshift = sum dxt mf, dfbt = sum (x - s) ds.
// ======================================================================================

__global__ void k_t_field_shifts(int nchol, double sqdt, const double* __restrict__ fields,
                                 const double2* __restrict__ fb, const double2* __restrict__ dfb,
                                 const double2* __restrict__ mf, double2* __restrict__ xt,
                                 double2* __restrict__ dxt, double2* __restrict__ shift,
                                 double2* __restrict__ dshift, double2* __restrict__ fbt,
                                 double2* __restrict__ dfbt) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int g = threadIdx.x; g < nchol; g += blockDim.x) {
    const double2 f = fb[(long)w * nchol + g], df = dfb[(long)w * nchol + g], m = mf[g];
    const double2 s = c2(-sqdt * (-f.y - m.x), -sqdt * (f.x - m.y));
    const double2 ds = c2(sqdt * df.y, -sqdt * df.x);
    const double x = fields[(long)w * nchol + g];
    const double2 t = c2(x - s.x, -s.y), dt_ = c2(-ds.x, -ds.y);
    xt[(long)w * nchol + g] = t;
    dxt[(long)w * nchol + g] = dt_;
    const double2 tm = cmul(t, m), dtm = cmul(dt_, m);
    const double2 s2 = cmul(s, s);
    const double2 xs = c2(x - s.x, -s.y);  // d(x s - s^2/2) = (x - s) ds
    const double2 dfx = cmul(xs, ds);
    acc[0] += tm.x; acc[1] += tm.y;
    acc[2] += x * s.x - 0.5 * s2.x; acc[3] += x * s.y - 0.5 * s2.y;
    acc[4] += dtm.x; acc[5] += dtm.y;
    acc[6] += dfx.x; acc[7] += dfx.y;
  }
  for (int q = 0; q < 8; ++q) acc[q] = block_sum(acc[q], red);
  if (threadIdx.x == 0) {
    shift[w] = c2(acc[0], acc[1]);
    fbt[w] = c2(acc[2], acc[3]);
    dshift[w] = c2(acc[4], acc[5]);
    dfbt[w] = c2(acc[6], acc[7]);
  }
}

// ======================================================================================
// Taylor propagator with tangents (propagation.py:67-92):
//   W1 = E W, dW1 = dE W + E dW; T_m = V T_{m-1} / m, dT_m = (dV T_{m-1} + V dT_{m-1}) / m;
//   acc = sum T_m; W = E acc, dW = dE acc + E dacc. One CTA per (walker of the chunk, slab).
// ======================================================================================

constexpr int kTMaxPT = 16;  // accumulator entries per thread: norb * k <= kTMaxPT * 256

__global__ void __launch_bounds__(256) k_t_taylor(const afq_ctx_dev c, int w0, const double2* __restrict__ vhs,
                                                  const double2* __restrict__ dvhs, const double* dexp_up,
                                                  const double* dexp_dn, double2* __restrict__ w_up,
                                                  double2* __restrict__ w_dn, double2* __restrict__ dw_up,
                                                  double2* __restrict__ dw_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wl = blockIdx.x, s = blockIdx.y, wlk = w0 + wl;
  const int norb = c.norb, ks = c.kslab[s], n = norb * ks;
  const int tid = threadIdx.x, nt = blockDim.x;
  double2* Ta = reinterpret_cast<double2*>(smem_raw);
  double2* Tb = Ta + n;
  double2* dTa = Tb + n;
  double2* dTb = dTa + n;
  const double* E = c.exp_h1[s];
  const double* dE = s == 0 ? dexp_up : dexp_dn;
  const double2* V = vhs + (size_t)wl * norb * norb;
  const double2* dV = dvhs + (size_t)wl * norb * norb;
  double2* W = (s == 0 ? w_up : w_dn) + (size_t)wlk * n;
  double2* dW = (s == 0 ? dw_up : dw_dn) + (size_t)wlk * n;
  for (int i = tid; i < n; i += nt) {
    Ta[i] = W[i];
    dTa[i] = dW[i];
  }
  __syncthreads();
  double2 acc[kTMaxPT], dacc[kTMaxPT];
#pragma unroll
  for (int j = 0; j < kTMaxPT; ++j) {
    const int i = tid + j * nt;
    acc[j] = dacc[j] = c2(0, 0);
    if (i < n) {
      const int p = i / ks, col = i % ks;
      double2 a = c2(0, 0), da = c2(0, 0);
      for (int q = 0; q < norb; ++q) {
        const double e = E[(size_t)p * norb + q], de = dE[(size_t)p * norb + q];
        const double2 t = Ta[q * ks + col], dt_ = dTa[q * ks + col];
        a.x = fma(e, t.x, a.x);
        a.y = fma(e, t.y, a.y);
        da.x = fma(de, t.x, fma(e, dt_.x, da.x));
        da.y = fma(de, t.y, fma(e, dt_.y, da.y));
      }
      Tb[i] = a;
      dTb[i] = da;
      acc[j] = a;
      dacc[j] = da;
    }
  }
  __syncthreads();
  double fact = 1.0;
  double2 *src = Tb, *dst = Ta, *dsrc = dTb, *ddst = dTa;
  for (int m = 1; m < c.n_exp_terms; ++m) {
    fact *= (double)m;
    const double invf = 1.0 / fact;
#pragma unroll
    for (int j = 0; j < kTMaxPT; ++j) {
      const int i = tid + j * nt;
      if (i < n) {
        const int p = i / ks, col = i % ks;
        double2 a = c2(0, 0), da = c2(0, 0);
        const double2* Vr = V + (size_t)p * norb;
        const double2* dVr = dV + (size_t)p * norb;
        for (int q = 0; q < norb; ++q) {
          const double2 t = src[q * ks + col];
          a = cadd(a, cmul(Vr[q], t));
          da = cadd(da, cadd(cmul(dVr[q], t), cmul(Vr[q], dsrc[q * ks + col])));
        }
        dst[i] = a;
        ddst[i] = da;
        acc[j] = cadd(acc[j], cscale(a, invf));
        dacc[j] = cadd(dacc[j], cscale(da, invf));
      }
    }
    __syncthreads();
    double2* t = src; src = dst; dst = t;
    t = dsrc; dsrc = ddst; ddst = t;
  }
#pragma unroll
  for (int j = 0; j < kTMaxPT; ++j) {
    const int i = tid + j * nt;
    if (i < n) {
      Ta[i] = acc[j];
      dTa[i] = dacc[j];
    }
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const int p = i / ks, col = i % ks;
    double2 a = c2(0, 0), da = c2(0, 0);
    for (int q = 0; q < norb; ++q) {
      const double e = E[(size_t)p * norb + q], de = dE[(size_t)p * norb + q];
      const double2 t = Ta[q * ks + col], dt_ = dTa[q * ks + col];
      a.x = fma(e, t.x, a.x);
      a.y = fma(e, t.y, a.y);
      da.x = fma(de, t.x, fma(e, dt_.x, da.x));
      da.y = fma(de, t.y, fma(e, dt_.y, da.y));
    }
    W[i] = a;
    dW[i] = da;
  }
}

// ======================================================================================
// Phaseless weights with tangents (propagation.py:133-160), one thread per walker.
// d log I = -sqrt(dt) dshift + dfbt + dt dE_pc + d log(O'/O);
// d theta = Im(-sqrt(dt) dshift + d log(O'/O)); v = |I| cos theta,
// dv = |I| (Re(d log I) cos theta - sin theta d theta). Clamped weights: zero tangent.
// ======================================================================================

__global__ void k_t_weights(int nw, double dt, double2 h0_prop, const double2* __restrict__ shift,
                            const double2* __restrict__ dshift, const double2* __restrict__ fbt,
                            const double2* __restrict__ dfbt, const double2* __restrict__ ovl_new,
                            const double2* __restrict__ dlo_new, double2* __restrict__ ovl,
                            double2* __restrict__ dlo, double* __restrict__ weights,
                            double* __restrict__ dweights, const double* __restrict__ scalars,
                            const double* __restrict__ dscalars) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const double sqdt = sqrt(dt);
  const double pcs = scalars[AFQ_S_POP_CONTROL_SHIFT], dpcs = dscalars[AFQ_S_POP_CONTROL_SHIFT];
  const double2 ratio = cdiv(ovl_new[w], ovl[w]);
  const double2 dlr = csub(dlo_new[w], dlo[w]);
  const double2 sh = shift[w], fb = fbt[w], dsh = dshift[w], dfb = dfbt[w];
  const double2 arg = c2(-sqdt * sh.x + fb.x + dt * (pcs + h0_prop.x), -sqdt * sh.y + fb.y + dt * h0_prop.y);
  const double2 darg = c2(-sqdt * dsh.x + dfb.x + dt * dpcs + dlr.x, -sqdt * dsh.y + dfb.y + dlr.y);
  const double2 imp = cmul(cexp_(arg), ratio);
  const double2 ph = cmul(cexp_(c2(-sqdt * sh.x, -sqdt * sh.y)), ratio);
  const double dtheta = -sqdt * dsh.y + dlr.y;
  const double theta = atan2(ph.y, ph.x);
  const double mag = hypot(imp.x, imp.y);
  double v = mag * cos(theta);
  double dv = mag * (darg.x * cos(theta) - sin(theta) * dtheta);
  if (isnan(v) || v < 1.0e-3 || v > 100.0) {
    v = 0.0;
    dv = 0.0;
  }
  const double w0 = weights[w], dw0 = dweights[w];
  double nwgt = v * w0, dn = dv * w0 + v * dw0;
  if (nwgt > 100.0) {
    nwgt = 0.0;
    dn = 0.0;
  }
  weights[w] = nwgt;
  dweights[w] = dn;
  ovl[w] = ovl_new[w];
  dlo[w] = dlo_new[w];
}

// E_pc = e_estimate - 0.1 log(sum w / nw) / dt (propagation.py:161-163); e_estimate has
// no tangent inside a block, so dE_pc = -0.1 (sum dw / sum w) / dt.
__global__ void k_t_pop_control(int nw, double dt, const double* __restrict__ weights,
                                const double* __restrict__ dweights, double* __restrict__ scalars,
                                double* __restrict__ dscalars) {
  __shared__ double red[32];
  double s = 0.0, ds = 0.0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    s += weights[w];
    ds += dweights[w];
  }
  s = block_sum(s, red);
  ds = block_sum(ds, red);
  if (threadIdx.x == 0) {
    scalars[AFQ_S_POP_CONTROL_SHIFT] = scalars[AFQ_S_E_ESTIMATE] - 0.1 * log(s / (double)nw) / dt;
    dscalars[AFQ_S_POP_CONTROL_SHIFT] = -0.1 * (ds / s) / dt;
  }
}

// ======================================================================================
// Tangent of the reduced QR W = Q R with real diag(R) (linalg_utils.py:51-65):
// R = Q^H W, X = dW R^-1, C = Q^H X, U = upper part of C - (C lower)^H with real diagonal,
// dQ = X - Q U. One CTA per (walker, slab); wold = W before the QR, w = Q after it.
// ======================================================================================

__global__ void __launch_bounds__(256) k_t_qr(const afq_ctx_dev c, const double2* __restrict__ wold_up,
                                              const double2* __restrict__ wold_dn,
                                              const double2* __restrict__ q_up, const double2* __restrict__ q_dn,
                                              double2* __restrict__ dw_up, double2* __restrict__ dw_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wlk = blockIdx.x, s = blockIdx.y;
  const int m = c.norb, k = c.kslab[s], tid = threadIdx.x, nt = blockDim.x;
  double2* Q = reinterpret_cast<double2*>(smem_raw);  // [m][k]
  double2* X = Q + (size_t)m * k;                      // [m][k]  dW, then X
  double2* R = X + (size_t)m * k;                      // [k][k]
  double2* U = R + (size_t)k * k;                      // [k][k]
  const size_t off = (size_t)wlk * m * k;
  const double2* Wo = (s == 0 ? wold_up : wold_dn) + off;
  const double2* Qg = (s == 0 ? q_up : q_dn) + off;
  double2* dW = (s == 0 ? dw_up : dw_dn) + off;
  for (int i = tid; i < m * k; i += nt) {
    Q[i] = Qg[i];
    X[i] = dW[i];
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += nt) {  // R = Q^H W
    const int i = e / k, j = e % k;
    double2 a = c2(0, 0);
    for (int p = 0; p < m; ++p) a = cadd(a, cmulc(Wo[(size_t)p * k + j], Q[p * k + i]));
    R[e] = a;
  }
  __syncthreads();
  for (int p = tid; p < m; p += nt) {  // X R = dW, row by row
    for (int j = 0; j < k; ++j) {
      double2 a = X[p * k + j];
      for (int l = 0; l < j; ++l) a = csub(a, cmul(X[p * k + l], R[l * k + j]));
      X[p * k + j] = cdiv(a, R[j * k + j]);
    }
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += nt) {  // C = Q^H X
    const int i = e / k, j = e % k;
    double2 a = c2(0, 0);
    for (int p = 0; p < m; ++p) a = cadd(a, cmulc(X[p * k + j], Q[p * k + i]));
    R[e] = a;  // R no longer needed: holds C
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += nt) {  // U = C - Omega
    const int i = e / k, j = e % k;
    double2 u = c2(0, 0);
    if (i < j) u = cadd(R[i * k + j], cconj(R[j * k + i]));
    else if (i == j) u = c2(R[e].x, 0.0);
    U[e] = u;
  }
  __syncthreads();
  for (int e = tid; e < m * k; e += nt) {  // dQ = X - Q U
    const int p = e / k, j = e % k;
    double2 a = X[e];
    for (int i = 0; i <= j; ++i) a = csub(a, cmul(Q[p * k + i], U[i * k + j]));
    dW[e] = a;
  }
}

// ======================================================================================
// Local-energy tangent (wavefunctions.py:529-561, 711-743): with f_g = RC_g G^T,
// d(sum c^2) = 2 sum c dc, d exc = 2 sum f_g[i,k] df_g[k,i], d ene1 = sum dG rot_h1 +
// G drot_h1. Pass 1 per (walker, chunk of g), pass 2 per walker.
// ======================================================================================

__global__ void __launch_bounds__(256) k_t_energy_part(const afq_ctx_dev c, int gchunk,
                                                       const double2* __restrict__ green,
                                                       const double2* __restrict__ dgreen,
                                                       double2* __restrict__ dpart,
                                                       const double* __restrict__ drc_up,
                                                       const double* __restrict__ drc_dn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = blockIdx.x, ch = blockIdx.y, norb = c.norb, tid = threadIdx.x, nt = blockDim.x;
  const int om = c.kmax;
  double2* Gs = reinterpret_cast<double2*>(smem_raw);  // [ktot]
  double2* dGs = Gs + c.ktot;                          // [ktot]
  double2* F = dGs + c.ktot;                           // [2][om*om]
  double2* dF = F + 2 * om * om;                       // [2][om*om]
  __shared__ double red[32];
  for (int i = tid; i < c.ktot; i += nt) {
    Gs[i] = green[(size_t)w * c.ktot + i];
    dGs[i] = dgreen[(size_t)w * c.ktot + i];
  }
  __syncthreads();
  double2 acc[5];
  for (int q = 0; q < 5; ++q) acc[q] = c2(0, 0);
  const int g0 = ch * gchunk, g1 = min(c.nchol, g0 + gchunk);
  for (int g = g0; g < g1; ++g) {
    double2 cc[2], dcc[2], dex[2];
    for (int s = 0; s < c.nspin_g; ++s) {
      const int o = c.gocc[s];
      const double* RC = c.rot_chol[s] + (size_t)g * o * norb;
      const size_t base = (size_t)s * c.gocc[0] * norb;
      double2* Fs = F + s * om * om;
      double2* dFs = dF + s * om * om;
      const double* dRC = s == 0 ? drc_up : drc_dn;  // orbital rotation: dF += dRC G^T
      for (int e = tid; e < o * o; e += nt) {
        const int i = e / o, kk = e % o;
        double2 a = c2(0, 0), da = c2(0, 0);
        const double* rr = RC + (size_t)i * norb;
        const double2* gg = Gs + base + (size_t)kk * norb;
        const double2* dg = dGs + base + (size_t)kk * norb;
        for (int p = 0; p < norb; ++p) {
          a.x = fma(rr[p], gg[p].x, a.x);
          a.y = fma(rr[p], gg[p].y, a.y);
          da.x = fma(rr[p], dg[p].x, da.x);
          da.y = fma(rr[p], dg[p].y, da.y);
        }
        if (dRC) {
          const double* dr = dRC + (size_t)g * o * norb + (size_t)i * norb;
          for (int p = 0; p < norb; ++p) {
            da.x = fma(dr[p], gg[p].x, da.x);
            da.y = fma(dr[p], gg[p].y, da.y);
          }
        }
        Fs[e] = a;
        dFs[e] = da;
      }
      __syncthreads();
      double v[6] = {0, 0, 0, 0, 0, 0};
      for (int e = tid; e < o * o; e += nt) {
        const int i = e / o, kk = e % o;
        const double2 p = cmul(Fs[i * o + kk], dFs[kk * o + i]);
        v[4] += p.x;
        v[5] += p.y;
        if (i == kk) {
          v[0] += Fs[e].x; v[1] += Fs[e].y;
          v[2] += dFs[e].x; v[3] += dFs[e].y;
        }
      }
      for (int q = 0; q < 6; ++q) v[q] = block_sum(v[q], red);
      cc[s] = c2(v[0], v[1]);
      dcc[s] = c2(v[2], v[3]);
      dex[s] = c2(2.0 * v[4], 2.0 * v[5]);
    }
    if (c.nspin_g == 1) {
      acc[0] = cadd(acc[0], cscale(cmul(cc[0], dcc[0]), 2.0));
      acc[1] = cadd(acc[1], dex[0]);
    } else {
      acc[0] = cadd(acc[0], cscale(cmul(cc[0], dcc[0]), 2.0));
      acc[1] = cadd(acc[1], cscale(cmul(cc[1], dcc[1]), 2.0));
      acc[2] = cadd(acc[2], cadd(cmul(dcc[0], cc[1]), cmul(cc[0], dcc[1])));
      acc[3] = cadd(acc[3], dex[0]);
      acc[4] = cadd(acc[4], dex[1]);
    }
  }
  if (tid == 0)
    for (int q = 0; q < 5; ++q) dpart[((size_t)w * gridDim.y + ch) * 5 + q] = acc[q];
}

__global__ void k_t_energy_final(const afq_ctx_dev c, int nchunks, const double2* __restrict__ green,
                                 const double2* __restrict__ dgreen, const double* drot_up,
                                 const double* drot_dn, const double2* __restrict__ dpart,
                                 double2* __restrict__ denergy) {
  __shared__ double red[32];
  const int w = blockIdx.x, norb = c.norb;
  double ex = 0, ey = 0;
  for (int s = 0; s < c.nspin_g; ++s) {
    const int o = c.gocc[s];
    const size_t base = (size_t)w * c.ktot + (size_t)s * c.gocc[0] * norb;
    const double* Rv = c.rot_h1[s];
    const double* dR = s == 0 ? drot_up : drot_dn;
    for (int e = threadIdx.x; e < o * norb; e += blockDim.x) {
      ex += dgreen[base + e].x * Rv[e] + green[base + e].x * dR[e];
      ey += dgreen[base + e].y * Rv[e] + green[base + e].y * dR[e];
    }
  }
  ex = block_sum(ex, red);
  ey = block_sum(ey, red);
  if (threadIdx.x == 0) {
    double2 a[5];
    for (int q = 0; q < 5; ++q) a[q] = c2(0, 0);
    for (int ch = 0; ch < nchunks; ++ch)
      for (int q = 0; q < 5; ++q) a[q] = cadd(a[q], dpart[((size_t)w * nchunks + ch) * 5 + q]);
    double2 de2, de1 = c2(ex, ey);
    if (c.energy_mode == 0) {
      de2 = csub(cscale(a[0], 2.0), a[1]);
      de1 = cscale(de1, 2.0);
    } else if (c.energy_mode == 1) {
      de2 = csub(a[0], a[1]);
    } else {
      de2 = cscale(csub(cadd(cadd(a[0], a[1]), cscale(a[2], 2.0)), cadd(a[3], a[4])), 0.5);
    }
    denergy[w] = cadd(de2, de1);
  }
}

// ======================================================================================
// Block statistics tangent (sampling.py:79-91): e = Re E clamped to e_estimate beyond
// sqrt(2/dt) (zero tangent when clamped), E_b = sum e w / sum w,
// dE_b = (sum (de w + e dw) - E_b sum dw) / sum w; dE_pc <- 0.9 dE_pc + 0.1 dE_b.
// Runs after the value kernel has written E_b into be[0].
// ======================================================================================

__global__ void k_t_block_stats(int nw, double dt, const double2* __restrict__ energy,
                                const double2* __restrict__ denergy, const double* __restrict__ weights,
                                const double* __restrict__ dweights, const double* __restrict__ scalars,
                                double* __restrict__ dscalars, const double* __restrict__ be,
                                double* __restrict__ dbe, double* __restrict__ dbw) {
  __shared__ double red[32];
  const double e_est = scalars[AFQ_S_E_ESTIMATE], lim = sqrt(2.0 / dt);
  double sw = 0, dsw = 0, a = 0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    double e = energy[w].x, de = denergy[w].x;
    if (fabs(e - e_est) > lim) {
      e = e_est;
      de = 0.0;
    }
    sw += weights[w];
    dsw += dweights[w];
    a += de * weights[w] + e * dweights[w];
  }
  sw = block_sum(sw, red);
  dsw = block_sum(dsw, red);
  a = block_sum(a, red);
  if (threadIdx.x == 0) {
    const double d = (a - be[0] * dsw) / sw;
    *dbe = d;
    *dbw = dsw;
    dscalars[AFQ_S_POP_CONTROL_SHIFT] = 0.9 * dscalars[AFQ_S_POP_CONTROL_SHIFT] + 0.1 * d;
  }
}

// sum of the weight tangents (SR keeps sum |w|; phaseless weights are non-negative)
__global__ void k_t_sum(int nw, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) s += x[w];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_t_sr_weights(int nw, const double* __restrict__ dsum, double* __restrict__ dweights) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) dweights[w] = *dsum / (double)nw;
}

__global__ void k_t_gather(int elems, const int32_t* __restrict__ idx, const double2* __restrict__ src,
                           double2* __restrict__ dst) {
  const int w = blockIdx.x;
  const double2* s = src + (size_t)idx[w] * elems;
  double2* d = dst + (size_t)w * elems;
  for (int i = threadIdx.x; i < elems; i += blockDim.x) d[i] = s[i];
}

// energy = sum E_b w_b / sum w_b and its tangent
__global__ void k_t_end(int nblk, const double* __restrict__ be, const double* __restrict__ bw,
                        const double* __restrict__ dbe, const double* __restrict__ dbw,
                        double* __restrict__ energy, double* __restrict__ denergy) {
  if (threadIdx.x == 0) {
    double a = 0, b = 0, da = 0, db = 0;
    for (int i = 0; i < nblk; ++i) {
      a += be[i] * bw[i];
      b += bw[i];
      da += dbe[i] * bw[i] + be[i] * dbw[i];
      db += dbw[i];
    }
    const double e = a / b;
    if (energy) *energy = e;
    *denergy = (da - e * db) / b;
  }
}

// ======================================================================================
// Launchers
// ======================================================================================

int t_launch_green(const afq_ctx_dev& c, const TangentBufs& t, const void* wu, const void* wd,
                   double2* green, double2* dgreen, double2* ovl, double2* dlog, cudaStream_t st) {
  const size_t km = c.kmax;
  const size_t smem = (2 * (size_t)c.norb * km + 2 * km * km + 2 * km * km) * sizeof(double2) +
                      (size_t)c.norb * km * sizeof(double);
  if (int e = t_smem(smem, "Green")) return e;
  cudaFuncSetAttribute(k_t_green, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_GREEN, st);
    k_t_green<<<c.nw, 256, smem, st>>>(c, (const double2*)wu, (const double2*)wd, t.dw[0], t.dw[1], green, dgreen,
                                       ovl, dlog, t.dtrial[0], c.nslab == 2 ? t.dtrial[1] : nullptr);
  }
  return t_err("t_green");
}

int t_launch_field_shifts(const afq_ctx_dev& c, const double* fields, const double2* fb, const double2* dfb,
                          double2* xt, double2* dxt, double2* shift, double2* dshift, double2* fbt, double2* dfbt,
                          cudaStream_t st) {
  {
    ProfScope _ps(K_FIELD, st);
    k_t_field_shifts<<<c.nw, 256, 0, st>>>(c.nchol, sqrt(c.dt), fields, fb, dfb, c.mf, xt, dxt, shift, dshift, fbt,
                                           dfbt);
  }
  return t_err("t_field_shifts");
}

int t_launch_taylor(const afq_ctx_dev& c, const TangentBufs& t, int w0, int nwc, const double2* vhs,
                    const double2* dvhs, void* wu, void* wd, cudaStream_t st) {
  const int n = c.norb * c.kmax;
  if (n > kTMaxPT * 256) {
    afq_set_error("tangent Taylor kernel: norb * nocc <= %d", kTMaxPT * 256);
    return -2;
  }
  const size_t smem = 4 * (size_t)n * sizeof(double2);
  if (int e = t_smem(smem, "Taylor")) return e;
  cudaFuncSetAttribute(k_t_taylor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_TAYLOR, st);
    k_t_taylor<<<dim3(nwc, c.nslab), 256, smem, st>>>(c, w0, vhs, dvhs, t.dexp[0], t.dexp[1], (double2*)wu,
                                                      (double2*)wd, t.dw[0], t.dw[1]);
  }
  return t_err("t_taylor");
}

int t_launch_weights(const afq_ctx_dev& c, const TangentBufs& t, const double2* shift, const double2* fbt,
                     const double2* ovl_new, double2* ovl, double* weights, double* scalars, cudaStream_t st) {
  {
    ProfScope _ps(K_WEIGHTS, st);
    k_t_weights<<<(c.nw + 127) / 128, 128, 0, st>>>(c.nw, c.dt, c2(c.h0_prop_re, c.h0_prop_im), shift, t.dshift, fbt,
                                                    t.dfbt, ovl_new, t.dlo_new, ovl, t.dlo, weights, t.dweights,
                                                    scalars, t.dscalars);
    k_t_pop_control<<<1, 1024, 0, st>>>(c.nw, c.dt, weights, t.dweights, scalars, t.dscalars);
  }
  return t_err("t_weights");
}

int t_launch_qr(const afq_ctx_dev& c, const TangentBufs& t, const void* wu, const void* wd, cudaStream_t st) {
  const size_t km = c.kmax;
  const size_t smem = (2 * (size_t)c.norb * km + 2 * km * km) * sizeof(double2);
  if (int e = t_smem(smem, "QR")) return e;
  cudaFuncSetAttribute(k_t_qr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_QR, st);
    k_t_qr<<<dim3(c.nw, c.nslab), 256, smem, st>>>(c, t.wold[0], t.wold[1], (const double2*)wu, (const double2*)wd,
                                                   t.dw[0], t.dw[1]);
  }
  return t_err("t_qr");
}

int t_launch_energy(const afq_ctx_dev& c, const TangentBufs& t, int nchunks, int gchunk, const double2* green,
                    cudaStream_t st) {
  const size_t smem = (2 * (size_t)c.ktot + 4 * (size_t)c.kmax * c.kmax) * sizeof(double2);
  if (int e = t_smem(smem, "energy")) return e;
  cudaFuncSetAttribute(k_t_energy_part, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_ENERGY, st);
    k_t_energy_part<<<dim3(c.nw, nchunks), 256, smem, st>>>(c, gchunk, green, t.dgreen, t.dpart, t.drc[0],
                                                            c.nspin_g == 2 ? t.drc[1] : nullptr);
  }
  int e = t_err("t_energy_part");
  if (e) return e;
  {
    ProfScope _ps(K_ENERGY_FIN, st);
    k_t_energy_final<<<c.nw, 256, 0, st>>>(c, nchunks, green, t.dgreen, t.drot[0], t.drot[1], t.dpart, t.dene);
  }
  return t_err("t_energy_final");
}

__global__ void k_t_add(long n, const double2* __restrict__ x, double2* __restrict__ y) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = cadd(y[i], x[i]);
}

int t_launch_add(long n, const double2* x, double2* y, cudaStream_t st) {
  {
    ProfScope _ps(K_FB, st);
    k_t_add<<<256, 256, 0, st>>>(n, x, y);
  }
  return t_err("t_add");
}

int t_launch_block_stats(const afq_ctx_dev& c, const TangentBufs& t, const double2* energy, const double* weights,
                         const double* scalars, const double* be, double* dbe, double* dbw, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_t_block_stats<<<1, 1024, 0, st>>>(c.nw, c.dt, energy, t.dene, weights, t.dweights, scalars, t.dscalars, be,
                                        dbe, dbw);
  }
  return t_err("t_block_stats");
}

int t_launch_sr_pre(const afq_ctx_dev& c, const TangentBufs& t, cudaStream_t st) {
  {
    ProfScope _ps(K_SR, st);
    k_t_sum<<<1, 1024, 0, st>>>(c.nw, t.dweights, t.dsum);
  }
  return t_err("t_sr_pre");
}

int t_launch_sr_post(const afq_ctx_dev& c, const TangentBufs& t, const int32_t* idx, cudaStream_t st) {
  for (int s = 0; s < c.nslab; ++s) {
    const size_t elems = (size_t)c.norb * c.kslab[s];
    cudaMemcpyAsync(t.wold[s], t.dw[s], elems * c.nw * sizeof(double2), cudaMemcpyDeviceToDevice, st);
    ProfScope _ps(K_SR, st);
    k_t_gather<<<c.nw, 256, 0, st>>>((int)elems, idx, t.wold[s], t.dw[s]);
  }
  {
    ProfScope _ps(K_SR, st);
    k_t_sr_weights<<<(c.nw + 255) / 256, 256, 0, st>>>(c.nw, t.dsum, t.dweights);
  }
  return t_err("t_sr_post");
}

int t_launch_end(int nblk, const double* be, const double* bw, const TangentBufs& t, double* energy, double* denergy,
                 cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_t_end<<<1, 32, 0, st>>>(nblk, be, bw, t.dbe, t.dbw, energy, denergy);
  }
  return t_err("t_end");
}

}  // namespace afq

// SIMT kernels of the AFQMC hot path: Green's function / overlap (FP64 Gauss-Jordan),
// complex x real GEMMs (FP64), field shifts, Taylor propagator (FP64), phaseless weights,
// local energy (FP64), Householder QR (FP64, LAPACK convention), comb SR, Philox RNG.
//
// Every kernel is templated on the walker storage type WT (double -> complex128 slabs,
// float -> complex64 slabs); arithmetic is FP64 throughout this file.

#include <math.h>
#include "afq_common.cuh"
#include "afq_kernels.cuh"
#include "afq_prof.cuh"

namespace afq {

// ======================================================================================
// Green's function and overlap.
// One CTA per walker. For each stored slab s: S = C_s^T W_s (C real), Gauss-Jordan with
// partial pivoting on [S | I] gives det(S) and S^-1, then G_s = (W_s S^-1)^T.
// wavefunctions.py:478-501 (rhf), 658-692 (uhf).
// ======================================================================================

template <typename WT>
__global__ void k_green_overlap(const afq_ctx_dev c, const WT* __restrict__ w_up,
                                const WT* __restrict__ w_dn, double2* __restrict__ green,
                                double2* __restrict__ overlap, int write_green) {
  using CT = typename CplxOf<WT>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wlk = blockIdx.x;
  const int norb = c.norb;
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ double red[32];
  __shared__ int piv_sh;
  __shared__ double2 det_sh;
  __shared__ double2 colj[64];
  // smem: W [norb][kmax] double2, Aug [o][2o] double2, C [norb][kmax] double
  double2* Ws = reinterpret_cast<double2*>(smem_raw);
  double2* Aug = Ws + (size_t)norb * c.kmax;
  double* Cs = reinterpret_cast<double*>(Aug + (size_t)c.kmax * 2 * c.kmax);

  double2 ovl = c2(1.0, 0.0);
  for (int s = 0; s < c.nslab; ++s) {
    const int ks = c.kslab[s];
    const int o = c.nocc_slab[s];  // occupied columns used from this slab
    const CT* W = reinterpret_cast<const CT*>(s == 0 ? w_up : w_dn) + (size_t)wlk * norb * ks;
    const double* C = c.trial[s];
    for (int i = tid; i < norb * o; i += nt) {
      int p = i / o, k = i % o;
      Ws[i] = ld_c(W + (size_t)p * ks + k);
      Cs[i] = C[(size_t)p * o + k];
    }
    __syncthreads();
    // S[i][k] = sum_p C[p][i] W[p][k];  Aug = [S | I]
    for (int e = tid; e < o * o; e += nt) {
      int i = e / o, k = e % o;
      double2 acc = c2(0, 0);
      for (int p = 0; p < norb; ++p) {
        double cv = Cs[p * o + i];
        double2 wv = Ws[p * o + k];
        acc.x += cv * wv.x;
        acc.y += cv * wv.y;
      }
      Aug[i * 2 * o + k] = acc;
      Aug[i * 2 * o + o + k] = c2(i == k ? 1.0 : 0.0, 0.0);
    }
    if (tid == 0) det_sh = c2(1.0, 0.0);
    __syncthreads();
    // Gauss-Jordan with partial pivoting (|re|+|im| pivot choice, as LAPACK izamax)
    for (int j = 0; j < o; ++j) {
      if (tid < 32) {
        double best = -1.0;
        int bi = j;
        for (int r = j + tid; r < o; r += 32) {
          double2 v = Aug[r * 2 * o + j];
          double m = fabs(v.x) + fabs(v.y);
          if (m > best) { best = m; bi = r; }
        }
        for (int off = 16; off > 0; off >>= 1) {
          double ob = __shfl_xor_sync(0xffffffffu, best, off);
          int oi = __shfl_xor_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (tid == 0) piv_sh = bi;
      }
      __syncthreads();
      const int pr = piv_sh;
      if (pr != j) {
        for (int e = tid; e < 2 * o; e += nt) {
          double2 t = Aug[j * 2 * o + e];
          Aug[j * 2 * o + e] = Aug[pr * 2 * o + e];
          Aug[pr * 2 * o + e] = t;
        }
      }
      __syncthreads();
      const double2 pv = Aug[j * 2 * o + j];
      if (tid == 0) {
        double2 d = cmul(det_sh, pv);
        det_sh = (pr != j) ? c2(-d.x, -d.y) : d;
      }
      const double2 inv = cdiv(c2(1.0, 0.0), pv);
      __syncthreads();
      for (int e = tid; e < 2 * o; e += nt) Aug[j * 2 * o + e] = cmul(Aug[j * 2 * o + e], inv);
      // snapshot the multipliers (column j) before any thread overwrites them
      for (int r = tid; r < o; r += nt) colj[r] = Aug[r * 2 * o + j];
      __syncthreads();
      for (int e = tid; e < o * 2 * o; e += nt) {
        int r = e / (2 * o), col = e % (2 * o);
        if (r == j) continue;
        Aug[e] = csub(Aug[e], cmul(colj[r], Aug[j * 2 * o + col]));
      }
      __syncthreads();
    }
    ovl = cmul(ovl, det_sh);
    if (c.nslab == 1 && c.restricted_square) ovl = cmul(ovl, det_sh);  // RHF restricted: det^2
    if (write_green) {
      // G[i][p] = sum_k W[p][k] Sinv[k][i]; Sinv[k][i] = Aug[k][o + i]
      const int gblk = (c.nspin_g == 2) ? s : 0;
      double2* Gw = green + (size_t)wlk * c.ktot + (size_t)gblk * c.nocc_slab[0] * norb;
      for (int e = tid; e < o * norb; e += nt) {
        int i = e / norb, p = e % norb;
        double2 acc = c2(0, 0);
        for (int k = 0; k < o; ++k) acc = cadd(acc, cmul(Ws[p * o + k], Aug[k * 2 * o + o + i]));
        if (c.nspin_g == 1 && s == 1) acc = cadd(acc, Gw[e]);  // RHF two-slab: G_up + G_dn
        Gw[e] = acc;
      }
    }
    __syncthreads();
  }
  if (tid == 0 && overlap) overlap[wlk] = ovl;
}

// ======================================================================================
// Complex x real GEMM, FP64:  C[m][n] = alpha * sum_k A[m][k] * B(k, n)
// B_KN: B(k,n) = B[k*ldb + n]; otherwise B(k,n) = B[n*ldb + k].
// ======================================================================================

template <bool B_KN>
__global__ void __launch_bounds__(256) k_gemm_cr(int M, int N, int K, const double2* __restrict__ A,
                                                 long lda, const double* __restrict__ B, long ldb,
                                                 double2* __restrict__ C, long ldc, double2 alpha) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ double2 As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = c2(0, 0);
  for (int k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      int e = tid + l * 256;
      int r = e >> 4, cc = e & 15;  // A: row r of 64, col cc of 16
      int gm = m0 + r, gk = k0 + cc;
      As[cc][r] = (gm < M && gk < K) ? A[(long)gm * lda + gk] : c2(0, 0);
      if (B_KN) {
        int br = e >> 6, bc = e & 63;  // k row br of 16, n col bc of 64
        int bk = k0 + br, bn = n0 + bc;
        Bs[br][bc] = (bk < K && bn < N) ? B[(long)bk * ldb + bn] : 0.0;
      } else {
        int bc = e >> 4, br = e & 15;  // n col bc of 64, k row br of 16
        int bk = k0 + br, bn = n0 + bc;
        Bs[br][bc] = (bk < K && bn < N) ? B[(long)bn * ldb + bk] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double2 a[4];
      double b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x = fma(a[i].x, b[j], acc[i][j].x);
          acc[i][j].y = fma(a[i].y, b[j], acc[i][j].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
      if (gm < M && gn < N) C[(long)gm * ldc + gn] = cmul(alpha, acc[i][j]);
    }
}

// ======================================================================================
// Field shifts (propagation.py:121-127):
//   s = -sqrt(dt) (i fb - mf);  xt = x - s;  shift = sum xt*mf;  fbt = sum x*s - s^2/2
// One CTA per walker.
// ======================================================================================

__global__ void k_field_shifts(int nchol, double sqdt, const double* __restrict__ fields,
                               const double2* __restrict__ fb, const double2* __restrict__ mf,
                               double2* __restrict__ xt, double2* __restrict__ shift,
                               double2* __restrict__ fbt) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  double sx = 0, sy = 0, fx = 0, fy = 0;
  for (int g = threadIdx.x; g < nchol; g += blockDim.x) {
    double2 f = fb[(long)w * nchol + g];
    double2 m = mf[g];
    // i*fb - mf = (-f.y - m.x, f.x - m.y)
    double2 s = c2(-sqdt * (-f.y - m.x), -sqdt * (f.x - m.y));
    double x = fields[(long)w * nchol + g];
    double2 t = c2(x - s.x, -s.y);
    xt[(long)w * nchol + g] = t;
    double2 tm = cmul(t, m);
    sx += tm.x;
    sy += tm.y;
    double2 s2 = cmul(s, s);
    fx += x * s.x - 0.5 * s2.x;
    fy += x * s.y - 0.5 * s2.y;
  }
  sx = block_sum(sx, red);
  sy = block_sum(sy, red);
  fx = block_sum(fx, red);
  fy = block_sum(fy, red);
  if (threadIdx.x == 0) {
    shift[w] = c2(sx, sy);
    fbt[w] = c2(fx, fy);
  }
}

// ======================================================================================
// Taylor propagator, FP64 (propagation.py:67-92):
//   W <- E W;  W <- W + sum_{m=1}^{nterms-1} V^m W / m!;  W <- E W
// One CTA per (walker in chunk, slab). V read from the chunk's vhs buffer (L2-resident).
// ======================================================================================

constexpr int TAYLOR_MAXPT = 32;  // accumulator entries per thread (norb*k <= 32*blockDim)

template <typename WT>
__global__ void __launch_bounds__(256) k_taylor_f64(const afq_ctx_dev c, int w0,
                                                    const double2* __restrict__ vhs,
                                                    WT* __restrict__ w_up, WT* __restrict__ w_dn) {
  using CT = typename CplxOf<WT>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wl = blockIdx.x, s = blockIdx.y;
  const int wlk = w0 + wl;
  const int norb = c.norb, ks = c.kslab[s];
  const int n = norb * ks;
  const int tid = threadIdx.x, nt = blockDim.x;
  double2* Ta = reinterpret_cast<double2*>(smem_raw);
  double2* Tb = Ta + n;
  const double* E = c.exp_h1[s];
  const double2* V = vhs + (size_t)wl * norb * norb;
  CT* W = reinterpret_cast<CT*>(s == 0 ? w_up : w_dn) + (size_t)wlk * n;
  for (int i = tid; i < n; i += nt) Ta[i] = ld_c(W + i);
  __syncthreads();
  double2 acc[TAYLOR_MAXPT];
  // Tb = E Ta ; acc = Tb
#pragma unroll
  for (int j = 0; j < TAYLOR_MAXPT; ++j) {
    int i = tid + j * nt;
    if (i < n) {
      int p = i / ks, col = i % ks;
      double2 a = c2(0, 0);
      for (int q = 0; q < norb; ++q) {
        double e = E[(size_t)p * norb + q];
        double2 t = Ta[q * ks + col];
        a.x = fma(e, t.x, a.x);
        a.y = fma(e, t.y, a.y);
      }
      Tb[i] = a;
      acc[j] = a;
    }
  }
  __syncthreads();
  double fact = 1.0;
  double2* src = Tb;
  double2* dst = Ta;
  for (int m = 1; m < c.n_exp_terms; ++m) {
    fact *= (double)m;
    const double invf = 1.0 / fact;
#pragma unroll
    for (int j = 0; j < TAYLOR_MAXPT; ++j) {
      int i = tid + j * nt;
      if (i < n) {
        int p = i / ks, col = i % ks;
        double2 a = c2(0, 0);
        const double2* Vr = V + (size_t)p * norb;
        for (int q = 0; q < norb; ++q) a = cadd(a, cmul(Vr[q], src[q * ks + col]));
        dst[i] = a;
        acc[j] = cadd(acc[j], cscale(a, invf));
      }
    }
    __syncthreads();
    double2* t = src;
    src = dst;
    dst = t;
  }
  // acc -> Ta, then W = E Ta
#pragma unroll
  for (int j = 0; j < TAYLOR_MAXPT; ++j) {
    int i = tid + j * nt;
    if (i < n) Ta[i] = acc[j];
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    int p = i / ks, col = i % ks;
    double2 a = c2(0, 0);
    for (int q = 0; q < norb; ++q) {
      double e = E[(size_t)p * norb + q];
      double2 t = Ta[q * ks + col];
      a.x = fma(e, t.x, a.x);
      a.y = fma(e, t.y, a.y);
    }
    st_c(W + i, a);
  }
}

// ======================================================================================
// Phaseless importance function and weights (propagation.py:133-164). One CTA.
// ======================================================================================

__global__ void k_weights(int nw, double dt, double2 h0_prop, const double2* __restrict__ shift,
                          const double2* __restrict__ fbt, int ntiles,
                          const double2* __restrict__ ovl_new, double2* __restrict__ ovl,
                          double* __restrict__ weights, const double* __restrict__ scalars) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const double sqdt = sqrt(dt);
  const double pcs = scalars[AFQ_S_POP_CONTROL_SHIFT];
  double2 ratio = cdiv(ovl_new[w], ovl[w]);
  double2 sh = c2(0, 0), fb = c2(0, 0);
  for (int t = 0; t < ntiles; ++t) {
    sh = cadd(sh, shift[(size_t)w * ntiles + t]);
    fb = cadd(fb, fbt[(size_t)w * ntiles + t]);
  }
  // |I| cos(angle(ph)) with I = exp(arg) O'/O and ph = exp(-sqrt(dt) shift) O'/O equals
  // exp(Re arg) Re(exp(i Im(-sqrt(dt) shift)) O'/O): one exp and one sincos instead of two
  // complex exponentials, atan2, hypot and cos (the same quantity; FP64 transcendentals are
  // slow on this part)
  const double re_arg = -sqdt * sh.x + fb.x + dt * (pcs + h0_prop.x);
  double sn, cs;
  sincos(-sqdt * sh.y, &sn, &cs);
  double v = exp(re_arg) * (cs * ratio.x - sn * ratio.y);
  if (isnan(v)) v = 0.0;
  if (v < 1.0e-3) v = 0.0;
  if (v > 100.0) v = 0.0;
  double nwgt = v * weights[w];
  if (nwgt > 100.0) nwgt = 0.0;
  weights[w] = nwgt;
  ovl[w] = ovl_new[w];
}

// pop_control_ene_shift = e_estimate - 0.1 log(sum w / nw) / dt (propagation.py:161-163)
// status (mixed path, may be NULL): the tensor-core pipeline's guard word, folded into
// scalars[AFQ_S_STATUS] so that callers see a timeout or a bad operand in the state
__global__ void k_pop_control(int nw, double dt, const double* __restrict__ weights,
                              double* __restrict__ scalars, const int* __restrict__ status) {
  __shared__ double red[32];
  double sum = 0.0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) sum += weights[w];
  sum = block_sum(sum, red);
  if (threadIdx.x == 0) {
    scalars[AFQ_S_POP_CONTROL_SHIFT] = scalars[AFQ_S_E_ESTIMATE] - 0.1 * log(sum / (double)nw) / dt;
    if (status && *status != 0)
      scalars[AFQ_S_STATUS] = (double)((int)scalars[AFQ_S_STATUS] | *status);
  }
}

// ======================================================================================
// Local energy, FP64 (wavefunctions.py:529-561, 711-743).
// Pass 1: CTA per (walker, chunk of g): f_g = RC_g G^T, c_g = tr f_g,
//         exc_g = sum_ik f_g[i,k] f_g[k,i]; per-chunk partial sums.
// Pass 2: CTA per walker: reduce chunks, add ene1 = sum G * rot_h1 and h0.
// Partial slots: RHF: [sum c^2, sum exc]; UHF: [sum cu^2, sum cd^2, sum cu cd, exc_u, exc_d].
// ======================================================================================

__global__ void __launch_bounds__(256) k_energy_f64_part(const afq_ctx_dev c, int gchunk,
                                                         const double2* __restrict__ green,
                                                         double2* __restrict__ epart) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = blockIdx.x, ch = blockIdx.y;
  const int norb = c.norb, tid = threadIdx.x, nt = blockDim.x;
  double2* Gs = reinterpret_cast<double2*>(smem_raw);            // [ktot]
  double2* F = Gs + c.ktot;                                      // [2][omax*omax]
  __shared__ double red[32];
  const int omax = c.kmax;
  for (int i = tid; i < c.ktot; i += nt) Gs[i] = green[(size_t)w * c.ktot + i];
  __syncthreads();
  double2 acc[5];
  for (int q = 0; q < 5; ++q) acc[q] = c2(0, 0);
  const int g0 = ch * gchunk, g1 = min(c.nchol, g0 + gchunk);
  for (int g = g0; g < g1; ++g) {
    double2 cc[2], ex[2];
    for (int s = 0; s < c.nspin_g; ++s) {
      const int o = c.gocc[s];
      const double* RC = c.rot_chol[s] + (size_t)g * o * norb;
      const double2* Gsp = Gs + (size_t)s * c.gocc[0] * norb;
      double2* Fs = F + s * omax * omax;
      for (int e = tid; e < o * o; e += nt) {
        int i = e / o, k = e % o;
        double2 a = c2(0, 0);
        const double* rr = RC + (size_t)i * norb;
        const double2* gg = Gsp + (size_t)k * norb;
        for (int p = 0; p < norb; ++p) {
          a.x = fma(rr[p], gg[p].x, a.x);
          a.y = fma(rr[p], gg[p].y, a.y);
        }
        Fs[e] = a;
      }
      __syncthreads();
      double tr_x = 0, tr_y = 0, ex_x = 0, ex_y = 0;
      for (int e = tid; e < o * o; e += nt) {
        int i = e / o, k = e % o;
        double2 p = cmul(Fs[i * o + k], Fs[k * o + i]);
        ex_x += p.x;
        ex_y += p.y;
        if (i == k) { tr_x += Fs[e].x; tr_y += Fs[e].y; }
      }
      tr_x = block_sum(tr_x, red);
      tr_y = block_sum(tr_y, red);
      ex_x = block_sum(ex_x, red);
      ex_y = block_sum(ex_y, red);
      cc[s] = c2(tr_x, tr_y);
      ex[s] = c2(ex_x, ex_y);
    }
    if (c.nspin_g == 1) {
      acc[0] = cadd(acc[0], cmul(cc[0], cc[0]));
      acc[1] = cadd(acc[1], ex[0]);
    } else {
      acc[0] = cadd(acc[0], cmul(cc[0], cc[0]));
      acc[1] = cadd(acc[1], cmul(cc[1], cc[1]));
      acc[2] = cadd(acc[2], cmul(cc[0], cc[1]));
      acc[3] = cadd(acc[3], ex[0]);
      acc[4] = cadd(acc[4], ex[1]);
    }
  }
  if (tid == 0) {
    for (int q = 0; q < 5; ++q) epart[((size_t)w * gridDim.y + ch) * 5 + q] = acc[q];
  }
}

__global__ void k_energy_final(const afq_ctx_dev c, int nchunks, const double2* __restrict__ green,
                               const double2* __restrict__ epart, double2* __restrict__ energy) {
  __shared__ double red[32];
  const int w = blockIdx.x, norb = c.norb;
  // ene1
  double e1x = 0, e1y = 0;
  for (int s = 0; s < c.nspin_g; ++s) {
    const int o = c.gocc[s];
    const double2* G = green + (size_t)w * c.ktot + (size_t)s * c.gocc[0] * norb;
    const double* R = c.rot_h1[s];
    for (int e = threadIdx.x; e < o * norb; e += blockDim.x) {
      e1x += G[e].x * R[e];
      e1y += G[e].y * R[e];
    }
  }
  e1x = block_sum(e1x, red);
  e1y = block_sum(e1y, red);
  if (threadIdx.x == 0) {
    double2 a[5];
    for (int q = 0; q < 5; ++q) a[q] = c2(0, 0);
    for (int ch = 0; ch < nchunks; ++ch)
      for (int q = 0; q < 5; ++q) a[q] = cadd(a[q], epart[((size_t)w * nchunks + ch) * 5 + q]);
    double2 e2, e1 = c2(e1x, e1y);
    if (c.energy_mode == 0) {  // RHF restricted: 2 sum c^2 - exc ; ene1 x2
      e2 = csub(cscale(a[0], 2.0), a[1]);
      e1 = cscale(e1, 2.0);
    } else if (c.energy_mode == 1) {  // RHF two-slab (G = G_up + G_dn): sum c^2 - exc
      e2 = csub(a[0], a[1]);
    } else {  // UHF
      e2 = cscale(csub(cadd(cadd(a[0], a[1]), cscale(a[2], 2.0)), cadd(a[3], a[4])), 0.5);
    }
    energy[w] = cadd(cadd(e2, e1), c2(c.h0, 0.0));
  }
}

// ======================================================================================
// Householder QR, LAPACK zgeqr2 + zung2r conventions (R has a real diagonal,
// beta = -sign(Re alpha) * |(alpha, x)|). One CTA per (walker, slab). Q overwrites W.
// Arithmetic in the walker's precision (FP64 for complex128 walkers, FP32 for complex64).
// linalg_utils.py:51-65 (jnp.linalg.qr, reduced mode).
// ======================================================================================

template <typename CT> struct QrT;
template <> struct QrT<double2> {
  using R = double;
  AFQ_D static double2 mk(double a, double b) { return make_double2(a, b); }
};
template <> struct QrT<float2> {
  using R = float;
  AFQ_D static float2 mk(float a, float b) { return make_float2(a, b); }
};

AFQ_D float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
AFQ_D double warp_sum_t(double v) { return warp_sum(v); }
AFQ_D float warp_sum_t(float v) { return warp_sumf(v); }

// rdiag (optional, [nslab][nw]): prod(diag R) per walker slab (linalg_utils.py:51-65 returns
// it as the norm factor; the free-projection step multiplies its norms by it)
template <typename WT>
__global__ void __launch_bounds__(256) k_qr_householder(const afq_ctx_dev c, WT* __restrict__ w_up,
                                                        WT* __restrict__ w_dn, double2* __restrict__ rdiag) {
  using CT = typename CplxOf<WT>::type;  // compute in the storage precision
  using R = typename QrT<CT>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wlk = blockIdx.x, s = blockIdx.y;
  const int m = c.norb, k = c.kslab[s];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5,
            nwarp = nt >> 5;
  CT* A = reinterpret_cast<CT*>(smem_raw);  // [m][k]
  CT* y = A + (size_t)m * k;                // [k]
  CT* tau = y + k;                          // [k]
  __shared__ double red[32];
  __shared__ CT sc_sh, beta_sh;
  CT* W = reinterpret_cast<CT*>(s == 0 ? w_up : w_dn) + (size_t)wlk * m * k;
  for (int i = tid; i < m * k; i += nt) A[i] = W[i];
  double2 rprod = c2(1.0, 0.0);  // thread 0
  __syncthreads();
  // ---- factorisation
  for (int j = 0; j < k; ++j) {
    double xnd = 0.0;
    for (int r = j + 1 + tid; r < m; r += nt) xnd += (double)cabs2(A[r * k + j]);
    xnd = block_sum(xnd, red);
    if (tid == 0) {
      const CT alpha = A[j * k + j];
      const R xn = (R)xnd;
      if (xn == (R)0 && alpha.y == (R)0) {
        tau[j] = QrT<CT>::mk(0, 0);
        beta_sh = alpha;
        sc_sh = QrT<CT>::mk(1, 0);
      } else {
        const R nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn);
        const R beta = (alpha.x >= (R)0) ? -nrm : nrm;
        tau[j] = QrT<CT>::mk((beta - alpha.x) / beta, -alpha.y / beta);
        sc_sh = cdiv(QrT<CT>::mk(1, 0), csub(alpha, QrT<CT>::mk(beta, 0)));
        beta_sh = QrT<CT>::mk(beta, 0);
      }
    }
    __syncthreads();
    const CT scl = sc_sh;
    for (int r = j + 1 + tid; r < m; r += nt) A[r * k + j] = cmul(A[r * k + j], scl);
    if (tid == 0) A[j * k + j] = QrT<CT>::mk(1, 0);
    __syncthreads();
    // y[col] = sum_r conj(v[r]) A[r][col], col > j ; then A -= conj(tau) v y
    for (int col = j + 1 + wid; col < k; col += nwarp) {
      R yx = 0, yy = 0;
      for (int r = j + lane; r < m; r += 32) {
        const CT pr = cmulc(A[r * k + col], A[r * k + j]);
        yx += pr.x;
        yy += pr.y;
      }
      yx = warp_sum_t(yx);
      yy = warp_sum_t(yy);
      if (lane == 0) y[col] = QrT<CT>::mk(yx, yy);
    }
    __syncthreads();
    const CT ct = cconj(tau[j]);
    const int ncol = k - j - 1;
    if (ncol > 0) {
      for (int e = tid; e < (m - j) * ncol; e += nt) {
        const int r = j + e / ncol, col = j + 1 + e % ncol;
        A[r * k + col] = csub(A[r * k + col], cmul(ct, cmul(A[r * k + j], y[col])));
      }
    }
    __syncthreads();
    if (tid == 0) {
      A[j * k + j] = beta_sh;
      rprod = cmul(rprod, c2((double)beta_sh.x, (double)beta_sh.y));
    }
    __syncthreads();
  }
  if (tid == 0 && rdiag) rdiag[(size_t)s * c.nw + wlk] = rprod;
  // ---- form Q (zung2r): columns from last to first
  for (int j = k - 1; j >= 0; --j) {
    if (j < k - 1) {
      if (tid == 0) A[j * k + j] = QrT<CT>::mk(1, 0);
      __syncthreads();
      for (int col = j + 1 + wid; col < k; col += nwarp) {
        R yx = 0, yy = 0;
        for (int r = j + lane; r < m; r += 32) {
          const CT pr = cmulc(A[r * k + col], A[r * k + j]);
          yx += pr.x;
          yy += pr.y;
        }
        yx = warp_sum_t(yx);
        yy = warp_sum_t(yy);
        if (lane == 0) y[col] = QrT<CT>::mk(yx, yy);
      }
      __syncthreads();
      const CT t = tau[j];
      const int ncol = k - j - 1;
      for (int e = tid; e < (m - j) * ncol; e += nt) {
        const int r = j + e / ncol, col = j + 1 + e % ncol;
        A[r * k + col] = csub(A[r * k + col], cmul(t, cmul(A[r * k + j], y[col])));
      }
      __syncthreads();
    }
    const CT t = tau[j];
    const CT mt = QrT<CT>::mk(-t.x, -t.y);
    for (int r = j + 1 + tid; r < m; r += nt) A[r * k + j] = cmul(mt, A[r * k + j]);
    if (tid == 0) A[j * k + j] = QrT<CT>::mk(1 - t.x, -t.y);
    for (int r = tid; r < j; r += nt) A[r * k + j] = QrT<CT>::mk(0, 0);
    __syncthreads();
  }
  for (int i = tid; i < m * k; i += nt) W[i] = A[i];
}

// ======================================================================================
// Comb stochastic reconfiguration (sr.py:24-47). One CTA computes the indices with a
// sequential cumulative sum (same summation order as numpy/jnp.cumsum), then a gather.
// ======================================================================================

// in_smem: the weights are staged in shared memory (coalesced), scanned there by one
// thread in index order (the summation order of numpy/jnp.cumsum) and searched there.
__global__ void k_sr_indices(int nw, const double* __restrict__ zeta, double* __restrict__ weights,
                             double* __restrict__ cum_g, int32_t* __restrict__ idx, int in_smem) {
  extern __shared__ double cum_s[];
  double* cum = in_smem ? cum_s : cum_g;
  if (in_smem) {
    for (int i = threadIdx.x; i < nw; i += blockDim.x) cum_s[i] = fabs(weights[i]);
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0;
      for (int i = 0; i < nw; ++i) {
        a += cum_s[i];
        cum_s[i] = a;
      }
    }
  } else if (threadIdx.x == 0) {
    double a = 0.0;
    for (int i = 0; i < nw; ++i) {
      a += fabs(weights[i]);
      cum[i] = a;
    }
  }
  __syncthreads();
  const double tw = cum[nw - 1];
  const double z0 = zeta[0];
  for (int i = threadIdx.x; i < nw; i += blockDim.x) {
    double z = tw * ((double)i + z0) / (double)nw;
    int lo = 0, hi = nw;  // first index with cum >= z
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (cum[mid] < z) lo = mid + 1; else hi = mid;
    }
    idx[i] = min(lo, nw - 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nw; i += blockDim.x) weights[i] = tw / (double)nw;
}

template <typename WT>
__global__ void k_gather_slab(int slab_elems, const int32_t* __restrict__ idx,
                              const WT* __restrict__ src, WT* __restrict__ dst) {
  using CT = typename CplxOf<WT>::type;
  const int w = blockIdx.x;
  const CT* s = reinterpret_cast<const CT*>(src) + (size_t)idx[w] * slab_elems;
  CT* d = reinterpret_cast<CT*>(dst) + (size_t)w * slab_elems;
  for (int i = threadIdx.x; i < slab_elems; i += blockDim.x) d[i] = s[i];
}

// ======================================================================================
// Block statistics (sampling.py:74-91) and the sampler total (sampling.py:337-341).
// ======================================================================================

__global__ void k_block_stats(int nw, double dt, const double2* __restrict__ energy,
                              const double* __restrict__ weights, double* __restrict__ scalars,
                              double* __restrict__ be_out, double* __restrict__ bw_out) {
  __shared__ double red[32];
  const double e_est = scalars[AFQ_S_E_ESTIMATE];
  const double lim = sqrt(2.0 / dt);
  double sw = 0, swe = 0, nz = 0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    double e = energy[w].x;
    if (fabs(e - e_est) > lim) e = e_est;
    double wt = weights[w];
    sw += wt;
    swe += e * wt;
    nz += (wt != 0.0) ? 1.0 : 0.0;
  }
  sw = block_sum(sw, red);
  swe = block_sum(swe, red);
  nz = block_sum(nz, red);
  if (threadIdx.x == 0) {
    double be = swe / sw;
    scalars[AFQ_S_N_KILLED] += (double)nw - nz;
    scalars[AFQ_S_BLOCK_ENERGY] = be;
    scalars[AFQ_S_BLOCK_WEIGHT] = sw;
    scalars[AFQ_S_POP_CONTROL_SHIFT] = 0.9 * scalars[AFQ_S_POP_CONTROL_SHIFT] + 0.1 * be;
    if (be_out) *be_out = be;
    if (bw_out) *bw_out = sw;
  }
}

// en_samples (corr_sample.py:482-491): Re(E) clamped to e_estimate beyond sqrt(2/dt)
__global__ void k_clamped_energies(int nw, double dt, const double2* __restrict__ energy,
                                   const double* __restrict__ scalars, double* __restrict__ out) {
  const double e_est = scalars[AFQ_S_E_ESTIMATE];
  const double lim = sqrt(2.0 / dt);
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
    const double e = energy[w].x;
    out[w] = (fabs(e - e_est) > lim) ? e_est : e;
  }
}

// corr_otler_rm (corr_sample.py:557-594) + the weighted sums of cs_step (673-694), one CTA.
// mean and population std in two passes, as jnp.mean / jnp.std; the larger z-score selected
// with jnp.where(z1 > z2, z1, z2) semantics (a NaN z1 selects z2).
__global__ void k_cs_outlier(int nw, double z_thresh, double* __restrict__ w1, double* __restrict__ w2,
                             const double* __restrict__ e1, const double* __restrict__ e2,
                             double* __restrict__ sums) {
  __shared__ double red[32];
  double s1 = 0, s2 = 0;
  for (int i = threadIdx.x; i < nw; i += blockDim.x) {
    s1 += w1[i];
    s2 += w2[i];
  }
  const double m1 = block_sum(s1, red) / nw, m2 = block_sum(s2, red) / nw;
  double v1 = 0, v2 = 0;
  for (int i = threadIdx.x; i < nw; i += blockDim.x) {
    v1 += (w1[i] - m1) * (w1[i] - m1);
    v2 += (w2[i] - m2) * (w2[i] - m2);
  }
  const double sd1 = sqrt(block_sum(v1, red) / nw), sd2 = sqrt(block_sum(v2, red) / nw);
  double a1 = 0, b1 = 0, a2 = 0, b2 = 0;
  for (int i = threadIdx.x; i < nw; i += blockDim.x) {
    const double z1 = fabs(w1[i] - m1) / sd1, z2 = fabs(w2[i] - m2) / sd2;
    const double z = (z1 > z2) ? z1 : z2;
    double x1 = w1[i], x2 = w2[i];
    if (z > z_thresh) {
      x1 = 0.0;
      x2 = 0.0;
    }
    w1[i] = x1;
    w2[i] = x2;
    a1 += e1[i] * x1;
    b1 += x1;
    a2 += e2[i] * x2;
    b2 += x2;
  }
  a1 = block_sum(a1, red);
  b1 = block_sum(b1, red);
  a2 = block_sum(a2, red);
  b2 = block_sum(b2, red);
  if (threadIdx.x == 0) {
    sums[0] = a1;
    sums[1] = b1;
    sums[2] = a2;
    sums[3] = b2;
  }
}

__global__ void k_phaseless_begin(double* scalars) {
  scalars[AFQ_S_N_KILLED] = 0.0;
  scalars[AFQ_S_POP_CONTROL_SHIFT] = scalars[AFQ_S_E_ESTIMATE];
}

__global__ void k_phaseless_end(int nblk, double denom, const double* __restrict__ be,
                                const double* __restrict__ bw, double* __restrict__ scalars,
                                double* __restrict__ energy) {
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < nblk; ++i) {
      a += be[i] * bw[i];
      b += bw[i];
    }
    *energy = a / b;
    scalars[AFQ_S_N_KILLED] /= denom;
  }
}

// driver.py:252 (block weight before QR/SR) and driver.py:308 (e_estimate update)
__global__ void k_driver_update(int nw, const double* __restrict__ weights,
                                const double* __restrict__ energy, double* __restrict__ scalars,
                                double* __restrict__ wsum) {
  __shared__ double red[32];
  double s = 0.0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) s += weights[w];
  s = block_sum(s, red);
  if (threadIdx.x == 0) {
    *wsum = s;
    scalars[AFQ_S_E_ESTIMATE] = 0.9 * scalars[AFQ_S_E_ESTIMATE] + 0.1 * energy[0];
  }
}

// ======================================================================================
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) + Box-Muller.
// ======================================================================================

AFQ_D void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2_, uint32_t& c3, uint32_t k0,
                        uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
  uint32_t hi1 = __umulhi(M1, c2_), lo1 = M1 * c2_;
  uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
  c0 = n0; c1 = n1; c2_ = n2; c3 = n3;
}

AFQ_D uint4 philox4x32(uint64_t ctr, uint64_t key) {
  uint32_t c0 = (uint32_t)ctr, c1 = (uint32_t)(ctr >> 32), c2_ = 0x5851F42Du, c3 = 0x14057B7Eu;
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(c0, c1, c2_, c3, k0, k1);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return make_uint4(c0, c1, c2_, c3);
}

// 53-bit uniform in (0, 1] from two words
AFQ_D double u53(uint32_t a, uint32_t b) {
  uint64_t v = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return ((double)v + 1.0) * (1.0 / 9007199254740992.0);
}

__global__ void k_fill_normal(double* out, int64_t n, uint64_t seed, uint64_t offset) {
  int64_t pair = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t i0 = 2 * pair;
  if (i0 >= n) return;
  uint64_t ctr = (offset >> 1) + (uint64_t)pair;
  uint4 r = philox4x32(ctr, seed);
  // Box-Muller in FP32 arithmetic (FP64 transcendentals are slow on this part); u1 uses
  // 32 random bits in (0, 1], so the radius reaches 6.7 sigma
  const float u1 = ((float)r.x + 1.0f) * 2.3283064365386963e-10f;
  const float u2 = (float)(r.z >> 8) * 5.9604644775390625e-08f;
  const float rad = sqrtf(-2.0f * logf(u1));
  float s, co;
  sincospif(2.0f * u2, &s, &co);
  out[i0] = (double)(rad * co);
  if (i0 + 1 < n) out[i0 + 1] = (double)(rad * s);
}

__global__ void k_fill_uniform(double* out, int64_t n, uint64_t seed, uint64_t offset) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint4 r = philox4x32(offset + (uint64_t)i, seed ^ 0x5bd1e995ull);
  out[i] = u53(r.x, r.y) - (1.0 / 9007199254740992.0);
}

// ======================================================================================
// host launchers
// ======================================================================================

static inline int launch_err(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    afq_set_error("%s: %s", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

int check_smem_optin(size_t smem, const char* what) {
  int dev = 0, lim = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;  // no limit known here: the launch reports it
  }
  if (smem > (size_t)lim) {
    afq_set_error("%s: needs %zu bytes of shared memory per block, the device allows %d", what, smem, lim);
    return -2;
  }
  return 0;
}

template <typename WT>
int launch_green(const afq_ctx_dev& c, const void* wu, const void* wd, double2* green,
                 double2* ovl, bool write_green, cudaStream_t st) {
  const size_t smem = green_f64_smem(c.norb, c.kmax);
  if (int rc = check_smem_optin(smem, "green_overlap (norb x occupied orbitals too large)")) return rc;
  auto kfn = k_green_overlap<WT>;
  cudaError_t ea = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (ea != cudaSuccess) {
    afq_set_error("green_overlap: shared-memory attribute: %s", cudaGetErrorString(ea));
    return (int)ea;
  }
  {
    ProfScope _ps(K_GREEN, st);
    kfn<<<c.nw, 256, smem, st>>>(c, (const WT*)wu, (const WT*)wd, green, ovl, write_green ? 1 : 0);
  }
  return launch_err("green_overlap");
}

int launch_gemm_cr(bool b_kn, int M, int N, int K, const double2* A, long lda, const double* B,
                   long ldb, double2* C, long ldc, double2 alpha, cudaStream_t st) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  ProfScope _ps(b_kn ? K_VHS : K_FB, st);
  if (b_kn)
    k_gemm_cr<true><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha);
  else
    k_gemm_cr<false><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha);
  return launch_err("gemm_cr");
}

int launch_field_shifts(const afq_ctx_dev& c, const double* fields, const double2* fb,
                        double2* xt, double2* shift, double2* fbt, cudaStream_t st) {
  {
    ProfScope _ps(K_FIELD, st);
    k_field_shifts<<<c.nw, 256, 0, st>>>(c.nchol, sqrt(c.dt), fields, fb, c.mf, xt, shift, fbt);
  }
  return launch_err("field_shifts");
}

template <typename WT>
int launch_taylor_f64(const afq_ctx_dev& c, int w0, int nwc, const double2* vhs, void* wu, void* wd,
                      cudaStream_t st) {
  size_t smem = 2 * (size_t)c.norb * c.kmax * sizeof(double2);
  auto kfn = k_taylor_f64<WT>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_TAYLOR, st);
    kfn<<<dim3(nwc, c.nslab), 256, smem, st>>>(c, w0, vhs, (WT*)wu, (WT*)wd);
  }
  return launch_err("taylor_f64");
}

int launch_weights(const afq_ctx_dev& c, const double2* shift, const double2* fbt, int ntiles,
                   const double2* ovl_new, double2* ovl, double* weights, double* scalars,
                   cudaStream_t st, const int* status) {
  {
    ProfScope _ps(K_WEIGHTS, st);
    // FP64 transcendentals per walker: 8 walkers per CTA spread them over the SMs' FP64 units
    k_weights<<<(c.nw + 7) / 8, 8, 0, st>>>(c.nw, c.dt, c2(c.h0_prop_re, c.h0_prop_im), shift, fbt, ntiles,
                                            ovl_new, ovl, weights, scalars);
  }
  {
    ProfScope _ps(K_WEIGHTS, st);
    k_pop_control<<<1, 1024, 0, st>>>(c.nw, c.dt, weights, scalars, status);
  }
  return launch_err("weights");
}

int launch_energy_f64(const afq_ctx_dev& c, int nchunks, int gchunk, const double2* green,
                      double2* epart, double2* energy, cudaStream_t st) {
  size_t smem = (size_t)c.ktot * sizeof(double2) + 2 * (size_t)c.kmax * c.kmax * sizeof(double2);
  cudaFuncSetAttribute(k_energy_f64_part, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_ENERGY, st);
    k_energy_f64_part<<<dim3(c.nw, nchunks), 256, smem, st>>>(c, gchunk, green, epart);
  }
  int e = launch_err("energy_part");
  if (e) return e;
  {
    ProfScope _ps(K_ENERGY_FIN, st);
    k_energy_final<<<c.nw, 256, 0, st>>>(c, nchunks, green, epart, energy);
  }
  return launch_err("energy_final");
}

template <typename WT>
int launch_qr(const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st, double2* rdiag) {
  size_t smem = ((size_t)c.norb * c.kmax + 2 * c.kmax) * sizeof(typename CplxOf<WT>::type);
  auto kfn = k_qr_householder<WT>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_QR, st);
    kfn<<<dim3(c.nw, c.nslab), 256, smem, st>>>(c, (WT*)wu, (WT*)wd, rdiag);
  }
  return launch_err("qr_householder");
}

template <typename WT>
int launch_sr(const afq_ctx_dev& c, const double* zeta, double* weights, double* cum, int32_t* idx,
              void* wu, void* wd, void* wcopy, cudaStream_t st) {
  {
    ProfScope _ps(K_SR, st);
    const int in_smem = c.nw * 8 <= 48 * 1024 ? 1 : 0;
    k_sr_indices<<<1, 1024, in_smem ? c.nw * 8 : 0, st>>>(c.nw, zeta, weights, cum, idx, in_smem);
  }
  int e = launch_err("sr_indices");
  if (e) return e;
  using CT = typename CplxOf<WT>::type;
  size_t off = 0;
  for (int s = 0; s < c.nslab; ++s) {
    void* w = s == 0 ? wu : wd;
    size_t elems = (size_t)c.norb * c.kslab[s];
    size_t bytes = elems * c.nw * sizeof(CT);
    char* cp = (char*)wcopy + off;
    cudaMemcpyAsync(cp, w, bytes, cudaMemcpyDeviceToDevice, st);
    {
      ProfScope _ps(K_SR, st);
      k_gather_slab<WT><<<c.nw, 256, 0, st>>>((int)elems, idx, (const WT*)cp, (WT*)w);
    }
    off += bytes;
  }
  return launch_err("sr_gather");
}

int launch_block_stats(const afq_ctx_dev& c, const double2* energy, const double* weights,
                       double* scalars, double* be, double* bw, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_block_stats<<<1, 1024, 0, st>>>(c.nw, c.dt, energy, weights, scalars, be, bw);
  }
  return launch_err("block_stats");
}

int launch_clamped_energies(const afq_ctx_dev& c, const double2* energy, const double* scalars,
                            double* out, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_clamped_energies<<<(c.nw + 255) / 256, 256, 0, st>>>(c.nw, c.dt, energy, scalars, out);
  }
  return launch_err("clamped_energies");
}

int launch_cs_outlier(double* w1, double* w2, const double* e1, const double* e2, int nw,
                      double z_thresh, double* sums, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_cs_outlier<<<1, 1024, 0, st>>>(nw, z_thresh, w1, w2, e1, e2, sums);
  }
  return launch_err("cs_outlier");
}

int launch_phaseless_begin(double* scalars, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_phaseless_begin<<<1, 1, 0, st>>>(scalars);
  }
  return launch_err("phaseless_begin");
}

int launch_phaseless_end(int nblk, double denom, const double* be, const double* bw,
                         double* scalars, double* energy, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_phaseless_end<<<1, 32, 0, st>>>(nblk, denom, be, bw, scalars, energy);
  }
  return launch_err("phaseless_end");
}

int launch_driver_update(const afq_ctx_dev& c, const double* weights, const double* energy,
                         double* scalars, double* wsum, cudaStream_t st) {
  {
    ProfScope _ps(K_STATS, st);
    k_driver_update<<<1, 1024, 0, st>>>(c.nw, weights, energy, scalars, wsum);
  }
  return launch_err("driver_update");
}

int launch_fill_normal(double* out, int64_t n, uint64_t seed, uint64_t offset, cudaStream_t st) {
  if (offset & 1ull) {
    afq_set_error("afq_fill_normal: offset must be even");
    return -1;
  }
  int64_t pairs = (n + 1) / 2;
  if (pairs == 0) return 0;
  {
    ProfScope _ps(K_RNG, st);
    k_fill_normal<<<(unsigned)((pairs + 255) / 256), 256, 0, st>>>(out, n, seed, offset);
  }
  return launch_err("fill_normal");
}

int launch_fill_uniform(double* out, int64_t n, uint64_t seed, uint64_t offset, cudaStream_t st) {
  if (n == 0) return 0;
  {
    ProfScope _ps(K_RNG, st);
    k_fill_uniform<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, seed, offset);
  }
  return launch_err("fill_uniform");
}

template int launch_green<double>(const afq_ctx_dev&, const void*, const void*, double2*, double2*, bool, cudaStream_t);
template int launch_green<float>(const afq_ctx_dev&, const void*, const void*, double2*, double2*, bool, cudaStream_t);
template int launch_taylor_f64<double>(const afq_ctx_dev&, int, int, const double2*, void*, void*, cudaStream_t);
template int launch_taylor_f64<float>(const afq_ctx_dev&, int, int, const double2*, void*, void*, cudaStream_t);
template int launch_qr<double>(const afq_ctx_dev&, void*, void*, cudaStream_t, double2*);
template int launch_qr<float>(const afq_ctx_dev&, void*, void*, cudaStream_t, double2*);
template int launch_sr<double>(const afq_ctx_dev&, const double*, double*, double*, int32_t*, void*, void*, void*, cudaStream_t);
template int launch_sr<float>(const afq_ctx_dev&, const double*, double*, double*, int32_t*, void*, void*, void*, cudaStream_t);

}  // namespace afq

// Constrained-path Monte Carlo for the Hubbard model with on-site U (propagation.py:515-657,
// uhf_cpmc trial wavefunctions.py:848-955), FP64 with real walkers, one CTA per walker:
// one-body half step, overlap and full Green's functions, a sweep over the sites choosing a
// discrete Hubbard-Stratonovich field per site from the overlap ratios with rank-one
// Green's-function updates, one-body half step, weights and the pop-control shift; the
// variant with a nearest-neighbour interaction (propagation.py:889-1230), whose neighbour
// sweep makes two-entry updates within one spin as well; and the continuous-field variant
// (propagation.py:1595-1675).

#include <math.h>

#include "afq_common.cuh"
#include "afq_kernels.cuh"
#include "afq_prof.cuh"

namespace afq {

constexpr int kCpmcThreads = 256;
constexpr int kCpmcMaxOcc = 32;

struct CpmcDev {
  int norb, no[2], nw;
  double dt;
  double hs[2][2];   // [field][spin] Hubbard-Stratonovich constants
  double hsn[2][2];  // [field][entry] constants of the neighbour interaction
  const int32_t* nbr;  // [npairs][2] neighbour sites
  int npairs;
  const double* unif;  // [nw][norb + 4 npairs] uniforms of the neighbour variant
  const double* exph[2];
  const double* trial[2];
  double* w[2];
  double* weights;
  double* overlaps;
  double* greens;  // [nw][2][norb][norb]
  double* scalars;
  const double* gauss;  // [nw][norb]
};

// shared memory: G [2][n][n], W [2][n][kmax], T [n][kmax], Aug [kmax][2 kmax]
static size_t cpmc_smem(int n, int kmax) {
  return (2 * (size_t)n * n + 3 * (size_t)n * kmax + 2 * (size_t)kmax * kmax) * sizeof(double);
}

// W_s <- E_s W_s; S_s = C_s^T W_s; Gauss-Jordan (partial pivoting, |.| of the real entries);
// det; A = W S^-1 into T; G_s = C_s A^T. Returns the product of both determinants
// (thread 0's value is the one used).
__device__ double cpmc_one_body(const CpmcDev& d, double* G, double* Ws, double* T, double* Aug, int kmax,
                                bool apply_exp, bool need_det = true, bool need_green = true) {
  __shared__ double colj[kCpmcMaxOcc];
  __shared__ int piv_sh;
  __shared__ double det_sh;
  const int n = d.norb, tid = threadIdx.x, nt = blockDim.x;
  double det = 1.0;
  for (int s = 0; s < 2; ++s) {
    const int o = d.no[s];
    double* W = Ws + (size_t)s * n * kmax;  // [n][o] (row stride o)
    const double* C = d.trial[s];
    if (apply_exp) {
      const double* E = d.exph[s];
      for (int e = tid; e < n * o; e += nt) {
        const int p = e / o, k = e % o;
        double a = 0.0;
        for (int q = 0; q < n; ++q) a = fma(E[(size_t)p * n + q], W[q * o + k], a);
        T[e] = a;
      }
      __syncthreads();
      for (int e = tid; e < n * o; e += nt) W[e] = T[e];
      __syncthreads();
    }
    if (!need_det) continue;
    for (int e = tid; e < o * o; e += nt) {  // Aug = [S | I]
      const int i = e / o, k = e % o;
      double a = 0.0;
      for (int p = 0; p < n; ++p) a = fma(C[(size_t)p * o + i], W[p * o + k], a);
      Aug[i * 2 * o + k] = a;
      Aug[i * 2 * o + o + k] = (i == k) ? 1.0 : 0.0;
    }
    if (tid == 0) det_sh = 1.0;
    __syncthreads();
    for (int j = 0; j < o; ++j) {
      if (tid < 32) {
        double best = -1.0;
        int bi = j;
        for (int r = j + tid; r < o; r += 32) {
          const double m = fabs(Aug[r * 2 * o + j]);
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
          const double t = Aug[j * 2 * o + e];
          Aug[j * 2 * o + e] = Aug[pr * 2 * o + e];
          Aug[pr * 2 * o + e] = t;
        }
      __syncthreads();
      const double pv = Aug[j * 2 * o + j];
      if (tid == 0) det_sh = (pr != j) ? -det_sh * pv : det_sh * pv;
      __syncthreads();
      for (int e = tid; e < 2 * o; e += nt) Aug[j * 2 * o + e] /= pv;
      for (int r = tid; r < o; r += nt) colj[r] = Aug[r * 2 * o + j];
      __syncthreads();
      for (int e = tid; e < o * 2 * o; e += nt) {
        const int r = e / (2 * o), col = e % (2 * o);
        if (r != j) Aug[e] -= colj[r] * Aug[j * 2 * o + col];
      }
      __syncthreads();
    }
    det *= det_sh;
    if (!need_green) {
      __syncthreads();  // det_sh and Aug are rewritten for the next spin
      continue;
    }
    for (int e = tid; e < n * o; e += nt) {  // A = W S^-1
      const int p = e / o, i = e % o;
      double a = 0.0;
      for (int k = 0; k < o; ++k) a = fma(W[p * o + k], Aug[k * 2 * o + o + i], a);
      T[e] = a;
    }
    __syncthreads();
    double* Gs = G + (size_t)s * n * n;
    for (int e = tid; e < n * n; e += nt) {  // G[i][j] = sum_k C[i][k] A[j][k]
      const int i = e / n, j = e % n;
      double a = 0.0;
      for (int k = 0; k < o; ++k) a = fma(C[(size_t)i * o + k], T[j * o + k], a);
      Gs[e] = a;
    }
    __syncthreads();
  }
  return det;
}

// Two-entry discrete-field update at (spin si, site i), (spin sj, site j)
// (wavefunctions.py:873-945 with propagation.py:949-1220): ratios of both fields from G,
// the field chosen with probability r0 / (r0 + r1) against `uni`, the walker rows scaled,
// overlap * ratio, weight * (r0 + r1) / 2 (thread 0's ov and w), and G updated with both
// steps built from G before the update: the exact rank-two update when si == sj (the
// reference's code reads column j after its first step, which is not; its test checks the
// fast form against the determinant form, which this one matches). Neighbour pairs have
// i != j, so the two scaled rows never coincide.
__device__ void cpmc_pair_update(const CpmcDev& d, double* G, double* Ws, int kmax, int si, int i, int sj, int j,
                                 bool nn, double uni, double& ov, double& w, double* sc, double* coli,
                                 double* colj, double* sgi, double* sgj) {
  const int n = d.norb, tid = threadIdx.x, nt = blockDim.x;
  double* Gi = G + (size_t)si * n * n;
  double* Gj = G + (size_t)sj * n * n;
  const bool same = si == sj;
  if (tid == 0) {
    const double gii = Gi[i * n + i], gjj = Gj[j * n + j];
    const double gij = same ? Gi[i * n + j] : 0.0, gji = same ? Gj[j * n + i] : 0.0;
    double r[2];
    for (int f = 0; f < 2; ++f) {
      const double c0 = (nn ? d.hsn[f][0] : d.hs[f][0]) - 1.0, c1 = (nn ? d.hsn[f][1] : d.hs[f][1]) - 1.0;
      r[f] = (1.0 + c0 * gii) * (1.0 + c1 * gjj) - c0 * c1 * gij * gji;
      if (r[f] < 1.0e-8) r[f] = 0.0;
    }
    double p0 = r[0] / 2.0;
    const double p1 = r[1] / 2.0, norm = p0 + p1;
    p0 /= norm;
    const int f = uni < p0 ? 0 : 1;
    sc[0] = nn ? d.hsn[f][0] : d.hs[f][0];
    sc[1] = nn ? d.hsn[f][1] : d.hs[f][1];
    sc[2] = r[f];
    sc[3] = gii;
    sc[4] = gjj;
    sc[5] = gij;
    sc[6] = gji;
    ov *= r[f];
    w *= norm;
  }
  for (int e = tid; e < n; e += nt) {
    coli[e] = Gi[(size_t)e * n + i];
    colj[e] = Gj[(size_t)e * n + j];
    sgi[e] = Gi[(size_t)i * n + e] - (e == i ? 1.0 : 0.0);
    sgj[e] = Gj[(size_t)j * n + e] - (e == j ? 1.0 : 0.0);
  }
  __syncthreads();
  const double c0 = sc[0], c1 = sc[1], ratio = sc[2], gii = sc[3], gjj = sc[4], gij = sc[5], gji = sc[6];
  const double uc0 = c0 - 1.0, uc1 = c1 - 1.0, fi = uc0 / ratio, fj = uc1 / ratio;
  const int oi = d.no[si], oj = d.no[sj];
  for (int e = tid; e < oi + oj; e += nt) {
    if (e < oi) Ws[(size_t)si * n * kmax + (size_t)i * oi + e] *= c0;
    else Ws[(size_t)sj * n * kmax + (size_t)j * oj + (e - oi)] *= c1;
  }
  for (int e = tid; e < n * n; e += nt) {
    const int a = e / n, b = e % n;
    const double vi = uc1 * (gij * sgj[b] - gjj * sgi[b]) - sgi[b];
    const double vj = uc0 * (gji * sgi[b] - gii * sgj[b]) - sgj[b];
    if (same) {
      Gi[e] += fi * coli[a] * vi + fj * colj[a] * vj;
    } else {
      Gi[e] += fi * coli[a] * vi;
      Gj[e] += fj * colj[a] * vj;
    }
  }
  __syncthreads();
}

// mode 0: overlaps and Green's functions of the given walkers; mode 1: one CPMC step;
// mode 2: one step of the continuous-field variant (no Green's functions); mode 3: one step
// with the nearest-neighbour interaction
__global__ void __launch_bounds__(kCpmcThreads) k_cpmc(const CpmcDev d, int mode) {
  extern __shared__ __align__(16) double csm[];
  __shared__ double colx[2][64], rowx[2][64];
  __shared__ double sc_sh[8];
  const int wl = blockIdx.x, tid = threadIdx.x, nt = blockDim.x, n = d.norb;
  const int kmax = d.no[0] > d.no[1] ? d.no[0] : d.no[1];
  double* G = csm;                             // [2][n][n]
  double* Ws = G + 2 * (size_t)n * n;          // [2][n][kmax]
  double* T = Ws + 2 * (size_t)n * kmax;       // [n][kmax]
  double* Aug = T + (size_t)n * kmax;          // [kmax][2 kmax]
  for (int s = 0; s < 2; ++s) {
    const int o = d.no[s];
    const double* src = d.w[s] + (size_t)wl * n * o;
    for (int e = tid; e < n * o; e += nt) Ws[(size_t)s * n * kmax + e] = src[e];
  }
  __syncthreads();
  // thread 0's copies are authoritative; mode 0 has no weights
  double w = mode ? d.weights[wl] : 0.0, ov = mode ? d.overlaps[wl] : 0.0;
  if (mode == 0) {
    const double det = cpmc_one_body(d, G, Ws, T, Aug, kmax, false);
    if (tid == 0) d.overlaps[wl] = det;
  } else if (mode == 2) {
    // continuous fields (propagator_cpmc_continuous, propagation.py:1595-1675; its force bias
    // is multiplied by zero): exp_h1, rows i times exp(+-x_i hs), exp_h1, overlap ratio
    cpmc_one_body(d, G, Ws, T, Aug, kmax, true, false, false);
    const double hs = d.hs[0][0];
    for (int e = tid; e < n * (d.no[0] + d.no[1]); e += nt) {
      const int s = e < n * d.no[0] ? 0 : 1;
      const int ee = s == 0 ? e : e - n * d.no[0], i = ee / d.no[s];
      const double x = d.gauss[(size_t)wl * n + i];
      Ws[(size_t)s * n * kmax + ee] *= exp(s == 0 ? x * hs : -x * hs);
    }
    __syncthreads();
    const double det = cpmc_one_body(d, G, Ws, T, Aug, kmax, true, true, false);
    if (tid == 0) {
      w *= exp(d.dt * d.scalars[AFQ_S_POP_CONTROL_SHIFT]) * det / ov;
      if (w < 1.0e-8) w = 0.0;
      if (w > 100.0) w = 0.0;
      d.weights[wl] = w;
      d.overlaps[wl] = det;
    }
    for (int s = 0; s < 2; ++s) {
      const int o = d.no[s];
      double* dst = d.w[s] + (size_t)wl * n * o;
      for (int e = tid; e < n * o; e += nt) dst[e] = Ws[(size_t)s * n * kmax + e];
    }
    return;
  } else {
    // one-body half step (propagation.py:539-563)
    double det = cpmc_one_body(d, G, Ws, T, Aug, kmax, true);
    if (tid == 0) {
      w *= det / ov;
      if (w < 1.0e-8) w = 0.0;
      ov = det;
    }
    if (mode == 3) {
      // on-site sweep, then four two-entry updates per neighbour pair (propagation.py:944-1218)
      const double* un = d.unif + (size_t)wl * (n + 4 * d.npairs);
      for (int x = 0; x < n; ++x)
        cpmc_pair_update(d, G, Ws, kmax, 0, x, 1, x, false, un[x], ov, w, sc_sh, colx[0], colx[1], rowx[0],
                         rowx[1]);
      for (int p = 0; p < d.npairs; ++p) {
        const int i = d.nbr[2 * p], j = d.nbr[2 * p + 1];
        if (i < 0 || i >= n || j < 0 || j >= n || i == j) {  // checked on the host as well
          if (tid == 0) d.scalars[AFQ_S_STATUS] = 3.0;
          continue;
        }
        for (int k = 0; k < 4; ++k)
          cpmc_pair_update(d, G, Ws, kmax, k >> 1, i, k & 1, j, true, un[n + k * d.npairs + p], ov, w, sc_sh,
                           colx[0], colx[1], rowx[0], rowx[1]);
      }
    }
    // sweep over the sites (propagation.py:594-648)
    for (int x = 0; x < (mode == 1 ? n : 0); ++x) {
      if (tid == 0) {
        const double guu = G[(size_t)x * n + x], gdd = G[(size_t)n * n + (size_t)x * n + x];
        double r[2];
        for (int f = 0; f < 2; ++f) {
          r[f] = (1.0 + (d.hs[f][0] - 1.0) * guu) * (1.0 + (d.hs[f][1] - 1.0) * gdd);
          if (r[f] < 1.0e-8) r[f] = 0.0;
        }
        double p0 = r[0] / 2.0;
        const double p1 = r[1] / 2.0, norm = p0 + p1;
        p0 /= norm;
        const double uni = (erf(d.gauss[(size_t)wl * n + x] / sqrt(2.0)) + 1.0) / 2.0;
        const int f = uni < p0 ? 0 : 1;
        sc_sh[0] = d.hs[f][0];
        sc_sh[1] = d.hs[f][1];
        sc_sh[2] = r[f];
        sc_sh[3] = guu;
        sc_sh[4] = gdd;
        ov *= r[f];
        w *= norm;
      }
      for (int e = tid; e < 2 * n; e += nt) {  // column x and row x (minus e_x) of both G
        const int s = e / n, i = e % n;
        colx[s][i] = G[(size_t)s * n * n + (size_t)i * n + x];
        rowx[s][i] = G[(size_t)s * n * n + (size_t)x * n + i] - (i == x ? 1.0 : 0.0);
      }
      __syncthreads();
      const double cu = sc_sh[0], cd = sc_sh[1], ratio = sc_sh[2], guu = sc_sh[3], gdd = sc_sh[4];
      const double uc0 = cu - 1.0, uc1 = cd - 1.0;
      // walker rows x times the chosen constants
      for (int e = tid; e < d.no[0] + d.no[1]; e += nt) {
        if (e < d.no[0]) Ws[(size_t)x * d.no[0] + e] *= cu;
        else Ws[(size_t)n * kmax + (size_t)x * d.no[1] + (e - d.no[0])] *= cd;
      }
      // wavefunctions.py:916-945 for the update indices (0, x), (1, x)
      const double fi = uc0 / ratio, fj = uc1 / ratio;
      for (int e = tid; e < n * n; e += nt) {
        const int i = e / n, j = e % n;
        G[e] += fi * colx[0][i] * (uc1 * (-gdd * rowx[0][j]) - rowx[0][j]);
        G[(size_t)n * n + e] += fj * colx[1][i] * (uc0 * (-guu * rowx[1][j]) - rowx[1][j]);
      }
      __syncthreads();
    }
    // one-body half step
    det = cpmc_one_body(d, G, Ws, T, Aug, kmax, true);
    if (tid == 0) {
      w *= det / ov;
      if (w < 1.0e-8) w = 0.0;
      ov = det;
      w *= exp(d.dt * d.scalars[AFQ_S_POP_CONTROL_SHIFT]);
      if (w > 100.0) w = 0.0;
      d.weights[wl] = w;
      d.overlaps[wl] = ov;
    }
    for (int s = 0; s < 2; ++s) {
      const int o = d.no[s];
      double* dst = d.w[s] + (size_t)wl * n * o;
      for (int e = tid; e < n * o; e += nt) dst[e] = Ws[(size_t)s * n * kmax + e];
    }
  }
  double* gout = d.greens + (size_t)wl * 2 * n * n;
  for (int e = tid; e < 2 * n * n; e += nt) gout[e] = G[e];
}

// pop_control_ene_shift = e_estimate - 0.1 log(sum w / nw) / dt (propagation.py:654-656)
__global__ void k_cpmc_pop_control(int nw, double dt, const double* __restrict__ weights,
                                   double* __restrict__ scalars) {
  __shared__ double red[32];
  double sum = 0.0;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) sum += weights[w];
  sum = block_sum(sum, red);
  if (threadIdx.x == 0)
    scalars[AFQ_S_POP_CONTROL_SHIFT] = scalars[AFQ_S_E_ESTIMATE] - 0.1 * log(sum / (double)nw) / dt;
}

int launch_cpmc(int norb, int n_up, int n_dn, int nw, double dt, double u, const double* exp_up,
                const double* exp_dn, const double* trial_up, const double* trial_dn, double* w_up, double* w_dn,
                double* weights, double* overlaps, double* greens, double* scalars, const double* gauss, int mode,
                cudaStream_t st, double u1, const int32_t* neighbors, int npairs, const double* uniforms) {
  if (norb < 1 || norb > 64 || n_up < 1 || n_dn < 1 || n_up > kCpmcMaxOcc || n_dn > kCpmcMaxOcc || n_up > norb ||
      n_dn > norb || nw < 1) {
    afq_set_error("cpmc: sizes out of range (norb <= 64, 1 <= n_up, n_dn <= min(32, norb))");
    return -1;
  }
  CpmcDev d;
  d.norb = norb;
  d.no[0] = n_up;
  d.no[1] = n_dn;
  d.nw = nw;
  d.dt = dt;
  if (mode == 2) {  // u is the continuous constant ham_data["hs_constant"]
    d.hs[0][0] = d.hs[0][1] = d.hs[1][0] = d.hs[1][1] = u;
  } else {
    const double gamma = acosh(exp(dt * u / 2.0)), cst = exp(-dt * u / 2.0);
    d.hs[0][0] = cst * exp(gamma);
    d.hs[0][1] = cst * exp(-gamma);
    d.hs[1][0] = cst * exp(-gamma);
    d.hs[1][1] = cst * exp(gamma);
  }
  if (mode == 3) {
    if (npairs < 0 || (npairs > 0 && !neighbors) || !uniforms) {
      afq_set_error("cpmc: neighbour variant needs the neighbour list and the uniforms");
      return -1;
    }
    const double g1 = acosh(exp(dt * u1 / 2.0)), c1 = exp(-dt * u1 / 2.0);
    d.hsn[0][0] = c1 * exp(g1);
    d.hsn[0][1] = c1 * exp(-g1);
    d.hsn[1][0] = c1 * exp(-g1);
    d.hsn[1][1] = c1 * exp(g1);
  } else {
    d.hsn[0][0] = d.hsn[0][1] = d.hsn[1][0] = d.hsn[1][1] = 0.0;
  }
  d.nbr = neighbors;
  d.npairs = mode == 3 ? npairs : 0;
  d.unif = uniforms;
  d.exph[0] = exp_up;
  d.exph[1] = exp_dn;
  d.trial[0] = trial_up;
  d.trial[1] = trial_dn;
  d.w[0] = w_up;
  d.w[1] = w_dn;
  d.weights = weights;
  d.overlaps = overlaps;
  d.greens = greens;
  d.scalars = scalars;
  d.gauss = gauss;
  const int kmax = n_up > n_dn ? n_up : n_dn;
  const size_t smem = cpmc_smem(norb, kmax);
  cudaFuncSetAttribute(k_cpmc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    ProfScope _ps(K_WEIGHTS, st);
    k_cpmc<<<nw, kCpmcThreads, smem, st>>>(d, mode);
    if (mode != 0) k_cpmc_pop_control<<<1, 1024, 0, st>>>(nw, dt, weights, scalars);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    afq_set_error("cpmc: %s", cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

}  // namespace afq

// Device code of the mixed-precision path: 16-bit operand packing, the Green's function /
// overlap kernel (FP32 Gauss-Jordan, FP64 log-determinant), GEMM epilogues (fused field
// shifts, vhs scatter into the Taylor layout, exp_h1 products, exchange/Coulomb energy),
// the per-walker tcgen05 Taylor kernel, and one-time operand preparation.
#pragma once
#include <cuda_fp16.h>

#include "afq_tc.cuh"

namespace afq {

// ---- 16-bit helpers -------------------------------------------------------------------

__device__ __forceinline__ uint16_t f2h(float x, bool bf) {
  return bf ? __bfloat16_as_ushort(__float2bfloat16_rn(x)) : __half_as_ushort(__float2half_rn(x));
}
__device__ __forceinline__ float h2f(uint16_t h, bool bf) {
  return bf ? __bfloat162float(__ushort_as_bfloat16(h)) : __half2float(__ushort_as_half(h));
}
// x ~ hi + lo with both parts 16-bit
__device__ __forceinline__ void split16(float x, bool bf, uint16_t& hi, uint16_t& lo) {
  hi = f2h(x, bf);
  lo = f2h(x - h2f(hi, bf), bf);
}
// byte offset of (row r, column k < 64) inside a [rows x 64] 16-bit tile, 128-byte swizzle
__device__ __forceinline__ uint32_t sw128(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 3) ^ (r & 7)) << 4) | ((k & 7) << 1)));
}
// exact power of two 2^-e with 2^-e * amax in (0.5, 1]; 1 for amax == 0
__device__ __forceinline__ float pow2_scale(float amax) {
  if (!(amax > 0.0f) || !isfinite(amax)) return 1.0f;
  int e;
  frexpf(amax, &e);  // amax = m * 2^e, m in [0.5, 1)
  return ldexpf(1.0f, -e);
}

// Plain-data view of the mixed state passed to kernels.
struct MixedDev {
  int n, nq, nk, ldfb, ldg, nw, nchol, nslab, nblk, kfb, restricted_square, energy_mode;
  int o_slab[2], R[2], o_blk[2], ldkb[2];
  int bf16;
  double h0;
  const float* trial32[2];
  const float* rh1_32[2];
  uint16_t* g_fb[2];
  uint16_t* g_blk[2][2];  // per-block Green operand (two Green blocks only)
  uint16_t* wt[2][2];
  float* g_inv;
  double2* ene1;
};

constexpr int kGreenMaxO = 40;  // occupied orbitals per slab (S is at most 40 x 40)

// dst[map(e)] = src[e] for e < n by a block of NT threads, 8 independent loads in flight per
// thread before the shared-memory stores (the copies are latency-bound otherwise)
template <int NT, class T, class Map>
__device__ __forceinline__ void copy_batched(T* dst, const T* __restrict__ src, int n, Map map) {
  for (int base = threadIdx.x; base < n; base += 8 * NT) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * NT;
      if (e < n) v[u] = src[e];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * NT;
      if (e < n) dst[map(e)] = v[u];
    }
  }
}

// Row stride (complex elements) of the walker copy in k_green_fused: a multiple of 4 columns
// rounded so that stride / 2 is odd (16-byte aligned rows; the row-per-thread reads of the
// operand packing then hit each shared-memory bank at most twice per half warp).
__host__ __device__ constexpr int green_s_ld(int o) {
  return ((((o + 3) & ~3) >> 1) & 1) ? ((o + 3) & ~3) : ((o + 3) & ~3) + 2;
}

// ======================================================================================
// Green's function, overlap and operands in one kernel, one CTA (NT = 128 or 256 threads)
// per walker (wavefunctions.py:478-501 rhf, 658-692 uhf). Per slab: the walker and trial
// copied to shared memory; S = C^T W (FP32, the orbital sum split over the NT / 128 thread
// groups); Gauss-Jordan with partial pivoting on S, double-buffered in shared memory with one
// barrier per pivot, thread (row group g = warp, column c = lane) updating rows g, g + NW, ..
// of column c (NW warps); the determinant as the FP64 signed product of the pivots (squared
// for restricted walkers); then, with kGreenG, G = (W S^-1)^T, its power-of-two scale, the
// 16-bit operands and ene1 = sum G * rot_h1, with thread (p = tid % 128, h = tid / 128) on
// orbital p and share h of the occupied columns.
// kGreenWT also writes the walker operand of the exp_h1 products.
// Pivoting is implicit, as in a row-per-lane register version: no rows move; the pivot of
// step j is the unused row with the largest |re| + |im| in column j (ties to the lower row).
// The working matrix ends as P^T S^-1 P^T for the pivot order P: its row r is row step(r)
// of S^-1 and its column c is column piv(c); det(S) = sign(P) * prod(pivots).
// ======================================================================================

constexpr int kGreenWT = 1, kGreenG = 2;
constexpr int kGfThreads = 128;  // threads per walker CTA (128 or 256; 128 measured faster)

// G lives in its own region when two slabs contribute to it or norb > 128 (each thread then
// owns two orbital rows); with one slab and norb <= 128 it overwrites the walker copy once
// G's inputs are in registers
__host__ __device__ constexpr size_t green_fused_smem(int n, int omax, int om, int gtot, bool g, int nslab) {
  return (((size_t)n * green_s_ld(omax) * 8 + 15) & ~(size_t)15) +
         (size_t)om * kGreenMaxO * 8 + ((g && (nslab == 2 || n > 128)) ? (size_t)gtot * n * 8 : 0);
}

// dst[(e / o) * ld + e % o] = src[e] for e < n * o, 8 loads in flight per thread, the row and
// column advanced incrementally (no division per element)
template <int NT>
__device__ __forceinline__ void copy_rows(float2* dst, const float2* __restrict__ src, int n, int o, int ld) {
  const int total = n * o, dq = NT / o, dr = NT - dq * o;
  int p = threadIdx.x / o, k = threadIdx.x - p * o;
  for (int base = threadIdx.x; base < total; base += 8 * NT) {
    float2 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * NT;
      if (e < total) v[u] = src[e];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * NT;
      if (e < total) dst[p * ld + k] = v[u];
      p += dq;
      k += dr;
      if (k >= o) {
        k -= o;
        ++p;
      }
    }
  }
}

template <int OM, int NT>
__global__ void __launch_bounds__(NT, (OM <= 24 ? 640 : 512) / NT) k_green_fused(const MixedDev md, const float2* __restrict__ wu,
                                                               const float2* __restrict__ wd,
                                                               double2* __restrict__ ovl, int flags) {
  extern __shared__ __align__(16) unsigned char sm[];
  constexpr int NW = NT / 32, NH = NT / 128;  // warps; thread groups of 128 (orbital rows)
  constexpr int RPT = (OM + NW - 1) / NW;     // rows of S per thread in the Gauss-Jordan phase
  constexpr int CPL = (OM + 31) / 32;          // columns of S per lane (lane, lane + 32)
  constexpr int RB = CPL == 1 ? 5 : 6;         // bits of the row index in the pivot-search key
  const int w = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, n = md.n;
  const int p0 = tid & 127, h = tid >> 7;  // orbital rows p0, p0 + 128 (norb <= 256)
  const bool overlay = md.nslab == 1 && n <= 128;  // G overwrites the walker copy
  const int omax = md.o_slab[0] > md.o_slab[1] ? md.o_slab[0] : md.o_slab[1];
  const int ldmax = green_s_ld(omax);
  const bool do_g = (flags & kGreenG) != 0;
  const int gtot = md.o_blk[0] + md.o_blk[1];
  float2* Ws = reinterpret_cast<float2*>(sm);                    // [n][ld] (columns >= o zero)
  float2* Si = reinterpret_cast<float2*>(sm + (((size_t)n * ldmax * 8 + 15) & ~(size_t)15));  // [OM][kGreenMaxO]
  // [gtot][n]: after the walker copy's last use when it overlays it (ld >= o = gtot)
  float2* Gs = overlay ? Ws : Si + OM * kGreenMaxO;
  __shared__ float2 Ssh[2][OM][OM + 1];  // S (partials), then the double-buffered working matrix
  __shared__ float2 pivv[OM];
  __shared__ int piv_s[OM], step_s[OM];
  __shared__ float2 e1w[NW], e1l[NW];
  __shared__ float fred[NW];
  const bool bf = md.bf16 != 0;
  double2 det = c2(1.0, 0.0);  // thread 0
  for (int s = 0; s < md.nslab; ++s) {
    const int o = md.o_slab[s], o4 = (o + 3) & ~3, ld = green_s_ld(o);
    const float2* W = (s == 0 ? wu : wd) + (size_t)w * n * o;
    const float* __restrict__ Ct = md.trial32[s];  // [n][o] trial in FP32
    if (o4 != o)
      for (int pp = tid; pp < n; pp += NT)
        for (int k = o; k < o4; ++k) Ws[pp * ld + k] = make_float2(0.f, 0.f);
    copy_rows<NT>(Ws, W, n, o, ld);
    __syncthreads();
    for (int p = p0; (flags & kGreenWT) && p < n; p += 128) {  // walker operand of the exp_h1 products: row (w, 2k + c), column p
      uint16_t* hi = md.wt[s][0] + (size_t)w * md.R[s] * md.nk + p;
      uint16_t* lo = md.wt[s][1] + (size_t)w * md.R[s] * md.nk + p;
      for (int k = h; k < o; k += NH) {
        const float2 v = Ws[p * ld + k];
        uint16_t hh, l;
        split16(v.x, bf, hh, l);
        hi[(size_t)(2 * k) * md.nk] = hh;
        lo[(size_t)(2 * k) * md.nk] = l;
        split16(v.y, bf, hh, l);
        hi[(size_t)(2 * k + 1) * md.nk] = hh;
        lo[(size_t)(2 * k + 1) * md.nk] = l;
      }
    }
    // S[i][k..k+3] = sum_p C[p][i] W[p][k..k+3], orbitals split in two halves (partials in
    // Ssh[0] and Ssh[1], then summed)
    const int nk4 = o4 / 4, nh = (n + NH - 1) / NH;
    for (int e = tid; e < NH * o * nk4; e += NT) {
      const int hh = e / (o * nk4), e2 = e - hh * o * nk4;
      const int i = e2 / nk4, k0 = (e2 - i * nk4) * 4;
      float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
      const int p1 = hh + 1 == NH ? n : (hh + 1) * nh;
#pragma unroll 4
      for (int pp = hh * nh; pp < p1; ++pp) {
        const float cv = __ldg(&Ct[pp * o + i]);  // the trial: the same for every walker (L1)
        const float4 x = *reinterpret_cast<const float4*>(&Ws[pp * ld + k0]);
        const float4 y = *reinterpret_cast<const float4*>(&Ws[pp * ld + k0 + 2]);
        a0.x = fmaf(cv, x.x, a0.x); a0.y = fmaf(cv, x.y, a0.y);
        a1.x = fmaf(cv, x.z, a1.x); a1.y = fmaf(cv, x.w, a1.y);
        a2.x = fmaf(cv, y.x, a2.x); a2.y = fmaf(cv, y.y, a2.y);
        a3.x = fmaf(cv, y.z, a3.x); a3.y = fmaf(cv, y.w, a3.y);
      }
      float2* Sr = &Ssh[hh][i][k0];
      Sr[0] = a0;
      if (k0 + 1 < o) Sr[1] = a1;
      if (k0 + 2 < o) Sr[2] = a2;
      if (k0 + 3 < o) Sr[3] = a3;
    }
    __syncthreads();
    if (NH == 2) {
#pragma unroll
      for (int cc = 0; cc < CPL; ++cc) {
        const int col = lane + 32 * cc;
        if (col < o) {
#pragma unroll
          for (int m = 0; m < RPT; ++m) {
            const int r = warp + NW * m;
            if (r < o) Ssh[0][r][col] = cadd(Ssh[0][r][col], Ssh[1][r][col]);
          }
        }
      }
      __syncthreads();
    }
    // Gauss-Jordan, double-buffered in shared memory: step j reads Ssh[j & 1] and writes
    // Ssh[(j & 1) ^ 1], so one barrier per pivot; thread (warp, lane) updates rows
    // warp, warp + 8, .. of columns lane (and lane + 32 for more than 32 electrons).
    bool used[CPL];  // row lane + 32 cc already pivoted (the same in every warp)
#pragma unroll
    for (int cc = 0; cc < CPL; ++cc) used[cc] = lane + 32 * cc >= o;
#pragma unroll 1
    for (int j = 0; j < o; ++j) {
      const int b = j & 1;
      // loads that do not depend on the pivot first: column j (search), own elements, and
      // the column-j factors of the own rows
      float2 own[RPT][CPL], fj[RPT];
#pragma unroll
      for (int m = 0; m < RPT; ++m) {
        const int r = warp + NW * m;
#pragma unroll
        for (int cc = 0; cc < CPL; ++cc)
          own[m][cc] = (r < o && lane + 32 * cc < o) ? Ssh[b][r][lane + 32 * cc] : make_float2(0.f, 0.f);
        fj[m] = r < o ? Ssh[b][r][j] : make_float2(0.f, 0.f);
      }
      unsigned key = 0u;  // |re| + |im| of the candidate rows with the row index in the low bits
#pragma unroll
      for (int cc = 0; cc < CPL; ++cc) {
        const int row = lane + 32 * cc;
        const float2 v = row < o ? Ssh[b][row][j] : make_float2(0.f, 0.f);
        const float mag = fabsf(v.x) + fabsf(v.y);
        const unsigned kc = used[cc] ? 0u
                                     : ((__float_as_uint(mag) & ~((1u << RB) - 1u)) |
                                        (unsigned)((1 << RB) - 1 - row));
        key = kc > key ? kc : key;
      }
      const int pr = (1 << RB) - 1 - (int)(__reduce_max_sync(0xffffffffu, key) & ((1u << RB) - 1u));
#pragma unroll
      for (int cc = 0; cc < CPL; ++cc)
        if (lane + 32 * cc == pr) used[cc] = true;
      const float2 pv = Ssh[b][pr][j];
      // 1 / pv = conj(pv) / |pv|^2 with pv scaled by a power of two first (no overflow)
      int ex;
      frexpf(fmaxf(fabsf(pv.x), fabsf(pv.y)), &ex);
      const float px = ldexpf(pv.x, -ex), py = ldexpf(pv.y, -ex);
      const float dd = ldexpf(__frcp_rn(fmaf(px, px, py * py)), -ex);
      const float2 inv = make_float2(px * dd, -py * dd);
#pragma unroll
      for (int cc = 0; cc < CPL; ++cc) {
        const int col = lane + 32 * cc;
        if (col < o) {
          const float2 ap = Ssh[b][pr][col];
          const float2 sp = (col == j) ? inv : cmul(ap, inv);
#pragma unroll
          for (int m = 0; m < RPT; ++m) {
            const int r = warp + NW * m;
            if (r < o)
              Ssh[b ^ 1][r][col] =
                  (r == pr) ? sp : csub((col == j) ? make_float2(0.f, 0.f) : own[m][cc], cmul(fj[m], sp));
          }
        }
      }
      if (tid == 0) {
        pivv[j] = pv;
        piv_s[j] = pr;
        step_s[pr] = j;
      }
      __syncthreads();
    }
    const int fbuf = o & 1;  // buffer holding the final working matrix
    if (warp == 0) {  // det: FP64 product of the pivots (a shuffle tree), sign of the pivot order
      int cnt = 0;
      double2 pd = c2(1.0, 0.0);
#pragma unroll
      for (int cc = 0; cc < CPL; ++cc) {
        const int x = lane + 32 * cc;
        if (x < o) {
          for (int y = x + 1; y < o; ++y) cnt += piv_s[x] > piv_s[y] ? 1 : 0;
          pd = cmul(pd, c2((double)pivv[x].x, (double)pivv[x].y));
        }
      }
      cnt = __reduce_add_sync(0xffffffffu, cnt);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        pd = cmul(pd, c2(__shfl_xor_sync(0xffffffffu, pd.x, off), __shfl_xor_sync(0xffffffffu, pd.y, off)));
      if (lane == 0) det = cmul(det, (cnt & 1) ? c2(-pd.x, -pd.y) : pd);
    }
    if (!do_g) {
      __syncthreads();  // the next slab rewrites Ws and Ssh
      continue;
    }
#pragma unroll
    for (int cc = 0; cc < CPL; ++cc) {
      const int col = lane + 32 * cc;
      if (col < o) {
#pragma unroll
        for (int m = 0; m < RPT; ++m) {
          const int r = warp + NW * m;
          if (r < o) Si[step_s[r] * kGreenMaxO + piv_s[col]] = Ssh[fbuf][r][col];
        }
      }
    }
    __syncthreads();
    // overlay: one row per thread and one pass, every thread reaching the barrier; otherwise
    // rows p0 and p0 + 128, G in its own region
    for (int p = p0; p < (overlay ? 128 : n); p += 128) {
      const bool prow_ok = p < n;
      float2 wr[OM];
#pragma unroll
      for (int k = 0; k < OM; ++k) wr[k] = (prow_ok && k < o) ? Ws[p * ld + k] : make_float2(0.f, 0.f);
      if (overlay) __syncthreads();  // G overwrites the walker copy
      if (!prow_ok) continue;
      const int b = md.nblk == 2 ? s : 0;
      float2* Gb = Gs + (size_t)(b == 0 ? 0 : md.o_blk[0]) * n;
      // four columns i at a time (this half's groups): independent accumulation chains,
      // 16-byte reads of S^-1
      for (int i0 = 4 * h; i0 < o; i0 += 4 * NH) {
        float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
#pragma unroll
        for (int k = 0; k < OM; ++k) {
          if (k < o) {
            const float4 s01 = *reinterpret_cast<const float4*>(&Si[k * kGreenMaxO + i0]);
            const float4 s23 = *reinterpret_cast<const float4*>(&Si[k * kGreenMaxO + i0 + 2]);
            a0 = cadd(a0, cmul(wr[k], make_float2(s01.x, s01.y)));
            a1 = cadd(a1, cmul(wr[k], make_float2(s01.z, s01.w)));
            a2 = cadd(a2, cmul(wr[k], make_float2(s23.x, s23.y)));
            a3 = cadd(a3, cmul(wr[k], make_float2(s23.z, s23.w)));
          }
        }
        const float2 av[4] = {a0, a1, a2, a3};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u;
          if (i < o) {
            float2 acc = av[u];
            if (md.nblk == 1 && s == 1) acc = cadd(acc, Gb[(size_t)i * n + p]);  // RHF two slabs
            Gb[(size_t)i * n + p] = acc;
          }
        }
      }
    }
    __syncthreads();  // Ws, Ssh and Si are rewritten by the next slab
  }
  if (tid == 0 && ovl) ovl[w] = md.restricted_square ? cmul(det, det) : det;
  if (!do_g) return;
  float mx = 0.f;
  for (int p = p0; p < n; p += 128)
    for (int i = h; i < gtot; i += NH) {
      const float2 g = Gs[(size_t)i * n + p];
      mx = fmaxf(mx, fmaxf(fabsf(g.x), fabsf(g.y)));
    }
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if (lane == 0) fred[warp] = mx;
  __syncthreads();
  float mall = fred[0];
#pragma unroll
  for (int q = 1; q < NW; ++q) mall = fmaxf(mall, fred[q]);
  const float scl = pow2_scale(mall);
  if (tid == 0) md.g_inv[w] = 1.0f / scl;
  float e1x = 0.f, e1y = 0.f;  // per-thread partials of <= 64 terms; FP64 across warps
  for (int p = p0; p < n; p += 128) {
    for (int i = h; i < gtot; i += NH) {
      const float2 g = Gs[(size_t)i * n + p];
      const int e = i * n + p;
      uint16_t hh, l;
      split16(g.x * scl, bf, hh, l);
      md.g_fb[0][(size_t)(2 * w) * md.ldfb + e] = hh;
      md.g_fb[1][(size_t)(2 * w) * md.ldfb + e] = l;
      split16(g.y * scl, bf, hh, l);
      md.g_fb[0][(size_t)(2 * w + 1) * md.ldfb + e] = hh;
      md.g_fb[1][(size_t)(2 * w + 1) * md.ldfb + e] = l;
      const int b = (md.nblk == 2 && i >= md.o_blk[0]) ? 1 : 0;
      const int eb = e - b * md.o_blk[0] * n;
      if (md.nblk == 2) {  // per-block operand (exchange / Coulomb of each spin separately)
        split16(g.x * scl, bf, hh, l);
        md.g_blk[b][0][(size_t)(2 * w) * md.ldkb[b] + eb] = hh;
        md.g_blk[b][1][(size_t)(2 * w) * md.ldkb[b] + eb] = l;
        split16(g.y * scl, bf, hh, l);
        md.g_blk[b][0][(size_t)(2 * w + 1) * md.ldkb[b] + eb] = hh;
        md.g_blk[b][1][(size_t)(2 * w + 1) * md.ldkb[b] + eb] = l;
      }
      const float r1 = md.rh1_32[b][eb];
      e1x = fmaf(g.x, r1, e1x);
      e1y = fmaf(g.y, r1, e1y);
    }
  }
  // warp sums as unevaluated float pairs (hi + lo, Knuth's TwoSum at every level)
  float lx = 0.f, ly = 0.f;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float ox = __shfl_xor_sync(0xffffffffu, e1x, off), oy = __shfl_xor_sync(0xffffffffu, e1y, off);
    const float olx = __shfl_xor_sync(0xffffffffu, lx, off), oly = __shfl_xor_sync(0xffffffffu, ly, off);
    float sx = e1x + ox, bx = sx - e1x;
    lx += olx + ((e1x - (sx - bx)) + (ox - bx));
    e1x = sx;
    float sy = e1y + oy, by = sy - e1y;
    ly += oly + ((e1y - (sy - by)) + (oy - by));
    e1y = sy;
  }
  if (lane == 0) {
    e1w[warp] = make_float2(e1x, e1y);
    e1l[warp] = make_float2(lx, ly);
  }
  __syncthreads();
  if (tid == 0) {
    double2 t = c2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < NW; ++q)
      t = c2(t.x + ((double)e1w[q].x + (double)e1l[q].x), t.y + ((double)e1w[q].y + (double)e1l[q].y));
    md.ene1[w] = t;
  }
}

// ======================================================================================
// Force-bias GEMM epilogue: rows (w, re/im) of fb = alpha * G . rot_chol^T, fused with the
// field shifts of propagation.py:121-127 (writes the shifted-field operand and per-tile
// partial sums of shift_term and fb_term), or, for calc_force_bias, the plain force bias.
// ======================================================================================

struct EpiFB {
  struct Params {
    const double* fields;
    const double2* mf;
    const float* rc_inv;
    const float* g_inv;
    float alpha, sqdt;
    int nw, nchol, ldg, ntiles, bf16;
    uint16_t* xt_hi;
    uint16_t* xt_lo;
    double2* part_shift;
    double2* part_fbt;
    double2* fb_out;  // non-null: write the force bias instead
  };
  static constexpr int kSmemBytes = 0;
  __device__ static void run(const Params& p, int m0, int n0, int bn, uint32_t tmem, int q, int lane,
                             unsigned char*, bool) {
    const int R = m0 + q * 32 + lane, w = R >> 1, c = R & 1;
    const bool valid = w < p.nw;
    const float gi = valid ? p.g_inv[w] : 0.f;
    const bool bf = p.bf16 != 0;
    float shx = 0.f, shy = 0.f, fbx = 0.f, fby = 0.f;
#pragma unroll 1
    for (int c0 = 0; c0 < bn; c0 += 16) {
      float v[16];
      ptx::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + c0, v);
      ptx::tmem_ld_wait();
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int g = n0 + c0 + j;
        const bool gv = g < p.nchol;
        const float val = v[j] * p.alpha * gi * (gv ? p.rc_inv[g] : 0.f);
        const float other = __shfl_xor_sync(0xffffffffu, val, 1);
        if (!valid || !gv) continue;
        const float fr = c ? other : val, fi = c ? val : other;
        if (p.fb_out) {
          if (c == 0) p.fb_out[(size_t)w * p.nchol + g] = c2(fr, fi);
          continue;
        }
        const double2 mfd = p.mf[g];
        const float mfr = (float)mfd.x, mfi = (float)mfd.y;
        const float sr = -p.sqdt * (-fi - mfr), si = -p.sqdt * (fr - mfi);
        const float x = (float)p.fields[(size_t)w * p.nchol + g];
        const float xtr = x - sr, xti = -si;
        uint16_t h, l;
        split16(c ? xti : xtr, bf, h, l);
        p.xt_hi[(size_t)R * p.ldg + g] = h;
        p.xt_lo[(size_t)R * p.ldg + g] = l;
        if (c == 0) {
          shx += xtr * mfr - xti * mfi;
          shy += xtr * mfi + xti * mfr;
          fbx += x * sr - 0.5f * (sr * sr - si * si);
          fby += x * si - sr * si;
        }
      }
    }
    if (valid && c == 0 && !p.fb_out) {
      p.part_shift[(size_t)w * p.ntiles + blockIdx.x] = c2(shx, shy);
      p.part_fbt[(size_t)w * p.ntiles + blockIdx.x] = c2(fbx, fby);
    }
  }
};

// Force bias from the K-split partials of fb = G . rot_chol^T (rows (w, re/im)), one CTA
// per walker: sums the partials in split order, then the same scaling, field shifts and
// shift_term / fb_term sums as EpiFB (propagation.py:121-127), the sums reduced over all
// Cholesky vectors (part_shift / part_fbt hold one entry per walker).
struct FbReduce {
  const float* part;  // [ksplit][2 nw][ldp]
  int ksplit, nw, nchol, ldg, bf16;
  long ldp, sst;
  const double* fields;
  const double2* mf;
  const float* rc_inv;
  const float* g_inv;
  float alpha, sqdt;
  uint16_t* xt_hi;
  uint16_t* xt_lo;
  double2* part_shift;  // [nw]
  double2* part_fbt;    // [nw]
  double2* fb_out;      // non-null: write the force bias instead
};

__global__ void __launch_bounds__(256, 3) k_fb_reduce(const FbReduce r) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  const float gi = r.g_inv[w];
  const bool bf = r.bf16 != 0;
  float shx = 0.f, shy = 0.f, fbx = 0.f, fby = 0.f;
  const float* pr = r.part + (long)(2 * w) * r.ldp;
  const float* pi = pr + r.ldp;
  // four Cholesky indices per thread at a time, all loads issued before any store (the
  // 16-bit stores may alias the loads for the compiler)
  for (int g0 = threadIdx.x; g0 < r.nchol; g0 += 4 * blockDim.x) {
    float ar[4], ai[4], rc[4], xv[4];
    double2 mfv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int g = g0 + u * blockDim.x;
      ar[u] = ai[u] = rc[u] = xv[u] = 0.f;
      mfv[u] = c2(0.0, 0.0);
      if (g < r.nchol) {
        for (int ks = 0; ks < r.ksplit; ++ks) {
          ar[u] += pr[(long)ks * r.sst + g];
          ai[u] += pi[(long)ks * r.sst + g];
        }
        rc[u] = r.rc_inv[g];
        if (!r.fb_out) {
          xv[u] = (float)r.fields[(size_t)w * r.nchol + g];
          mfv[u] = r.mf[g];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int g = g0 + u * blockDim.x;
      if (g >= r.nchol) continue;
      const float fr = ar[u] * r.alpha * gi * rc[u], fi = ai[u] * r.alpha * gi * rc[u];
      if (r.fb_out) {
        r.fb_out[(size_t)w * r.nchol + g] = c2(fr, fi);
        continue;
      }
      const float mfr = (float)mfv[u].x, mfi = (float)mfv[u].y;
      const float sr = -r.sqdt * (-fi - mfr), si = -r.sqdt * (fr - mfi);
      const float x = xv[u];
      const float xtr = x - sr, xti = -si;
      uint16_t h, l;
      split16(xtr, bf, h, l);
      r.xt_hi[(size_t)(2 * w) * r.ldg + g] = h;
      r.xt_lo[(size_t)(2 * w) * r.ldg + g] = l;
      split16(xti, bf, h, l);
      r.xt_hi[(size_t)(2 * w + 1) * r.ldg + g] = h;
      r.xt_lo[(size_t)(2 * w + 1) * r.ldg + g] = l;
      shx += xtr * mfr - xti * mfi;
      shy += xtr * mfi + xti * mfr;
      fbx += x * sr - 0.5f * (sr * sr - si * si);
      fby += x * si - sr * si;
    }
  }
  if (r.fb_out) return;
  // the four sums reduced together: warp shuffles on unevaluated float pairs (hi + lo,
  // Knuth's TwoSum at every level: no FP64 on the shuffle path), then one FP64 pass over the
  // warps in shared memory
  float v[4] = {shx, shy, fbx, fby}, vl[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float o = __shfl_xor_sync(0xffffffffu, v[j], off), ol = __shfl_xor_sync(0xffffffffu, vl[j], off);
      const float sum = v[j] + o, bb = sum - v[j];
      vl[j] += ol + ((v[j] - (sum - bb)) + (o - bb));
      v[j] = sum;
    }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < 4; ++j) red[4 * wid + j] = (double)v[j] + (double)vl[j];
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int i = 0; i < nwarp; ++i) t += red[4 * i + threadIdx.x];
    red[threadIdx.x] = t;  // each thread wrote only its own slot of warp 0's row
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    r.part_shift[w] = c2(red[0], red[1]);
    r.part_fbt[w] = c2(red[2], red[3]);
  }
}

// ======================================================================================
// vhs GEMM epilogue (propagation.py:265-271): rows (w, re/im) of xt . chol give
// V = i sqrt(dt) xt . chol = sqrt(dt) (-(xt_i.L) + i (xt_r.L)); write the Taylor A operand
// [Vr | Vi] (hi and lo) for each walker of the chunk. Columns are (p, q) with q padded to nq.
// ======================================================================================

struct EpiVHS {
  struct Params {
    uint16_t* v_hi;
    uint16_t* v_lo;
    int n, nq, rows, bf16, want_lo;
    float sqdt;
    int sym;  // split GEMM only: columns are the packed (p, q) pairs of sym_decode
    int mr;   // rows per walker of the V operand (128, or 256 for norb > 128)
  };
  static constexpr int kSmemBytes = 0;
  __device__ static void run(const Params& p, int m0, int n0, int bn, uint32_t tmem, int q, int lane,
                             unsigned char*, bool) {
    const int R = m0 + q * 32 + lane, wl = R >> 1, c = R & 1;
    const bool bf = p.bf16 != 0;
    const float scale = c == 0 ? p.sqdt : -p.sqdt;
#pragma unroll 1
    for (int c0 = 0; c0 < bn; c0 += 16) {
      float v[16];
      ptx::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + c0, v);
      ptx::tmem_ld_wait();
      const int col = n0 + c0, pr = col / p.nq, q0 = col % p.nq;
      if (R >= p.rows || pr >= p.n) continue;
      const size_t off = ((size_t)wl * p.mr + pr) * (2 * p.nq) + (c == 0 ? p.nq : 0) + q0;
      uint32_t hw[8], lw[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        uint16_t h0, l0, h1, l1;
        split16(v[2 * j] * scale, bf, h0, l0);
        split16(v[2 * j + 1] * scale, bf, h1, l1);
        hw[j] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        lw[j] = (uint32_t)l0 | ((uint32_t)l1 << 16);
      }
      uint4* dh = reinterpret_cast<uint4*>(p.v_hi + off);
      dh[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
      dh[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
      if (p.want_lo) {
        uint4* dl = reinterpret_cast<uint4*>(p.v_lo + off);
        dl[0] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        dl[1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
      }
    }
  }
};

// The same scatter for the persistent split GEMM: row R of the chunk, 128 columns from col0.
struct EpiVHSSplit {
  using Params = EpiVHS::Params;
  static constexpr bool kWarpStore = true;
  // Rows R0 + lane (walker R / 2, real (even R) or imaginary part) and 128 columns col0.. of
  // vhs, i.e. (orbital pr, q) pairs, into the Taylor operand V = [Vr | Vi] per walker. Per 32
  // columns each lane converts its row to fp16 hi / lo (two values per conversion
  // instruction) and stages one plane at a time in shared memory (80-byte rows), then four
  // lanes store each row's 64 contiguous bytes: a warp's stores cover 8 rows x 64 B instead of
  // 32 separate 16-byte pieces. A 32-column group never crosses a row run (runs are multiples
  // of 32 long and start at multiples of 32), so (pr, q0) is decoded once per tile and then
  // advanced.
  __device__ __forceinline__ static void store_warp(const Params& p, int R0, int lane, int col0, const float* v, int,
                                                    unsigned char* stage) {
    const int R = R0 + lane;
    const bool bf = p.bf16 != 0;
    const float scale = (R & 1) == 0 ? p.sqdt : -p.sqdt;
    int pr, q0;
    if (p.sym)
      sym_decode(p.n, p.nq, col0, pr, q0);
    else {
      pr = col0 / p.nq;
      q0 = col0 % p.nq;
    }
#pragma unroll
    for (int c32 = 0; c32 < 128; c32 += 32) {
      if (pr >= p.n) break;  // warp-uniform
      uint32_t hw[16], lw[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float a = v[c32 + 2 * j] * scale, b = v[c32 + 2 * j + 1] * scale;
        if (bf) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
          const float2 hf = __bfloat1622float2(h);
          const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
          hw[j] = *reinterpret_cast<const uint32_t*>(&h);
          lw[j] = *reinterpret_cast<const uint32_t*>(&l);
        } else {
          const __half2 h = __floats2half2_rn(a, b);
          const float2 hf = __half22float2(h);
          const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
          hw[j] = *reinterpret_cast<const uint32_t*>(&h);
          lw[j] = *reinterpret_cast<const uint32_t*>(&l);
        }
      }
#pragma unroll
      for (int plane = 0; plane < 2; ++plane) {
        if (plane == 1 && !p.want_lo) break;
        const uint32_t* src = plane ? lw : hw;
        uint4* srow = reinterpret_cast<uint4*>(stage + lane * kSplitStageRow);
#pragma unroll
        for (int u = 0; u < 4; ++u) srow[u] = make_uint4(src[4 * u], src[4 * u + 1], src[4 * u + 2], src[4 * u + 3]);
        __syncwarp();
        uint16_t* base = plane ? p.v_lo : p.v_hi;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = lane + 32 * u, row = t >> 2, part = t & 3, Rr = R0 + row;
          if (Rr < p.rows) {
            const int wl = Rr >> 1, c = Rr & 1;
            const size_t off = ((size_t)wl * p.mr + pr) * (2 * p.nq) + (c == 0 ? p.nq : 0) + q0 + part * 8;
            *reinterpret_cast<uint4*>(base + off) =
                *reinterpret_cast<const uint4*>(stage + row * kSplitStageRow + part * 16);
          }
        }
        __syncwarp();
      }
      // next 32 columns: same row run, or the start of the next row's run
      q0 += 32;
      if (q0 >= p.nq) {
        ++pr;
        q0 = p.sym ? 32 * (pr >> 5) : 0;
      }
    }
  }
};

// vhs B operand for symmetric vectors: chol [nchol][n*n] -> lop[c][g] for the packed columns
// c = (p, q) of sym_decode, 32 x 32 tiles through shared memory
__global__ void k_prep_lop_sym(const double* __restrict__ chol, int nchol, int n, int nq, int total, int ldg,
                               int bf16, uint16_t* __restrict__ hi, uint16_t* __restrict__ lo) {
  __shared__ float tile[32][33];
  const int c0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  int pp = n, qq = 0;
  if (c0 + tx < total) sym_decode(n, nq, c0 + tx, pp, qq);
  for (int r = ty; r < 32; r += 8) {
    const int g = g0 + r;
    tile[r][tx] = (g < nchol && pp < n && qq < n) ? (float)chol[(size_t)g * n * n + (size_t)pp * n + qq] : 0.f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int c = c0 + r, g = g0 + tx;
    if (c < total && g < nchol) {
      uint16_t h, l;
      split16(tile[tx][r], bf16 != 0, h, l);
      hi[(size_t)c * ldg + g] = h;
      lo[(size_t)c * ldg + g] = l;
    }
  }
}

// ======================================================================================
// QR of the FP32 walker slabs (propagation.py:251-253 -> linalg_utils.py:51-65): the
// LAPACK Householder factorisation (zgeqr2) and explicit Q (zung2r), one warp per slab with
// the slab in shared memory (row stride k | 1: conflict-free column walks) and only
// warp-level synchronisation. Column sums (the reflector applied to the trailing columns)
// are owned by lanes per column (qr_colsum); the rank-1 updates by lane = row. The squared
// norm below the diagonal is accumulated as a float pair.
// ======================================================================================

constexpr int kQrWarps = 4;

__host__ __device__ constexpr int qr_ld(int k) { return k | 1; }

// y[c] = sum_{r >= j} conj(A[r][c]) A[r][j] for c in (j, k) by one warp: lpc = the largest
// power of two with lpc * (k - j - 1) <= 32 lanes per column, each summing every lpc-th row,
// combined by shuffles (the rows of a column are the serial part otherwise).
__device__ __forceinline__ void qr_colsum(const float2* A, int ld, int m, int k, int j, int lane, float2* y) {
  const int nc = k - j - 1;
  if (nc <= 0) return;
  int lpc = 1;
  while (lpc * 2 * nc <= 32) lpc *= 2;
  const int col = j + 1 + lane / lpc, part = lane % lpc;
  const bool active = lane < lpc * nc;
  float yx = 0.f, yy = 0.f;
  if (active) {
#pragma unroll 4
    for (int r = j + part; r < m; r += lpc) {
      const float2 pr = cmulc(A[r * ld + col], A[r * ld + j]);
      yx += pr.x;
      yy += pr.y;
    }
  }
  for (int off = 1; off < lpc; off <<= 1) {  // lpc is warp-uniform
    yx += __shfl_xor_sync(0xffffffffu, yx, off);
    yy += __shfl_xor_sync(0xffffffffu, yy, off);
  }
  if (active && part == 0) y[col] = make_float2(yx, yy);
}

__global__ void __launch_bounds__(32 * kQrWarps) k_qr_warp(int nw, int m, int k, float2* __restrict__ wbase) {
  extern __shared__ __align__(16) unsigned char qsm_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wlk = blockIdx.x * kQrWarps + warp;
  if (wlk >= nw) return;  // warp-level work only: no block barrier below
  const int ld = qr_ld(k);
  float2* A = reinterpret_cast<float2*>(qsm_raw) + (size_t)warp * ((size_t)m * ld + 64);
  float2* y = A + (size_t)m * ld;
  float2* tau = y + 32;
  float2* W = wbase + (size_t)wlk * m * k;
  for (int i = lane; i < m * k; i += 32) {
    const int r = i / k;
    A[r * ld + (i - r * k)] = W[i];
  }
  __syncwarp();
  // ---- factorisation
  for (int j = 0; j < k; ++j) {
    // squared norm below the diagonal as an unevaluated float pair (TwoSum per term and per
    // shuffle level): FP64-class accuracy without the FP64 pipe
    float xh = 0.f, xl = 0.f;
    for (int r = j + 1 + lane; r < m; r += 32) {
      const float a2 = cabs2(A[r * ld + j]), sum = xh + a2, bb = sum - xh;
      xl += (xh - (sum - bb)) + (a2 - bb);
      xh = sum;
    }
    for (int off = 16; off > 0; off >>= 1) {
      const float o = __shfl_xor_sync(0xffffffffu, xh, off), ol = __shfl_xor_sync(0xffffffffu, xl, off);
      const float sum = xh + o, bb = sum - xh;
      xl += ol + ((xh - (sum - bb)) + (o - bb));
      xh = sum;
    }
    const float2 alpha = A[j * ld + j];
    const float xn = xh + xl;
    float2 t, scl, beta;
    if (xn == 0.f && alpha.y == 0.f) {
      t = make_float2(0.f, 0.f);
      beta = alpha;
      scl = make_float2(1.f, 0.f);
    } else {
      const float nrm = sqrtf(alpha.x * alpha.x + alpha.y * alpha.y + xn);
      const float b = (alpha.x >= 0.f) ? -nrm : nrm;
      t = make_float2((b - alpha.x) / b, -alpha.y / b);
      scl = cdiv(make_float2(1.f, 0.f), csub(alpha, make_float2(b, 0.f)));
      beta = make_float2(b, 0.f);
    }
    __syncwarp();
    for (int r = j + 1 + lane; r < m; r += 32) A[r * ld + j] = cmul(A[r * ld + j], scl);
    if (lane == 0) {
      A[j * ld + j] = make_float2(1.f, 0.f);
      tau[j] = t;
    }
    __syncwarp();
    qr_colsum(A, ld, m, k, j, lane, y);
    __syncwarp();
    const float2 ct = make_float2(t.x, -t.y);
    for (int r = j + lane; r < m; r += 32) {
      const float2 v = A[r * ld + j];
#pragma unroll 4
      for (int cc = j + 1; cc < k; ++cc)
        A[r * ld + cc] = csub(A[r * ld + cc], cmul(ct, cmul(v, y[cc])));
    }
    __syncwarp();
    if (lane == 0) A[j * ld + j] = beta;
    __syncwarp();
  }
  // ---- form Q (zung2r): columns from last to first
  for (int j = k - 1; j >= 0; --j) {
    const float2 t = tau[j];
    if (j < k - 1) {
      if (lane == 0) A[j * ld + j] = make_float2(1.f, 0.f);
      __syncwarp();
      qr_colsum(A, ld, m, k, j, lane, y);
      __syncwarp();
      for (int r = j + lane; r < m; r += 32) {
        const float2 v = A[r * ld + j];
#pragma unroll 4
        for (int cc = j + 1; cc < k; ++cc)
          A[r * ld + cc] = csub(A[r * ld + cc], cmul(t, cmul(v, y[cc])));
      }
      __syncwarp();
    }
    const float2 mt = make_float2(-t.x, -t.y);
    for (int r = j + 1 + lane; r < m; r += 32) A[r * ld + j] = cmul(mt, A[r * ld + j]);
    if (lane == 0) A[j * ld + j] = make_float2(1.f - t.x, -t.y);
    for (int r = lane; r < j; r += 32) A[r * ld + j] = make_float2(0.f, 0.f);
    __syncwarp();
  }
  for (int i = lane; i < m * k; i += 32) {
    const int r = i / k;
    W[i] = A[r * ld + (i - r * k)];
  }
}

// ======================================================================================
// exp_h1 products: D[p][(w, 2k + c)] = ((E - I) X)[p][k].c for the walker (X = W) or the
// Taylor sum (X = acc). First product: W1 = W + D into the Taylor B operand (hi/lo);
// last product: W_new = acc + D back into the FP32 walker slab. propagation.py:73, 91.
// ======================================================================================

struct EpiExp {
  struct Params {
    float* w;                 // walker slab [nw][n][o] complex64
    const uint16_t* acc_hi;   // last product: Taylor sum operand [nw*R][nk]
    const uint16_t* acc_lo;
    uint16_t* t0_hi;          // first product: Taylor B operand [nw][NT][2nq]
    uint16_t* t0_lo;
    int n, o, R, nk, nq, NT, nw, bf16, last;
  };
  static constexpr int kSmemBytes = 0;
  // Walker-major: R (a multiple of 16) columns per walker, so each walker is R/16 whole
  // TMEM chunks; thread p handles orbital row p of every walker of the tile.
  __device__ static void run(const Params& p, int m0, int n0, int bn, uint32_t tmem, int q, int lane,
                             unsigned char*, bool) {
    const int pr = m0 + q * 32 + lane;
    const bool bf = p.bf16 != 0;
    const int wpt = bn / p.R, w0 = n0 / p.R;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
#pragma unroll 1
    for (int wl = 0; wl < wpt; ++wl) {
      float v[64];
#pragma unroll
      for (int c0 = 0; c0 < 64; c0 += 16) {
        if (c0 < p.R) {
          float t[16];
          ptx::tmem_ld16(tmem + lane_off + (uint32_t)(wl * p.R + c0), t);
#pragma unroll
          for (int j = 0; j < 16; ++j) v[c0 + j] = t[j];
        }
      }
      ptx::tmem_ld_wait();
      const int w = w0 + wl;
      if (pr >= p.n || w >= p.nw) continue;
      float2* wrow = reinterpret_cast<float2*>(p.w) + ((size_t)w * p.n + pr) * p.o;
      // loads are issued 8 orbitals at a time before the stores of those orbitals (the stores
      // may alias the loads for the compiler, which would otherwise wait one load latency per k)
      if (p.last) {
        const size_t ab = (size_t)w * p.R * p.nk + pr;
#pragma unroll
        for (int k0 = 0; k0 < 32; k0 += 8) {
          if (k0 < p.o) {
            uint16_t ah[16], al[16];
#pragma unroll
            for (int r = 0; r < 16; ++r)
              if (2 * k0 + r < 2 * p.o) {
                ah[r] = p.acc_hi[ab + (size_t)(2 * k0 + r) * p.nk];
                al[r] = p.acc_lo[ab + (size_t)(2 * k0 + r) * p.nk];
              }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
              const int k = k0 + kk;
              if (k < p.o) {
                const float ar = h2f(ah[2 * kk], bf) + h2f(al[2 * kk], bf);
                const float ai = h2f(ah[2 * kk + 1], bf) + h2f(al[2 * kk + 1], bf);
                wrow[k] = make_float2(ar + v[2 * k], ai + v[2 * k + 1]);
              }
            }
          }
        }
      } else {
        const size_t base = (size_t)w * p.NT * 2 * p.nq;
#pragma unroll
        for (int k0 = 0; k0 < 32; k0 += 8) {
          if (k0 < p.o) {
            float2 xw[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
              if (k0 + kk < p.o) xw[kk] = wrow[k0 + kk];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
              const int k = k0 + kk;
              if (k < p.o) {
                const float wr = xw[kk].x + v[2 * k], wi = xw[kk].y + v[2 * k + 1];
                uint16_t hr, lr, hi_, li, hn, ln;
                split16(wr, bf, hr, lr);
                split16(wi, bf, hi_, li);
                split16(-wi, bf, hn, ln);
                const size_t r0 = base + (size_t)(2 * k) * 2 * p.nq, r1 = r0 + 2 * p.nq;
                // row 2k: [Tr | -Ti], row 2k+1: [Ti | Tr]
                p.t0_hi[r0 + pr] = hr;
                p.t0_lo[r0 + pr] = lr;
                p.t0_hi[r0 + p.nq + pr] = hn;
                p.t0_lo[r0 + p.nq + pr] = ln;
                p.t0_hi[r1 + pr] = hi_;
                p.t0_lo[r1 + pr] = li;
                p.t0_hi[r1 + p.nq + pr] = hr;
                p.t0_lo[r1 + p.nq + pr] = lr;
              }
            }
          }
        }
      }
    }
  }
};

// ======================================================================================
// Exchange epilogue of the split GEMM, on the transposed product D = G U (U symmetric):
// D[(w, re/im)][(i,q)] = Z_w[(i,q)] = sum_(k,p) U[(i,q),(k,p)] G_w[k,p] with
// U[(i,q),(k,p)] = sum_g rot_chol_g[i,p] rot_chol_g[k,q], so that the exchange sum of
// wavefunctions.py:539 (and 737-738), exc = sum_g sum_ik f_g[i,k] f_g[k,i] with
// f_g = rot_chol_g G^T, equals sum_(i,q) Z_w[(i,q)] G_w[i,q]. A thread holds row (w, part)
// of D over 128 consecutive (i,q): it reads the same 128 entries of G_w's re and im rows
// (contiguous 16-byte loads, hi + lo) and forms Z_part . G_re and Z_part . G_im; the
// neighbouring lane (the other part of the same walker) completes the complex product. The
// walker's partial of exc for these 128 columns and this K range goes, scaled, to slot
// ks * n128 + col0 / 128 of its row of partials: exc is linear in Z, so K-split partials
// need no separate reduction, and the final energy kernel sums the slots in a fixed order.
// ======================================================================================

struct EpiExcSplit {
  static constexpr bool kWarpStore = true;
  struct Params {
    const uint16_t* g_hi;  // [2 nw][ldk] Green operand (rows 2w, 2w+1 = re, im)
    const uint16_t* g_lo;
    const float* g_inv;    // [nw]
    float u_inv;
    int kb, ldk, nw, bf16;
    int n128, slots;       // 128-column groups of kb; partial slots per walker (K splits * n128)
    double2* exc_part;     // [nw][slots]
  };
  __device__ __forceinline__ static void store_warp(const Params& p, int row0, int lane, int col0, const float* v,
                                                    int ks, unsigned char*) {
    if (row0 >= 2 * p.nw || col0 >= p.kb) return;  // warp-uniform: padding rows / columns of the last tiles
    const int R = row0 + lane, w = R >> 1;
    const bool rv = R < 2 * p.nw, bf = p.bf16 != 0;
    // Z_part . G_re and Z_part . G_im: 8-column chunk sums added with Kahan compensation
    float a_re = 0.f, a_im = 0.f, k_re = 0.f, k_im = 0.f;
    if (rv) {
      const uint16_t* gr_h = p.g_hi + (size_t)(2 * w) * p.ldk;
      const uint16_t* gr_l = p.g_lo + (size_t)(2 * w) * p.ldk;
      const uint16_t* gi_h = gr_h + p.ldk;
      const uint16_t* gi_l = gr_l + p.ldk;
#pragma unroll
      for (int c8 = 0; c8 < 128; c8 += 8) {
        const int c = col0 + c8;
        if (c < p.kb) {  // 8 columns at a time (c + 8 <= ldk: rows padded to multiples of 8)
          const uint4 rh = *reinterpret_cast<const uint4*>(gr_h + c), rl = *reinterpret_cast<const uint4*>(gr_l + c);
          const uint4 ih = *reinterpret_cast<const uint4*>(gi_h + c), il = *reinterpret_cast<const uint4*>(gi_l + c);
          const uint32_t rhw[4] = {rh.x, rh.y, rh.z, rh.w}, rlw[4] = {rl.x, rl.y, rl.z, rl.w};
          const uint32_t ihw[4] = {ih.x, ih.y, ih.z, ih.w}, ilw[4] = {il.x, il.y, il.z, il.w};
          float s_re = 0.f, s_im = 0.f;
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const int sh = 16 * (e & 1);
            const float gre = h2f((uint16_t)(rhw[e >> 1] >> sh), bf) + h2f((uint16_t)(rlw[e >> 1] >> sh), bf);
            const float gim = h2f((uint16_t)(ihw[e >> 1] >> sh), bf) + h2f((uint16_t)(ilw[e >> 1] >> sh), bf);
            if (c + e < p.kb) {  // the row's padding columns are never written
              s_re = fmaf(v[c8 + e], gre, s_re);
              s_im = fmaf(v[c8 + e], gim, s_im);
            }
          }
          const float y_re = s_re - k_re, t_re = a_re + y_re;
          k_re = (t_re - a_re) - y_re;
          a_re = t_re;
          const float y_im = s_im - k_im, t_im = a_im + y_im;
          k_im = (t_im - a_im) - y_im;
          a_im = t_im;
        }
      }
      a_re -= k_re;
      a_im -= k_im;
    }
    // lane 2k: Z_re . G (part 0), lane 2k + 1: Z_im . G (part 1)
    const float o_re = __shfl_xor_sync(0xffffffffu, a_re, 1), o_im = __shfl_xor_sync(0xffffffffu, a_im, 1);
    if (rv && (R & 1) == 0) {
      const double sc = (double)p.g_inv[w] * (double)p.g_inv[w] * (double)p.u_inv;
      const double ex = (double)a_re - (double)o_im, ey = (double)a_im + (double)o_re;
      p.exc_part[(size_t)w * p.slots + ks * p.n128 + col0 / 128] = c2(ex * sc, ey * sc);
    }
  }
};

}  // namespace afq

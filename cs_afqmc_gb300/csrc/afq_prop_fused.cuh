// Fused walker propagation of the mixed path (propagation.py:67-92, _apply_trotprop_det):
// per walker slab W,
//   W1 = exp_h1 W                      (exp_h1 = I + (E - I))
//   acc = sum_{m=0..nterms-1} V^m W1 / m!   (V = vhs of the walker, Taylor by repeated V T)
//   W' = exp_h1 acc
// in one persistent kernel, all products on tcgen05 with FP32 accumulators in TMEM.
//
// Operands (16-bit hi/lo planes):
//   A (in tensor memory, row p in lane p, K packed two per column): E - I [128][nq] (loaded
//     once), Vr and Vi [128][nq] of the current walker. Keeping A in TMEM leaves the tensor
//     core only the small B operand to read from shared memory per instruction.
//   B (shared memory, K-major, 128-byte swizzle): [2 NT rows][nq] written by the epilogue
//     threads, row 2k + c = part c (re / im) of column k of the current term, K = orbital q.
// The complex product V T is two real products, D0 = Vr B and D1 = Vi B, combined in the
// epilogue: Re(VT) = D0[2k] - D1[2k+1], Im(VT) = D0[2k+1] + D1[2k]; (E - I) T is D0 alone.
//
// Every product is one MMA chain with N = NT (all of the walker's B rows): a tcgen05.mma of
// M = 128, K = 16 costs the same ~60 cycles for any N <= 128 (measured on GB300), so the
// instruction count, not N, sets the time. The epilogue runs on 4 NT / 16 warps: warp
// (part, quadrant) reads TMEM lanes 32 quadrant.. (thread = orbital row p) and owns the 16
// B rows 16 part.. (8 orbitals). One control thread issues the TMA loads and every MMA. The
// next walker's V is brought into shared memory by TMA while the current walker is
// propagated; four loader warps move it into TMEM once the current walker's last Taylor
// products have completed, which overlaps the final exp_h1 product and the next walker's
// first one.
//
// Those two exp_h1 products are independent and share the A operand (E - I), so with a
// Taylor series (nterms > 1) they are one MMA chain of N = 2 NT: B rows 0 .. NT-1 hold this
// walker's Taylor sum, rows NT .. 2 NT-1 the next walker's slab, and the products land in D0
// and D1. Each output element is the same K sum as in two separate chains; per walker this
// saves one exp_h1 chain and one epilogue round trip.
//
// Precision: every product accumulates its correction terms (lo * hi, hi * lo) first, then
// hi * hi, in one FP32 accumulator over K <= 128 (two K tiles); the Taylor sum, W1 and W'
// are formed in FP32 registers. The first `split` Taylor products use V_lo and T_lo; the
// exp_h1 products use E_lo (e_lo) and W_lo / acc_lo (w_lo).
//
// Every wait is bounded (ptx::kWaitLimit polls): on a timeout the CTA sets bit 2 of
// *status, stops, waits (bounded) for its own copies and MMAs in flight and frees TMEM.
#pragma once
#include "afq_mixed_kernels.cuh"

namespace afq {

struct PropDev {
  int n, o, nq, NT, nterms, split, bf16, nwc;
  int e_lo, w_lo;   // exp_h1 products: E_lo * B_hi and E_hi * B_lo terms
  int sym;          // V is symmetric and stored only for q >= 32 floor(p / 32) (packed vhs)
  float2* w;        // walker slab of the chunk's first walker, [nwc][n][o] complex64
};

__device__ __forceinline__ void sts16(uint32_t addr, uint16_t v) {
  asm volatile("st.shared.u16 [%0], %1;" ::"r"(addr), "h"(v) : "memory");
}

constexpr int kPropMaxChains = 4;     // NT <= 64: at most 32 orbitals per slab
constexpr uint32_t kPropTile = 16384;  // one 128-row x 64-column 16-bit operand tile

__host__ __device__ constexpr size_t prop_fused_smem(int nq, int NT) {
  return 1024 + (size_t)(nq / 64) * kPropTile * 4  // V staging: hi / lo, Vr and Vi tiles
         + (size_t)(nq / 64) * 2 * NT * 128 * 2   // B hi / lo (2 NT rows: the merged exp_h1 chain)
         + 256;                                   // barriers, TMEM address
}

// TMEM columns (kw = nq / 2 columns per 128 x nq operand): E_hi, E_lo, Vr_hi, Vi_hi, Vr_lo,
// Vi_lo at 0, kw, .., 5 kw; the accumulators D0, D1 at 6 kw and 6 kw + NT
__host__ __device__ constexpr int prop_tmem_cols(int nq, int NT) { return 3 * nq + 2 * NT; }

template <int NP>  // NT = 16 NP B rows
__global__ void __launch_bounds__(128 * NP + 160, 1)
    k_prop_fused(const __grid_constant__ CUtensorMap mv_hi, const __grid_constant__ CUtensorMap mv_lo,
                 const uint16_t* __restrict__ e_hi, const uint16_t* __restrict__ e_lo, int nk,
                 const PropDev pd, int* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int KQ = pd.nq / 64, kw = pd.nq / 2;
  const uint32_t BT = (uint32_t)pd.NT * 2 * 128;  // bytes per B K tile (2 NT rows)
  unsigned char* Sv = smem;                   // staging: [plane][part][kt] tiles
  unsigned char* Bh = Sv + 4 * KQ * kPropTile;
  unsigned char* Bl = Bh + KQ * BT;
  uint64_t* bars = reinterpret_cast<uint64_t*>(Bl + KQ * BT);
  uint64_t* v_bar = bars;          // the next walker's V landed in the staging tiles
  uint64_t* vready = bars + 1;     // V moved into TMEM (staging free)
  uint64_t* vfree = bars + 2;      // the walker's last Taylor products completed (V in TMEM free)
  uint64_t* eready = bars + 3;     // E - I in TMEM
  uint64_t* ready = bars + 4;      // B rows written and the accumulators read
  uint64_t* done = bars + 5;       // the step's MMAs completed
  uint64_t* fin = bars + 6;        // every MMA issued has completed (teardown)
  uint64_t* vlofree = bars + 7;    // the walker's last product with V_lo completed (V_lo in TMEM free)
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 8);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int NT = 16 * NP;
  constexpr int kLoad = 4 * NP, kCtrl = 4 * NP + 4;  // loader warps, control warp
  const bool bf = pd.bf16 != 0;
  const bool need_v = pd.nterms > 1;
  const bool merge = need_v;  // final exp_h1 chain of a walker merged with the next walker's first
  const bool v_lo = pd.split > 0;
  const int nsteps = pd.nterms + 1;  // exp_h1, nterms - 1 Taylor products, exp_h1
  // V_lo is last used by Taylor product `split`: when that is not the last product, the next
  // walker's V_lo is moved into TMEM as soon as it completes, before the rest of V
  const bool early_lo = v_lo && pd.split < nsteps - 2;

  if (tid == 0) {
    ptx::mbar_init(v_bar, 1);
    ptx::mbar_init(vready, 4);
    ptx::mbar_init(vfree, 1);
    ptx::mbar_init(eready, 4);
    ptx::mbar_init(ready, 4 * NP);  // one arrival per epilogue warp
    ptx::mbar_init(done, 1);
    ptx::mbar_init(fin, 1);
    ptx::mbar_init(vlofree, 1);
    ptx::fence_mbar_init();
  }
  if (warp == kCtrl) {
    ptx::tmem_alloc(tmem_holder, 512);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t c_eh = 0, c_el = kw, c_vh = 2 * kw, c_vl = 4 * kw, c_d = 6 * kw;
  bool ok = true;

  if (warp == kCtrl) {
    if (lane == 0) {
      const uint32_t sBh = ptx::smem_u32(Bh), sBl = ptx::smem_u32(Bl);
      const uint32_t idesc1 = ptx::idesc_f16(128, NT, bf ? 1 : 0), idesc2 = ptx::idesc_f16(128, 2 * NT, bf ? 1 : 0);
      uint32_t idesc = idesc1;
      const uint32_t vbytes = 2 * KQ * kPropTile * (v_lo ? 2 : 1);
      auto load_v = [&](int wl) {
        ptx::mbar_expect_tx(v_bar, vbytes);
        for (int kt = 0; kt < 2 * KQ; ++kt) {  // [Vr | Vi] K tiles of the hi, then the lo plane
          ptx::tma_load_2d(Sv + kt * kPropTile, &mv_hi, v_bar, kt * 64, wl * 128);
          if (v_lo) ptx::tma_load_2d(Sv + (2 * KQ + kt) * kPropTile, &mv_lo, v_bar, kt * 64, wl * 128);
        }
      };
      // D (+)= A[tmem columns a ..] B[b ..] over K = nq
      auto run = [&](uint32_t d, uint32_t a, uint32_t b, bool& first) {
        for (int kt = 0; kt < KQ; ++kt)
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            ptx::mma_f16_ts(d, a + (uint32_t)(32 * kt + 8 * kk), ptx::desc_kmajor_sw128(b + kt * BT + kk * 32),
                            idesc, first ? 0u : 1u);
            first = false;
          }
      };
      ptx::prefetch_tmap(&mv_hi);
      int v_issued = 0, v_moved = 0;
      if (need_v && blockIdx.x < pd.nwc) {
        load_v(blockIdx.x);
        ++v_issued;
      }
      if (!ptx::mbar_wait(eready, 0)) ok = false;
      uint32_t sc = 0;  // steps issued so far (phase of ready / done)
      int it = 0;       // walkers started
      for (int wl = blockIdx.x; wl < pd.nwc && ok; wl += gridDim.x, ++it) {
        const bool has_next = wl + (int)gridDim.x < pd.nwc;
        // after the first walker, a walker's first exp_h1 product ran in the previous one's last chain
        for (int st = (merge && it > 0) ? 1 : 0; st < nsteps && ok; ++st, ++sc) {
          const bool expo = st == 0 || st == nsteps - 1;
          idesc = (merge && has_next && st == nsteps - 1) ? idesc2 : idesc1;
          if (!ptx::mbar_wait(ready, sc & 1)) {
            ok = false;
            break;
          }
          if (!expo && st == 1) {  // first Taylor product: this walker's V in TMEM
            if (!ptx::mbar_wait(vready, v_moved & 1)) {
              ok = false;
              break;
            }
            ++v_moved;
            if (wl + (int)gridDim.x < pd.nwc) {  // the staging tiles are free: next walker's V
              load_v(wl + gridDim.x);
              ++v_issued;
            }
          }
          ptx::tc_fence_after();
          const uint32_t d0 = tmem + c_d;
          if (expo) {
            bool first = true;
            if (pd.e_lo) run(d0, tmem + c_el, sBh, first);
            if (pd.w_lo) run(d0, tmem + c_eh, sBl, first);
            run(d0, tmem + c_eh, sBh, first);
          } else {
            const bool lo = st <= pd.split;
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {  // Vr -> D0, Vi -> D1
              const uint32_t d = d0 + NT * h, ah = tmem + c_vh + h * kw, al = tmem + c_vl + h * kw;
              bool f = true;
              if (lo) {
                run(d, al, sBh, f);
                run(d, ah, sBl, f);
              }
              run(d, ah, sBh, f);
            }
          }
          ptx::mma_commit(done);
          // the walker's last Taylor products are issued: V in TMEM is free once they complete
          if (ok && need_v && st == nsteps - 2) ptx::mma_commit(vfree);
          if (ok && early_lo && st == pd.split) ptx::mma_commit(vlofree);
        }
      }
      ptx::mma_commit(fin);
      if (!ptx::mbar_wait(fin, 0)) ok = false;
      // never leave a copy in flight: a load whose walker was not reached
      if (v_issued > v_moved && !ptx::mbar_wait(v_bar, (v_issued - 1) & 1)) ok = false;
    }
  } else if (warp >= kLoad) {
    // ---- loader warps: E - I once, then every walker's V, staging tiles -> TMEM
    const int q = warp & 3, p = 32 * q + lane;
    const uint32_t lane_off = (uint32_t)(32 * q) << 16;
    {
      const uint32_t* eh32 = reinterpret_cast<const uint32_t*>(e_hi) + (size_t)p * (nk / 2);
      const uint32_t* el32 = reinterpret_cast<const uint32_t*>(e_lo) + (size_t)p * (nk / 2);
      for (int plane = 0; plane < (pd.e_lo ? 2 : 1); ++plane) {
        const uint32_t* src = plane ? el32 : eh32;
        for (int j0 = 0; j0 < kw; j0 += 16) {
          uint32_t v[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = (2 * (j0 + j) < nk) ? src[j0 + j] : 0u;
          ptx::tmem_st16u(tmem + lane_off + (plane ? c_el : c_eh) + j0, v);
        }
      }
      ptx::tmem_st_wait();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(eready);
    }
    // with symmetric V the staged row p holds only q >= 32 quadrant: the columns below come
    // from row q, column p (for a fixed q the warp reads 32 consecutive elements of row q)
    const int q_lo = pd.sym ? 32 * q : 0;
    const bool pv = p < pd.n;
    auto copy_plane = [&](int plane) {
      for (int t = 0; t < 2 * KQ; ++t) {  // tiles: Vr kt = 0..KQ-1, then Vi
        const unsigned char* tile = Sv + (plane * 2 * KQ + t) * kPropTile + p * 128;
        const uint32_t col = (plane ? c_vl : c_vh) + (t / KQ) * kw + (t % KQ) * 32;
        const int k_tile = (t % KQ) * 64;
        // column p of the part's staged tiles (K tile p / 64 of the same part and plane)
        const unsigned char* ctile = Sv + (plane * 2 * KQ + (t / KQ) * KQ + (p >> 6)) * kPropTile;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          uint32_t v[16];
#pragma unroll
          for (int c = 0; c < 4; ++c) {  // 16-byte chunks 4 half + c of the row (swizzled)
            const int k0 = k_tile + 8 * (4 * half + c);
            if (k0 >= q_lo) {  // warp-uniform: q_lo and k0 are multiples of 8 and 32
              const uint4 x = *reinterpret_cast<const uint4*>(tile + (((4 * half + c) ^ (p & 7)) << 4));
              v[4 * c] = x.x;
              v[4 * c + 1] = x.y;
              v[4 * c + 2] = x.z;
              v[4 * c + 3] = x.w;
            } else {
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                uint32_t wd = 0;
                if (pv) {
#pragma unroll
                  for (int e = 0; e < 2; ++e) {
                    const int qq = k0 + 2 * j + e;  // row qq < 32 quadrant <= p
                    const uint16_t x = *reinterpret_cast<const uint16_t*>(
                        ctile + qq * 128 + (((((p & 63) >> 3) ^ (qq & 7))) << 4) + ((p & 7) << 1));
                    wd |= (uint32_t)x << (16 * e);
                  }
                }
                v[4 * c + j] = wd;
              }
            }
          }
          ptx::tmem_st16u(tmem + lane_off + col + 16 * half, v);
        }
      }
    };
    int it = 0;
    for (int wl = blockIdx.x; need_v && wl < pd.nwc && ok; wl += gridDim.x, ++it) {
      bool w_ok = ptx::mbar_wait(v_bar, it & 1);
      if (early_lo) {  // V_lo first, once the previous walker's last split product completed
        if (it > 0) w_ok = w_ok && ptx::mbar_wait(vlofree, (it - 1) & 1);
        if (!__all_sync(0xffffffffu, w_ok)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        copy_plane(1);
      }
      if (it > 0) w_ok = w_ok && ptx::mbar_wait(vfree, (it - 1) & 1);
      if (!__all_sync(0xffffffffu, w_ok)) {
        ok = false;
        break;
      }
      ptx::tc_fence_after();
      copy_plane(0);
      if (v_lo && !early_lo) copy_plane(1);
      ptx::tmem_st_wait();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(vready);
    }
  } else {
    const int g = warp >> 2, q = warp & 3;  // 16-row part of the B operand, lane quadrant
    const int p = 32 * q + lane;
    const bool prow = p < pd.n, pk = p < pd.nq;  // orbital row; K index inside the B tiles
    const int kt_p = p >> 6, kc_p = p & 63;
    const int k0 = 8 * g;  // first orbital of the part
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16) + c_d + (uint32_t)(16 * g);
    const float2* wbase = pd.w;
    // write val[0..15] (rows 16g + r, K = p) as the part's B rows; rows of orbitals >= o
    // and K indices >= n are zero
    // byte offsets of rows 16g + r (r < 8; r + 8 is 1024 bytes further) at K = p inside the
    // swizzled B tile, as 32-bit shared-memory addresses
    const uint32_t b_row0 = (uint32_t)(kt_p * BT + 2048 * g) + ((uint32_t)(kc_p & 7) << 1);
    const uint32_t sBh_e = ptx::smem_u32(Bh) + b_row0, sBl_e = ptx::smem_u32(Bl) + b_row0;
    const int c8 = kc_p >> 3;
    // rows0: 0 for this walker's rows, NT for the next walker's rows of the merged exp_h1 chain
    auto put = [&](const float* val, bool lo, int rows0) {
      if (!pk) return;
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const uint32_t off = (uint32_t)(128 * (rows0 + r)) + ((uint32_t)(c8 ^ (r & 7)) << 4);
        const float x = (prow && k0 + (r >> 1) < pd.o) ? val[r] : 0.f;
        uint16_t h, l;
        split16(x, bf, h, l);
        sts16(sBh_e + off, h);
        if (lo) sts16(sBl_e + off, l);
      }
    };
    auto signal = [&]() {  // B rows visible to the tensor core, TMEM reads complete
      ptx::fence_proxy_async();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(ready);
    };
    auto wait_done = [&](uint32_t sc) {
      return __all_sync(0xffffffffu, ptx::mbar_wait(done, sc & 1)) != 0;
    };
    auto load_w = [&](int wl, float* wv) {
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        float2 v = make_float2(0.f, 0.f);
        if (prow && k0 + kk < pd.o) v = wbase[((size_t)wl * pd.n + p) * pd.o + k0 + kk];
        wv[2 * kk] = v.x;
        wv[2 * kk + 1] = v.y;
      }
    };
    uint32_t sc = 0;
    float wv[16], acc[16];
    bool have_w1 = false;  // acc holds W1 of the walker (its first exp_h1 product ran merged)
    if (blockIdx.x < pd.nwc) load_w(blockIdx.x, wv);
    for (int wl = blockIdx.x; wl < pd.nwc && ok; wl += gridDim.x) {
      const int wn = wl + gridDim.x;
      const bool next = merge && wn < pd.nwc;
      if (!have_w1) {
        // ---- W1 = W + (E - I) W
        put(wv, pd.w_lo != 0, 0);
        signal();
        if (!wait_done(sc++)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        float d0[16];
        ptx::tmem_ld16p(lane_base, d0);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j] = wv[j] + d0[j];
        put(acc, pd.nterms > 1 ? pd.split >= 1 : pd.w_lo != 0, 0);
        signal();
      }
      // ---- T_m = V T_{m-1} / m, acc += T_m
      for (int m = 1; m < pd.nterms; ++m) {
        // the next walker's slab rows (B rows of the merged chain), loaded while the last
        // Taylor product runs
        if (next && m + 1 == pd.nterms) load_w(wn, wv);
        if (!wait_done(sc++)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        float d0[16], d1[16];
        ptx::tmem_ld16p(lane_base, d0);
        ptx::tmem_ld16p(lane_base + NT, d1);
        ptx::tmem_ld_wait();
        const float invm = 1.0f / (float)m;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {  // T_m into d0
          const float tr = (d0[2 * kk] - d1[2 * kk + 1]) * invm, ti = (d0[2 * kk + 1] + d1[2 * kk]) * invm;
          d0[2 * kk] = tr;
          d0[2 * kk + 1] = ti;
          acc[2 * kk] += tr;
          acc[2 * kk + 1] += ti;
        }
        if (m + 1 < pd.nterms) {
          put(d0, m + 1 <= pd.split, 0);
        } else {
          put(acc, pd.w_lo != 0, 0);            // operand of the final exp_h1 product
          if (next) put(wv, pd.w_lo != 0, NT);  // and of the next walker's first
        }
        signal();
      }
      if (!ok) break;
      // without the merge: the next walker's slab rows, loaded before this walker's results are stored
      if (!merge && wn < pd.nwc) load_w(wn, wv);
      // ---- W' = acc + (E - I) acc (merged: and the next walker's W1 = W + (E - I) W)
      if (!wait_done(sc++)) {
        ok = false;
        break;
      }
      ptx::tc_fence_after();
      {
        float d0[16];
        ptx::tmem_ld16p(lane_base, d0);
        ptx::tmem_ld_wait();
        if (prow) {
          float2* dst = pd.w + ((size_t)wl * pd.n + p) * pd.o;
#pragma unroll
          for (int kk = 0; kk < 8; ++kk)
            if (k0 + kk < pd.o) dst[k0 + kk] = make_float2(acc[2 * kk] + d0[2 * kk], acc[2 * kk + 1] + d0[2 * kk + 1]);
        }
      }
      have_w1 = next;
      if (next) {
        float d1[16];
        ptx::tmem_ld16p(lane_base + NT, d1);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j] = wv[j] + d1[j];
        put(acc, pd.split >= 1, 0);
        signal();
      }
    }
  }
  if (!ok) atomicOr(status, 2);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == kCtrl) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
}

}  // namespace afq

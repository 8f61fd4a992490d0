// Fused walker propagation for wide slabs (128 < norb <= 256; propagation.py:67-92): the
// same chain as k_prop_fused - W1 = exp_h1 W, acc = sum_m V^m W1 / m!, W' = exp_h1 acc -
// with the orbital dimension in two 128-row M tiles. Operands of that size do not fit in
// tensor memory, so the A tiles (exp_h1 - I, and Vr, Vi of the walker; 16-bit hi / lo planes)
// are streamed from L2 by TMA through a ring of shared-memory stages for every product:
//   per step, for M tile mt (2), part h (1 for exp_h1; Vr, Vi for a Taylor product) and
//   K tile kt (4): A_hi (and A_lo when the step has split terms) -> MMAs into D[mt][h].
// B (shared memory, K-major, 128-byte swizzle): [NT][nq = 256] written by the epilogue warps,
// row 2k + c = part c of column k of the current term, K = orbital q; each epilogue thread
// owns orbital rows p and p + 128 (TMEM lane p of both M tiles' accumulators).
//
// Warp roles: 4 NT / 16 epilogue warps (16-row part of B, TMEM lane quadrant), one producer
// warp (lane 0 issues the TMA loads, running ahead through the ring across steps and
// walkers), one control warp (TMEM allocation; lane 0 issues the MMAs and releases stages).
// Accumulation: per K tile the correction products (lo * hi, hi * lo) precede hi * hi, into
// one FP32 accumulator over K = 256. Every wait is bounded; on a timeout the CTA sets bit 2
// of *status, stops, waits (bounded) for its copies and MMAs in flight and frees TMEM.
#pragma once
#include "afq_prop_fused.cuh"

namespace afq {

constexpr int kWideStages = 3;                  // ring units of (A_hi, A_lo) tiles
constexpr int kWideMR = 256;                    // rows of the per-walker V and exp_h1 operands
constexpr int kWideKQ = 4;                      // K tiles of 64 (nq = 256)

__host__ __device__ constexpr size_t prop_wide_smem(int NT) {
  return 1024 + (size_t)kWideStages * 2 * kPropTile + (size_t)kWideKQ * NT * 128 * 2 + 256;
}

template <int NP>  // NT = 16 NP B rows
__global__ void __launch_bounds__(128 * NP + 64, 1)
    k_prop_wide(const __grid_constant__ CUtensorMap mv_hi, const __grid_constant__ CUtensorMap mv_lo,
                const __grid_constant__ CUtensorMap me_hi, const __grid_constant__ CUtensorMap me_lo,
                const PropDev pd, int* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr int NT = 16 * NP, KQ = kWideKQ, S = kWideStages;
  constexpr uint32_t BT = (uint32_t)NT * 128;  // bytes per B K tile
  constexpr int kProd = 4 * NP, kCtrl = 4 * NP + 1;
  constexpr uint32_t kCols = 4 * NT <= 256 ? 256 : 512;  // TMEM columns allocated
  unsigned char* ring = smem;  // unit s: A_hi tile, then A_lo tile
  unsigned char* Bh = ring + S * 2 * kPropTile;
  unsigned char* Bl = Bh + KQ * BT;
  uint64_t* bars = reinterpret_cast<uint64_t*>(Bl + KQ * BT);
  uint64_t* full = bars;           // [S]
  uint64_t* empty = bars + S;      // [S]
  uint64_t* ready = bars + 2 * S;  // B rows written and the accumulators read
  uint64_t* done = ready + 1;      // the step's MMAs completed
  uint64_t* fin = ready + 2;       // every MMA issued has completed (teardown)
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(ready + 3);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool bf = pd.bf16 != 0;
  const int nsteps = pd.nterms + 1;  // exp_h1, nterms - 1 Taylor products, exp_h1
  // step st: exp_h1 (one A part, lo plane with e_lo) or Taylor product st (Vr and Vi, lo
  // plane for the first `split` products)
  auto step_expo = [&](int st) { return st == 0 || st == nsteps - 1; };
  auto step_alo = [&](int st) { return step_expo(st) ? pd.e_lo != 0 : st <= pd.split; };

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    ptx::mbar_init(ready, 4 * NP);
    ptx::mbar_init(done, 1);
    ptx::mbar_init(fin, 1);
    ptx::fence_mbar_init();
  }
  if (warp == kCtrl) {
    ptx::tmem_alloc(tmem_holder, kCols);  // D[mt][h] at (2 mt + h) NT
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  bool ok = true;

  if (warp == kProd) {
    if (lane == 0) {
      ptx::prefetch_tmap(&mv_hi);
      ptx::prefetch_tmap(&me_hi);
      int u = 0;
      for (int wl = blockIdx.x; wl < pd.nwc && ok; wl += gridDim.x)
        for (int st = 0; st < nsteps && ok; ++st) {
          const bool expo = step_expo(st), alo = step_alo(st);
          const int nparts = expo ? 1 : 2;
          for (int mt = 0; mt < 2 && ok; ++mt)
            for (int h = 0; h < nparts && ok; ++h)
              for (int kt = 0; kt < KQ; ++kt, ++u) {
                const int s = u % S, r = u / S;
                if (r > 0 && !ptx::mbar_wait(&empty[s], (r - 1) & 1)) {
                  ok = false;
                  break;
                }
                unsigned char* a = ring + s * 2 * kPropTile;
                ptx::mbar_expect_tx(&full[s], kPropTile * (alo ? 2 : 1));
                if (expo) {
                  ptx::tma_load_2d(a, &me_hi, &full[s], kt * 64, mt * 128);
                  if (alo) ptx::tma_load_2d(a + kPropTile, &me_lo, &full[s], kt * 64, mt * 128);
                } else {
                  const int x = h * 256 + kt * 64, y = wl * kWideMR + mt * 128;
                  ptx::tma_load_2d(a, &mv_hi, &full[s], x, y);
                  if (alo) ptx::tma_load_2d(a + kPropTile, &mv_lo, &full[s], x, y);
                }
              }
        }
      // never leave a copy in flight: the last round issued on each stage
      for (int j = u - 1; j >= 0 && j >= u - S; --j)
        if (!ptx::mbar_wait(&full[j % S], (j / S) & 1)) ok = false;
    }
  } else if (warp == kCtrl) {
    if (lane == 0) {
      const uint32_t sBh = ptx::smem_u32(Bh), sBl = ptx::smem_u32(Bl);
      const uint32_t idesc = ptx::idesc_f16(128, NT, bf ? 1 : 0);
      int u = 0;
      uint32_t sc = 0;
      for (int wl = blockIdx.x; wl < pd.nwc && ok; wl += gridDim.x)
        for (int st = 0; st < nsteps && ok; ++st, ++sc) {
          if (!ptx::mbar_wait(ready, sc & 1)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const bool expo = step_expo(st), alo = step_alo(st);
          const bool blo = expo ? pd.w_lo != 0 : st <= pd.split;
          const int nparts = expo ? 1 : 2;
          for (int mt = 0; mt < 2 && ok; ++mt)
            for (int h = 0; h < nparts && ok; ++h) {
              const uint32_t d = tmem + (uint32_t)((2 * mt + h) * NT);
              bool first = true;
              for (int kt = 0; kt < KQ; ++kt, ++u) {
                const int s = u % S;
                if (!ptx::mbar_wait(&full[s], (u / S) & 1)) {
                  ok = false;
                  break;
                }
                ptx::tc_fence_after();
                const uint32_t ah = ptx::smem_u32(ring + s * 2 * kPropTile), al = ah + kPropTile;
                const uint32_t bh = sBh + kt * BT, bl = sBl + kt * BT;
                auto mma4 = [&](uint32_t a, uint32_t b) {
#pragma unroll
                  for (int kk = 0; kk < 4; ++kk) {
                    ptx::mma_f16(d, ptx::desc_kmajor_sw128(a + kk * 32), ptx::desc_kmajor_sw128(b + kk * 32), idesc,
                                 first ? 0u : 1u);
                    first = false;
                  }
                };
                if (alo) mma4(al, bh);
                if (blo) mma4(ah, bl);
                mma4(ah, bh);
                ptx::mma_commit(&empty[s]);  // the stage is free once these MMAs completed
              }
            }
          if (ok) ptx::mma_commit(done);
        }
      ptx::mma_commit(fin);
      if (!ptx::mbar_wait(fin, 0)) ok = false;
    }
  } else {
    const int g = warp >> 2, q = warp & 3;  // 16-row part of the B operand, lane quadrant
    const int p0 = 32 * q + lane;           // rows p0 (M tile 0) and p0 + 128 (M tile 1)
    const int k0 = 8 * g;                   // first orbital of the part
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(16 * g);
    const int c8 = (p0 & 63) >> 3;
    // B rows 16g + r at K = p0 + 128 mt: K tile 2 mt + p0 / 64, swizzled within the tile
    const uint32_t b_off = (uint32_t)((p0 >> 6) * BT + 2048 * g) + ((uint32_t)(p0 & 7) << 1);
    const uint32_t sBh = ptx::smem_u32(Bh), sBl = ptx::smem_u32(Bl);
    auto put = [&](const float (&val)[2][16], bool lo) {
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int p = p0 + 128 * mt;
        const uint32_t base = b_off + (uint32_t)(2 * mt) * BT;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
          const uint32_t off = base + (uint32_t)(128 * r) + ((uint32_t)(c8 ^ (r & 7)) << 4);
          const float x = (p < pd.n && k0 + (r >> 1) < pd.o) ? val[mt][r] : 0.f;
          uint16_t h, l;
          split16(x, bf, h, l);
          sts16(sBh + off, h);
          if (lo) sts16(sBl + off, l);
        }
      }
    };
    auto signal = [&]() {
      ptx::fence_proxy_async();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(ready);
    };
    auto wait_done = [&](uint32_t sc) {
      return __all_sync(0xffffffffu, ptx::mbar_wait(done, sc & 1)) != 0;
    };
    uint32_t sc = 0;
    for (int wl = blockIdx.x; wl < pd.nwc && ok; wl += gridDim.x) {
      float acc[2][16];
      // ---- W1 = W + (E - I) W (acc holds W, then W1)
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int p = p0 + 128 * mt;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          float2 v = make_float2(0.f, 0.f);
          if (p < pd.n && k0 + kk < pd.o) v = pd.w[((size_t)wl * pd.n + p) * pd.o + k0 + kk];
          acc[mt][2 * kk] = v.x;
          acc[mt][2 * kk + 1] = v.y;
        }
      }
      put(acc, pd.w_lo != 0);
      signal();
      if (!wait_done(sc++)) {
        ok = false;
        break;
      }
      ptx::tc_fence_after();
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        float d0[16];
        ptx::tmem_ld16p(lane_base + (uint32_t)(2 * mt * NT), d0);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[mt][j] += d0[j];
      }
      put(acc, pd.nterms > 1 ? pd.split >= 1 : pd.w_lo != 0);
      signal();
      // ---- T_m = V T_{m-1} / m, acc += T_m
      for (int m = 1; m < pd.nterms; ++m) {
        if (!wait_done(sc++)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        float t[2][16];
        const float invm = 1.0f / (float)m;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          float d0[16], d1[16];
          ptx::tmem_ld16p(lane_base + (uint32_t)(2 * mt * NT), d0);
          ptx::tmem_ld16p(lane_base + (uint32_t)((2 * mt + 1) * NT), d1);
          ptx::tmem_ld_wait();
#pragma unroll
          for (int kk = 0; kk < 8; ++kk) {
            t[mt][2 * kk] = (d0[2 * kk] - d1[2 * kk + 1]) * invm;
            t[mt][2 * kk + 1] = (d0[2 * kk + 1] + d1[2 * kk]) * invm;
            acc[mt][2 * kk] += t[mt][2 * kk];
            acc[mt][2 * kk + 1] += t[mt][2 * kk + 1];
          }
        }
        if (m + 1 < pd.nterms)
          put(t, m + 1 <= pd.split);
        else
          put(acc, pd.w_lo != 0);  // operand of the final exp_h1 product
        signal();
      }
      if (!ok) break;
      // ---- W' = acc + (E - I) acc
      if (!wait_done(sc++)) {
        ok = false;
        break;
      }
      ptx::tc_fence_after();
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        float d0[16];
        ptx::tmem_ld16p(lane_base + (uint32_t)(2 * mt * NT), d0);
        ptx::tmem_ld_wait();
        const int p = p0 + 128 * mt;
        if (p < pd.n) {
          float2* dst = pd.w + ((size_t)wl * pd.n + p) * pd.o;
#pragma unroll
          for (int kk = 0; kk < 8; ++kk)
            if (k0 + kk < pd.o)
              dst[k0 + kk] = make_float2(acc[mt][2 * kk] + d0[2 * kk], acc[mt][2 * kk + 1] + d0[2 * kk + 1]);
        }
      }
    }
  }
  if (!ok) atomicOr(status, 2);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == kCtrl) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, kCols);
  }
}

}  // namespace afq

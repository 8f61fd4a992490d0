// Persistent split-precision tcgen05 GEMM: D[M x N] = A_hi B_hi^T + A_lo B_hi^T + A_hi B_lo^T
// (x ~ hi + lo, 16-bit planes; the lo terms are optional), for the large contractions whose
// operands are both dense planes (vhs = i sqrt(dt) x~ . chol).
//
// Against the tile-per-CTA core (afq_gemm.cuh) it changes three things:
//  * each K tile loads the four planes once (A_hi, A_lo, B_hi, B_lo) and issues the three
//    products from them, instead of re-loading A_hi and B_hi for every term;
//  * 128 x 256 output tiles (131 flop per loaded byte with both lo terms);
//  * one CTA per SM loops over tiles. The TMA warp runs ahead across tile boundaries, the
//    MMA warp alternates between two 256-column TMEM accumulators, and eight epilogue warps
//    keep the running FP32 sums in registers, so a tile's stores overlap the next tile's
//    main loop.
//
// Accumulation: the tensor core truncates when it adds into its FP32 accumulator (about
// 6e-9 * K relative bias over a long sum). The MMAs of every `drain` K tiles go into a fresh
// accumulator and the epilogue adds it to its register sums with round-to-nearest; inside a
// K tile the small correction products are issued before hi*hi so that they meet a small
// accumulator.
//
// Warp roles (320 threads): warp 0 lane 0 issues TMA loads into a two-deep ring of K-tile
// units; warp 1 owns the TMEM allocation (512 columns) and lane 0 issues the MMAs; warps
// 2..9 drain the accumulators: warp w reads TMEM lanes 32*(w%4).. and columns
// 128*((w-2)/4).. (thread = output row, 128 columns per thread). Every wait is bounded: on a
// timeout the CTA records a nonzero word in *status, stops, and still frees its TMEM.
#pragma once
#include "afq_ptx.cuh"

namespace afq {

struct SplitMaps {
  CUtensorMap a_hi, a_lo, b_hi, b_lo;  // A boxes 64 x 128 rows, B boxes 64 x kSplitBBox rows
};

constexpr int kSplitThreads = 320;
constexpr int kSplitBN = 256;
constexpr int kSplitStages = 2;
constexpr int kSplitA = 128 * 128;                      // bytes of one A plane per K tile
constexpr int kSplitB = kSplitBN * 128;                 // bytes of one B plane per K tile
constexpr int kSplitBBox = 128;                         // rows per B TMA box (half a tile)
constexpr int kSplitUnit = 2 * kSplitA + 2 * kSplitB;   // one K tile, four planes
constexpr int kSplitStageRow = 80;                      // bytes per row of an epilogue staging buffer
constexpr int kSplitStageWarp = 32 * kSplitStageRow;     // one buffer per epilogue warp
constexpr int kSplitSmem = 1024 + kSplitStages * kSplitUnit + 256 + 8 * kSplitStageWarp;

struct SplitArgs {
  int m_tiles, n_tiles, k_tiles;
  int k_splits;    // K split into this many ranges (tiles = m_tiles * n_tiles * k_splits)
  int a_row0;      // first A row (walker chunk)
  int has_alo;     // A_lo * B_hi term
  int has_blo;     // B_lo * A_hi term
  int drain;       // K tiles per accumulation run (>= 1)
  uint32_t idesc;  // M = 128, N = 256
};

// Epi::store(params, row, col0, v, ks): row of D (global row index without a_row0), 128
// consecutive columns col0.. in v[0..127], K range ks; columns >= N must be ignored by the
// epilogue. With k_splits > 1 each K range produces a partial result. An epilogue with
// kWarpStore provides store_warp(params, row0, lane, col0, v, ks, stage) instead, called by
// all 32 lanes of the warp (rows row0 + lane) with a kSplitStageWarp-byte shared-memory
// buffer of its own.
template <class Epi>
__global__ void __launch_bounds__(kSplitThreads, 1)
    k_gemm_split(const __grid_constant__ SplitMaps maps, const SplitArgs g,
                 const __grid_constant__ typename Epi::Params ep, int* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kSplitStages * kSplitUnit);
  uint64_t* empty = full + kSplitStages;
  uint64_t* accfull = empty + kSplitStages;  // [2]
  uint64_t* accempty = accfull + 2;          // [2]
  uint64_t* done = accempty + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cid = blockIdx.x, ncl = gridDim.x;
  const int mt = g.m_tiles;
  const int ntiles = mt * g.n_tiles * g.k_splits;
  const int kps = (g.k_tiles + g.k_splits - 1) / g.k_splits;  // K tiles per split
  const uint32_t tx_bytes = kSplitA * (g.has_alo ? 2 : 1) + kSplitB * (g.has_blo ? 2 : 1);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kSplitStages; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      ptx::mbar_init(&accfull[a], 1);
      ptx::mbar_init(&accempty[a], 8);  // one arrival per epilogue warp
    }
    ptx::mbar_init(done, 1);
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_holder, 512);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      ptx::prefetch_tmap(&maps.a_hi);
      ptx::prefetch_tmap(&maps.b_hi);
      if (g.has_alo) ptx::prefetch_tmap(&maps.a_lo);
      if (g.has_blo) ptx::prefetch_tmap(&maps.b_lo);
      int it = 0;
      for (int tile = cid; tile < ntiles && ok; tile += ncl) {
        const int m0 = (tile % mt) * 128, n0 = ((tile / mt) % g.n_tiles) * kSplitBN;
        const int ks = tile / (mt * g.n_tiles);
        const int ka = ks * kps, kb = min(g.k_tiles, ka + kps);
        for (int kt = ka; kt < kb; ++kt, ++it) {
          const int s = it % kSplitStages, r = it / kSplitStages;
          if (r > 0 && !ptx::mbar_wait(&empty[s], (r - 1) & 1)) {
            ok = false;
            break;
          }
          unsigned char* u = smem + s * kSplitUnit;
          ptx::mbar_expect_tx(&full[s], tx_bytes);
          ptx::tma_load_2d(u, &maps.a_hi, &full[s], kt * 64, g.a_row0 + m0);
          if (g.has_alo) ptx::tma_load_2d(u + kSplitA, &maps.a_lo, &full[s], kt * 64, g.a_row0 + m0);
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            const int hb = hh * kSplitBBox * 128;
            ptx::tma_load_2d(u + 2 * kSplitA + hb, &maps.b_hi, &full[s], kt * 64, n0 + hh * kSplitBBox);
            if (g.has_blo)
              ptx::tma_load_2d(u + 2 * kSplitA + kSplitB + hb, &maps.b_lo, &full[s], kt * 64, n0 + hh * kSplitBBox);
          }
        }
      }
      // never leave a copy in flight: wait for the last round issued on each stage
      for (int j = it - 1; j >= 0 && j >= it - kSplitStages; --j)
        if (!ptx::mbar_wait(&full[j % kSplitStages], (j / kSplitStages) & 1)) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int it = 0, grun = 0;
      for (int tile = cid; tile < ntiles && ok; tile += ncl) {
        const int ks = tile / (mt * g.n_tiles);
        const int ka = ks * kps, kb = min(g.k_tiles, ka + kps);
        const int runs_per_tile = kb > ka ? (kb - ka + g.drain - 1) / g.drain : 0;
        for (int run = 0; run < runs_per_tile && ok; ++run, ++grun) {
          const int a = grun & 1;
          if (grun >= 2 && !ptx::mbar_wait(&accempty[a], ((grun - 2) >> 1) & 1)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t dacc = tmem + (uint32_t)(a * kSplitBN);
          const int kt0 = ka + run * g.drain, kt1 = min(kb, kt0 + g.drain);
          for (int kt = kt0; kt < kt1; ++kt, ++it) {
            const int s = it % kSplitStages, r = it / kSplitStages;
            if (!ptx::mbar_wait(&full[s], r & 1)) {
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            const uint32_t ua = ptx::smem_u32(smem + s * kSplitUnit);
            const uint32_t ahi = ua, alo = ua + kSplitA, bhi = ua + 2 * kSplitA, blo = bhi + kSplitB;
            bool first = kt == kt0;
            // correction products first, then hi * hi
            if (g.has_alo) {
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) {
                ptx::mma_f16(dacc, ptx::desc_kmajor_sw128(alo + kk * 32), ptx::desc_kmajor_sw128(bhi + kk * 32),
                             g.idesc, first ? 0u : 1u);
                first = false;
              }
            }
            if (g.has_blo) {
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) {
                ptx::mma_f16(dacc, ptx::desc_kmajor_sw128(ahi + kk * 32), ptx::desc_kmajor_sw128(blo + kk * 32),
                             g.idesc, first ? 0u : 1u);
                first = false;
              }
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              ptx::mma_f16(dacc, ptx::desc_kmajor_sw128(ahi + kk * 32), ptx::desc_kmajor_sw128(bhi + kk * 32),
                           g.idesc, first ? 0u : 1u);
              first = false;
            }
            ptx::mma_commit(&empty[s]);
          }
          ptx::mma_commit(&accfull[a]);
        }
      }
      // every MMA issued has completed before TMEM is released
      ptx::mma_commit(done);
      if (!ptx::mbar_wait(done, 0)) ok = false;
    }
  } else {
    const int q = warp & 3, half = (warp - 2) >> 2;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    int grun = 0;
    for (int tile = cid; tile < ntiles && ok; tile += ncl) {
      const int m0 = (tile % mt) * 128, n0 = ((tile / mt) % g.n_tiles) * kSplitBN;
      const int ks = tile / (mt * g.n_tiles);
      const int ka = ks * kps, kb = min(g.k_tiles, ka + kps);
      const int runs_per_tile = kb > ka ? (kb - ka + g.drain - 1) / g.drain : 0;
      float sum[128];
#pragma unroll
      for (int j = 0; j < 128; ++j) sum[j] = 0.f;
      for (int run = 0; run < runs_per_tile; ++run, ++grun) {
        const int a = grun & 1;
        // warp-uniform outcome: the TMEM loads below are .sync.aligned
        if (!__all_sync(0xffffffffu, ptx::mbar_wait(&accfull[a], (grun >> 1) & 1))) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        const uint32_t src = tmem + lane_off + (uint32_t)(a * kSplitBN + half * 128);
#pragma unroll
        for (int h = 0; h < 128; h += 32) {
          float v[32];
          ptx::tmem_ld16p(src + h, v);
          ptx::tmem_ld16p(src + h + 16, v + 16);
          ptx::tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 32; ++j) sum[h + j] += v[j];
        }
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&accempty[a]);
      }
      if (!ok) break;
      if constexpr (Epi::kWarpStore)
        Epi::store_warp(ep, m0 + q * 32, lane, n0 + half * 128, sum, ks,
                        smem + kSplitStages * kSplitUnit + 256 + (warp - 2) * kSplitStageWarp);
      else
        Epi::store(ep, m0 + q * 32 + lane, n0 + half * 128, sum, ks);
    }
  }
  if (!ok) atomicOr(status, 4);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
}

// Plain epilogue for tests: D (fp32, row-major, ldd) clipped to M x N.
struct SplitStoreF32 {
  static constexpr bool kWarpStore = false;
  struct Params {
    float* d;
    int M, N;
    long ldd;
  };
  __device__ __forceinline__ static void store(const Params& p, int row, int col0, const float* v, int) {
    if (row >= p.M) return;
#pragma unroll
    for (int j = 0; j < 128; ++j)
      if (col0 + j < p.N) p.d[(long)row * p.ldd + col0 + j] = v[j];
  }
};

// Partial results of a K-split GEMM: d[ks][row][col] (fp32, row stride ldd, split stride sst).
// K-split partials: D_ks (fp32, row-major, ldd; partial ks at d + ks * sst), rows < M, groups
// of 4 columns starting below N (ldd covers the last group). Per 16 columns the warp stages its 32 rows in shared memory, then four
// lanes store each row's 64 contiguous bytes.
struct SplitPartialF32 {
  static constexpr bool kWarpStore = true;
  struct Params {
    float* d;
    int M, N;
    long ldd, sst;
  };
  __device__ __forceinline__ static void store_warp(const Params& p, int row0, int lane, int col0, const float* v,
                                                    int ks, unsigned char* stage) {
    float* base = p.d + (long)ks * p.sst;
#pragma unroll
    for (int c16 = 0; c16 < 128; c16 += 16) {
      if (col0 + c16 >= p.N) break;  // warp-uniform
      float4* srow = reinterpret_cast<float4*>(stage + lane * kSplitStageRow);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        srow[u] = make_float4(v[c16 + 4 * u], v[c16 + 4 * u + 1], v[c16 + 4 * u + 2], v[c16 + 4 * u + 3]);
      __syncwarp();
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int t = lane + 32 * u, row = t >> 2, part = t & 3;
        const int r = row0 + row, c = col0 + c16 + 4 * part;
        if (r < p.M && c < p.N)
          *reinterpret_cast<float4*>(base + (long)r * p.ldd + c) =
              *reinterpret_cast<const float4*>(stage + row * kSplitStageRow + 16 * part);
      }
      __syncwarp();
    }
  }
};

}  // namespace afq

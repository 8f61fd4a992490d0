// Persistent split-precision tcgen05 GEMM: D[M x N] = A_hi B_hi^T + A_lo B_hi^T + A_hi B_lo^T
// (x ~ hi + lo, 16-bit planes; the lo terms are optional), for the large contractions whose
// operands are both dense planes (vhs = i sqrt(dt) x~ . chol, force bias, exchange matrix).
//
// Against the tile-per-CTA core (afq_gemm.cuh) it changes three things:
//  * each K tile loads the four planes once (A_hi, A_lo, B_hi, B_lo) and issues the three
//    products from them, instead of re-loading A_hi and B_hi for every term;
//  * 128 x 256 output tiles (131 flop per loaded byte with both lo terms);
//  * one CTA (or CTA pair) per SM loops over tiles. The TMA warp runs ahead across tile
//    boundaries, the MMA warp alternates between two 256-column TMEM accumulators, and eight
//    epilogue warps keep the running FP32 sums in registers, so a tile's stores overlap the
//    next tile's main loop for two accumulation runs. (A tcgen05.mma costs about the same
//    for N = 128 as for N = 256, so narrower tiles with more accumulators run slower.)
//
// Accumulation: the tensor core truncates when it adds into its FP32 accumulator (about
// 6e-9 * K relative bias over a long sum). The MMAs of every `drain` K tiles go into a fresh
// accumulator and the epilogue adds it to its register sums with round-to-nearest; inside a
// K tile the small correction products are issued before hi*hi so that they meet a small
// accumulator.
//
// Warp roles (320 threads): warp 0 lane 0 issues TMA loads into a ring of K-tile units; warp
// 1 owns the TMEM allocation (512 columns) and lane 0 issues the MMAs; warps 2..9 drain the
// accumulators: warp w reads TMEM lanes 32*(w%4).. and columns 128*((w-2)/4).. (thread =
// output row, 128 columns per thread). Every wait is bounded: on a timeout the CTA records a
// nonzero word in *status, stops, and still frees its TMEM.
//
// CTA pairs (CG = 2, clusters of two CTAs): a tile is 256 rows x 256 columns and one
// tcgen05.mma.cta_group::2 (M = 256) issued by the even CTA covers both SMs. Each CTA loads
// its own 128 A rows and its own half (128 rows) of the B tile with plain TMA loads into its
// own shared memory (64 KB per K tile instead of 96 KB; three-deep ring). The loads of both
// CTAs complete on the even CTA's `full` barrier; the even CTA's MMA thread releases stages
// and accumulators with one commit per CTA; the odd CTA's epilogue warps arrive remotely on
// the even CTA's `accempty` barriers. Each CTA drains and stores its own 128 accumulator rows
// from its own TMEM.
#pragma once
#include "afq_ptx.cuh"

namespace afq {

struct SplitMaps {
  CUtensorMap a_hi, a_lo, b_hi, b_lo;  // A boxes 64 x 128 rows, B boxes 64 x kSplitBBox rows
};

constexpr int kSplitThreads = 320;
constexpr int kSplitBN = 256;                            // output columns per tile
constexpr int kSplitBBox = 128;                          // rows per B TMA box
constexpr int kSplitA = 128 * 128;                       // bytes of one A plane per K tile
constexpr int kSplitB = kSplitBN * 128;                  // bytes of one B plane (all tile rows) per K tile
constexpr int kSplitRing = 3 * 65536;                    // K-tile ring in shared memory
constexpr int kSplitStages = 2;                          // single CTA: 96 KB units
constexpr int kSplitUnit = 2 * kSplitA + 2 * kSplitB;
constexpr int kSplitStages2 = 3;                         // CTA pair: 64 KB units (half of B)
constexpr int kSplitUnit2 = 2 * kSplitA + 2 * (kSplitB / 2);
constexpr int kSplitStageRow = 80;                       // bytes per row of an epilogue staging buffer
constexpr int kSplitStageWarp = 32 * kSplitStageRow;     // one buffer per epilogue warp
constexpr int kSplitSmem = 1024 + kSplitRing + 256 + 8 * kSplitStageWarp;
static_assert(kSplitStages * kSplitUnit <= kSplitRing && kSplitStages2 * kSplitUnit2 <= kSplitRing,
              "K-tile ring");

struct SplitArgs {
  int m_tiles, n_tiles, k_tiles;
  int k_splits;    // K split into this many ranges (tiles = m_tiles * n_tiles * k_splits)
  int a_row0;      // first A row (walker chunk)
  int has_alo;     // A_lo * B_hi term
  int has_blo;     // B_lo * A_hi term
  int drain;       // K tiles per accumulation run (>= 1)
  uint32_t idesc;  // M = 128 (256 for CTA pairs), N = kSplitBN
};

// Epi::store(params, row, col0, v, ks): row of D (global row index without a_row0), 128
// consecutive columns col0.. in v[0..127], K range ks; columns >= N must be ignored by the
// epilogue. With k_splits > 1 each K range produces a partial result. An epilogue with
// kWarpStore provides store_warp(params, row0, lane, col0, v, ks, stage) instead, called by
// all 32 lanes of the warp (rows row0 + lane) with a kSplitStageWarp-byte shared-memory
// buffer of its own.
template <class Epi, int CG = 1>
__global__ void __launch_bounds__(kSplitThreads, 1)
    k_gemm_split(const __grid_constant__ SplitMaps maps, const SplitArgs g,
                 const __grid_constant__ typename Epi::Params ep, int* status) {
  static_assert(CG == 1 || CG == 2, "one CTA or a CTA pair per tile");
  constexpr int STAGES = CG == 2 ? kSplitStages2 : kSplitStages;
  constexpr int UNIT = CG == 2 ? kSplitUnit2 : kSplitUnit;
  constexpr int BPL = kSplitB / CG;  // bytes of one B plane per CTA and K tile
  constexpr int NBOX = kSplitBN / CG / kSplitBBox;  // B boxes per plane per CTA
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kSplitRing);
  uint64_t* empty = full + STAGES;
  uint64_t* accfull = empty + STAGES;  // [2]
  uint64_t* accempty = accfull + 2;    // [2]
  uint64_t* done = accempty + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(done + 1);
  unsigned char* stage_base = smem + kSplitRing + 256;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = CG == 2 ? ptx::cluster_ctarank() : 0u;
  const bool leader = rank == 0;
  const int cid = blockIdx.x / CG, ncl = gridDim.x / CG;
  const int mt = (g.m_tiles + CG - 1) / CG;  // row blocks of 128 * CG rows
  const int ntiles = mt * g.n_tiles * g.k_splits;
  const int kps = (g.k_tiles + g.k_splits - 1) / g.k_splits;  // K tiles per split
  const uint32_t tx_cta = kSplitA * (g.has_alo ? 2 : 1) + BPL * (g.has_blo ? 2 : 1);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      ptx::mbar_init(&accfull[a], 1);
      ptx::mbar_init(&accempty[a], 8 * CG);  // one arrival per epilogue warp of the pair
    }
    ptx::mbar_init(done, 1);
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    if constexpr (CG == 2) {
      ptx::tmem_alloc_pair(tmem_holder, 512);
      ptx::tmem_relinquish_pair();
    } else {
      ptx::tmem_alloc(tmem_holder, 512);
      ptx::tmem_relinquish();
    }
  }
  ptx::tc_fence_before();
  if constexpr (CG == 2)
    ptx::cluster_sync();  // the peer's barriers are initialised before any remote arrival
  else
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
        const int m0 = (tile % mt) * 128 * CG + (int)rank * 128;
        const int nb = ((tile / mt) % g.n_tiles) * kSplitBN + (int)rank * (kSplitBN / CG);
        const int ks = tile / (mt * g.n_tiles);
        const int ka = ks * kps, kb = min(g.k_tiles, ka + kps);
        for (int kt = ka; kt < kb; ++kt, ++it) {
          const int s = it % STAGES, r = it / STAGES;
          if (r > 0) {
            const bool got = CG == 2 ? ptx::mbar_wait_cluster(&empty[s], (r - 1) & 1)
                                     : ptx::mbar_wait(&empty[s], (r - 1) & 1);
            if (!got) {
              ok = false;
              break;
            }
          }
          unsigned char* u = smem + s * UNIT;
          if constexpr (CG == 2) {
            // both CTAs' loads complete on the even CTA's barrier, which expects the pair's bytes
            const uint32_t fb = ptx::mapa_shared(&full[s], 0);
            if (leader) ptx::mbar_expect_tx(&full[s], 2 * tx_cta);
            ptx::tma_load_2d_pair(u, &maps.a_hi, fb, kt * 64, g.a_row0 + m0);
            if (g.has_alo) ptx::tma_load_2d_pair(u + kSplitA, &maps.a_lo, fb, kt * 64, g.a_row0 + m0);
#pragma unroll
            for (int hh = 0; hh < NBOX; ++hh) {
              const int hb = hh * kSplitBBox * 128;
              ptx::tma_load_2d_pair(u + 2 * kSplitA + hb, &maps.b_hi, fb, kt * 64, nb + hh * kSplitBBox);
              if (g.has_blo)
                ptx::tma_load_2d_pair(u + 2 * kSplitA + BPL + hb, &maps.b_lo, fb, kt * 64, nb + hh * kSplitBBox);
            }
          } else {
            ptx::mbar_expect_tx(&full[s], tx_cta);
            ptx::tma_load_2d(u, &maps.a_hi, &full[s], kt * 64, g.a_row0 + m0);
            if (g.has_alo) ptx::tma_load_2d(u + kSplitA, &maps.a_lo, &full[s], kt * 64, g.a_row0 + m0);
#pragma unroll
            for (int hh = 0; hh < NBOX; ++hh) {
              const int hb = hh * kSplitBBox * 128;
              ptx::tma_load_2d(u + 2 * kSplitA + hb, &maps.b_hi, &full[s], kt * 64, nb + hh * kSplitBBox);
              if (g.has_blo)
                ptx::tma_load_2d(u + 2 * kSplitA + BPL + hb, &maps.b_lo, &full[s], kt * 64, nb + hh * kSplitBBox);
            }
          }
        }
      }
      // never leave a copy in flight: wait for the last round issued on each stage (the even
      // CTA's barrier counts the odd CTA's bytes too; the odd CTA cannot leave before the
      // closing cluster barrier, which the even CTA reaches after this wait)
      if (leader)
        for (int j = it - 1; j >= 0 && j >= it - STAGES; --j) {
          const bool got = CG == 2 ? ptx::mbar_wait_cluster(&full[j % STAGES], (j / STAGES) & 1)
                                   : ptx::mbar_wait(&full[j % STAGES], (j / STAGES) & 1);
          if (!got) ok = false;
        }
    }
  } else if (warp == 1) {
    if (lane == 0 && leader) {
      int it = 0, grun = 0;
      uint32_t peer_empty = 0, peer_accfull = 0;
      if constexpr (CG == 2) {
        peer_empty = ptx::mapa_shared(empty, 1);
        peer_accfull = ptx::mapa_shared(accfull, 1);
      }
      for (int tile = cid; tile < ntiles && ok; tile += ncl) {
        const int ks = tile / (mt * g.n_tiles);
        const int ka = ks * kps, kb = min(g.k_tiles, ka + kps);
        const int runs_per_tile = kb > ka ? (kb - ka + g.drain - 1) / g.drain : 0;
        for (int run = 0; run < runs_per_tile && ok; ++run, ++grun) {
          const int a = grun & 1;
          if (grun >= 2) {
            const bool got = CG == 2 ? ptx::mbar_wait_cluster(&accempty[a], ((grun - 2) >> 1) & 1)
                                     : ptx::mbar_wait(&accempty[a], ((grun - 2) >> 1) & 1);
            if (!got) {
              ok = false;
              break;
            }
          }
          ptx::tc_fence_after();
          const uint32_t dacc = tmem + (uint32_t)(a * kSplitBN);
          const int kt0 = ka + run * g.drain, kt1 = min(kb, kt0 + g.drain);
          for (int kt = kt0; kt < kt1; ++kt, ++it) {
            const int s = it % STAGES, r = it / STAGES;
            const bool got = CG == 2 ? ptx::mbar_wait_cluster(&full[s], r & 1) : ptx::mbar_wait(&full[s], r & 1);
            if (!got) {
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            const uint32_t ua = ptx::smem_u32(smem + s * UNIT);
            const uint32_t ahi = ua, alo = ua + kSplitA, bhi = ua + 2 * kSplitA, blo = bhi + BPL;
            bool first = kt == kt0;
            auto mma = [&](uint32_t ad, uint32_t bd) {
              const uint64_t da = ptx::desc_kmajor_sw128(ad), db = ptx::desc_kmajor_sw128(bd);
              if constexpr (CG == 2)
                ptx::mma_f16_pair(dacc, da, db, g.idesc, first ? 0u : 1u);
              else
                ptx::mma_f16(dacc, da, db, g.idesc, first ? 0u : 1u);
              first = false;
            };
            // correction products first, then hi * hi
            if (g.has_alo) {
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) mma(alo + kk * 32, bhi + kk * 32);
            }
            if (g.has_blo) {
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) mma(ahi + kk * 32, blo + kk * 32);
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) mma(ahi + kk * 32, bhi + kk * 32);
            if constexpr (CG == 2) {
              ptx::mma_commit_pair(ptx::smem_u32(&empty[s]));
              ptx::mma_commit_pair(peer_empty + (uint32_t)(s * 8));
            } else {
              ptx::mma_commit(&empty[s]);
            }
          }
          if constexpr (CG == 2) {
            ptx::mma_commit_pair(ptx::smem_u32(&accfull[a]));
            ptx::mma_commit_pair(peer_accfull + (uint32_t)(a * 8));
          } else {
            ptx::mma_commit(&accfull[a]);
          }
        }
      }
      // every MMA issued has completed before TMEM is released
      if constexpr (CG == 2)
        ptx::mma_commit_pair(ptx::smem_u32(done));
      else
        ptx::mma_commit(done);
      if (!ptx::mbar_wait(done, 0)) ok = false;
    }
  } else {
    const int q = warp & 3, half = (warp - 2) >> 2;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    uint32_t acc_empty_bar = 0;
    if constexpr (CG == 2) acc_empty_bar = ptx::mapa_shared(accempty, 0);
    int grun = 0;
    for (int tile = cid; tile < ntiles && ok; tile += ncl) {
      const int m0 = (tile % mt) * 128 * CG + (int)rank * 128, n0 = ((tile / mt) % g.n_tiles) * kSplitBN;
      const int ks = tile / (mt * g.n_tiles);
      const int ka = ks * kps, kb = min(g.k_tiles, ka + kps);
      const int runs_per_tile = kb > ka ? (kb - ka + g.drain - 1) / g.drain : 0;
      float sum[128];
#pragma unroll
      for (int j = 0; j < 128; ++j) sum[j] = 0.f;
      for (int run = 0; run < runs_per_tile; ++run, ++grun) {
        const int a = grun & 1;
        // warp-uniform outcome: the TMEM loads below are .sync.aligned
        const bool got = CG == 2 ? ptx::mbar_wait_cluster(&accfull[a], (grun >> 1) & 1)
                                 : ptx::mbar_wait(&accfull[a], (grun >> 1) & 1);
        if (!__all_sync(0xffffffffu, got)) {
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
        if (lane == 0) {
          if constexpr (CG == 2)
            ptx::mbar_arrive_cluster(acc_empty_bar + (uint32_t)(a * 8));
          else
            ptx::mbar_arrive(&accempty[a]);
        }
      }
      if (!ok) break;
      if constexpr (Epi::kWarpStore)
        Epi::store_warp(ep, m0 + q * 32, lane, n0 + half * 128, sum, ks, stage_base + (warp - 2) * kSplitStageWarp);
      else
        Epi::store(ep, m0 + q * 32 + lane, n0 + half * 128, sum, ks);
    }
  }
  if (!ok) atomicOr(status, 4);
  ptx::tc_fence_before();
  if constexpr (CG == 2)
    ptx::cluster_sync();  // the even CTA's MMAs into this CTA's TMEM and shared memory are done
  else
    __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    if constexpr (CG == 2)
      ptx::tmem_dealloc_pair(tmem, 512);
    else
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

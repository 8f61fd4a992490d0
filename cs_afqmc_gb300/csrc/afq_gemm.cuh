// Warp-specialised tcgen05 GEMM core: D[M x N] (fp32, TMEM) = sum_t A_t[M x K] * B_t[N x K]^T
// over up to three (A_t, B_t) operand pairs (the split-precision hi/lo terms), 16-bit inputs
// (bf16 or fp16), both operands K-major in global memory, loaded by TMA with the 128-byte
// swizzle. One 128 x bn output tile per CTA; bn (runtime, multiple of 16, <= BNMAX) sets the
// MMA N, the B box and the epilogue width; BNMAX sizes the shared-memory ring.
//
// The A rows of the tile start at a_row0 + 128 * blockIdx.y (a_row0 selects a walker chunk);
// the epilogue sees the tile origin without a_row0.
//
// Warp roles (192 threads): warp 0 lane 0 issues TMA loads into a STAGES-deep ring;
// warp 1 owns the TMEM allocation and lane 0 issues the MMAs; warps 2..5 run the epilogue
// (warp w reads TMEM lanes 32*(w%4) .. 32*(w%4)+31). Every wait is bounded: on a timeout the
// CTA records a nonzero word in *status and still frees its TMEM.
//
// Accumulation. The tensor core adds each MMA's products into the FP32 accumulator with
// truncation, which biases long sums toward zero by about 6e-9 * K relative (measured on
// GB300: -1.5e-5 at K = 2400). With drain = d > 0 the MMAs of every d consecutive K tiles go
// into a fresh accumulator (two, used alternately), and the epilogue warps add each finished
// accumulator into a third TMEM region with round-to-nearest FP32 adds while the tensor
// core fills the other one. Every truncated run then spans 4 d MMAs only.
#pragma once
#include "afq_ptx.cuh"

namespace afq {

struct GemmMaps {
  CUtensorMap a[3];
  CUtensorMap b[3];
};

constexpr int kGemmThreads = 192;

__host__ __device__ constexpr int gemm_tmem_cols(int bn) {
  return bn <= 32 ? 32 : bn <= 64 ? 64 : bn <= 128 ? 128 : bn <= 256 ? 256 : 512;
}

template <int BNMAX, int STAGES>
__host__ __device__ constexpr int gemm_pipe_bytes() {
  return STAGES * (128 * 128 + BNMAX * 128);
}

// Dynamic shared memory for the core: pipeline + 256 B of barriers + epilogue scratch,
// plus 1 KB of alignment slack.
template <int BNMAX, int STAGES, class Epi>
__host__ __device__ constexpr int gemm_smem_bytes() {
  return 1024 + gemm_pipe_bytes<BNMAX, STAGES>() + 256 + Epi::kSmemBytes;
}

template <int BNMAX, int STAGES, class Epi>
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_gemm_tc(const __grid_constant__ GemmMaps maps, int nterms, int k_tiles, int bn, int a_row0,
              int drain, uint32_t idesc, const __grid_constant__ typename Epi::Params ep,
              int* status) {
  static_assert(BNMAX % 16 == 0 && BNMAX >= 16 && BNMAX <= 256, "BNMAX");
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr int A_BYTES = 128 * 128;  // 128 rows x 64 x 16-bit
  constexpr int STAGE = A_BYTES + BNMAX * 128;
  const uint32_t TMEM_COLS = gemm_tmem_cols(drain ? 3 * bn : bn);
  const uint32_t tx_bytes = A_BYTES + bn * 128;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE);
  uint64_t* empty = full + STAGES;
  uint64_t* accb = empty + STAGES;
  uint64_t* accfull = accb + 1;    // [2]
  uint64_t* accempty = accb + 3;   // [2]
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(accb + 5);
  unsigned char* epi_smem = smem + STAGES * STAGE + 256;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * bn;
  const int total = nterms * k_tiles;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    ptx::mbar_init(accb, 1);
    for (int a = 0; a < 2; ++a) {
      ptx::mbar_init(&accfull[a], 1);
      ptx::mbar_init(&accempty[a], 4);  // one arrival per epilogue warp
    }
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_holder, TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      for (int t = 0; t < nterms; ++t) {
        ptx::prefetch_tmap(&maps.a[t]);
        ptx::prefetch_tmap(&maps.b[t]);
      }
      int issued = 0;
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES, r = it / STAGES;
        if (r > 0 && !ptx::mbar_wait(&empty[s], (r - 1) & 1)) {
          ok = false;
          break;
        }
        const int t = it / k_tiles, kt = it % k_tiles;
        unsigned char* sa = smem + s * STAGE;
        ptx::mbar_expect_tx(&full[s], tx_bytes);
        ptx::tma_load_2d(sa, &maps.a[t], &full[s], kt * 64, a_row0 + m0);
        ptx::tma_load_2d(sa + A_BYTES, &maps.b[t], &full[s], kt * 64, n0);
        ++issued;
      }
      // never leave a copy in flight: wait for the last round issued on each stage
      for (int it = issued - 1; it >= 0 && it >= issued - STAGES; --it)
        if (!ptx::mbar_wait(&full[it % STAGES], (it / STAGES) & 1)) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      if (!drain) {
        for (int it = 0; it < total; ++it) {
          const int s = it % STAGES, r = it / STAGES;
          if (!ptx::mbar_wait(&full[s], r & 1)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t sa = ptx::smem_u32(smem + s * STAGE), sb = sa + A_BYTES;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            ptx::mma_f16(tmem, ptx::desc_kmajor_sw128(sa + kk * 32), ptx::desc_kmajor_sw128(sb + kk * 32),
                         idesc, (it > 0 || kk > 0) ? 1u : 0u);
          }
          ptx::mma_commit(&empty[s]);
        }
        ptx::mma_commit(accb);
      } else {
        const int nruns = (total + drain - 1) / drain;
        for (int run = 0; run < nruns && ok; ++run) {
          const int a = run & 1;
          if (run >= 2 && !ptx::mbar_wait(&accempty[a], ((run - 2) >> 1) & 1)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t dacc = tmem + (uint32_t)((1 + a) * bn);
          const int it0 = run * drain, it1 = min(total, it0 + drain);
          for (int it = it0; it < it1; ++it) {
            const int s = it % STAGES, r = it / STAGES;
            if (!ptx::mbar_wait(&full[s], r & 1)) {
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            const uint32_t sa = ptx::smem_u32(smem + s * STAGE), sb = sa + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              ptx::mma_f16(dacc, ptx::desc_kmajor_sw128(sa + kk * 32), ptx::desc_kmajor_sw128(sb + kk * 32),
                           idesc, (it > it0 || kk > 0) ? 1u : 0u);
            }
            ptx::mma_commit(&empty[s]);
          }
          ptx::mma_commit(&accfull[a]);
        }
        // every MMA this thread issued has completed before TMEM is released
        ptx::mma_commit(accb);
        if (!ptx::mbar_wait(accb, 0)) ok = false;
      }
    }
  } else {
    const int q = warp & 3;
    bool got = true;
    if (!drain) {
      got = ptx::mbar_wait(accb, 0);
      ptx::tc_fence_after();
    } else if constexpr (BNMAX <= 128) {
      // Running sum in registers (thread = TMEM lane = output row, BNMAX columns): a drain
      // is one TMEM read of the finished accumulator; the sum goes to TMEM columns [0, bn)
      // once, after the last run, for the epilogue.
      const int nruns = (total + drain - 1) / drain;
      const uint32_t lane_off = (uint32_t)(q * 32) << 16;
      float sum[BNMAX];
#pragma unroll
      for (int j = 0; j < BNMAX; ++j) sum[j] = 0.f;
      for (int run = 0; run < nruns; ++run) {
        const int a = run & 1;
        if (!ptx::mbar_wait(&accfull[a], (run >> 1) & 1)) {
          got = false;
          break;
        }
        ptx::tc_fence_after();
        const uint32_t src = tmem + lane_off + (uint32_t)((1 + a) * bn);
#pragma unroll
        for (int h = 0; h < BNMAX; h += 64) {
          if (h < bn) {
            float v[64];
#pragma unroll
            for (int c = 0; c < 64; c += 16)
              if (h + c < bn) ptx::tmem_ld16p(src + h + c, v + c);
            ptx::tmem_ld_wait();
#pragma unroll
            for (int c = 0; c < 64; c += 16)
              if (h + c < bn) {
#pragma unroll
                for (int j = 0; j < 16; ++j) sum[h + c + j] += v[c + j];
              }
          }
        }
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&accempty[a]);
      }
      if (got) {
#pragma unroll
        for (int c = 0; c < BNMAX; c += 16)
          if (c < bn) ptx::tmem_st16p(tmem + lane_off + (uint32_t)c, sum + c);
        ptx::tmem_st_wait();
      }
      ptx::tc_fence_after();
    } else {
      const int nruns = (total + drain - 1) / drain;
      const uint32_t lane_off = (uint32_t)(q * 32) << 16;
      for (int run = 0; run < nruns; ++run) {
        const int a = run & 1;
        if (!ptx::mbar_wait(&accfull[a], (run >> 1) & 1)) {
          got = false;
          break;
        }
        ptx::tc_fence_after();
#pragma unroll 1
        for (int c0 = 0; c0 < bn; c0 += 16) {
          float v[16];
          ptx::tmem_ld16(tmem + lane_off + (uint32_t)((1 + a) * bn + c0), v);
          if (run > 0) {
            float sum[16];
            ptx::tmem_ld16(tmem + lane_off + (uint32_t)c0, sum);
            ptx::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += sum[j];
          } else {
            ptx::tmem_ld_wait();
          }
          ptx::tmem_st16(tmem + lane_off + (uint32_t)c0, v);
        }
        ptx::tmem_st_wait();
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&accempty[a]);
      }
      ptx::tc_fence_after();
    }
    if (!got) ok = false;
    Epi::run(ep, m0, n0, bn, tmem, q, lane, epi_smem, got);
  }
  if (!ok) atomicOr(status, 1);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// Plain epilogue: D (fp32, row-major, ldd) = accumulator, clipped to M x N. Used by tests.
struct EpiStoreF32 {
  struct Params {
    float* d;
    int M, N;
    long ldd;
  };
  static constexpr int kSmemBytes = 0;
  __device__ static void run(const Params& p, int m0, int n0, int bn, uint32_t tmem, int q,
                             int lane, unsigned char*, bool) {
    const int row = m0 + q * 32 + lane;
#pragma unroll 1
    for (int c = 0; c < bn; c += 16) {
      float v[16];
      ptx::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + c, v);
      ptx::tmem_ld_wait();
      if (row < p.M) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (n0 + c + j < p.N) p.d[(long)row * p.ldd + n0 + c + j] = v[j];
      }
    }
  }
};

// Host: tensor map for a row-major 16-bit matrix [rows][cols] (row stride ld elements),
// box = 64 columns x box_rows rows, 128-byte swizzle, zero fill out of bounds.
int make_tmap_16(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint64_t ld,
                 uint32_t box_rows, bool bf16);

}  // namespace afq

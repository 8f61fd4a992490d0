// Mixed-precision (16-bit tcgen05) path: tensor maps, workspace layout, one-time operand
// preparation, the per-walker Taylor kernel, GEMM launches and the test hook.
#include <stdio.h>
#include <string.h>

#include "afq_mixed_kernels.cuh"
#include "afq_prof.cuh"
#include "afq_prop_fused.cuh"
#include "afq_prop_wide.cuh"

namespace afq {

// ---- tensor maps ----------------------------------------------------------------------

typedef CUresult (*PFN_tmapEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                         const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                         const cuuint32_t*, CUtensorMapInterleave,
                                         CUtensorMapSwizzle, CUtensorMapL2promotion,
                                         CUtensorMapFloatOOBfill);

static PFN_tmapEncodeTiled encode_fn() {
  static PFN_tmapEncodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_tmapEncodeTiled>(p);
  }
  return fn;
}

int make_tmap_16(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint64_t ld,
                 uint32_t box_rows, bool bf16) {
  PFN_tmapEncodeTiled enc = encode_fn();
  if (!enc) {
    afq_set_error("cuTensorMapEncodeTiled unavailable");
    return -3;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 2) % 16 || box_rows < 1 || box_rows > 256) {
    afq_set_error("tensor map: base/stride must be 16-byte aligned, box rows in [1,256]");
    return -1;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {ld * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                   const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    afq_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return -3;
  }
  return 0;
}

static int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    afq_set_error("%s: %s", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

#define TC_CHECK(x)    \
  do {                 \
    int _e = (x);      \
    if (_e) return _e; \
  } while (0)

// drain > 0: K tiles per truncated accumulation run (see afq_gemm.cuh); needs 3 bn <= 512
template <int BNMAX, int STAGES, class Epi>
static int launch_gemm(int cls, const GemmMaps& maps, int nterms, int k_tiles, int m_tiles, int n_tiles,
                       int bn, bool bf16, const typename Epi::Params& ep, int* status,
                       cudaStream_t st, int a_row0 = 0, int drain = 0) {
  if (bn % 16 || bn < 16 || bn > BNMAX || (drain && 3 * bn > 512)) {
    afq_set_error("gemm: bn %d invalid", bn);
    return -1;
  }
  constexpr int smem = gemm_smem_bytes<BNMAX, STAGES, Epi>();
  static_assert(smem <= 232448, "shared memory");
  auto kfn = k_gemm_tc<BNMAX, STAGES, Epi>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  {
    ProfScope _ps(cls, st);
    kfn<<<dim3(n_tiles, m_tiles), kGemmThreads, smem, st>>>(
        maps, nterms, k_tiles, bn, a_row0, drain, ptx::idesc_f16(128, bn, bf16 ? 1 : 0), ep, status);
  }
  return launch_check("gemm_tc");
}

// persistent split-precision GEMM (afq_gemm_split.cuh): one CTA per SM, at most one per tile.
// With two or more M tiles the tiles go to CTA pairs (clusters of two, one 256-row MMA over
// both SMs, each CTA loading its own half of B); the grid is then twice the number of
// co-resident pairs, or of tiles if fewer. split_pairs(0) keeps the single-CTA kernel.
static int g_split_pairs = 1;

template <class Epi>
static int launch_split(int cls, const SplitMaps& maps, SplitArgs g, int num_sms,
                        const typename Epi::Params& ep, int* status, cudaStream_t st) {
  const int ntiles = g.m_tiles * g.n_tiles * g.k_splits;
  if (ntiles < 1 || g.k_tiles < 1 || g.drain < 1 || g.k_splits < 1 || g.k_splits > g.k_tiles) {
    afq_set_error("split gemm: bad sizes");
    return -1;
  }
  const bool bf16 = ((g.idesc >> 7) & 1u) != 0;
  if (g_split_pairs && g.m_tiles >= 2) {
    auto kfn = k_gemm_split<Epi, 2>;
    cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, kSplitSmem);
    g.idesc = ptx::idesc_f16(256, kSplitBN, bf16 ? 1 : 0);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kSplitThreads);
    cfg.dynamicSmemBytes = kSplitSmem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(num_sms - (num_sms & 1));
    int maxc = 0;
    if (cudaOccupancyMaxActiveClusters(&maxc, kfn, &cfg) != cudaSuccess || maxc < 1) {
      cudaGetLastError();
      maxc = num_sms / 2;
    }
    const int pair_tiles = (g.m_tiles + 1) / 2 * g.n_tiles * g.k_splits;
    const int npairs = pair_tiles < maxc ? pair_tiles : maxc;
    cfg.gridDim = dim3(2 * npairs);
    cudaError_t e;
    {
      ProfScope _ps(cls, st);
      e = cudaLaunchKernelEx(&cfg, kfn, maps, g, ep, status);
    }
    if (e != cudaSuccess) {
      afq_set_error("gemm_split (CTA pairs): %s", cudaGetErrorString(e));
      return (int)e;
    }
    return launch_check("gemm_split");
  }
  auto kfn = k_gemm_split<Epi, 1>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, kSplitSmem);
  const int grid = ntiles < num_sms ? ntiles : num_sms;
  {
    ProfScope _ps(cls, st);
    kfn<<<grid, kSplitThreads, kSplitSmem, st>>>(maps, g, ep, status);
  }
  return launch_check("gemm_split");
}

// K splits of a split GEMM over m_tiles x n_tiles output tiles (128 x 256) and k_tiles K
// tiles: the count minimising (tile rounds) x (K tiles per split) over the CTAs, or CTA
// pairs when the launch takes that form; ties go to fewer partials
static int choose_ksplit(int m_tiles, int n_tiles, int k_tiles, int sms) {
  const bool pairs = g_split_pairs && m_tiles >= 2;
  const int workers = pairs ? sms / 2 : sms, units = (pairs ? (m_tiles + 1) / 2 : m_tiles) * n_tiles;
  int best = 1;
  long best_cost = -1;
  for (int ks = 1; ks <= (k_tiles / 4 > 1 ? k_tiles / 4 : 1); ++ks) {
    const long rounds = ((long)units * ks + workers - 1) / workers;
    const long cost = rounds * ((k_tiles + ks - 1) / ks);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = ks;
    }
  }
  return best;
}

// ======================================================================================
// Taylor kernel (propagation.py:76-90): per walker slab, T_0 = W1 (B operand from the
// first exp_h1 product), T_m = V T_{m-1} / m on the tensor cores with V = [Vr | Vi] held in
// shared memory, acc = sum_m T_m in FP32 registers. The first `split` products use
// V_hi T_hi + V_hi T_lo + V_lo T_hi. Writes acc as the B operand of the last exp_h1 product.
//
// Persistent: one CTA per SM loops over the walkers of the chunk. 4 * NT / CW warps: warp w
// reads TMEM lanes 32*(w%4).. (thread <-> orbital row p) and owns the CW output columns
// CW*(w/4).. (CW / 2 orbitals), so the per-product epilogue (TMEM readout, Taylor sum, next
// B operand) is spread over several warps per lane quadrant. As soon as the last product's MMAs of a
// walker have completed, the TMA loads of the next walker's V and T_0 are issued, so they
// overlap that walker's last epilogue and its output.
// Each K tile of V_hi T_hi, and each correction product, accumulates in its own 64-column
// TMEM region (the tensor core truncates when it accumulates), summed with round-to-nearest.
// ======================================================================================

struct TaylorDev {
  int n, o, nq, NT, R, nk, nterms, split, bf16, w0, nwc;
  uint16_t* acc_hi;
  uint16_t* acc_lo;
};

constexpr int kTaylorDrain = 2;  // K tiles accumulated per TMEM region of the main product
// TMEM regions read per product: the main product's (K <= 256: at most 4 K tiles) + 2 corrections
constexpr int kTaylorRegions = (4 + kTaylorDrain - 1) / kTaylorDrain + 2;
constexpr int kTaylorCW = 16;  // B-operand columns per warp of the epilogue (8 or 16; 16 measured faster)
constexpr int kTaylorMaxThreads = 128 * 64 / kTaylorCW;  // NT <= 64

static inline size_t taylor_smem(int nq, int NT, bool lo) {
  const int KT = 2 * nq / 64;
  return 1024 + (size_t)KT * 128 * 128 * (lo ? 2 : 1) + (size_t)KT * NT * 128 * 2 + 64;
}

template <int MAXT, int CW>
__global__ void __launch_bounds__(MAXT, 1)
    k_taylor_tc(const __grid_constant__ CUtensorMap mv_hi, const __grid_constant__ CUtensorMap mv_lo,
                const __grid_constant__ CUtensorMap mt_hi, const __grid_constant__ CUtensorMap mt_lo,
                const TaylorDev td, int* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int KT = 2 * td.nq / 64;
  const bool has_lo = td.split > 0;
  const uint32_t VT = 128 * 128;    // bytes per V k-tile
  const uint32_t BT = td.NT * 128;  // bytes per B k-tile
  unsigned char* Vh = smem;
  unsigned char* Vl = Vh + KT * VT;
  unsigned char* Bh = Vl + (has_lo ? KT * VT : 0);
  unsigned char* Bl = Bh + KT * BT;
  uint64_t* bars = reinterpret_cast<uint64_t*>(Bl + KT * BT);
  uint64_t* ld_bar = bars;
  uint64_t* mma_bar = bars + 1;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3, part = warp >> 2;
  const int KR = (KT + kTaylorDrain - 1) / kTaylorDrain;  // TMEM regions of the main product
  const uint32_t tcols = gemm_tmem_cols((KR + 2) * 64);
  const bool bf = td.bf16 != 0;
  const uint32_t ld_bytes = KT * VT * (has_lo ? 2 : 1) + KT * BT * 2;
  bool ok = true;

  if (tid == 0) {
    ptx::mbar_init(ld_bar, 1);
    ptx::mbar_init(mma_bar, 1);
    ptx::fence_mbar_init();
  }
  if (warp == 0) {
    ptx::tmem_alloc(tmem_holder, tcols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  auto issue_loads = [&](int wl) {
    const int wg = td.w0 + wl;
    ptx::mbar_expect_tx(ld_bar, ld_bytes);
    for (int kt = 0; kt < KT; ++kt) {
      ptx::tma_load_2d(Vh + kt * VT, &mv_hi, ld_bar, kt * 64, wl * 128);
      if (has_lo) ptx::tma_load_2d(Vl + kt * VT, &mv_lo, ld_bar, kt * 64, wl * 128);
      ptx::tma_load_2d(Bh + kt * BT, &mt_hi, ld_bar, kt * 64, wg * td.NT);
      ptx::tma_load_2d(Bl + kt * BT, &mt_lo, ld_bar, kt * 64, wg * td.NT);
    }
  };

  const int p = q * 32 + lane;
  const bool prow = p < td.n;
  const int o2 = 2 * td.o;
  const int c_begin = part * CW;  // this thread's CW columns (orbitals k = c_begin/2 ..)
  const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
  const uint32_t idesc = ptx::idesc_f16(128, td.NT, bf ? 1 : 0);
  const uint32_t sVh = ptx::smem_u32(Vh), sVl = ptx::smem_u32(Vl), sBh = ptx::smem_u32(Bh),
                 sBl = ptx::smem_u32(Bl);
  const int kt0 = p / 64, kc0 = p % 64;                      // K = p
  const int kt1 = (td.nq + p) / 64, kc1 = (td.nq + p) % 64;  // K = nq + p

  if (tid == 0 && blockIdx.x < td.nwc) issue_loads(blockIdx.x);
  int iter = 0, prod = 0;
  for (int wl = blockIdx.x; wl < td.nwc && ok; wl += gridDim.x, ++iter) {
    if (!ptx::mbar_wait(ld_bar, iter & 1)) ok = false;
    float acc[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) {
      const int r = c_begin + j;
      if (r < o2 && prow) {
        const uint32_t off = kt0 * BT + sw128(r, kc0);
        acc[j] = h2f(*reinterpret_cast<const uint16_t*>(Bh + off), bf) +
                 h2f(*reinterpret_cast<const uint16_t*>(Bl + off), bf);
      } else {
        acc[j] = 0.f;
      }
    }
    if (td.nterms <= 1) {  // no products: T_0 alone; the operands are free after the read above
      __syncthreads();
      if (tid == 0 && wl + gridDim.x < td.nwc) issue_loads(wl + gridDim.x);
    }
    for (int m = 1; m < td.nterms; ++m, ++prod) {
      // every thread has read the B operand (acc init or previous product) before the MMAs
      ptx::tc_fence_before();
      __syncthreads();
      if (tid == 0 && ok) {
        ptx::tc_fence_after();
        const int ngroups = (m <= td.split) ? 3 : 1;
        for (int gi = 0; gi < ngroups; ++gi) {
          const uint32_t va = gi == 2 ? sVl : sVh;
          const uint32_t ba = gi == 1 ? sBl : sBh;
          for (int kt = 0; kt < KT; ++kt) {
            // region: one per K tile for the main product, one per correction product
            const uint32_t dreg = tmem + (uint32_t)(64 * (gi == 0 ? kt / kTaylorDrain : KR + gi - 1));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              ptx::mma_f16(dreg, ptx::desc_kmajor_sw128(va + kt * VT + kk * 32),
                           ptx::desc_kmajor_sw128(ba + kt * BT + kk * 32), idesc,
                           (kk > 0 || (gi == 0 ? kt % kTaylorDrain != 0 : kt > 0)) ? 1u : 0u);
          }
        }
        ptx::mma_commit(mma_bar);
      }
      if (ok && !ptx::mbar_wait(mma_bar, prod & 1)) ok = false;
      ok = __syncthreads_and(ok);
      if (!ok) break;
      ptx::tc_fence_after();
      const bool last = m + 1 == td.nterms;
      // the smem operands are free once the last product's MMAs are done: fetch the next walker
      if (last && tid == 0 && wl + gridDim.x < td.nwc) issue_loads(wl + gridDim.x);
      const int nreg = KR + ((m <= td.split) ? 2 : 0);
      const float invm = 1.0f / (float)m;
      const bool lo_next = (m + 1) <= td.split;
      {
        constexpr int cc = 0;
        const int c0 = c_begin;
        if (c0 < td.NT) {
          float dd[CW];
#pragma unroll
          for (int j = 0; j < CW; ++j) dd[j] = 0.f;
#pragma unroll
          for (int g0 = 0; g0 < kTaylorRegions; g0 += 2) {  // regions in groups of two
            if (g0 < nreg) {
              float v[2][CW];
#pragma unroll
              for (int rg = 0; rg < 2; ++rg)
                if (g0 + rg < nreg) ptx::tmem_ldp<CW>(lane_base + (uint32_t)(64 * (g0 + rg) + c0), v[rg]);
              ptx::tmem_ld_wait();
#pragma unroll
              for (int j = 0; j < CW; ++j) {
#pragma unroll
                for (int rg = 0; rg < 2; ++rg)
                  if (g0 + rg < nreg) dd[j] += v[rg][j];
              }
            }
          }
#pragma unroll
          for (int j = 0; j < CW; ++j) {
            dd[j] = (c0 + j < o2) ? dd[j] * invm : 0.f;
            acc[cc + j] += dd[j];
          }
          if (!last && prow) {
#pragma unroll
            for (int kk = 0; kk < CW / 2; ++kk) {
              const int k = c0 / 2 + kk;
              if (k < td.o) {
                const float tr = dd[2 * kk], ti = dd[2 * kk + 1];
                uint16_t hr, lr, hi_, li, hni, lni;
                split16(tr, bf, hr, lr);
                split16(ti, bf, hi_, li);
                split16(-ti, bf, hni, lni);
                const uint32_t a0 = kt0 * BT + sw128(2 * k, kc0), a1 = kt1 * BT + sw128(2 * k, kc1);
                const uint32_t b0 = kt0 * BT + sw128(2 * k + 1, kc0), b1 = kt1 * BT + sw128(2 * k + 1, kc1);
                *reinterpret_cast<uint16_t*>(Bh + a0) = hr;
                *reinterpret_cast<uint16_t*>(Bh + a1) = hni;
                *reinterpret_cast<uint16_t*>(Bh + b0) = hi_;
                *reinterpret_cast<uint16_t*>(Bh + b1) = hr;
                if (lo_next) {
                  *reinterpret_cast<uint16_t*>(Bl + a0) = lr;
                  *reinterpret_cast<uint16_t*>(Bl + a1) = lni;
                  *reinterpret_cast<uint16_t*>(Bl + b0) = li;
                  *reinterpret_cast<uint16_t*>(Bl + b1) = lr;
                }
              }
            }
          }
        }
      }
      if (!last) ptx::fence_proxy_async();  // generic-proxy smem writes -> async-proxy MMA reads
    }
    if (!ok) break;
    if (prow) {
      const int wg = td.w0 + wl;
      uint16_t* oh = td.acc_hi + (size_t)wg * td.R * td.nk + p;
      uint16_t* ol = td.acc_lo + (size_t)wg * td.R * td.nk + p;
#pragma unroll
      for (int j = 0; j < CW; ++j) {
        const int r = c_begin + j;
        if (r < o2) {
          uint16_t h, l;
          split16(acc[j], bf, h, l);
          oh[(size_t)r * td.nk] = h;
          ol[(size_t)r * td.nk] = l;
        }
      }
    }
  }
  // never leave a copy in flight (a walker whose loads were issued but that was not reached)
  if (tid == 0 && !ok) ptx::mbar_wait(ld_bar, iter & 1);
  if (!ok) atomicOr(status, 2);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, tcols);
  }
}

// ======================================================================================
// One-time operand preparation
// ======================================================================================

__global__ void k_to_f32(const double* __restrict__ src, float* __restrict__ dst, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

// 2^-e_g with 2^e_g max|src[g][:]| in (0.5, 1]
__global__ void k_row_scale(const double* __restrict__ src, int len, float* __restrict__ inv) {
  __shared__ float mx_sh[32];
  const int g = blockIdx.x;
  float mx = 0.f;
  for (int i = threadIdx.x; i < len; i += blockDim.x) mx = fmaxf(mx, fabsf((float)src[(size_t)g * len + i]));
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) mx_sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    float v = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) v = fmaxf(v, mx_sh[i]);
    inv[g] = 1.0f / pow2_scale(v);
  }
}

// rows g of src [nchol][len] -> dst[g][ld] (hi/lo) scaled by 1/inv[g]
__global__ void k_prep_rows_scaled(const double* __restrict__ src, int len, int ld, int bf16,
                                   const float* __restrict__ inv, uint16_t* __restrict__ hi,
                                   uint16_t* __restrict__ lo) {
  const int g = blockIdx.x;
  const double scl = 1.0 / (double)inv[g];
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    uint16_t h, l;
    split16((float)(src[(size_t)g * len + i] * scl), bf16 != 0, h, l);
    hi[(size_t)g * ld + i] = h;
    lo[(size_t)g * ld + i] = l;
  }
}

// exchange matrix: V[(i,p),(k,q)] = sum_g rc[g][i*n+p] rc[g][k*n+q] in FP64, written as
// U[(i,q),(k,p)] (FP32 scratch, row stride ldk); *amax <- max |U| (float bits, non-negative)
__global__ void k_prep_u(const double* __restrict__ rc, int nchol, int kb, int n, int ldk,
                         float* __restrict__ u, unsigned* __restrict__ amax) {
  __shared__ double xa[16][33], xb[16][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  double acc[4] = {0, 0, 0, 0};
  for (int g0 = 0; g0 < nchol; g0 += 16) {
    for (int e = threadIdx.x; e < 16 * 32; e += 256) {
      const int gg = e / 32, cc = e % 32, g = g0 + gg;
      xa[gg][cc] = (g < nchol && r0 + cc < kb) ? rc[(size_t)g * kb + r0 + cc] : 0.0;
      xb[gg][cc] = (g < nchol && c0 + cc < kb) ? rc[(size_t)g * kb + c0 + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int gg = 0; gg < 16; ++gg) {
      const double bv = xb[gg][tx];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] = fma(xa[gg][ty + 8 * j], bv, acc[j]);
    }
    __syncthreads();
  }
  float mx = 0.f;
  for (int j = 0; j < 4; ++j) {
    const int vr = r0 + ty + 8 * j, vc = c0 + tx;  // V row (i,p), V column (k,q)
    if (vr < kb && vc < kb) {
      const int i = vr / n, pp = vr % n, k = vc / n, qq = vc % n;
      const float val = (float)acc[j];
      u[(size_t)(i * n + qq) * ldk + (k * n + pp)] = val;
      mx = fmaxf(mx, fabsf(val));
    }
  }
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if (tx == 0) atomicMax(amax, __float_as_uint(mx));
}

// U (FP32 scratch) * 2^e -> hi/lo, 2^e from the max
__global__ void k_split_u(const float* __restrict__ u, long n, const unsigned* __restrict__ amax, int bf16,
                          uint16_t* __restrict__ hi, uint16_t* __restrict__ lo) {
  const float scl = pow2_scale(__uint_as_float(*amax));
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    uint16_t h, l;
    split16(u[i] * scl, bf16 != 0, h, l);
    hi[i] = h;
    lo[i] = l;
  }
}

// ---- exchange matrix on the tensor cores (large systems) --------------------------------
// U[(i,q),(k,p)] = sum_g rc[g][i,p] rc[g][k,q] is a permutation of X X^T with
// X[(i,p)][g] = rc[g][i n + p]: X is split into fp16 hi / lo planes under one power-of-two
// scale, X X^T runs on the persistent split GEMM (three products, drained FP32 accumulation)
// and the epilogue writes U permuted and unscaled into the FP32 scratch with its max |U|.
constexpr int kExchangeTensorMinKb = 4096;  // below this the FP64 build (k_prep_u) is kept

// *amax <- max |src| as float bits (non-negative floats order like their bits)
__global__ void k_amax_f64(const double* __restrict__ src, long n, unsigned* __restrict__ amax) {
  float mx = 0.f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    mx = fmaxf(mx, fabsf((float)src[i]));
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) atomicMax(amax, __float_as_uint(mx));
}

// X[(i,p)][g] (hi / lo, row stride ldg) from rc [nchol][kb] scaled by pow2_scale(*amax_x);
// 32 x 32 tiles through shared memory
__global__ void k_prep_xu(const double* __restrict__ rc, int nchol, int kb, int ldg, const unsigned* amax_x,
                          int bf16, uint16_t* __restrict__ hi, uint16_t* __restrict__ lo) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const float scl = pow2_scale(__uint_as_float(*amax_x));
  for (int r = ty; r < 32; r += 8) {
    const int g = g0 + r, k = r0 + tx;
    tile[r][tx] = (g < nchol && k < kb) ? (float)(rc[(size_t)g * kb + k] * (double)scl) : 0.f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int k = r0 + r, g = g0 + tx;
    if (k < kb && g < nchol) {
      uint16_t h, l;
      split16(tile[tx][r], bf16 != 0, h, l);
      hi[(size_t)k * ldg + g] = h;
      lo[(size_t)k * ldg + g] = l;
    }
  }
}

// split-GEMM epilogue for U: D[(i,p)][(k,q)] -> u[(i n + q) ldk + k n + p] / scale^2
struct SplitStoreU {
  static constexpr bool kWarpStore = false;
  struct Params {
    float* u;
    int kb, n, ldk;
    const unsigned* amax_x;
    unsigned* amax_u;
  };
  __device__ __forceinline__ static void store(const Params& p, int row, int col0, const float* v, int) {
    if (row >= p.kb) return;
    const float s = pow2_scale(__uint_as_float(*p.amax_x)), unscale = 1.0f / (s * s);
    const int i = row / p.n, pp = row - i * p.n;
    int k = col0 / p.n, q = col0 - k * p.n;
    float mx = 0.f;
#pragma unroll 4
    for (int j = 0; j < 128; ++j) {
      if (col0 + j < p.kb) {
        const float val = v[j] * unscale;
        p.u[(size_t)(i * p.n + q) * p.ldk + k * p.n + pp] = val;
        mx = fmaxf(mx, fabsf(val));
      }
      if (++q == p.n) {
        q = 0;
        ++k;
      }
    }
    atomicMax(p.amax_u, __float_as_uint(mx));
  }
};

// vhs B operand: chol [nchol][n*n] -> lop[(p*nq + q)][g], 32x32 tiles through shared memory
__global__ void k_prep_lop(const double* __restrict__ chol, int nchol, int n, int nq, int ldg, int bf16,
                           uint16_t* __restrict__ hi, uint16_t* __restrict__ lo) {
  __shared__ float tile[32][33];
  const int pq0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int g = g0 + r, pq = pq0 + tx;
    tile[r][tx] = (g < nchol && pq < n * n) ? (float)chol[(size_t)g * n * n + pq] : 0.f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int pq = pq0 + r, g = g0 + tx;
    if (pq < n * n && g < nchol) {
      const int pp = pq / n, qq = pq % n;
      uint16_t h, l;
      split16(tile[tx][r], bf16 != 0, h, l);
      hi[((size_t)pp * nq + qq) * ldg + g] = h;
      lo[((size_t)pp * nq + qq) * ldg + g] = l;
    }
  }
}

// kDiagChol: the diagonal of every Cholesky vector in FP32 ([nchol][n]); an off-diagonal
// nonzero sets status bit 4 (the caller promised diagonal vectors). CTA per vector.
__global__ void k_prep_diag(const double* __restrict__ chol, int n, float* __restrict__ d, int* status) {
  const int g = blockIdx.x;
  const double* L = chol + (size_t)g * n * n;
  bool off = false;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int p = e / n, q = e % n;
    if (p == q) d[(size_t)g * n + p] = (float)L[e];
    else if (L[e] != 0.0) off = true;
  }
  if (off) atomicOr(status, 4);
}

// exp(vhs) W1 for diagonal Cholesky vectors (propagation.py:67-92 with a diagonal V):
// vhs = i sqrt(dt) diag(v), v_p = sum_g xt_g d_g[p], so sum_m vhs^m W1 / m! scales row p of
// W1 by the Taylor polynomial of i sqrt(dt) v_p (Horner form). Reads the first exp_h1
// product's Taylor operand (t0: row 2k = [Tr | -Ti], row 2k+1 = [Ti | Tr]) and writes the
// last product's operand (acc: rows 2k + re/im, cols p), both fp16 hi + lo. CTA per
// (walker, slab); HBM-bound.
struct TaylorDiag {
  const float* dchol;
  const uint16_t *xt_hi, *xt_lo;
  const uint16_t *t0_hi[2], *t0_lo[2];
  uint16_t *acc_hi[2], *acc_lo[2];
  int nchol, ldg, n, o[2], nq, NT[2], R[2], nk, nterms, bf16;
  float sqdt;
};

constexpr int kDiagSplit = 8;  // partial sums over g per orbital (256 threads: 8 x 32 orbitals)

__global__ void __launch_bounds__(256) k_taylor_diag(const TaylorDiag td) {
  __shared__ float2 poly[128];
  __shared__ float2 part[kDiagSplit][128];
  const int w = blockIdx.x, s = blockIdx.y, n = td.n, tid = threadIdx.x;
  const bool bf = td.bf16 != 0;
  // v_p = sum_g xt_g d_g[p]: thread (j, lane) takes orbitals lane, lane + 32, ... and every
  // kDiagSplit-th g from j; xt_g is a broadcast load, d_g[p] coalesced over the warp
  {
    const int j = tid >> 5, lane = tid & 31;
    const size_t r0 = (size_t)(2 * w) * td.ldg, r1 = r0 + td.ldg;
    for (int p0 = 0; p0 < n; p0 += 32) {
      const int p = p0 + lane;
      float vr = 0.f, vi = 0.f;
      if (p < n)
        for (int g = j; g < td.nchol; g += kDiagSplit) {
          const float dg = td.dchol[(size_t)g * n + p];
          vr = fmaf(h2f(td.xt_hi[r0 + g], bf) + h2f(td.xt_lo[r0 + g], bf), dg, vr);
          vi = fmaf(h2f(td.xt_hi[r1 + g], bf) + h2f(td.xt_lo[r1 + g], bf), dg, vi);
        }
      if (p < n) part[j][p] = make_float2(vr, vi);
    }
  }
  __syncthreads();
  for (int p = tid; p < n; p += blockDim.x) {
    float vr = 0.f, vi = 0.f;
    for (int j = 0; j < kDiagSplit; ++j) {
      vr += part[j][p].x;
      vi += part[j][p].y;
    }
    const float ar = -td.sqdt * vi, ai = td.sqdt * vr;  // i sqrt(dt) v
    float pr = 1.f, pi = 0.f;
    for (int m = td.nterms - 1; m >= 1; --m) {  // P <- 1 + a P / m
      const float inv = 1.f / (float)m;
      const float qr = (ar * pr - ai * pi) * inv, qi = (ar * pi + ai * pr) * inv;
      pr = 1.f + qr;
      pi = qi;
    }
    poly[p] = make_float2(pr, pi);
  }
  __syncthreads();
  const int o = td.o[s];
  const size_t tb = (size_t)w * td.NT[s] * 2 * td.nq, ab = (size_t)w * td.R[s] * td.nk;
  // four orbitals per thread: 8-byte loads and stores (rows start on 8-byte boundaries: the
  // row pitches 2 nq and nk are multiples of 4 elements); a partial last group goes one by one
  const int ng = (n + 3) / 4;
  for (int e = tid; e < o * ng; e += blockDim.x) {
    const int k = e / ng, p0 = (e - k * ng) * 4;
    const size_t ir = tb + (size_t)(2 * k) * 2 * td.nq + p0, ii = ir + 2 * td.nq;
    const size_t ar = ab + (size_t)(2 * k) * td.nk + p0, ai = ar + td.nk;
    if (p0 + 4 <= n) {
      const uint2 vhr = *reinterpret_cast<const uint2*>(td.t0_hi[s] + ir);
      const uint2 vlr = *reinterpret_cast<const uint2*>(td.t0_lo[s] + ir);
      const uint2 vhi = *reinterpret_cast<const uint2*>(td.t0_hi[s] + ii);
      const uint2 vli = *reinterpret_cast<const uint2*>(td.t0_lo[s] + ii);
      uint32_t ohr[2] = {0, 0}, olr[2] = {0, 0}, ohi[2] = {0, 0}, oli[2] = {0, 0};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int sh = 16 * (j & 1);
        const uint32_t whr = j < 2 ? vhr.x : vhr.y, wlr = j < 2 ? vlr.x : vlr.y;
        const uint32_t whi = j < 2 ? vhi.x : vhi.y, wli = j < 2 ? vli.x : vli.y;
        const float tr = h2f((uint16_t)(whr >> sh), bf) + h2f((uint16_t)(wlr >> sh), bf);
        const float ti = h2f((uint16_t)(whi >> sh), bf) + h2f((uint16_t)(wli >> sh), bf);
        const float2 c = poly[p0 + j];
        uint16_t h, l;
        split16(c.x * tr - c.y * ti, bf, h, l);
        ohr[j >> 1] |= (uint32_t)h << sh;
        olr[j >> 1] |= (uint32_t)l << sh;
        split16(c.x * ti + c.y * tr, bf, h, l);
        ohi[j >> 1] |= (uint32_t)h << sh;
        oli[j >> 1] |= (uint32_t)l << sh;
      }
      *reinterpret_cast<uint2*>(td.acc_hi[s] + ar) = make_uint2(ohr[0], ohr[1]);
      *reinterpret_cast<uint2*>(td.acc_lo[s] + ar) = make_uint2(olr[0], olr[1]);
      *reinterpret_cast<uint2*>(td.acc_hi[s] + ai) = make_uint2(ohi[0], ohi[1]);
      *reinterpret_cast<uint2*>(td.acc_lo[s] + ai) = make_uint2(oli[0], oli[1]);
    } else {
      for (int j = 0; j < n - p0; ++j) {
        const float tr = h2f(td.t0_hi[s][ir + j], bf) + h2f(td.t0_lo[s][ir + j], bf);
        const float ti = h2f(td.t0_hi[s][ii + j], bf) + h2f(td.t0_lo[s][ii + j], bf);
        const float2 c = poly[p0 + j];
        uint16_t h, l;
        split16(c.x * tr - c.y * ti, bf, h, l);
        td.acc_hi[s][ar + j] = h;
        td.acc_lo[s][ar + j] = l;
        split16(c.x * ti + c.y * tr, bf, h, l);
        td.acc_hi[s][ai + j] = h;
        td.acc_lo[s][ai + j] = l;
      }
    }
  }
}

// exp_h1 A operand: E - I -> [128][nk]
__global__ void k_prep_eop(const double* __restrict__ e, int n, int nk, int bf16, uint16_t* __restrict__ hi,
                           uint16_t* __restrict__ lo) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * n; i += gridDim.x * blockDim.x) {
    const int p = i / n, q = i % n;
    const double v = e[i] - (p == q ? 1.0 : 0.0);
    uint16_t h, l;
    split16((float)v, bf16 != 0, h, l);
    hi[(size_t)p * nk + q] = h;
    lo[(size_t)p * nk + q] = l;
  }
}

// local energy from c_g and exchange partials (wavefunctions.py:540, 735-741)
__global__ void k_energy_final_mixed(int nw, int nchol, int nblk, int mt0, int mt1, int mode, double h0,
                                     const double2* __restrict__ c_out, const double2* __restrict__ exc,
                                     const double2* __restrict__ ene1, double2* __restrict__ out) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  double a[5][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
  const double2* c0 = c_out + (size_t)w * nchol;
  const double2* c1 = c_out + ((size_t)nw + w) * nchol;
  for (int g = threadIdx.x; g < nchol; g += blockDim.x) {
    const double2 u = c0[g];
    const double2 uu = cmul(u, u);
    a[0][0] += uu.x;
    a[0][1] += uu.y;
    if (nblk == 2) {
      const double2 d = c1[g];
      const double2 dd = cmul(d, d), ud = cmul(u, d);
      a[1][0] += dd.x;
      a[1][1] += dd.y;
      a[2][0] += ud.x;
      a[2][1] += ud.y;
    }
  }
  for (int t = threadIdx.x; t < mt0; t += blockDim.x) {
    const double2 e = exc[(size_t)w * mt0 + t];
    a[3][0] += e.x;
    a[3][1] += e.y;
  }
  if (nblk == 2)
    for (int t = threadIdx.x; t < mt1; t += blockDim.x) {
      const double2 e = exc[(size_t)nw * mt0 + (size_t)w * mt1 + t];
      a[4][0] += e.x;
      a[4][1] += e.y;
    }
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 2; ++j) a[i][j] = block_sum(a[i][j], red);
  if (threadIdx.x == 0) {
    double2 e1 = ene1[w], e2;
    const double2 s0 = c2(a[0][0], a[0][1]), s1 = c2(a[1][0], a[1][1]), s2 = c2(a[2][0], a[2][1]);
    const double2 x0 = c2(a[3][0], a[3][1]), x1 = c2(a[4][0], a[4][1]);
    if (mode == 0) {
      e2 = csub(cscale(s0, 2.0), x0);
      e1 = cscale(e1, 2.0);
    } else if (mode == 1) {
      e2 = csub(s0, x0);
    } else {
      e2 = cscale(csub(cadd(cadd(s0, s1), cscale(s2, 2.0)), cadd(x0, x1)), 0.5);
    }
    out[w] = cadd(cadd(e2, e1), c2(h0, 0.0));
  }
}

// ======================================================================================
// host side
// ======================================================================================

namespace {

struct TcLayout {
  size_t off = 0;
  size_t take(size_t b) {
    size_t o = off;
    off += (b + 1023) & ~(size_t)1023;
    return o;
  }
};

inline int rup(int x, int m) { return (x + m - 1) / m * m; }

// rows per walker R = 2o rounded up to a multiple of 16 (each walker is a whole number of
// 16-column TMEM chunks in the exp_h1 products), walkers per N tile wpt with R * wpt <= 256
void walker_rows(int o, int* R, int* wpt) {
  const int r = rup(2 * o, 16);
  int w = 256 / r;
  if (w < 1) w = 1;
  *R = r;
  *wpt = w;
}

struct Plan {
  TcState t;
  size_t total;
  size_t o_rc_fb[2], o_rc_inv, o_lop[2], o_eop[2][2], o_u[2][2], o_rcb[2][2], o_rcb_inv[2], o_utmp;
  size_t o_gfb[2], o_xt[2], o_vbuf[2], o_wt[2][2], o_acc[2][2], o_t0[2][2], o_gblk[2][2];
  size_t o_fbpart;
  size_t o_ginv, o_ene1, o_pshift, o_pfbt, o_cout, o_exc, o_status, o_amax, o_trial32[2], o_rh1[2];
  size_t o_dchol, o_xu[2];
};

int make_plan(const afq_ctx_dev& c, int nwc, int32_t cfg, Plan* P) {
  TcState& t = P->t;
  memset(P, 0, sizeof(*P));
  if (cfg == 0) cfg = kMixedDefault;
  t.cfg = cfg;
  t.bf16 = (cfg & kUseBf16) != 0;
  t.n = c.norb;
  if (t.n > 256) {
    afq_set_error("mixed precision path: norb <= 256");
    return -2;
  }
  // norb > 128: two 128-row M tiles in the propagation kernel (k_prop_wide)
  t.wide = t.n > 128;
  if (t.wide && (cfg & (kLegacyTaylor | kDiagChol))) {
    afq_set_error("mixed precision path: norb > 128 runs on the streamed propagation kernel only "
                  "(no separate Taylor kernel, no diagonal-vector path)");
    return -2;
  }
  t.nq = t.n <= 64 ? 64 : t.n <= 128 ? 128 : 256;
  t.mr = t.wide ? kWideMR : 128;
  t.nk = rup(t.n, 8);
  t.nw = c.nw;
  t.nwc = nwc;
  t.nslab = c.nslab;
  t.nblk = c.nspin_g;
  t.kfb = c.ktot;
  t.ldfb = rup(t.kfb, 8);
  t.ldg = rup(c.nchol, 8);
  for (int s = 0; s < t.nslab; ++s) {
    t.o_slab[s] = c.kslab[s];
    walker_rows(t.o_slab[s], &t.R[s], &t.wpt[s]);
    t.bn_w[s] = t.R[s] * t.wpt[s];
    t.NT[s] = rup(2 * t.o_slab[s], 16);
    if (t.NT[s] > (t.wide ? 80 : 64)) {
      afq_set_error("mixed precision path: at most %d electrons per spin%s", t.wide ? 40 : 32,
                    t.wide ? "" : " for norb <= 128");
      return -2;
    }
  }
  {  // the fused propagation kernel takes every non-diagonal configuration it has room for
    int ntmax = 0;
    for (int s = 0; s < t.nslab; ++s) ntmax = t.NT[s] > ntmax ? t.NT[s] : ntmax;
    t.fused = !(cfg & (kLegacyTaylor | kDiagChol)) && t.n <= 128 && ntmax <= 16 * kPropMaxChains &&
              prop_fused_smem(t.nq, ntmax) <= 232448 && prop_tmem_cols(t.nq, ntmax) <= 512;
    // symmetric vectors: packed vhs columns, mirrored in the fused kernel
    t.sym = t.fused && (cfg & kSymChol) != 0;
    t.n_vcols = t.sym ? sym_total(t.n, t.nq) : t.n * t.nq;
  }
  size_t umax = 0;
  for (int b = 0; b < t.nblk; ++b) {
    t.o_blk[b] = c.gocc[b];
    t.kb[b] = t.o_blk[b] * t.n;
    t.ldkb[b] = rup(t.kb[b], 8);
    const size_t ub = (size_t)t.kb[b] * t.ldkb[b];
    if (ub > umax) umax = ub;
  }
  // force-bias tile width: the widest of 256/128/64 that still gives >= 148 CTAs
  {
    const int mtl = (2 * c.nw + 127) / 128;
    t.fb_bn = c.nchol >= 128 ? 128 : rup(c.nchol, 16);
    while (mtl * ((c.nchol + t.fb_bn - 1) / t.fb_bn) < 148) {
      const int next = rup(t.fb_bn / 2, 16);
      if (next < 64) break;
      t.fb_bn = next;
    }
    t.fb_ntiles = (c.nchol + t.fb_bn - 1) / t.fb_bn;
  }
  {  // force bias on the persistent split GEMM: enough K splits to cover the SMs
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
      sms = 148;
    cudaGetLastError();  // a host without a device leaves an error behind
    const int mt2 = (2 * c.nw + 127) / 128, nt2 = (c.nchol + kSplitBN - 1) / kSplitBN;
    const int kt = (t.kfb + 63) / 64;
    t.fb_ks = choose_ksplit(mt2, nt2, kt, sms);
    for (int b = 0; b < t.nblk; ++b) {  // exchange: Z = U . G on the split GEMM, K-split partials of exc
      t.z_ks[b] = choose_ksplit(mt2, (t.kb[b] + kSplitBN - 1) / kSplitBN, (t.kb[b] + 63) / 64, sms);
      t.mt_z[b] = t.z_ks[b] * ((t.kb[b] + 127) / 128);
    }
    t.fb_npad = nt2 * kSplitBN;
  }
  t.n_fb_terms = 1 + ((cfg & kFbDyn) ? 1 : 0) + ((cfg & kFbStat) ? 1 : 0);
  t.n_vhs_terms = 1 + ((cfg & kVhsDyn) ? 1 : 0) + ((cfg & kVhsStat) ? 1 : 0);
  t.n_e_terms = 1 + ((cfg & kExpDyn) ? 1 : 0) + ((cfg & kExpStat) ? 1 : 0);
  t.n_en_terms = 1 + ((cfg & kEneDyn) ? 1 : 0) + ((cfg & kEneStat) ? 1 : 0);
  t.taylor_split = (cfg >> kTaylorShift) & 7;
  {
    const int d = (cfg >> kDrainShift) & 7;
    t.drain = d == 0 ? kDrainDefault : d == 7 ? 0 : d;
  }
  TcLayout L;
  const size_t H = 2;  // bytes per 16-bit element
  for (int i = 0; i < 2; ++i) P->o_rc_fb[i] = L.take((size_t)c.nchol * t.ldfb * H);
  P->o_rc_inv = L.take((size_t)c.nchol * 4);
  for (int i = 0; i < 2; ++i) P->o_lop[i] = L.take((size_t)t.n * t.nq * t.ldg * H);
  for (int s = 0; s < t.nslab; ++s)
    for (int i = 0; i < 2; ++i) P->o_eop[s][i] = L.take((size_t)t.mr * t.nk * H);
  for (int b = 0; b < t.nblk; ++b) {
    for (int i = 0; i < 2; ++i) P->o_u[b][i] = L.take((size_t)t.kb[b] * t.ldkb[b] * H);
    if (t.nblk == 2) {
      for (int i = 0; i < 2; ++i) P->o_rcb[b][i] = L.take((size_t)c.nchol * t.ldkb[b] * H);
      P->o_rcb_inv[b] = L.take((size_t)c.nchol * 4);
    }
  }
  P->o_utmp = L.take(umax * 4);
  {  // X planes of the tensor-core exchange build (the largest block; blocks reuse them)
    int kbmax = 0;
    for (int b = 0; b < t.nblk; ++b) kbmax = t.kb[b] > kbmax ? t.kb[b] : kbmax;
    for (int i = 0; i < 2; ++i)
      P->o_xu[i] = L.take(kbmax > kExchangeTensorMinKb ? (size_t)kbmax * t.ldg * H : 256);
  }
  for (int i = 0; i < 2; ++i) P->o_gfb[i] = L.take((size_t)2 * t.nw * t.ldfb * H);
  for (int i = 0; i < 2; ++i) P->o_xt[i] = L.take((size_t)2 * t.nw * t.ldg * H);
  for (int i = 0; i < 2; ++i) P->o_vbuf[i] = L.take((size_t)nwc * t.mr * 2 * t.nq * H);
  for (int s = 0; s < t.nslab; ++s)
    for (int i = 0; i < 2; ++i) {
      P->o_wt[s][i] = L.take((size_t)t.nw * t.R[s] * t.nk * H);
      P->o_acc[s][i] = L.take((size_t)t.nw * t.R[s] * t.nk * H);
      P->o_t0[s][i] = L.take((size_t)t.nw * t.NT[s] * 2 * t.nq * H);
    }
  if (t.nblk == 2)
    for (int b = 0; b < t.nblk; ++b)
      for (int i = 0; i < 2; ++i) P->o_gblk[b][i] = L.take((size_t)2 * t.nw * t.ldkb[b] * H);
  P->o_ginv = L.take((size_t)t.nw * 4);
  P->o_ene1 = L.take((size_t)t.nw * 16);
  P->o_fbpart = L.take((size_t)t.fb_ks * ((2 * t.nw + 127) / 128 * 128) * t.fb_npad * 4);
  P->o_pshift = L.take((size_t)t.nw * t.fb_ntiles * 16);
  P->o_pfbt = L.take((size_t)t.nw * t.fb_ntiles * 16);
  P->o_cout = L.take((size_t)t.nblk * t.nw * c.nchol * 16);
  P->o_exc = L.take((size_t)t.nw * (t.mt_z[0] + t.mt_z[1]) * 16);
  P->o_status = L.take(256);
  P->o_amax = L.take(256);
  P->o_dchol = L.take((cfg & kDiagChol) ? (size_t)c.nchol * t.n * 4 : 256);
  for (int s = 0; s < 2; ++s) P->o_trial32[s] = L.take((size_t)t.n * 64 * 4);
  for (int b = 0; b < 2; ++b) P->o_rh1[b] = L.take((size_t)t.n * 64 * 4);
  P->total = L.off + 1024;
  return 0;
}

MixedDev mixed_dev(const TcState& t, const afq_ctx_dev& c) {
  MixedDev m;
  memset(&m, 0, sizeof(m));
  m.n = t.n;
  m.nq = t.nq;
  m.nk = t.nk;
  m.ldfb = t.ldfb;
  m.ldg = t.ldg;
  m.nw = t.nw;
  m.nchol = c.nchol;
  m.nslab = t.nslab;
  m.nblk = t.nblk;
  m.kfb = t.kfb;
  m.restricted_square = c.restricted_square;
  m.energy_mode = c.energy_mode;
  m.bf16 = t.bf16 ? 1 : 0;
  m.h0 = c.h0;
  for (int s = 0; s < 2; ++s) {
    m.o_slab[s] = s < t.nslab ? t.o_slab[s] : 0;
    m.R[s] = t.R[s];
    m.o_blk[s] = s < t.nblk ? t.o_blk[s] : 0;
    m.ldkb[s] = t.ldkb[s];
    m.trial32[s] = t.trial32[s];
    m.rh1_32[s] = t.rh1_32[s];
    m.g_fb[s] = t.g_fb[s];
    for (int i = 0; i < 2; ++i) {
      m.g_blk[s][i] = t.g_blk[s][i];
      m.wt[s][i] = t.wt[s][i];
    }
  }
  m.g_inv = t.g_inv;
  m.ene1 = t.ene1;
  return m;
}

}  // namespace

size_t tc_workspace_bytes(const afq_ctx_dev& c, int nwc, int32_t cfg) {
  Plan P;
  if (make_plan(c, nwc, cfg, &P)) return 0;
  return P.total;
}

int tc_init(TcState* out, const afq_ctx_dev& c, const afq_hamiltonian& h, const double* rccat, int nwc,
            int32_t cfg, char* ws, cudaStream_t st) {
  Plan P;
  TC_CHECK(make_plan(c, nwc, cfg, &P));
  TcState& t = P.t;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(ws) + 1023) & ~uintptr_t(1023));
  auto U = [&](size_t o) { return reinterpret_cast<uint16_t*>(base + o); };
  for (int i = 0; i < 2; ++i) {
    t.rc_fb[i] = U(P.o_rc_fb[i]);
    t.lop[i] = U(P.o_lop[i]);
    t.g_fb[i] = U(P.o_gfb[i]);
    t.xt[i] = U(P.o_xt[i]);
    t.vbuf[i] = U(P.o_vbuf[i]);
    for (int s = 0; s < t.nslab; ++s) {
      t.eop[s][i] = U(P.o_eop[s][i]);
      t.wt[s][i] = U(P.o_wt[s][i]);
      t.acc[s][i] = U(P.o_acc[s][i]);
      t.t0[s][i] = U(P.o_t0[s][i]);
    }
    for (int b = 0; b < t.nblk; ++b) {
      t.u[b][i] = U(P.o_u[b][i]);
      // one Green block (RHF): the block operands are the force-bias operands themselves
      t.g_blk[b][i] = t.nblk == 2 ? U(P.o_gblk[b][i]) : t.g_fb[i];
      t.rc_blk[b][i] = t.nblk == 2 ? U(P.o_rcb[b][i]) : t.rc_fb[i];
    }
  }
  t.rc_inv = reinterpret_cast<float*>(base + P.o_rc_inv);
  for (int b = 0; b < t.nblk; ++b)
    t.rc_blk_inv[b] = t.nblk == 2 ? reinterpret_cast<float*>(base + P.o_rcb_inv[b]) : t.rc_inv;
  t.u_tmp = reinterpret_cast<float*>(base + P.o_utmp);
  unsigned* amax = reinterpret_cast<unsigned*>(base + P.o_amax);
  t.g_inv = reinterpret_cast<float*>(base + P.o_ginv);
  t.ene1 = reinterpret_cast<double2*>(base + P.o_ene1);
  t.part_shift = reinterpret_cast<double2*>(base + P.o_pshift);
  t.fb_part = reinterpret_cast<float*>(base + P.o_fbpart);
  t.part_fbt = reinterpret_cast<double2*>(base + P.o_pfbt);
  t.c_out = reinterpret_cast<double2*>(base + P.o_cout);
  t.exc_part = reinterpret_cast<double2*>(base + P.o_exc);
  t.status = reinterpret_cast<int*>(base + P.o_status);
  t.dchol = reinterpret_cast<float*>(base + P.o_dchol);
  for (int s = 0; s < 2; ++s) {
    t.trial32[s] = reinterpret_cast<float*>(base + P.o_trial32[s]);
    t.rh1_32[s] = reinterpret_cast<float*>(base + P.o_rh1[s]);
  }
  // zero everything once: padding rows and columns of every operand stay zero afterwards
  cudaError_t e = cudaMemsetAsync(base, 0, P.total - 1024, st);
  if (e != cudaSuccess) {
    afq_set_error("memset: %s", cudaGetErrorString(e));
    return (int)e;
  }
  const int bf = t.bf16 ? 1 : 0;
  ProfScope _ps(K_PREP, st);
  if (t.cfg & kDiagChol) k_prep_diag<<<c.nchol, 256, 0, st>>>(h.chol, t.n, t.dchol, t.status);
  for (int s = 0; s < t.nslab; ++s) {
    k_to_f32<<<64, 256, 0, st>>>(c.trial[s], const_cast<float*>(t.trial32[s]), (long)t.n * t.o_slab[s]);
    k_prep_eop<<<64, 256, 0, st>>>(c.exp_h1[s], t.n, t.nk, bf, t.eop[s][0], t.eop[s][1]);
  }
  for (int b = 0; b < t.nblk; ++b) {
    k_to_f32<<<64, 256, 0, st>>>(c.rot_h1[b], const_cast<float*>(t.rh1_32[b]), (long)t.n * t.o_blk[b]);
    if (t.nblk == 2) {
      k_row_scale<<<c.nchol, 256, 0, st>>>(c.rot_chol[b], t.kb[b], t.rc_blk_inv[b]);
      k_prep_rows_scaled<<<c.nchol, 256, 0, st>>>(c.rot_chol[b], t.kb[b], t.ldkb[b], bf, t.rc_blk_inv[b],
                                                  t.rc_blk[b][0], t.rc_blk[b][1]);
    }
    // exchange matrix of this block: power-of-two scaling, hi/lo split; built in FP64 on the
    // SIMT cores, or for large blocks as X X^T on the split tensor-core GEMM
    cudaMemsetAsync(amax, 0, 8, st);
    if (t.kb[b] > kExchangeTensorMinKb) {
      uint16_t* xh = U(P.o_xu[0]);
      uint16_t* xl = U(P.o_xu[1]);
      k_amax_f64<<<1024, 256, 0, st>>>(c.rot_chol[b], (long)c.nchol * t.kb[b], amax + 1);
      k_prep_xu<<<dim3((t.kb[b] + 31) / 32, (c.nchol + 31) / 32), 256, 0, st>>>(c.rot_chol[b], c.nchol, t.kb[b],
                                                                               t.ldg, amax + 1, bf, xh, xl);
      SplitMaps xm;
      memset(&xm, 0, sizeof(xm));
      TC_CHECK(make_tmap_16(&xm.a_hi, xh, t.kb[b], c.nchol, t.ldg, 128, t.bf16));
      TC_CHECK(make_tmap_16(&xm.a_lo, xl, t.kb[b], c.nchol, t.ldg, 128, t.bf16));
      TC_CHECK(make_tmap_16(&xm.b_hi, xh, t.kb[b], c.nchol, t.ldg, kSplitBBox, t.bf16));
      TC_CHECK(make_tmap_16(&xm.b_lo, xl, t.kb[b], c.nchol, t.ldg, kSplitBBox, t.bf16));
      SplitArgs ga;
      ga.m_tiles = (t.kb[b] + 127) / 128;
      ga.n_tiles = (t.kb[b] + kSplitBN - 1) / kSplitBN;
      ga.k_tiles = (c.nchol + 63) / 64;
      ga.k_splits = 1;
      ga.a_row0 = 0;
      ga.has_alo = 1;
      ga.has_blo = 1;
      ga.drain = t.drain > 0 ? t.drain : ga.k_tiles;
      ga.idesc = ptx::idesc_f16(128, kSplitBN, t.bf16 ? 1 : 0);
      int dev = 0, sms = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 148;
      SplitStoreU::Params up{t.u_tmp, t.kb[b], t.n, t.ldkb[b], amax + 1, amax};
      TC_CHECK(launch_split<SplitStoreU>(K_PREP, xm, ga, sms, up, t.status, st));
    } else {
      k_prep_u<<<dim3((t.kb[b] + 31) / 32, (t.kb[b] + 31) / 32), 256, 0, st>>>(c.rot_chol[b], c.nchol, t.kb[b],
                                                                             t.n, t.ldkb[b], t.u_tmp, amax);
    }
    const long ucount = (long)t.kb[b] * t.ldkb[b];
    k_split_u<<<1024, 256, 0, st>>>(t.u_tmp, ucount, amax, bf, t.u[b][0], t.u[b][1]);
    unsigned amax_h = 0;
    cudaMemcpyAsync(&amax_h, amax, 4, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);  // set-up only: the unscale factor is a host constant
    float am;
    memcpy(&am, &amax_h, 4);
    int ex = 0;
    if (am > 0.f) frexpf(am, &ex);
    t.u_inv[b] = ldexpf(1.0f, ex);
  }
  const double* rcsrc = c.nspin_g == 2 ? rccat : c.rot_chol[0];
  k_row_scale<<<c.nchol, 256, 0, st>>>(rcsrc, t.kfb, t.rc_inv);
  k_prep_rows_scaled<<<c.nchol, 256, 0, st>>>(rcsrc, t.kfb, t.ldfb, bf, t.rc_inv, t.rc_fb[0], t.rc_fb[1]);
  if (t.sym)
    k_prep_lop_sym<<<dim3((t.n_vcols + 31) / 32, (c.nchol + 31) / 32), 256, 0, st>>>(
        h.chol, c.nchol, t.n, t.nq, t.n_vcols, t.ldg, bf, t.lop[0], t.lop[1]);
  else
    k_prep_lop<<<dim3((t.n * t.n + 31) / 32, (c.nchol + 31) / 32), 256, 0, st>>>(h.chol, c.nchol, t.n, t.nq,
                                                                               t.ldg, bf, t.lop[0], t.lop[1]);
  TC_CHECK(launch_check("mixed operand preparation"));
  // ---- tensor maps
  const bool b16 = t.bf16;
  auto mk = [&](CUtensorMap* m, const void* p, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box) {
    return make_tmap_16(m, p, rows, cols, ld, box, b16);
  };
  {  // force bias: A = g_fb (walker-dependent), B = rc_fb (static)
    int i = 0;
    TC_CHECK(mk(&t.m_fb.a[i], t.g_fb[0], 2 * t.nw, t.kfb, t.ldfb, 128));
    TC_CHECK(mk(&t.m_fb.b[i++], t.rc_fb[0], c.nchol, t.kfb, t.ldfb, t.fb_bn));
    if (t.cfg & kFbDyn) {
      TC_CHECK(mk(&t.m_fb.a[i], t.g_fb[1], 2 * t.nw, t.kfb, t.ldfb, 128));
      TC_CHECK(mk(&t.m_fb.b[i++], t.rc_fb[0], c.nchol, t.kfb, t.ldfb, t.fb_bn));
    }
    if (t.cfg & kFbStat) {
      TC_CHECK(mk(&t.m_fb.a[i], t.g_fb[0], 2 * t.nw, t.kfb, t.ldfb, 128));
      TC_CHECK(mk(&t.m_fb.b[i++], t.rc_fb[1], c.nchol, t.kfb, t.ldfb, t.fb_bn));
    }
  }
  {  // force-bias planes for the persistent split GEMM
    TC_CHECK(mk(&t.m_fb_split.a_hi, t.g_fb[0], 2 * t.nw, t.kfb, t.ldfb, 128));
    TC_CHECK(mk(&t.m_fb_split.a_lo, t.g_fb[1], 2 * t.nw, t.kfb, t.ldfb, 128));
    TC_CHECK(mk(&t.m_fb_split.b_hi, t.rc_fb[0], c.nchol, t.kfb, t.ldfb, kSplitBBox));
    TC_CHECK(mk(&t.m_fb_split.b_lo, t.rc_fb[1], c.nchol, t.kfb, t.ldfb, kSplitBBox));
  }
  {  // vhs planes for the persistent split GEMM (B boxes of 256 rows)
    const uint64_t nrows = (uint64_t)t.n * t.nq;
    TC_CHECK(mk(&t.m_vhs_split.a_hi, t.xt[0], 2 * t.nw, c.nchol, t.ldg, 128));
    TC_CHECK(mk(&t.m_vhs_split.a_lo, t.xt[1], 2 * t.nw, c.nchol, t.ldg, 128));
    TC_CHECK(mk(&t.m_vhs_split.b_hi, t.lop[0], (uint64_t)t.n_vcols, c.nchol, t.ldg, kSplitBBox));
    TC_CHECK(mk(&t.m_vhs_split.b_lo, t.lop[1], (uint64_t)t.n_vcols, c.nchol, t.ldg, kSplitBBox));
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&t.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || t.num_sms < 1)
      t.num_sms = 148;
  }
  {  // vhs: A = xt (walker-dependent), B = lop (static)
    int i = 0;
    const uint64_t nrows = (uint64_t)t.n * t.nq;
    TC_CHECK(mk(&t.m_vhs.a[i], t.xt[0], 2 * t.nw, c.nchol, t.ldg, 128));
    TC_CHECK(mk(&t.m_vhs.b[i++], t.lop[0], nrows, c.nchol, t.ldg, 128));
    if (t.cfg & kVhsDyn) {
      TC_CHECK(mk(&t.m_vhs.a[i], t.xt[1], 2 * t.nw, c.nchol, t.ldg, 128));
      TC_CHECK(mk(&t.m_vhs.b[i++], t.lop[0], nrows, c.nchol, t.ldg, 128));
    }
    if (t.cfg & kVhsStat) {
      TC_CHECK(mk(&t.m_vhs.a[i], t.xt[0], 2 * t.nw, c.nchol, t.ldg, 128));
      TC_CHECK(mk(&t.m_vhs.b[i++], t.lop[1], nrows, c.nchol, t.ldg, 128));
    }
  }
  for (int s = 0; s < t.nslab; ++s) {  // exp_h1 products: A = eop (static), B = wt / acc
    const uint64_t rows = (uint64_t)t.nw * t.R[s];
    for (int which = 0; which < 2; ++which) {
      GemmMaps& m = which == 0 ? t.m_e1[s] : t.m_e2[s];
      uint16_t** bop = which == 0 ? t.wt[s] : t.acc[s];
      int i = 0;
      TC_CHECK(mk(&m.a[i], t.eop[s][0], 128, t.n, t.nk, 128));
      TC_CHECK(mk(&m.b[i++], bop[0], rows, t.n, t.nk, t.bn_w[s]));
      if (t.cfg & kExpDyn) {
        TC_CHECK(mk(&m.a[i], t.eop[s][0], 128, t.n, t.nk, 128));
        TC_CHECK(mk(&m.b[i++], bop[1], rows, t.n, t.nk, t.bn_w[s]));
      }
      if (t.cfg & kExpStat) {
        TC_CHECK(mk(&m.a[i], t.eop[s][1], 128, t.n, t.nk, 128));
        TC_CHECK(mk(&m.b[i++], bop[0], rows, t.n, t.nk, t.bn_w[s]));
      }
    }
    TC_CHECK(mk(&t.m_vt[s][0], t.vbuf[0], (uint64_t)nwc * t.mr, 2 * t.nq, 2 * t.nq, 128));
    TC_CHECK(mk(&t.m_vt[s][1], t.vbuf[1], (uint64_t)nwc * t.mr, 2 * t.nq, 2 * t.nq, 128));
    TC_CHECK(mk(&t.m_ew[s][0], t.eop[s][0], (uint64_t)t.mr, t.n, t.nk, 128));
    TC_CHECK(mk(&t.m_ew[s][1], t.eop[s][1], (uint64_t)t.mr, t.n, t.nk, 128));
    TC_CHECK(mk(&t.m_t0[s][0], t.t0[s][0], (uint64_t)t.nw * t.NT[s], 2 * t.nq, 2 * t.nq, t.NT[s]));
    TC_CHECK(mk(&t.m_t0[s][1], t.t0[s][1], (uint64_t)t.nw * t.NT[s], 2 * t.nq, 2 * t.nq, t.NT[s]));
  }
  for (int b = 0; b < t.nblk; ++b) {
    // Coulomb: c_g = G_b . rot_chol_b (A = Green operand, B = rot_chol operand)
    {
      int i = 0;
      TC_CHECK(mk(&t.m_c[b].a[i], t.g_blk[b][0], 2 * t.nw, t.kb[b], t.ldkb[b], 128));
      TC_CHECK(mk(&t.m_c[b].b[i++], t.rc_blk[b][0], c.nchol, t.kb[b], t.ldkb[b], t.fb_bn));
      if (t.cfg & kEneDyn) {
        TC_CHECK(mk(&t.m_c[b].a[i], t.g_blk[b][1], 2 * t.nw, t.kb[b], t.ldkb[b], 128));
        TC_CHECK(mk(&t.m_c[b].b[i++], t.rc_blk[b][0], c.nchol, t.kb[b], t.ldkb[b], t.fb_bn));
      }
      if (t.cfg & kEneStat) {
        TC_CHECK(mk(&t.m_c[b].a[i], t.g_blk[b][0], 2 * t.nw, t.kb[b], t.ldkb[b], 128));
        TC_CHECK(mk(&t.m_c[b].b[i++], t.rc_blk[b][1], c.nchol, t.kb[b], t.ldkb[b], t.fb_bn));
      }
    }
    // exchange: Z^T = G_b . U_b (U symmetric) on the split GEMM (A = Green operand planes, B = U planes)
    memset(&t.m_zs[b], 0, sizeof(SplitMaps));
    TC_CHECK(mk(&t.m_zs[b].a_hi, t.g_blk[b][0], 2 * t.nw, t.kb[b], t.ldkb[b], 128));
    if (t.cfg & kEneDyn) TC_CHECK(mk(&t.m_zs[b].a_lo, t.g_blk[b][1], 2 * t.nw, t.kb[b], t.ldkb[b], 128));
    TC_CHECK(mk(&t.m_zs[b].b_hi, t.u[b][0], t.kb[b], t.kb[b], t.ldkb[b], kSplitBBox));
    if (t.cfg & kEneStat) TC_CHECK(mk(&t.m_zs[b].b_lo, t.u[b][1], t.kb[b], t.kb[b], t.ldkb[b], kSplitBBox));
  }
  t.ready = 1;
  *out = t;
  return 0;
}

template <int OM>
static void launch_green_fused(const MixedDev& md, size_t smem, const float2* w0, const float2* w1, double2* ovl,
                               int flags, cudaStream_t st) {
  // a refused attribute surfaces as the launch error checked by the caller
  cudaFuncSetAttribute(k_green_fused<OM, kGfThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_green_fused<OM, kGfThreads><<<md.nw, kGfThreads, smem, st>>>(md, w0, w1, ovl, flags);
}

int tc_green(TcState& t, const afq_ctx_dev& c, const void* wu, const void* wd, double2* ovl, bool write_ops,
             cudaStream_t st, bool for_propagation) {
  MixedDev md = mixed_dev(t, c);
  const int omax = md.o_slab[0] > md.o_slab[1] ? md.o_slab[0] : md.o_slab[1];
  if (omax > kGreenMaxO) {
    afq_set_error("mixed precision path: at most %d electrons per spin", kGreenMaxO);
    return -2;
  }
  const float2* w0 = static_cast<const float2*>(wu);
  const float2* w1 = static_cast<const float2*>(wd);
  // the walker operand of the exp_h1 GEMMs is needed only when they run as separate launches
  const int flags = (write_ops || for_propagation) ? ((t.fused || t.wide ? 0 : kGreenWT) | kGreenG) : 0;
  const int om = omax <= 8 ? 8 : omax <= 16 ? 16 : omax <= 24 ? 24 : omax <= 32 ? 32 : 40;
  const size_t smem =
      green_fused_smem(t.n, omax, om, md.o_blk[0] + md.o_blk[1], (flags & kGreenG) != 0, md.nslab);
  if (int rc = check_smem_optin(smem + sizeof(float2) * 2 * om * (om + 1) + 1024,
                                "mixed Green's-function kernel (norb x electrons too large for one CTA)"))
    return rc;
  {
    ProfScope _ps(K_GREEN, st);
    if (om == 8) launch_green_fused<8>(md, smem, w0, w1, ovl, flags, st);
    else if (om == 16) launch_green_fused<16>(md, smem, w0, w1, ovl, flags, st);
    else if (om == 24) launch_green_fused<24>(md, smem, w0, w1, ovl, flags, st);
    else if (om == 32) launch_green_fused<32>(md, smem, w0, w1, ovl, flags, st);
    else launch_green_fused<40>(md, smem, w0, w1, ovl, flags, st);
  }
  return launch_check("green_fused");
}

// energy (with maps == nullptr): the Coulomb contraction of the local energy on the split
// path (RHF: the same operands as the force bias), with the energy's split-term options
static int fb_gemm(TcState& t, const afq_ctx_dev& c, const double* fields, double2* fb_out, cudaStream_t st,
                   const GemmMaps* maps = nullptr, const float* rc_inv = nullptr, float alpha = 0.f,
                   int kdim = 0, bool energy = false) {
  EpiFB::Params ep;
  memset(&ep, 0, sizeof(ep));
  ep.fields = fields;
  ep.mf = c.mf;
  ep.rc_inv = rc_inv ? rc_inv : t.rc_inv;
  ep.g_inv = t.g_inv;
  ep.alpha = alpha != 0.f ? alpha : (c.energy_mode == 0 ? 2.0f : 1.0f);
  ep.sqdt = (float)sqrt(c.dt);
  ep.nw = t.nw;
  ep.nchol = c.nchol;
  ep.ldg = t.ldg;
  ep.ntiles = t.fb_ntiles;
  ep.bf16 = t.bf16 ? 1 : 0;
  ep.xt_hi = t.xt[0];
  ep.xt_lo = t.xt[1];
  ep.part_shift = t.part_shift;
  ep.part_fbt = t.part_fbt;
  ep.fb_out = fb_out;
  const int kt = ((kdim ? kdim : t.kfb) + 63) / 64, mt = (2 * t.nw + 127) / 128;
  if (!maps) {
    // force bias: K-split partials on the persistent split GEMM, then one reduction per
    // walker fused with the field shifts
    SplitArgs sa;
    sa.m_tiles = mt;
    sa.n_tiles = t.fb_npad / kSplitBN;
    sa.k_tiles = kt;
    sa.k_splits = t.fb_ks;
    sa.a_row0 = 0;
    sa.has_alo = (t.cfg & (energy ? kEneDyn : kFbDyn)) ? 1 : 0;
    sa.has_blo = (t.cfg & (energy ? kEneStat : kFbStat)) ? 1 : 0;
    sa.drain = t.drain > 0 ? t.drain : kt;
    sa.idesc = ptx::idesc_f16(128, kSplitBN, t.bf16 ? 1 : 0);
    const long ldp = t.fb_npad, sst = (long)mt * 128 * t.fb_npad;
    SplitPartialF32::Params pp{t.fb_part, 2 * t.nw, c.nchol, ldp, sst};
    const int cls = energy ? K_ENERGY : K_FB;
    TC_CHECK(launch_split<SplitPartialF32>(cls, t.m_fb_split, sa, t.num_sms, pp, t.status, st));
    FbReduce r;
    r.part = t.fb_part;
    r.ksplit = t.fb_ks;
    r.nw = t.nw;
    r.nchol = c.nchol;
    r.ldg = t.ldg;
    r.bf16 = ep.bf16;
    r.ldp = ldp;
    r.sst = sst;
    r.fields = fields;
    r.mf = c.mf;
    r.rc_inv = ep.rc_inv;
    r.g_inv = t.g_inv;
    r.alpha = ep.alpha;
    r.sqdt = ep.sqdt;
    r.xt_hi = t.xt[0];
    r.xt_lo = t.xt[1];
    r.part_shift = t.part_shift;
    r.part_fbt = t.part_fbt;
    r.fb_out = fb_out;
    {
      ProfScope _ps(cls, st);
      k_fb_reduce<<<t.nw, 256, 0, st>>>(r);
    }
    return launch_check("fb_reduce");
  }
  const int cls = maps ? K_ENERGY : K_FB;
  const GemmMaps& m = maps ? *maps : t.m_fb;
  const int nterms = maps ? t.n_en_terms : t.n_fb_terms;
  if (t.fb_bn <= 64)  // narrow tiles: a smaller ring lets two CTAs share an SM
    return launch_gemm<64, 4, EpiFB>(cls, m, nterms, kt, mt, t.fb_ntiles, t.fb_bn, t.bf16, ep, t.status, st, 0,
                                     t.drain);
  return launch_gemm<128, 4, EpiFB>(cls, m, nterms, kt, mt, t.fb_ntiles, t.fb_bn, t.bf16, ep, t.status, st, 0,
                                    t.drain);
}

int tc_force_bias(TcState& t, const afq_ctx_dev& c, double2* out, cudaStream_t st) {
  return fb_gemm(t, c, nullptr, out, st);
}

int tc_field_shifts(TcState& t, const afq_ctx_dev& c, const double* fields, cudaStream_t st) {
  return fb_gemm(t, c, fields, nullptr, st);
}

static int exp_gemm(TcState& t, const afq_ctx_dev& c, int s, bool last, float2* w, cudaStream_t st) {
  EpiExp::Params ep;
  memset(&ep, 0, sizeof(ep));
  ep.w = reinterpret_cast<float*>(w);
  ep.acc_hi = t.acc[s][0];
  ep.acc_lo = t.acc[s][1];
  ep.t0_hi = t.t0[s][0];
  ep.t0_lo = t.t0[s][1];
  ep.n = t.n;
  ep.o = t.o_slab[s];
  ep.R = t.R[s];
  ep.nk = t.nk;
  ep.nq = t.nq;
  ep.NT = t.NT[s];
  ep.nw = t.nw;
  ep.bf16 = t.bf16 ? 1 : 0;
  ep.last = last ? 1 : 0;
  const int kt = (t.n + 63) / 64, nt = (t.nw * t.R[s] + t.bn_w[s] - 1) / t.bn_w[s];
  return launch_gemm<256, 2, EpiExp>(K_EXP, last ? t.m_e2[s] : t.m_e1[s], t.n_e_terms, kt, 1, nt, t.bn_w[s], t.bf16,
                                     ep, t.status, st);
}

template <int NP>
static int launch_prop_fused(const TcState& t, int s, const PropDev& pd, cudaStream_t st) {
  const size_t smem = prop_fused_smem(t.nq, t.NT[s]);
  auto kfn = k_prop_fused<NP>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    afq_set_error("prop_fused: shared-memory attribute: %s", cudaGetErrorString(e));
    return (int)e;
  }
  {
    ProfScope _ps(K_PROP, st);
    kfn<<<pd.nwc < t.num_sms ? pd.nwc : t.num_sms, 128 * NP + 160, smem, st>>>(
        t.m_vt[s][0], t.m_vt[s][1], t.eop[s][0], t.eop[s][1], t.nk, pd, t.status);
  }
  return launch_check("prop_fused");
}

template <int NP>
static int launch_prop_wide(const TcState& t, int s, const PropDev& pd, cudaStream_t st) {
  const size_t smem = prop_wide_smem(t.NT[s]);
  auto kfn = k_prop_wide<NP>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    afq_set_error("prop_wide: shared-memory attribute: %s", cudaGetErrorString(e));
    return (int)e;
  }
  {
    ProfScope _ps(K_PROP, st);
    kfn<<<pd.nwc < t.num_sms ? pd.nwc : t.num_sms, 128 * NP + 64, smem, st>>>(
        t.m_vt[s][0], t.m_vt[s][1], t.m_ew[s][0], t.m_ew[s][1], pd, t.status);
  }
  return launch_check("prop_wide");
}

// vhs GEMM, then exp_h1 * Taylor * exp_h1 in one kernel per slab, chunk by chunk
static int propagate_fused(TcState& t, const afq_ctx_dev& c, float2* const* W, cudaStream_t st) {
  const int nchunks = t.nw / t.nwc;
  const bool want_lo = t.taylor_split > 0;
  for (int ch = 0; ch < nchunks; ++ch) {
    const int w0 = ch * t.nwc;
    EpiVHS::Params ev;
    ev.v_hi = t.vbuf[0];
    ev.v_lo = t.vbuf[1];
    ev.n = t.n;
    ev.nq = t.nq;
    ev.rows = 2 * t.nwc;
    ev.bf16 = t.bf16 ? 1 : 0;
    ev.want_lo = want_lo ? 1 : 0;
    ev.sqdt = (float)sqrt(c.dt);
    ev.sym = t.sym ? 1 : 0;
    ev.mr = t.mr;
    SplitArgs sa;
    sa.k_tiles = (c.nchol + 63) / 64;
    sa.k_splits = 1;
    sa.m_tiles = (2 * t.nwc + 127) / 128;
    sa.n_tiles = (t.n_vcols + kSplitBN - 1) / kSplitBN;
    sa.a_row0 = 2 * w0;
    sa.has_alo = (t.cfg & kVhsDyn) ? 1 : 0;
    sa.has_blo = (t.cfg & kVhsStat) ? 1 : 0;
    sa.drain = t.drain > 0 ? t.drain : sa.k_tiles;
    sa.idesc = ptx::idesc_f16(128, kSplitBN, t.bf16 ? 1 : 0);
    if (c.n_exp_terms > 1)
      TC_CHECK(launch_split<EpiVHSSplit>(K_VHS, t.m_vhs_split, sa, t.num_sms, ev, t.status, st));
    for (int s = 0; s < t.nslab; ++s) {
      PropDev pd;
      pd.n = t.n;
      pd.o = t.o_slab[s];
      pd.nq = t.nq;
      pd.NT = t.NT[s];
      pd.nterms = c.n_exp_terms;
      pd.split = t.taylor_split;
      pd.bf16 = t.bf16 ? 1 : 0;
      pd.nwc = t.nwc;
      pd.e_lo = (t.cfg & kExpStat) ? 1 : 0;
      pd.w_lo = (t.cfg & kExpDyn) ? 1 : 0;
      pd.sym = t.sym ? 1 : 0;
      pd.w = W[s] + (size_t)w0 * t.n * t.o_slab[s];
      const int np = t.NT[s] / 16;
      if (t.wide) {
        if (np == 1) TC_CHECK(launch_prop_wide<1>(t, s, pd, st));
        else if (np == 2) TC_CHECK(launch_prop_wide<2>(t, s, pd, st));
        else if (np == 3) TC_CHECK(launch_prop_wide<3>(t, s, pd, st));
        else if (np == 4) TC_CHECK(launch_prop_wide<4>(t, s, pd, st));
        else TC_CHECK(launch_prop_wide<5>(t, s, pd, st));
        continue;
      }
      if (np == 1) TC_CHECK(launch_prop_fused<1>(t, s, pd, st));
      else if (np == 2) TC_CHECK(launch_prop_fused<2>(t, s, pd, st));
      else if (np == 3) TC_CHECK(launch_prop_fused<3>(t, s, pd, st));
      else TC_CHECK(launch_prop_fused<4>(t, s, pd, st));
    }
  }
  return 0;
}

int tc_propagate_walkers(TcState& t, const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st) {
  float2* W[2] = {static_cast<float2*>(wu), static_cast<float2*>(wd)};
  if (t.fused || t.wide) return propagate_fused(t, c, W, st);
  for (int s = 0; s < t.nslab; ++s) TC_CHECK(exp_gemm(t, c, s, false, W[s], st));
  if (t.cfg & kDiagChol) {
    if (t.n > 128) {
      afq_set_error("diagonal Cholesky path: norb <= 128");
      return -2;
    }
    TaylorDiag td;
    td.dchol = t.dchol;
    td.xt_hi = t.xt[0];
    td.xt_lo = t.xt[1];
    for (int s = 0; s < 2; ++s) {
      td.t0_hi[s] = t.t0[s][0];
      td.t0_lo[s] = t.t0[s][1];
      td.acc_hi[s] = t.acc[s][0];
      td.acc_lo[s] = t.acc[s][1];
      td.o[s] = t.o_slab[s];
      td.NT[s] = t.NT[s];
      td.R[s] = t.R[s];
    }
    td.nchol = c.nchol;
    td.ldg = t.ldg;
    td.n = t.n;
    td.nq = t.nq;
    td.nk = t.nk;
    td.nterms = c.n_exp_terms;
    td.bf16 = t.bf16 ? 1 : 0;
    td.sqdt = (float)sqrt(c.dt);
    {
      ProfScope _ps(K_TAYLOR, st);
      k_taylor_diag<<<dim3(t.nw, t.nslab), 256, 0, st>>>(td);
    }
    TC_CHECK(launch_check("taylor_diag"));
    for (int s = 0; s < t.nslab; ++s) TC_CHECK(exp_gemm(t, c, s, true, W[s], st));
    return 0;
  }
  const int nchunks = t.nw / t.nwc;
  const bool want_lo = t.taylor_split > 0;
  for (int ch = 0; ch < nchunks; ++ch) {
    const int w0 = ch * t.nwc;
    EpiVHS::Params ev;
    ev.v_hi = t.vbuf[0];
    ev.v_lo = t.vbuf[1];
    ev.n = t.n;
    ev.nq = t.nq;
    ev.rows = 2 * t.nwc;
    ev.bf16 = t.bf16 ? 1 : 0;
    ev.want_lo = want_lo ? 1 : 0;
    ev.sym = 0;  // the separate Taylor kernel reads the full V
    ev.mr = 128;
    ev.sqdt = (float)sqrt(c.dt);
    SplitArgs sa;
    sa.k_tiles = (c.nchol + 63) / 64;
    sa.k_splits = 1;
    sa.m_tiles = (2 * t.nwc + 127) / 128;
    sa.n_tiles = (t.n * t.nq + kSplitBN - 1) / kSplitBN;
    sa.a_row0 = 2 * w0;
    sa.has_alo = (t.cfg & kVhsDyn) ? 1 : 0;
    sa.has_blo = (t.cfg & kVhsStat) ? 1 : 0;
    sa.drain = t.drain > 0 ? t.drain : sa.k_tiles;
    sa.idesc = ptx::idesc_f16(128, kSplitBN, t.bf16 ? 1 : 0);
    TC_CHECK(launch_split<EpiVHSSplit>(K_VHS, t.m_vhs_split, sa, t.num_sms, ev, t.status, st));
    for (int s = 0; s < t.nslab; ++s) {
      TaylorDev td;
      td.n = t.n;
      td.o = t.o_slab[s];
      td.nq = t.nq;
      td.NT = t.NT[s];
      td.R = t.R[s];
      td.nk = t.nk;
      td.nterms = c.n_exp_terms;
      td.split = t.taylor_split;
      td.bf16 = t.bf16 ? 1 : 0;
      td.w0 = w0;
      td.nwc = t.nwc;
      td.acc_hi = t.acc[s][0];
      td.acc_lo = t.acc[s][1];
      const size_t smem = taylor_smem(t.nq, t.NT[s], want_lo);
      // one warp per kTaylorCW columns of the B operand and TMEM lane quadrant; the register
      // budget follows the block size
      const int threads = 128 * ((t.NT[s] + kTaylorCW - 1) / kTaylorCW);
      if (threads > kTaylorMaxThreads) {
        afq_set_error("Taylor kernel: B operand of %d rows (at most %d)", t.NT[s], kTaylorMaxThreads * kTaylorCW / 128);
        return -2;
      }
      auto kfn = threads <= kTaylorMaxThreads * 3 / 4 ? k_taylor_tc<kTaylorMaxThreads * 3 / 4, kTaylorCW>
                                                      : k_taylor_tc<kTaylorMaxThreads, kTaylorCW>;
      cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      {
        ProfScope _ps(K_TAYLOR, st);
        kfn<<<t.nwc < t.num_sms ? t.nwc : t.num_sms, threads, smem, st>>>(t.m_vt[s][0], t.m_vt[s][1], t.m_t0[s][0],
                                                                          t.m_t0[s][1], td, t.status);
      }
      TC_CHECK(launch_check("taylor_tc"));
    }
  }
  for (int s = 0; s < t.nslab; ++s) TC_CHECK(exp_gemm(t, c, s, true, W[s], st));
  return 0;
}

int tc_weights(TcState& t, const afq_ctx_dev& c, const double2* ovl_new, double2* ovl, double* weights,
               double* scalars, cudaStream_t st) {
  // the force-bias reduction leaves one shift_term / fb_term sum per walker
  return launch_weights(c, t.part_shift, t.part_fbt, 1, ovl_new, ovl, weights, scalars, st, t.status);
}

// local energy (wavefunctions.py:529-561, 711-743): Coulomb c_g from a force-bias-like GEMM,
// exchange from the U GEMM, both per spin block; ene1 comes from the Green kernel.
int tc_energy(TcState& t, const afq_ctx_dev& c, double2* out, cudaStream_t st) {
  for (int b = 0; b < t.nblk; ++b) {
    if (t.nblk == 1)  // RHF: the force-bias operands, on the persistent split GEMM
      TC_CHECK(fb_gemm(t, c, nullptr, t.c_out, st, nullptr, nullptr, 1.0f, 0, true));
    else
      TC_CHECK(fb_gemm(t, c, nullptr, t.c_out + (size_t)b * t.nw * c.nchol, st, &t.m_c[b], t.rc_blk_inv[b], 1.0f,
                       t.kb[b]));
    EpiExcSplit::Params ep;
    ep.g_hi = t.g_blk[b][0];
    ep.g_lo = t.g_blk[b][1];
    ep.g_inv = t.g_inv;
    ep.u_inv = t.u_inv[b];
    ep.kb = t.kb[b];
    ep.ldk = t.ldkb[b];
    ep.nw = t.nw;
    ep.bf16 = t.bf16 ? 1 : 0;
    ep.n128 = (t.kb[b] + 127) / 128;
    ep.slots = t.mt_z[b];
    ep.exc_part = t.exc_part + (b == 0 ? 0 : (size_t)t.nw * t.mt_z[0]);
    SplitArgs sa;
    sa.m_tiles = (2 * t.nw + 127) / 128;
    sa.n_tiles = (t.kb[b] + kSplitBN - 1) / kSplitBN;
    sa.k_tiles = (t.kb[b] + 63) / 64;
    sa.k_splits = t.z_ks[b];
    sa.a_row0 = 0;
    sa.has_alo = (t.cfg & kEneDyn) ? 1 : 0;   // G_lo * U_hi
    sa.has_blo = (t.cfg & kEneStat) ? 1 : 0;  // G_hi * U_lo
    sa.drain = t.drain > 0 ? t.drain : sa.k_tiles;
    sa.idesc = ptx::idesc_f16(128, kSplitBN, t.bf16 ? 1 : 0);
    TC_CHECK(launch_split<EpiExcSplit>(K_ENERGY, t.m_zs[b], sa, t.num_sms, ep, t.status, st));
  }
  {
    ProfScope _ps(K_ENERGY_FIN, st);
    k_energy_final_mixed<<<t.nw, 256, 0, st>>>(t.nw, c.nchol, t.nblk, t.mt_z[0], t.nblk == 2 ? t.mt_z[1] : 0,
                                               c.energy_mode, c.h0, t.c_out, t.exc_part, t.ene1, out);
  }
  return launch_check("energy_final_mixed");
}

int tc_orthonormalize(TcState& t, const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st) {
  for (int s = 0; s < c.nslab; ++s) {
    const int k = c.kslab[s];
    const size_t smem = (size_t)kQrWarps * ((size_t)c.norb * qr_ld(k) + 64) * sizeof(float2);
    // the warp kernel holds kQrWarps slabs in shared memory; wider or longer slabs take the
    // one-CTA-per-slab Householder kernel
    if (k > 32 || smem > 227 * 1024) return launch_qr<float>(c, wu, wd, st);
    cudaFuncSetAttribute(k_qr_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    {
      ProfScope _ps(K_QR, st);
      k_qr_warp<<<(c.nw + kQrWarps - 1) / kQrWarps, 32 * kQrWarps, smem, st>>>(
          c.nw, c.norb, k, static_cast<float2*>(s == 0 ? wu : wd));
    }
    TC_CHECK(launch_check("qr_warp"));
  }
  return 0;
}

}  // namespace afq

// ---- test hooks (include/afqmc_gb300_testing.h) ---------------------------------------

extern "C" int afq_test_gemm_split(const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo,
                                   float* d, int M, int N, int K, int lda, int ldb, int bf16, int drain,
                                   int* status, void* stream) {
  using namespace afq;
  if (!a_hi || !b_hi || !d || !status || M < 1 || N < 1 || K < 1 || drain < 0) {
    afq_set_error("afq_test_gemm_split: bad arguments");
    return -1;
  }
  SplitMaps maps;
  memset(&maps, 0, sizeof(maps));
  int e = make_tmap_16(&maps.a_hi, a_hi, M, K, lda, 128, bf16 != 0);
  if (!e && a_lo) e = make_tmap_16(&maps.a_lo, a_lo, M, K, lda, 128, bf16 != 0);
  if (!e) e = make_tmap_16(&maps.b_hi, b_hi, N, K, ldb, kSplitBBox, bf16 != 0);
  if (!e && b_lo) e = make_tmap_16(&maps.b_lo, b_lo, N, K, ldb, kSplitBBox, bf16 != 0);
  if (e) return e;
  SplitArgs g;
  g.k_tiles = (K + 63) / 64;
  g.k_splits = 1;
  g.m_tiles = (M + 127) / 128;
  g.n_tiles = (N + kSplitBN - 1) / kSplitBN;
  g.a_row0 = 0;
  g.has_alo = a_lo ? 1 : 0;
  g.has_blo = b_lo ? 1 : 0;
  g.drain = drain > 0 ? drain : g.k_tiles;
  g.idesc = ptx::idesc_f16(128, kSplitBN, bf16 ? 1 : 0);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 148;
  SplitStoreF32::Params ep{d, M, N, (long)N};
  return launch_split<SplitStoreF32>(K_PREP, maps, g, sms, ep, status, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int afq_test_split_pairs(int enable) {
  const int prev = afq::g_split_pairs;
  if (enable >= 0) afq::g_split_pairs = enable ? 1 : 0;
  return prev;
}

extern "C" int afq_test_gemm_f16(const void* a, const void* b, int nterms, long a_term_stride,
                                 long b_term_stride, float* d, int M, int N, int K, int lda,
                                 int ldb, int bf16, int bn, int drain, int* status, void* stream) {
  using namespace afq;
  if (!a || !b || !d || !status || M < 1 || N < 1 || K < 1 || nterms < 1 || nterms > 3) {
    afq_set_error("afq_test_gemm_f16: bad arguments");
    return -1;
  }
  if (bn % 16 || bn < 16 || bn > 256) {
    afq_set_error("afq_test_gemm_f16: bn must be a multiple of 16 in [16, 256]");
    return -1;
  }
  GemmMaps maps;
  memset(&maps, 0, sizeof(maps));
  for (int t = 0; t < nterms; ++t) {
    const char* at = static_cast<const char*>(a) + (size_t)t * a_term_stride * 2;
    const char* bt = static_cast<const char*>(b) + (size_t)t * b_term_stride * 2;
    int e = make_tmap_16(&maps.a[t], at, M, K, lda, 128, bf16 != 0);
    if (!e) e = make_tmap_16(&maps.b[t], bt, N, K, ldb, bn, bf16 != 0);
    if (e) return e;
  }
  EpiStoreF32::Params ep{d, M, N, (long)N};
  const int kt = (K + 63) / 64, mt = (M + 127) / 128, nt = (N + bn - 1) / bn;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // bn <= 128 runs the instantiation the product GEMMs use (register-resident drain)
  if (bn <= 128)
    return launch_gemm<128, 4, EpiStoreF32>(K_PREP, maps, nterms, kt, mt, nt, bn, bf16, ep, status, st, 0,
                                            drain);
  return launch_gemm<256, 4, EpiStoreF32>(K_PREP, maps, nterms, kt, mt, nt, bn, bf16, ep, status, st, 0,
                                          drain);
}

// Allocation-free force bias for callers that cannot allocate device memory.
//
// Some hosts cannot call cudaMalloc at all: code running inside another runtime's memory
// arena (a JAX/XLA custom call or a plugin that only receives pre-allocated buffers), or a
// process whose device memory is fully reserved up front. For them this file provides one
// entry point that computes the force bias with no allocation and no context: the
// Green's function it needs as scratch lives in a file-scope device array of fixed size,
// which every GPU that loads the library keeps until the process exits.

#include <string.h>

#include <mutex>

#include <cuda.h>

#include "afq_common.cuh"
#include "afq_kernels.cuh"

namespace {

// 40 MiB of scratch: the Green's functions of n_walkers * nocc * norb <= 2,621,440
// complex128 values (for example 1024 walkers x 20 electrons x 128 orbitals).
constexpr size_t kNoAllocScratchBytes = size_t(40) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// per device: the scratch address and the CUDA context it was looked up in
void* g_scratch_addr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};

typedef CUresult (*PFN_ctxGetCurrent)(CUcontext*);

// The driver's current context (its handle changes when the primary context is torn down
// and created again, e.g. after cudaDeviceReset, which also reloads this module's array).
CUcontext current_context() {
  static PFN_ctxGetCurrent fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_ctxGetCurrent>(p);
    cudaGetLastError();
  }
  CUcontext ctx = nullptr;
  if (fn && fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  return ctx;
}

// Device address of the scratch array on the current device. Host code cannot use the
// array's name as a device pointer; the address is looked up with cudaGetSymbolAddress the
// first time a device (and context) is seen, with that device current, and cached.
int scratch_on_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    afq_set_error("afq_calc_force_bias_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return (int)e;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    afq_set_error("afq_calc_force_bias_noalloc: device index %d out of range", dev);
    return -1;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  const CUcontext ctx = current_context();
  if (!g_scratch_addr[dev] || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      afq_set_error("afq_calc_force_bias_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return e != cudaSuccess ? (int)e : -1;
    }
    g_scratch_addr[dev] = p;
    // the context is current now (cudaGetSymbolAddress initialises it if needed)
    g_scratch_ctx[dev] = current_context();
  }
  *out = g_scratch_addr[dev];
  return 0;
}

}  // namespace

extern "C" int afq_calc_force_bias_noalloc(int32_t norb, int32_t nocc, int32_t nchol, int32_t n_walkers,
                                           const double* trial, const double* rot_chol,
                                           const void* walkers, double* force_bias, void* stream) {
  if (norb < 1 || nocc < 1 || nocc > norb || nocc > 64 || nchol < 1 || n_walkers < 1 ||
      (size_t)norb * nocc > 7000) {
    afq_set_error("afq_calc_force_bias_noalloc: bad sizes norb=%d nocc=%d nchol=%d n_walkers=%d", norb,
                  nocc, nchol, n_walkers);
    return -1;
  }
  const size_t need = (size_t)n_walkers * nocc * norb * sizeof(double2);
  if (need > kNoAllocScratchBytes) {
    afq_set_error(
        "afq_calc_force_bias_noalloc: needs %zu bytes of scratch, the static scratch holds %zu "
        "(n_walkers * nocc * norb <= %zu)",
        need, kNoAllocScratchBytes, kNoAllocScratchBytes / sizeof(double2));
    return -1;
  }
  if (!trial || !rot_chol || !walkers || !force_bias) {
    afq_set_error("afq_calc_force_bias_noalloc: NULL argument");
    return -1;
  }
  // the Green's-function kernel holds the walker, trial and S^-1 in shared memory
  if (int rc = afq::check_smem_optin(afq::green_f64_smem(norb, nocc),
                                     "afq_calc_force_bias_noalloc: norb x nocc too large for the Green kernel"))
    return rc;
  void* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc) return rc;
  // RHF trial, restricted walkers, FP64: the sizes a context would derive
  afq_ctx_dev c;
  memset(&c, 0, sizeof(c));
  c.norb = norb;
  c.nchol = nchol;
  c.nw = n_walkers;
  c.nslab = 1;
  c.kslab[0] = c.nocc_slab[0] = nocc;
  c.kmax = nocc;
  c.restricted_square = 1;
  c.nspin_g = 1;
  c.gocc[0] = nocc;
  c.ktot = nocc * norb;
  c.trial[0] = c.trial[1] = trial;
  c.rot_chol[0] = c.rot_chol[1] = rot_chol;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  double2* green = static_cast<double2*>(scratch);  // every element is overwritten below
  rc = afq::launch_green<double>(c, walkers, nullptr, green, nullptr, true, st);
  if (rc) return rc;
  return afq::launch_gemm_cr(false, n_walkers, nchol, c.ktot, green, c.ktot, rot_chol, c.ktot,
                             reinterpret_cast<double2*>(force_bias), nchol, c2(2.0, 0.0), st);
}

// Launch accounting and optional CUDA-event timing per kernel class. Every kernel launch of
// the library sits inside a ProfScope; with timing enabled the scope records an event pair
// on the launch stream around the launch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace afq {

enum KClass {
  K_GREEN = 0,   // Green's function / overlap / operand packing
  K_FB,          // force-bias GEMM (+ fused field shifts)
  K_FIELD,       // FP64 field shifts
  K_VHS,         // vhs GEMM
  K_TAYLOR,      // Taylor series of exp(vhs)
  K_EXP,         // exp_h1 products
  K_ENERGY,      // local energy contraction
  K_ENERGY_FIN,  // local energy reduction
  K_WEIGHTS,     // phaseless weights / pop control
  K_QR,          // orthonormalisation
  K_SR,          // stochastic reconfiguration
  K_STATS,       // block statistics and bookkeeping
  K_RNG,         // Philox draws
  K_PREP,        // one-time operand preparation
  K_PROP,        // fused exp_h1 * Taylor * exp_h1 walker propagation
  K_NCLASS
};

void prof_begin(int cls, cudaStream_t st);
void prof_end(int cls, cudaStream_t st);

struct ProfScope {
  int cls;
  cudaStream_t st;
  ProfScope(int c, cudaStream_t s) : cls(c), st(s) { prof_begin(c, s); }
  ~ProfScope() { prof_end(cls, st); }
};

}  // namespace afq

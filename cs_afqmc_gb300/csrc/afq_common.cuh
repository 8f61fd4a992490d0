// Shared device helpers and the context layout of the AFQMC hot path.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/afqmc_gb300.h"

#define AFQ_HD __host__ __device__ __forceinline__
#define AFQ_D __device__ __forceinline__

// ---- complex arithmetic on double2 / float2 ------------------------------------------

AFQ_HD double2 c2(double re, double im) { return make_double2(re, im); }
AFQ_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
AFQ_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
AFQ_HD double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
AFQ_HD double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
AFQ_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a * conj(b)
AFQ_HD double2 cmulc(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
AFQ_HD double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
// Smith's algorithm for a / b.
AFQ_HD double2 cdiv(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  } else {
    double r = b.x / b.y, den = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
}
AFQ_HD double2 cexp_(double2 a) {
  double e = exp(a.x);
  return make_double2(e * cos(a.y), e * sin(a.y));
}

// float2 complex arithmetic (mixed-precision kernels)
AFQ_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
AFQ_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
AFQ_HD float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
AFQ_HD float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
AFQ_HD float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
AFQ_HD float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }
AFQ_HD float2 cdiv(float2 a, float2 b) {
  if (fabsf(b.x) >= fabsf(b.y)) {
    float r = b.y / b.x, den = b.x + b.y * r;
    return make_float2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  } else {
    float r = b.x / b.y, den = b.x * r + b.y;
    return make_float2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
}

// walker storage <-> double2
AFQ_D double2 ld_c(const double2* p) { return *p; }
AFQ_D double2 ld_c(const float2* p) {
  float2 v = *p;
  return make_double2((double)v.x, (double)v.y);
}
AFQ_D void st_c(double2* p, double2 v) { *p = v; }
AFQ_D void st_c(float2* p, double2 v) { *p = make_float2((float)v.x, (float)v.y); }

template <typename WT> struct CplxOf;
template <> struct CplxOf<double> { using type = double2; };
template <> struct CplxOf<float> { using type = float2; };

// ---- block reductions ----------------------------------------------------------------

AFQ_D double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; every thread gets the result. `red` holds >= 32 doubles.
AFQ_D double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nwarp) ? red[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

// Host helpers implemented in afq_capi.cu
void afq_set_error(const char* fmt, ...);

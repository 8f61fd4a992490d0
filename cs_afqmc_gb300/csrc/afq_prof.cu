// Launch counters and event timing per kernel class (see afq_prof.cuh).
#include <mutex>
#include <vector>

#include "afq_common.cuh"
#include "afq_prof.cuh"

namespace afq {
namespace {

struct ClassProf {
  std::vector<cudaEvent_t> ev;  // pairs: 2*i start, 2*i+1 end
  size_t used = 0;
  int64_t launches = 0;
  cudaEvent_t pending = nullptr;
};

std::mutex g_mu;
bool g_timing = false;
ClassProf g_prof[K_NCLASS];

const char* kNames[K_NCLASS] = {"green", "force_bias_gemm", "field_shifts", "vhs_gemm", "taylor",
                                "exp_h1_gemm", "energy_gemm", "energy_reduce", "weights", "qr", "sr",
                                "block_stats", "rng", "prep", "prop_fused"};

}  // namespace

void prof_begin(int cls, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_mu);
  ClassProf& p = g_prof[cls];
  if (!g_timing) return;
  if (p.used * 2 + 2 > p.ev.size()) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    p.ev.push_back(a);
    p.ev.push_back(b);
  }
  cudaEventRecord(p.ev[p.used * 2], st);
}

void prof_end(int cls, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_mu);
  ClassProf& p = g_prof[cls];
  p.launches += 1;
  if (!g_timing) return;
  cudaEventRecord(p.ev[p.used * 2 + 1], st);
  p.used += 1;
}

}  // namespace afq

using namespace afq;

extern "C" {

int afq_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_timing = on != 0;
  for (auto& p : g_prof) {
    p.used = 0;
    p.launches = 0;
  }
  return 0;
}

int afq_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& p : g_prof) {
    p.used = 0;
    p.launches = 0;
  }
  return 0;
}

int afq_profile_read(int cls, double* total_ms, int64_t* launches) {
  if (cls < 0 || cls >= K_NCLASS || !total_ms || !launches) {
    afq_set_error("afq_profile_read: bad arguments");
    return -1;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  ClassProf& p = g_prof[cls];
  double t = 0.0;
  for (size_t i = 0; i < p.used; ++i) {
    float ms = 0.f;
    cudaEventSynchronize(p.ev[2 * i + 1]);
    if (cudaEventElapsedTime(&ms, p.ev[2 * i], p.ev[2 * i + 1]) == cudaSuccess) t += ms;
  }
  *total_ms = t;
  *launches = p.launches;
  return 0;
}

const char* afq_profile_class_name(int cls) {
  return (cls >= 0 && cls < K_NCLASS) ? kNames[cls] : "";
}

int afq_profile_num_classes(void) { return K_NCLASS; }

}  // extern "C"

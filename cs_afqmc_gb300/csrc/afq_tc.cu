// Mixed-precision (BF16 tcgen05) path.
#include "afq_tc.cuh"

namespace afq {

static int not_ready() {
  afq_set_error("mixed precision path is not built yet");
  return -2;
}

size_t tc_workspace_bytes(const afq_ctx_dev&, int) { return 256; }
int tc_init(TcState*, const afq_ctx_dev&, const afq_hamiltonian&, const double*, int, char*, cudaStream_t) {
  return not_ready();
}
int tc_force_bias(TcState&, const afq_ctx_dev&, const double2*, double2*, double, cudaStream_t) { return not_ready(); }
int tc_energy(TcState&, const afq_ctx_dev&, const double2*, double2*, double2*, cudaStream_t) { return not_ready(); }
int tc_propagate_chunk(TcState&, const afq_ctx_dev&, int, int, const double2*, void*, void*, cudaStream_t) {
  return not_ready();
}
int tc_orthonormalize(TcState&, const afq_ctx_dev&, void*, void*, cudaStream_t) { return not_ready(); }

}  // namespace afq

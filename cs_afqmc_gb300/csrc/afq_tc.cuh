// Mixed-precision (BF16 tensor-core) path: operands, plans and launchers.
#pragma once
#include "afq_kernels.cuh"

namespace afq {

struct TcState {
  int ready;
};

size_t tc_workspace_bytes(const afq_ctx_dev& c, int nw_chunk);
int tc_init(TcState* t, const afq_ctx_dev& c, const afq_hamiltonian& h, const double* rccat,
            int nw_chunk, char* ws, cudaStream_t st);
int tc_force_bias(TcState& t, const afq_ctx_dev& c, const double2* green, double2* out,
                  double alpha, cudaStream_t st);
int tc_energy(TcState& t, const afq_ctx_dev& c, const double2* green, double2* epart,
              double2* out, cudaStream_t st);
int tc_propagate_chunk(TcState& t, const afq_ctx_dev& c, int w0, int nwc, const double2* xt,
                       void* wu, void* wd, cudaStream_t st);
int tc_orthonormalize(TcState& t, const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st);

}  // namespace afq

// Mixed-precision path: FP32 walkers, FP16 (or BF16) tcgen05 contractions with hi/lo
// split correction, FP32 small dense algebra with FP64 log-determinants, FP64 weights and
// energy sums. Operand layouts (16-bit, row-major, K contiguous; "hi/lo" = x ~ hi + lo):
//   g_fb   [2 nw][ldfb]       rows (w, re/im), cols (spin block, i, p) = G_s[i][p] * 2^e_w
//   rc_fb  [nchol][ldfb]      rows g, cols (spin block, i, p) = rot_chol_s[g][i][p] * 2^e_g
//   xt     [2 nw][ldg]        rows (w, re/im), cols g = shifted fields
//   lop    [norb * nq][ldg]   rows (p, q) (q padded to nq), cols g = chol_g[p][q]; with
//                             symmetric vectors rows are the packed (p, q) pairs of sym_decode
//   vbuf   [nwc][mr][2 nq]    per walker [Vr | Vi] (rows >= norb and q >= norb zero); mr = 128,
//                             or 256 for norb > 128
//   eop[s] [mr][nk]           exp_h1_s - I (rows >= norb zero)
//   wt[s], acc[s] [nw * R_s][nk]  rows (w, 2k + re/im), cols p: walker / Taylor sum
//   t0[s]  [nw][NT_s][2 nq]   Taylor B operand: row 2k = [Tr | -Ti], row 2k+1 = [Ti | Tr]
//   u[b]   [kb][ldkb]         rows (i, q), cols (k, p): sum_g rot_chol_b[g,i,p] rot_chol_b[g,k,q]
//                             (exchange matrix, scaled by a power of two)
//   g_blk[b] [2 nw][ldkb]     Green operand of spin block b alone (UHF; RHF uses g_fb)
//   rc_blk[b] [nchol][ldkb]   rot_chol of spin block b alone (UHF; RHF uses rc_fb)
#pragma once
#include "afq_gemm.cuh"
#include "afq_gemm_split.cuh"
#include "afq_kernels.cuh"

namespace afq {

// accuracy options of the mixed path (afq_dims.mixed_config; 0 selects kMixedDefault)
enum MixedBits : int32_t {
  kFbDyn = 1 << 0,      // force bias: lo part of G
  kFbStat = 1 << 1,     // force bias: lo part of rot_chol
  kVhsDyn = 1 << 2,     // vhs: lo part of the shifted fields
  kVhsStat = 1 << 3,    // vhs: lo part of chol
  kExpDyn = 1 << 4,     // exp_h1 products: lo part of the walker / Taylor sum
  kExpStat = 1 << 5,    // exp_h1 products: lo part of exp_h1 - I
  kEneDyn = 1 << 6,     // energy: lo part of G
  kEneStat = 1 << 7,    // energy: lo part of rot_chol
  kTaylorShift = 8,     // bits 8..10: Taylor products computed with split operands
  kUseBf16 = 1 << 11,   // bf16 operands instead of fp16
  kDrainShift = 12,     // bits 12..14: K tiles per truncated accumulation run in the force
                        // bias, vhs and exchange GEMMs (0: default, 7: no draining)
  kDiagChol = 1 << 15,  // every Cholesky vector is a diagonal matrix (on-site lattice terms):
                        // exp(vhs) W1 is a per-row polynomial scale, no vhs GEMM / Taylor MMA
  kLegacyTaylor = 1 << 16,  // separate exp_h1 GEMMs around the Taylor kernel (k_taylor_tc)
                            // instead of the fused propagation kernel
  kSymChol = 1 << 17,   // every Cholesky vector is a symmetric matrix: the vhs GEMM computes
                        // V only for q >= 32 floor(p / 32) and the fused kernel mirrors the rest
  kExplicit = 1 << 30,  // set by callers that pass an explicit configuration
};
constexpr int kDrainDefault = 2;  // K tiles per drained run unless the configuration says
constexpr int32_t kMixedDefault = kFbDyn | kFbStat | kVhsDyn | kVhsStat | kExpDyn | kExpStat |
                                  kEneDyn | kEneStat | (2 << kTaylorShift);

// Symmetric Cholesky vectors (V = V^T): row p of V, in row blocks of 32 (b = p / 32), keeps
// the columns q >= 32 b only; the packed column of (p, q) is
// sym_base(b) + (p - 32 b) (nq - 32 b) + (q - 32 b). Every row run is a multiple of 32 long
// and starts at a multiple of 32.
__host__ __device__ inline int sym_rows(int n, int b) { return n - 32 * b < 32 ? n - 32 * b : 32; }
__host__ __device__ inline int sym_total(int n, int nq) {
  int t = 0;
  for (int b = 0; 32 * b < n; ++b) t += sym_rows(n, b) * (nq - 32 * b);
  return t;
}
// (p, q) of packed column c < sym_total(n, nq)
__host__ __device__ inline void sym_decode(int n, int nq, int c, int& p, int& q) {
  for (int b = 0; 32 * b < n; ++b) {
    const int len = nq - 32 * b, size = sym_rows(n, b) * len;
    if (c < size) {
      p = 32 * b + c / len;
      q = 32 * b + c % len;
      return;
    }
    c -= size;
  }
  p = n;  // past the end
  q = 0;
}

struct TcState {
  int ready;
  int cfg;
  bool bf16;
  int n, nq, nk, ldfb, ldg, kfb;
  int nw, nwc;
  int nslab, nblk;          // walker slabs, Green blocks
  int o_slab[2], R[2], wpt[2], bn_w[2], NT[2];
  int o_blk[2], kb[2], ldkb[2], mt_z[2];  // mt_z: exchange partial slots per walker (K splits x 32-row groups)
  int z_ks[2];                              // exchange GEMM K splits per spin block
  int fb_bn, fb_ntiles;
  int fb_ks, fb_npad;       // force bias on the split GEMM: K splits, padded N of the partials
  float* fb_part;           // [fb_ks][2 nw][fb_npad] K-split partials of the force bias
  SplitMaps m_fb_split;     // force-bias operand planes (B boxes of 256 rows)
  // static operands [hi, lo]
  uint16_t *rc_fb[2], *lop[2], *eop[2][2], *u[2][2], *rc_blk[2][2];
  float* rc_inv;            // [nchol] 2^-e_g for rc_fb
  float* rc_blk_inv[2];     // [nchol] 2^-e_g for rc_blk
  float u_inv[2];           // 2^-e of u[b]
  float* u_tmp;             // FP32 scratch for building u (set-up only)
  // dynamic operands
  uint16_t *g_fb[2], *xt[2], *vbuf[2], *wt[2][2], *acc[2][2], *t0[2][2], *g_blk[2][2];
  float* g_inv;             // [nw] 2^-e_w
  double2* ene1;            // [nw]
  double2* part_shift;      // [nw][fb_ntiles]
  double2* part_fbt;        // [nw][fb_ntiles]
  double2* c_out;           // [nblk][nw][nchol]
  double2* exc_part;        // [nblk][nw][mt_z]
  const float* trial32[2];  // [norb][o_s] trial in FP32
  const float* rh1_32[2];   // [o_b][norb] rot_h1 in FP32
  int* status;              // device word: nonzero after a pipeline timeout (2, 1) or a
                            // non-diagonal Cholesky vector under kDiagChol (4)
  float* dchol;             // kDiagChol: [nchol][n] diagonals of the Cholesky vectors
  // tensor maps
  GemmMaps m_fb, m_vhs, m_e1[2], m_e2[2], m_c[2];
  SplitMaps m_zs[2];  // exchange: A = U planes, B = Green operand planes
  CUtensorMap m_vt[2][2];   // Taylor: vbuf hi/lo (unused index for slab)
  CUtensorMap m_t0[2][2];   // Taylor: t0[s] hi/lo
  bool fused;               // fused propagation kernel (norb <= 128, <= 32 orbitals per slab)
  bool sym;                 // symmetric Cholesky vectors on the fused path: packed vhs columns
  bool wide;                // norb > 128: streamed propagation kernel (k_prop_wide)
  int mr;                   // rows of the per-walker V and exp_h1 - I operands (128 or 256)
  CUtensorMap m_ew[2][2];   // wide propagation: exp_h1[s] - I hi/lo, boxes of 128 rows
  int n_vcols;              // vhs GEMM columns: norb * nq, or the packed count with sym
  int n_fb_terms, n_vhs_terms, n_e_terms, n_en_terms, taylor_split;
  int drain;                // K tiles per drained accumulation run (0: not drained)
  int num_sms;              // persistent grid size
  SplitMaps m_vhs_split;    // vhs operand planes for the persistent split GEMM
};

size_t tc_workspace_bytes(const afq_ctx_dev& c, int nw_chunk, int32_t mixed_config);
int tc_init(TcState* t, const afq_ctx_dev& c, const afq_hamiltonian& h, const double* rccat,
            int nw_chunk, int32_t mixed_config, char* ws, cudaStream_t st);
// Overlap (when ovl is not NULL); with write_ops or for_propagation also G, its 16-bit
// operands, ene1 and the walker operand of the exp_h1 products, all in one launch.
int tc_green(TcState& t, const afq_ctx_dev& c, const void* wu, const void* wd, double2* ovl,
             bool write_ops, cudaStream_t st, bool for_propagation = false);
int tc_force_bias(TcState& t, const afq_ctx_dev& c, double2* out, cudaStream_t st);
int tc_energy(TcState& t, const afq_ctx_dev& c, double2* out, cudaStream_t st);
int tc_field_shifts(TcState& t, const afq_ctx_dev& c, const double* fields, cudaStream_t st);
int tc_propagate_walkers(TcState& t, const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st);
int tc_weights(TcState& t, const afq_ctx_dev& c, const double2* ovl_new, double2* ovl,
               double* weights, double* scalars, cudaStream_t st);
int tc_orthonormalize(TcState& t, const afq_ctx_dev& c, void* wu, void* wd, cudaStream_t st);

}  // namespace afq

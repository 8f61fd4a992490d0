/*
 * afqmc_gb300_testing.h - test hooks of libafqmc_gb300.so.
 *
 * These entry points have no counterpart in the reference: they expose single kernels of
 * the mixed-precision path so that tests can compare each one with a PyTorch FP32
 * computation of the same operation. Same conventions as afqmc_gb300.h (device pointers,
 * stream-ordered, 0 on success, afq_last_error() on failure).
 */
#ifndef AFQMC_GB300_TESTING_H
#define AFQMC_GB300_TESTING_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* D[M,N] (fp32, row-major) = sum_{t < nterms} A_t[M,K] * B_t[N,K]^T on the tcgen05 tensor
 * cores. A_t = a + t*a_term_stride, B_t = b + t*b_term_stride (elements); rows of A and B
 * are K-major with leading dimensions lda/ldb (multiples of 8). bf16 != 0: bfloat16 inputs,
 * else float16. bn: output tile width (multiple of 16, <= 256; <= 160 with drain).
 * drain: 0 = one accumulator; d > 0 = a fresh accumulator every d K tiles, summed with
 * round-to-nearest. *status (device int) becomes nonzero if a pipeline wait timed out. */
int afq_test_gemm_f16(const void* a, const void* b, int nterms, long a_term_stride,
                      long b_term_stride, float* d, int M, int N, int K, int lda, int ldb,
                      int bf16, int bn, int drain, int* status, void* stream);

/* D[M,N] (fp32) = A_hi B_hi^T + A_lo B_hi^T + A_hi B_lo^T with the persistent split GEMM
 * (128 x 256 tiles per CTA; with M > 128, 256 x 256 tiles per CTA pair unless pairs are
 * switched off). a_lo / b_lo may be NULL (term left out). All planes K-major with leading
 * dimensions lda / ldb (multiples of 8). drain: K tiles per accumulation run, 0 = one run
 * over all of K. */
int afq_test_gemm_split(const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo,
                        float* d, int M, int N, int K, int lda, int ldb, int bf16, int drain,
                        int* status, void* stream);

/* Library-wide choice of the split GEMM's form for every later launch (library GEMMs
 * included): enable = 1 CTA pairs (the default), 0 one CTA per tile, < 0 no change.
 * Returns the previous setting. Not thread-safe: for tests and timing comparisons. */
int afq_test_split_pairs(int enable);

#ifdef __cplusplus
}
#endif
#endif

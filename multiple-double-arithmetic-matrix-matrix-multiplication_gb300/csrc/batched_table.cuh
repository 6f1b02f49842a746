// The problem table of the batched slice-digit GEMM (batched.cu) and the
// lookup of a block's problem, shared by the planning code and the stage
// kernels of batched_w{4,6,10,16}.cu.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace mdgi {

struct BatchProblem {
  int p, s, D, m, n, k, Mp, Np, Kp;
  const double *A, *B;
  double *C;
  int lda, ldb, ldc;
  int offE, offF;  // row maxima / exponents of A at offE, of B's columns at offF
  __nv_bfloat16 *dA, *dB;
  int *chunks;
  long long plane_a, plane_b, plane_c;
  int rowblk_begin;  // absmax of A: blocks of 256 rows
  int colblk_begin;  // absmax of B: blocks of 256 rows of B (k)
  int digA_begin;    // digits of A: rows Mp
  int digB_begin;    // digits of B: rows Np
  int out_begin;     // renorm: rows m
};

// First problem whose prefix count (Field: 0 row blocks of A, 1 row blocks
// of B, 2 digit rows of A, 3 digit rows of B, 4 output rows) is <= x.
template <int Field>
__device__ __forceinline__ int find_problem(const BatchProblem *pr, int count, int x) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const int b = Field == 0 ? pr[mid].rowblk_begin
                  : Field == 1 ? pr[mid].colblk_begin
                  : Field == 2 ? pr[mid].digA_begin
                  : Field == 3 ? pr[mid].digB_begin
                               : pr[mid].out_begin;
    if (b <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Digits of the A and B of one P group (digit-row blocks from xa / xb),
// and the renormalisation of its C (`rows` output rows from x0), with NW-word
// integers (instantiated in batched_w{4,6,10,16}.cu).
template <int NW>
int launch_batch_digits(const BatchProblem *pr, int count, const int *E, dim3 ga, dim3 gb,
                        int xa, int xb, cudaStream_t st);
template <int NW>
int launch_batch_renorm(int p, const BatchProblem *pr, int count, const int *E, int rows,
                        int max_n, int x0, cudaStream_t st);

}  // namespace mdgi

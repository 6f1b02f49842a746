// The problem table of the batched slice-digit GEMM (batched.cu) and the
// lookup of a block's problem, shared by the planning code and the stage
// kernels of batched_w{4,6,10,16}.cu.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace mdgi {

// Integer words of the digit and renormalisation stages for P limbs at the
// default digit count (words_for(s, 1) and words_for(1, D), s = D).
__host__ __device__ constexpr int batch_words(int p) {
  return p == 2 ? 4 : p == 4 ? 6 : p == 8 ? 10 : 16;
}

// Columns per thread of the renormalisation for P limbs (vector loads of
// the chunk planes; fewer for the wider integers to bound registers).
__host__ __device__ constexpr int batch_cols_per_thread(int p) {
  return p <= 4 ? 4 : p == 8 ? 2 : 1;
}

// Every stage kernel runs over a flat list of work units (thread blocks);
// each problem owns a contiguous range of units in every list.
//   scale:  ceil(m / 8) blocks of 8 rows of A, then ceil(n / 32) blocks of
//           32 columns of B
//   digits: Mp x ceil(Kp / 128) blocks of A's digit rows, then
//           Np x ceil(Kp / 128) of B's
//   renorm: one row of blocks per output row (m rows), per limb count
struct BatchProblem {
  int p, s, D, m, n, k, Mp, Np, Kp;
  const double *A, *B;
  double *C;
  int lda, ldb, ldc;
  int offE, offF;  // exponents of A's rows at offE, of B's columns at offF
  __nv_bfloat16 *dA, *dB;
  int *chunks;
  long long plane_a, plane_b, plane_c;
  int scale_begin, scale_b_off;  // first scale unit; units of A's rows
  int dig_begin, dig_b_off;      // first digit unit; units of A's digit rows
  int out_begin;                 // first output row among those of its P
};

enum { kScaleUnits = 0, kDigitUnits = 1, kRenormUnits = 2 };

// The problem whose range of units (Field) holds unit x: the last problem
// whose first unit is <= x.
template <int Field>
__device__ __forceinline__ int find_problem(const BatchProblem *pr, int count, int x) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const int b = Field == kScaleUnits ? pr[mid].scale_begin
                  : Field == kDigitUnits ? pr[mid].dig_begin
                                         : pr[mid].out_begin;
    if (b <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One launch each over every problem of the batch for the exponents and
// the digits: NWMAX is the widest integer of the batch (4, 6, 10 or 16
// words, the P of its widest problem); the kernels switch on each problem's
// P.  The renormalisation: one launch per P over that P's output rows
// [row0, row0 + rows), columns up to the widest n of the group.  (Instantiated in batched_w{4,6,10,16}.cu.)
template <int NWMAX>
int launch_batch_scale(const BatchProblem *pr, int count, int units, int *exps, cudaStream_t st);
template <int NWMAX>
int launch_batch_digits(const BatchProblem *pr, int count, int units, const int *exps,
                        cudaStream_t st);
template <int P>
int launch_batch_renorm(const BatchProblem *pr, int count, int row0, int rows, int max_n,
                        const int *exps, cudaStream_t st);

}  // namespace mdgi

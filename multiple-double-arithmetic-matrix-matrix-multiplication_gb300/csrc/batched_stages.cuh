// Exponent, digit and renormalisation kernels of the batched slice-digit
// GEMM.  The exponent and digit kernels run once over every problem of the
// batch, whatever its P: each block finds its problem in the table
// (batched_table.cuh) and branches on the problem's P to the integer width
// that P needs; the branches of wider integers than the batch holds are not
// compiled into the instance that is launched (NWMAX).  The
// renormalisation runs once per limb count present.  One translation unit
// per width (batched_w{4,6,10,16}.cu) so that the wide-integer code
// compiles in parallel.
#pragma once

#include "batched_table.cuh"
#include "slice_stages.cuh"

namespace mdgi {

// Row exponents of A (one warp per row) and column exponents of B (32
// columns x 8 row groups per block), each from the maximum over the whole
// row / column of sum_l |x_l| -- the value, order of additions and rounding
// of the single-problem absmax kernel -- so no atomics and no cleared
// maxima are needed.  (A template only so that each translation unit
// holds its own instance.)
template <int NWMAX>
__global__ void __launch_bounds__(256)
    scale_all(const BatchProblem *__restrict__ pr, int count, int *__restrict__ exps) {
  const int u = blockIdx.x;
  const BatchProblem &b = pr[find_problem<kScaleUnits>(pr, count, u)];
  const int lu = u - b.scale_begin;
  const int P = b.p;
  if (lu < b.scale_b_off) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = 8 * lu + warp;
    if (r >= b.m) return;
    unsigned long long mx = 0;
    for (int c = lane; c < b.k; c += 32)
      mx = umax64(mx, abs_sum_bits(b.A + ((size_t)r * b.lda + c) * P, P));
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) exps[b.offE + r] = scale_exp(__longlong_as_double((long long)mx));
  } else {
    __shared__ unsigned long long red[8][32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c = 32 * (lu - b.scale_b_off) + tx;
    unsigned long long mx = 0;
    if (c < b.n)
      for (int r = ty; r < b.k; r += 8)
        mx = umax64(mx, abs_sum_bits(b.B + ((size_t)r * b.ldb + c) * P, P));
    red[ty][tx] = mx;
    __syncthreads();
    if (ty == 0 && c < b.n) {
#pragma unroll
      for (int y = 1; y < 8; ++y) mx = umax64(mx, red[y][tx]);
      exps[b.offF + c] = scale_exp(__longlong_as_double((long long)mx));
    }
  }
}

// Digits of one unit: a digit row (row of A's planes or, transposed, column
// of B's) over 128 k-positions, one per thread (one element per thread
// keeps the wide integers of the octo- and hexa-double branches few, so
// the merged kernel's register count stays near the single-width ones').
// Only the valid rows and k-positions: the padding of every plane was
// cleared when the plan was made and nothing writes it afterwards.
template <int NW>
__device__ __forceinline__ void digits_unit(const BatchProblem &b, const int *exps, int lu) {
  const int kblocks = (b.k + 127) / 128;
  const bool side_b = lu >= b.dig_b_off;
  if (side_b) lu -= b.dig_b_off;
  const int prow = lu / kblocks, pc = (lu - prow * kblocks) * 128 + (int)threadIdx.x;
  if (pc >= b.k) return;
  if (!side_b)
    digits_elem<NW>(b.p, b.s, b.m, b.k, b.A, b.lda, exps + b.offE, 0, b.dA, b.Kp, b.plane_a,
                    b.Mp, b.Kp, prow, pc);
  else
    digits_elem<NW>(b.p, b.s, b.n, b.k, b.B, b.ldb, exps + b.offF, 1, b.dB, b.Kp, b.plane_b,
                    b.Np, b.Kp, prow, pc);
}

template <int NWMAX>
__global__ void __launch_bounds__(128)
    digits_all(const BatchProblem *__restrict__ pr, int count, const int *__restrict__ exps) {
  const int u = blockIdx.x;
  const BatchProblem &b = pr[find_problem<kDigitUnits>(pr, count, u)];
  const int lu = u - b.dig_begin;
  switch (batch_words(b.p)) {
    case 4: digits_unit<4>(b, exps, lu); break;
    case 6: if constexpr (NWMAX >= 6) digits_unit<6>(b, exps, lu); break;
    case 10: if constexpr (NWMAX >= 10) digits_unit<10>(b, exps, lu); break;
    default: if constexpr (NWMAX >= 16) digits_unit<16>(b, exps, lu); break;
  }
}

// The renormalisation runs one launch per P (a kernel holding the bodies of
// several widths measured 15 % slower): block (x, y) takes output row
// row0 + x of the P group, columns 128 V y .. +128 V - 1.
template <int P>
__global__ void __launch_bounds__(128)
    renorm_p(const BatchProblem *__restrict__ pr, int count, const int *__restrict__ exps,
             int row0) {
  constexpr int V = batch_cols_per_thread(P);
  const int x = row0 + (int)blockIdx.x;
  const BatchProblem &b = pr[find_problem<kRenormUnits>(pr, count, x)];
  const int r = x - b.out_begin, c0 = ((int)blockIdx.y * 128 + (int)threadIdx.x) * V;
  renorm_elems<P, batch_words(P), V>(b.s, b.D, b.Kp / 64, b.m, b.n, b.chunks, b.plane_c, b.Np,
                                     exps + b.offE, exps + b.offF, b.C, b.ldc, r, c0);
}

template <int NWMAX>
int launch_batch_scale(const BatchProblem *pr, int count, int units, int *exps, cudaStream_t st) {
  if (units == 0) return MDG_SUCCESS;
  scale_all<NWMAX><<<units, 256, 0, st>>>(pr, count, exps);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

template <int NWMAX>
int launch_batch_digits(const BatchProblem *pr, int count, int units, const int *exps,
                        cudaStream_t st) {
  if (units == 0) return MDG_SUCCESS;
  digits_all<NWMAX><<<units, 128, 0, st>>>(pr, count, exps);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

template <int P>
int launch_batch_renorm(const BatchProblem *pr, int count, int row0, int rows, int max_n,
                        const int *exps, cudaStream_t st) {
  if (rows == 0 || max_n == 0) return MDG_SUCCESS;
  constexpr int V = batch_cols_per_thread(P);
  renorm_p<P><<<dim3(rows, ceil_div(ceil_div(max_n, V), 128)), 128, 0, st>>>(pr, count, exps,
                                                                             row0);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

}  // namespace mdgi

// Digit and renormalisation kernels of the batched slice-digit GEMM, one
// translation unit per integer width (batched_w{4,6,10,16}.cu) so that the
// wide-integer code compiles in parallel.
#pragma once

#include "batched_table.cuh"
#include "slice_stages.cuh"

namespace mdgi {

// Blocks x0 + blockIdx.x of the problems' digit rows (one P group of the
// table, which the plan sorts by P).
template <int NW, int Side>
__global__ void digits_b(const BatchProblem *__restrict__ pr, int count, const int *__restrict__ E,
                         int x0) {
  const int x = x0 + (int)blockIdx.x;
  const int q = find_problem<Side == 0 ? 2 : 3>(pr, count, x);
  const BatchProblem &b = pr[q];
  const int pc = blockIdx.y * blockDim.x + threadIdx.x;
  if (pc >= b.Kp) return;
  if (Side == 0)
    mdgi::digits_elem<NW>(b.p, b.s, b.m, b.k, b.A, b.lda, E + b.offE, 0, b.dA, b.Kp, b.plane_a,
                          b.Mp, b.Kp, x - b.digA_begin, pc);
  else
    mdgi::digits_elem<NW>(b.p, b.s, b.n, b.k, b.B, b.ldb, E + b.offF, 1, b.dB, b.Kp, b.plane_b,
                          b.Np, b.Kp, x - b.digB_begin, pc);
}

// Output rows x0 + blockIdx.x of one P group, V adjacent columns per thread
// (chunk planes are Np wide with Np a multiple of 256 and start 256-byte
// aligned, so V-wide loads stay aligned).
template <int P, int NW, int V>
__global__ void __launch_bounds__(128) renorm_b(const BatchProblem *__restrict__ pr, int count,
                                                const int *__restrict__ E, int x0) {
  const int x = x0 + (int)blockIdx.x;
  const int q = find_problem<4>(pr, count, x);
  const BatchProblem &b = pr[q];
  const int r = x - b.out_begin, c = (blockIdx.y * blockDim.x + threadIdx.x) * V;
  mdgi::renorm_elems<P, NW, V>(b.s, b.D, b.Kp / 64, b.m, b.n, b.chunks, b.plane_c, b.Np,
                               E + b.offE, E + b.offF, b.C, b.ldc, r, c);
}

template <int NW>
int launch_batch_digits(const BatchProblem *pr, int count, const int *E, dim3 ga, dim3 gb,
                        int xa, int xb, cudaStream_t st) {
  digits_b<NW, 0><<<ga, 128, 0, st>>>(pr, count, E, xa);
  MDG_TRY_LAUNCH();
  digits_b<NW, 1><<<gb, 128, 0, st>>>(pr, count, E, xb);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

template <int P, int NW>
int launch_renorm_group(const BatchProblem *pr, int count, const int *E, int rows, int max_n,
                        int x0, cudaStream_t st) {
  constexpr int V = NW <= 6 ? 4 : NW <= 10 ? 2 : 1;
  const dim3 g(rows, ceil_div(ceil_div(max_n, V), 128));
  renorm_b<P, NW, V><<<g, 128, 0, st>>>(pr, count, E, x0);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

template <int NW>
int launch_batch_renorm(int p, const BatchProblem *pr, int count, const int *E, int rows,
                        int max_n, int x0, cudaStream_t st) {
  switch (p) {
    case 2: return launch_renorm_group<2, NW>(pr, count, E, rows, max_n, x0, st);
    case 4: return launch_renorm_group<4, NW>(pr, count, E, rows, max_n, x0, st);
    case 8: return launch_renorm_group<8, NW>(pr, count, E, rows, max_n, x0, st);
    default: return launch_renorm_group<16, NW>(pr, count, E, rows, max_n, x0, st);
  }
}

}  // namespace mdgi

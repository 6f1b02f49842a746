// Digit and renormalisation kernels of the batched slice-digit GEMM, one
// translation unit per integer width (batched_w{4,6,10,16}.cu) so that the
// wide-integer code compiles in parallel.
#pragma once

#include "batched_table.cuh"
#include "slice_stages.cuh"

namespace mdgi {

template <int NW, int Side>
__global__ void digits_b(const BatchProblem *__restrict__ pr, int count, const int *__restrict__ E) {
  const int q = find_problem<Side == 0 ? 2 : 3>(pr, count, blockIdx.x);
  const BatchProblem &b = pr[q];
  const int pc = blockIdx.y * blockDim.x + threadIdx.x;
  if (pc >= b.Kp) return;
  if (Side == 0)
    mdgi::digits_elem<NW>(b.p, b.s, b.m, b.k, b.A, b.lda, E + b.offE, 0, b.dA, b.Kp, b.plane_a,
                          b.Mp, b.Kp, blockIdx.x - b.digA_begin, pc);
  else
    mdgi::digits_elem<NW>(b.p, b.s, b.n, b.k, b.B, b.ldb, E + b.offF, 1, b.dB, b.Kp, b.plane_b,
                          b.Np, b.Kp, blockIdx.x - b.digB_begin, pc);
}

template <int NW>
__global__ void __launch_bounds__(128) renorm_b(const BatchProblem *__restrict__ pr, int count,
                                                const int *__restrict__ E) {
  const int q = find_problem<4>(pr, count, blockIdx.x);
  const BatchProblem &b = pr[q];
  const int r = blockIdx.x - b.out_begin, c = blockIdx.y * blockDim.x + threadIdx.x;
  const int KB = b.Kp / 64;
  switch (b.p) {
    case 2:
      mdgi::renorm_elems<2, NW, 1>(b.s, b.D, KB, b.m, b.n, b.chunks, b.plane_c, b.Np,
                                   E + b.offE, E + b.offF, b.C, b.ldc, r, c);
      break;
    case 4:
      mdgi::renorm_elems<4, NW, 1>(b.s, b.D, KB, b.m, b.n, b.chunks, b.plane_c, b.Np,
                                   E + b.offE, E + b.offF, b.C, b.ldc, r, c);
      break;
    case 8:
      mdgi::renorm_elems<8, NW, 1>(b.s, b.D, KB, b.m, b.n, b.chunks, b.plane_c, b.Np,
                                   E + b.offE, E + b.offF, b.C, b.ldc, r, c);
      break;
    default:
      mdgi::renorm_elems<16, NW, 1>(b.s, b.D, KB, b.m, b.n, b.chunks, b.plane_c, b.Np,
                                    E + b.offE, E + b.offF, b.C, b.ldc, r, c);
      break;
  }
}

template <int NW>
int launch_batch_digits(const BatchProblem *pr, int count, const int *E, dim3 ga, dim3 gb,
                        cudaStream_t st) {
  digits_b<NW, 0><<<ga, 128, 0, st>>>(pr, count, E);
  MDG_TRY_LAUNCH();
  digits_b<NW, 1><<<gb, 128, 0, st>>>(pr, count, E);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

template <int NW>
int launch_batch_renorm(const BatchProblem *pr, int count, const int *E, dim3 gr,
                        cudaStream_t st) {
  renorm_b<NW><<<gr, 128, 0, st>>>(pr, count, E);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

}  // namespace mdgi

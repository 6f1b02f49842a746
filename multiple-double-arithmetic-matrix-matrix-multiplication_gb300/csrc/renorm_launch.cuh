// Renormalisation kernels of the slice-digit form, instantiated per limb
// count P in renorm_p{2,4,8,16}.cu so that the wide-integer code of the
// sixteen (P, words) pairs compiles in parallel translation units.
#pragma once

#include "common.cuh"
#include "slice_common.cuh"
#include "slice_stages.cuh"
#include "slice_tc.cuh"

namespace mdgi {

template <int P, int NW, int V, bool PAIRED = false>
__global__ void __launch_bounds__(128)
    renorm_kernel(int s, int D, int KB, int m, int n, const int *__restrict__ chunks,
                  long long plane_c, int ldcd, const int *__restrict__ E,
                  const int *__restrict__ F, double *__restrict__ C, int ldc) {
  renorm_elems<P, NW, V, PAIRED>(s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc,
                                 blockIdx.y, (blockIdx.x * blockDim.x + threadIdx.x) * V);
}

// V columns per thread: 4 only for NW <= 6, 2 only for NW <= 10 (the
// launcher never asks for more), so wider pairs are not instantiated.
// Paired chunk loads (renorm_elems) where some diagonal spans two or more
// chunks, for 6 words with 4 columns a thread, where they measured faster
// (quad-double 8192^3: 7.6 -> 5.9 ms); with 4 or 10 words they were 8-11 %
// slower, and the 16-word variant (3.7 instead of 4.8 ms at hexa-double
// 2048^3) tripled the compile time of every limb count's unit.
template <int P, int NW>
int launch_renorm_w(int V, int s, int D, int KB, int m, int n, const int *chunks,
                    long long plane_c, int ldcd, const int *E, const int *F, double *C, int ldc,
                    cudaStream_t st) {
  int widest = 0;
  for (int d = 0; d < D; ++d) widest = std::max(widest, diag_chunks(d, s, KB));
  if constexpr (NW == 6) {
    if (widest >= 2 && V == 4) {
      renorm_kernel<P, NW, 4, true><<<dim3(ceil_div(ceil_div(n, 4), 128), m), 128, 0, st>>>(
          s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc);
      MDG_TRY_LAUNCH();
      return MDG_SUCCESS;
    }
  }
  if constexpr (NW <= 6) {
    if (V == 4) {
      renorm_kernel<P, NW, 4><<<dim3(ceil_div(ceil_div(n, 4), 128), m), 128, 0, st>>>(
          s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc);
      MDG_TRY_LAUNCH();
      return MDG_SUCCESS;
    }
  }
  if constexpr (NW <= 10) {
    if (V >= 2) {
      renorm_kernel<P, NW, 2><<<dim3(ceil_div(ceil_div(n, 2), 128), m), 128, 0, st>>>(
          s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc);
      MDG_TRY_LAUNCH();
      return MDG_SUCCESS;
    }
  }
  renorm_kernel<P, NW, 1><<<dim3(ceil_div(n, 128), m), 128, 0, st>>>(s, D, KB, m, n, chunks,
                                                                     plane_c, ldcd, E, F, C, ldc);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

template <int P>
int launch_renorm_p(int NW, int V, int s, int D, int KB, int m, int n, const int *chunks,
                    long long plane_c, int ldcd, const int *E, const int *F, double *C, int ldc,
                    cudaStream_t st) {
  switch (NW) {
    case 4:
      return launch_renorm_w<P, 4>(V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    case 6:
      return launch_renorm_w<P, 6>(V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    case 10:
      return launch_renorm_w<P, 10>(V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    default:
      return launch_renorm_w<P, 16>(V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
  }
}

}  // namespace mdgi

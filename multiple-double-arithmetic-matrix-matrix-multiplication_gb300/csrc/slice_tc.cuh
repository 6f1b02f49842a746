// Internal interface of the slice-digit form (slice_tc.cu, diag_gemm_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace mdgi {

// Workspace layout of one slice-digit GEMM (byte offsets, 256-aligned).
struct SlicePlan {
  int p, s, D, m, n, k;
  int Mp, Np, Kp;  // padded to 128, 128, 64
  long long plane_a, plane_b, plane_c;  // elements between digit / diagonal planes
  size_t off_rowbits, off_colbits, off_E, off_F, off_dA, off_dB, off_Cd, total;
};

SlicePlan make_slice_plan(int p, int s, int D, int m, int n, int k);
int words_for(int s, int D);

int launch_scale_exponents(int p, int m, int n, int k, const double *A, int lda,
                           const double *B, int ldb, unsigned long long *rowbits,
                           unsigned long long *colbits, int *E, int *F, cudaStream_t st);
int launch_digits(int p, int s, int rows, int cols, const double *X, int ldx, const int *E,
                  int trans, void *planes, int ld_out, long long plane_stride, int rows_pad,
                  int cols_pad, cudaStream_t st);
// mma.sync engine (Mp % 128, Np % 64, Kp % 32)
int launch_diag_gemm_v0(int s, int D, int Mp, int Np, int Kp, const void *dA, const void *dB,
                        int ld, long long plane_a, long long plane_b, long long *Cd,
                        long long plane_c, int ldc, cudaStream_t st);
// tcgen05 engine (Mp % 128, Np % 128, Kp % 64)
int launch_diag_gemm_tc(int s, int D, int Mp, int Np, int Kp, const void *dA, const void *dB,
                        int ld, long long plane_a, long long plane_b, long long *Cd,
                        long long plane_c, int ldc, cudaStream_t st);
int launch_renorm(int p, int D, int m, int n, const long long *Cd, long long plane_c, int ldcd,
                  const int *E, const int *F, double *C, int ldc, cudaStream_t st);

// engine: 0 = mma.sync, 1 = tcgen05
int run_slice_gemm(const SlicePlan &pl, const double *A, int lda, const double *B, int ldb,
                   double *C, int ldc, void *ws, int engine, cudaStream_t st);

// Which engine mdg_gemm uses for the BF16 form (MDG_SLICE_ENGINE=0/1 overrides).
int default_engine();

}  // namespace mdgi

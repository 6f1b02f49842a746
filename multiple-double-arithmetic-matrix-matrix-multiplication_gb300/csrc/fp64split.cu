// Truncated slice convolution on FP64 tensor cores (DMMA m8n8k4).
//
// Cq[r][c][i] = sum_k sum_{j<=i} Aq[r][k][j] * Bq[k][c][i-j]
//
// This is the product the reference forms with one FP64 wmma GEMM against
// the block-Toeplitz matrix bigB2 (TCtest.cu:21-46, TCcuda.cu:79-95): its
// K index is the flattened (k, j) = k*pp + j, consumed four at a time by
// each m8n8k4 DMMA.  Here bigB2 is never formed.  For every output entry the
// DMMAs run over the same chunks (k, j0..j0+3), k outer, j0 inner, with the
// same four operands per chunk, and the chunks whose B part is zero for the
// whole tile (j0 > i) are skipped, which removes half of the reference's
// tensor work.  Operands are addressed through element strides: the
// reference's AoS layout (m x k x pp; four consecutive slices of one entry
// per 32-byte sector) for mdg_slice_conv, and slice planes (pp planes of
// m x k, the layout of the CPU convolution driver TCcudant.cpp:172-276) for
// mdg_plane_conv.
//
// GB300 note: FP64 tensor throughput on this part is a small fraction of its
// BF16 rate; this kernel is the baseline the BF16 slice form is measured
// against, and it is DMMA-bound, not memory-bound.
#include "common.cuh"

namespace {

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(c[0]), "+d"(c[1])
      : "d"(a), "d"(b));
}

// Element (row, k, slice) of A sits at row * ar + kk * ak + j * aj, and so
// on for B (k, column, slice) and C (row, column, slice).
struct ConvStrides {
  long long ar, ak, aj, bk, bc, bj, cr, cc, ci;
};

// Block: 4 warps as 2 x 2, tile 64 rows x 32 columns of diagonal i =
// blockIdx.z.  Warp tile: 32 rows (4 m8 tiles) x 16 columns (2 n8 tiles).
__global__ void __launch_bounds__(128)
    slice_conv_kernel(int pp, int m, int n, int k, const double *__restrict__ Aq,
                      const double *__restrict__ Bq, double *__restrict__ Cq,
                      const ConvStrides sd) {
  const int i = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int row_base = blockIdx.y * 64 + (warp >> 1) * 32;
  const int col_base = blockIdx.x * 32 + (warp & 1) * 16;
  double acc[4][2][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;

  int rows[4], cols[2];
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) rows[mi] = row_base + mi * 8 + g;
#pragma unroll
  for (int ni = 0; ni < 2; ++ni) cols[ni] = col_base + ni * 8 + g;

  for (int kk = 0; kk < k; ++kk) {
    for (int j0 = 0; j0 <= i; j0 += 4) {
      const int ja = j0 + t, jb = i - ja;
      double a[4], b[2];
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
        a[mi] = (rows[mi] < m && ja < pp)
                    ? __ldg(Aq + rows[mi] * sd.ar + kk * sd.ak + ja * sd.aj)
                    : 0.0;
#pragma unroll
      for (int ni = 0; ni < 2; ++ni)
        b[ni] = (cols[ni] < n && jb >= 0)
                    ? __ldg(Bq + kk * sd.bk + cols[ni] * sd.bc + jb * sd.bj)
                    : 0.0;
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 2; ++ni) dmma(acc[mi][ni], a[mi], b[ni]);
    }
  }
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) {
    const int r = row_base + mi * 8 + g;
    if (r >= m) continue;
#pragma unroll
    for (int ni = 0; ni < 2; ++ni)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int c = col_base + ni * 8 + 2 * t + h;
        if (c < n) Cq[r * sd.cr + c * sd.cc + i * sd.ci] = acc[mi][ni][h];
      }
  }
}

}  // namespace

namespace mdgi {

int launch_slice_conv(int pp, int m, int n, int k, const double *Aq, const double *Bq,
                      double *Cq, int planes, cudaStream_t st) {
  if (m == 0 || n == 0 || pp == 0) return MDG_SUCCESS;
  if (pp > 65535) return MDG_ERROR_INVALID_SIZE;
  const long long P = pp, M = m, N = n, K = k;
  const ConvStrides aos{K * P, P, 1, N * P, P, 1, N * P, P, 1};
  const ConvStrides soa{K, 1, M * K, N, 1, K * N, N, 1, M * N};
  dim3 grid(ceil_div(n, 32), ceil_div(m, 64), pp);
  slice_conv_kernel<<<grid, 128, 0, st>>>(pp, m, n, k, Aq, Bq, Cq, planes ? soa : aos);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

}  // namespace mdgi

// Plain multi-double GEMM on FP64 CUDA cores.
//
// Replaces matmulTCnt and its kernels ddmm/qdmm/odmm/hdmm (TCcuda.cu:119-302):
// one thread per entry C(r, c), the k loop of one P-double product followed
// by one P-double addition into the running sum, in increasing k.  The
// arithmetic is mdg_arith.h; with contraction off (this file is built with
// -fmad=false) every entry is bit for bit the reference's host result
// matmul{dd,qd,od,hd}f (TCcuda.cu:320-372).
//
// GB300 notes.  The work is FP64-bound: a quad-double product-and-add is a
// few hundred FP64 operations against 64 bytes of operands, so the kernel
// stages 16 x 16 tiles of A and B in shared memory (each operand loaded once
// per block, reused 16 times) and spends its time in the FP64 pipe.  Unlike
// the reference it takes any m, n, k (the reference requires n % nfrag == 0)
// and leading dimensions; a k tail never touches padding, so the sum is the
// reference's sum exactly.
#include "common.cuh"

namespace {

constexpr int T = 16;  // tile edge; 256 threads per block

template <int P>
__global__ void __launch_bounds__(T * T)
    plain_gemm_kernel(int m, int n, int k, const double *__restrict__ A, int lda,
                      const double *__restrict__ B, int ldb, double *__restrict__ C, int ldc) {
  extern __shared__ double smem[];
  double *As = smem;              // [T rows][T k][P]
  double *Bs = smem + T * T * P;  // [T k][T cols][P]
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * T + tx;
  const int row0 = blockIdx.y * T, col0 = blockIdx.x * T;
  const int r = row0 + ty, c = col0 + tx;
  double acc[P];
#pragma unroll
  for (int l = 0; l < P; ++l) acc[l] = 0.0;

  for (int k0 = 0; k0 < k; k0 += T) {
    const int kt = min(T, k - k0);
    for (int idx = tid; idx < T * T * P; idx += T * T) {
      const int i = idx / (T * P), rem = idx % (T * P);
      const int gr = row0 + i, gk = k0 + rem / P;
      As[idx] = (gr < m && gk < k) ? A[((size_t)gr * lda + gk) * P + rem % P] : 0.0;
      const int gk2 = k0 + i, gc = col0 + rem / P;
      Bs[idx] = (gk2 < k && gc < n) ? B[((size_t)gk2 * ldb + gc) * P + rem % P] : 0.0;
    }
    __syncthreads();
    for (int kk = 0; kk < kt; ++kk) {
      double a[P], b[P];
#pragma unroll
      for (int l = 0; l < P; ++l) {
        a[l] = As[(ty * T + kk) * P + l];
        b[l] = Bs[(kk * T + tx) * P + l];
      }
      mdg::madd<P>(acc, a, b);
    }
    __syncthreads();
  }
  if (r < m && c < n) {
#pragma unroll
    for (int l = 0; l < P; ++l) C[((size_t)r * ldc + c) * P + l] = acc[l];
  }
}

template <int P>
int launch(int m, int n, int k, const double *A, int lda, const double *B, int ldb, double *C,
           int ldc, cudaStream_t st) {
  const size_t smem = 2 * T * T * P * sizeof(double);
  // the attribute belongs to the current device: set it on every launch
  // (a host-side call of about a microsecond) rather than remember it
  MDG_TRY_CUDA(cudaFuncSetAttribute(plain_gemm_kernel<P>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(mdgi::ceil_div(n, T), mdgi::ceil_div(m, T)), block(T, T);
  plain_gemm_kernel<P><<<grid, block, smem, st>>>(m, n, k, A, lda, B, ldb, C, ldc);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

// ---------------------------------------------------------------- batched --
// One launch over the tiles of many problems with mixed P.  Each block finds
// its problem by binary search over the prefix sums of tile counts and runs
// the same tile loop as above.  Shared memory is sized for the largest P.

template <int P>
__device__ void plain_tile(const mdg_problem &pr, int tile, double *smem) {
  const int tiles_n = (pr.n + T - 1) / T;
  const int by = tile / tiles_n, bx = tile % tiles_n;
  double *As = smem, *Bs = smem + T * T * P;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * T + tx;
  const int row0 = by * T, col0 = bx * T, r = row0 + ty, c = col0 + tx;
  const int m = pr.m, n = pr.n, k = pr.k;
  double acc[P];
#pragma unroll
  for (int l = 0; l < P; ++l) acc[l] = 0.0;
  for (int k0 = 0; k0 < k; k0 += T) {
    const int kt = min(T, k - k0);
    for (int idx = tid; idx < T * T * P; idx += T * T) {
      const int i = idx / (T * P), rem = idx % (T * P);
      const int gr = row0 + i, gk = k0 + rem / P;
      As[idx] = (gr < m && gk < k) ? pr.A[((size_t)gr * pr.lda + gk) * P + rem % P] : 0.0;
      const int gk2 = k0 + i, gc = col0 + rem / P;
      Bs[idx] = (gk2 < k && gc < n) ? pr.B[((size_t)gk2 * pr.ldb + gc) * P + rem % P] : 0.0;
    }
    __syncthreads();
    for (int kk = 0; kk < kt; ++kk) {
      double a[P], b[P];
#pragma unroll
      for (int l = 0; l < P; ++l) {
        a[l] = As[(ty * T + kk) * P + l];
        b[l] = Bs[(kk * T + tx) * P + l];
      }
      mdg::madd<P>(acc, a, b);
    }
    __syncthreads();
  }
  if (r < m && c < n) {
#pragma unroll
    for (int l = 0; l < P; ++l) pr.C[((size_t)r * pr.ldc + c) * P + l] = acc[l];
  }
}

__global__ void __launch_bounds__(T * T)
    plain_batched_kernel(const mdg_problem *__restrict__ probs, int count,
                         const int *__restrict__ tile_starts, int total_tiles) {
  extern __shared__ double smem[];
  // persistent: blocks stride over the global tile list
  for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {  // last problem whose start <= t
      const int mid = (lo + hi + 1) >> 1;
      if (tile_starts[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const mdg_problem pr = probs[lo];
    const int tile = t - tile_starts[lo];
    switch (pr.p) {
      case 2: plain_tile<2>(pr, tile, smem); break;
      case 4: plain_tile<4>(pr, tile, smem); break;
      case 8: plain_tile<8>(pr, tile, smem); break;
      default: plain_tile<16>(pr, tile, smem); break;
    }
  }
}

}  // namespace

namespace mdgi {

int launch_plain_gemm(int p, int m, int n, int k, const double *A, int lda, const double *B,
                      int ldb, double *C, int ldc, cudaStream_t st) {
  if (m == 0 || n == 0) return MDG_SUCCESS;
  switch (p) {
    case 2: return launch<2>(m, n, k, A, lda, B, ldb, C, ldc, st);
    case 4: return launch<4>(m, n, k, A, lda, B, ldb, C, ldc, st);
    case 8: return launch<8>(m, n, k, A, lda, B, ldb, C, ldc, st);
    case 16: return launch<16>(m, n, k, A, lda, B, ldb, C, ldc, st);
  }
  return MDG_ERROR_INVALID_LIMBS;
}

int launch_plain_batched(const mdg_problem *dev_problems, int count, int max_p,
                         const int *dev_tile_starts, int total_tiles, cudaStream_t st) {
  if (total_tiles == 0) return MDG_SUCCESS;
  const size_t smem = 2 * T * T * (size_t)max_p * sizeof(double);
  MDG_TRY_CUDA(cudaFuncSetAttribute(plain_batched_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int dev = 0, sms = 0, per_sm = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  MDG_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MDG_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, plain_batched_kernel,
                                                             T * T, smem));
  const int grid = std::min(total_tiles, sms * std::max(per_sm, 1));
  plain_batched_kernel<<<grid, dim3(T, T), smem, st>>>(dev_problems, count, dev_tile_starts,
                                                       total_tiles);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

}  // namespace mdgi

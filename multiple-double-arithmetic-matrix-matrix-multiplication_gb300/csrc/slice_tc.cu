// The slice-digit form of the multi-double GEMM: split, diagonal GEMM on
// BF16 tensor cores, renormalisation.
//
// 1. scale exponents.  E[r] for each row of A and F[c] for each column of B
//    from the largest sum of absolute limbs; 2^E bounds every entry.
// 2. digits.  Each P-double a of row r becomes the integer
//       V = sum_l floor(a_l * 2^(S - E[r])),  S = 7 + 8 (s - 1),
//    written as s balanced base-256 digits d_0 (most significant) ..
//    d_{s-1} in [-128, 128].  Digit i of every entry forms one BF16 plane
//    (the integers up to 256 are exact in BF16).  A's planes are m x k,
//    B's are transposed to n x k so both operands are K-major.
// 3. diagonal GEMM.  C_d = sum_{i+j=d} A_i B_j^T for d < D.  One product
//    of two digits is at most 2^14, so an FP32 accumulator holds the exact
//    sum of 1024 of them (|sum| <= 2^24); every 1024 products (256 in the
//    mma.sync engine) the FP32 accumulator is flushed into 32-bit
//    integers, and every 2032 k-steps (130048 products) the integers are
//    stored as one "chunk" plane (|sum| < 2^31).  All sums are exact.
// 4. renormalisation.  W = sum_d C_d 256^(D-1-d), C_d the sum of the
//    chunks of diagonal d, is formed exactly in
//    wide integers and rounded to P limbs, each to nearest, scaled by
//    2^(E[r] + F[c] - 14 - 8 (D - 1)).
// The reference has no counterpart of steps 1-4; its split form cuts limbs
// into FP64 slices for FP64 DMMA (floatybits.cu, TCtest.cu).  The oracle's
// section 8 restates these steps on the CPU, and the GPU result equals it
// bit for bit.
#include "common.cuh"
#include "slice_common.cuh"
#include "slice_tc.cuh"
#include "slice_stages.cuh"

#include <cuda_bf16.h>

namespace {

using mdgi::wide_add_shifted;

// ------------------------------------------------------------ exponents --
__global__ void absmax_kernel(int P, int R, int Cn, const double *__restrict__ X, int ldx,
                              unsigned long long *rowbits, unsigned long long *colbits) {
  mdgi::absmax_block(P, R, Cn, X, ldx, rowbits, colbits, blockIdx.x, blockIdx.y);
}

__global__ void exps_kernel(int count, const unsigned long long *__restrict__ bits,
                            int *__restrict__ E) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) E[i] = mdgi::scale_exp(__longlong_as_double((long long)bits[i]));
}

// --------------------------------------------------------------- digits --
template <int NW>
__global__ void digits_kernel(int P, int s, int rows, int cols, const double *__restrict__ X,
                              int ldx, const int *__restrict__ E, int trans,
                              __nv_bfloat16 *__restrict__ planes, int ld_out,
                              long long plane_stride, int rows_pad, int cols_pad) {
  mdgi::digits_elem<NW>(P, s, rows, cols, X, ldx, E, trans, planes, ld_out, plane_stride,
                        rows_pad, cols_pad, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

// 4 k-positions per thread, consecutive threads on consecutive positions of
// one plane row, so plane stores are coalesced for A and B alike.
template <int NW>
__global__ void __launch_bounds__(256)
    digits4_kernel(int P, int s, int rows, int cols, const double *__restrict__ X, int ldx,
                   const int *__restrict__ E, int trans, __nv_bfloat16 *__restrict__ planes,
                   int ld_out, long long plane_stride, int rows_pad, int cols_pad) {
  mdgi::digits_elem4<NW>(P, s, rows, cols, X, ldx, E, trans, planes, ld_out, plane_stride,
                         rows_pad, cols_pad, blockIdx.y,
                         (blockIdx.x * blockDim.x + threadIdx.x) * 4);
}

// ---------------------------------------------------- diagonal GEMM v0 --
// mma.sync m16n8k16 BF16 -> FP32.  Block 128 x 64, 8 warps as 4 x 2, warp
// tile 32 x 32 (2 x 4 MMA tiles), K chunk 32 through shared memory.
constexpr int BM = 128, BN = 64, BK = 32, SK = BK + 8;
// k-steps of 64 per FP32 flush in this engine: 256 products, |sum| <= 2^22,
// the range of the exact_int conversion below
constexpr int V0_GROUP_STEPS = 4;

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// x is an integer-valued float with |x| <= 2^22: adding 1.5 * 2^23 puts it
// in the significand exactly; the bits minus those of 1.5 * 2^23 are x.
__device__ __forceinline__ int64_t exact_int(float x) {
  return (int64_t)(__float_as_int(x + 12582912.0f) - 0x4B400000);
}

__global__ void __launch_bounds__(256)
    diag_gemm_v0(int s, int D, int Kp, const __nv_bfloat16 *__restrict__ dA,
                 const __nv_bfloat16 *__restrict__ dB, int ld, long long plane_a,
                 long long plane_b, int *__restrict__ out, long long plane_c, int ldc) {
  __shared__ __align__(16) __nv_bfloat16 As[BM][SK];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][SK];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
  const int KB = Kp / 64;
  int chunk = 0;

  for (int d = 0; d < D; ++d) {
    float acc[2][4][4];
    int tot[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          acc[a][b][c] = 0.f;
          tot[a][b][c] = 0;
        }
    const int ilo = max(0, d - (s - 1));
    const int S = mdgi::diag_pairs(d, s) * KB;
    for (int step = 0; step < S; ++step) {
      const int i = ilo + step / KB, kb = step % KB;
      const __nv_bfloat16 *Ai = dA + i * plane_a + (size_t)row0 * ld + kb * 64;
      const __nv_bfloat16 *Bj = dB + (d - i) * plane_b + (size_t)col0 * ld + kb * 64;
      for (int half = 0; half < 2; ++half) {
#pragma unroll
        for (int v = tid; v < BM * BK / 8; v += 256) {
          const int r = v >> 2, cc = (v & 3) * 8;
          *reinterpret_cast<uint4 *>(&As[r][cc]) =
              *reinterpret_cast<const uint4 *>(Ai + (size_t)r * ld + half * BK + cc);
        }
        {
          const int r = tid >> 2, cc = (tid & 3) * 8;
          *reinterpret_cast<uint4 *>(&Bs[r][cc]) =
              *reinterpret_cast<const uint4 *>(Bj + (size_t)r * ld + half * BK + cc);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
          uint32_t af[2][4], bf[4][2];
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            const int r = wm + mt * 16 + g;
            af[mt][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 2 * t]);
            af[mt][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 2 * t]);
            af[mt][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 8 + 2 * t]);
            af[mt][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 8 + 2 * t]);
          }
#pragma unroll
          for (int nt = 0; nt < 4; ++nt) {
            const int c = wn + nt * 8 + g;
            bf[nt][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + 2 * t]);
            bf[nt][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + 8 + 2 * t]);
          }
#pragma unroll
          for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bf[nt]);
        }
        __syncthreads();
      }
      const bool group_end = (step % V0_GROUP_STEPS == V0_GROUP_STEPS - 1) || step == S - 1;
      const bool chunk_end = (step % mdgi::CHUNK_STEPS == mdgi::CHUNK_STEPS - 1) || step == S - 1;
      if (group_end) {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              tot[a][b][c] += (int)exact_int(acc[a][b][c]);
              acc[a][b][c] = 0.f;
            }
      }
      if (chunk_end) {
        int *o = out + (size_t)chunk * plane_c;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int r = row0 + wm + mt * 16 + g + h * 8;
              const int c = col0 + wn + nt * 8 + 2 * t;
              *reinterpret_cast<int2 *>(o + (size_t)r * ldc + c) =
                  make_int2(tot[mt][nt][2 * h], tot[mt][nt][2 * h + 1]);
              tot[mt][nt][2 * h] = tot[mt][nt][2 * h + 1] = 0;
            }
        ++chunk;
      }
    }
  }
}

}  // namespace

namespace mdgi {

int words_for(int s, int D) {
  // digits need S + 2 bits plus a word of headroom; W needs 8 (D - 1) + 64
  const int bits = std::max(7 + 8 * (s - 1) + 2, 8 * (D - 1) + 72);
  const int w = (bits + 63) / 64 + 1;
  if (w <= 4) return 4;
  if (w <= 6) return 6;
  if (w <= 10) return 10;
  if (w <= 16) return 16;
  return 0;
}

SlicePlan make_slice_plan(int p, int s, int D, int m, int n, int k) {
  SlicePlan pl{};
  pl.p = p;
  pl.s = s;
  pl.D = D;
  pl.m = m;
  pl.n = n;
  pl.k = k;
  pl.Mp = (int)align_up(std::max(m, 1), 256);
  pl.Np = (int)align_up(std::max(n, 1), 256);
  pl.Kp = (int)align_up(std::max(k, 1), 64);
  pl.chunks = total_chunks(s, D, pl.Kp / 64);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  pl.off_rowbits = take(sizeof(unsigned long long) * pl.Mp);
  pl.off_colbits = take(sizeof(unsigned long long) * pl.Np);
  pl.off_E = take(sizeof(int) * pl.Mp);
  pl.off_F = take(sizeof(int) * pl.Np);
  pl.plane_a = (long long)pl.Mp * pl.Kp;
  pl.plane_b = (long long)pl.Np * pl.Kp;
  pl.plane_c = (long long)pl.Mp * pl.Np;
  pl.off_dA = take(sizeof(__nv_bfloat16) * (size_t)s * pl.plane_a);
  pl.off_dB = take(sizeof(__nv_bfloat16) * (size_t)s * pl.plane_b);
  pl.off_Cd = take(sizeof(int) * (size_t)pl.chunks * pl.plane_c);
  pl.total = off;
  return pl;
}

int launch_scale_exponents(int p, int m, int n, int k, const double *A, int lda,
                           const double *B, int ldb, unsigned long long *rowbits,
                           unsigned long long *colbits, int *E, int *F, cudaStream_t st) {
  MDG_TRY_CUDA(cudaMemsetAsync(rowbits, 0, sizeof(unsigned long long) * std::max(m, 1), st));
  MDG_TRY_CUDA(cudaMemsetAsync(colbits, 0, sizeof(unsigned long long) * std::max(n, 1), st));
  if (k > 0 && m > 0) {
    dim3 grid(ceil_div(k, 32), ceil_div(m, 256));
    absmax_kernel<<<grid, dim3(32, 8), 0, st>>>(p, m, k, A, lda, rowbits, nullptr);
    MDG_TRY_LAUNCH();
  }
  if (k > 0 && n > 0) {
    dim3 grid(ceil_div(n, 32), ceil_div(k, 256));
    absmax_kernel<<<grid, dim3(32, 8), 0, st>>>(p, k, n, B, ldb, nullptr, colbits);
    MDG_TRY_LAUNCH();
  }
  if (m > 0) {
    exps_kernel<<<ceil_div(m, 256), 256, 0, st>>>(m, rowbits, E);
    MDG_TRY_LAUNCH();
  }
  if (n > 0) {
    exps_kernel<<<ceil_div(n, 256), 256, 0, st>>>(n, colbits, F);
    MDG_TRY_LAUNCH();
  }
  return MDG_SUCCESS;
}

int launch_digits(int p, int s, int rows, int cols, const double *X, int ldx, const int *E,
                  int trans, void *planes, int ld_out, long long plane_stride, int rows_pad,
                  int cols_pad, cudaStream_t st) {
  const int NW = words_for(s, 1);
  if (!NW) return MDG_ERROR_NOT_SUPPORTED;
  if (rows_pad == 0 || cols_pad == 0) return MDG_SUCCESS;
  auto *pl = reinterpret_cast<__nv_bfloat16 *>(planes);
  const bool vec = (cols_pad % 4 == 0) && (ld_out % 4 == 0) && (plane_stride % 4 == 0) &&
                   (reinterpret_cast<uintptr_t>(planes) % 8 == 0);
  if (vec) {
    const dim3 grid(ceil_div(cols_pad / 4, 256), rows_pad);
#define MDG_DIGITS8(W)                                                                      \
  digits4_kernel<W><<<grid, 256, 0, st>>>(p, s, rows, cols, X, ldx, E, trans, pl, ld_out,   \
                                           plane_stride, rows_pad, cols_pad)
    switch (NW) {
      case 4: MDG_DIGITS8(4); break;
      case 6: MDG_DIGITS8(6); break;
      case 10: MDG_DIGITS8(10); break;
      default: MDG_DIGITS8(16); break;
    }
#undef MDG_DIGITS8
    MDG_TRY_LAUNCH();
    return MDG_SUCCESS;
  }
  dim3 grid(ceil_div(cols_pad, 128), rows_pad);
#define MDG_DIGITS(W)                                                                    \
  digits_kernel<W><<<grid, 128, 0, st>>>(p, s, rows, cols, X, ldx, E, trans, pl, ld_out, \
                                          plane_stride, rows_pad, cols_pad)
  switch (NW) {
    case 4: MDG_DIGITS(4); break;
    case 6: MDG_DIGITS(6); break;
    case 10: MDG_DIGITS(10); break;
    default: MDG_DIGITS(16); break;
  }
#undef MDG_DIGITS
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

int launch_diag_gemm_v0(int s, int D, int Mp, int Np, int Kp, const void *dA, const void *dB,
                        int ld, long long plane_a, long long plane_b, int *chunks,
                        long long plane_c, cudaStream_t st) {
  if (Mp % BM || Np % BN || Kp % 64) return MDG_ERROR_INVALID_SIZE;
  dim3 grid(Np / BN, Mp / BM);
  diag_gemm_v0<<<grid, 256, 0, st>>>(s, D, Kp, reinterpret_cast<const __nv_bfloat16 *>(dA),
                                     reinterpret_cast<const __nv_bfloat16 *>(dB), ld, plane_a,
                                     plane_b, chunks, plane_c, Np);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

int launch_renorm(int p, int s, int D, int KB, int m, int n, const int *chunks,
                  long long plane_c, int ldcd, const int *E, const int *F, double *C, int ldc,
                  cudaStream_t st) {
  if (m == 0 || n == 0) return MDG_SUCCESS;
  const int NW = words_for(1, D);
  if (!NW) return MDG_ERROR_NOT_SUPPORTED;
  // V adjacent columns per thread need V-aligned rows of chunk planes
  const int Vmax = NW <= 6 ? 4 : NW <= 10 ? 2 : 1;
  int V = Vmax;
  while (V > 1 && ((ldcd % V) || (plane_c % V) ||
                   (reinterpret_cast<uintptr_t>(chunks) % (4 * V))))
    V >>= 1;
  switch (p) {
    case 2:
      return launch_renorm_p<2>(NW, V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    case 4:
      return launch_renorm_p<4>(NW, V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    case 8:
      return launch_renorm_p<8>(NW, V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    case 16:
      return launch_renorm_p<16>(NW, V, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, st);
    default:
      return MDG_ERROR_INVALID_LIMBS;
  }
}

int slice_prepare_b(const SlicePlan &pl, const double *B, int ldb, void *ws, cudaStream_t st) {
  char *base = reinterpret_cast<char *>(ws);
  auto *rowbits = reinterpret_cast<unsigned long long *>(base + pl.off_rowbits);
  auto *colbits = reinterpret_cast<unsigned long long *>(base + pl.off_colbits);
  int *E = reinterpret_cast<int *>(base + pl.off_E);
  int *F = reinterpret_cast<int *>(base + pl.off_F);
  MDG_TRY(launch_scale_exponents(pl.p, 0, pl.n, pl.k, nullptr, 1, B, ldb, rowbits, colbits, E, F,
                                 st));
  return launch_digits(pl.p, pl.s, pl.n, pl.k, B, ldb, F, 1, base + pl.off_dB, pl.Kp,
                       pl.plane_b, pl.Np, pl.Kp, st);
}

int slice_panel_a(const SlicePlan &pl, int rows, const double *A, int lda, void *ws,
                  cudaStream_t st) {
  if (rows <= 0) return MDG_SUCCESS;
  if (rows > pl.m) return MDG_ERROR_INVALID_SIZE;
  char *base = reinterpret_cast<char *>(ws);
  auto *rowbits = reinterpret_cast<unsigned long long *>(base + pl.off_rowbits);
  auto *colbits = reinterpret_cast<unsigned long long *>(base + pl.off_colbits);
  int *E = reinterpret_cast<int *>(base + pl.off_E);
  int *F = reinterpret_cast<int *>(base + pl.off_F);
  // E only (n = 0 leaves F, computed by slice_prepare_b, alone)
  MDG_TRY(launch_scale_exponents(pl.p, rows, 0, pl.k, A, lda, nullptr, 1, rowbits, colbits, E,
                                 F, st));
  // rows beyond `rows` up to the plan's padded Mp get zero digits
  return launch_digits(pl.p, pl.s, rows, pl.k, A, lda, E, 0, base + pl.off_dA, pl.Kp,
                       pl.plane_a, pl.Mp, pl.Kp, st);
}

int slice_block(const SlicePlan &pla, const void *wsa, const SlicePlan &plb, void *wsb, int rows,
                double *C, int ldc, int engine, int parts, int raster, cudaStream_t st,
                int pace) {
  if (rows <= 0) return MDG_SUCCESS;
  if (rows > pla.m || pla.Mp != plb.Mp || pla.Kp != plb.Kp || pla.s != plb.s ||
      pla.D != plb.D || pla.p != plb.p)
    return MDG_ERROR_INVALID_SIZE;
  const char *abase = reinterpret_cast<const char *>(wsa);
  char *bbase = reinterpret_cast<char *>(wsb);
  const int *E = reinterpret_cast<const int *>(abase + pla.off_E);
  const int *F = reinterpret_cast<const int *>(bbase + plb.off_F);
  const void *dA = abase + pla.off_dA;
  const void *dB = bbase + plb.off_dB;
  auto *Cd = reinterpret_cast<int *>(bbase + plb.off_Cd);
  const SlicePlan &pl = plb;
  if (engine != 0) {
    MDG_TRY(launch_diag_gemm_tc(pl.s, pl.D, pl.Mp, pl.Np, pl.Kp, dA, dB, pl.Kp, pla.plane_a,
                                pl.plane_b, Cd, pl.plane_c, engine == 2 ? 1 : 0, parts, raster, st,
                                pace));
  } else {
    MDG_TRY(launch_diag_gemm_v0(pl.s, pl.D, pl.Mp, pl.Np, pl.Kp, dA, dB, pl.Kp, pla.plane_a,
                                pl.plane_b, Cd, pl.plane_c, st));
  }
  return launch_renorm(pl.p, pl.s, pl.D, pl.Kp / 64, rows, pl.n, Cd, pl.plane_c, pl.Np, E, F, C,
                       ldc, st);
}

int slice_panel(const SlicePlan &pl, int rows, const double *A, int lda, double *C, int ldc,
                void *ws, int engine, int parts, int raster, cudaStream_t st, int pace) {
  MDG_TRY(slice_panel_a(pl, rows, A, lda, ws, st));
  return slice_block(pl, ws, pl, ws, rows, C, ldc, engine, parts, raster, st, pace);
}

int run_slice_gemm(const SlicePlan &pl, const double *A, int lda, const double *B, int ldb,
                   double *C, int ldc, void *ws, int engine, int parts, int raster,
                   cudaStream_t st, int pace) {
  char *base = reinterpret_cast<char *>(ws);
  auto *rowbits = reinterpret_cast<unsigned long long *>(base + pl.off_rowbits);
  auto *colbits = reinterpret_cast<unsigned long long *>(base + pl.off_colbits);
  int *E = reinterpret_cast<int *>(base + pl.off_E);
  int *F = reinterpret_cast<int *>(base + pl.off_F);
  void *dA = base + pl.off_dA;
  void *dB = base + pl.off_dB;
  auto *Cd = reinterpret_cast<int *>(base + pl.off_Cd);
  NvtxRange range("mdg slice_bf16");
  {
    NvtxRange r("split: scale exponents and digits");
    MDG_TRY(launch_scale_exponents(pl.p, pl.m, pl.n, pl.k, A, lda, B, ldb, rowbits, colbits, E,
                                   F, st));
    MDG_TRY(launch_digits(pl.p, pl.s, pl.m, pl.k, A, lda, E, 0, dA, pl.Kp, pl.plane_a, pl.Mp,
                          pl.Kp, st));
    MDG_TRY(launch_digits(pl.p, pl.s, pl.n, pl.k, B, ldb, F, 1, dB, pl.Kp, pl.plane_b, pl.Np,
                          pl.Kp, st));
  }
  NvtxRange r2("diagonal GEMM and renormalisation");
  if (engine != 0) {
    MDG_TRY(launch_diag_gemm_tc(pl.s, pl.D, pl.Mp, pl.Np, pl.Kp, dA, dB, pl.Kp, pl.plane_a,
                                pl.plane_b, Cd, pl.plane_c, engine == 2 ? 1 : 0, parts, raster, st,
                                pace));
  } else {
    MDG_TRY(launch_diag_gemm_v0(pl.s, pl.D, pl.Mp, pl.Np, pl.Kp, dA, dB, pl.Kp, pl.plane_a,
                                pl.plane_b, Cd, pl.plane_c, st));
  }
  MDG_TRY(launch_renorm(pl.p, pl.s, pl.D, pl.Kp / 64, pl.m, pl.n, Cd, pl.plane_c, pl.Np, E, F,
                        C, ldc, st));
  return MDG_SUCCESS;
}

}  // namespace mdgi

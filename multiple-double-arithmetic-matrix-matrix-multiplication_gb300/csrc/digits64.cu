// Slice digits on the FP64 tensor cores (MDG_FORM_FP64_DIGITS): the
// reference's own hardware path (FP64 DMMA, TCtest.cu:21-46) run on the
// slice-digit scheme of the BF16 form, so that the two tensor-core paths can
// be compared at the same accuracy.
//
// The scale exponents are the BF16 form's (E[r] for the rows of A, F[c] for
// the columns of B).  Each P-double a of row r becomes the integer
// V = sum_l floor(a_l 2^(S - E[r])), S = (DB - 1) + DB (s - 1), written as s
// balanced base-2^DB digits d_0 (most significant) .. d_{s-1}, each in
// [-2^(DB-1), 2^(DB-1)] and stored as a double.  With DB = 19 a digit
// product is at most 2^36 and a sum of 2^16 of them stays below 2^53, so
// DMMA's FP64 sums of up to 65536 products per entry are exact; they are
// added into int64 diagonal sums C_d = sum_{i+j=d} A_i B_j^T for d < D.
// The result is W = sum_d C_d 2^(DB (D-1-d)) times 2^(E + F - 2 (DB - 1) -
// DB (D - 1)), rounded to P limbs exactly as the BF16 form rounds.  Every
// stage is exact integer arithmetic or a defined rounding, so the result is
// the oracle's bit for bit (oracle.c, orc_gemm_digits).
//
// 19-bit digits need far fewer digit pairs than 8-bit ones for the same
// accuracy (quad-double: 12 digits, 78 pairs, against 28 and 406), which is
// the best use of GB300's narrow FP64 tensor rate.
#include <algorithm>

#include "common.cuh"
#include "slice_common.cuh"
#include "slice_stages.cuh"
#include "slice_tc.cuh"

namespace {

constexpr int DB = 19;          // bits per digit
constexpr int SEG = 1 << 16;    // products per entry summed in FP64 before a flush

// Digits of one entry: planes are rows x cols (K-major), plane i at
// planes + i * plane_stride.  trans = 1: X is cols x rows (B, k x n).
template <int NW>
__global__ void __launch_bounds__(128)
    digits64_kernel(int P, int s, int rows, int cols, const double *__restrict__ X, int ldx,
                    const int *__restrict__ E, int trans, double *__restrict__ planes,
                    long long plane_stride) {
  const int pr = blockIdx.y, pc = blockIdx.x * 128 + threadIdx.x;
  if (pc >= cols || pr >= rows) return;
  const double *a = trans ? X + ((size_t)pc * ldx + pr) * P : X + ((size_t)pr * ldx + pc) * P;
  const int S = (DB - 1) + DB * (s - 1);
  const int Er = E[pr];
  uint64_t w[NW];
#pragma unroll
  for (int i = 0; i < NW; ++i) w[i] = 0;
  for (int l = 0; l < P; ++l) {
    int e2;
    const int64_t m = mdgi::exact_significand(a[l], e2);
    if (m == 0) continue;
    const int q = e2 + S - Er;
    if (q >= 0) {
      mdgi::wide_add_shifted<NW>(w, m, q);
    } else if (q > -64) {
      mdgi::wide_add_shifted<NW>(w, m >> (-q), 0);
    } else {
      mdgi::wide_add_shifted<NW>(w, m < 0 ? -1 : 0, 0);
    }
  }
  // balanced digits from the bottom: t = chunk + carry, t >= 2^(DB-1) -> t - 2^DB
  double *out = planes + (size_t)pr * cols + pc;
  int carry = 0;
  for (int p = 0; p < s - 1; ++p) {
    const int t = (int)(mdgi::wide_bits64<NW>(w, DB * p) & ((1u << DB) - 1)) + carry;
    const int d = t >= (1 << (DB - 1)) ? t - (1 << DB) : t;
    carry = t >= (1 << (DB - 1)) ? 1 : 0;
    out[(size_t)(s - 1 - p) * plane_stride] = (double)d;
  }
  out[0] = (double)((int64_t)mdgi::wide_bits64<NW>(w, DB * (s - 1)) + carry);
}

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(c[0]), "+d"(c[1])
      : "d"(a), "d"(b));
}

// C_d for a 64 x 32 tile (4 warps as 2 x 2, each 32 rows x 16 columns of
// m8n8k4 DMMA tiles), diagonal d = blockIdx.z.  A: s planes m x k; B: s
// planes n x k; Cd: D planes m x n of int64.
__global__ void __launch_bounds__(128)
    diag64_kernel(int s, int m, int n, int k, const double *__restrict__ A,
                  const double *__restrict__ B, long long plane_a, long long plane_b,
                  long long *__restrict__ Cd) {
  const int d = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int row_base = blockIdx.y * 64 + (warp >> 1) * 32;
  const int col_base = blockIdx.x * 32 + (warp & 1) * 16;
  long long acc[4][2][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) acc[a][b][0] = acc[a][b][1] = 0;
  int rows[4], cols[2];
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) rows[mi] = row_base + mi * 8 + g;
#pragma unroll
  for (int ni = 0; ni < 2; ++ni) cols[ni] = col_base + ni * 8 + g;
  const int ilo = d - (s - 1) > 0 ? d - (s - 1) : 0, ihi = d < s - 1 ? d : s - 1;
  for (int i = ilo; i <= ihi; ++i) {
    const double *Ai = A + (size_t)i * plane_a;
    const double *Bj = B + (size_t)(d - i) * plane_b;
    for (int k0 = 0; k0 < k; k0 += SEG) {
      const int k1 = k0 + SEG < k ? k0 + SEG : k;
      double f[4][2][2];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) f[a][b][0] = f[a][b][1] = 0.0;
      for (int kk = k0; kk < k1; kk += 4) {
        const int kt = kk + t;
        double av[4], bv[2];
#pragma unroll
        for (int mi = 0; mi < 4; ++mi)
          av[mi] = (rows[mi] < m && kt < k1) ? __ldg(Ai + (size_t)rows[mi] * k + kt) : 0.0;
#pragma unroll
        for (int ni = 0; ni < 2; ++ni)
          bv[ni] = (cols[ni] < n && kt < k1) ? __ldg(Bj + (size_t)cols[ni] * k + kt) : 0.0;
#pragma unroll
        for (int mi = 0; mi < 4; ++mi)
#pragma unroll
          for (int ni = 0; ni < 2; ++ni) dmma(f[mi][ni], av[mi], bv[ni]);
      }
      // integer-valued and below 2^53: the conversion is exact
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 2; ++ni) {
          acc[mi][ni][0] += __double2ll_rn(f[mi][ni][0]);
          acc[mi][ni][1] += __double2ll_rn(f[mi][ni][1]);
        }
    }
  }
  long long *out = Cd + (size_t)d * m * n;
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) {
    const int r = row_base + mi * 8 + g;
    if (r >= m) continue;
#pragma unroll
    for (int ni = 0; ni < 2; ++ni)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int c = col_base + ni * 8 + 2 * t + h;
        if (c < n) out[(size_t)r * n + c] = acc[mi][ni][h];
      }
  }
}

// C[r][c] = RN_P(W * 2^(E[r] + F[c] - 2 (DB - 1) - DB (D - 1))), W built
// from the top diagonal down: W = W 2^DB + C_d.
template <int P, int NW>
__global__ void __launch_bounds__(128)
    renorm64_kernel(int D, int m, int n, const long long *__restrict__ Cd,
                    const int *__restrict__ E, const int *__restrict__ F, double *__restrict__ C,
                    int ldc) {
  const int r = blockIdx.y, c = blockIdx.x * 128 + threadIdx.x;
  if (c >= n || r >= m) return;
  uint64_t w[NW];
#pragma unroll
  for (int i = 0; i < NW; ++i) w[i] = 0;
  const long long *src = Cd + (size_t)r * n + c;
  for (int d = 0; d < D; ++d) {
#pragma unroll
    for (int i = NW - 1; i > 0; --i) w[i] = (w[i] << DB) | (w[i - 1] >> (64 - DB));
    w[0] <<= DB;
    mdgi::wide_add_shifted<NW>(w, src[(size_t)d * m * n], 0);
  }
  const int scale = E[r] + F[c] - 2 * (DB - 1) - DB * (D - 1);
  mdgi::emit_limbs<P, NW>(w, scale, C + ((size_t)r * ldc + c) * P);
}

template <int NW>
int launch_renorm64_w(int p, int D, int m, int n, const long long *Cd, const int *E,
                      const int *F, double *C, int ldc, cudaStream_t st) {
  const dim3 grid(mdgi::ceil_div(n, 128), m);
  switch (p) {
    case 2: renorm64_kernel<2, NW><<<grid, 128, 0, st>>>(D, m, n, Cd, E, F, C, ldc); break;
    case 4: renorm64_kernel<4, NW><<<grid, 128, 0, st>>>(D, m, n, Cd, E, F, C, ldc); break;
    case 8: renorm64_kernel<8, NW><<<grid, 128, 0, st>>>(D, m, n, Cd, E, F, C, ldc); break;
    default: renorm64_kernel<16, NW><<<grid, 128, 0, st>>>(D, m, n, Cd, E, F, C, ldc); break;
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

}  // namespace

namespace mdgi {

int digits64_default(int p) {
  switch (p) {
    case 2: return 6;    // 113 bits (the BF16 form: 111)
    case 4: return 12;   // 227 bits (223)
    case 8: return 24;   // 455 bits (439)
    case 16: return 47;  // 892 bits (879)
  }
  return 0;
}

// Words of the wide integers: the digits need S + 2 bits, W needs
// DB (D - 1) + 72 (the int64 sums and their carries), plus a word of headroom.
int words64_for(int s, int D) {
  const int bits = std::max((DB - 1) + DB * (s - 1) + 2, DB * (D - 1) + 72);
  const int w = (bits + 63) / 64 + 1;
  if (w <= 4) return 4;
  if (w <= 6) return 6;
  if (w <= 10) return 10;
  if (w <= 16) return 16;
  return 0;
}

Digits64Plan make_digits64_plan(int p, int s, int D, int m, int n, int k) {
  Digits64Plan pl{};
  pl.p = p;
  pl.s = s;
  pl.D = D;
  pl.m = m;
  pl.n = n;
  pl.k = k;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  pl.off_rowbits = take(sizeof(unsigned long long) * std::max(m, 1));
  pl.off_colbits = take(sizeof(unsigned long long) * std::max(n, 1));
  pl.off_E = take(sizeof(int) * std::max(m, 1));
  pl.off_F = take(sizeof(int) * std::max(n, 1));
  pl.off_dA = take(sizeof(double) * (size_t)s * m * k);
  pl.off_dB = take(sizeof(double) * (size_t)s * n * k);
  pl.off_Cd = take(sizeof(long long) * (size_t)D * m * n);
  pl.total = off;
  return pl;
}

int run_digits64_gemm(const Digits64Plan &pl, const double *A, int lda, const double *B, int ldb,
                      double *C, int ldc, void *ws, cudaStream_t st) {
  const int NW = words64_for(pl.s, pl.D);
  if (!NW) return MDG_ERROR_NOT_SUPPORTED;
  if (pl.m > 65535 || pl.n > 65535 || pl.D > 65535) return MDG_ERROR_NOT_SUPPORTED;
  char *base = reinterpret_cast<char *>(ws);
  auto *rowbits = reinterpret_cast<unsigned long long *>(base + pl.off_rowbits);
  auto *colbits = reinterpret_cast<unsigned long long *>(base + pl.off_colbits);
  int *E = reinterpret_cast<int *>(base + pl.off_E);
  int *F = reinterpret_cast<int *>(base + pl.off_F);
  double *dA = reinterpret_cast<double *>(base + pl.off_dA);
  double *dB = reinterpret_cast<double *>(base + pl.off_dB);
  long long *Cd = reinterpret_cast<long long *>(base + pl.off_Cd);
  NvtxRange range("mdg fp64_digits");
  MDG_TRY(launch_scale_exponents(pl.p, pl.m, pl.n, pl.k, A, lda, B, ldb, rowbits, colbits, E, F,
                                 st));
  const long long pa = (long long)pl.m * pl.k, pb = (long long)pl.n * pl.k;
#define MDG_DIGITS64(W)                                                                        \
  digits64_kernel<W><<<dim3(ceil_div(pl.k, 128), pl.m), 128, 0, st>>>(pl.p, pl.s, pl.m, pl.k, \
                                                                      A, lda, E, 0, dA, pa);   \
  MDG_TRY_LAUNCH();                                                                            \
  digits64_kernel<W><<<dim3(ceil_div(pl.k, 128), pl.n), 128, 0, st>>>(pl.p, pl.s, pl.n, pl.k, \
                                                                      B, ldb, F, 1, dB, pb);   \
  MDG_TRY_LAUNCH()
  switch (NW) {
    case 4: MDG_DIGITS64(4); break;
    case 6: MDG_DIGITS64(6); break;
    case 10: MDG_DIGITS64(10); break;
    default: MDG_DIGITS64(16); break;
  }
#undef MDG_DIGITS64
  diag64_kernel<<<dim3(ceil_div(pl.n, 32), ceil_div(pl.m, 64), pl.D), 128, 0, st>>>(
      pl.s, pl.m, pl.n, pl.k, dA, dB, pa, pb, Cd);
  MDG_TRY_LAUNCH();
  switch (NW) {
    case 4: return launch_renorm64_w<4>(pl.p, pl.D, pl.m, pl.n, Cd, E, F, C, ldc, st);
    case 6: return launch_renorm64_w<6>(pl.p, pl.D, pl.m, pl.n, Cd, E, F, C, ldc, st);
    case 10: return launch_renorm64_w<10>(pl.p, pl.D, pl.m, pl.n, Cd, E, F, C, ldc, st);
    default: return launch_renorm64_w<16>(pl.p, pl.D, pl.m, pl.n, Cd, E, F, C, ldc, st);
  }
}

}  // namespace mdgi

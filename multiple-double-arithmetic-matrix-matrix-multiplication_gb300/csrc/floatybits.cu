// Limb slicing and squeezing on the GPU (the FP64 split form's two ends).
//
// split: every limb of a P-double is cut into FP64 slices holding fixed
// ranges of its significand bits, then adjacent slices of one P-double are
// "balanced" so that their exponents differ by at most 13 (or 7/6) bits.
// Reference: split4 / split4pd / balance4 (floatybits.cu:134-206), split8 /
// split8pd / balance8 (:208-313), mixsplit2 / mixbalance (:315-342), and
// the unbalanced split4pd of the CPU convolution driver (TCcudant.cpp:163).  The
// reference goes through vector<int> bit arrays and pow() loops on the host;
// here one thread per P-double reads the IEEE fields with frexp/ldexp.
//
// Two modes.  exact = 0 reproduces the reference bit for bit, including the
// two properties of its bit expansion (floatybits.cu:16-33, 54-68, 92-102):
// only 52 of the 53 significand bits are kept, and a negative limb expands
// to an all-zero fraction, i.e. slices -0.0.  exact = 1 splits |x| with all
// 53 bits (the last range takes the 53rd bit) and gives every slice the sign
// of its limb; balancing then only pairs slices of the same sign.
//
// squeeze: y = sum of pp partial sums through the P-double inc_d, in order
// (pllsqueeze_{2,4,8,16}_pp_old, TCcuda.cu:876-906); one thread per entry
// and no barrier (the reference's __syncthreads in that loop guards no
// shared data).
#include "common.cuh"

namespace {

__device__ __forceinline__ double slice_ref(double x, int lo, int hi) {
  if (!(x >= 0)) return -0.0;
  int e;
  const double f = frexp(x, &e);
  if (f <= 0.0) return 0.0;
  const uint64_t F = (uint64_t)ldexp(f, 52);  // first 52 fraction bits
  const uint64_t bits = (F >> (52 - hi)) & ((1ull << (hi - lo)) - 1);
  return ldexp((double)bits, e - hi);
}

__device__ __forceinline__ double trunc52(double x) {
  if (!(x >= 0)) return -0.0;
  int e;
  const double f = frexp(x, &e);
  if (f <= 0.0) return 0.0;
  return ldexp((double)(uint64_t)ldexp(f, 52), e - 52);
}

__device__ __forceinline__ void split_exact(double x, const int *ranges, int nr, double *out) {
  const double ax = fabs(x);
  if (ax == 0.0) {
    for (int t = 0; t < nr; ++t) out[t] = 0.0;
    return;
  }
  int e;
  const double f = frexp(ax, &e);
  const uint64_t F = (uint64_t)ldexp(f, 53);
  for (int t = 0; t < nr; ++t) {
    const int lo = ranges[t], hi = (t == nr - 1) ? 53 : ranges[t + 1];
    const uint64_t bits = (F >> (53 - hi)) & ((1ull << (hi - lo)) - 1);
    const double v = ldexp((double)bits, e - hi);
    out[t] = x < 0 ? -v : v;
  }
}

__constant__ int kRanges4[5] = {0, 13, 26, 39, 52};
__constant__ int kRanges8[8] = {0, 7, 14, 21, 28, 34, 40, 52};

__device__ __forceinline__ void balance(double &x, double &y, int th, int exact) {
  if (x == 0.0 || y == 0.0) return;
  if (exact && ((x < 0) != (y < 0))) return;
  int xe, ye;
  frexp(x, &xe);
  frexp(y, &ye);
  if (!(xe - ye > th - 1)) return;
  double bit = ldexp(1.0, xe - th);
  if (exact && x < 0) bit = -bit;
  x = x - bit;
  y = y + bit;
}

// One thread per P-double.  pp <= 128.
__global__ void split_kernel(int kind, int exact, int P, long long count,
                             const double *__restrict__ x, double *__restrict__ out, int soa,
                             long long plane_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int pp = (kind == 0 || kind == 3) ? 4 * P : kind == 1 ? 8 * P : 12;
  double w[128];
  int pos = 0;
  for (int l = 0; l < P; ++l) {
    const double v = x[i * P + l];
    const bool use8 = (kind == 1) || (kind == 2 && l == 1);
    if (!exact) {
      if (use8) {
        double s = 0.0;
        for (int t = 0; t < 7; ++t) {
          w[pos + t] = slice_ref(v, kRanges8[t], kRanges8[t + 1]);
          s = (t == 0) ? w[pos] : s + w[pos + t];
        }
        w[pos + 7] = trunc52(v) - s;
      } else {
        for (int t = 0; t < 3; ++t) w[pos + t] = slice_ref(v, kRanges4[t], kRanges4[t + 1]);
        const double s = (w[pos] + w[pos + 1]) + w[pos + 2];
        w[pos + 3] = trunc52(v) - s;
      }
    } else {
      if (use8) {
        split_exact(v, kRanges8, 7, w + pos);
        w[pos + 7] = 0.0;
      } else {
        split_exact(v, kRanges4, 4, w + pos);
      }
    }
    pos += use8 ? 8 : 4;
  }
  // kind 3 (split4pd of TCcudant.cpp:163) keeps the slices unbalanced
  for (int j = 0; j + 1 < pp && kind != 3; ++j) {
    int th;
    if (kind == 0) {
      if (j >= pp - 2) break;
      th = 14;
    } else if (kind == 1) {
      if (j >= pp - 3) break;
      th = (j % 8 < 4) ? 8 : 7;
    } else {
      if (j >= pp - 3) break;
      th = (j % 12 < 4) ? 14 : (j % 12 < 8) ? 8 : 7;
    }
    balance(w[j], w[j + 1], th, exact);
  }
  if (soa) {
    for (int j = 0; j < pp; ++j) out[j * plane_stride + i] = w[j];
  } else {
    for (int j = 0; j < pp; ++j) out[i * pp + j] = w[j];
  }
}

template <int P>
__global__ void squeeze_kernel(long long count, int pp, const double *__restrict__ x,
                               long long x_stride, long long x_plane, double *__restrict__ y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double acc[P];
#pragma unroll
  for (int l = 0; l < P; ++l) acc[l] = 0.0;
  for (int j = 0; j < pp; ++j) mdg::inc_d<P>(acc, x[i * x_stride + j * x_plane]);
#pragma unroll
  for (int l = 0; l < P; ++l) y[i * P + l] = acc[l];
}

}  // namespace

namespace mdgi {

int launch_split(int kind, int exact, int p, long long count, const double *x, double *out,
                 int soa, long long plane_stride, cudaStream_t st) {
  if (count == 0) return MDG_SUCCESS;
  const int threads = 128;
  split_kernel<<<ceil_div(count, threads), threads, 0, st>>>(kind, exact, p, count, x, out, soa,
                                                              plane_stride);
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

// x_stride: distance between entries; x_plane: distance between partials
// (AoS: x_stride = pp, x_plane = 1;  SoA: x_stride = 1, x_plane = count).
int launch_squeeze(int p, int pp, long long count, const double *x, long long x_stride,
                   long long x_plane, double *y, cudaStream_t st) {
  if (count == 0) return MDG_SUCCESS;
  const int threads = 128;
  const unsigned grid = ceil_div(count, threads);
  switch (p) {
    case 2: squeeze_kernel<2><<<grid, threads, 0, st>>>(count, pp, x, x_stride, x_plane, y); break;
    case 4: squeeze_kernel<4><<<grid, threads, 0, st>>>(count, pp, x, x_stride, x_plane, y); break;
    case 8: squeeze_kernel<8><<<grid, threads, 0, st>>>(count, pp, x, x_stride, x_plane, y); break;
    case 16: squeeze_kernel<16><<<grid, threads, 0, st>>>(count, pp, x, x_stride, x_plane, y); break;
    default: return MDG_ERROR_INVALID_LIMBS;
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

}  // namespace mdgi

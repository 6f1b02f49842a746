// Per-element / per-block bodies of the slice-digit stage kernels, shared
// by the single-problem kernels (slice_tc.cu) and the batched kernels
// (batched.cu).  See slice_tc.cu for what each stage computes.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "slice_common.cuh"
#include "slice_tc.cuh"

namespace mdgi {

// ------------------------------------------------------------ exponents --
// sum_l |x_l| of one entry (FP64 additions in limb order), as its bit
// pattern: maxima of non-negative doubles are taken as 64-bit unsigned
// integers, which orders them like the doubles and keeps the reductions off
// the FP64 pipe (narrow on this GPU).  A NaN sum counts as 0, so that a
// maximum skips it as a floating-point comparison would.
__device__ __forceinline__ unsigned long long abs_sum_bits(const double *x, int P) {
  double v = fabs(x[0]);
  for (int l = 1; l < P; ++l) v = v + fabs(x[l]);
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return b > 0x7ff0000000000000ull ? 0ull : b;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// Block 32 x 8 covers 32 columns x 256 rows; each warp walks 32 rows of
// one 32-column strip.  Row maxima: warp reduction, one atomic per row per
// warp.  Column maxima: one atomic per thread.
__device__ __forceinline__ void absmax_block(int P, int R, int Cn, const double *__restrict__ X,
                                             int ldx, unsigned long long *rowbits,
                                             unsigned long long *colbits, int bx, int by) {
  const int c = bx * 32 + threadIdx.x;
  const int r0 = by * 256 + threadIdx.y * 32;
  unsigned long long cm = 0;
  for (int rr = 0; rr < 32; ++rr) {
    const int r = r0 + rr;
    if (r >= R) break;
    const unsigned long long v = c < Cn ? abs_sum_bits(X + ((size_t)r * ldx + c) * P, P) : 0ull;
    cm = umax64(cm, v);
    if (rowbits) {
      unsigned long long w = v;
#pragma unroll
      for (int o = 16; o; o >>= 1) w = umax64(w, __shfl_xor_sync(0xffffffffu, w, o));
      if (threadIdx.x == 0) atomicMax(rowbits + r, w);
    }
  }
  if (colbits && c < Cn) atomicMax(colbits + c, cm);
}

// --------------------------------------------------------------- digits --
// BF16 bits of an integer d in [-128, 127] without a conversion instruction
// (conversions run at a fraction of the FP32 rate): 2^23 + 128 + d written
// into the bit pattern of 2^23 is that integer as a float, and subtracting
// 2^23 + 128 in FP32 leaves d exactly; a float with at most 8 significant
// bits has its low 16 bits clear, so its top half is d in BF16.
__device__ __forceinline__ uint32_t bf16_bits_of_digit(int d) {
  const float f = __int_as_float(0x4B000000 + 128 + d) - 8388736.0f;
  return __float_as_uint(f) >> 16;
}

// One thread per element of the padded plane (prow, pcol); pcol (the k
// index) is the fastest, so plane stores are coalesced.  Outside the valid
// region every digit is zero.
template <int NW>
__device__ __forceinline__ void digits_elem(int P, int s, int rows, int cols,
                                            const double *__restrict__ X, int ldx,
                                            const int *__restrict__ E, int trans,
                                            __nv_bfloat16 *__restrict__ planes, int ld_out,
                                            long long plane_stride, int rows_pad, int cols_pad,
                                            int pr, int pc) {
  if (pc >= cols_pad || pr >= rows_pad) return;
  __nv_bfloat16 *out = planes + (size_t)pr * ld_out + pc;
  if (pr >= rows || pc >= cols) {
    for (int i = 0; i < s; ++i) out[i * plane_stride] = __float2bfloat16_rn(0.0f);
    return;
  }
  const double *a = trans ? X + ((size_t)pc * ldx + pr) * P : X + ((size_t)pr * ldx + pc) * P;
  const int S = 7 + 8 * (s - 1);
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
  // balanced digits from the bottom: t = byte + carry, t >= 128 -> t - 256
  int carry = 0;
#pragma unroll
  for (int wi = 0; wi < NW; ++wi) {
    const uint64_t word = w[wi];
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int p = wi * 8 + b;
      if (p < s - 1) {
        const int t = (int)((word >> (8 * b)) & 255) + carry;
        const int d = t >= 128 ? t - 256 : t;
        carry = t >= 128 ? 1 : 0;
        out[(s - 1 - p) * plane_stride] =
            __ushort_as_bfloat16((unsigned short)bf16_bits_of_digit(d));
      }
    }
  }
  const int top = (int)(int64_t)mdgi::wide_bits64<NW>(w, 8 * (s - 1)) + carry;
  out[0] = __float2bfloat16_rn((float)top);
}

// Four consecutive k-positions per thread: the same digits as digits_elem,
// written as one 8-byte vector (4 BF16) per plane.  pc0 is a multiple of 4;
// cols_pad, ld_out and plane_stride are multiples of 4.
template <int NW>
__device__ __forceinline__ void digits_elem4(int P, int s, int rows, int cols,
                                             const double *__restrict__ X, int ldx,
                                             const int *__restrict__ E, int trans,
                                             __nv_bfloat16 *__restrict__ planes, int ld_out,
                                             long long plane_stride, int rows_pad, int cols_pad,
                                             int pr, int pc0) {
  if (pc0 >= cols_pad || pr >= rows_pad) return;
  uint2 *out = reinterpret_cast<uint2 *>(planes + (size_t)pr * ld_out + pc0);
  const long long vstride = plane_stride / 4;
  if (pr >= rows || pc0 >= cols) {
    for (int i = 0; i < s; ++i) out[i * vstride] = make_uint2(0, 0);
    return;
  }
  const int S = 7 + 8 * (s - 1);
  const int Er = E[pr];
  uint64_t w[4][NW];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
#pragma unroll
    for (int i = 0; i < NW; ++i) w[e][i] = 0;
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int pc = pc0 + e;
    const double *a = trans ? X + ((size_t)pc * ldx + pr) * P : X + ((size_t)pr * ldx + pc) * P;
    for (int l = 0; l < P; ++l) {
      int e2;
      const int64_t m = pc < cols ? mdgi::exact_significand(a[l], e2) : 0;
      if (m == 0) continue;
      const int q = e2 + S - Er;
      if (q >= 0) {
        mdgi::wide_add_shifted<NW>(w[e], m, q);
      } else if (q > -64) {
        mdgi::wide_add_shifted<NW>(w[e], m >> (-q), 0);
      } else {
        mdgi::wide_add_shifted<NW>(w[e], m < 0 ? -1 : 0, 0);
      }
    }
  }
  int carry[4] = {0, 0, 0, 0};
#pragma unroll
  for (int wi = 0; wi < NW; ++wi) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int p = wi * 8 + b;
      if (p < s - 1) {
        uint32_t packed[2];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int t = (int)((w[e][wi] >> (8 * b)) & 255) + carry[e];
          const int d = t >= 128 ? t - 256 : t;
          carry[e] = t >= 128 ? 1 : 0;
          const uint32_t bits = bf16_bits_of_digit(d);
          if (e & 1) packed[e >> 1] |= bits << 16; else packed[e >> 1] = bits;
        }
        out[(s - 1 - p) * vstride] = make_uint2(packed[0], packed[1]);
      }
    }
  }
  uint32_t packed[2];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int top = (int)(int64_t)mdgi::wide_bits64<NW>(w[e], 8 * (s - 1)) + carry[e];
    const uint32_t bits = __bfloat16_as_ushort(__float2bfloat16_rn((float)top));
    if (e & 1) packed[e >> 1] |= bits << 16; else packed[e >> 1] = bits;
  }
  out[0] = make_uint2(packed[0], packed[1]);
}

// --------------------------------------------------------------- renorm --
// W = sum_d C_d 256^(D-1-d) is built bottom-up (Horner from the least
// significant diagonal): T = C_{D-1}; repeatedly emit the low byte of T as
// the next byte of W and continue with floor(T / 256) + C_{d-1}; after
// diagonal 0, T is the top part of W, above bit 8 (D - 1).  The emitted
// bytes land at positions fixed at compile time, so W stays in registers.
// Each thread takes V adjacent columns and loads their chunk sums as one
// vector per chunk plane.
// V adjacent int32 as one vector load.
template <int V>
struct IntV;
template <>
struct IntV<4> {
  static __device__ __forceinline__ void load(const int *p, int (&x)[4]) {
    const int4 t = *reinterpret_cast<const int4 *>(p);
    x[0] = t.x; x[1] = t.y; x[2] = t.z; x[3] = t.w;
  }
};
template <>
struct IntV<2> {
  static __device__ __forceinline__ void load(const int *p, int (&x)[2]) {
    const int2 t = *reinterpret_cast<const int2 *>(p);
    x[0] = t.x; x[1] = t.y;
  }
};
template <>
struct IntV<1> {
  static __device__ __forceinline__ void load(const int *p, int (&x)[1]) { x[0] = *p; }
};

// The P limbs of W * 2^scale (W a wide two's complement integer): limb l
// is the residual R_l = W - (limbs 0..l-1), rounded to nearest-even to 53
// bits.  W itself is never modified: after a limb rounded at bit sh, the
// residual is W's bits below sh with every bit from sh up equal to f, where
// f is all ones if that limb was rounded up and zero otherwise (rounding up
// leaves a negative remainder, rounding down a non-negative one, and |R|
// is below 2^sh either way).  So each limb needs: the highest bit of R
// that differs from f (its magnitude), a 64-bit window of R at that bit,
// and whether any bit of W lies below the rounding position (the sticky
// bit, from W's lowest set bit, found once).  The search looks at a
// 128-bit window of R ending at the current cut h and moves down 64 bits
// at a time while the window's upper half carries nothing but f.
template <int P, int NW>
__device__ __forceinline__ void emit_limbs(const uint64_t (&w)[NW], int scale, double *out) {
  const int lsb = mdgi::wide_lsb<NW>(w);
  uint64_t f = (uint64_t)((int64_t)w[NW - 1] >> 63);
  int h = 64 * NW;  // bits of R from h up all equal f
#pragma unroll 1
  for (int l = 0; l < P; ++l) {
    if (f == 0 && lsb >= h) {  // R = 0
      out[l] = 0.0;
      continue;
    }
    int b0, t;
    uint64_t lo, hi;
    for (;;) {  // at most NW passes: h drops by 64 per pass
      b0 = h > 128 ? h - 128 : 0;
      mdgi::wide_bits128<NW>(w, b0, lo, hi);
      const int cut = h - b0;  // 0..128: window bits from cut up are f
      if (cut < 64) {
        const uint64_t keep = cut ? ((1ull << cut) - 1) : 0ull;
        lo = (lo & keep) | (f & ~keep);
        hi = f;
      } else if (cut < 128) {
        const uint64_t keep = cut > 64 ? ((1ull << (cut - 64)) - 1) : 0ull;
        hi = (hi & keep) | (f & ~keep);
      }
      const uint64_t xh = hi ^ f, xl = lo ^ f;
      if (xh) {
        t = b0 + 127 - __clzll((long long)xh);
        break;
      }
      if (b0 == 0) {
        t = xl ? 63 - __clzll((long long)xl) : -1;  // -1: R = -1
        break;
      }
      h = b0 + 64;
    }
    // rounding position sh; x = bits [sh - 1, sh + 63) of R: the round bit,
    // then m = floor(R / 2^sh), |m| <= 2^53 (sh = 0: R itself, b0 = 0)
    const int sh = t > 52 ? t - 52 : 0;
    uint64_t x;
    if (sh == 0) {
      x = lo << 1;
    } else {
      const int o = sh - 1 - b0;  // 0..127
      if (o < 64)
        x = o ? ((lo >> o) | (hi << (64 - o))) : lo;
      else
        x = o > 64 ? ((hi >> (o - 64)) | (f << (128 - o))) : hi;
    }
    const int64_t m = (int64_t)x >> 1;
    const bool up = sh > 0 && (x & 1ull) && (lsb < sh - 1 || (m & 1));
    const int64_t mr = up ? m + 1 : m;
    f = up ? ~0ull : 0ull;
    h = sh;
    // mr 2^(sh + scale) as a double; with the top bit at 52 (or 53) and a
    // normal exponent it is assembled from its fields by integer
    // instructions, otherwise converted and scaled in FP64
    const bool neg = mr < 0;
    const uint64_t mm = neg ? (uint64_t)(-mr) : (uint64_t)mr;
    const bool top = mm >> 53;
    const uint64_t frac = top ? (mm >> 1) : mm;
    const int be = sh + scale + 52 + (top ? 1 : 0) + 1023;
    double val;
    if ((frac >> 52) == 1 && be >= 1 && be <= 2046)
      val = __longlong_as_double((long long)(((uint64_t)be << 52) | (frac & ((1ull << 52) - 1))));
    else
      val = ldexp((double)mm, sh + scale);
    out[l] = neg ? -val : val;
  }
}

// PAIRED: the first two chunk planes of each diagonal are loaded together
// (the second load repeats the first when the diagonal has one chunk), so
// that two loads are in flight where diagonals span two chunks.
template <int P, int NW, int V, bool PAIRED = false>
__device__ __forceinline__ void renorm_elems(int s, int D, int KB, int m, int n,
                                             const int *__restrict__ chunks, long long plane_c,
                                             int ldcd, const int *__restrict__ E,
                                             const int *__restrict__ F, double *__restrict__ C,
                                             int ldc, int r, int c0) {
  if (c0 >= n || r >= m) return;
  const int *src = chunks + (size_t)r * ldcd + c0;
  int q = 0;
  for (int d = 0; d < D; ++d) q += mdgi::diag_chunks(d, s, KB);
  uint64_t w[V][NW];
  long long T[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    T[v] = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) w[v][i] = 0;
  }
#pragma unroll
  for (int wi = 0; wi < NW; ++wi) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int k = wi * 8 + b;
      if (k < D) {
        const int d = D - 1 - k;
        const int nc = mdgi::diag_chunks(d, s, KB);
        q -= nc;
        int j = 0;
        if constexpr (PAIRED) {
          int x[V], y[V];
          IntV<V>::load(src + (size_t)q * plane_c, x);
          IntV<V>::load(src + (size_t)(q + (nc > 1 ? 1 : 0)) * plane_c, y);
#pragma unroll
          for (int v = 0; v < V; ++v) T[v] += (long long)x[v] + (nc > 1 ? y[v] : 0);
          j = 2;
        }
        for (; j < nc; ++j) {
          int x[V];
          IntV<V>::load(src + (size_t)(q + j) * plane_c, x);
#pragma unroll
          for (int v = 0; v < V; ++v) T[v] += x[v];
        }
        if (k < D - 1) {
#pragma unroll
          for (int v = 0; v < V; ++v) {
            w[v][wi] |= (uint64_t)(T[v] & 255) << (8 * b);
            T[v] >>= 8;
          }
        }
      }
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int c = c0 + v;
    if (c >= n) break;
    mdgi::wide_add_shifted<NW>(w[v], T[v], 8 * (D - 1));
    const int scale = E[r] + F[c] - 14 - 8 * (D - 1);
    double *out = C + ((size_t)r * ldc + c) * P;
    emit_limbs<P, NW>(w[v], scale, out);
  }
}

}  // namespace mdgi

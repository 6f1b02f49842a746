// Fixed-width two's complement integers in registers, used by the digit
// split and by the renormalisation of the slice-digit form.  Word 0 is the
// least significant.  Every loop is unrolled over the compile-time width so
// that the words stay in registers; positions that vary at run time are
// handled with predicated selects instead of indexed accesses.
#pragma once

#include <stdint.h>

namespace mdgi {

// w += v * 2^q for q >= 0 (v sign-extended).
template <int NW>
__device__ __forceinline__ void wide_add_shifted(uint64_t (&w)[NW], int64_t v, int q) {
  const int qw = q >> 6, r = q & 63;
  const uint64_t fill = (uint64_t)(v >> 63);
  const uint64_t lo = (uint64_t)v << r;
  const uint64_t hi = r ? (uint64_t)(v >> (64 - r)) : fill;
  uint64_t carry = 0;
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    const uint64_t add = (i < qw) ? 0ull : (i == qw) ? lo : (i == qw + 1) ? hi : fill;
    const uint64_t s = w[i] + add;
    const uint64_t c1 = s < add;
    const uint64_t s2 = s + carry;
    const uint64_t c2 = s2 < s;
    w[i] = s2;
    carry = c1 | c2;
  }
}

// The 64 bits of w starting at bit pos (0 <= pos < 64 NW); bits above the
// top word read as the sign.  The word offset is applied as a barrel shift
// (one predicated shift per bit of the offset) so that every access has a
// compile-time index and w stays in registers.
template <int NW>
__device__ __forceinline__ uint64_t wide_bits64(const uint64_t (&w)[NW], int pos) {
  const int qw = pos >> 6, r = pos & 63;
  const uint64_t fill = (uint64_t)((int64_t)w[NW - 1] >> 63);
  uint64_t t[NW + 1];
#pragma unroll
  for (int i = 0; i < NW; ++i) t[i] = w[i];
  t[NW] = fill;
#pragma unroll
  for (int bit = 1; bit <= NW; bit <<= 1) {
    const bool on = (qw & bit) != 0;
#pragma unroll
    for (int i = 0; i <= NW; ++i) {
      const uint64_t src = (i + bit <= NW) ? t[i + bit] : fill;
      t[i] = on ? src : t[i];
    }
  }
  const uint64_t lo = t[0], hi = NW >= 1 ? t[1] : fill;
  return r ? ((lo >> r) | (hi << (64 - r))) : lo;
}

// Bits [pos, pos + 128) of w (0 <= pos < 64 NW) as lo and hi; bits above the
// top word read as the sign.  The same barrel shift as wide_bits64, over
// one more word.
template <int NW>
__device__ __forceinline__ void wide_bits128(const uint64_t (&w)[NW], int pos, uint64_t &lo,
                                             uint64_t &hi) {
  const int qw = pos >> 6, r = pos & 63;
  const uint64_t fill = (uint64_t)((int64_t)w[NW - 1] >> 63);
  uint64_t t[NW + 2];
#pragma unroll
  for (int i = 0; i < NW; ++i) t[i] = w[i];
  t[NW] = fill;
  t[NW + 1] = fill;
#pragma unroll
  for (int bit = 1; bit <= NW; bit <<= 1) {
    const bool on = (qw & bit) != 0;
#pragma unroll
    for (int i = 0; i <= NW + 1; ++i) {
      const uint64_t src = (i + bit <= NW + 1) ? t[i + bit] : fill;
      t[i] = on ? src : t[i];
    }
  }
  lo = r ? ((t[0] >> r) | (t[1] << (64 - r))) : t[0];
  hi = r ? ((t[1] >> r) | (t[2] << (64 - r))) : t[1];
}

// Index of the lowest set bit of w, 64 NW for zero.
template <int NW>
__device__ __forceinline__ int wide_lsb(const uint64_t (&w)[NW]) {
  int b = 64 * NW;
#pragma unroll
  for (int i = NW - 1; i >= 0; --i)
    if (w[i]) b = 64 * i + __ffsll((long long)w[i]) - 1;
  return b;
}

// x = m 2^e2 with m an integer, |m| < 2^53 (0 for x = +-0), read from the
// IEEE fields of a finite x with integer instructions only: the FP64 units
// of this GPU are narrow, and frexp / ldexp / an FP64-to-int conversion per
// limb kept them 80 % busy in the digit split.  Normal x: m = +-(fraction +
// 2^52), e2 = biased exponent - 1075; subnormal x: m = +-fraction,
// e2 = -1074.  m 2^e2 equals x exactly, so floor(x 2^q) is unchanged.
__device__ __forceinline__ int64_t exact_significand(double x, int &e2) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7ff);
  const int64_t frac = (int64_t)(b & 0xfffffffffffffull);
  const int64_t mag = be ? (frac | (1ll << 52)) : frac;
  e2 = (be ? be : 1) - 1075;
  return (b >> 63) ? -mag : mag;
}

// Scale exponent of a row / column from the largest sum of absolute limbs
// M: the frexp exponent of M, plus one when M lies within 2^-29 of 2^e.
__device__ __forceinline__ int scale_exp(double M) {
  if (!(M > 0.0)) return 0;
  int e;
  frexp(M, &e);
  if (M > ldexp(1.0 - ldexp(1.0, -29), e)) e += 1;
  return e;
}

}  // namespace mdgi

/*
 * oracle.c -- CPU restatement of the reference's multi-double GEMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  It is plain C, compiled with -ffp-contract=off so that every product
 * is rounded on its own as the reference's host code is.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the reference's
 * own functions (built from its sources by oracle/Makefile into oracle/_ref)
 * and tests/test_oracle_golden.py checks this file against them bit for bit.
 *
 * Sections and the reference code each one restates:
 *   1. error-free transforms        double_double_functions.cu:11-53,150-195
 *   2. double-double operations     double_double_functions.cu:26-279
 *   3. P-double operations          quad_double_functions.cu:14-537 and the
 *                                   octo/hexa files (same algorithms, P=8,16)
 *   4. plain GEMM                   TCcuda.cu:320-372 (matmul{dd,qd,od,hd}f)
 *   5. floatybits split + balance   floatybits.cu:122-342
 *   6. squeeze                      TCcuda.cu:876-958 (pllsqueeze_*_pp_old)
 *   7. FP64 split-form GEMM         TCtest.cu:21-46 with TCcuda.cu:79-95
 *   8. slice-digit form             the tensor-core form of this library:
 *                                   exact integer digits, exact diagonal
 *                                   sums, rounding back to P limbs
 *   9. input generator              this library's counter-based generator
 *                                   (mdg_generate); its reference family is
 *                                   random_pd, floatybits.cu:107-120
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PMAX 16

/* ------------------------------------------------------------------ 1 -- */

static double qts(double a, double b, double *e) {
  double s = a + b;
  *e = b - (s - a);
  return s;
}
static double tsum(double a, double b, double *e) {
  double s = a + b, bb = s - a;
  *e = (a - (s - bb)) + (b - bb);
  return s;
}
static double tdiff(double a, double b, double *e) {
  double s = a - b, bb = s - a;
  *e = (a - (s - bb)) - (b + bb);
  return s;
}
static void vsplit(double a, double *hi, double *lo) {
  const double sp = 134217729.0, th = 6.69692879491417e+299;
  double t;
  if (a > th || a < -th) {
    a *= 3.7252902984619140625e-09;
    t = sp * a;
    *hi = t - (t - a);
    *lo = a - *hi;
    *hi *= 268435456.0;
    *lo *= 268435456.0;
  } else {
    t = sp * a;
    *hi = t - (t - a);
    *lo = a - *hi;
  }
}
static double tprod(double a, double b, double *e) {
  double p = a * b, ah, al, bh, bl;
  vsplit(a, &ah, &al);
  vsplit(b, &bh, &bl);
  *e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
  return p;
}

/* ------------------------------------------------------------------ 2 -- */

void orc_dd_add(double ah, double al, double bh, double bl, double *ch,
                double *cl) {
  double s1, s2, t1, t2;
  s1 = tsum(ah, bh, &s2);
  t1 = tsum(al, bl, &t2);
  s2 += t1;
  s1 = qts(s1, s2, &s2);
  s2 += t2;
  *ch = qts(s1, s2, cl);
}
void orc_dd_sub(double ah, double al, double bh, double bl, double *ch,
                double *cl) {
  double s1, s2, t1, t2;
  s1 = tdiff(ah, bh, &s2);
  t1 = tdiff(al, bl, &t2);
  s2 += t1;
  s1 = qts(s1, s2, &s2);
  s2 += t2;
  *ch = qts(s1, s2, cl);
}
void orc_dd_mul(double ah, double al, double bh, double bl, double *ch,
                double *cl) {
  double p1, p2;
  p1 = tprod(ah, bh, &p2);
  p2 += (ah * bl + al * bh);
  *ch = qts(p1, p2, cl);
}
void orc_dd_inc_d(double *ah, double *al, double b) {
  double s1, s2;
  s1 = tsum(*ah, b, &s2);
  s2 += *al;
  *ah = qts(s1, s2, al);
}
static void dd_mul_d_dd(double a, double bh, double bl, double *ch,
                        double *cl) {
  double p1, p2;
  p1 = tprod(a, bh, &p2);
  p2 += (bl * a);
  *ch = qts(p1, p2, cl);
}
void orc_dd_div(double ah, double al, double bh, double bl, double *ch,
                double *cl) {
  double q1, q2, q3, xh, xl;
  q1 = ah / bh;
  dd_mul_d_dd(q1, bh, bl, &xh, &xl);
  orc_dd_sub(ah, al, xh, xl, ch, cl);
  q2 = *ch / bh;
  dd_mul_d_dd(q2, bh, bl, &xh, &xl);
  orc_dd_sub(*ch, *cl, xh, xl, ch, cl);
  q3 = *ch / bh;
  *ch = qts(q1, q2, cl);
  orc_dd_inc_d(ch, cl, q3);
}
static void dd_sqr(double ah, double al, double *bh, double *bl) {
  double p1, p2, h, l;
  double q = ah * ah;
  vsplit(ah, &h, &l);
  p2 = ((h * h - q) + 2.0 * h * l) + l * l;
  p1 = q;
  p2 += 2.0 * ah * al;
  p2 += al * al;
  *bh = qts(p1, p2, bl);
}
void orc_dd_sqrt(double ah, double al, double *bh, double *bl) {
  if (ah == 0.0 && al == 0.0) {
    *bh = 0.0;
    *bl = 0.0;
  } else if (ah < 0.0) {
    *bh = -1.0;
    *bl = 0.0;
  } else {
    double x = 1.0 / sqrt(ah), ax = ah * x, sh, sl, yh, yl;
    dd_sqr(ax, 0.0, &sh, &sl);
    orc_dd_sub(ah, al, sh, sl, &yh, &yl);
    *bh = tsum(ax, yh * x * 0.5, bl);
  }
}

/* ------------------------------------------------------------------ 3 -- */

/* Hida-Li-Bailey renormalisation of f[0..P] into r[0..P-1]
 * (quad_double_functions.cu:14-152 for P=4). */
double orc_renorm(int P, const double *f, double *r) {
  double pr, e;
  int ptr, i;
  if (f[1] == 0.0) {
    pr = f[0];
    ptr = 0;
  } else {
    r[0] = f[0];
    pr = f[1];
    ptr = 1;
  }
  for (i = 2; i <= P; ++i) {
    r[ptr] = qts(pr, f[i], &e);
    if (e == 0.0) {
      pr = r[ptr];
    } else {
      pr = e;
      ++ptr;
    }
  }
  if (ptr < P && pr != 0.0) r[ptr++] = pr;
  for (i = ptr; i < P; ++i) r[i] = 0.0;
  return pr;
}

void orc_fast_renorm(int P, const double *x, double *r) {
  double f[PMAX + 1], pr;
  int i;
  pr = qts(x[P - 1], x[P], &f[P]);
  for (i = P - 2; i >= 1; --i) pr = qts(x[i], pr, &f[i + 1]);
  f[0] = qts(x[0], pr, &f[1]);
  orc_renorm(P, f, r);
}

void orc_renorm_add1(int P, const double *x, double y, double *r) {
  double f[PMAX + 1], pr;
  int i;
  pr = tsum(x[P - 1], y, &f[P]);
  for (i = P - 2; i >= 1; --i) pr = tsum(x[i], pr, &f[i + 1]);
  f[0] = tsum(x[0], pr, &f[1]);
  orc_renorm(P, f, r);
}

/* baileyAdd_fast<P,P,P> (quad_double_functions.cu:216-242). */
void orc_pd_add(int P, const double *a, const double *b, double *c) {
  double f[PMAX + 1], e;
  int i, t;
  if (P == 2) {
    orc_dd_add(a[0], a[1], b[0], b[1], &c[0], &c[1]);
    return;
  }
  f[P] = 0.0;
  for (i = P - 1; i >= 0; --i) {
    f[i] = tsum(a[i], b[i], &e);
    for (t = i + 1; t < P; ++t) f[t] = tsum(f[t], e, &e);
    f[P] += e;
  }
  orc_fast_renorm(P, f, c);
}

/* baileyMul_fast<P,P,P> (quad_double_functions.cu:321-381). */
void orc_pd_mul(int P, const double *a, const double *b, double *c) {
  double f[PMAX + 1], p, e;
  int i, d, t;
  if (P == 2) {
    orc_dd_mul(a[0], a[1], b[0], b[1], &c[0], &c[1]);
    return;
  }
  f[P] = a[1] * b[P - 1];
  for (i = 2; i < P; ++i) f[P] += a[i] * b[P - i];
  for (d = P - 1; d >= 0; --d) {
    f[d] = tprod(a[0], b[d], &e);
    for (t = d + 1; t < P; ++t) f[t] = tsum(f[t], e, &e);
    f[P] += e;
    for (i = 1; i <= d; ++i) {
      p = tprod(a[i], b[d - i], &e);
      for (t = d + 1; t < P; ++t) f[t] = tsum(f[t], e, &e);
      f[P] += e;
      f[d] = tsum(f[d], p, &e);
      for (t = d + 1; t < P; ++t) f[t] = tsum(f[t], e, &e);
      f[P] += e;
    }
  }
  orc_fast_renorm(P, f, c);
}

/* baileyMul_fast<P,1,P> (quad_double_functions.cu:442-468). */
void orc_pd_mul_d(int P, const double *a, double b, double *c) {
  double f[PMAX + 1], e;
  int i, t;
  f[P] = 0.0;
  for (i = P - 1; i >= 0; --i) {
    f[i] = tprod(a[i], b, &e);
    for (t = i + 1; t < P; ++t) f[t] = tsum(f[t], e, &e);
    f[P] += e;
  }
  orc_fast_renorm(P, f, c);
}

void orc_pd_sub(int P, const double *a, const double *b, double *c) {
  double nb[PMAX];
  int i;
  if (P == 2) {
    orc_dd_sub(a[0], a[1], b[0], b[1], &c[0], &c[1]);
    return;
  }
  for (i = 0; i < P; ++i) nb[i] = -b[i];
  orc_pd_add(P, nb, a, c);
}

/* Long division (quad_double_functions.cu:485-520). */
void orc_pd_div(int P, const double *a, const double *b, double *c) {
  double q[PMAX + 1], acc[PMAX], rem[PMAX], t[PMAX];
  int i, j;
  if (P == 2) {
    orc_dd_div(a[0], a[1], b[0], b[1], &c[0], &c[1]);
    return;
  }
  for (i = 0; i < P; ++i) rem[i] = a[i];
  for (i = 0; i < P; ++i) {
    q[i] = rem[0] / b[0];
    orc_pd_mul_d(P, b, q[i], acc);
    orc_pd_sub(P, rem, acc, t);
    for (j = 0; j < P; ++j) rem[j] = t[j];
  }
  q[P] = rem[0] / b[0];
  orc_fast_renorm(P, q, c);
}

/* Newton step on the square root of the leading half
 * (quad_double_functions.cu:524-537). */
void orc_pd_sqrt(int P, const double *a, double *b) {
  double h[PMAX], z[PMAX], t[PMAX];
  int i;
  if (P == 2) {
    orc_dd_sqrt(a[0], a[1], &b[0], &b[1]);
    return;
  }
  for (i = 0; i < P; ++i) h[i] = 0.0;
  orc_pd_sqrt(P / 2, a, h);
  orc_pd_mul(P, h, h, z);
  orc_pd_add(P, z, a, t);
  orc_pd_div(P, t, h, z);
  for (i = 0; i < P; ++i) b[i] = z[i] * 0.5;
}

void orc_pd_inc_d(int P, double *y, double x) {
  double r[PMAX];
  int i;
  if (P == 2) {
    orc_dd_inc_d(&y[0], &y[1], x);
    return;
  }
  orc_renorm_add1(P, y, x, r);
  for (i = 0; i < P; ++i) y[i] = r[i];
}

/* Element-wise kernels over n P-doubles, used by the golden tests. */
void orc_vec_binop(int op, int P, long n, const double *a, const double *b,
                   double *c) {
  long i;
  for (i = 0; i < n; ++i) {
    const double *x = a + i * P, *y = b + i * P;
    double *z = c + i * P;
    switch (op) {
      case 0: orc_pd_add(P, x, y, z); break;
      case 1: orc_pd_mul(P, x, y, z); break;
      case 2: orc_pd_sub(P, x, y, z); break;
      case 3: orc_pd_div(P, x, y, z); break;
      case 4: orc_pd_sqrt(P, x, z); break;
      case 5: {
        int j;
        for (j = 0; j < P; ++j) z[j] = x[j];
        orc_pd_inc_d(P, z, y[0]);
        break;
      }
      case 6:
        if (P == 2) dd_mul_d_dd(y[0], x[0], x[1], &z[0], &z[1]);
        else orc_pd_mul_d(P, x, y[0], z);
        break;
      default: break;
    }
  }
}

/* ------------------------------------------------------------------ 4 -- */

/* C = A*B for row-major arrays of P-doubles (limbs contiguous), the loop of
 * matmul{dd,qd,od,hd}f (TCcuda.cu:320-372) generalised to m x k by k x n.
 * Rows [r0, r1) only; threads > 1 splits the rows with OpenMP. */
void orc_gemm_plain_rows(int P, int m, int n, int k, const double *A,
                         const double *B, double *C, int r0, int r1,
                         int threads) {
  int r;
  (void)m;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
#endif
  for (r = r0; r < r1; ++r) {
    int c, kk, l;
    for (c = 0; c < n; ++c) {
      double acc[PMAX], t[PMAX], s[PMAX];
      for (l = 0; l < P; ++l) acc[l] = 0.0;
      for (kk = 0; kk < k; ++kk) {
        orc_pd_mul(P, A + ((long)r * k + kk) * P, B + ((long)kk * n + c) * P,
                   t);
        orc_pd_add(P, acc, t, s);
        for (l = 0; l < P; ++l) acc[l] = s[l];
      }
      for (l = 0; l < P; ++l) C[((long)r * n + c) * P + l] = acc[l];
    }
  }
  (void)threads;
}

void orc_gemm_plain(int P, int m, int n, int k, const double *A,
                    const double *B, double *C) {
  orc_gemm_plain_rows(P, m, n, k, A, B, C, 0, m, 1);
}

/* ------------------------------------------------------------------ 5 -- */

/* The reference turns a double into a vector of 64 ints (floatybits.cu:54,
 * 16-33): a sign, the frexp exponent, and the binary expansion of the frexp
 * fraction.  The expansion loop only runs for positive fractions, so the
 * fraction of a negative double is all zeros, and only the first 52 bits of
 * the 53-bit expansion are read back (floatybits.cu:92-102).  Slices are the
 * values of fraction-bit ranges [lo, hi) times 2^e; a zero slice of a
 * negative number is -0.0 (pow(-1,1) * 0 * 2^e). */
static double slice_of(double x, int lo, int hi, int *is_neg) {
  int e;
  double f = frexp(x, &e);
  uint64_t F, bits;
  *is_neg = !(x >= 0);
  if (*is_neg) return -0.0;
  if (f <= 0.0) return 0.0;                 /* +0 or -0 input */
  F = (uint64_t)ldexp(f, 52);               /* first 52 fraction bits */
  bits = (F >> (52 - hi)) & ((((uint64_t)1) << (hi - lo)) - 1);
  return ldexp((double)bits, e - hi);
}

static double trunc52(double x) {
  int e;
  double f = frexp(x, &e);
  if (!(x >= 0)) return -0.0;
  if (f <= 0.0) return 0.0;
  return ldexp((double)(uint64_t)ldexp(f, 52), e - 52);
}

static const int RANGES4[5] = {0, 13, 26, 39, 52};
static const int RANGES8[8] = {0, 7, 14, 21, 28, 34, 40, 52};

/* split4 (floatybits.cu:159-191): three 13-bit ranges and the remainder. */
static void split4_ref(double x, double *out) {
  int neg, t;
  double s = 0.0;
  for (t = 0; t < 3; ++t) out[t] = slice_of(x, RANGES4[t], RANGES4[t + 1], &neg);
  s = (out[0] + out[1]) + out[2];
  out[3] = trunc52(x) - s;
}

/* split8 (floatybits.cu:218-301): seven ranges 7,7,7,7,6,6,12 and the
 * remainder, which is zero for every input. */
static void split8_ref(double x, double *out) {
  int neg, t;
  double s;
  for (t = 0; t < 7; ++t) out[t] = slice_of(x, RANGES8[t], RANGES8[t + 1], &neg);
  s = out[0];
  for (t = 1; t < 7; ++t) s = s + out[t];
  out[7] = trunc52(x) - s;
}

/* balance (floatybits.cu:122-148): move one unit 2^(ex - th) from x to y
 * when the frexp exponents of x and y are more than th-1 apart. */
static void balance_ref(double *x, double *y, int th) {
  int xe, ye;
  if (*x == 0.0 || *y == 0.0) return;
  frexp(*x, &xe);
  frexp(*y, &ye);
  if (!(xe - ye > th - 1)) return;
  {
    double bit = ldexp(1.0, xe - th);
    *x = *x - bit;
    *y = *y + bit;
  }
}

/* Signed variant used by the exact mode: move the unit toward zero on both
 * sides when x and y share a sign, leave mixed-sign pairs alone. */
static void balance_exact(double *x, double *y, int th) {
  int xe, ye;
  if (*x == 0.0 || *y == 0.0) return;
  if ((*x < 0) != (*y < 0)) return;
  frexp(*x, &xe);
  frexp(*y, &ye);
  if (!(xe - ye > th - 1)) return;
  {
    double bit = ldexp(1.0, xe - th);
    if (*x < 0) bit = -bit;
    *x = *x - bit;
    *y = *y + bit;
  }
}

/* Exact splits: the ranges of the reference, applied to |x| with all 53
 * significand bits (the last range takes the 53rd bit), sign restored. */
static void split_exact(double x, const int *ranges, int nr, double *out) {
  int e, t;
  double f, ax = fabs(x);
  uint64_t F;
  if (ax == 0.0) {
    for (t = 0; t < nr; ++t) out[t] = 0.0;
    return;
  }
  f = frexp(ax, &e);
  F = (uint64_t)ldexp(f, 53);
  for (t = 0; t < nr; ++t) {
    int lo = ranges[t], hi = (t == nr - 1) ? 53 : ranges[t + 1];
    uint64_t bits = (F >> (53 - hi)) & ((((uint64_t)1) << (hi - lo)) - 1);
    double v = ldexp((double)bits, e - hi);
    out[t] = (x < 0) ? -v : v;
  }
}

/* kind: 0 = split4 (pp = 4p), 1 = split8 (pp = 8p), 2 = mixed dd split
 * (pp = 12, p must be 2).  exact: 0 reproduces the reference bit for bit,
 * 1 keeps signs and the 53rd bit.  x holds n P-doubles; out n*pp slices. */
void orc_split(int kind, int exact, int P, long n, const double *x,
               double *out) {
  long i;
  int l, j;
  for (i = 0; i < n; ++i) {
    const double *xi = x + i * P;
    int pp = kind == 0 ? 4 * P : kind == 1 ? 8 * P : 12;
    double *o = out + i * pp, *w = o;
    for (l = 0; l < P; ++l) {
      int use8 = (kind == 1) || (kind == 2 && l == 1);
      if (!exact) {
        if (use8) split8_ref(xi[l], w);
        else split4_ref(xi[l], w);
      } else {
        static const int r8x[7] = {0, 7, 14, 21, 28, 34, 40};
        if (use8) {
          split_exact(xi[l], r8x, 7, w);
          w[7] = 0.0;
        } else {
          split_exact(xi[l], RANGES4, 4, w);
        }
      }
      w += use8 ? 8 : 4;
    }
    /* balance4 / balance8 / mixbalance (floatybits.cu:150-154, 208-216,
     * 315-325) over the slices of one p-double, last pair(s) excluded. */
    for (j = 0; j + 1 < pp; ++j) {
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
      if (exact) balance_exact(&o[j], &o[j + 1], th);
      else balance_ref(&o[j], &o[j + 1], th);
    }
  }
}

/* ------------------------------------------------------------------ 6 -- */

/* y = sum_j x[j] over pp partial sums per entry, added one at a time with
 * the P-double inc_d (TCcuda.cu:876-906). */
void orc_squeeze(int P, int pp, long n, const double *x, double *y) {
  long i;
  int j, l;
  for (i = 0; i < n; ++i) {
    double acc[PMAX];
    for (l = 0; l < P; ++l) acc[l] = 0.0;
    for (j = 0; j < pp; ++j) orc_pd_inc_d(P, acc, x[i * pp + j]);
    for (l = 0; l < P; ++l) y[i * P + l] = acc[l];
  }
}

/* ------------------------------------------------------------------ 7 -- */

/* Truncated Cauchy product of slice sequences, FP64 accumulation:
 * Cq[r][c][i] = sum_k sum_{j<=i} Aq[r][k][j] * Bq[k][c][i-j], the product
 * the DMMA kernel forms against the block-Toeplitz matrix (TCtest.cu:21-46,
 * TCcuda.cu:79-95).  The sum runs over k outer, j inner, like the flattened
 * index k*pp+j of the reference.  Aq is m x k x pp, Bq is k x n x pp. */
void orc_slice_conv_rows(int pp, int m, int n, int k, const double *Aq,
                         const double *Bq, double *Cq, int r0, int r1,
                         int threads) {
  int r;
  (void)m;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
#endif
  for (r = r0; r < r1; ++r) {
    int c, i, kk, j;
    for (c = 0; c < n; ++c)
      for (i = 0; i < pp; ++i) {
        double s = 0.0;
        for (kk = 0; kk < k; ++kk)
          for (j = 0; j <= i; ++j)
            s += Aq[((long)r * k + kk) * pp + j] *
                 Bq[((long)kk * n + c) * pp + (i - j)];
        Cq[((long)r * n + c) * pp + i] = s;
      }
  }
  (void)threads;
}

/* The reference's CPU path on slice planes (TCcudant.cpp:216-250): every
 * plane pair (i, j) multiplied with k increasing (convmult2), then
 * C_i = sum_{j <= i} aux[j][i-j] in increasing j (convadd2).  A and B are pp
 * planes of n x n, row-major. */
void orc_plane_conv(int n, int pp, const double *A, const double *B,
                    double *C) {
  long nn = (long)n * n;
  double *aux = (double *)calloc((size_t)pp * pp * nn, sizeof(double));
  int i, j, r, c, kk;
  for (i = 0; i < pp; ++i)
    for (j = 0; j < pp; ++j)
      for (r = 0; r < n; ++r)
        for (c = 0; c < n; ++c) {
          double s = 0.0;
          for (kk = 0; kk < n; ++kk)
            s += A[i * nn + (long)r * n + kk] * B[j * nn + (long)kk * n + c];
          aux[((long)i * pp + j) * nn + (long)r * n + c] = s;
        }
  for (i = 0; i < pp; ++i)
    for (r = 0; r < n; ++r)
      for (c = 0; c < n; ++c) {
        double s = 0.0;
        for (j = 0; j <= i; ++j)
          s += aux[((long)j * pp + (i - j)) * nn + (long)r * n + c];
        C[i * nn + (long)r * n + c] = s;
      }
  free(aux);
}

/* ------------------------------------------------------------------ 8 -- */

/* Slice-digit form.  Every row r of A gets a scale exponent E[r] and every
 * column c of B a scale exponent F[c]; each P-double a is written exactly
 * as a signed integer V = sum_l floor(a_l * 2^(S - E)), S = 7 + 8 (s - 1),
 * and V as s balanced base-256 digits d_0 (most significant) .. d_{s-1},
 * each in [-128, 128].  The product of two digit planes is exact in BF16
 * with FP32 accumulation; the sums C_d = sum_{i+j=d} A_i B_j over the
 * D diagonals d < D are exact integers; the result is
 * W = sum_d C_d 256^(D-1-d) scaled by 2^(E + F - 14 - 8 (D-1)), rounded to
 * P limbs, each to nearest. */

#define NW 16 /* 64-bit words of the fixed-point integers: 1024 bits */

typedef struct { uint64_t w[NW]; } bigint; /* two's complement, w[0] low */

static void bi_zero(bigint *a) { memset(a, 0, sizeof *a); }
static void bi_add(bigint *a, const bigint *b) {
  unsigned __int128 c = 0;
  int i;
  for (i = 0; i < NW; ++i) {
    c += (unsigned __int128)a->w[i] + b->w[i];
    a->w[i] = (uint64_t)c;
    c >>= 64;
  }
}
static void bi_neg(bigint *a) {
  int i;
  unsigned __int128 c = 1;
  for (i = 0; i < NW; ++i) {
    c += (uint64_t)~a->w[i];
    a->w[i] = (uint64_t)c;
    c >>= 64;
  }
}
static int bi_sign(const bigint *a) { return (int64_t)a->w[NW - 1] < 0; }
static int bi_is_zero(const bigint *a) {
  int i;
  for (i = 0; i < NW; ++i)
    if (a->w[i]) return 0;
  return 1;
}
/* a = (int64) v << sh, sh >= 0 */
static void bi_from_i64_shl(bigint *a, int64_t v, int sh) {
  int i, q = sh / 64, rr = sh % 64;
  uint64_t fill = v < 0 ? ~(uint64_t)0 : 0;
  for (i = 0; i < NW; ++i) a->w[i] = (i < q) ? 0 : fill;
  if (q < NW) {
    a->w[q] = (uint64_t)v << rr;
    if (q + 1 < NW)
      a->w[q + 1] = rr ? (uint64_t)(v >> (64 - rr)) : fill;
  }
}
/* arithmetic right shift by 0 < sh < 64 */
static void bi_sar(bigint *a, int sh) {
  int i;
  for (i = 0; i < NW - 1; ++i)
    a->w[i] = (a->w[i] >> sh) | (a->w[i + 1] << (64 - sh));
  a->w[NW - 1] = (uint64_t)((int64_t)a->w[NW - 1] >> sh);
}
static int bi_msb(const bigint *a) { /* of a non-negative value, -1 if 0 */
  int i;
  for (i = NW - 1; i >= 0; --i)
    if (a->w[i]) return i * 64 + 63 - __builtin_clzll(a->w[i]);
  return -1;
}
static int bi_bit(const bigint *a, int b) {
  return (int)((a->w[b / 64] >> (b % 64)) & 1);
}

/* Scale exponent of a row / column: M = max over entries of the sum of the
 * absolute limbs (added left to right), e = frexp exponent of M, plus one
 * when M lies within 2^-29 of 2^e, so that every entry is at most 2^e. */
int orc_scale_exp(double M) {
  int e;
  if (!(M > 0.0)) return 0;
  frexp(M, &e);
  if (M > ldexp(1.0 - ldexp(1.0, -29), e)) e += 1;
  return e;
}

double orc_abs_limb_sum(int P, const double *a) {
  double s = fabs(a[0]);
  int l;
  for (l = 1; l < P; ++l) s = s + fabs(a[l]);
  return s;
}

/* Row exponents of A (m x k) and column exponents of B (k x n). */
void orc_scale_exps(int P, int m, int n, int k, const double *A,
                    const double *B, int *E, int *F) {
  int r, c, kk;
  for (r = 0; r < m; ++r) {
    double M = 0.0;
    for (kk = 0; kk < k; ++kk) {
      double v = orc_abs_limb_sum(P, A + ((long)r * k + kk) * P);
      if (v > M) M = v;
    }
    E[r] = orc_scale_exp(M);
  }
  for (c = 0; c < n; ++c) {
    double M = 0.0;
    for (kk = 0; kk < k; ++kk) {
      double v = orc_abs_limb_sum(P, B + ((long)kk * n + c) * P);
      if (v > M) M = v;
    }
    F[c] = orc_scale_exp(M);
  }
}

/* V = sum_l floor(a_l * 2^(S - E)) for a P-double a. */
static void fixed_point(int P, const double *a, int S, int E, bigint *V) {
  int l;
  bi_zero(V);
  for (l = 0; l < P; ++l) {
    double x = a[l];
    int e, q;
    double f;
    int64_t m;
    bigint t;
    if (x == 0.0) continue;
    f = frexp(x, &e);
    m = (int64_t)ldexp(f, 53);      /* |m| in [2^52, 2^53) */
    q = e - 53 + S - E;             /* x * 2^(S-E) = m * 2^q */
    if (q >= 0) {
      bi_from_i64_shl(&t, m, q);
    } else if (q > -64) {
      bi_from_i64_shl(&t, m >> (-q), 0); /* arithmetic shift = floor */
    } else {
      bi_from_i64_shl(&t, m < 0 ? -1 : 0, 0);
    }
    bi_add(V, &t);
  }
}

/* Balanced base-2^b digits of V: d[s-1] .. d[1] from the bottom, each
 * ((V + h) mod 2^b) - h with h = 2^(b-1), V <- floor((V + h) / 2^b);
 * d[0] = V.  b = 8 for the BF16 form, 19 for the FP64 digit form. */
static void digits_of_b(bigint *V, int s, int b, int *d) {
  int i;
  bigint half;
  bi_from_i64_shl(&half, (int64_t)1 << (b - 1), 0);
  for (i = s - 1; i >= 1; --i) {
    bi_add(V, &half);
    d[i] = (int)(V->w[0] & (((uint64_t)1 << b) - 1)) - (1 << (b - 1));
    bi_sar(V, b);
  }
  d[0] = (int)(int64_t)V->w[0];
}

/* Digit planes of A: out[i][r][kk] for i < s (int8 values stored as int32
 * here).  trans = 0: x is m x k (rows scaled by E);  trans = 1: x is k x n
 * (columns scaled by E) and the planes are n x k. */
static void digits_b(int P, int s, int bits, int rows, int cols, const double *x,
                     const int *E, int trans, int *out);

void orc_digits(int P, int s, int rows, int cols, const double *x,
                const int *E, int trans, int *out) {
  digits_b(P, s, 8, rows, cols, x, E, trans, out);
}

/* The same with b-bit digits, S = (b - 1) + b (s - 1). */
static void digits_b(int P, int s, int bits, int rows, int cols, const double *x,
                     const int *E, int trans, int *out) {
  int S = (bits - 1) + bits * (s - 1);
  int r, c, i, d[512];
  long plane = (long)rows * cols;
  for (r = 0; r < rows; ++r)
    for (c = 0; c < cols; ++c) {
      bigint V;
      const double *a;
      int e;
      long o;
      if (!trans) {
        a = x + ((long)r * cols + c) * P;
        e = E[r];
        o = (long)r * cols + c;
      } else {
        /* x is cols(k) x rows(n): entry (kk = c, col = r) */
        a = x + ((long)c * rows + r) * P;
        e = E[r];
        o = (long)r * cols + c;
      }
      fixed_point(P, a, S, e, &V);
      digits_of_b(&V, s, bits, d);
      for (i = 0; i < s; ++i) out[i * plane + o] = d[i];
    }
}

/* Exact diagonal sums C_d[r][c] = sum_{i+j=d} sum_kk dA_i[r][kk] dB_j[c][kk]
 * for d < D (int64).  dA: s planes m x k;  dB: s planes n x k. */
void orc_diag_sums(int s, int D, int m, int n, int k, const int *dA,
                   const int *dB, int64_t *Cd) {
  long pa = (long)m * k, pb = (long)n * k, pc = (long)m * n;
  int d, i, r, c, kk;
  for (d = 0; d < D; ++d)
    for (r = 0; r < m; ++r)
      for (c = 0; c < n; ++c) {
        int64_t acc = 0;
        for (i = 0; i <= d; ++i) {
          int j = d - i;
          const int *a, *b;
          if (i >= s || j >= s) continue;
          a = dA + i * pa + (long)r * k;
          b = dB + j * pb + (long)c * k;
          for (kk = 0; kk < k; ++kk) acc += (int64_t)a[kk] * b[kk];
        }
        Cd[d * pc + (long)r * n + c] = acc;
      }
}

/* Round the integer W (non-negative or negative) to nearest-even double. */
static double bi_round_to_double(const bigint *W, bigint *rounded) {
  bigint a = *W;
  int neg = bi_sign(&a), t, i;
  double v;
  if (neg) bi_neg(&a);
  t = bi_msb(&a);
  if (t < 0) {
    bi_zero(rounded);
    return 0.0;
  }
  if (t < 53) {
    uint64_t m = a.w[0];
    v = (double)m;
    *rounded = *W;
    return neg ? -v : v;
  }
  {
    int sh = t - 52; /* keep bits t..sh (53 bits) */
    uint64_t m = 0;
    int rb, sticky = 0;
    for (i = 52; i >= 0; --i) m = (m << 1) | (uint64_t)bi_bit(&a, sh + i);
    rb = bi_bit(&a, sh - 1);
    for (i = 0; i < sh - 1 && !sticky; ++i) sticky |= bi_bit(&a, i);
    if (rb && (sticky || (m & 1))) m += 1;
    v = ldexp((double)m, sh);
    bi_from_i64_shl(rounded, (int64_t)m, sh);
    if (neg) {
      bi_neg(rounded);
      v = -v;
    }
    return v;
  }
}

/* Limbs of W * 2^scale: limb i = RN(W - limbs 0..i-1), then scaled. */
static void to_limbs(int P, bigint *W, int scale, double *out) {
  int l;
  for (l = 0; l < P; ++l) {
    bigint R;
    double v = bi_round_to_double(W, &R);
    out[l] = ldexp(v, scale);
    bi_neg(&R);
    bi_add(W, &R);
  }
}

static void renorm_diags_b(int P, int D, int bits, int m, int n, const int64_t *Cd,
                           const int *E, const int *F, double *C);

void orc_renorm_diags(int P, int D, int m, int n, const int64_t *Cd,
                      const int *E, const int *F, double *C) {
  renorm_diags_b(P, D, 8, m, n, Cd, E, F, C);
}

/* W = sum_d C_d 2^(b (D-1-d)), times 2^(E + F - 2 (b - 1) - b (D - 1)). */
static void renorm_diags_b(int P, int D, int bits, int m, int n, const int64_t *Cd,
                           const int *E, const int *F, double *C) {
  long pc = (long)m * n;
  int r, c, d;
  for (r = 0; r < m; ++r)
    for (c = 0; c < n; ++c) {
      bigint W, t;
      bi_zero(&W);
      for (d = 0; d < D; ++d) {
        int64_t v = Cd[d * pc + (long)r * n + c];
        if (!v) continue;
        bi_from_i64_shl(&t, v, bits * (D - 1 - d));
        bi_add(&W, &t);
      }
      to_limbs(P, &W, E[r] + F[c] - 2 * (bits - 1) - bits * (D - 1),
               C + ((long)r * n + c) * P);
    }
}

static void gemm_digits_b(int P, int s, int D, int bits, int m, int n, int k,
                          const double *A, const double *B, double *C);

/* Whole slice-digit GEMM on the CPU, for small sizes. */
void orc_gemm_slices(int P, int s, int D, int m, int n, int k,
                     const double *A, const double *B, double *C) {
  gemm_digits_b(P, s, D, 8, m, n, k, A, B, C);
}

/* The FP64 digit form: the same scheme with 19-bit digits (the library's
 * MDG_FORM_FP64_DIGITS).  Its digit products are summed exactly, so the
 * result does not depend on the order of the FP64 tensor-core sums. */
void orc_gemm_digits(int P, int s, int D, int m, int n, int k,
                     const double *A, const double *B, double *C) {
  gemm_digits_b(P, s, D, 19, m, n, k, A, B, C);
}

static void gemm_digits_b(int P, int s, int D, int bits, int m, int n, int k,
                          const double *A, const double *B, double *C) {
  int *E = (int *)malloc(sizeof(int) * m), *F = (int *)malloc(sizeof(int) * n);
  int *dA = (int *)malloc(sizeof(int) * (size_t)s * m * k);
  int *dB = (int *)malloc(sizeof(int) * (size_t)s * n * k);
  int64_t *Cd = (int64_t *)malloc(sizeof(int64_t) * (size_t)D * m * n);
  orc_scale_exps(P, m, n, k, A, B, E, F);
  digits_b(P, s, bits, m, k, A, E, 0, dA);
  digits_b(P, s, bits, n, k, B, F, 1, dB);
  orc_diag_sums(s, D, m, n, k, dA, dB, Cd);
  renorm_diags_b(P, D, bits, m, n, Cd, E, F, C);
  free(E);
  free(F);
  free(dA);
  free(dB);
  free(Cd);
}

/* ------------------------------------------------------------------ 9 -- */

/* splitmix64 finaliser (Vigna), the only source of randomness. */
static uint64_t gen_mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* Word j of the stream with base b (streams: one per entry, row, column). */
static uint64_t gen_word(uint64_t key, uint64_t index, int j) {
  const uint64_t b = gen_mix(key ^ (index * 0xd1342543de82ef95ull));
  return gen_mix(b + (uint64_t)(j + 1) * 0x9e3779b97f4a7c15ull);
}

static double gen_unit(uint64_t w) { /* (k - 2^52) 2^-52, k the top 53 bits */
  return ldexp((double)((int64_t)(w >> 11) - ((int64_t)1 << 52)), -52);
}

/* dist: 0 uniform, 1 normal (Irwin-Hall of 12), 2 random_pd family; +4 row
 * scales, +8 column scales 2^U{e0..e1}.  X is rows x cols x P, dense. */
void orc_generate(int dist, int P, int rows, int cols, uint64_t seed, int e0, int e1,
                  double *X) {
  const uint64_t key = gen_mix(seed);
  const uint64_t ke = gen_mix(key ^ 0x5851f42d4c957f2dull);
  const uint64_t kr = gen_mix(key ^ 0xa0761d6478bd642full);
  const uint64_t kc = gen_mix(key ^ 0xe7037ed1a0b428dbull);
  const int kind = dist & 3;
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) {
      const uint64_t e = (uint64_t)r * (uint64_t)cols + (uint64_t)c;
      double *x = X + e * (uint64_t)P;
      if (kind == 2) {
        int ex = e0;
        if (e1 != e0) ex += (int)(gen_word(ke, e, 0) % (uint64_t)(e1 - e0));
        for (int i = 0; i < P; ++i) {
          const uint64_t f = ((uint64_t)1 << 51) | (gen_word(ke, e, 1 + i) >> 13);
          x[i] = ldexp((double)f, ex - 52 * i - 52);
        }
        continue;
      }
      int j = 0;
      if (kind == 1) {
        int64_t t = -((int64_t)6 << 53);
        for (; j < 12; ++j) t += (int64_t)(gen_word(ke, e, j) >> 11);
        x[0] = ldexp((double)t, -53);
      } else {
        x[0] = gen_unit(gen_word(ke, e, j++));
      }
      for (int i = 1; i < P; ++i) {
        const double ulp = x[i - 1] == 0.0 ? 0.0 : ldexp(1.0, ilogb(x[i - 1]) - 52);
        x[i] = gen_unit(gen_word(ke, e, j + i - 1)) * ulp * 0.5;
      }
      for (int i = P - 2; i >= 0; --i) {
        double err;
        const double s = qts(x[i], x[i + 1], &err);
        x[i] = s;
        x[i + 1] = err;
      }
      for (int i = 0; i < P - 1; ++i) {
        double err;
        const double s = qts(x[i], x[i + 1], &err);
        x[i] = s;
        x[i + 1] = err;
      }
      int sc = 0;
      if (dist & 4) sc += e0 + (int)(gen_word(kr, (uint64_t)r, 0) % (uint64_t)(e1 - e0 + 1));
      if (dist & 8) sc += e0 + (int)(gen_word(kc, (uint64_t)c, 0) % (uint64_t)(e1 - e0 + 1));
      if (sc)
        for (int i = 0; i < P; ++i) x[i] = ldexp(x[i], sc);
    }
}

int orc_has_openmp(void) {
#ifdef _OPENMP
  return 1;
#else
  return 0;
#endif
}

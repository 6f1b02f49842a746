/*
 * mdg_arith.h -- multi-double arithmetic (double-double, quad-double,
 * octo-double, hexa-double) for host and device, written as one set of
 * templates over the limb count P.
 *
 * A P-double is an unevaluated sum of P doubles, most significant first.
 * The algorithms are the published ones:
 *   - Knuth two-sum, Dekker quick-two-sum, Dekker/Veltkamp two-product
 *     (Dekker 1971; Knuth TAOCP vol. 2);
 *   - the double-double and quad-double renormalisation of Hida, Li and
 *     Bailey ("Algorithms for quad-double precision floating point
 *     arithmetic", ARITH-15, 2001);
 *   - the "fast" Bailey-style addition and multiplication that CAMPARY
 *     generates for P-term expansions (Joldes, Muller, Popescu, Tucker,
 *     "CAMPARY: Cuda Multiple Precision Arithmetic Library", 2016).
 *
 * The order of every floating-point operation follows the functions of the
 * reference library so that a GEMM built on these templates returns the same
 * bits as the reference's:
 *   double_double_functions.cu:11-246, quad_double_functions.cu:14-537,
 *   octo_double_functions.cu:15-1540, hexa_double_functions.cu:16-6360.
 * Those files are unrolled by hand for each P; here one loop nest serves all
 * P in {4, 8, 16}, and P = 2 uses the double-double forms.
 *
 * Floating-point contraction must be off (nvcc -fmad=false, gcc
 * -ffp-contract=off): a fused a*b+c changes the rounding of the plain
 * products that the CAMPARY multiplication accumulates without error terms.
 * On the device the two-product uses one FMA for the error term; on the host
 * it uses Veltkamp splitting. Both return the exact error a*b - fl(a*b) when
 * neither overflow nor underflow occurs, so both give identical bits there.
 */
#ifndef MDG_ARITH_H
#define MDG_ARITH_H

#include <math.h>

#if defined(__CUDACC__)
#define MDG_HD __host__ __device__ __forceinline__
#define MDG_UNROLL _Pragma("unroll")
#else
#define MDG_HD static inline
#define MDG_UNROLL _Pragma("GCC unroll 32")
#endif

namespace mdg {

/* ---------------------------------------------------------------- EFTs -- */

/* s + err == a + b exactly, valid when |a| >= |b| (Dekker). */
MDG_HD double quick_two_sum(double a, double b, double *err) {
  double s = a + b;
  *err = b - (s - a);
  return s;
}

/* s + err == a + b exactly for any a, b (Knuth). */
MDG_HD double two_sum(double a, double b, double *err) {
  double s = a + b;
  double bb = s - a;
  *err = (a - (s - bb)) + (b - bb);
  return s;
}

MDG_HD double quick_two_diff(double a, double b, double *err) {
  double s = a - b;
  *err = (a - s) - b;
  return s;
}

MDG_HD double two_diff(double a, double b, double *err) {
  double s = a - b;
  double bb = s - a;
  *err = (a - (s - bb)) - (b + bb);
  return s;
}

/* Veltkamp splitting of a into two 26-bit halves, with the usual rescale
 * for |a| > 2^996 so that 2^27+1 times a cannot overflow. */
MDG_HD void veltkamp_split(double a, double *hi, double *lo) {
  const double splitter = 134217729.0;            /* 2^27 + 1 */
  const double thresh = 6.69692879491417e+299;    /* 2^996 */
  if (a > thresh || a < -thresh) {
    a *= 3.7252902984619140625e-09;               /* 2^-28 */
    double t = splitter * a;
    *hi = t - (t - a);
    *lo = a - *hi;
    *hi *= 268435456.0;                           /* 2^28 */
    *lo *= 268435456.0;
  } else {
    double t = splitter * a;
    *hi = t - (t - a);
    *lo = a - *hi;
  }
}

/* p + err == a * b exactly (no overflow / underflow). */
MDG_HD double two_prod(double a, double b, double *err) {
  double p = a * b;
#if defined(__CUDA_ARCH__)
  *err = fma(a, b, -p);
#else
  double ah, al, bh, bl;
  veltkamp_split(a, &ah, &al);
  veltkamp_split(b, &bh, &bl);
  *err = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
#endif
  return p;
}

MDG_HD double two_sqr(double a, double *err) {
  double q = a * a;
#if defined(__CUDA_ARCH__)
  *err = fma(a, a, -q);
#else
  double h, l;
  veltkamp_split(a, &h, &l);
  *err = ((h * h - q) + 2.0 * h * l) + l * l;
#endif
  return q;
}

/* ------------------------------------------------------ double-double -- */

MDG_HD void dd_add(double ah, double al, double bh, double bl, double *ch,
                   double *cl) {
  double s1, s2, t1, t2;
  s1 = two_sum(ah, bh, &s2);
  t1 = two_sum(al, bl, &t2);
  s2 += t1;
  s1 = quick_two_sum(s1, s2, &s2);
  s2 += t2;
  *ch = quick_two_sum(s1, s2, cl);
}

MDG_HD void dd_sub(double ah, double al, double bh, double bl, double *ch,
                   double *cl) {
  double s1, s2, t1, t2;
  s1 = two_diff(ah, bh, &s2);
  t1 = two_diff(al, bl, &t2);
  s2 += t1;
  s1 = quick_two_sum(s1, s2, &s2);
  s2 += t2;
  *ch = quick_two_sum(s1, s2, cl);
}

MDG_HD void dd_sub_dd_d(double ah, double al, double b, double *ch,
                        double *cl) {
  double s1, s2;
  s1 = two_diff(ah, b, &s2);
  s2 += al;
  *ch = quick_two_sum(s1, s2, cl);
}

MDG_HD void dd_inc_d(double *ah, double *al, double b) {
  double s1, s2;
  s1 = two_sum(*ah, b, &s2);
  s2 += *al;
  *ah = quick_two_sum(s1, s2, al);
}

MDG_HD void dd_dec_d(double *ah, double *al, double b) {
  double s1, s2;
  s1 = two_diff(*ah, b, &s2);
  s2 += *al;
  *ah = quick_two_sum(s1, s2, al);
}

MDG_HD void dd_mul(double ah, double al, double bh, double bl, double *ch,
                   double *cl) {
  double p1, p2;
  p1 = two_prod(ah, bh, &p2);
  p2 += (ah * bl + al * bh);
  *ch = quick_two_sum(p1, p2, cl);
}

MDG_HD void dd_sqr(double ah, double al, double *bh, double *bl) {
  double p1, p2;
  p1 = two_sqr(ah, &p2);
  p2 += 2.0 * ah * al;
  p2 += al * al;
  *bh = quick_two_sum(p1, p2, bl);
}

MDG_HD void dd_mul_d_dd(double a, double bh, double bl, double *ch,
                        double *cl) {
  double p1, p2;
  p1 = two_prod(a, bh, &p2);
  p2 += (bl * a);
  *ch = quick_two_sum(p1, p2, cl);
}

MDG_HD void dd_mlt_d(double *ah, double *al, double b) {
  double p1, p2;
  p1 = two_prod(*ah, b, &p2);
  p2 += *al * b;
  *ah = quick_two_sum(p1, p2, al);
}

/* Long division with three quotient digits. */
MDG_HD void dd_div(double ah, double al, double bh, double bl, double *ch,
                   double *cl) {
  double q1, q2, q3, xh, xl;
  q1 = ah / bh;
  dd_mul_d_dd(q1, bh, bl, &xh, &xl);
  dd_sub(ah, al, xh, xl, ch, cl);
  q2 = *ch / bh;
  dd_mul_d_dd(q2, bh, bl, &xh, &xl);
  dd_sub(*ch, *cl, xh, xl, ch, cl);
  q3 = *ch / bh;
  *ch = quick_two_sum(q1, q2, cl);
  dd_inc_d(ch, cl, q3);
}

/* Karp's square root: one Newton correction of 1/sqrt(a_hi). */
MDG_HD void dd_sqrt(double ah, double al, double *bh, double *bl) {
  if (ah == 0.0 && al == 0.0) {
    *bh = 0.0;
    *bl = 0.0;
  } else if (ah < 0.0) {
    *bh = -1.0;
    *bl = 0.0;
  } else {
    const double x = 1.0 / sqrt(ah);
    double ax = ah * x;
    double sh, sl, yh, yl;
    dd_sqr(ax, 0.0, &sh, &sl);
    dd_sub(ah, al, sh, sl, &yh, &yl);
    *bh = two_sum(ax, yh * x * 0.5, bl);
  }
}

/* ------------------------------------------- P-double, P in {4,8,16} -- */

/* Renormalise P+1 overlapping terms f[0..P] (decreasing magnitude, as left
 * by the quick-two-sum sweeps below) into P limbs r[0..P-1]; the trailing
 * limbs that receive nothing are zero.  This is the Hida-Li-Bailey
 * renormalisation in the form the reference spells out for P = 4, 8, 16
 * (quad_double_functions.cu:14-152).  The output slot is chosen by a
 * running index; every write is predicated over all slots so that the
 * limbs stay in registers on the device. */
template <int P>
MDG_HD double renorm(const double *f, double *r) {
  double pr;
  int ptr;
  MDG_UNROLL
  for (int j = 0; j < P; ++j) r[j] = 0.0;
  if (f[1] == 0.0) {
    pr = f[0];
    ptr = 0;
  } else {
    r[0] = f[0];
    pr = f[1];
    ptr = 1;
  }
  MDG_UNROLL
  for (int i = 2; i <= P; ++i) {
    double e;
    double s = quick_two_sum(pr, f[i], &e);
    MDG_UNROLL
    for (int j = 0; j < i; ++j)
      if (j == ptr) r[j] = s;
    if (e == 0.0) {
      pr = s;
    } else {
      pr = e;
      ++ptr;
    }
  }
  if (ptr < P && pr != 0.0) {
    MDG_UNROLL
    for (int j = 0; j < P; ++j)
      if (j == ptr) r[j] = pr;
    ++ptr;
  }
  MDG_UNROLL
  for (int j = 1; j < P; ++j)
    if (j >= ptr) r[j] = 0.0;
  if (ptr < 1) r[0] = 0.0;
  return pr;
}

/* Quick-two-sum sweep from the bottom, then renormalise. */
template <int P>
MDG_HD void fast_renorm(const double *x, double *r) {
  double f[P + 1];
  double pr = quick_two_sum(x[P - 1], x[P], &f[P]);
  MDG_UNROLL
  for (int i = P - 2; i >= 1; --i) pr = quick_two_sum(x[i], pr, &f[i + 1]);
  f[0] = quick_two_sum(x[0], pr, &f[1]);
  renorm<P>(f, r);
}

/* r = x + y for a P-double x and a double y (two-sum sweep, renormalise). */
template <int P>
MDG_HD void renorm_add1(const double *x, double y, double *r) {
  double f[P + 1];
  double pr = two_sum(x[P - 1], y, &f[P]);
  MDG_UNROLL
  for (int i = P - 2; i >= 1; --i) pr = two_sum(x[i], pr, &f[i + 1]);
  f[0] = two_sum(x[0], pr, &f[1]);
  renorm<P>(f, r);
}

/* c = a + b: CAMPARY baileyAdd_fast<P,P,P>.  Limbs are added from the
 * bottom; each error term ripples down through the lower partial sums and
 * lands in the guard term f[P]. */
template <int P>
MDG_HD void add(const double *a, const double *b, double *c) {
  double f[P + 1], e;
  f[P] = 0.0;
  MDG_UNROLL
  for (int i = P - 1; i >= 0; --i) {
    f[i] = two_sum(a[i], b[i], &e);
    MDG_UNROLL
    for (int t = i + 1; t < P; ++t) f[t] = two_sum(f[t], e, &e);
    f[P] += e;
  }
  fast_renorm<P>(f, c);
}

/* c = a * b: CAMPARY baileyMul_fast<P,P,P>.  Diagonal P is summed with
 * plain products; diagonals P-1..0 use exact two-products whose errors
 * ripple down to the guard term. */
template <int P>
MDG_HD void mul(const double *a, const double *b, double *c) {
  double f[P + 1], p, e;
  f[P] = a[1] * b[P - 1];
  MDG_UNROLL
  for (int i = 2; i < P; ++i) f[P] += a[i] * b[P - i];
  MDG_UNROLL
  for (int d = P - 1; d >= 0; --d) {
    f[d] = two_prod(a[0], b[d], &e);
    MDG_UNROLL
    for (int t = d + 1; t < P; ++t) f[t] = two_sum(f[t], e, &e);
    f[P] += e;
    MDG_UNROLL
    for (int i = 1; i <= d; ++i) {
      p = two_prod(a[i], b[d - i], &e);
      MDG_UNROLL
      for (int t = d + 1; t < P; ++t) f[t] = two_sum(f[t], e, &e);
      f[P] += e;
      f[d] = two_sum(f[d], p, &e);
      MDG_UNROLL
      for (int t = d + 1; t < P; ++t) f[t] = two_sum(f[t], e, &e);
      f[P] += e;
    }
  }
  fast_renorm<P>(f, c);
}

/* c = a * a with the same operation order as mul(a, a). */
template <int P>
MDG_HD void sqr(const double *a, double *c) { mul<P>(a, a, c); }

/* c = a * b for a P-double a and a double b: baileyMul_fast<P,1,P>. */
template <int P>
MDG_HD void mul_d(const double *a, double b, double *c) {
  double f[P + 1], e;
  f[P] = 0.0;
  MDG_UNROLL
  for (int i = P - 1; i >= 0; --i) {
    f[i] = two_prod(a[i], b, &e);
    MDG_UNROLL
    for (int t = i + 1; t < P; ++t) f[t] = two_sum(f[t], e, &e);
    f[P] += e;
  }
  fast_renorm<P>(f, c);
}

template <int P>
MDG_HD void mul_pwr2(const double *a, double b, double *c) {
  MDG_UNROLL
  for (int i = 0; i < P; ++i) c[i] = a[i] * b;
}

/* c = a - b, evaluated as (-b) + a like the reference. */
template <int P>
MDG_HD void sub(const double *a, const double *b, double *c) {
  double nb[P];
  MDG_UNROLL
  for (int i = 0; i < P; ++i) nb[i] = -b[i];
  add<P>(nb, a, c);
}

/* Long division with P+1 quotient digits. */
template <int P>
MDG_HD void div(const double *a, const double *b, double *c) {
  double q[P + 1], acc[P], rem[P];
  MDG_UNROLL
  for (int i = 0; i < P; ++i) rem[i] = a[i];
  MDG_UNROLL
  for (int i = 0; i < P; ++i) {
    q[i] = rem[0] / b[0];
    mul_d<P>(b, q[i], acc);
    double t[P];
    sub<P>(rem, acc, t);
    MDG_UNROLL
    for (int j = 0; j < P; ++j) rem[j] = t[j];
  }
  q[P] = rem[0] / b[0];
  fast_renorm<P>(q, c);
}

template <int P> struct half_sqrt;

/* Square root by one Newton step on the square root of the leading half:
 * b = (b0^2 + a) / (2 b0). */
template <int P>
MDG_HD void sqrt_md(const double *a, double *b) {
  double h[P], z[P], t[P];
  MDG_UNROLL
  for (int i = 0; i < P; ++i) h[i] = 0.0;
  half_sqrt<P>::run(a, h);
  sqr<P>(h, z);
  add<P>(z, a, t);
  div<P>(t, h, z);
  mul_pwr2<P>(z, 0.5, b);
}

template <> struct half_sqrt<4> {
  MDG_HD static void run(const double *a, double *h) {
    dd_sqrt(a[0], a[1], &h[0], &h[1]);
  }
};
template <> struct half_sqrt<8> {
  MDG_HD static void run(const double *a, double *h) { sqrt_md<4>(a, h); }
};
template <> struct half_sqrt<16> {
  MDG_HD static void run(const double *a, double *h) { sqrt_md<8>(a, h); }
};

/* -------------------------------------- generic entry used by kernels -- */

/* acc = acc + a*b with the reference's plain-GEMM step: a product followed
 * by an addition into the running sum (TCcuda.cu:119-246). */
template <int P>
MDG_HD void madd(double *acc, const double *a, const double *b) {
  double t[P], s[P];
  mul<P>(a, b, t);
  add<P>(acc, t, s);
  MDG_UNROLL
  for (int i = 0; i < P; ++i) acc[i] = s[i];
}

template <>
MDG_HD void madd<2>(double *acc, const double *a, const double *b) {
  double th, tl;
  dd_mul(a[0], a[1], b[0], b[1], &th, &tl);
  dd_add(acc[0], acc[1], th, tl, &acc[0], &acc[1]);
}

/* y = y + x for a double x: the squeeze step (the *_inc_d functions). */
template <int P>
MDG_HD void inc_d(double *y, double x) {
  double r[P];
  renorm_add1<P>(y, x, r);
  MDG_UNROLL
  for (int i = 0; i < P; ++i) y[i] = r[i];
}

template <>
MDG_HD void inc_d<2>(double *y, double x) { dd_inc_d(&y[0], &y[1], x); }

}  // namespace mdg

#endif /* MDG_ARITH_H */

/* Generated by gen_dropin_headers.py: quad-double functions with the
 * signatures of the reference header quad_double_functions.h; every body
 * forwards to the limb-count templates of mdg_arith.h. */
#ifndef MDG_DROPIN_QUAD_DOUBLE_FUNCTIONS_H
#define MDG_DROPIN_QUAD_DOUBLE_FUNCTIONS_H

#include "mdg_arith.h"
#include "double_double_functions.h"
#include <stdio.h>

MDG_HD void qdf_renorm4(double f0, double f1, double f2, double f3, double f4, double *pr, double *r0, double *r1, double *r2, double *r3) {
  const double f[5] = {f0, f1, f2, f3, f4}; double r[4];
  *pr = mdg::renorm<4>(f, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3];
}
MDG_HD void qdf_fast_renorm(double x0, double x1, double x2, double x3, double x4, double *r0, double *r1, double *r2, double *r3) {
  const double x[5] = {x0, x1, x2, x3, x4}; double r[4];
  mdg::fast_renorm<4>(x, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3];
}
MDG_HD void qdf_renorm_add1(double x0, double x1, double x2, double x3, double y, double *r0, double *r1, double *r2, double *r3) {
  const double x[4] = {x0, x1, x2, x3}; double r[4];
  mdg::renorm_add1<4>(x, y, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3];
}
MDG_HD void qdf_copy(double a0, double a1, double a2, double a3, double *b0, double *b1, double *b2, double *b3) {
  *b0 = a0; *b1 = a1; *b2 = a2; *b3 = a3;
}
MDG_HD void qdf_abs(double a0, double a1, double a2, double a3, double *b0, double *b1, double *b2, double *b3) {
  if (a0 < 0.0) { *b0 = -a0; *b1 = -a1; *b2 = -a2; *b3 = -a3; }
  else { *b0 = a0; *b1 = a1; *b2 = a2; *b3 = a3; }
}
MDG_HD void qdf_add(double a0, double a1, double a2, double a3, double b0, double b1, double b2, double b3, double *c0, double *c1, double *c2, double *c3) {
  const double a[4] = {a0, a1, a2, a3}, b[4] = {b0, b1, b2, b3}; double c[4];
  mdg::add<4>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3];
}
MDG_HD void qdf_inc(double *a0, double *a1, double *a2, double *a3, double b0, double b1, double b2, double b3) {
  const double a[4] = {*a0, *a1, *a2, *a3}, b[4] = {b0, b1, b2, b3}; double c[4];
  mdg::add<4>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3];
}
MDG_HD void qdf_inc_d(double *a0, double *a1, double *a2, double *a3, double b) {
  const double a[4] = {*a0, *a1, *a2, *a3}; double c[4];
  mdg::renorm_add1<4>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3];
}
MDG_HD void qdf_dec(double *a0, double *a1, double *a2, double *a3, double b0, double b1, double b2, double b3) {
  const double a[4] = {*a0, *a1, *a2, *a3}, b[4] = {-b0, -b1, -b2, -b3}; double c[4];
  mdg::add<4>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3];
}
MDG_HD void qdf_minus(double *a0, double *a1, double *a2, double *a3) {
  *a0 = -(*a0); *a1 = -(*a1); *a2 = -(*a2); *a3 = -(*a3);
}
MDG_HD void qdf_sub(double a0, double a1, double a2, double a3, double b0, double b1, double b2, double b3, double *c0, double *c1, double *c2, double *c3) {
  const double a[4] = {a0, a1, a2, a3}, b[4] = {b0, b1, b2, b3}; double c[4];
  mdg::sub<4>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3];
}
MDG_HD void qdf_mul_pwr2(double a0, double a1, double a2, double a3, double b, double *c0, double *c1, double *c2, double *c3) {
  *c0 = a0 * b; *c1 = a1 * b; *c2 = a2 * b; *c3 = a3 * b;
}
MDG_HD void qdf_mul(double a0, double a1, double a2, double a3, double b0, double b1, double b2, double b3, double *c0, double *c1, double *c2, double *c3) {
  const double a[4] = {a0, a1, a2, a3}, b[4] = {b0, b1, b2, b3}; double c[4];
  mdg::mul<4>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3];
}
MDG_HD void qdf_sqr(double a0, double a1, double a2, double a3, double *c0, double *c1, double *c2, double *c3) {
  const double a[4] = {a0, a1, a2, a3}; double c[4];
  mdg::sqr<4>(a, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3];
}
MDG_HD void qdf_mul_qd_d(double a0, double a1, double a2, double a3, double b, double *c0, double *c1, double *c2, double *c3) {
  const double a[4] = {a0, a1, a2, a3}; double c[4];
  mdg::mul_d<4>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3];
}
MDG_HD void qdf_mlt_d(double *a0, double *a1, double *a2, double *a3, double b) {
  const double a[4] = {*a0, *a1, *a2, *a3}; double c[4];
  mdg::mul_d<4>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3];
}
MDG_HD void qdf_div(double a0, double a1, double a2, double a3, double b0, double b1, double b2, double b3, double *c0, double *c1, double *c2, double *c3) {
  const double a[4] = {a0, a1, a2, a3}, b[4] = {b0, b1, b2, b3}; double c[4];
  mdg::div<4>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3];
}
MDG_HD void qdf_sqrt(double a0, double a1, double a2, double a3, double *b0, double *b1, double *b2, double *b3) {
  const double a[4] = {a0, a1, a2, a3}; double c[4];
  mdg::sqrt_md<4>(a, c); *b0 = c[0]; *b1 = c[1]; *b2 = c[2]; *b3 = c[3];
}
static inline void qdf_write_doubles(double a0, double a1, double a2, double a3) {
  const double a[4] = {a0, a1, a2, a3};
  for (int i = 0; i < 4; ++i) printf("  limb %2d : %.16e\n", i, a[i]);
}

#endif /* MDG_DROPIN_QUAD_DOUBLE_FUNCTIONS_H */

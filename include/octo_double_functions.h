/* Generated by gen_dropin_headers.py: octo-double functions with the
 * signatures of the reference header octo_double_functions.h; every body
 * forwards to the limb-count templates of mdg_arith.h. */
#ifndef MDG_DROPIN_OCTO_DOUBLE_FUNCTIONS_H
#define MDG_DROPIN_OCTO_DOUBLE_FUNCTIONS_H

#include "mdg_arith.h"
#include "double_double_functions.h"
#include "quad_double_functions.h"
#include <stdio.h>

MDG_HD void odf_renorm8(double f0, double f1, double f2, double f3, double f4, double f5, double f6, double f7, double f8, double *pr, double *r0, double *r1, double *r2, double *r3, double *r4, double *r5, double *r6, double *r7) {
  const double f[9] = {f0, f1, f2, f3, f4, f5, f6, f7, f8}; double r[8];
  *pr = mdg::renorm<8>(f, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3]; *r4 = r[4]; *r5 = r[5]; *r6 = r[6]; *r7 = r[7];
}
MDG_HD void odf_fast_renorm(double x0, double x1, double x2, double x3, double x4, double x5, double x6, double x7, double x8, double *r0, double *r1, double *r2, double *r3, double *r4, double *r5, double *r6, double *r7) {
  const double x[9] = {x0, x1, x2, x3, x4, x5, x6, x7, x8}; double r[8];
  mdg::fast_renorm<8>(x, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3]; *r4 = r[4]; *r5 = r[5]; *r6 = r[6]; *r7 = r[7];
}
MDG_HD void odf_renorm_add1(double x0, double x1, double x2, double x3, double x4, double x5, double x6, double x7, double y, double *r0, double *r1, double *r2, double *r3, double *r4, double *r5, double *r6, double *r7) {
  const double x[8] = {x0, x1, x2, x3, x4, x5, x6, x7}; double r[8];
  mdg::renorm_add1<8>(x, y, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3]; *r4 = r[4]; *r5 = r[5]; *r6 = r[6]; *r7 = r[7];
}
MDG_HD void odf_copy(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double *b0, double *b1, double *b2, double *b3, double *b4, double *b5, double *b6, double *b7) {
  *b0 = a0; *b1 = a1; *b2 = a2; *b3 = a3; *b4 = a4; *b5 = a5; *b6 = a6; *b7 = a7;
}
MDG_HD void odf_abs(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double *b0, double *b1, double *b2, double *b3, double *b4, double *b5, double *b6, double *b7) {
  if (a0 < 0.0) { *b0 = -a0; *b1 = -a1; *b2 = -a2; *b3 = -a3; *b4 = -a4; *b5 = -a5; *b6 = -a6; *b7 = -a7; }
  else { *b0 = a0; *b1 = a1; *b2 = a2; *b3 = a3; *b4 = a4; *b5 = a5; *b6 = a6; *b7 = a7; }
}
MDG_HD void odf_add(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}, b[8] = {b0, b1, b2, b3, b4, b5, b6, b7}; double c[8];
  mdg::add<8>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7];
}
MDG_HD void odf_inc(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7) {
  const double a[8] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7}, b[8] = {b0, b1, b2, b3, b4, b5, b6, b7}; double c[8];
  mdg::add<8>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7];
}
MDG_HD void odf_inc_d(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double b) {
  const double a[8] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7}; double c[8];
  mdg::renorm_add1<8>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7];
}
MDG_HD void odf_dec(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7) {
  const double a[8] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7}, b[8] = {-b0, -b1, -b2, -b3, -b4, -b5, -b6, -b7}; double c[8];
  mdg::add<8>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7];
}
MDG_HD void odf_minus(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7) {
  *a0 = -(*a0); *a1 = -(*a1); *a2 = -(*a2); *a3 = -(*a3); *a4 = -(*a4); *a5 = -(*a5); *a6 = -(*a6); *a7 = -(*a7);
}
MDG_HD void odf_sub(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}, b[8] = {b0, b1, b2, b3, b4, b5, b6, b7}; double c[8];
  mdg::sub<8>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7];
}
MDG_HD void odf_mul_pwr2(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double b, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  *c0 = a0 * b; *c1 = a1 * b; *c2 = a2 * b; *c3 = a3 * b; *c4 = a4 * b; *c5 = a5 * b; *c6 = a6 * b; *c7 = a7 * b;
}
MDG_HD void odf_mul(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}, b[8] = {b0, b1, b2, b3, b4, b5, b6, b7}; double c[8];
  mdg::mul<8>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7];
}
MDG_HD void odf_sqr(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}; double c[8];
  mdg::sqr<8>(a, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7];
}
MDG_HD void odf_mul_od_d(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double b, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}; double c[8];
  mdg::mul_d<8>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7];
}
MDG_HD void odf_mlt_d(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double b) {
  const double a[8] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7}; double c[8];
  mdg::mul_d<8>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7];
}
MDG_HD void odf_div(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}, b[8] = {b0, b1, b2, b3, b4, b5, b6, b7}; double c[8];
  mdg::div<8>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7];
}
MDG_HD void odf_sqrt(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double *b0, double *b1, double *b2, double *b3, double *b4, double *b5, double *b6, double *b7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7}; double c[8];
  mdg::sqrt_md<8>(a, c); *b0 = c[0]; *b1 = c[1]; *b2 = c[2]; *b3 = c[3]; *b4 = c[4]; *b5 = c[5]; *b6 = c[6]; *b7 = c[7];
}
static inline void odf_write_doubles(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7) {
  const double a[8] = {a0, a1, a2, a3, a4, a5, a6, a7};
  for (int i = 0; i < 8; ++i) printf("  limb %2d : %.16e\n", i, a[i]);
}

#endif /* MDG_DROPIN_OCTO_DOUBLE_FUNCTIONS_H */

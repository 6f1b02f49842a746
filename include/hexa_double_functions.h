/* Generated by gen_dropin_headers.py: hexa-double functions with the
 * signatures of the reference header hexa_double_functions.h; every body
 * forwards to the limb-count templates of mdg_arith.h. */
#ifndef MDG_DROPIN_HEXA_DOUBLE_FUNCTIONS_H
#define MDG_DROPIN_HEXA_DOUBLE_FUNCTIONS_H

#include "mdg_arith.h"
#include "double_double_functions.h"
#include "quad_double_functions.h"
#include "octo_double_functions.h"
#include <stdio.h>

MDG_HD void hdf_renorm16(double f0, double f1, double f2, double f3, double f4, double f5, double f6, double f7, double f8, double f9, double f10, double f11, double f12, double f13, double f14, double f15, double f16, double *pr, double *r0, double *r1, double *r2, double *r3, double *r4, double *r5, double *r6, double *r7, double *r8, double *r9, double *r10, double *r11, double *r12, double *r13, double *r14, double *r15) {
  const double f[17] = {f0, f1, f2, f3, f4, f5, f6, f7, f8, f9, f10, f11, f12, f13, f14, f15, f16}; double r[16];
  *pr = mdg::renorm<16>(f, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3]; *r4 = r[4]; *r5 = r[5]; *r6 = r[6]; *r7 = r[7]; *r8 = r[8]; *r9 = r[9]; *r10 = r[10]; *r11 = r[11]; *r12 = r[12]; *r13 = r[13]; *r14 = r[14]; *r15 = r[15];
}
MDG_HD void hdf_fast_renorm(double x0, double x1, double x2, double x3, double x4, double x5, double x6, double x7, double x8, double x9, double x10, double x11, double x12, double x13, double x14, double x15, double x16, double *r0, double *r1, double *r2, double *r3, double *r4, double *r5, double *r6, double *r7, double *r8, double *r9, double *r10, double *r11, double *r12, double *r13, double *r14, double *r15) {
  const double x[17] = {x0, x1, x2, x3, x4, x5, x6, x7, x8, x9, x10, x11, x12, x13, x14, x15, x16}; double r[16];
  mdg::fast_renorm<16>(x, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3]; *r4 = r[4]; *r5 = r[5]; *r6 = r[6]; *r7 = r[7]; *r8 = r[8]; *r9 = r[9]; *r10 = r[10]; *r11 = r[11]; *r12 = r[12]; *r13 = r[13]; *r14 = r[14]; *r15 = r[15];
}
MDG_HD void hdf_renorm_add1(double x0, double x1, double x2, double x3, double x4, double x5, double x6, double x7, double x8, double x9, double x10, double x11, double x12, double x13, double x14, double x15, double y, double *r0, double *r1, double *r2, double *r3, double *r4, double *r5, double *r6, double *r7, double *r8, double *r9, double *r10, double *r11, double *r12, double *r13, double *r14, double *r15) {
  const double x[16] = {x0, x1, x2, x3, x4, x5, x6, x7, x8, x9, x10, x11, x12, x13, x14, x15}; double r[16];
  mdg::renorm_add1<16>(x, y, r); *r0 = r[0]; *r1 = r[1]; *r2 = r[2]; *r3 = r[3]; *r4 = r[4]; *r5 = r[5]; *r6 = r[6]; *r7 = r[7]; *r8 = r[8]; *r9 = r[9]; *r10 = r[10]; *r11 = r[11]; *r12 = r[12]; *r13 = r[13]; *r14 = r[14]; *r15 = r[15];
}
MDG_HD void hdf_copy(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double *b0, double *b1, double *b2, double *b3, double *b4, double *b5, double *b6, double *b7, double *b8, double *b9, double *b10, double *b11, double *b12, double *b13, double *b14, double *b15) {
  *b0 = a0; *b1 = a1; *b2 = a2; *b3 = a3; *b4 = a4; *b5 = a5; *b6 = a6; *b7 = a7; *b8 = a8; *b9 = a9; *b10 = a10; *b11 = a11; *b12 = a12; *b13 = a13; *b14 = a14; *b15 = a15;
}
MDG_HD void hdf_abs(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double *b0, double *b1, double *b2, double *b3, double *b4, double *b5, double *b6, double *b7, double *b8, double *b9, double *b10, double *b11, double *b12, double *b13, double *b14, double *b15) {
  if (a0 < 0.0) { *b0 = -a0; *b1 = -a1; *b2 = -a2; *b3 = -a3; *b4 = -a4; *b5 = -a5; *b6 = -a6; *b7 = -a7; *b8 = -a8; *b9 = -a9; *b10 = -a10; *b11 = -a11; *b12 = -a12; *b13 = -a13; *b14 = -a14; *b15 = -a15; }
  else { *b0 = a0; *b1 = a1; *b2 = a2; *b3 = a3; *b4 = a4; *b5 = a5; *b6 = a6; *b7 = a7; *b8 = a8; *b9 = a9; *b10 = a10; *b11 = a11; *b12 = a12; *b13 = a13; *b14 = a14; *b15 = a15; }
}
MDG_HD void hdf_add(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double b8, double b9, double b10, double b11, double b12, double b13, double b14, double b15, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}, b[16] = {b0, b1, b2, b3, b4, b5, b6, b7, b8, b9, b10, b11, b12, b13, b14, b15}; double c[16];
  mdg::add<16>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7]; *c8 = c[8]; *c9 = c[9]; *c10 = c[10]; *c11 = c[11]; *c12 = c[12]; *c13 = c[13]; *c14 = c[14]; *c15 = c[15];
}
MDG_HD void hdf_inc(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double *a8, double *a9, double *a10, double *a11, double *a12, double *a13, double *a14, double *a15, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double b8, double b9, double b10, double b11, double b12, double b13, double b14, double b15) {
  const double a[16] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7, *a8, *a9, *a10, *a11, *a12, *a13, *a14, *a15}, b[16] = {b0, b1, b2, b3, b4, b5, b6, b7, b8, b9, b10, b11, b12, b13, b14, b15}; double c[16];
  mdg::add<16>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7]; *a8 = c[8]; *a9 = c[9]; *a10 = c[10]; *a11 = c[11]; *a12 = c[12]; *a13 = c[13]; *a14 = c[14]; *a15 = c[15];
}
MDG_HD void hdf_inc_d(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double *a8, double *a9, double *a10, double *a11, double *a12, double *a13, double *a14, double *a15, double b) {
  const double a[16] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7, *a8, *a9, *a10, *a11, *a12, *a13, *a14, *a15}; double c[16];
  mdg::renorm_add1<16>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7]; *a8 = c[8]; *a9 = c[9]; *a10 = c[10]; *a11 = c[11]; *a12 = c[12]; *a13 = c[13]; *a14 = c[14]; *a15 = c[15];
}
MDG_HD void hdf_dec(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double *a8, double *a9, double *a10, double *a11, double *a12, double *a13, double *a14, double *a15, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double b8, double b9, double b10, double b11, double b12, double b13, double b14, double b15) {
  const double a[16] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7, *a8, *a9, *a10, *a11, *a12, *a13, *a14, *a15}, b[16] = {-b0, -b1, -b2, -b3, -b4, -b5, -b6, -b7, -b8, -b9, -b10, -b11, -b12, -b13, -b14, -b15}; double c[16];
  mdg::add<16>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7]; *a8 = c[8]; *a9 = c[9]; *a10 = c[10]; *a11 = c[11]; *a12 = c[12]; *a13 = c[13]; *a14 = c[14]; *a15 = c[15];
}
MDG_HD void hdf_minus(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double *a8, double *a9, double *a10, double *a11, double *a12, double *a13, double *a14, double *a15) {
  *a0 = -(*a0); *a1 = -(*a1); *a2 = -(*a2); *a3 = -(*a3); *a4 = -(*a4); *a5 = -(*a5); *a6 = -(*a6); *a7 = -(*a7); *a8 = -(*a8); *a9 = -(*a9); *a10 = -(*a10); *a11 = -(*a11); *a12 = -(*a12); *a13 = -(*a13); *a14 = -(*a14); *a15 = -(*a15);
}
MDG_HD void hdf_sub(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double b8, double b9, double b10, double b11, double b12, double b13, double b14, double b15, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}, b[16] = {b0, b1, b2, b3, b4, b5, b6, b7, b8, b9, b10, b11, b12, b13, b14, b15}; double c[16];
  mdg::sub<16>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7]; *c8 = c[8]; *c9 = c[9]; *c10 = c[10]; *c11 = c[11]; *c12 = c[12]; *c13 = c[13]; *c14 = c[14]; *c15 = c[15];
}
MDG_HD void hdf_mul_pwr2(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double b, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  *c0 = a0 * b; *c1 = a1 * b; *c2 = a2 * b; *c3 = a3 * b; *c4 = a4 * b; *c5 = a5 * b; *c6 = a6 * b; *c7 = a7 * b; *c8 = a8 * b; *c9 = a9 * b; *c10 = a10 * b; *c11 = a11 * b; *c12 = a12 * b; *c13 = a13 * b; *c14 = a14 * b; *c15 = a15 * b;
}
MDG_HD void hdf_mul(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double b8, double b9, double b10, double b11, double b12, double b13, double b14, double b15, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}, b[16] = {b0, b1, b2, b3, b4, b5, b6, b7, b8, b9, b10, b11, b12, b13, b14, b15}; double c[16];
  mdg::mul<16>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7]; *c8 = c[8]; *c9 = c[9]; *c10 = c[10]; *c11 = c[11]; *c12 = c[12]; *c13 = c[13]; *c14 = c[14]; *c15 = c[15];
}
MDG_HD void hdf_sqr(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}; double c[16];
  mdg::sqr<16>(a, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7]; *c8 = c[8]; *c9 = c[9]; *c10 = c[10]; *c11 = c[11]; *c12 = c[12]; *c13 = c[13]; *c14 = c[14]; *c15 = c[15];
}
MDG_HD void hdf_mul_hd_d(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double b, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}; double c[16];
  mdg::mul_d<16>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7]; *c8 = c[8]; *c9 = c[9]; *c10 = c[10]; *c11 = c[11]; *c12 = c[12]; *c13 = c[13]; *c14 = c[14]; *c15 = c[15];
}
MDG_HD void hdf_mlt_d(double *a0, double *a1, double *a2, double *a3, double *a4, double *a5, double *a6, double *a7, double *a8, double *a9, double *a10, double *a11, double *a12, double *a13, double *a14, double *a15, double b) {
  const double a[16] = {*a0, *a1, *a2, *a3, *a4, *a5, *a6, *a7, *a8, *a9, *a10, *a11, *a12, *a13, *a14, *a15}; double c[16];
  mdg::mul_d<16>(a, b, c); *a0 = c[0]; *a1 = c[1]; *a2 = c[2]; *a3 = c[3]; *a4 = c[4]; *a5 = c[5]; *a6 = c[6]; *a7 = c[7]; *a8 = c[8]; *a9 = c[9]; *a10 = c[10]; *a11 = c[11]; *a12 = c[12]; *a13 = c[13]; *a14 = c[14]; *a15 = c[15];
}
MDG_HD void hdf_div(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double b0, double b1, double b2, double b3, double b4, double b5, double b6, double b7, double b8, double b9, double b10, double b11, double b12, double b13, double b14, double b15, double *c0, double *c1, double *c2, double *c3, double *c4, double *c5, double *c6, double *c7, double *c8, double *c9, double *c10, double *c11, double *c12, double *c13, double *c14, double *c15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}, b[16] = {b0, b1, b2, b3, b4, b5, b6, b7, b8, b9, b10, b11, b12, b13, b14, b15}; double c[16];
  mdg::div<16>(a, b, c); *c0 = c[0]; *c1 = c[1]; *c2 = c[2]; *c3 = c[3]; *c4 = c[4]; *c5 = c[5]; *c6 = c[6]; *c7 = c[7]; *c8 = c[8]; *c9 = c[9]; *c10 = c[10]; *c11 = c[11]; *c12 = c[12]; *c13 = c[13]; *c14 = c[14]; *c15 = c[15];
}
MDG_HD void hdf_sqrt(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15, double *b0, double *b1, double *b2, double *b3, double *b4, double *b5, double *b6, double *b7, double *b8, double *b9, double *b10, double *b11, double *b12, double *b13, double *b14, double *b15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15}; double c[16];
  mdg::sqrt_md<16>(a, c); *b0 = c[0]; *b1 = c[1]; *b2 = c[2]; *b3 = c[3]; *b4 = c[4]; *b5 = c[5]; *b6 = c[6]; *b7 = c[7]; *b8 = c[8]; *b9 = c[9]; *b10 = c[10]; *b11 = c[11]; *b12 = c[12]; *b13 = c[13]; *b14 = c[14]; *b15 = c[15];
}
static inline void hdf_write_doubles(double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8, double a9, double a10, double a11, double a12, double a13, double a14, double a15) {
  const double a[16] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15};
  for (int i = 0; i < 16; ++i) printf("  limb %2d : %.16e\n", i, a[i]);
}

#endif /* MDG_DROPIN_HEXA_DOUBLE_FUNCTIONS_H */

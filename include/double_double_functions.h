/* Generated by gen_dropin_headers.py: double-double functions with the
 * signatures of the reference header double_double_functions.h; every body
 * forwards to mdg_arith.h.  One deliberate difference: ddf_mlt computes the
 * product a*b (the reference adds b_hi*a_hi where b_hi*a_lo belongs,
 * double_double_functions.cu:135). */
#ifndef MDG_DROPIN_DOUBLE_DOUBLE_FUNCTIONS_H
#define MDG_DROPIN_DOUBLE_DOUBLE_FUNCTIONS_H

#include "mdg_arith.h"
#include <stdio.h>

MDG_HD double ddf_quick_two_sum(double a, double b, double *err) { return mdg::quick_two_sum(a, b, err); }
MDG_HD double ddf_two_sum(double a, double b, double *err) { return mdg::two_sum(a, b, err); }
MDG_HD void ddf_add(double a_hi, double a_lo, double b_hi, double b_lo, double *c_hi, double *c_lo) { mdg::dd_add(a_hi, a_lo, b_hi, b_lo, c_hi, c_lo); }
MDG_HD double ddf_quick_two_diff(double a, double b, double *err) { return mdg::quick_two_diff(a, b, err); }
MDG_HD double ddf_two_diff(double a, double b, double *err) { return mdg::two_diff(a, b, err); }
MDG_HD void ddf_minus(double *a_hi, double *a_lo) { *a_hi = -(*a_hi); *a_lo = -(*a_lo); }
MDG_HD void ddf_sub(double a_hi, double a_lo, double b_hi, double b_lo, double *c_hi, double *c_lo) { mdg::dd_sub(a_hi, a_lo, b_hi, b_lo, c_hi, c_lo); }
MDG_HD void ddf_sub_dd_d(double a_hi, double a_lo, double b, double *c_hi, double *c_lo) { mdg::dd_sub_dd_d(a_hi, a_lo, b, c_hi, c_lo); }
MDG_HD void ddf_inc(double *a_hi, double *a_lo, double b_hi, double b_lo) { mdg::dd_add(*a_hi, *a_lo, b_hi, b_lo, a_hi, a_lo); }
MDG_HD void ddf_inc_d(double *a_hi, double *a_lo, double b) { mdg::dd_inc_d(a_hi, a_lo, b); }
MDG_HD void ddf_dec(double *a_hi, double *a_lo, double b_hi, double b_lo) { mdg::dd_sub(*a_hi, *a_lo, b_hi, b_lo, a_hi, a_lo); }
MDG_HD void ddf_dec_d(double *a_hi, double *a_lo, double b) { mdg::dd_dec_d(a_hi, a_lo, b); }
MDG_HD void ddf_mlt(double *a_hi, double *a_lo, double b_hi, double b_lo) { mdg::dd_mul(*a_hi, *a_lo, b_hi, b_lo, a_hi, a_lo); }
MDG_HD void ddf_mlt_d(double *a_hi, double *a_lo, double b) { mdg::dd_mlt_d(a_hi, a_lo, b); }
MDG_HD void ddf_split(double a, double *hi, double *lo) { mdg::veltkamp_split(a, hi, lo); }
MDG_HD double ddf_two_prod(double a, double b, double *err) { return mdg::two_prod(a, b, err); }
MDG_HD double ddf_two_sqr(double a, double *err) { return mdg::two_sqr(a, err); }
MDG_HD void ddf_mul(double a_hi, double a_lo, double b_hi, double b_lo, double *c_hi, double *c_lo) { mdg::dd_mul(a_hi, a_lo, b_hi, b_lo, c_hi, c_lo); }
MDG_HD void ddf_sqr(double a_hi, double a_lo, double *b_hi, double *b_lo) { mdg::dd_sqr(a_hi, a_lo, b_hi, b_lo); }
MDG_HD void ddf_mul_d_dd(double a, double b_hi, double b_lo, double *c_hi, double *c_lo) { mdg::dd_mul_d_dd(a, b_hi, b_lo, c_hi, c_lo); }
MDG_HD void ddf_div(double a_hi, double a_lo, double b_hi, double b_lo, double *c_hi, double *c_lo) { mdg::dd_div(a_hi, a_lo, b_hi, b_lo, c_hi, c_lo); }
MDG_HD void ddf_sqrt(double a_hi, double a_lo, double *b_hi, double *b_lo) { mdg::dd_sqrt(a_hi, a_lo, b_hi, b_lo); }
MDG_HD void ddf_abs(double a_hi, double a_lo, double *b_hi, double *b_lo) {
  if (a_hi < 0.0) { *b_hi = -a_hi; *b_lo = -a_lo; } else { *b_hi = a_hi; *b_lo = a_lo; }
}
static inline void ddf_write_doubles(double a_hi, double a_lo) {
  printf("  hi : %.16e  lo : %.16e\n", a_hi, a_lo);
}

#endif /* MDG_DROPIN_DOUBLE_DOUBLE_FUNCTIONS_H */

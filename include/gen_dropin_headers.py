"""Writes the four drop-in arithmetic headers next to this script.

double_double_functions.h, quad_double_functions.h, octo_double_functions.h
and hexa_double_functions.h declare the same functions, with the same names,
argument order and argument meaning, as the reference headers of the same
names (C++/double_double_functions.h:17-341, quad_double_functions.h:19-398,
octo_double_functions.h:21-599, hexa_double_functions.h:26-526).  Each body
forwards to the templates in mdg_arith.h.  Limb arguments are spelled
<name>0 .. <name>{P-1}, most significant first.

Run:  python include/gen_dropin_headers.py
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))

PREFIX = {4: "qdf", 8: "odf", 16: "hdf"}
GUARD = {4: "quad", 8: "octo", 16: "hexa"}
DSUFFIX = {4: "qd", 8: "od", 16: "hd"}


def vals(name, P):
    return ", ".join(f"double {name}{i}" for i in range(P))


def ptrs(name, P):
    return ", ".join(f"double *{name}{i}" for i in range(P))


def arr(name, P, deref=False):
    star = "*" if deref else ""
    return "{" + ", ".join(f"{star}{name}{i}" for i in range(P)) + "}"


def store(dst, src, P):
    return " ".join(f"*{dst}{i} = {src}[{i}];" for i in range(P))


def gen_pd(P):
    f = PREFIX[P]
    ds = DSUFFIX[P]
    out = []
    w = out.append
    g = f"MDG_DROPIN_{GUARD[P].upper()}_DOUBLE_FUNCTIONS_H"
    w(f"/* Generated by gen_dropin_headers.py: {GUARD[P]}-double functions with the")
    w(f" * signatures of the reference header {GUARD[P]}_double_functions.h; every body")
    w(" * forwards to the limb-count templates of mdg_arith.h. */")
    w(f"#ifndef {g}\n#define {g}\n")
    w('#include "mdg_arith.h"')
    w('#include "double_double_functions.h"')
    if P >= 8:
        w('#include "quad_double_functions.h"')
    if P >= 16:
        w('#include "octo_double_functions.h"')
    w("#include <stdio.h>\n")
    fin = ", ".join(f"double f{i}" for i in range(P + 1))
    w(f"MDG_HD void {f}_renorm{P}({fin}, double *pr, {ptrs('r', P)}) {{")
    w(f"  const double f[{P + 1}] = {arr('f', P + 1)}; double r[{P}];")
    w(f"  *pr = mdg::renorm<{P}>(f, r); {store('r', 'r', P)}\n}}")
    xin = ", ".join(f"double x{i}" for i in range(P + 1))
    w(f"MDG_HD void {f}_fast_renorm({xin}, {ptrs('r', P)}) {{")
    w(f"  const double x[{P + 1}] = {arr('x', P + 1)}; double r[{P}];")
    w(f"  mdg::fast_renorm<{P}>(x, r); {store('r', 'r', P)}\n}}")
    w(f"MDG_HD void {f}_renorm_add1({vals('x', P)}, double y, {ptrs('r', P)}) {{")
    w(f"  const double x[{P}] = {arr('x', P)}; double r[{P}];")
    w(f"  mdg::renorm_add1<{P}>(x, y, r); {store('r', 'r', P)}\n}}")
    w(f"MDG_HD void {f}_copy({vals('a', P)}, {ptrs('b', P)}) {{")
    w("  " + " ".join(f"*b{i} = a{i};" for i in range(P)) + "\n}")
    w(f"MDG_HD void {f}_abs({vals('a', P)}, {ptrs('b', P)}) {{")
    w("  if (a0 < 0.0) { " + " ".join(f"*b{i} = -a{i};" for i in range(P)) + " }")
    w("  else { " + " ".join(f"*b{i} = a{i};" for i in range(P)) + " }\n}")
    binop = f"const double a[{P}] = {arr('a', P)}, b[{P}] = {arr('b', P)}; double c[{P}];"
    w(f"MDG_HD void {f}_add({vals('a', P)}, {vals('b', P)}, {ptrs('c', P)}) {{")
    w(f"  {binop}\n  mdg::add<{P}>(a, b, c); {store('c', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_inc({ptrs('a', P)}, {vals('b', P)}) {{")
    w(f"  const double a[{P}] = {arr('a', P, True)}, b[{P}] = {arr('b', P)}; double c[{P}];")
    w(f"  mdg::add<{P}>(a, b, c); {store('a', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_inc_d({ptrs('a', P)}, double b) {{")
    w(f"  const double a[{P}] = {arr('a', P, True)}; double c[{P}];")
    w(f"  mdg::renorm_add1<{P}>(a, b, c); {store('a', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_dec({ptrs('a', P)}, {vals('b', P)}) {{")
    w(f"  const double a[{P}] = {arr('a', P, True)}, b[{P}] = {{" +
      ", ".join(f"-b{i}" for i in range(P)) + f"}}; double c[{P}];")
    w(f"  mdg::add<{P}>(a, b, c); {store('a', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_minus({ptrs('a', P)}) {{")
    w("  " + " ".join(f"*a{i} = -(*a{i});" for i in range(P)) + "\n}")
    w(f"MDG_HD void {f}_sub({vals('a', P)}, {vals('b', P)}, {ptrs('c', P)}) {{")
    w(f"  {binop}\n  mdg::sub<{P}>(a, b, c); {store('c', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_mul_pwr2({vals('a', P)}, double b, {ptrs('c', P)}) {{")
    w("  " + " ".join(f"*c{i} = a{i} * b;" for i in range(P)) + "\n}")
    w(f"MDG_HD void {f}_mul({vals('a', P)}, {vals('b', P)}, {ptrs('c', P)}) {{")
    w(f"  {binop}\n  mdg::mul<{P}>(a, b, c); {store('c', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_sqr({vals('a', P)}, {ptrs('c', P)}) {{")
    w(f"  const double a[{P}] = {arr('a', P)}; double c[{P}];")
    w(f"  mdg::sqr<{P}>(a, c); {store('c', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_mul_{ds}_d({vals('a', P)}, double b, {ptrs('c', P)}) {{")
    w(f"  const double a[{P}] = {arr('a', P)}; double c[{P}];")
    w(f"  mdg::mul_d<{P}>(a, b, c); {store('c', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_mlt_d({ptrs('a', P)}, double b) {{")
    w(f"  const double a[{P}] = {arr('a', P, True)}; double c[{P}];")
    w(f"  mdg::mul_d<{P}>(a, b, c); {store('a', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_div({vals('a', P)}, {vals('b', P)}, {ptrs('c', P)}) {{")
    w(f"  {binop}\n  mdg::div<{P}>(a, b, c); {store('c', 'c', P)}\n}}")
    w(f"MDG_HD void {f}_sqrt({vals('a', P)}, {ptrs('b', P)}) {{")
    w(f"  const double a[{P}] = {arr('a', P)}; double c[{P}];")
    w(f"  mdg::sqrt_md<{P}>(a, c); {store('b', 'c', P)}\n}}")
    w(f"static inline void {f}_write_doubles({vals('a', P)}) {{")
    w(f"  const double a[{P}] = {arr('a', P)};")
    w(f"  for (int i = 0; i < {P}; ++i) printf(\"  limb %2d : %.16e\\n\", i, a[i]);\n}}")
    w(f"\n#endif /* {g} */")
    return "\n".join(out) + "\n"


DD = r'''/* Generated by gen_dropin_headers.py: double-double functions with the
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
'''


def main():
    with open(os.path.join(HERE, "double_double_functions.h"), "w") as fh:
        fh.write(DD)
    for P in (4, 8, 16):
        with open(os.path.join(HERE, f"{GUARD[P]}_double_functions.h"), "w") as fh:
            fh.write(gen_pd(P))


if __name__ == "__main__":
    main()

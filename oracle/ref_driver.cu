/*
 * ref_driver.cu -- C entry points around the reference's own host functions.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together
 * with the reference's C++/floatybits.cu and C++/TCcuda.cu (which includes
 * the four *_double_functions.cu files) into oracle/_ref/libref.so.  It is
 * used in the build container to produce the golden vectors in
 * tests/golden/ and to cross-check oracle.c; nothing on the GPU path loads
 * it.  The functions called here are the reference's, unmodified:
 *   ddf_/qdf_/odf_/hdf_ add, mul, sub, div, sqrt, inc_d, mul_*_d
 *                                        (*_double_functions.cu)
 *   matmulddf / matmulqdf / matmulodf / matmulhdf   (TCcuda.cu:320-372)
 *   split4pd / split8pd / mixsplit2                 (floatybits.cu:196,303,327)
 *   mat -> random_pd                                (TCcuda.cu:14, floatybits.cu:107)
 *   bigB2                                           (TCcuda.cu:79)
 */
#include "TCcuda.h"
#include <vector>
#include <cstdlib>
#include <cstring>

using std::vector;

#define LIMBS2(x) x[0], x[1]
#define LIMBS4(x) x[0], x[1], x[2], x[3]
#define LIMBS8(x) x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7]
#define LIMBS16(x) \
  x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8], x[9], x[10], x[11], x[12], x[13], x[14], x[15]
#define PTRS2(x) &x[0], &x[1]
#define PTRS4(x) &x[0], &x[1], &x[2], &x[3]
#define PTRS8(x) &x[0], &x[1], &x[2], &x[3], &x[4], &x[5], &x[6], &x[7]
#define PTRS16(x)                                                                            \
  &x[0], &x[1], &x[2], &x[3], &x[4], &x[5], &x[6], &x[7], &x[8], &x[9], &x[10], &x[11], &x[12], \
      &x[13], &x[14], &x[15]

extern "C" {

/* op: 0 add, 1 mul, 2 sub, 3 div, 4 sqrt (b unused), 5 inc_d (b[0]),
 * 6 mul by double (b[0]) */
int ref_binop(int op, int P, long n, const double *a, const double *b,
              double *c) {
  for (long i = 0; i < n; ++i) {
    const double *x = a + i * P, *y = b + i * P;
    double *z = c + i * P;
    if (op == 5) memcpy(z, x, sizeof(double) * P);
    if (P == 2) {
      switch (op) {
        case 0: ddf_add(LIMBS2(x), LIMBS2(y), PTRS2(z)); break;
        case 1: ddf_mul(LIMBS2(x), LIMBS2(y), PTRS2(z)); break;
        case 2: ddf_sub(LIMBS2(x), LIMBS2(y), PTRS2(z)); break;
        case 3: ddf_div(LIMBS2(x), LIMBS2(y), PTRS2(z)); break;
        case 4: ddf_sqrt(LIMBS2(x), PTRS2(z)); break;
        case 5: ddf_inc_d(PTRS2(z), y[0]); break;
        case 6: ddf_mul_d_dd(y[0], LIMBS2(x), PTRS2(z)); break;
        default: return -1;
      }
    } else if (P == 4) {
      switch (op) {
        case 0: qdf_add(LIMBS4(x), LIMBS4(y), PTRS4(z)); break;
        case 1: qdf_mul(LIMBS4(x), LIMBS4(y), PTRS4(z)); break;
        case 2: qdf_sub(LIMBS4(x), LIMBS4(y), PTRS4(z)); break;
        case 3: qdf_div(LIMBS4(x), LIMBS4(y), PTRS4(z)); break;
        case 4: qdf_sqrt(LIMBS4(x), PTRS4(z)); break;
        case 5: qdf_inc_d(PTRS4(z), y[0]); break;
        case 6: qdf_mul_qd_d(LIMBS4(x), y[0], PTRS4(z)); break;
        default: return -1;
      }
    } else if (P == 8) {
      switch (op) {
        case 0: odf_add(LIMBS8(x), LIMBS8(y), PTRS8(z)); break;
        case 1: odf_mul(LIMBS8(x), LIMBS8(y), PTRS8(z)); break;
        case 2: odf_sub(LIMBS8(x), LIMBS8(y), PTRS8(z)); break;
        case 3: odf_div(LIMBS8(x), LIMBS8(y), PTRS8(z)); break;
        case 4: odf_sqrt(LIMBS8(x), PTRS8(z)); break;
        case 5: odf_inc_d(PTRS8(z), y[0]); break;
        case 6: odf_mul_od_d(LIMBS8(x), y[0], PTRS8(z)); break;
        default: return -1;
      }
    } else if (P == 16) {
      switch (op) {
        case 0: hdf_add(LIMBS16(x), LIMBS16(y), PTRS16(z)); break;
        case 1: hdf_mul(LIMBS16(x), LIMBS16(y), PTRS16(z)); break;
        case 2: hdf_sub(LIMBS16(x), LIMBS16(y), PTRS16(z)); break;
        case 3: hdf_div(LIMBS16(x), LIMBS16(y), PTRS16(z)); break;
        case 4: hdf_sqrt(LIMBS16(x), PTRS16(z)); break;
        case 5: hdf_inc_d(PTRS16(z), y[0]); break;
        case 6: hdf_mul_hd_d(LIMBS16(x), y[0], PTRS16(z)); break;
        default: return -1;
      }
    } else {
      return -1;
    }
  }
  return 0;
}

/* square n x n plain GEMM on the host, C = A*B */
int ref_matmul(int P, int n, const double *A, const double *B, double *C) {
  vector<double> a(A, A + (size_t)n * n * P), b(B, B + (size_t)n * n * P), c;
  switch (P) {
    case 2: c = matmulddf(a, b, n); break;
    case 4: c = matmulqdf(a, b, n); break;
    case 8: c = matmulodf(a, b, n); break;
    case 16: c = matmulhdf(a, b, n); break;
    default: return -1;
  }
  memcpy(C, c.data(), sizeof(double) * c.size());
  return 0;
}

/* kind 0 split4pd, 1 split8pd, 2 mixsplit2; x holds n P-doubles */
int ref_split(int kind, int P, long n, const double *x, double *out) {
  vector<double> v(x, x + n * P), o;
  if (kind == 0) o = split4pd(v, P);
  else if (kind == 1) o = split8pd(v, P);
  else if (kind == 2 && P == 2) o = mixsplit2(v);
  else return -1;
  memcpy(out, o.data(), sizeof(double) * o.size());
  return 0;
}

/* The squeeze of pllsqueeze_{p}_pp_old (TCcuda.cu:876-906) run on the
 * host: y_i = sum_j x[i*pp + j] through the reference's *_inc_d. */
int ref_squeeze(int P, int pp, long n, const double *x, double *y) {
  for (long i = 0; i < n; ++i) {
    double *z = y + i * P;
    for (int l = 0; l < P; ++l) z[l] = 0.0;
    for (int j = 0; j < pp; ++j) {
      double v = x[i * pp + j];
      if (P == 2) ddf_inc_d(PTRS2(z), v);
      else if (P == 4) qdf_inc_d(PTRS4(z), v);
      else if (P == 8) odf_inc_d(PTRS8(z), v);
      else if (P == 16) hdf_inc_d(PTRS16(z), v);
      else return -1;
    }
  }
  return 0;
}

/* srand(seed) then mat(n, p, expmin, expmax): n*n random p-doubles */
int ref_mat(unsigned seed, int n, int P, int expmin, int expmax, double *out) {
  srand(seed);
  vector<double> a = mat(n, P, expmin, expmax);
  memcpy(out, a.data(), sizeof(double) * a.size());
  return 0;
}

/* bigB2(B, n, pp): (n pp) x (n pp) block-Toeplitz matrix, column-major */
int ref_bigB2(const double *Bq, int n, int pp, double *out) {
  vector<double> b(Bq, Bq + (size_t)n * n * pp);
  vector<double> o = bigB2(b, n, pp);
  memcpy(out, o.data(), sizeof(double) * o.size());
  return 0;
}

/* Layout helpers and host functions of TCcuda.cu (TCcuda.h:33-81):
 * which 0 part(x, p, i) of n P-doubles, 1 bigA(A, n, p), 2 bigB(B, n, p),
 * 3 matmulhost(A, B, n, p), 4 renormhost(A, n, p), 5 renormhostbig(A, n, p)
 * (the last two in place on a copy).  Returns the number of doubles
 * written to out, -1 for an unknown `which`. */
long ref_host(int which, int n, int p, int i, const double *A, const double *B, double *out) {
  const size_t np2 = (size_t)n * n * p;
  vector<double> a(A, A + (which == 0 ? (size_t)n * p : np2)), o;
  switch (which) {
    case 0: o = part(a, p, i); break;
    case 1: o = bigA(a, n, p); break;
    case 2: o = bigB(a, n, p); break;
    case 3: {
      vector<double> b(B, B + np2);
      o = matmulhost(a, b, n, p);
      break;
    }
    case 4: renormhost(a, n, p); o = a; break;
    case 5: renormhostbig(a, n, p); o = a; break;
    default: return -1;
  }
  memcpy(out, o.data(), sizeof(double) * o.size());
  return (long)o.size();
}

}  // extern "C"

/*
 * TCcuda.h -- drop-in declarations of the reference's C++/TCcuda.h
 * (TCcuda.h:23-103): the same names, argument order and meaning, on top of
 * the C ABI of mdgemm.h.  Implemented in dropin.cu (libmdgemm.so).
 *
 * Differences a caller can see, all documented in dropin.cu: device memory
 * is freed (the reference leaks every buffer), matmulTCnt accepts any n
 * (the reference needs n % nfrag == 0, nfrag <= 32), pllsqueeze_old
 * accepts any n (the reference needs 64 | n when n >= 64), and the
 * dispatchers return zeros for an unsupported p instead of falling off the
 * end of the function.  Every CUDA status is checked: a failed allocation,
 * copy or launch returns the zero result (t_CUDA = 0) that the reference
 * returns for an unsupported p.
 *
 * The exported kernels keep the reference's launch contract: no bounds
 * checks, so a launch must cover exactly the entries (ddmm..hdmm: an n x n
 * grid of threads, r = blockIdx.x * blockDim.x + threadIdx.x, c from y;
 * renormA / renormbigA: one block of n x n threads; the squeeze kernels:
 * exactly one thread per entry, with y holding the starting values).
 */
#ifndef MDG_DROPIN_TCCUDA_H
#define MDG_DROPIN_TCCUDA_H

#include "floatybits.h"
#include "double_double_functions.h"
#include "quad_double_functions.h"
#include "octo_double_functions.h"
#include "hexa_double_functions.h"
#include "mdgemm.h"

#include <stdio.h>
#include <cuda_runtime.h>
#ifdef __CUDACC__
#include <cublas_v2.h>
#include <curand.h>
#include <mma.h>
using namespace nvcuda;  // the reference's drivers use wmma:: unqualified
#endif

/* The kernels below are exported from libmdgemm.so (CUDA gives __global__
 * functions of a shared library hidden visibility by default) so that a
 * caller can launch them as with the reference's sources.  The launch goes
 * through the library's CUDA runtime; a program built with the static
 * runtime then has two runtimes in the process, which share the primary
 * context (device pointers pass between them), or links with
 * -cudart shared. */
#if defined(__GNUC__)
#define MDG_KERNEL_EXPORT __attribute__((visibility("default")))
#else
#define MDG_KERNEL_EXPORT
#endif

vector<double> mat(int n, int p, int expmin = 0, int expmax = 0);  /* TCcuda.h:23 */
vector<double> zeros(int m, int n, int p);  /* TCcuda.h:28 */
vector<double> part(vector<double> x, int p, int i);  /* TCcuda.h:33 */
vector<double> bigA(vector<double> A, int n, int p);  /* TCcuda.h:36 */
vector<double> bigB(vector<double> B, int n, int p);  /* TCcuda.h:44 */
vector<double> bigB2(vector<double> B, int n, int p);  /* TCcuda.h:53 */

MDG_KERNEL_EXPORT __global__ void renormbigA(double *A, int n, int p);  /* TCcuda.h:56 */
MDG_KERNEL_EXPORT __global__ void renormA(double *A, int n, int p);  /* TCcuda.h:59 */

MDG_KERNEL_EXPORT __global__ void ddmm(double *A, double *B, double *C, int n);  /* TCcuda.h:62 */
MDG_KERNEL_EXPORT __global__ void qdmm(double *A, double *B, double *C, int n);  /* TCcuda.h:63 */
MDG_KERNEL_EXPORT __global__ void odmm(double *A, double *B, double *C, int n);  /* TCcuda.h:64 */
MDG_KERNEL_EXPORT __global__ void hdmm(double *A, double *B, double *C, int n);  /* TCcuda.h:65 */
vector<double> matmulTCnt(vector<double> A, vector<double> B, int n, int nfrag, int p,
                          int loop_ct, float &t_CUDA);  /* TCcuda.h:66 */

vector<double> matmulhost(vector<double> A, vector<double> B, int n, int p);  /* TCcuda.h:69 */
vector<double> matmulddf(vector<double> A, vector<double> B, int n);  /* TCcuda.h:72 */
vector<double> matmulqdf(vector<double> A, vector<double> B, int n);  /* TCcuda.h:73 */
vector<double> matmulodf(vector<double> A, vector<double> B, int n);  /* TCcuda.h:74 */
vector<double> matmulhdf(vector<double> A, vector<double> B, int n);  /* TCcuda.h:75 */

void renormhost(vector<double> &A, int n, int p);  /* TCcuda.h:78 */
void renormhostbig(vector<double> &A, int n, int p);  /* TCcuda.h:81 */

MDG_KERNEL_EXPORT __global__ void pllsqueeze_kernel_2_8(double *x1, double *x2, double *x3, double *x4, double *x5,
                                      double *x6, double *x7, double *x8, double *y1,
                                      double *y2);  /* TCcuda.h:86 */
MDG_KERNEL_EXPORT __global__ void pllsqueeze_kernel_2_12(double *x1, double *x2, double *x3, double *x4, double *x5,
                                       double *x6, double *x7, double *x8, double *x9,
                                       double *x10, double *x11, double *x12, double *y1,
                                       double *y2);  /* TCcuda.h:89 */
MDG_KERNEL_EXPORT __global__ void pllsqueeze_kernel_2_16(double *x1, double *x2, double *x3, double *x4, double *x5,
                                       double *x6, double *x7, double *x8, double *x9,
                                       double *x10, double *x11, double *x12, double *x13,
                                       double *x14, double *x15, double *x16, double *y1,
                                       double *y2);  /* TCcuda.h:92 */
vector<double> pllsqueeze_2_8(vector<double> x);  /* TCcuda.h:87 */
vector<double> pllntsqueeze_2_8(vector<double> x);  /* TCcuda.h:88 */
vector<double> pllsqueeze_2_12(vector<double> x);  /* TCcuda.h:90 */
vector<double> pllntsqueeze_2_12(vector<double> x);  /* TCcuda.h:91 */
vector<double> pllsqueeze_2_16(vector<double> x);  /* TCcuda.h:93 */
vector<double> pllntsqueeze_2_16(vector<double> x);  /* TCcuda.h:94 */
vector<double> pllsqueeze(vector<double> x, int p, int pp);  /* TCcuda.h:95 */
vector<double> pllntsqueeze(vector<double> x, int p, int pp);  /* TCcuda.h:96 */

MDG_KERNEL_EXPORT __global__ void pllsqueeze_2_pp_old(double *x, double *y, int pp);  /* TCcuda.h:99 */
MDG_KERNEL_EXPORT __global__ void pllsqueeze_4_pp_old(double *x, double *y, int pp);  /* TCcuda.h:100 */
MDG_KERNEL_EXPORT __global__ void pllsqueeze_8_pp_old(double *x, double *y, int pp);  /* TCcuda.h:101 */
MDG_KERNEL_EXPORT __global__ void pllsqueeze_16_pp_old(double *x, double *y, int pp);  /* TCcuda.h:102 */
vector<double> pllsqueeze_old(vector<double> x, int p, int pp, float &t_CUDA);  /* TCcuda.h:103 */

/* Not in the reference header: the split GEMM of its driver (TCtest.cu:48-
 * 114) as one call, and the BF16 slice-digit form.  form is MDG_FORM_*. */
vector<double> matmulTC(vector<double> A, vector<double> B, int n, int p, int form,
                        const mdg_options *opt, float &t_CUDA);

#endif

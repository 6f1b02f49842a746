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
 * end of the function.
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

vector<double> mat(int n, int p, int expmin = 0, int expmax = 0);
vector<double> zeros(int m, int n, int p);
vector<double> part(vector<double> x, int p, int i);
vector<double> bigA(vector<double> A, int n, int p);
vector<double> bigB(vector<double> B, int n, int p);
vector<double> bigB2(vector<double> B, int n, int p);

__global__ void renormbigA(double *A, int n, int p);
__global__ void renormA(double *A, int n, int p);

__global__ void ddmm(double *A, double *B, double *C, int n);
__global__ void qdmm(double *A, double *B, double *C, int n);
__global__ void odmm(double *A, double *B, double *C, int n);
__global__ void hdmm(double *A, double *B, double *C, int n);
vector<double> matmulTCnt(vector<double> A, vector<double> B, int n, int nfrag, int p,
                          int loop_ct, float &t_CUDA);

vector<double> matmulhost(vector<double> A, vector<double> B, int n, int p);
vector<double> matmulddf(vector<double> A, vector<double> B, int n);
vector<double> matmulqdf(vector<double> A, vector<double> B, int n);
vector<double> matmulodf(vector<double> A, vector<double> B, int n);
vector<double> matmulhdf(vector<double> A, vector<double> B, int n);

void renormhost(vector<double> &A, int n, int p);
void renormhostbig(vector<double> &A, int n, int p);

vector<double> pllsqueeze_2_8(vector<double> x);
vector<double> pllntsqueeze_2_8(vector<double> x);
vector<double> pllsqueeze_2_12(vector<double> x);
vector<double> pllntsqueeze_2_12(vector<double> x);
vector<double> pllsqueeze_2_16(vector<double> x);
vector<double> pllntsqueeze_2_16(vector<double> x);
vector<double> pllsqueeze(vector<double> x, int p, int pp);
vector<double> pllntsqueeze(vector<double> x, int p, int pp);

__global__ void pllsqueeze_2_pp_old(double *x, double *y, int pp);
__global__ void pllsqueeze_4_pp_old(double *x, double *y, int pp);
__global__ void pllsqueeze_8_pp_old(double *x, double *y, int pp);
__global__ void pllsqueeze_16_pp_old(double *x, double *y, int pp);
vector<double> pllsqueeze_old(vector<double> x, int p, int pp, float &t_CUDA);

/* Not in the reference header: the split GEMM of its driver (TCtest.cu:48-
 * 114) as one call, and the BF16 slice-digit form.  form is MDG_FORM_*. */
vector<double> matmulTC(vector<double> A, vector<double> B, int n, int p, int form,
                        const mdg_options *opt, float &t_CUDA);

#endif

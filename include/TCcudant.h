/*
 * TCcudant.h -- drop-in declarations for the reference's CPU convolution
 * driver, C++/TCcudant.cpp.  That driver defines these functions itself and
 * has no header; a program that includes this header instead of defining
 * them gets the same names, argument order and meaning, with the slicing
 * and the plane convolutions on the GPU (mdg_split kind 3, mdg_plane_conv
 * of mdgemm.h).  The bit-vector helpers come from floatybits.h.
 * Implemented in dropin.cu (libmdgemm.so); compiles with g++ or nvcc.
 *
 * Differences a caller can see:
 *   splitp returns exactly p planes of A.size() / p entries.  The
 *   reference's loop (TCcudant.cpp:176, `while (j <= A.size())`) reads one
 *   element past the end of A into the first plane and so shifts every later
 *   plane by one entry.
 *   The FP64 convolutions (matmul2, convmult2, manualconvmult,
 *   dotconvbutbetter, directdotconv) sum in the FP64 tensor cores' order,
 *   so they agree with the reference's single-core loops to within a few
 *   units of 2^-53 of sum |a| |b| per entry, not bit for bit.  convadd2 is
 *   the reference's host loop and is bit-identical given the same C_aux.
 */
#ifndef MDG_DROPIN_TCCUDANT_H
#define MDG_DROPIN_TCCUDANT_H

#include "floatybits.h"

#ifndef MDG_DROPIN_TCCUDA_H
vector<double> mat(int n, int p, int expmin = 0, int expmax = 0);  /* TCcudant.cpp:186 */
#endif
vector<double> zeros(int n, int p);                                 /* TCcudant.cpp:198 */

/* split4 of every double of x without balancing (TCcudant.cpp:163): 4 slices
 * per double, the reference's bits (negative doubles give zero slices). */
vector<double> split4pd(vector<double> x);
/* AoS -> planes: plane i holds element i of every group of p (TCcudant.cpp:172). */
vector<double> splitp(vector<double> A, int p);
/* C += A B for n x n FP64 matrices (TCcudant.cpp:206). */
void matmul2(vector<double> A, vector<double> B, vector<double> &C, int n);
/* C_aux plane (i, j) += A_i B_j for all i, j < p; C_aux holds p*p planes of
 * n x n, plane (i, j) at (i p + j) n^2 (TCcudant.cpp:216). */
void convmult2(vector<double> A, vector<double> B, vector<double> &C_aux, int n, int p);
/* C_i += sum_{j<=i} C_aux plane (j, i - j) (TCcudant.cpp:232). */
void convadd2(vector<double> &C, vector<double> &C_aux, int n, int p);
/* C_i = sum_{j<=i} A_j B_{i-j} on p slice planes of n x n (TCcudant.cpp:242). */
vector<double> manualconvmult(vector<double> A, vector<double> B, int n, int p);
/* C += the same convolution (TCcudant.cpp:252). */
void dotconvbutbetter(vector<double> A, vector<double> B, vector<double> &C, int n, int p);
/* The same convolution into a new matrix (TCcudant.cpp:270). */
vector<double> directdotconv(vector<double> A, vector<double> B, int n, int p);

#endif

/*
 * cudant_shim.cpp -- C entry points around the reference's CPU path,
 * C++/TCcudant.cpp, linked with it into oracle/_ref/libcudant.so.
 * TEST INFRASTRUCTURE ONLY (golden vectors, CPU baseline in the build
 * container).  The reference functions are called unmodified:
 *   split4pd (no balancing)        TCcudant.cpp:163
 *   manualconvmult = convmult2 + convadd2   TCcudant.cpp:216-250
 *   directdotconv  = dotconvbutbetter       TCcudant.cpp:252-276
 * splitp (TCcudant.cpp:172) is not called: its loop reads one element past
 * the end of its input; the slice planes are laid out here instead.
 */
#include <cstring>
#include <vector>

using std::vector;

vector<double> split4pd(vector<double> x);
vector<double> manualconvmult(vector<double> A, vector<double> B, int n, int p);
vector<double> directdotconv(vector<double> A, vector<double> B, int n, int p);

extern "C" {

/* x: cnt doubles -> cnt*4 slices (AoS, 4 per double, no balancing) */
int cudant_split4(long cnt, const double *x, double *out) {
  vector<double> v(x, x + cnt), o = split4pd(v);
  memcpy(out, o.data(), sizeof(double) * o.size());
  return 0;
}

/* A, B: pp planes of n*n (row-major); C: pp planes of n*n partial sums
 * C_i = sum_{j<=i} A_j B_{i-j}.  how: 0 manualconvmult, 1 directdotconv. */
int cudant_conv(int how, int n, int pp, const double *A, const double *B,
                double *C) {
  size_t sz = (size_t)pp * n * n;
  vector<double> a(A, A + sz), b(B, B + sz), c;
  c = how == 0 ? manualconvmult(a, b, n, pp) : directdotconv(a, b, n, pp);
  memcpy(C, c.data(), sizeof(double) * sz);
  return 0;
}

}  // extern "C"

// The flow of the reference's CPU convolution driver (TCcudant.cpp:278-314)
// on the drop-in header include/TCcudant.h, built with the host compiler
// alone and linked against libmdgemm.so.  Reads the P-double matrices A and
// B (n x n, raw little-endian doubles) and writes, into <outdir>:
//   split.bin   split4pd(A)                        (AoS, 4P slices per entry)
//   planes.bin  splitp(split4pd(A), 4P)            (4P planes of n x n)
//   manual.bin  manualconvmult(A8, B8, n, 4P)
//   direct.bin  directdotconv(A8, B8, n, 4P)
//   twostep.bin convmult2 + convadd2 into zeros
//   accum.bin   dotconvbutbetter into a matrix of ones
//   matmul.bin  matmul2 of the first planes into a matrix of ones
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>

#include "TCcudant.h"

static vector<double> load(const std::string &path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const size_t n = (size_t)f.tellg() / sizeof(double);
  vector<double> v(n);
  f.seekg(0);
  f.read(reinterpret_cast<char *>(v.data()), n * sizeof(double));
  return v;
}

static void save(const std::string &path, const vector<double> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

int main(int argc, char **argv) {
  if (argc == 2 && std::string(argv[1]) == "short") {
    // operands one plane entry short: the two-step path leaves C and C_aux as
    // they are, the one-step paths return zeros without touching the device
    const int n = 3, p = 2;
    const vector<double> S((size_t)n * n * p - 1, 1.0), F((size_t)n * n * p, 1.0);
    vector<double> aux = zeros(n, p * p), C = zeros(n, p);
    convmult2(S, F, aux, n, p);
    vector<double> aux_short((size_t)n * n * p * p - 1, 0.0);
    convmult2(F, F, aux_short, n, p);
    convadd2(C, aux_short, n, p);
    double t = 0.0;
    for (double x : aux) t += x;
    for (double x : aux_short) t += x;
    for (double x : C) t += x;
    for (double x : manualconvmult(S, F, n, p)) t += x;
    for (double x : directdotconv(F, S, n, p)) t += x;
    printf("short %g\n", t);
    return 0;
  }
  if (argc != 6) return 2;
  const int p = atoi(argv[1]), n = atoi(argv[2]), pp = 4 * p;
  const std::string out = argv[5];
  const vector<double> A = load(argv[3]), B = load(argv[4]);
  const vector<double> As = split4pd(A);
  const vector<double> A8 = splitp(As, pp), B8 = splitp(split4pd(B), pp);
  save(out + "/split.bin", As);
  save(out + "/planes.bin", A8);
  save(out + "/manual.bin", manualconvmult(A8, B8, n, pp));
  save(out + "/direct.bin", directdotconv(A8, B8, n, pp));
  vector<double> aux = zeros(n, pp * pp), C = zeros(n, pp);
  convmult2(A8, B8, aux, n, pp);
  convadd2(C, aux, n, pp);
  save(out + "/twostep.bin", C);
  vector<double> acc(C.size(), 1.0);
  dotconvbutbetter(A8, B8, acc, n, pp);
  save(out + "/accum.bin", acc);
  vector<double> M((size_t)n * n, 1.0);
  matmul2(vector<double>(A8.begin(), A8.begin() + (size_t)n * n),
          vector<double>(B8.begin(), B8.begin() + (size_t)n * n), M, n);
  save(out + "/matmul.bin", M);
  return 0;
}

// Host-side checks of the drop-in C++ surface (include/TCcuda.h,
// include/floatybits.h) linked against libmdgemm.so.  Each command reads and
// writes raw little-endian doubles; tests/test_dropin_cpp.py drives it and
// compares with the golden vectors made by the reference.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

#include "TCcuda.h"

static vector<double> load(const char *path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const size_t n = (size_t)f.tellg() / sizeof(double);
  vector<double> v(n);
  f.seekg(0);
  f.read(reinterpret_cast<char *>(v.data()), n * sizeof(double));
  return v;
}

static void save(const char *path, const vector<double> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const std::string cmd = argv[1];
  if (cmd == "mat") {  // mat <n> <p> <seed> <out> [<expmin> <expmax>]
    srand((unsigned)atoi(argv[4]));
    const int e0 = argc > 7 ? atoi(argv[6]) : 0, e1 = argc > 7 ? atoi(argv[7]) : 0;
    save(argv[5], mat(atoi(argv[2]), atoi(argv[3]), e0, e1));
  } else if (cmd == "matmul") {  // matmul <p> <n> <A> <B> <out>
    const int p = atoi(argv[2]), n = atoi(argv[3]);
    vector<double> A = load(argv[4]), B = load(argv[5]), C;
    if (p == 2) C = matmulddf(A, B, n);
    else if (p == 4) C = matmulqdf(A, B, n);
    else if (p == 8) C = matmulodf(A, B, n);
    else C = matmulhdf(A, B, n);
    save(argv[6], C);
  } else if (cmd == "bigB2") {  // bigB2 <n> <pp> <in> <out>
    save(argv[5], bigB2(load(argv[4]), atoi(argv[2]), atoi(argv[3])));
  } else if (cmd == "squeeze") {  // squeeze <p> <pp> <in> <out>
    save(argv[5], pllntsqueeze(load(argv[4]), atoi(argv[2]), atoi(argv[3])));
  } else if (cmd == "host") {  // host <name> <p> <n> <A> <B> <out>: TCcuda.h:33-81
    const std::string name = argv[2];
    const int p = atoi(argv[3]), n = atoi(argv[4]);
    vector<double> A = load(argv[5]), B = load(argv[6]), out;
    if (name == "part1") out = part(A, p, 1);
    else if (name == "bigA") out = bigA(A, n, p);
    else if (name == "bigB") out = bigB(B, n, p);
    else if (name == "matmulhost") out = matmulhost(A, B, n, p);
    else if (name == "renormhost") { renormhost(A, n, p); out = A; }
    else if (name == "renormhostbig") { renormhostbig(A, n, p); out = A; }
    else return 3;
    save(argv[7], out);
  } else if (cmd == "short") {  // short <p> <n>: n x n x p operands one double short
    const int p = atoi(argv[2]), n = atoi(argv[3]);
    const vector<double> S((size_t)n * n * p - 1, 1.0), F((size_t)n * n * p, 1.0);
    auto sum = [](const vector<double> &v) {
      double t = 0.0;
      for (double x : v) t += x;
      return t;
    };
    vector<double> R = S, Rb = S;
    renormhost(R, n, p);
    renormhostbig(Rb, n, p);
    float t = 1.0f;
    const vector<double> C1 = matmulhost(S, F, n, p), C2 = matmulhost(F, S, n, p);
    const vector<double> C3 = matmulTCnt(S, F, n, 8, p, 1, t);
    printf("bigA %zu\nbigB %zu\nbigB2 %zu\n", bigA(S, n, p).size(), bigB(S, n, p).size(),
           bigB2(S, n, p).size());
    printf("matmulhost %zu %g %zu %g\n", C1.size(), sum(C1), C2.size(), sum(C2));
    printf("renormhost %g\nrenormhostbig %g\n", sum(R), sum(Rb));
    printf("matmulTCnt %zu %g %g\n", C3.size(), sum(C3), (double)t);
    if (p == 2) printf("matmulddf %g\n", sum(matmulddf(S, F, n)));
    if (p == 4) printf("matmulqdf %g\n", sum(matmulqdf(F, S, n)));
    printf("pllntsqueeze %zu\n", pllntsqueeze(F, p, 0).size());
  } else if (cmd == "kernels") {  // kernels: every __global__ of TCcuda.h links from the library
    const void *k[] = {(const void *)&renormbigA,           (const void *)&renormA,
                       (const void *)&ddmm,                 (const void *)&qdmm,
                       (const void *)&odmm,                 (const void *)&hdmm,
                       (const void *)&pllsqueeze_kernel_2_8, (const void *)&pllsqueeze_kernel_2_12,
                       (const void *)&pllsqueeze_kernel_2_16, (const void *)&pllsqueeze_2_pp_old,
                       (const void *)&pllsqueeze_4_pp_old,  (const void *)&pllsqueeze_8_pp_old,
                       (const void *)&pllsqueeze_16_pp_old};
    int n = 0;
    for (const void *f : k) n += f != nullptr;
    printf("%d\n", n);
  } else if (cmd == "bits") {  // bits <x> : bitform / double_rep round trip
    const double x = atof(argv[2]);
    printf("%.17g\n", double_rep(bitform(x)));
  } else {
    return 2;
  }
  return 0;
}

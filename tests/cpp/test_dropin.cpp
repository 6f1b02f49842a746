// Checks of the drop-in C++ surface (include/TCcuda.h, include/floatybits.h)
// linked against libmdgemm.so.  Each command reads and writes raw
// little-endian doubles; tests/test_dropin_cpp.py drives it and compares with
// the golden vectors made by the reference.  The host commands run anywhere;
// the GPU commands (tcnt, tc, gsplit, gsqueeze, kmm, krenorm, ksqpp, ksq2)
// call the std::vector wrappers and launch the exported kernels the way the
// reference's drivers do.  Build with -cudart shared so that the <<<>>>
// launches and the library use one CUDA runtime.
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

#define CHECK_CUDA(call)                                                        \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 4;                                                                 \
    }                                                                           \
  } while (0)

// A device copy of a host vector (freed at scope exit).
struct Dev {
  double *p = nullptr;
  size_t n = 0;
  explicit Dev(size_t count) : n(count) {
    if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess) p = nullptr;
  }
  ~Dev() {
    if (p) cudaFree(p);
  }
};

// GPU commands of the drop-in; 0 on success, 4 on a CUDA failure.
static int gpu_command(const std::string &cmd, int argc, char **argv) {
  if (cmd == "tcnt") {  // tcnt <p> <n> <nfrag> <A> <B> <out>: matmulTCnt, two launches
    const int p = atoi(argv[2]), n = atoi(argv[3]), nfrag = atoi(argv[4]);
    float t = -1.0f;
    const vector<double> C = matmulTCnt(load(argv[5]), load(argv[6]), n, nfrag, p, 2, t);
    printf("%g\n", (double)t);
    save(argv[7], C);
    return t > 0.0f ? 0 : 5;
  }
  if (cmd == "tc") {  // tc <form> <p> <n> <A> <B> <out>: matmulTC, default options
    const int form = atoi(argv[2]), p = atoi(argv[3]), n = atoi(argv[4]);
    float t = -1.0f;
    const vector<double> C = matmulTC(load(argv[5]), load(argv[6]), n, p, form, nullptr, t);
    printf("%g\n", (double)t);
    save(argv[7], C);
    return t > 0.0f ? 0 : 5;
  }
  if (cmd == "gsplit") {  // gsplit <split4|split8|mix> <p> <in> <out>
    const std::string kind = argv[2];
    const int p = atoi(argv[3]);
    const vector<double> x = load(argv[4]);
    save(argv[5], kind == "split4" ? split4pd(x, p) : kind == "split8" ? split8pd(x, p)
                                                                         : mixsplit2(x));
    return 0;
  }
  if (cmd == "gsqueeze") {  // gsqueeze <old|any|dd> <p> <pp> <in> <out>
    const std::string how = argv[2];
    const int p = atoi(argv[3]), pp = atoi(argv[4]);
    const vector<double> x = load(argv[5]);
    float t = -1.0f;
    vector<double> y;
    if (how == "old") y = pllsqueeze_old(x, p, pp, t);
    else if (how == "any") y = pllsqueeze(x, p, pp);
    else y = pp == 8 ? pllsqueeze_2_8(x) : pp == 12 ? pllsqueeze_2_12(x) : pllsqueeze_2_16(x);
    save(argv[6], y);
    return (how == "old" && !(t > 0.0f)) ? 5 : 0;
  }
  if (cmd == "kmm") {  // kmm <p> <n> <nfrag> <A> <B> <out>: {dd,qd,od,hd}mm as matmulTCnt launches them
    const int p = atoi(argv[2]), n = atoi(argv[3]), nfrag = atoi(argv[4]);
    const vector<double> A = load(argv[5]), B = load(argv[6]);
    const size_t sz = (size_t)n * n * p;
    if (A.size() != sz || B.size() != sz || n % nfrag) return 3;
    Dev dA(sz), dB(sz), dC(sz);
    if (!dA.p || !dB.p || !dC.p) return 4;
    CHECK_CUDA(cudaMemcpy(dA.p, A.data(), sz * 8, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(dB.p, B.data(), sz * 8, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemset(dC.p, 0, sz * 8));
    const dim3 grid(n / nfrag, n / nfrag), block(nfrag, nfrag);
    if (p == 2) ddmm<<<grid, block>>>(dA.p, dB.p, dC.p, n);
    else if (p == 4) qdmm<<<grid, block>>>(dA.p, dB.p, dC.p, n);
    else if (p == 8) odmm<<<grid, block>>>(dA.p, dB.p, dC.p, n);
    else hdmm<<<grid, block>>>(dA.p, dB.p, dC.p, n);
    CHECK_CUDA(cudaGetLastError());
    CHECK_CUDA(cudaDeviceSynchronize());
    vector<double> C(sz);
    CHECK_CUDA(cudaMemcpy(C.data(), dC.p, sz * 8, cudaMemcpyDeviceToHost));
    save(argv[7], C);
    return 0;
  }
  if (cmd == "krenorm") {  // krenorm <A|bigA> <p> <n> <in> <out>: one block of n x n threads
    const std::string which = argv[2];
    const int p = atoi(argv[3]), n = atoi(argv[4]);
    vector<double> A = load(argv[5]);
    if (A.size() != (size_t)n * n * p || n * n > 1024) return 3;
    Dev dA(A.size());
    if (!dA.p) return 4;
    CHECK_CUDA(cudaMemcpy(dA.p, A.data(), A.size() * 8, cudaMemcpyHostToDevice));
    if (which == "A") renormA<<<1, dim3(n, n)>>>(dA.p, n, p);
    else renormbigA<<<1, dim3(n, n)>>>(dA.p, n, p);
    CHECK_CUDA(cudaGetLastError());
    CHECK_CUDA(cudaMemcpy(A.data(), dA.p, A.size() * 8, cudaMemcpyDeviceToHost));
    save(argv[6], A);
    return 0;
  }
  if (cmd == "ksqpp") {  // ksqpp <p> <pp> <blocks> <threads> <in> <out>: pllsqueeze_{p}_pp_old
    const int p = atoi(argv[2]), pp = atoi(argv[3]), nb = atoi(argv[4]), nt = atoi(argv[5]);
    const vector<double> x = load(argv[6]);
    const size_t cnt = (size_t)nb * nt;
    if (x.size() != cnt * pp) return 3;  // exactly one thread per entry
    Dev dx(x.size()), dy(cnt * p);
    if (!dx.p || !dy.p) return 4;
    CHECK_CUDA(cudaMemcpy(dx.p, x.data(), x.size() * 8, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemset(dy.p, 0, cnt * p * 8));
    if (p == 2) pllsqueeze_2_pp_old<<<nb, nt>>>(dx.p, dy.p, pp);
    else if (p == 4) pllsqueeze_4_pp_old<<<nb, nt>>>(dx.p, dy.p, pp);
    else if (p == 8) pllsqueeze_8_pp_old<<<nb, nt>>>(dx.p, dy.p, pp);
    else pllsqueeze_16_pp_old<<<nb, nt>>>(dx.p, dy.p, pp);
    CHECK_CUDA(cudaGetLastError());
    vector<double> y(cnt * p);
    CHECK_CUDA(cudaMemcpy(y.data(), dy.p, y.size() * 8, cudaMemcpyDeviceToHost));
    save(argv[7], y);
    return 0;
  }
  if (cmd == "ksq2") {  // ksq2 <pp> <blocks> <threads> <in> <out>: the separate-plane dd squeeze
    const int pp = atoi(argv[2]), nb = atoi(argv[3]), nt = atoi(argv[4]);
    const vector<double> x = load(argv[5]);
    const size_t cnt = (size_t)nb * nt;
    if (x.size() != cnt * pp || (pp != 8 && pp != 12 && pp != 16)) return 3;
    // slice j of every entry into plane j, as the reference's part() gathers
    vector<double> planes(x.size());
    for (int j = 0; j < pp; ++j)
      for (size_t i = 0; i < cnt; ++i) planes[j * cnt + i] = x[i * pp + j];
    Dev dx(x.size()), dy(2 * cnt);
    if (!dx.p || !dy.p) return 4;
    CHECK_CUDA(cudaMemcpy(dx.p, planes.data(), x.size() * 8, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemset(dy.p, 0, 2 * cnt * 8));
    double *q[16];
    for (int j = 0; j < 16; ++j) q[j] = dx.p + (size_t)(j < pp ? j : 0) * cnt;
    double *y1 = dy.p, *y2 = dy.p + cnt;
    if (pp == 8) pllsqueeze_kernel_2_8<<<nb, nt>>>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7],
                                                  y1, y2);
    else if (pp == 12)
      pllsqueeze_kernel_2_12<<<nb, nt>>>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8],
                                         q[9], q[10], q[11], y1, y2);
    else
      pllsqueeze_kernel_2_16<<<nb, nt>>>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8],
                                         q[9], q[10], q[11], q[12], q[13], q[14], q[15], y1, y2);
    CHECK_CUDA(cudaGetLastError());
    vector<double> yy(2 * cnt), y(2 * cnt);
    CHECK_CUDA(cudaMemcpy(yy.data(), dy.p, yy.size() * 8, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < cnt; ++i) {
      y[2 * i] = yy[i];
      y[2 * i + 1] = yy[cnt + i];
    }
    save(argv[6], y);
    return 0;
  }
  return -1;
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
    const int r = gpu_command(cmd, argc, argv);
    return r < 0 ? 2 : r;
  }
  return 0;
}

// Drop-in C++ surface of the reference (TCcuda.h:23-103, floatybits.h:17-97,
// and the functions of the CPU convolution driver TCcudant.cpp:163-276)
// over the C ABI.  std::vector in, std::vector out, like the reference; the
// GPU work goes through mdg_* entry points.
//
// Behaviour kept from the reference: argument order and meaning, the
// sequence of rand() calls of mat/random_pd (so srand(s) gives the same
// matrices), reference-compatible slices in split4pd/split8pd/mixsplit2,
// zeros for an unsupported p in matmulTCnt and pllsqueeze_old, extended to
// every failure: a device allocation, copy or launch that fails gives the
// zero result (and t_CUDA = 0), with the CUDA error text kept for
// mdg_last_cuda_error().
// Behaviour changed: device memory is freed; any n is accepted where the
// reference needs n % nfrag == 0 or 64 | n; the pllsqueeze / pllntsqueeze
// dispatchers return zeros for an unsupported p (the reference has no
// return statement on that path, TCcuda.cu:810-853); a vector shorter than
// its n x n x p (or planes) shape gives the empty / zero result instead of
// a read past its end, on the host or, through the device copies, on the GPU.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "TCcuda.h"
#include "TCcudant.h"
#include "common.cuh"

namespace {

struct DevBuf {
  double *p = nullptr;
  explicit DevBuf(size_t n) {
    if (n && cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) p = nullptr;
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

// The call succeeded; otherwise its error is recorded (mdg_last_cuda_error).
bool cuda_ok(cudaError_t e) {
  if (e == cudaSuccess) return true;
  mdgi::set_cuda_error(e);
  return false;
}

bool to_device(double *dst, const vector<double> &src, size_t count) {
  return count == 0 ||
         cuda_ok(cudaMemcpy(dst, src.data(), count * sizeof(double), cudaMemcpyHostToDevice));
}

// Copies count doubles back; on failure the host vector is cleared to zeros
// (the reference's result for a call that did not run).
bool to_host(vector<double> &dst, const double *src, size_t count) {
  if (count == 0) return true;
  if (cuda_ok(cudaMemcpy(dst.data(), src, count * sizeof(double), cudaMemcpyDeviceToHost)))
    return true;
  std::fill(dst.begin(), dst.end(), 0.0);
  return false;
}

// Two events on the legacy default stream around the work of a wrapper;
// elapsed() is the time between them in ms, or a failure.
struct Timer {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool ok = false;
  Timer() { ok = cuda_ok(cudaEventCreate(&e0)) && cuda_ok(cudaEventCreate(&e1)); }
  ~Timer() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
  bool start() { return ok && cuda_ok(cudaEventRecord(e0)); }
  bool stop(float &ms) {
    return cuda_ok(cudaEventRecord(e1)) && cuda_ok(cudaEventSynchronize(e1)) &&
           cuda_ok(cudaEventElapsedTime(&ms, e0, e1));
  }
};

// v holds at least `count` doubles (a negative count never fits)
bool holds(const vector<double> &v, long long count) {
  return count >= 0 && v.size() >= (size_t)count;
}

// n x n entries of p doubles, or -1 for a negative size
long long nnp(int n, int p) { return (n < 0 || p < 0) ? -1 : (long long)n * n * p; }

vector<double> gpu_split(int kind, vector<double> x, int p) {
  if (p <= 0) return vector<double>();
  const int pp = kind == 0 ? 4 * p : kind == 1 ? 8 * p : 12;
  const long long count = (long long)x.size() / p;
  vector<double> out((size_t)count * pp, 0.0);
  if (!count) return out;
  DevBuf dx(x.size()), dout(out.size());
  if (!dx.p || !dout.p || !to_device(dx.p, x, x.size())) return out;
  if (mdg_split(kind, 0, p, count, dx.p, dout.p, nullptr) == MDG_SUCCESS)
    to_host(out, dout.p, out.size());
  return out;
}

template <int P>
vector<double> host_plain(const vector<double> &A, const vector<double> &B, int n) {
  if (n < 0) return vector<double>();
  vector<double> C((size_t)n * n * P, 0.0);
  if (!holds(A, nnp(n, P)) || !holds(B, nnp(n, P))) return C;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      double acc[P];
      for (int l = 0; l < P; ++l) acc[l] = 0.0;
      for (int k = 0; k < n; ++k)
        mdg::madd<P>(acc, &A[((size_t)r * n + k) * P], &B[((size_t)k * n + c) * P]);
      for (int l = 0; l < P; ++l) C[((size_t)r * n + c) * P + l] = acc[l];
    }
  return C;
}

template <int P>
vector<double> host_squeeze(const vector<double> &x, int pp) {
  if (pp <= 0) return vector<double>();
  const size_t n = x.size() / pp;
  vector<double> y(n * P, 0.0);
  for (size_t i = 0; i < n; ++i) {
    double acc[P];
    for (int l = 0; l < P; ++l) acc[l] = 0.0;
    for (int j = 0; j < pp; ++j) mdg::inc_d<P>(acc, x[i * pp + j]);
    for (int l = 0; l < P; ++l) y[i * P + l] = acc[l];
  }
  return y;
}

}  // namespace

// ------------------------------------------------------------ floatybits --

int val_bits(vector<int> bits) {
  int s = 0;
  for (size_t i = 0; i < bits.size(); ++i) s = 2 * s + bits[i];
  return s;
}

// Binary expansion of a fraction in [0, 1]; a non-positive input expands to
// nothing (then zero-padded to 52 entries), as in the reference.
vector<int> expandfracbits(double fr) {
  vector<int> bits;
  double t = fr;
  int i = -1;
  while (t > 0) {
    const double w = ldexp(1.0, i);
    if (t >= w) {
      bits.push_back(1);
      t -= w;
    } else {
      bits.push_back(0);
    }
    --i;
  }
  while (bits.size() < 52) bits.push_back(0);
  return bits;
}

vector<int> expandexpbits(int n) {
  vector<int> bits;
  for (int t = n; t > 0; t /= 2) bits.insert(bits.begin(), t % 2);
  while (bits.size() < 11) bits.insert(bits.begin(), 0);
  return bits;
}

vector<int> bitform(double x) {
  int e;
  const double f = frexp(x, &e);
  vector<int> bits;
  bits.push_back(x >= 0 ? 0 : 1);
  vector<int> eb = expandexpbits(e + 1023), fb = expandfracbits(f);
  bits.insert(bits.end(), eb.begin(), eb.end());
  bits.insert(bits.end(), fb.begin(), fb.end());
  return bits;
}

vector<int> random_double_bits(int signbit, int exponent, bool fixfirst) {
  vector<int> bits;
  bits.push_back(signbit);
  vector<int> eb = expandexpbits(exponent);
  bits.insert(bits.end(), eb.begin(), eb.end());
  for (int i = 0; i < 52; ++i) bits.push_back(rand() % 2);
  if (fixfirst) bits[12] = 1;
  return bits;
}

double double_rep(vector<int> bits) {
  vector<int> eb(bits.begin() + 1, bits.begin() + 12);
  const int exponent = val_bits(eb) - 1023;
  uint64_t F = 0;
  for (int i = 1; i <= 52; ++i) F = (F << 1) | (uint64_t)(bits[11 + i] & 1);
  const double fraction = ldexp((double)F, -52);
  return (bits[0] ? -1.0 : 1.0) * fraction * ldexp(1.0, exponent);
}

vector<double> random_pd(int expmin, int expmax, int p) {
  const int hiexp = (expmax == expmin) ? expmin + 1023 : expmin + 1023 + rand() % (expmax - expmin);
  vector<double> parts;
  for (int i = 0; i < p; ++i) parts.push_back(double_rep(random_double_bits(0, hiexp - 52 * i)));
  return parts;
}

bool is_balanced(double x, double y, int threshold) {
  int xe, ye;
  frexp(x, &xe);
  frexp(y, &ye);
  return !(xe - ye > threshold);
}

void balance(double &x, double &y, int threshold) {
  if (x == 0.0 || y == 0.0) return;
  if (is_balanced(x, y, threshold - 1)) return;
  int xe;
  frexp(x, &xe);
  const double bit = ldexp(1.0, xe - threshold);
  x = x - bit;
  y = y + bit;
}

void balance4(vector<double> &x, int a, int b) {
  for (int i = a; i < b; ++i) balance(x[i], x[i + 1], 14);
}

void balance8(vector<double> &x, int a, int b) {
  for (int i = a; i < b - 1; ++i) balance(x[i], x[i + 1], (i - a) % 8 < 4 ? 8 : 7);
}

void mixbalance(vector<double> &x, int a, int b) {
  for (int i = a; i < b - 1; ++i) {
    const int j = (i - a) % 12;
    balance(x[i], x[i + 1], j < 4 ? 14 : j < 8 ? 8 : 7);
  }
}

static vector<double> split_bits(const vector<int> &bits, const int *ranges, int nr) {
  vector<double> D;
  double s = 0.0;
  for (int t = 0; t < nr; ++t) {
    vector<int> b = bits;
    for (int i = 0; i < 52; ++i)
      if (i < ranges[t] || i >= ranges[t + 1]) b[12 + i] = 0;
    const double d = double_rep(b);
    D.push_back(d);
    s = (t == 0) ? d : s + d;
  }
  D.push_back(double_rep(bits) - s);
  return D;
}

vector<double> split4(vector<int> bits) {
  static const int r[4] = {0, 13, 26, 39};
  return split_bits(bits, r, 3);
}

vector<double> split8(vector<int> bits) {
  static const int r[8] = {0, 7, 14, 21, 28, 34, 40, 52};
  return split_bits(bits, r, 7);
}

vector<double> split4pd(vector<double> x, int p) { return gpu_split(0, x, p); }
vector<double> split8pd(vector<double> x, int p) { return gpu_split(1, x, p); }
vector<double> mixsplit2(vector<double> x) { return gpu_split(2, x, 2); }

// ---------------------------------------------------------------- TCcuda --

vector<double> mat(int n, int p, int expmin, int expmax) {
  vector<double> A;
  for (int i = 0; i < n * n; ++i) {
    vector<double> a = random_pd(expmin, expmax, p);
    A.insert(A.end(), a.begin(), a.end());
  }
  return A;
}

vector<double> zeros(int m, int n, int p) { return vector<double>((size_t)m * n * p, 0.0); }

vector<double> part(vector<double> x, int p, int i) {
  vector<double> xi;
  for (size_t j = i; j < x.size(); j += p) xi.push_back(x[j]);
  return xi;
}

vector<double> bigA(vector<double> A, int n, int p) {
  vector<double> AA;
  if (!holds(A, nnp(n, p))) return AA;
  for (int r = 0; r < n; ++r)
    for (int i = 0; i < p; ++i)
      for (int c = 0; c < n; ++c) AA.push_back(A[((size_t)r * n + c) * p + i]);
  return AA;
}

vector<double> bigB(vector<double> B, int n, int p) {
  vector<double> BB;
  if (!holds(B, nnp(n, p))) return BB;
  for (int i = 0; i < p; ++i)
    for (int c = 0; c < n; ++c)
      for (int j = 0; j < p; ++j)
        for (int r = 0; r < n; ++r)
          BB.push_back(j <= i ? B[((size_t)r * n + c) * p + (i - j)] : 0.0);
  return BB;
}

vector<double> bigB2(vector<double> B, int n, int p) {
  vector<double> BB;
  if (!holds(B, nnp(n, p))) return BB;
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < p; ++i)
      for (int r = 0; r < n; ++r)
        for (int j = 0; j < p; ++j)
          BB.push_back(j <= i ? B[((size_t)r * n + c) * p + (i - j)] : 0.0);
  return BB;
}

// One pass of hi = a_k + a_k+1, lo = hi - a_k over the limbs; kept as the
// reference defines it (TCcuda.cu:97-117): it is not an error-free
// transformation.  One thread per (i, j) of an n x n block.
__global__ void renormbigA(double *A, int n, int p) {
  const int i = threadIdx.x, j = threadIdx.y;
  for (int k = 0; k < p - 1; ++k) {
    const double hi = A[i * n * p + k * n + j] + A[i * n * p + (k + 1) * n + j];
    const double lo = hi - A[i * n * p + k * n + j];
    A[i * n * p + k * n + j] = hi;
    A[i * n * p + (k + 1) * n + j] = lo;
  }
}

__global__ void renormA(double *A, int n, int p) {
  const int i = threadIdx.x, j = threadIdx.y;
  for (int k = 0; k < p - 1; ++k) {
    const double hi = A[i * n * p + j * p + k] + A[i * n * p + j * p + k + 1];
    const double lo = hi - A[i * n * p + j * p + k];
    A[i * n * p + j * p + k] = hi;
    A[i * n * p + j * p + k + 1] = lo;
  }
}

void renormhost(vector<double> &A, int n, int p) {
  if (!holds(A, nnp(n, p))) return;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double *e = A.data() + ((size_t)i * n + j) * p;  // entry (i, j), limbs adjacent
      for (int k = 0; k < p - 1; ++k) {
        const double hi = e[k] + e[k + 1];
        const double lo = hi - e[k];
        e[k] = hi;
        e[k + 1] = lo;
      }
    }
}

void renormhostbig(vector<double> &A, int n, int p) {
  if (!holds(A, nnp(n, p))) return;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double *e = A.data() + (size_t)i * n * p + j;  // row i, column j: limbs n apart
      for (int k = 0; k < p - 1; ++k) {
        const double hi = e[(size_t)k * n] + e[(size_t)(k + 1) * n];
        const double lo = hi - e[(size_t)k * n];
        e[(size_t)k * n] = hi;
        e[(size_t)(k + 1) * n] = lo;
      }
    }
}

// One thread per entry C(r, c) with r from x and c from y, as the
// reference's kernels (TCcuda.cu:119-246); n x n, no bounds check (the
// launch must cover exactly n x n).
template <int P>
__device__ void plain_entry(const double *A, const double *B, double *C, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y * blockDim.y + threadIdx.y;
  double acc[P];
  for (int l = 0; l < P; ++l) acc[l] = 0.0;
  for (int k = 0; k < n; ++k) mdg::madd<P>(acc, A + ((size_t)r * n + k) * P, B + ((size_t)k * n + c) * P);
  for (int l = 0; l < P; ++l) C[((size_t)r * n + c) * P + l] = acc[l];
}
__global__ void ddmm(double *A, double *B, double *C, int n) { plain_entry<2>(A, B, C, n); }
__global__ void qdmm(double *A, double *B, double *C, int n) { plain_entry<4>(A, B, C, n); }
__global__ void odmm(double *A, double *B, double *C, int n) { plain_entry<8>(A, B, C, n); }
__global__ void hdmm(double *A, double *B, double *C, int n) { plain_entry<16>(A, B, C, n); }

// matmulTCnt: the plain form on the GPU, loop_ct launches timed with events.
// Any failure (allocation, copy, launch) returns zeros and t_CUDA = 0, the
// reference's result when no kernel ran (TCcuda.cu:269-298).
vector<double> matmulTCnt(vector<double> A, vector<double> B, int n, int nfrag, int p,
                          int loop_ct, float &t_CUDA) {
  (void)nfrag;  // the tiling is the library's; any n works
  vector<double> C = zeros(n, n, p);
  t_CUDA = 0.0f;
  if (!mdgi::valid_p(p) || n <= 0) return C;
  const size_t sz = (size_t)n * n * p;
  if (!holds(A, nnp(n, p)) || !holds(B, nnp(n, p))) return C;
  DevBuf dA(sz), dB(sz), dC(sz);
  if (!dA.p || !dB.p || !dC.p) return C;
  if (!to_device(dA.p, A, sz) || !to_device(dB.p, B, sz) ||
      !cuda_ok(cudaMemset(dC.p, 0, sz * sizeof(double))))
    return C;
  Timer tm;
  float ms = 0.0f;
  if (!tm.start()) return C;
  int st = MDG_SUCCESS;
  for (int l = 0; l < loop_ct && st == MDG_SUCCESS; ++l)
    st = mdg_gemm(MDG_FORM_PLAIN, p, n, n, n, dA.p, n, dB.p, n, dC.p, n, nullptr, nullptr, 0,
                  nullptr);
  if (!tm.stop(ms) || st != MDG_SUCCESS || !to_host(C, dC.p, sz)) return C;
  t_CUDA = ms;
  return C;
}

// The same contract for any form: zeros and t_CUDA = 0 on a failure.
vector<double> matmulTC(vector<double> A, vector<double> B, int n, int p, int form,
                        const mdg_options *opt, float &t_CUDA) {
  vector<double> C = zeros(n, n, p);
  t_CUDA = 0.0f;
  if (!mdgi::valid_p(p) || n <= 0) return C;
  const size_t sz = (size_t)n * n * p;
  if (!holds(A, nnp(n, p)) || !holds(B, nnp(n, p))) return C;
  DevBuf dA(sz), dB(sz), dC(sz);
  if (!dA.p || !dB.p || !dC.p) return C;
  const size_t ws_bytes = mdg_gemm_workspace_size(form, p, n, n, n, opt);
  DevBuf ws((ws_bytes + sizeof(double) - 1) / sizeof(double));
  if (ws_bytes && !ws.p) return C;
  if (!to_device(dA.p, A, sz) || !to_device(dB.p, B, sz)) return C;
  Timer tm;
  float ms = 0.0f;
  if (!tm.start()) return C;
  const int st = mdg_gemm(form, p, n, n, n, dA.p, n, dB.p, n, dC.p, n, opt, ws.p, ws_bytes,
                          nullptr);
  if (!tm.stop(ms) || st != MDG_SUCCESS || !to_host(C, dC.p, sz)) return C;
  t_CUDA = ms;
  return C;
}

// Naive FP64 slice convolution without error-free transformations
// (TCcuda.cu:304-318).
vector<double> matmulhost(vector<double> A, vector<double> B, int n, int p) {
  if (nnp(n, p) < 0) return vector<double>();
  vector<double> C = zeros(n, n, p);
  if (!holds(A, nnp(n, p)) || !holds(B, nnp(n, p))) return C;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      for (int k = 0; k < n; ++k)
        for (int i = 0; i < p; ++i)
          for (int j = 0; j <= i; ++j)
            C[((size_t)r * n + c) * p + i] +=
                A[((size_t)r * n + k) * p + j] * B[((size_t)k * n + c) * p + (i - j)];
  return C;
}

vector<double> matmulddf(vector<double> A, vector<double> B, int n) { return host_plain<2>(A, B, n); }
vector<double> matmulqdf(vector<double> A, vector<double> B, int n) { return host_plain<4>(A, B, n); }
vector<double> matmulodf(vector<double> A, vector<double> B, int n) { return host_plain<8>(A, B, n); }
vector<double> matmulhdf(vector<double> A, vector<double> B, int n) { return host_plain<16>(A, B, n); }

// ------------------------------------------------------------ squeezing --

vector<double> pllsqueeze_old(vector<double> x, int p, int pp, float &t_CUDA) {
  t_CUDA = 0.0f;
  const long long n = pp > 0 ? (long long)x.size() / pp : 0;
  vector<double> y = zeros((int)n, 1, mdgi::valid_p(p) ? p : 1);
  if (!mdgi::valid_p(p) || n == 0) return y;
  DevBuf dx(x.size()), dy(y.size());
  if (!dx.p || !dy.p || !to_device(dx.p, x, x.size())) return y;
  Timer tm;
  float ms = 0.0f;
  if (!tm.start()) return y;
  const int st = mdg_squeeze(p, pp, n, dx.p, dy.p, nullptr);
  if (!tm.stop(ms) || st != MDG_SUCCESS || !to_host(y, dy.p, y.size())) return y;
  t_CUDA = ms;
  return y;
}

vector<double> pllsqueeze(vector<double> x, int p, int pp) {
  float t;
  return pllsqueeze_old(x, p, pp, t);
}

vector<double> pllntsqueeze(vector<double> x, int p, int pp) {
  switch (p) {
    case 2: return host_squeeze<2>(x, pp);
    case 4: return host_squeeze<4>(x, pp);
    case 8: return host_squeeze<8>(x, pp);
    case 16: return host_squeeze<16>(x, pp);
  }
  return vector<double>();
}

vector<double> pllsqueeze_2_8(vector<double> x) { return pllsqueeze(x, 2, 8); }
vector<double> pllsqueeze_2_12(vector<double> x) { return pllsqueeze(x, 2, 12); }
vector<double> pllsqueeze_2_16(vector<double> x) { return pllsqueeze(x, 2, 16); }
vector<double> pllntsqueeze_2_8(vector<double> x) { return pllntsqueeze(x, 2, 8); }
vector<double> pllntsqueeze_2_12(vector<double> x) { return pllntsqueeze(x, 2, 12); }
vector<double> pllntsqueeze_2_16(vector<double> x) { return pllntsqueeze(x, 2, 16); }

template <int P>
__device__ void squeeze_entry(const double *x, double *y, int pp) {
  const int i = blockDim.x * blockIdx.x + threadIdx.x;
  double acc[P];
  for (int l = 0; l < P; ++l) acc[l] = y[(size_t)P * i + l];
  for (int j = 0; j < pp; ++j) mdg::inc_d<P>(acc, x[(size_t)pp * i + j]);
  for (int l = 0; l < P; ++l) y[(size_t)P * i + l] = acc[l];
}
__global__ void pllsqueeze_2_pp_old(double *x, double *y, int pp) { squeeze_entry<2>(x, y, pp); }
__global__ void pllsqueeze_4_pp_old(double *x, double *y, int pp) { squeeze_entry<4>(x, y, pp); }
__global__ void pllsqueeze_8_pp_old(double *x, double *y, int pp) { squeeze_entry<8>(x, y, pp); }
__global__ void pllsqueeze_16_pp_old(double *x, double *y, int pp) { squeeze_entry<16>(x, y, pp); }

// The double-double squeeze on separate partial planes (TCcuda.cu:400, 508,
// 646): entry i of (y1, y2) takes x1[i], x2[i], ... in order through the
// double-double inc_d.  One thread per entry and no bounds check, as in the
// reference: the launch must cover exactly the entries.
template <int Q>
__device__ void squeeze_planes_dd(const double *const (&x)[Q], double *y1, double *y2) {
  const int i = blockDim.x * blockIdx.x + threadIdx.x;
  double acc[2] = {y1[i], y2[i]};
#pragma unroll
  for (int j = 0; j < Q; ++j) mdg::inc_d<2>(acc, x[j][i]);
  y1[i] = acc[0];
  y2[i] = acc[1];
}
__global__ void pllsqueeze_kernel_2_8(double *x1, double *x2, double *x3, double *x4, double *x5,
                                      double *x6, double *x7, double *x8, double *y1,
                                      double *y2) {
  const double *const x[8] = {x1, x2, x3, x4, x5, x6, x7, x8};
  squeeze_planes_dd<8>(x, y1, y2);
}
__global__ void pllsqueeze_kernel_2_12(double *x1, double *x2, double *x3, double *x4, double *x5,
                                       double *x6, double *x7, double *x8, double *x9,
                                       double *x10, double *x11, double *x12, double *y1,
                                       double *y2) {
  const double *const x[12] = {x1, x2, x3, x4, x5, x6, x7, x8, x9, x10, x11, x12};
  squeeze_planes_dd<12>(x, y1, y2);
}
__global__ void pllsqueeze_kernel_2_16(double *x1, double *x2, double *x3, double *x4, double *x5,
                                       double *x6, double *x7, double *x8, double *x9,
                                       double *x10, double *x11, double *x12, double *x13,
                                       double *x14, double *x15, double *x16, double *y1,
                                       double *y2) {
  const double *const x[16] = {x1, x2, x3, x4, x5, x6, x7, x8,
                               x9, x10, x11, x12, x13, x14, x15, x16};
  squeeze_planes_dd<16>(x, y1, y2);
}

// ------------------------------------------------------------------------
// The CPU convolution driver's functions (include/TCcudant.h,
// TCcudant.cpp:163-276): slicing and FP64 plane products on the GPU.

namespace {

// C (pp planes of m x n) = the truncated convolution of A (pp planes of
// m x k) and B (pp planes of k x n) through mdg_plane_conv; zeros if the
// device cannot be used.
vector<double> gpu_plane_conv(const vector<double> &A, const vector<double> &B, int pp, int m,
                              int n, int k) {
  if (pp <= 0 || m < 0 || n < 0 || k < 0) return vector<double>();
  vector<double> C((size_t)pp * m * n, 0.0);
  if (m == 0 || n == 0) return C;
  if (!holds(A, (long long)pp * m * k) || !holds(B, (long long)pp * k * n)) return C;
  DevBuf dA(A.size()), dB(B.size()), dC(C.size());
  if ((A.size() && !dA.p) || (B.size() && !dB.p) || !dC.p) return C;
  if (!to_device(dA.p, A, A.size()) || !to_device(dB.p, B, B.size())) return C;
  if (mdg_plane_conv(pp, m, n, k, dA.p, dB.p, dC.p, nullptr) == MDG_SUCCESS)
    to_host(C, dC.p, C.size());
  return C;
}

}  // namespace

vector<double> zeros(int n, int p) { return vector<double>((size_t)n * n * p, 0.0); }

vector<double> split4pd(vector<double> x) {
  const long long count = (long long)x.size();
  vector<double> out((size_t)count * 4, 0.0);
  if (!count) return out;
  DevBuf dx(x.size()), dout(out.size());
  if (!dx.p || !dout.p || !to_device(dx.p, x, x.size())) return out;
  // one double per entry (P = 1): the slices of each double on its own
  if (mdgi::launch_split(3, 0, 1, count, dx.p, dout.p, 0, 0, nullptr) == MDG_SUCCESS)
    to_host(out, dout.p, out.size());
  return out;
}

vector<double> splitp(vector<double> A, int p) {
  if (p <= 0) return vector<double>();
  const size_t cnt = A.size() / (size_t)p;
  vector<double> out(cnt * (size_t)p);
  for (int i = 0; i < p; ++i)
    for (size_t e = 0; e < cnt; ++e) out[(size_t)i * cnt + e] = A[e * (size_t)p + i];
  return out;
}

void matmul2(vector<double> A, vector<double> B, vector<double> &C, int n) {
  const vector<double> P = gpu_plane_conv(A, B, 1, n, n, n);
  for (size_t i = 0; i < P.size() && i < C.size(); ++i) C[i] += P[i];
}

void convmult2(vector<double> A, vector<double> B, vector<double> &C_aux, int n, int p) {
  if (n < 0 || p <= 0 || !holds(A, nnp(n, p)) || !holds(B, nnp(n, p)) ||
      !holds(C_aux, nnp(n, p) * p))
    return;
  const size_t nn = (size_t)n * n;
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) {
      const vector<double> Ai(A.begin() + i * nn, A.begin() + (i + 1) * nn);
      const vector<double> Bj(B.begin() + j * nn, B.begin() + (j + 1) * nn);
      const vector<double> P = gpu_plane_conv(Ai, Bj, 1, n, n, n);
      double *dst = C_aux.data() + ((size_t)i * p + j) * nn;
      for (size_t e = 0; e < nn; ++e) dst[e] += P[e];
    }
}

void convadd2(vector<double> &C, vector<double> &C_aux, int n, int p) {
  if (n < 0 || p <= 0 || !holds(C, nnp(n, p)) || !holds(C_aux, nnp(n, p) * p)) return;
  const size_t nn = (size_t)n * n;
  for (int i = 0; i < p; ++i)
    for (size_t e = 0; e < nn; ++e)
      for (int j = 0; j <= i; ++j) C[i * nn + e] += C_aux[((size_t)j * p + (i - j)) * nn + e];
}

vector<double> manualconvmult(vector<double> A, vector<double> B, int n, int p) {
  return gpu_plane_conv(A, B, p, n, n, n);
}

void dotconvbutbetter(vector<double> A, vector<double> B, vector<double> &C, int n, int p) {
  const vector<double> P = gpu_plane_conv(A, B, p, n, n, n);
  for (size_t i = 0; i < P.size() && i < C.size(); ++i) C[i] += P[i];
}

vector<double> directdotconv(vector<double> A, vector<double> B, int n, int p) {
  return gpu_plane_conv(A, B, p, n, n, n);
}

// C = op(A) op(B), optionally accumulated into C (mdg_gemm_ex).
//
// The reference's entry points take square, non-transposed operands and
// overwrite C (TCcuda.h:66).  Here an operand given transposed is first
// copied into the workspace by an exact P-double transpose (O(mk) bytes
// against the O(mnk) product: 0.2 % of a quad-double 8192^3 GEMM), the
// product is formed by mdg_gemm of the chosen form, and accumulation adds
// the product to C entry by entry with the reference's P-double addition
// (ddf_add for P = 2, else baileyAdd_fast, quad_double_functions.cu:216).
// So the result is exactly mdg_gemm on the transposed operands, then
// C (+) product.
#include <algorithm>

#include "common.cuh"

namespace {

// out[c][r] = in[r][c] for a rows x cols P-double matrix (leading
// dimensions in entries).  Reads are coalesced along c; each thread writes
// one entry of P contiguous doubles (whole 32-byte sectors for P >= 4).
// Scalar accesses: caller pointers need only be 8-byte aligned.
template <int P>
__global__ void pd_transpose(int rows, int cols, const double *__restrict__ in, int ld_in,
                             double *__restrict__ out, int ld_out) {
  const long long total = (long long)rows * cols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / cols), c = (int)(e - (long long)r * cols);
    const double *src = in + ((size_t)r * ld_in + c) * P;
    double *dst = out + ((size_t)c * ld_out + r) * P;
#pragma unroll
    for (int l = 0; l < P; ++l) dst[l] = src[l];
  }
}

// C[r][c] = C[r][c] (+) T[r][c], the reference's addition for each P:
// ddf_add (double_double_functions.cu) for P = 2, baileyAdd_fast
// (quad_double_functions.cu:216 and the octo / hexa files) otherwise.
template <int P>
__global__ void pd_accumulate(int m, int n, const double *__restrict__ T, int ldt,
                              double *__restrict__ C, int ldc) {
  const long long total = (long long)m * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / n), c = (int)(e - (long long)r * n);
    double *cp = C + ((size_t)r * ldc + c) * P;
    const double *tp = T + ((size_t)r * ldt + c) * P;
    double a[P], b[P], s[P];
#pragma unroll
    for (int l = 0; l < P; ++l) {
      a[l] = cp[l];
      b[l] = tp[l];
    }
    if (P == 2)
      mdg::dd_add(a[0], a[1], b[0], b[1], &s[0], &s[1]);
    else
      mdg::add<P>(a, b, s);
#pragma unroll
    for (int l = 0; l < P; ++l) cp[l] = s[l];
  }
}

unsigned grid_for(long long total, int threads) {
  const long long g = (total + threads - 1) / threads;
  return (unsigned)(g < 4096 ? (g > 0 ? g : 1) : 4096);
}

int launch_transpose(int p, int rows, int cols, const double *in, int ld_in, double *out,
                     int ld_out, cudaStream_t st) {
  const unsigned g = grid_for((long long)rows * cols, 256);
  switch (p) {
    case 2: pd_transpose<2><<<g, 256, 0, st>>>(rows, cols, in, ld_in, out, ld_out); break;
    case 4: pd_transpose<4><<<g, 256, 0, st>>>(rows, cols, in, ld_in, out, ld_out); break;
    case 8: pd_transpose<8><<<g, 256, 0, st>>>(rows, cols, in, ld_in, out, ld_out); break;
    default: pd_transpose<16><<<g, 256, 0, st>>>(rows, cols, in, ld_in, out, ld_out);
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

int launch_accumulate(int p, int m, int n, const double *T, int ldt, double *C, int ldc,
                      cudaStream_t st) {
  const unsigned g = grid_for((long long)m * n, 128);
  switch (p) {
    case 2: pd_accumulate<2><<<g, 128, 0, st>>>(m, n, T, ldt, C, ldc); break;
    case 4: pd_accumulate<4><<<g, 128, 0, st>>>(m, n, T, ldt, C, ldc); break;
    case 8: pd_accumulate<8><<<g, 128, 0, st>>>(m, n, T, ldt, C, ldc); break;
    default: pd_accumulate<16><<<g, 128, 0, st>>>(m, n, T, ldt, C, ldc);
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

// Workspace of mdg_gemm_ex: the inner mdg_gemm's, then op(A), op(B) and the
// product, each 256-byte aligned.
struct ExLayout {
  size_t inner, off_a, off_b, off_t, total;
};

ExLayout ex_layout(size_t inner, int trans_a, int trans_b, int accumulate, int p, int m, int n,
                   int k) {
  ExLayout L;
  L.inner = inner;
  size_t off = mdgi::align_up(inner, 256);
  L.off_a = off;
  if (trans_a) off = mdgi::align_up(off + sizeof(double) * (size_t)m * k * p, 256);
  L.off_b = off;
  if (trans_b) off = mdgi::align_up(off + sizeof(double) * (size_t)k * n * p, 256);
  L.off_t = off;
  if (accumulate) off = mdgi::align_up(off + sizeof(double) * (size_t)m * n * p, 256);
  L.total = off;
  return L;
}

int check_ex(int form, int trans_a, int trans_b, int accumulate, int p, int m, int n, int k,
             int lda, int ldb, int ldc) {
  if (!mdgi::valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (form < MDG_FORM_PLAIN || form > MDG_FORM_FP64_DIGITS) return MDG_ERROR_INVALID_FORM;
  if ((trans_a | trans_b | accumulate) & ~1) return MDG_ERROR_INVALID_FORM;
  if (m < 0 || n < 0 || k < 0) return MDG_ERROR_INVALID_SIZE;
  if (lda < std::max(trans_a ? m : k, 1) || ldb < std::max(trans_b ? k : n, 1) ||
      ldc < std::max(n, 1))
    return MDG_ERROR_INVALID_SIZE;
  return MDG_SUCCESS;
}

}  // namespace

extern "C" {

size_t mdg_gemm_ex_workspace_size(int form, int trans_a, int trans_b, int accumulate, int p,
                                  int m, int n, int k, const mdg_options *opt) {
  const int lda = std::max(trans_a ? m : k, 1), ldb = std::max(trans_b ? k : n, 1);
  if (check_ex(form, trans_a, trans_b, accumulate, p, m, n, k, lda, ldb, std::max(n, 1)) !=
      MDG_SUCCESS)
    return 0;
  const size_t inner = mdg_gemm_workspace_size(form, p, m, n, k, opt);
  if (form != MDG_FORM_PLAIN && inner == 0) return 0;  // options rejected
  return ex_layout(inner, trans_a, trans_b, accumulate, p, m, n, k).total;
}

int mdg_gemm_ex(int form, int trans_a, int trans_b, int accumulate, int p, int m, int n, int k,
                const double *A, int lda, const double *B, int ldb, double *C, int ldc,
                const mdg_options *opt, void *workspace, size_t workspace_bytes,
                void *stream) {
  MDG_TRY(check_ex(form, trans_a, trans_b, accumulate, p, m, n, k, lda, ldb, ldc));
  const size_t inner = mdg_gemm_workspace_size(form, p, m, n, k, opt);
  if (form != MDG_FORM_PLAIN && inner == 0) return MDG_ERROR_INVALID_FORM;
  if (m == 0 || n == 0) return MDG_SUCCESS;  // nothing is read or written
  if (!C || (k > 0 && (!A || !B))) return MDG_ERROR_NULL_POINTER;
  cudaStream_t st = mdgi::as_stream(stream);
  if (k == 0) {  // the product is zero: C is kept (accumulate) or cleared
    if (!accumulate)
      MDG_TRY_CUDA(
          cudaMemset2DAsync(C, sizeof(double) * ldc * p, 0, sizeof(double) * n * p, m, st));
    return MDG_SUCCESS;
  }
  const ExLayout L = ex_layout(inner, trans_a, trans_b, accumulate, p, m, n, k);
  if (L.total > 0 && (!workspace || workspace_bytes < L.total)) return MDG_ERROR_WORKSPACE;
  char *ws = reinterpret_cast<char *>(workspace);
  const double *Aop = A, *Bop = B;
  int lda_op = lda, ldb_op = ldb;
  if (trans_a) {  // stored k x m -> m x k
    double *At = reinterpret_cast<double *>(ws + L.off_a);
    MDG_TRY(launch_transpose(p, k, m, A, lda, At, k, st));
    Aop = At;
    lda_op = k;
  }
  if (trans_b) {  // stored n x k -> k x n
    double *Bt = reinterpret_cast<double *>(ws + L.off_b);
    MDG_TRY(launch_transpose(p, n, k, B, ldb, Bt, n, st));
    Bop = Bt;
    ldb_op = n;
  }
  double *Cout = accumulate ? reinterpret_cast<double *>(ws + L.off_t) : C;
  const int ldc_out = accumulate ? n : ldc;
  MDG_TRY(mdg_gemm(form, p, m, n, k, Aop, lda_op, Bop, ldb_op, Cout, ldc_out, opt,
                   inner ? ws : nullptr, inner, stream));
  if (accumulate) MDG_TRY(launch_accumulate(p, m, n, Cout, n, C, ldc, st));
  return MDG_SUCCESS;
}

}  // extern "C"

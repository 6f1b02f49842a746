// The slice-digit GEMM for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc at all: code that runs while a CUDA
// graph is being captured by someone else, plug-in hosts that own every
// device allocation and hand out only the operand buffers, and real-time
// or embedded integrations that forbid allocation after start-up.
// mdg_gemm_slice_static serves them: it takes only the operands and uses a
// scratch array of fixed size compiled into this library instead of a
// caller-supplied workspace.
//
// The array is a file-scope __device__ variable, so every GPU on which the
// library is loaded holds its kStaticScratchBytes until the process exits.
// Host code cannot use the array's name as a device address; the first call
// on each device looks the address up with cudaGetSymbolAddress (with that
// device current) and caches it, so that first call should come before any
// stream capture.  All calls share the array and it keeps the previous
// call's contents: every region the pipeline reads is written first (the
// row / column maxima are cleared, digit planes are written in full
// including padding, every chunk plane is written by the diagonal GEMM), and
// calls that overlap on the GPU race on the array, so a caller must order
// them (one stream, or events).
#include <mutex>

#include "common.cuh"
#include "slice_tc.cuh"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device with that device current).
int scratch_address(void **out) {
  int dev = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return MDG_ERROR_NOT_SUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    MDG_TRY_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return MDG_SUCCESS;
}

}  // namespace

extern "C" {

size_t mdg_static_scratch_bytes(void) { return kStaticScratchBytes; }

int mdg_gemm_slice_static(int p, int m, int n, int k, const double *A, int lda, const double *B,
                          int ldb, double *C, int ldc, void *stream) {
  if (!mdgi::valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (m < 0 || n < 0 || k < 0 || lda < std::max(k, 1) || ldb < std::max(n, 1) ||
      ldc < std::max(n, 1))
    return MDG_ERROR_INVALID_SIZE;
  if (m == 0 || n == 0) return MDG_SUCCESS;
  if (!C || (k > 0 && (!A || !B))) return MDG_ERROR_NULL_POINTER;
  const int s = mdg_default_slices(p);
  const mdgi::SlicePlan pl = mdgi::make_slice_plan(p, s, s, m, n, k);
  if (pl.total > kStaticScratchBytes || pl.Mp > 65535 || pl.Np > 65535)
    return MDG_ERROR_TOO_LARGE;
  cudaStream_t st = mdgi::as_stream(stream);
  if (k == 0) {
    MDG_TRY_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc * p, 0, sizeof(double) * n * p, m, st));
    return MDG_SUCCESS;
  }
  void *scratch = nullptr;
  MDG_TRY(scratch_address(&scratch));
  return mdgi::run_slice_gemm(pl, A, lda, B, ldb, C, ldc, scratch, mdgi::engine_choice(0), 0, 0,
                              st);
}

}  // extern "C"

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
// in each CUDA context (normally the device's primary context) looks the
// address up with cudaGetSymbolAddress, with that context current, and
// caches it under the context's unique id, so that first call should come
// before any stream capture.  A context created later (after
// cudaDeviceReset, or a driver-API context the caller makes current) has its
// own id and gets its own lookup.  All calls share the array and it keeps
// the previous call's contents: every region the pipeline reads is written
// first (the row / column maxima are cleared, digit planes are written in
// full including padding, every chunk plane is written by the diagonal
// GEMM), and calls that overlap on the GPU race on the array, so a caller
// must order them (one stream, or events).
#include <cuda.h>

#include <mutex>

#include "common.cuh"
#include "slice_tc.cuh"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kMaxContexts = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

template <typename Fn>
Fn driver_entry(const char *name, int version) {
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    return reinterpret_cast<Fn>(p);
  return nullptr;
}

// Unique id of the current context (0 when none is current yet).
int current_context_id(unsigned long long *id) {
  static const CtxGetCurrentFn get_current = driver_entry<CtxGetCurrentFn>("cuCtxGetCurrent", 4000);
  static const CtxGetIdFn get_id = driver_entry<CtxGetIdFn>("cuCtxGetId", 12000);
  if (!get_current || !get_id) return MDG_ERROR_NOT_SUPPORTED;
  CUcontext ctx = nullptr;
  *id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS) return MDG_ERROR_CUDA;
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return MDG_ERROR_CUDA;
  return MDG_SUCCESS;
}

std::mutex g_mu;
struct Entry {
  unsigned long long ctx;
  void *ptr;
};
Entry g_entries[kMaxContexts] = {};
int g_next = 0;

// Device address of the scratch array in the current context.
int scratch_address(void **out) {
  unsigned long long id = 0;
  MDG_TRY(current_context_id(&id));
  std::lock_guard<std::mutex> lk(g_mu);
  if (id)
    for (const Entry &e : g_entries)
      if (e.ctx == id) {
        *out = e.ptr;
        return MDG_SUCCESS;
      }
  // first call in this context: the runtime call below also makes the
  // device's primary context current when no context was
  void *p = nullptr;
  MDG_TRY_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
  MDG_TRY(current_context_id(&id));
  if (!id) return MDG_ERROR_CUDA;
  g_entries[g_next] = Entry{id, p};
  g_next = (g_next + 1) % kMaxContexts;
  *out = p;
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

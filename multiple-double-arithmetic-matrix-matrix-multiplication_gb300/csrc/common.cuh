// Shared helpers of the CUDA sources: status plumbing, launch checks.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "mdg_arith.h"
#include "mdgemm.h"

namespace mdgi {

// Records the text of a failed CUDA call for mdg_last_cuda_error().
void set_cuda_error(cudaError_t e);

inline bool valid_p(int p) { return p == 2 || p == 4 || p == 8 || p == 16; }

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// An NVTX range for the scope (host side): names the stages of a GEMM in
// profiler timelines and lets ncu select them (--nvtx --nvtx-include).
// Without a tool attached the calls return at once.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Host-side fault injection: with MDG_ALLOC_LIMIT_BYTES set, every device
// allocation the library makes for itself (the host-entry cache, plans)
// larger than that many bytes fails with MDG_ERROR_ALLOCATION, before any
// CUDA call (a simulated out-of-memory; nothing is asked of the device).
bool alloc_over_limit(size_t bytes);

}  // namespace mdgi

#define MDG_TRY_CUDA(call)                        \
  do {                                            \
    cudaError_t mdg_e_ = (call);                  \
    if (mdg_e_ != cudaSuccess) {                  \
      mdgi::set_cuda_error(mdg_e_);               \
      return MDG_ERROR_CUDA;                      \
    }                                             \
  } while (0)

#define MDG_TRY_LAUNCH() MDG_TRY_CUDA(cudaGetLastError())

#define MDG_TRY(call)                    \
  do {                                   \
    int mdg_s_ = (call);                 \
    if (mdg_s_ != MDG_SUCCESS) return mdg_s_; \
  } while (0)

// Internal launchers (one translation unit each); all return mdg_status.
namespace mdgi {
int launch_plain_gemm(int p, int m, int n, int k, const double *A, int lda, const double *B,
                      int ldb, double *C, int ldc, cudaStream_t st);
int launch_plain_batched(const mdg_problem *dev_problems, int count, int max_p,
                         const int *dev_tile_starts, int total_tiles, cudaStream_t st);
int launch_split(int kind, int exact, int p, long long count, const double *x, double *out,
                 int soa, long long plane_stride, cudaStream_t st);
int launch_squeeze(int p, int pp, long long count, const double *x, long long x_stride,
                   long long x_plane, double *y, cudaStream_t st);
// planes = 0: AoS (m x k x pp, ...); 1: pp slice planes of m x k, k x n, m x n
int launch_slice_conv(int pp, int m, int n, int k, const double *Aq, const double *Bq,
                      double *Cq, int planes, cudaStream_t st);
}  // namespace mdgi

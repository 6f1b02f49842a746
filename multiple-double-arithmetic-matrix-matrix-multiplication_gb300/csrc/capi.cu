// The C ABI (include/mdgemm.h): argument checks, workspace layout, form
// dispatch, the host-buffer entry and the batched entry.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "slice_tc.cuh"

namespace mdgi {

static thread_local char g_cuda_error[256] = "";

void set_cuda_error(cudaError_t e) {
  std::snprintf(g_cuda_error, sizeof g_cuda_error, "%s: %s", cudaGetErrorName(e),
                cudaGetErrorString(e));
}

int default_engine() {
  const char *v = std::getenv("MDG_SLICE_ENGINE");
  if (v && *v) return std::atoi(v) ? 1 : 0;
  return 1;
}

// Option value -> engine code of run_slice_gemm: 0 mma.sync, 1 tcgen05
// (auto tile shape), 2 tcgen05 single CTA, 3 tcgen05 CTA pairs.  The
// MDG_SLICE_ENGINE / MDG_TC_PAIR environment variables override "auto".
int engine_choice(int opt) {
  switch (opt) {
    case 1: return 2;
    case 2: return 3;
    case 3: return 0;
  }
  if (default_engine() == 0) return 0;
  const char *pv = std::getenv("MDG_TC_PAIR");
  if (pv && *pv == '0') return 2;
  return 1;
}

bool alloc_over_limit(size_t bytes) {
  const char *e = std::getenv("MDG_ALLOC_LIMIT_BYTES");
  if (!e || !*e) return false;
  return bytes > std::strtoull(e, nullptr, 10);
}

// ------------------------------------------------------------------ cache --
// Grow-only device buffers owned by the library, for calls that take no
// workspace argument (mdg_gemm_host, mdg_scale_exponents).  One per slot.
// The buffers, streams and events belong to one device; a call on another
// device releases them first.
constexpr int kMaxPanels = 4, kMaxStrips = 2;
struct DeviceCache {
  std::mutex mu;
  int dev = -1;
  // A, B, C, then one workspace per column strip of the host entry
  void *ptr[3 + kMaxStrips] = {};
  size_t cap[3 + kMaxStrips] = {};
  cudaStream_t streams[3] = {nullptr, nullptr, nullptr};  // compute, copies in, copies out
  // start, B strips in, A panels in, C blocks done
  cudaEvent_t events[1 + kMaxStrips + kMaxPanels + kMaxPanels * kMaxStrips] = {};
  // caller holds mu
  int bind_device() {
    int d = 0;
    MDG_TRY_CUDA(cudaGetDevice(&d));
    if (d != dev) {
      release_locked();
      dev = d;
    }
    return MDG_SUCCESS;
  }
  int make_streams() {
    for (auto &st : streams)
      if (!st) MDG_TRY_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (auto &ev : events)
      if (!ev) MDG_TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    return MDG_SUCCESS;
  }
  void release_locked() {
    for (int i = 0; i < 3 + kMaxStrips; ++i) {
      if (ptr[i]) cudaFree(ptr[i]);
      ptr[i] = nullptr;
      cap[i] = 0;
    }
    for (auto &st : streams) {
      if (st) cudaStreamDestroy(st);
      st = nullptr;
    }
    for (auto &ev : events) {
      if (ev) cudaEventDestroy(ev);
      ev = nullptr;
    }
  }
  int get(int slot, size_t bytes, void **out) {
    if (bytes == 0) bytes = 256;
    if (alloc_over_limit(bytes)) return MDG_ERROR_ALLOCATION;
    if (cap[slot] < bytes) {
      if (ptr[slot]) cudaFree(ptr[slot]);
      ptr[slot] = nullptr;
      cap[slot] = 0;
      cudaError_t e = cudaMalloc(&ptr[slot], bytes);
      if (e != cudaSuccess) {
        set_cuda_error(e);
        return MDG_ERROR_ALLOCATION;
      }
      cap[slot] = bytes;
    }
    *out = ptr[slot];
    return MDG_SUCCESS;
  }
  void release() {
    std::lock_guard<std::mutex> lk(mu);
    release_locked();
    dev = -1;
  }
};
static DeviceCache g_cache;

// ---------------------------------------------------------------- checks --
static int check_gemm_args(int form, int p, int m, int n, int k, const void *A, int lda,
                           const void *B, int ldb, const void *C, int ldc) {
  if (form < MDG_FORM_PLAIN || form > MDG_FORM_FP64_DIGITS) return MDG_ERROR_INVALID_FORM;
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (m < 0 || n < 0 || k < 0) return MDG_ERROR_INVALID_SIZE;
  if (lda < std::max(k, 1) || ldb < std::max(n, 1) || ldc < std::max(n, 1))
    return MDG_ERROR_INVALID_SIZE;
  if (m == 0 || n == 0) return MDG_SUCCESS;  // nothing is read or written
  if (!C || (k > 0 && (!A || !B))) return MDG_ERROR_NULL_POINTER;
  return MDG_SUCCESS;
}

struct Opts {
  int slices, diagonals, split_kind, split_exact, engine, parts, raster, pace;
};

// Options with the defaults filled in; the digit count and its limits
// depend on the form (8-bit digits for the BF16 form, 19-bit for FP64).
static int resolve_opts(int form, int p, const mdg_options *o, Opts *r) {
  const bool d64 = form == MDG_FORM_FP64_DIGITS;
  r->slices = (o && o->slices) ? o->slices : d64 ? digits64_default(p) : mdg_default_slices(p);
  r->diagonals = (o && o->diagonals) ? o->diagonals : r->slices;
  r->split_kind = o ? o->split_kind : 0;
  if (o && (o->split_exact < 0 || o->split_exact > 2)) return MDG_ERROR_INVALID_FORM;
  r->split_exact = (o && o->split_exact == 2) ? 0 : 1;
  r->engine = o ? o->engine : 0;
  r->parts = o ? o->parts : 0;
  r->raster = o ? o->raster : 0;
  r->pace = o ? o->pace : 0;
  if (r->engine < 0 || r->engine > 3 || r->parts < 0 || r->parts > 8 || r->raster < 0 ||
      r->pace < -1 || r->pace > 65536)
    return MDG_ERROR_INVALID_FORM;
  if (r->slices < 1 || r->slices > 128) return MDG_ERROR_INVALID_FORM;
  if (r->diagonals < 1 || r->diagonals > 2 * r->slices - 1) return MDG_ERROR_INVALID_FORM;
  if (r->split_kind < 0 || r->split_kind > 2) return MDG_ERROR_INVALID_FORM;
  if (r->split_kind == 2 && p != 2) return MDG_ERROR_INVALID_LIMBS;
  if (!(d64 ? words64_for(r->slices, r->diagonals) : words_for(r->slices, r->diagonals)))
    return MDG_ERROR_NOT_SUPPORTED;
  return MDG_SUCCESS;
}

static int split_pp(int kind, int p) { return kind == 0 ? 4 * p : kind == 1 ? 8 * p : 12; }

// FP64 split form workspace: packed A/B (when strided), slices, partials,
// packed C (when strided).
struct SplitPlan {
  int pp;
  size_t off_Ap, off_Bp, off_Aq, off_Bq, off_Cq, off_Cp, total;
};

static SplitPlan make_split_plan(int p, int kind, int m, int n, int k) {
  SplitPlan s{};
  s.pp = split_pp(kind, p);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  s.off_Ap = take(sizeof(double) * (size_t)m * k * p);
  s.off_Bp = take(sizeof(double) * (size_t)k * n * p);
  s.off_Aq = take(sizeof(double) * (size_t)m * k * s.pp);
  s.off_Bq = take(sizeof(double) * (size_t)k * n * s.pp);
  s.off_Cq = take(sizeof(double) * (size_t)m * n * s.pp);
  s.off_Cp = take(sizeof(double) * (size_t)m * n * p);
  s.total = off;
  return s;
}

static int run_split_gemm(int p, const Opts &o, int m, int n, int k, const double *A, int lda,
                          const double *B, int ldb, double *C, int ldc, void *ws,
                          cudaStream_t st) {
  const SplitPlan sp = make_split_plan(p, o.split_kind, m, n, k);
  char *base = reinterpret_cast<char *>(ws);
  const double *Ac = A, *Bc = B;
  if (lda != k && m > 0 && k > 0) {
    double *Ap = reinterpret_cast<double *>(base + sp.off_Ap);
    MDG_TRY_CUDA(cudaMemcpy2DAsync(Ap, sizeof(double) * k * p, A, sizeof(double) * lda * p,
                                   sizeof(double) * k * p, m, cudaMemcpyDeviceToDevice, st));
    Ac = Ap;
  }
  if (ldb != n && k > 0 && n > 0) {
    double *Bp = reinterpret_cast<double *>(base + sp.off_Bp);
    MDG_TRY_CUDA(cudaMemcpy2DAsync(Bp, sizeof(double) * n * p, B, sizeof(double) * ldb * p,
                                   sizeof(double) * n * p, k, cudaMemcpyDeviceToDevice, st));
    Bc = Bp;
  }
  double *Aq = reinterpret_cast<double *>(base + sp.off_Aq);
  double *Bq = reinterpret_cast<double *>(base + sp.off_Bq);
  double *Cq = reinterpret_cast<double *>(base + sp.off_Cq);
  NvtxRange range("mdg fp64split");
  MDG_TRY(launch_split(o.split_kind, o.split_exact, p, (long long)m * k, Ac, Aq, 0, 0, st));
  MDG_TRY(launch_split(o.split_kind, o.split_exact, p, (long long)k * n, Bc, Bq, 0, 0, st));
  MDG_TRY(launch_slice_conv(sp.pp, m, n, k, Aq, Bq, Cq, 0, st));
  double *Cout = (ldc == n) ? C : reinterpret_cast<double *>(base + sp.off_Cp);
  MDG_TRY(launch_squeeze(p, sp.pp, (long long)m * n, Cq, sp.pp, 1, Cout, st));
  if (ldc != n && m > 0 && n > 0) {
    MDG_TRY_CUDA(cudaMemcpy2DAsync(C, sizeof(double) * ldc * p, Cout, sizeof(double) * n * p,
                                   sizeof(double) * n * p, m, cudaMemcpyDeviceToDevice, st));
  }
  return MDG_SUCCESS;
}

static size_t workspace_bytes(int form, int p, int m, int n, int k, const Opts &o) {
  if (form == MDG_FORM_PLAIN) return 0;
  if (form == MDG_FORM_FP64_SPLIT) return make_split_plan(p, o.split_kind, m, n, k).total;
  if (form == MDG_FORM_FP64_DIGITS) return make_digits64_plan(p, o.slices, o.diagonals, m, n, k).total;
  return make_slice_plan(p, o.slices, o.diagonals, m, n, k).total;
}

}  // namespace mdgi

using namespace mdgi;

// mdg_gemm_host for the BF16 form on tall problems: C is computed in blocks
// of row panels of A (up to four) by column strips of B (two when n >=
// 4096).  The first block waits only for the first strip of B and the
// first panel of A; the other strips and panels are copied in on one copy
// stream while earlier blocks compute (each strip's exponents and digits
// are computed once, each panel's once), and every finished block of C goes
// back on a second copy stream, so most of the host-link traffic hides
// behind the tensor-core work.  Bits as one mdg_gemm (slice_panel_a,
// slice_block).  The work starts after everything queued before it on the
// legacy default stream and the blocking streams, as the single-stream
// path would.
static int host_slice_panels_issue(int p, const Opts &o, int m, int n, int k, const double *A,
                                   const double *B, double *C, double *dA, double *dB,
                                   double *dC);

static int host_slice_panels(int p, const Opts &o, int m, int n, int k, const double *A,
                             const double *B, double *C, double *dA, double *dB, double *dC) {
  const int st = host_slice_panels_issue(p, o, m, n, k, A, B, C, dA, dB, dC);
  if (st != MDG_SUCCESS)
    // copies into the caller's host buffers may still be queued: let them
    // finish before returning, so that the caller may free the buffers
    for (cudaStream_t s : g_cache.streams)
      if (s) cudaStreamSynchronize(s);
  return st;
}

static int host_slice_panels_issue(int p, const Opts &o, int m, int n, int k, const double *A,
                                   const double *B, double *C, double *dA, double *dB,
                                   double *dC) {
  NvtxRange range("mdg host: B strips and A panels overlapped");
  const int want = std::min(kMaxPanels, m / 1024);
  const int mp = (int)align_up((m + want - 1) / want, 256);
  const int panels = (m + mp - 1) / mp;
  // strips of ns columns (a multiple of 256); with two strips and n >= 4096
  // the last one holds at least n / 2 - 255 columns
  const int strips = n >= 4096 ? kMaxStrips : 1;
  const int ns = strips > 1 ? (int)align_up((n + strips - 1) / strips, 256) : n;
  SlicePlan pls[kMaxStrips];
  void *ws[kMaxStrips] = {};
  for (int j = 0; j < strips; ++j) {
    pls[j] = make_slice_plan(p, o.slices, o.diagonals, mp, std::min(ns, n - j * ns), k);
    if (pls[j].Mp > 65535 || pls[j].Np > 65535) return MDG_ERROR_NOT_SUPPORTED;
    MDG_TRY(g_cache.get(3 + j, pls[j].total, &ws[j]));
  }
  MDG_TRY(g_cache.make_streams());
  cudaStream_t sc = g_cache.streams[0], si = g_cache.streams[1], so = g_cache.streams[2];
  cudaEvent_t ev0 = g_cache.events[0];
  cudaEvent_t *evB = g_cache.events + 1, *evA = evB + kMaxStrips, *evC = evA + kMaxPanels;
  const size_t ea = (size_t)k * p, ec = (size_t)n * p;  // doubles per row of A / of B and C
  const size_t row_a = sizeof(double) * ea, pitch = sizeof(double) * ec;
  MDG_TRY_CUDA(cudaEventRecord(ev0, 0));
  MDG_TRY_CUDA(cudaStreamWaitEvent(si, ev0, 0));
  MDG_TRY_CUDA(cudaStreamWaitEvent(sc, ev0, 0));
  // copies in, in the order the blocks need them: strip 0 of B, panel 0 of
  // A, the other strips, then (in the loop) the next panel of A
  auto copy_strip = [&](int j) -> int {
    const size_t c0 = (size_t)j * ns * p;
    MDG_TRY_CUDA(cudaMemcpy2DAsync(dB + c0, pitch, B + c0, pitch,
                                   sizeof(double) * (size_t)pls[j].n * p, k,
                                   cudaMemcpyHostToDevice, si));
    MDG_TRY_CUDA(cudaEventRecord(evB[j], si));
    return MDG_SUCCESS;
  };
  MDG_TRY(copy_strip(0));
  MDG_TRY_CUDA(cudaMemcpyAsync(dA, A, row_a * std::min(mp, m), cudaMemcpyHostToDevice, si));
  MDG_TRY_CUDA(cudaEventRecord(evA[0], si));
  for (int j = 1; j < strips; ++j) MDG_TRY(copy_strip(j));
  MDG_TRY_CUDA(cudaStreamWaitEvent(sc, evB[0], 0));
  MDG_TRY(slice_prepare_b(pls[0], dB, n, ws[0], sc));
  const int engine = engine_choice(o.engine);
  for (int i = 0; i < panels; ++i) {
    const int r0 = i * mp, rows = std::min(mp, m - r0);
    if (i + 1 < panels) {
      const int r1 = r0 + mp, rows1 = std::min(mp, m - r1);
      MDG_TRY_CUDA(cudaMemcpyAsync(dA + r1 * ea, A + r1 * ea, row_a * rows1,
                                   cudaMemcpyHostToDevice, si));
      MDG_TRY_CUDA(cudaEventRecord(evA[i + 1], si));
    }
    MDG_TRY_CUDA(cudaStreamWaitEvent(sc, evA[i], 0));
    // the panel's exponents and digits live in strip 0's workspace
    MDG_TRY(slice_panel_a(pls[0], rows, dA + r0 * ea, k, ws[0], sc));
    for (int j = 0; j < strips; ++j) {
      if (i == 0 && j > 0) {
        MDG_TRY_CUDA(cudaStreamWaitEvent(sc, evB[j], 0));
        MDG_TRY(slice_prepare_b(pls[j], dB + (size_t)j * ns * p, n, ws[j], sc));
      }
      const size_t off = r0 * ec + (size_t)j * ns * p;
      MDG_TRY(slice_block(pls[0], ws[0], pls[j], ws[j], rows, dC + off, n, engine, o.parts,
                          o.raster, sc, o.pace));
      cudaEvent_t done = evC[i * kMaxStrips + j];
      MDG_TRY_CUDA(cudaEventRecord(done, sc));
      MDG_TRY_CUDA(cudaStreamWaitEvent(so, done, 0));
      MDG_TRY_CUDA(cudaMemcpy2DAsync(C + off, pitch, dC + off, pitch,
                                     sizeof(double) * (size_t)pls[j].n * p, rows,
                                     cudaMemcpyDeviceToHost, so));
    }
  }
  MDG_TRY_CUDA(cudaStreamSynchronize(si));
  MDG_TRY_CUDA(cudaStreamSynchronize(sc));
  MDG_TRY_CUDA(cudaStreamSynchronize(so));
  return MDG_SUCCESS;
}

extern "C" {

const char *mdg_status_string(int status) {
  switch (status) {
    case MDG_SUCCESS: return "success";
    case MDG_ERROR_INVALID_LIMBS: return "invalid limb count (P must be 2, 4, 8 or 16)";
    case MDG_ERROR_INVALID_SIZE: return "invalid size or leading dimension";
    case MDG_ERROR_NULL_POINTER: return "null pointer";
    case MDG_ERROR_INVALID_FORM: return "invalid form or option";
    case MDG_ERROR_WORKSPACE: return "workspace missing or too small";
    case MDG_ERROR_CUDA: return "CUDA error";
    case MDG_ERROR_NOT_SUPPORTED: return "not supported";
    case MDG_ERROR_TIMEOUT: return "device wait timed out";
    case MDG_ERROR_ALLOCATION: return "allocation failed";
    case MDG_ERROR_TOO_LARGE: return "problem exceeds the fixed scratch of the allocation-free entry";
  }
  return "unknown status";
}

const char *mdg_last_cuda_error(void) { return g_cuda_error; }

int mdg_version(void) { return 100; }

int mdg_default_fp64_digits(int p) { return digits64_default(p); }

int mdg_default_slices(int p) {
  switch (p) {
    case 2: return 14;
    case 4: return 28;
    case 8: return 55;
    case 16: return 110;  /* 879 bits: above the plain hexa-double GEMM's ~870 */
  }
  return 0;
}

size_t mdg_gemm_workspace_size(int form, int p, int m, int n, int k, const mdg_options *opt) {
  Opts o;
  if (!valid_p(p) || m < 0 || n < 0 || k < 0) return 0;
  if (resolve_opts(form, p, opt, &o) != MDG_SUCCESS) return 0;
  return workspace_bytes(form, p, m, n, k, o);
}

int mdg_gemm(int form, int p, int m, int n, int k, const double *A, int lda, const double *B,
             int ldb, double *C, int ldc, const mdg_options *opt, void *workspace,
             size_t workspace_bytes_, void *stream) {
  MDG_TRY(check_gemm_args(form, p, m, n, k, A, lda, B, ldb, C, ldc));
  Opts o;
  MDG_TRY(resolve_opts(form, p, opt, &o));
  cudaStream_t st = as_stream(stream);
  if (m == 0 || n == 0) return MDG_SUCCESS;
  if (k == 0) {  // empty sum: C = 0
    MDG_TRY_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc * p, 0, sizeof(double) * n * p, m, st));
    return MDG_SUCCESS;
  }
  if (form == MDG_FORM_PLAIN) {
    NvtxRange range("mdg plain");
    return launch_plain_gemm(p, m, n, k, A, lda, B, ldb, C, ldc, st);
  }
  const size_t need = workspace_bytes(form, p, m, n, k, o);
  if (!workspace || workspace_bytes_ < need) return MDG_ERROR_WORKSPACE;
  if (form == MDG_FORM_FP64_SPLIT)
    return run_split_gemm(p, o, m, n, k, A, lda, B, ldb, C, ldc, workspace, st);
  if (form == MDG_FORM_FP64_DIGITS)
    return run_digits64_gemm(make_digits64_plan(p, o.slices, o.diagonals, m, n, k), A, lda, B,
                             ldb, C, ldc, workspace, st);
  const SlicePlan pl = make_slice_plan(p, o.slices, o.diagonals, m, n, k);
  if (pl.Mp > 65535 || pl.Np > 65535) return MDG_ERROR_NOT_SUPPORTED;
  return run_slice_gemm(pl, A, lda, B, ldb, C, ldc, workspace, engine_choice(o.engine), o.parts,
                        o.raster, st, o.pace);
}

int mdg_gemm_host(int form, int p, int m, int n, int k, const double *A, const double *B,
                  double *C, const mdg_options *opt) {
  MDG_TRY(check_gemm_args(form, p, m, n, k, A, std::max(k, 1), B, std::max(n, 1), C,
                          std::max(n, 1)));
  Opts o;
  MDG_TRY(resolve_opts(form, p, opt, &o));
  if (m == 0 || n == 0) return MDG_SUCCESS;
  const size_t sa = sizeof(double) * (size_t)m * k * p, sb = sizeof(double) * (size_t)k * n * p,
               sc = sizeof(double) * (size_t)m * n * p;
  if (alloc_over_limit(sa) || alloc_over_limit(sb) || alloc_over_limit(sc) ||
      alloc_over_limit(workspace_bytes(form, p, m, n, k, o)))
    return MDG_ERROR_ALLOCATION;
  std::lock_guard<std::mutex> lk(g_cache.mu);
  MDG_TRY(g_cache.bind_device());
  void *dA, *dB, *dC, *ws = nullptr;
  MDG_TRY(g_cache.get(0, sa, &dA));
  MDG_TRY(g_cache.get(1, sb, &dB));
  MDG_TRY(g_cache.get(2, sc, &dC));
  if (form == MDG_FORM_SLICE_BF16 && k > 0 && m >= 2048)
    return host_slice_panels(p, o, m, n, k, A, B, C, (double *)dA, (double *)dB, (double *)dC);
  const size_t need = workspace_bytes(form, p, m, n, k, o);
  if (need) MDG_TRY(g_cache.get(3, need, &ws));
  cudaStream_t st = 0;
  if (sa) MDG_TRY_CUDA(cudaMemcpyAsync(dA, A, sa, cudaMemcpyHostToDevice, st));
  if (sb) MDG_TRY_CUDA(cudaMemcpyAsync(dB, B, sb, cudaMemcpyHostToDevice, st));
  MDG_TRY(mdg_gemm(form, p, m, n, k, (const double *)dA, std::max(k, 1), (const double *)dB, n,
                   (double *)dC, n, opt, ws, need, st));
  MDG_TRY_CUDA(cudaMemcpyAsync(C, dC, sc, cudaMemcpyDeviceToHost, st));
  MDG_TRY_CUDA(cudaStreamSynchronize(st));
  return MDG_SUCCESS;
}

void mdg_release_cache(void) { g_cache.release(); }

int mdg_host_alloc(size_t bytes, void **out) {
  if (!out) return MDG_ERROR_NULL_POINTER;
  *out = nullptr;
  if (alloc_over_limit(bytes)) return MDG_ERROR_ALLOCATION;
  cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    set_cuda_error(e);
    *out = nullptr;
    return MDG_ERROR_ALLOCATION;
  }
  return MDG_SUCCESS;
}

void mdg_host_free(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
}

// ---------------------------------------------------------------- batched --

size_t mdg_gemm_batched_workspace_size(int form, const mdg_problem *problems, int count,
                                       const mdg_options *opt) {
  if (!problems || count < 0) return 0;
  size_t total = align_up(sizeof(mdg_problem) * (size_t)count, 256) +
                 align_up(sizeof(int) * (size_t)(count + 1), 256);
  if (form == MDG_FORM_PLAIN) return total;
  if (form == MDG_FORM_SLICE_BF16) {
    std::vector<mdg_problem> live;
    for (int i = 0; i < count; ++i)
      if (problems[i].m > 0 && problems[i].n > 0 && problems[i].k > 0) live.push_back(problems[i]);
    return live.empty() ? 0 : mdg_batch_workspace_size(live.data(), (int)live.size());
  }
  size_t mx = 0;
  for (int i = 0; i < count; ++i) {
    const mdg_problem &q = problems[i];
    mx = std::max(mx, mdg_gemm_workspace_size(form, q.p, q.m, q.n, q.k, opt));
  }
  return total + mx;
}

int mdg_gemm_batched(int form, const mdg_problem *problems, int count, const mdg_options *opt,
                     void *workspace, size_t wsb, void *stream) {
  if (count < 0) return MDG_ERROR_INVALID_SIZE;
  if (count == 0) return MDG_SUCCESS;
  if (!problems) return MDG_ERROR_NULL_POINTER;
  int max_p = 2;
  for (int i = 0; i < count; ++i) {
    const mdg_problem &q = problems[i];
    MDG_TRY(check_gemm_args(form, q.p, q.m, q.n, q.k, q.A, q.lda, q.B, q.ldb, q.C, q.ldc));
    max_p = std::max(max_p, q.p);
  }
  const size_t need = mdg_gemm_batched_workspace_size(form, problems, count, opt);
  if (!workspace || wsb < need) return MDG_ERROR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  char *base = reinterpret_cast<char *>(workspace);
  if (form == MDG_FORM_PLAIN) {
    std::vector<int> starts(count + 1, 0);
    for (int i = 0; i < count; ++i) {
      const mdg_problem &q = problems[i];
      const long long tiles = (q.k == 0) ? 0 : (long long)((q.m + 15) / 16) * ((q.n + 15) / 16);
      starts[i + 1] = starts[i] + (int)tiles;
    }
    for (int i = 0; i < count; ++i)
      if (problems[i].k == 0 && problems[i].m > 0 && problems[i].n > 0)
        MDG_TRY_CUDA(cudaMemset2DAsync(problems[i].C, sizeof(double) * problems[i].ldc * problems[i].p,
                                       0, sizeof(double) * problems[i].n * problems[i].p,
                                       problems[i].m, st));
    auto *dprobs = reinterpret_cast<mdg_problem *>(base);
    auto *dstarts =
        reinterpret_cast<int *>(base + align_up(sizeof(mdg_problem) * (size_t)count, 256));
    // the table travels with the launch stream: pinned staging would need a
    // host allocation, so the copy waits for the host data to be read
    MDG_TRY_CUDA(cudaMemcpyAsync(dprobs, problems, sizeof(mdg_problem) * count,
                                 cudaMemcpyHostToDevice, st));
    MDG_TRY_CUDA(cudaMemcpyAsync(dstarts, starts.data(), sizeof(int) * (count + 1),
                                 cudaMemcpyHostToDevice, st));
    MDG_TRY_CUDA(cudaStreamSynchronize(st));
    return launch_plain_batched(dprobs, count, max_p, dstarts, starts[count], st);
  }
  if (form == MDG_FORM_SLICE_BF16) {
    // empty problems: nothing (m or n = 0) or C = 0 (k = 0); the plan takes the rest
    std::vector<mdg_problem> live;
    for (int i = 0; i < count; ++i) {
      const mdg_problem &q = problems[i];
      if (q.m == 0 || q.n == 0) continue;
      if (q.k == 0) {
        MDG_TRY_CUDA(cudaMemset2DAsync(q.C, sizeof(double) * q.ldc * q.p, 0,
                                       sizeof(double) * q.n * q.p, q.m, st));
        continue;
      }
      live.push_back(q);
    }
    if (live.empty()) return MDG_SUCCESS;
    mdg_batch b = nullptr;
    MDG_TRY(mdg_batch_create(live.data(), (int)live.size(), workspace, wsb, stream, &b));
    const int st2 = mdg_batch_run(b, stream);
    mdg_batch_destroy(b);
    return st2;
  }
  // FP64 split form: the stages of each problem in turn on one stream,
  // sharing the largest workspace
  void *ws = base + align_up(sizeof(mdg_problem) * (size_t)count, 256) +
             align_up(sizeof(int) * (size_t)(count + 1), 256);
  const size_t wsz = need - (static_cast<char *>(ws) - base);
  for (int i = 0; i < count; ++i) {
    const mdg_problem &q = problems[i];
    MDG_TRY(mdg_gemm(form, q.p, q.m, q.n, q.k, q.A, q.lda, q.B, q.ldb, q.C, q.ldc, opt, ws, wsz,
                     stream));
  }
  return MDG_SUCCESS;
}

// ------------------------------------------------------- stage entries --

int mdg_split(int kind, int exact, int p, long long count, const double *x, double *out,
              void *stream) {
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (kind < 0 || kind > 3 || (exact != 0 && exact != 1)) return MDG_ERROR_INVALID_FORM;
  if (kind == 2 && p != 2) return MDG_ERROR_INVALID_LIMBS;
  if (count < 0) return MDG_ERROR_INVALID_SIZE;
  if (count > 0 && (!x || !out)) return MDG_ERROR_NULL_POINTER;
  return launch_split(kind, exact, p, count, x, out, 0, 0, as_stream(stream));
}

int mdg_split_planes(int kind, int exact, int p, long long count, const double *x,
                     double *planes, long long plane_stride, void *stream) {
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (kind < 0 || kind > 3 || (exact != 0 && exact != 1)) return MDG_ERROR_INVALID_FORM;
  if (kind == 2 && p != 2) return MDG_ERROR_INVALID_LIMBS;
  if (count < 0 || plane_stride < count) return MDG_ERROR_INVALID_SIZE;
  if (count > 0 && (!x || !planes)) return MDG_ERROR_NULL_POINTER;
  return launch_split(kind, exact, p, count, x, planes, 1, plane_stride, as_stream(stream));
}

int mdg_squeeze(int p, int pp, long long count, const double *x, double *y, void *stream) {
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (pp < 1 || count < 0) return MDG_ERROR_INVALID_SIZE;
  if (count > 0 && (!x || !y)) return MDG_ERROR_NULL_POINTER;
  return launch_squeeze(p, pp, count, x, pp, 1, y, as_stream(stream));
}

size_t mdg_slice_conv_workspace_size(int pp, int m, int n, int k) {
  (void)pp; (void)m; (void)n; (void)k;
  return 0;
}

int mdg_slice_conv(int pp, int m, int n, int k, const double *Aq, const double *Bq, double *Cq,
                   void *workspace, size_t workspace_bytes_, void *stream) {
  (void)workspace;
  (void)workspace_bytes_;
  if (pp < 1 || m < 0 || n < 0 || k < 0) return MDG_ERROR_INVALID_SIZE;
  if (m == 0 || n == 0) return MDG_SUCCESS;  // nothing is read or written
  if (!Cq || (k > 0 && (!Aq || !Bq))) return MDG_ERROR_NULL_POINTER;
  return launch_slice_conv(pp, m, n, k, Aq, Bq, Cq, 0, as_stream(stream));
}

int mdg_plane_conv(int pp, int m, int n, int k, const double *A, const double *B, double *C,
                   void *stream) {
  if (pp < 1 || m < 0 || n < 0 || k < 0) return MDG_ERROR_INVALID_SIZE;
  if (m == 0 || n == 0) return MDG_SUCCESS;  // nothing is read or written
  if (!C || (k > 0 && (!A || !B))) return MDG_ERROR_NULL_POINTER;
  return launch_slice_conv(pp, m, n, k, A, B, C, 1, as_stream(stream));
}

int mdg_scale_exponents(int p, int m, int n, int k, const double *A, int lda, const double *B,
                        int ldb, int *E, int *F, void *stream) {
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (m < 0 || n < 0 || k < 0 || lda < std::max(k, 1) || ldb < std::max(n, 1))
    return MDG_ERROR_INVALID_SIZE;
  if ((m > 0 && (!E || (k > 0 && !A))) || (n > 0 && (!F || (k > 0 && !B))))
    return MDG_ERROR_NULL_POINTER;
  std::lock_guard<std::mutex> lk(g_cache.mu);
  MDG_TRY(g_cache.bind_device());
  void *bits;
  MDG_TRY(g_cache.get(3, sizeof(unsigned long long) * (size_t)(std::max(m, 1) + std::max(n, 1)),
                      &bits));
  auto *rb = reinterpret_cast<unsigned long long *>(bits);
  return launch_scale_exponents(p, m, n, k, A, lda, B, ldb, rb, rb + std::max(m, 1), E, F,
                                as_stream(stream));
}

int mdg_slice_digits(int p, int s, int rows, int cols, const double *X, int ldx, const int *E,
                     int trans, void *planes, int ld_out, long long plane_stride,
                     void *stream) {
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (s < 1 || s > 128 || rows < 0 || cols < 0 || ld_out < cols) return MDG_ERROR_INVALID_SIZE;
  if (plane_stride < (long long)rows * ld_out) return MDG_ERROR_INVALID_SIZE;
  if (trans ? (ldx < std::max(rows, 1)) : (ldx < std::max(cols, 1))) return MDG_ERROR_INVALID_SIZE;
  if (rows > 0 && cols > 0 && (!X || !E || !planes)) return MDG_ERROR_NULL_POINTER;
  if (rows > 65535) return MDG_ERROR_NOT_SUPPORTED;
  return launch_digits(p, s, rows, cols, X, ldx, E, trans, planes, ld_out, plane_stride, rows,
                       cols, as_stream(stream));
}

int mdg_slice_chunk_count(int s, int D, int k) {
  if (s < 1 || D < 1 || D > 2 * s - 1 || k < 0) return 0;
  return total_chunks(s, D, (int)(align_up(std::max(k, 1), 64) / 64));
}

int mdg_slice_diagonals(int s, int D, int m, int n, int k, const void *dA, const void *dB, int ld,
                        long long plane_a, long long plane_b, int *chunks, void *stream) {
  if (s < 1 || D < 1 || D > 2 * s - 1 || m < 0 || n < 0 || k < 0) return MDG_ERROR_INVALID_SIZE;
  if (m % 128 || n % 256 || k % 64 || ld < k) return MDG_ERROR_INVALID_SIZE;
  // each digit plane holds its rows at stride ld: planes that overlap would
  // have the last one read past the caller's buffer
  if (plane_a < (long long)m * ld || plane_b < (long long)n * ld) return MDG_ERROR_INVALID_SIZE;
  if (m == 0 || n == 0 || k == 0) return MDG_SUCCESS;
  if (!dA || !dB || !chunks) return MDG_ERROR_NULL_POINTER;
  const long long plane_c = (long long)m * n;
  const int eng = engine_choice(0);
  if (eng != 0 && ld == k)
    return launch_diag_gemm_tc(s, D, m, n, k, dA, dB, ld, plane_a, plane_b, chunks, plane_c,
                               eng == 2 ? 1 : 0, 0, 0, as_stream(stream));
  return launch_diag_gemm_v0(s, D, m, n, k, dA, dB, ld, plane_a, plane_b, chunks, plane_c,
                             as_stream(stream));
}

int mdg_renorm_diagonals(int p, int s, int D, int k, int m, int n, const int *chunks,
                         long long plane_c, int ldcd, const int *E, const int *F, double *C,
                         int ldc, void *stream) {
  if (!valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (s < 1 || D < 1 || D > 2 * s - 1 || k < 0 || m < 0 || n < 0 || ldc < std::max(n, 1) ||
      ldcd < n || plane_c < (long long)m * ldcd)
    return MDG_ERROR_INVALID_SIZE;
  if (!words_for(1, D)) return MDG_ERROR_NOT_SUPPORTED;
  if (m == 0 || n == 0) return MDG_SUCCESS;
  if (!chunks || !E || !F || !C) return MDG_ERROR_NULL_POINTER;
  if (m > 65535) return MDG_ERROR_NOT_SUPPORTED;
  const int KB = (int)(align_up(std::max(k, 1), 64) / 64);
  return launch_renorm(p, s, D, KB, m, n, chunks, plane_c, ldcd, E, F, C, ldc, as_stream(stream));
}

int mdg_device_status(void) { return tc_device_status(); }

}  // extern "C"

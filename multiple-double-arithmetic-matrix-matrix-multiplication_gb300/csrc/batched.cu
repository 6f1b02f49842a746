// Batched slice-digit GEMM: many problems of uneven m, n, k and mixed P in
// one launch per stage.
//
// mdg_batch_create lays out the caller's workspace (a table of problems,
// the scale exponents of all problems side by side, every problem's digit
// and chunk planes) and uploads the tables, tensor maps included;
// mdg_batch_run only launches kernels, so it can be captured into a CUDA
// graph and replayed.  Per run, whatever the mix of P:
//   one launch: exponents of every row of every A and column of every B
//   one launch: digits of every A and every B
//   one launch: grouped tcgen05 diagonal GEMM over the tiles of all problems
//   one launch per limb count present: renormalisation of its C
// Each stage kernel finds its problem from its block index by binary search
// over per-problem prefix counts, and branches on the problem's P to the
// integer width that P needs (batched_stages.cuh).  The grouped GEMM's tiles
// are 128 rows by 256 or 128 columns per problem, or 256 x 256 on CTA pairs
// (a tile policy the plan can tune); heavy tiles can be cut into ranges of
// diagonals (the split mode, tuned too).  Each problem's result equals the
// single-problem mdg_gemm result bit for bit.  The reference runs one square problem per call; it
// has no counterpart of this entry.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "slice_stages.cuh"
#include "slice_tc.cuh"

#include "batched_table.cuh"

struct mdg_batch_s {
  int count = 0, nwmax = 4, total_units = 0;
  int scale_units = 0, digit_units = 0, renorm_units = 0;
  // per P = 2, 4, 8, 16: first output row, rows, widest n
  int renorm_begin[4] = {0, 0, 0, 0}, renorm_count[4] = {0, 0, 0, 0}, renorm_n[4] = {0, 0, 0, 0};
  int tiles_policy = MDG_BATCH_TILES_256, split = 1;
  mdgi::BatchProblem *dprobs = nullptr;
  mdgi::GroupedProblem *dgroups = nullptr;
  int *exps = nullptr;  // E of all problems then F
  std::vector<mdgi::BatchProblem> hprobs;  // host copy of the table
};

namespace {

using mdgi::BatchProblem;

// Tile width of a problem's single-CTA grouped-GEMM tiles under a policy:
// 256 columns (the wider tile reads fewer operand bytes per product), or 128
// where that pads fewer columns (n mod 256 in 1..128), or 128 always.  The
// CTA-pair policy uses 256 x 256 tiles.
int tile_width(int policy, int n) {
  const int w128 = (int)mdgi::align_up(std::max(n, 1), 128);
  const int w256 = (int)mdgi::align_up(std::max(n, 1), 256);
  switch (policy) {
    case MDG_BATCH_TILES_128: return 128;
    case MDG_BATCH_TILES_AUTO: return w128 < w256 ? 128 : 256;
    default: return 256;
  }
}

// Work units per worker (CTA, or CTA pair) that the split mode aims for:
// heavy tiles are cut into diagonal ranges of about total / (workers x this)
// k-steps of work.  Small units keep the units of one problem side by side
// on the GPU, so that its digit planes are read from DRAM about once rather
// than once per digit pair.
constexpr int kSplitUnitsPerWorker = 16;

// The grouped GEMM's table for a tile policy and split mode: B tensor maps
// with the policy's box, units dealt heaviest first.
int grouped_table(const std::vector<BatchProblem> &hp, int policy, int split, int workers,
                  std::vector<mdgi::GroupedProblem> *hg, int *total_units) {
  hg->clear();
  const bool pair = policy == MDG_BATCH_TILES_PAIR;
  for (const BatchProblem &b : hp) {
    mdgi::GroupedProblem g{};
    const int tn = tile_width(policy, b.n);
    MDG_TRY(mdgi::encode_plane_map(g.tmA, b.dA, b.Kp, (long long)b.s * b.Mp, 128));
    MDG_TRY(mdgi::encode_plane_map(g.tmB, b.dB, b.Kp, (long long)b.s * b.Np, pair ? 128 : tn));
    g.s = b.s; g.D = b.D; g.Mp = b.Mp; g.Np = b.Np; g.KB = b.Kp / 64;
    g.tn = tn;
    g.mt = pair ? b.Mp / 256 : (b.m + 127) / 128;
    g.nt = (b.n + tn - 1) / tn;
    g.ktail = (b.k - (g.KB - 1) * 64 + 15) / 16;
    g.parts = 1;
    g.out = b.chunks;
    g.plane_c = b.plane_c;
    hg->push_back(g);
  }
  // work of one tile in k-steps of 128 x 128 output: digit pairs x k-blocks
  // x tile area
  auto tile_work = [&](const mdgi::GroupedProblem &g) {
    long long pairs = 0;
    for (int d = 0; d < g.D; ++d) pairs += mdgi::diag_pairs(d, g.s);
    return pairs * g.KB * (pair ? 4 : g.tn / 128);
  };
  if (split) {
    long long total = 0;
    for (const mdgi::GroupedProblem &g : *hg) total += tile_work(g) * g.mt * g.nt;
    const long long target =
        std::max(1LL, total / ((long long)std::max(workers, 1) * kSplitUnitsPerWorker));
    for (mdgi::GroupedProblem &g : *hg)
      g.parts = (int)std::min<long long>(g.D, std::max(1LL, (tile_work(g) + target - 1) / target));
  }
  // The grouped kernel deals units to CTAs round-robin in table order.
  // Heaviest units first (a quad-double tile carries ~4x the work of a
  // double-double one, an octo-double tile ~15x), so that the deal
  // approximates longest-processing-time-first and the CTAs finish
  // together; a problem's units stay consecutive.  Only the order changes;
  // each unit still writes its own problem's chunk planes.
  auto unit_work = [&](const mdgi::GroupedProblem &g) {
    return (tile_work(g) + g.parts - 1) / g.parts;
  };
  std::stable_sort(hg->begin(), hg->end(),
                   [&](const mdgi::GroupedProblem &a, const mdgi::GroupedProblem &b) {
                     return unit_work(a) > unit_work(b);
                   });
  long long u = 0;
  for (mdgi::GroupedProblem &g : *hg) {
    g.unit_begin = (int)u;
    u += (long long)g.mt * g.nt * g.parts;
  }
  if (u > (1LL << 30)) return MDG_ERROR_INVALID_SIZE;
  *total_units = (int)u;
  return MDG_SUCCESS;
}

struct Layout {
  size_t off_probs, off_groups, off_exps, total;
  std::vector<size_t> off_dA, off_dB, off_chunks;
};

// Sizes and offsets; fills the host table when `ws` is non-null.
int plan_batch(const mdg_problem *problems, int count, Layout *L, mdg_batch_s *h,
               std::vector<BatchProblem> *hp, char *ws) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = mdgi::align_up(off + bytes, 256);
    return o;
  };
  L->off_probs = take(sizeof(BatchProblem) * count);
  L->off_groups = take(sizeof(mdgi::GroupedProblem) * count);
  int rows = 0, cols = 0;
  for (int i = 0; i < count; ++i) {
    rows += std::max(problems[i].m, 1);
    cols += std::max(problems[i].n, 1);
  }
  L->off_exps = take(sizeof(int) * (size_t)(rows + cols));
  L->off_dA.resize(count);
  L->off_dB.resize(count);
  L->off_chunks.resize(count);
  int scale_u = 0, digit_u = 0, renorm_u = 0, offE = 0, offF = rows;
  h->nwmax = 4;
  for (int i = 0; i < 4; ++i) h->renorm_begin[i] = h->renorm_count[i] = h->renorm_n[i] = 0;
  // the table is kept in order of P (stable): blocks of one P sit together
  // in every stage's launch
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return problems[a].p < problems[b].p; });
  for (int oi = 0; oi < count; ++oi) {
    const int i = order[oi];
    const mdg_problem &q = problems[i];
    const int s = mdg_default_slices(q.p), D = s;
    // rows padded to 256 so that every tile policy, CTA pairs included, fits
    const int Mp = (int)mdgi::align_up(std::max(q.m, 1), 256);
    const int Np = (int)mdgi::align_up(std::max(q.n, 1), 256);
    const int Kp = (int)mdgi::align_up(std::max(q.k, 1), 64);
    const int nch = mdgi::total_chunks(s, D, Kp / 64);
    L->off_dA[i] = take(sizeof(__nv_bfloat16) * (size_t)s * Mp * Kp);
    L->off_dB[i] = take(sizeof(__nv_bfloat16) * (size_t)s * Np * Kp);
    L->off_chunks[i] = take(sizeof(int) * (size_t)nch * Mp * Np);
    const int nw = std::max(mdgi::words_for(s, 1), mdgi::words_for(1, D));
    if (!nw || nw > mdgi::batch_words(q.p)) return MDG_ERROR_NOT_SUPPORTED;
    h->nwmax = std::max(h->nwmax, mdgi::batch_words(q.p));
    const int kblocks = (q.k + 127) / 128;
    const int scale_a = (q.m + 7) / 8, scale_b = (q.n + 31) / 32;
    // digits: valid rows and k-positions only (the padding is cleared once,
    // by mdg_batch_create)
    const int digit_a = q.m * kblocks, digit_b = q.n * kblocks;
    const int out_u = q.m;  // renormalisation: one row of blocks per output row
    if (ws) {
      BatchProblem b{};
      b.p = q.p; b.s = s; b.D = D; b.m = q.m; b.n = q.n; b.k = q.k;
      b.Mp = Mp; b.Np = Np; b.Kp = Kp;
      b.A = q.A; b.B = q.B; b.C = q.C; b.lda = q.lda; b.ldb = q.ldb; b.ldc = q.ldc;
      b.offE = offE; b.offF = offF;
      b.dA = reinterpret_cast<__nv_bfloat16 *>(ws + L->off_dA[i]);
      b.dB = reinterpret_cast<__nv_bfloat16 *>(ws + L->off_dB[i]);
      b.chunks = reinterpret_cast<int *>(ws + L->off_chunks[i]);
      b.plane_a = (long long)Mp * Kp;
      b.plane_b = (long long)Np * Kp;
      b.plane_c = (long long)Mp * Np;
      b.scale_begin = scale_u; b.scale_b_off = scale_a;
      b.dig_begin = digit_u; b.dig_b_off = digit_a;
      b.out_begin = renorm_u;
      hp->push_back(b);
    }
    const int pi = q.p == 2 ? 0 : q.p == 4 ? 1 : q.p == 8 ? 2 : 3;
    if (h->renorm_count[pi] == 0) h->renorm_begin[pi] = renorm_u;
    h->renorm_count[pi] += out_u;
    h->renorm_n[pi] = std::max(h->renorm_n[pi], q.n);
    scale_u += scale_a + scale_b;
    digit_u += digit_a + digit_b;
    renorm_u += out_u;
    offE += std::max(q.m, 1);
    offF += std::max(q.n, 1);
  }
  h->count = count;
  h->scale_units = scale_u;
  h->digit_units = digit_u;
  h->renorm_units = renorm_u;
  L->total = off;
  return MDG_SUCCESS;
}

int check_problems(const mdg_problem *problems, int count) {
  if (count < 0) return MDG_ERROR_INVALID_SIZE;
  if (count > 0 && !problems) return MDG_ERROR_NULL_POINTER;
  for (int i = 0; i < count; ++i) {
    const mdg_problem &q = problems[i];
    if (!mdgi::valid_p(q.p)) return MDG_ERROR_INVALID_LIMBS;
    if (q.m <= 0 || q.n <= 0 || q.k <= 0) return MDG_ERROR_INVALID_SIZE;
    if (q.lda < q.k || q.ldb < q.n || q.ldc < q.n) return MDG_ERROR_INVALID_SIZE;
    if (!q.A || !q.B || !q.C) return MDG_ERROR_NULL_POINTER;
  }
  return MDG_SUCCESS;
}

// Key of a batch in the tuning cache: its problem shapes (P, m, n, k), in
// table order, hashed (FNV-1a 64).
std::string batch_key(const std::vector<BatchProblem> &hp) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](int v) {
    for (int b = 0; b < 4; ++b) {
      h ^= (uint64_t)((v >> (8 * b)) & 255);
      h *= 1099511628211ull;
    }
  };
  for (const BatchProblem &b : hp) {
    mix(b.p);
    mix(b.m);
    mix(b.n);
    mix(b.k);
  }
  char buf[64];
  std::snprintf(buf, sizeof(buf), "batch %d %016llx", (int)hp.size(), (unsigned long long)h);
  return buf;
}

// Builds and uploads the grouped GEMM's table for a tile policy and split
// mode; waits for the copy (the host table is a local).
int apply_tiles(mdg_batch_s *h, int policy, int split, cudaStream_t st) {
  int dev = 0, sms = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  MDG_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  std::vector<mdgi::GroupedProblem> hg;
  int units = 0;
  MDG_TRY(grouped_table(h->hprobs, policy, split,
                        policy == MDG_BATCH_TILES_PAIR ? sms / 2 : sms, &hg, &units));
  MDG_TRY_CUDA(cudaMemcpyAsync(h->dgroups, hg.data(), sizeof(mdgi::GroupedProblem) * h->count,
                               cudaMemcpyHostToDevice, st));
  MDG_TRY_CUDA(cudaStreamSynchronize(st));
  h->total_units = units;
  h->tiles_policy = policy;
  h->split = split;
  return MDG_SUCCESS;
}

}  // namespace

extern "C" {

size_t mdg_batch_workspace_size(const mdg_problem *problems, int count) {
  if (check_problems(problems, count) != MDG_SUCCESS || count == 0) return 0;
  Layout L;
  mdg_batch_s h;
  if (plan_batch(problems, count, &L, &h, nullptr, nullptr) != MDG_SUCCESS) return 0;
  return L.total;
}

int mdg_batch_create(const mdg_problem *problems, int count, void *workspace,
                     size_t workspace_bytes, void *stream, mdg_batch_s **out) {
  if (!out) return MDG_ERROR_NULL_POINTER;
  *out = nullptr;
  MDG_TRY(check_problems(problems, count));
  if (count == 0) return MDG_ERROR_INVALID_SIZE;
  Layout L;
  mdg_batch_s probe;
  MDG_TRY(plan_batch(problems, count, &L, &probe, nullptr, nullptr));
  if (!workspace || workspace_bytes < L.total) return MDG_ERROR_WORKSPACE;
  char *ws = reinterpret_cast<char *>(workspace);
  auto *h = new mdg_batch_s();
  int st = plan_batch(problems, count, &L, h, &h->hprobs, ws);
  if (st != MDG_SUCCESS) {
    delete h;
    return st;
  }
  h->dprobs = reinterpret_cast<BatchProblem *>(ws + L.off_probs);
  h->dgroups = reinterpret_cast<mdgi::GroupedProblem *>(ws + L.off_groups);
  h->exps = reinterpret_cast<int *>(ws + L.off_exps);
  cudaStream_t s = mdgi::as_stream(stream);
  // zero digit planes: the digit kernel writes only the valid rows and
  // k-positions of each problem, so the padding stays zero for every run
  for (const BatchProblem &b : h->hprobs) {
    cudaError_t e = cudaMemsetAsync(b.dA, 0, sizeof(__nv_bfloat16) * (size_t)b.s * b.Mp * b.Kp, s);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(b.dB, 0, sizeof(__nv_bfloat16) * (size_t)b.s * b.Np * b.Kp, s);
    if (e != cudaSuccess) {
      mdgi::set_cuda_error(e);
      delete h;
      return MDG_ERROR_CUDA;
    }
  }
  // a tile policy and split mode tuned earlier for the same shapes, else
  // 256-column tiles, split
  int policy = MDG_BATCH_TILES_256, split = 1;
  mdgi::tune_lookup_batch(batch_key(h->hprobs), &policy, &split);
  cudaError_t e = cudaMemcpyAsync(h->dprobs, h->hprobs.data(), sizeof(BatchProblem) * count,
                                  cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    mdgi::set_cuda_error(e);
    delete h;
    return MDG_ERROR_CUDA;
  }
  st = apply_tiles(h, policy, split, s);
  if (st != MDG_SUCCESS) {
    delete h;
    return st;
  }
  *out = h;
  return MDG_SUCCESS;
}

int mdg_batch_run(mdg_batch_s *h, void *stream) {
  if (!h) return MDG_ERROR_NULL_POINTER;
  cudaStream_t st = mdgi::as_stream(stream);
#define MDG_BATCH_STAGES(W)                                                               \
  MDG_TRY(mdgi::launch_batch_scale<W>(h->dprobs, h->count, h->scale_units, h->exps, st)); \
  MDG_TRY(mdgi::launch_batch_digits<W>(h->dprobs, h->count, h->digit_units, h->exps, st))
  switch (h->nwmax) {
    case 4: MDG_BATCH_STAGES(4); break;
    case 6: MDG_BATCH_STAGES(6); break;
    case 10: MDG_BATCH_STAGES(10); break;
    default: MDG_BATCH_STAGES(16); break;
  }
#undef MDG_BATCH_STAGES
  MDG_TRY(mdgi::launch_diag_gemm_grouped(h->dgroups, h->count, h->total_units,
                                         h->tiles_policy == MDG_BATCH_TILES_PAIR, st));
  const int *rb = h->renorm_begin, *rc = h->renorm_count, *rn = h->renorm_n;
  MDG_TRY(mdgi::launch_batch_renorm<2>(h->dprobs, h->count, rb[0], rc[0], rn[0], h->exps, st));
  MDG_TRY(mdgi::launch_batch_renorm<4>(h->dprobs, h->count, rb[1], rc[1], rn[1], h->exps, st));
  MDG_TRY(mdgi::launch_batch_renorm<8>(h->dprobs, h->count, rb[2], rc[2], rn[2], h->exps, st));
  MDG_TRY(mdgi::launch_batch_renorm<16>(h->dprobs, h->count, rb[3], rc[3], rn[3], h->exps, st));
  return MDG_SUCCESS;
}

int mdg_batch_set_tiles(mdg_batch_s *h, int policy, void *stream) {
  if (!h) return MDG_ERROR_NULL_POINTER;
  if (policy < MDG_BATCH_TILES_AUTO || policy > MDG_BATCH_TILES_PAIR) return MDG_ERROR_INVALID_FORM;
  return apply_tiles(h, policy, h->split, mdgi::as_stream(stream));
}

int mdg_batch_tiles(mdg_batch_s *h) { return h ? h->tiles_policy : -1; }

int mdg_batch_set_split(mdg_batch_s *h, int split, void *stream) {
  if (!h) return MDG_ERROR_NULL_POINTER;
  if (split != 0 && split != 1) return MDG_ERROR_INVALID_FORM;
  return apply_tiles(h, h->tiles_policy, split, mdgi::as_stream(stream));
}

int mdg_batch_split(mdg_batch_s *h) { return h ? h->split : -1; }

int mdg_batch_tune(mdg_batch_s *h, void *stream) {
  if (!h) return MDG_ERROR_NULL_POINTER;
  mdgi::NvtxRange range("mdg batch tune");
  cudaStream_t st = mdgi::as_stream(stream);
  cudaEvent_t e0, e1;
  MDG_TRY_CUDA(cudaEventCreate(&e0));
  MDG_TRY_CUDA(cudaEventCreate(&e1));
  int best = h->tiles_policy, best_split = h->split, status = MDG_SUCCESS;
  float best_ms = 0.0f;
  for (int choice = 0; choice < 8 && status == MDG_SUCCESS; ++choice) {
    static const int kPolicies[4] = {MDG_BATCH_TILES_256, MDG_BATCH_TILES_AUTO,
                                     MDG_BATCH_TILES_128, MDG_BATCH_TILES_PAIR};
    const int policy = kPolicies[choice >> 1], split = 1 - (choice & 1);
    status = apply_tiles(h, policy, split, st);
    if (status == MDG_SUCCESS) status = mdg_batch_run(h, stream);  // warm-up
    if (status != MDG_SUCCESS) break;
    cudaEventRecord(e0, st);
    status = mdg_batch_run(h, stream);
    cudaEventRecord(e1, st);
    float ms = 0.0f;
    if (status != MDG_SUCCESS) break;
    if (cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      status = MDG_ERROR_CUDA;
      break;
    }
    if (best_ms == 0.0f || ms < best_ms) {
      best_ms = ms;
      best = policy;
      best_split = split;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MDG_TRY(status);
  MDG_TRY(mdg_device_status());  // a bounded wait that gave up fails the tuning
  MDG_TRY(apply_tiles(h, best, best_split, st));
  mdgi::tune_record_batch(batch_key(h->hprobs), best, best_split, best_ms);
  return MDG_SUCCESS;
}

void mdg_batch_destroy(mdg_batch_s *h) { delete h; }

}  // extern "C"

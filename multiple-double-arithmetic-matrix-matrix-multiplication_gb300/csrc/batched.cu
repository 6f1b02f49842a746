// Batched slice-digit GEMM: many problems of uneven m, n, k and mixed P in
// one launch per stage.
//
// mdg_batch_create lays out the caller's workspace (a table of problems,
// the scale-exponent arrays of all problems side by side, every problem's
// digit and chunk planes) and uploads the tables, tensor maps included;
// mdg_batch_run only launches kernels, so it can be captured into a CUDA
// graph and replayed:
//   memset of the row / column maxima
//   absmax over the rows of every A, absmax over the columns of every B
//   exponents of all rows and columns
//   digits of every A, digits of every B
//   one grouped tcgen05 diagonal GEMM over the tiles of all problems
//   renormalisation of every C
// Each stage kernel finds its problem from its block index by binary search
// over per-problem prefix counts.  Digit and renorm kernels use the widest
// integer the batch needs for every problem (a wider integer gives the same
// bits).  Each problem's result equals the single-problem mdg_gemm result
// bit for bit.  The reference runs one square problem per call; it has no
// counterpart of this entry.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "slice_stages.cuh"
#include "slice_tc.cuh"

#include "batched_table.cuh"

// Problems of one limb count P: a contiguous range of the problem table
// (sorted by P), digit and renorm kernels launched with its own integer width.
struct BatchGroup {
  int p = 0, nw = 4;
  int digA0 = 0, digA = 0, digB0 = 0, digB = 0, out0 = 0, out = 0;  // first block, blocks
  int max_Kp = 0, max_n = 0;
};

struct mdg_batch_s {
  int count = 0, nw = 4, total_tiles = 0;
  std::vector<BatchGroup> groups;
  int total_rowblk = 0, total_colblk = 0, total_digA = 0, total_digB = 0, total_out = 0;
  int max_k = 0, max_n = 0, max_Kp = 0;
  int total_exps = 0;
  mdgi::BatchProblem *dprobs = nullptr;
  mdgi::GroupedProblem *dgroups = nullptr;
  unsigned long long *bits = nullptr;  // row maxima then column maxima
  int *exps = nullptr;                 // E of all problems then F
};

namespace {

using mdgi::BatchProblem;
using mdgi::find_problem;

__global__ void absmax_rows_b(const BatchProblem *__restrict__ pr, int count,
                              unsigned long long *bits) {
  const int q = find_problem<0>(pr, count, blockIdx.y);
  const BatchProblem &b = pr[q];
  if ((int)blockIdx.x * 32 >= b.k) return;
  mdgi::absmax_block(b.p, b.m, b.k, b.A, b.lda, bits + b.offE, nullptr, blockIdx.x,
                     blockIdx.y - b.rowblk_begin);
}

__global__ void absmax_cols_b(const BatchProblem *__restrict__ pr, int count,
                              unsigned long long *bits) {
  const int q = find_problem<1>(pr, count, blockIdx.y);
  const BatchProblem &b = pr[q];
  if ((int)blockIdx.x * 32 >= b.n) return;
  mdgi::absmax_block(b.p, b.k, b.n, b.B, b.ldb, nullptr, bits + b.offF, blockIdx.x,
                     blockIdx.y - b.colblk_begin);
}

__global__ void exps_b(int count, const unsigned long long *__restrict__ bits, int *__restrict__ E) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) E[i] = mdgi::scale_exp(__longlong_as_double((long long)bits[i]));
}

struct Layout {
  size_t off_probs, off_groups, off_bits, off_exps, total;
  std::vector<size_t> off_dA, off_dB, off_chunks;
};

// Sizes and offsets; fills the host tables when `ws` is non-null.
int plan_batch(const mdg_problem *problems, int count, Layout *L, mdg_batch_s *h,
               std::vector<BatchProblem> *hp, std::vector<mdgi::GroupedProblem> *hg, char *ws) {
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
  L->off_bits = take(sizeof(unsigned long long) * (size_t)(rows + cols));
  L->off_exps = take(sizeof(int) * (size_t)(rows + cols));
  L->off_dA.resize(count);
  L->off_dB.resize(count);
  L->off_chunks.resize(count);
  int rowblk = 0, colblk = 0, digA = 0, digB = 0, outr = 0, tiles = 0, offE = 0, offF = rows;
  h->nw = 4;
  h->groups.clear();
  // the table is built in order of P (stable), so that every P group is one
  // contiguous range of blocks for the digit and renorm launches
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return problems[a].p < problems[b].p; });
  for (int oi = 0; oi < count; ++oi) {
    const int i = order[oi];
    const mdg_problem &q = problems[i];
    const int s = mdg_default_slices(q.p), D = s;
    const int Mp = (int)mdgi::align_up(std::max(q.m, 1), 128);
    const int Np = (int)mdgi::align_up(std::max(q.n, 1), 256);
    const int Kp = (int)mdgi::align_up(std::max(q.k, 1), 64);
    const int nch = mdgi::total_chunks(s, D, Kp / 64);
    L->off_dA[i] = take(sizeof(__nv_bfloat16) * (size_t)s * Mp * Kp);
    L->off_dB[i] = take(sizeof(__nv_bfloat16) * (size_t)s * Np * Kp);
    L->off_chunks[i] = take(sizeof(int) * (size_t)nch * Mp * Np);
    const int nw = std::max(mdgi::words_for(s, 1), mdgi::words_for(1, D));
    if (!nw) return MDG_ERROR_NOT_SUPPORTED;
    h->nw = std::max(h->nw, nw);
    if (h->groups.empty() || h->groups.back().p != q.p) {
      BatchGroup g;
      g.p = q.p;
      g.digA0 = digA;
      g.digB0 = digB;
      g.out0 = outr;
      h->groups.push_back(g);
    }
    BatchGroup &grp = h->groups.back();
    grp.nw = std::max(grp.nw, nw);
    grp.digA += Mp;
    grp.digB += Np;
    grp.out += std::max(q.m, 1);
    grp.max_Kp = std::max(grp.max_Kp, Kp);
    grp.max_n = std::max(grp.max_n, q.n);
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
      b.rowblk_begin = rowblk; b.colblk_begin = colblk;
      b.digA_begin = digA; b.digB_begin = digB; b.out_begin = outr;
      hp->push_back(b);
      mdgi::GroupedProblem g{};
      MDG_TRY(mdgi::encode_plane_map(g.tmA, b.dA, Kp, (long long)s * Mp, 128));
      MDG_TRY(mdgi::encode_plane_map(g.tmB, b.dB, Kp, (long long)s * Np, 256));
      g.s = s; g.D = D; g.Mp = Mp; g.Np = Np; g.KB = Kp / 64; g.tile_begin = tiles;
      g.out = b.chunks;
      g.plane_c = b.plane_c;
      hg->push_back(g);
    }
    rowblk += (std::max(q.m, 1) + 255) / 256;
    colblk += (std::max(q.k, 1) + 255) / 256;
    digA += Mp;
    digB += Np;
    outr += std::max(q.m, 1);
    tiles += (Mp / 128) * (Np / 256);
    offE += std::max(q.m, 1);
    offF += std::max(q.n, 1);
    h->max_k = std::max(h->max_k, q.k);
    h->max_n = std::max(h->max_n, q.n);
    h->max_Kp = std::max(h->max_Kp, Kp);
  }
  if (ws) {
    // The grouped kernel deals tiles to CTAs round-robin in table order.
    // Heaviest tiles first (digit pairs x k-steps per tile: a quad-double
    // tile carries ~4x the work of a double-double one, an octo-double
    // tile ~15x), so that the deal approximates longest-processing-time-
    // first and the CTAs finish together.  Only the order of the tiles
    // changes; each still writes its own problem's chunk planes.
    auto work = [](const mdgi::GroupedProblem &g) {
      long long pairs = 0;
      for (int d = 0; d < g.D; ++d) pairs += mdgi::diag_pairs(d, g.s);
      return pairs * g.KB;
    };
    std::stable_sort(hg->begin(), hg->end(),
                     [&](const mdgi::GroupedProblem &a, const mdgi::GroupedProblem &b) {
                       return work(a) > work(b);
                     });
    int t = 0;
    for (auto &g : *hg) {
      g.tile_begin = t;
      t += (g.Mp / 128) * (g.Np / 256);
    }
  }
  h->count = count;
  h->total_rowblk = rowblk;
  h->total_colblk = colblk;
  h->total_digA = digA;
  h->total_digB = digB;
  h->total_out = outr;
  h->total_tiles = tiles;
  h->total_exps = rows + cols;
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

}  // namespace

extern "C" {

size_t mdg_batch_workspace_size(const mdg_problem *problems, int count) {
  if (check_problems(problems, count) != MDG_SUCCESS || count == 0) return 0;
  Layout L;
  mdg_batch_s h;
  if (plan_batch(problems, count, &L, &h, nullptr, nullptr, nullptr) != MDG_SUCCESS) return 0;
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
  MDG_TRY(plan_batch(problems, count, &L, &probe, nullptr, nullptr, nullptr));
  if (!workspace || workspace_bytes < L.total) return MDG_ERROR_WORKSPACE;
  char *ws = reinterpret_cast<char *>(workspace);
  auto *h = new mdg_batch_s();
  std::vector<BatchProblem> hp;
  std::vector<mdgi::GroupedProblem> hg;
  int st = plan_batch(problems, count, &L, h, &hp, &hg, ws);
  if (st != MDG_SUCCESS) {
    delete h;
    return st;
  }
  h->dprobs = reinterpret_cast<BatchProblem *>(ws + L.off_probs);
  h->dgroups = reinterpret_cast<mdgi::GroupedProblem *>(ws + L.off_groups);
  h->bits = reinterpret_cast<unsigned long long *>(ws + L.off_bits);
  h->exps = reinterpret_cast<int *>(ws + L.off_exps);
  cudaStream_t s = mdgi::as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(h->dprobs, hp.data(), sizeof(BatchProblem) * count,
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->dgroups, hg.data(), sizeof(mdgi::GroupedProblem) * count,
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    mdgi::set_cuda_error(e);
    delete h;
    return MDG_ERROR_CUDA;
  }
  *out = h;
  return MDG_SUCCESS;
}

int mdg_batch_run(mdg_batch_s *h, void *stream) {
  if (!h) return MDG_ERROR_NULL_POINTER;
  cudaStream_t st = mdgi::as_stream(stream);
  MDG_TRY_CUDA(cudaMemsetAsync(h->bits, 0, sizeof(unsigned long long) * h->total_exps, st));
  absmax_rows_b<<<dim3(mdgi::ceil_div(h->max_k, 32), h->total_rowblk), dim3(32, 8), 0, st>>>(
      h->dprobs, h->count, h->bits);
  MDG_TRY_LAUNCH();
  absmax_cols_b<<<dim3(mdgi::ceil_div(h->max_n, 32), h->total_colblk), dim3(32, 8), 0, st>>>(
      h->dprobs, h->count, h->bits);
  MDG_TRY_LAUNCH();
  exps_b<<<mdgi::ceil_div(h->total_exps, 256), 256, 0, st>>>(h->total_exps, h->bits, h->exps);
  MDG_TRY_LAUNCH();
  // digits and renorm per P group, each with its own integer width
  for (const BatchGroup &g : h->groups) {
    if (!g.digA && !g.digB) continue;
    const dim3 ga(std::max(g.digA, 1), mdgi::ceil_div(g.max_Kp, 128));
    const dim3 gb(std::max(g.digB, 1), mdgi::ceil_div(g.max_Kp, 128));
#define MDG_BATCH_DIGITS(W) \
  MDG_TRY(mdgi::launch_batch_digits<W>(h->dprobs, h->count, h->exps, ga, gb, g.digA0, g.digB0, st))
    switch (g.nw) {
      case 4: MDG_BATCH_DIGITS(4); break;
      case 6: MDG_BATCH_DIGITS(6); break;
      case 10: MDG_BATCH_DIGITS(10); break;
      default: MDG_BATCH_DIGITS(16); break;
    }
#undef MDG_BATCH_DIGITS
  }
  MDG_TRY(mdgi::launch_diag_gemm_grouped(h->dgroups, h->count, h->total_tiles, st));
  for (const BatchGroup &g : h->groups) {
    if (!g.out || !g.max_n) continue;
#define MDG_BATCH_RENORM(W)                                                                   \
  MDG_TRY(mdgi::launch_batch_renorm<W>(g.p, h->dprobs, h->count, h->exps, g.out, g.max_n, g.out0, \
                                       st))
    switch (g.nw) {
      case 4: MDG_BATCH_RENORM(4); break;
      case 6: MDG_BATCH_RENORM(6); break;
      case 10: MDG_BATCH_RENORM(10); break;
      default: MDG_BATCH_RENORM(16); break;
    }
#undef MDG_BATCH_RENORM
  }
  return MDG_SUCCESS;
}

void mdg_batch_destroy(mdg_batch_s *h) { delete h; }

}  // extern "C"

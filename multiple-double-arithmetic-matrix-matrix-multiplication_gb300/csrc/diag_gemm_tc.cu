// Diagonal GEMM of digit planes on the 5th-generation tensor cores.
//
// For every output tile (128 rows x 256 columns) and every diagonal d < D,
// the products A_i B_j^T with i + j = d are summed over k exactly: BF16
// digits in [-128, 128], FP32 accumulation in tensor memory (TMEM), flushed
// every 1024 products (|partial| <= 2^24) into int32 registers, stored every
// 2032 k-steps (130048 products) as one int32 chunk plane (|sum| < 2^31).
//
// One CTA per SM, persistent over tiles; 10 warps with fixed roles:
//   warp 0      TMA producer: A_i (128 x 64) and B_j (256 x 64) k-blocks
//               into a 4-stage shared-memory ring (128-byte swizzle),
//   warp 1      TMEM allocator and MMA issuer: tcgen05.mma kind::f16,
//               M=128 N=256 K=16, BF16 x BF16 -> FP32, into one of two
//               256-column accumulators (all 512 TMEM columns),
//   warps 2-9   epilogue: tcgen05.ld of the accumulator (warp w reads TMEM
//               lanes 32 (w % 4) .. +31, columns 128 ((w - 2) / 4) .. +127)
//               every 16 k-steps, exact float -> int conversion, int32
//               accumulation, chunk stores.
// Barriers: full/empty per stage (TMA <-> MMA), accfull/accempty per
// accumulator (MMA <-> epilogue).  Every wait is bounded (2 s of
// %globaltimer); on a timeout the CTA records the error, stops issuing,
// waits (bounded) for its copies and MMAs in flight, frees TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "common.cuh"
#include "slice_tc.cuh"

namespace {

constexpr int TM = 128, TN = 256, TK = 64;
constexpr int STAGES = 4;
constexpr int A_BYTES = TM * TK * 2;  // 16 KiB
constexpr int B_BYTES = TN * TK * 2;  // 32 KiB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr int TMEM_COLS = 512;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /* align */ + 256 /* barriers */;
constexpr unsigned long long TIMEOUT_NS = 2000000000ull;

// kind::f16 instruction descriptor: D F32 (bits 4-5 = 1), A BF16 (7-9 = 1),
// B BF16 (10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);

__device__ int g_tc_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait.  Returns false on a timeout (and raises the CTA's abort
// flag) or when another role has already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (true) {
    if (mbar_test(bar, parity)) return true;
    if (*abort) return false;
    if (now_ns() - t0 > TIMEOUT_NS) {
      *abort = 1;
      return false;
    }
  }
}

// Bounded wait that ignores the abort flag (draining in-flight work).
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
  const unsigned long long t0 = now_ns();
  while (!mbar_test(bar, parity) && now_ns() - t0 < TIMEOUT_NS) {
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *tm, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor, K-major, 128-byte swizzle: start address
// >> 4 (bits 0-13), leading byte offset 16 B (unused for this layout,
// bits 16-29), stride byte offset 1024 B between 8-row groups (bits 32-45),
// descriptor version 1 (bits 46-47), swizzle mode 2 = 128 B (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(16 >> 4) << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc));
}

// The same with a run-time instruction descriptor (tile width per job).
__device__ __forceinline__ void mma_bf16_n(uint32_t d_tmem, uint64_t a, uint64_t b,
                                           uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Asynchronous TMEM load of 32 columns of this warp's 32 lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
}

// Waits for this thread's outstanding TMEM loads.  The registers of the
// last load are operands, so no read of them can move above the wait.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]),
                 "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]),
                 "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]),
                 "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
}

// The accumulator holds integer-valued floats with |x| <= 2^24; the
// conversion to int32 is exact.
__device__ __forceinline__ void add_exact(int *acc, const uint32_t (&r)[32]) {
#pragma unroll
  for (int j = 0; j < 32; ++j) acc[j] += __float2int_rn(__uint_as_float(r[j]));
}

// Adds 128 accumulator columns (starting at taddr) into acc: four 32-column
// loads, each issued before the previous block is converted so that the
// load latency overlaps the integer work.
__device__ __forceinline__ void drain128(uint32_t taddr, int (&acc)[128]) {
  uint32_t ra[32], rb[32];
  tmem_ld32(taddr, ra);
  tmem_wait(ra);
  tmem_ld32(taddr + 32, rb);
  add_exact(acc, ra);
  tmem_wait(rb);
  tmem_ld32(taddr + 64, ra);
  add_exact(acc + 32, rb);
  tmem_wait(ra);
  tmem_ld32(taddr + 96, rb);
  add_exact(acc + 64, ra);
  tmem_wait(rb);
  add_exact(acc + 96, rb);
}

// Diagonals [d0, d1) of part `part` of a tile cut into `parts` ranges whose
// digit-pair counts add up to about 1/parts of the tile's pairs each (empty
// when parts exceeds what the pair counts allow).
__device__ __forceinline__ void part_diagonals(int s, int D, int part, int parts, int &d0,
                                               int &d1) {
  int total = 0;
  for (int d = 0; d < D; ++d) total += mdgi::diag_pairs(d, s);
  const long long lo = (long long)total * part / parts, hi = (long long)total * (part + 1) / parts;
  int cum = 0;
  d0 = D;
  d1 = D;
  for (int d = 0; d < D; ++d) {
    if (cum >= lo && d0 == D) d0 = d;
    if (cum >= hi) {
      d1 = d;
      break;
    }
    cum += mdgi::diag_pairs(d, s);
  }
  if (d0 > d1) d0 = d1;
}

// One unit of work: where its operands and output live, which of its
// problem's rows / columns it covers and which diagonals [d0, d1) it
// computes.  tn: tile width, 256 or 128 columns (the B box of tmB is tn
// rows); ktail: MMAs of K = 16 issued for the last k-block (1..4; the rest
// of that block is the zero padding of k).
struct TileJob {
  const CUtensorMap *tmA, *tmB;
  int s, D, Mp, Np, KB, row, col, tn, ktail, d0, d1;
  int *out;
  long long plane_c;
};

// A single problem cut into 128 x 256 tiles.
struct SingleJobs {
  const CUtensorMap *tmA, *tmB;
  int s, D, Mp, Np, KB;
  int *out;
  long long plane_c;
  __device__ int tiles() const { return (Mp / TM) * (Np / TN); }
  __device__ TileJob job(int t) const {
    const int MB = Mp / TM;
    return TileJob{tmA, tmB, s, D, Mp, Np, KB, (t % MB) * TM, (t / MB) * TN, TN, TK / 16,
                   0, D, out, plane_c};
  }
};

template <class Jobs>
__device__ __forceinline__ void tc1_body(const Jobs &jobs) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
  // bars: [0,4) full, [4,8) empty, [8,10) accfull, [10,12) accempty, 12 mma drain
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bars + 16);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 17);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t smem_base = smem_u32(smem);
  auto full = [&](int st) { return smem_u32(bars + st); };
  auto empty = [&](int st) { return smem_u32(bars + STAGES + st); };
  auto accfull = [&](int b) { return smem_u32(bars + 2 * STAGES + b); };
  auto accempty = [&](int b) { return smem_u32(bars + 2 * STAGES + 2 + b); };
  const uint32_t drain_bar = smem_u32(bars + 2 * STAGES + 4);

  if (threadIdx.x == 0) {
    for (int st = 0; st < STAGES; ++st) {
      mbar_init(full(st), 1);
      mbar_init(empty(st), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accfull(b), 1);
      mbar_init(accempty(b), EPI_WARPS);
    }
    mbar_init(drain_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_holder)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_base = *tmem_holder;

  const int tiles = jobs.tiles();

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------ producer --
      int st = 0;
      uint32_t ph = 0;
      // per stage: a copy was issued (bit of `issued`), parity of its phase
      // (bit of `last_par`); bit masks so that they stay in registers
      uint32_t issued = 0, last_par = 0;
      for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const TileJob jb = jobs.job(tile);
        const int s = jb.s, KB = jb.KB;
        for (int d = jb.d0; d < jb.d1; ++d) {
          const int ilo = d - (s - 1) > 0 ? d - (s - 1) : 0;
          const int S = mdgi::diag_pairs(d, s) * KB;
          for (int t = 0; t < S; ++t) {
            const int i = ilo + t / KB, kb = t - (t / KB) * KB, j = d - i;
            if (!mbar_wait(empty(st), ph ^ 1, abort_flag)) goto producer_done;
            mbar_expect_tx(full(st), A_BYTES + jb.tn * TK * 2);
            const uint32_t a_dst = smem_base + st * STAGE_BYTES;
            tma_load_2d(a_dst, jb.tmA, kb * TK, i * jb.Mp + jb.row, full(st));
            tma_load_2d(a_dst + A_BYTES, jb.tmB, kb * TK, j * jb.Np + jb.col, full(st));
            last_par = (last_par & ~(1u << st)) | (ph << st);
            issued |= 1u << st;
            if (++st == STAGES) {
              st = 0;
              ph ^= 1;
            }
          }
        }
      }
    producer_done:
      if (*abort_flag)
        for (int i = 0; i < STAGES; ++i)
          if ((issued >> i) & 1u) mbar_drain(full(i), (last_par >> i) & 1u);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------------------------------------------- MMA issuer --
      int st = 0, buf = 0;
      uint32_t ph = 0, aph[2] = {0, 0};
      bool any = false;
      for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const TileJob jb = jobs.job(tile);
        const uint32_t idesc = (IDESC & ~(0x3Fu << 17)) | ((uint32_t)(jb.tn >> 3) << 17);
        for (int d = jb.d0; d < jb.d1; ++d) {
          const int S = mdgi::diag_pairs(d, jb.s) * jb.KB;
          int kb = 0;  // k-block of step t within its digit pair
          for (int g0 = 0; g0 < S; g0 += mdgi::GROUP_STEPS) {
            if (!mbar_wait(accempty(buf), aph[buf] ^ 1, abort_flag)) goto mma_done;
            fence_after();
            const uint32_t dt = tmem_base + buf * TN;
            const int g1 = g0 + mdgi::GROUP_STEPS < S ? g0 + mdgi::GROUP_STEPS : S;
            for (int t = g0; t < g1; ++t) {
              if (!mbar_wait(full(st), ph, abort_flag)) goto mma_done;
              fence_after();
              const uint32_t a_addr = smem_base + st * STAGE_BYTES;
              const uint64_t da = sw128_desc(a_addr), db = sw128_desc(a_addr + A_BYTES);
              // the last k-block of a pair: only the MMAs that reach data
              const bool short_block = kb == jb.KB - 1 && jb.ktail < TK / 16;
              if (++kb == jb.KB) kb = 0;
              if (!short_block) {
#pragma unroll
                for (int kk = 0; kk < TK / 16; ++kk)
                  mma_bf16_n(dt, da + 2 * kk, db + 2 * kk, idesc, (t > g0 || kk > 0) ? 1u : 0u);
              } else {
                for (int kk = 0; kk < jb.ktail; ++kk)
                  mma_bf16_n(dt, da + 2 * kk, db + 2 * kk, idesc, (t > g0 || kk > 0) ? 1u : 0u);
              }
              mma_commit(empty(st));
              any = true;
              if (++st == STAGES) {
                st = 0;
                ph ^= 1;
              }
            }
            mma_commit(accfull(buf));
            aph[buf] ^= 1;
            buf ^= 1;
          }
        }
      }
    mma_done:
      if (*abort_flag && any) {
        mma_commit(drain_bar);
        mbar_drain(drain_bar, 0);
      }
    }
  } else {
    // -------------------------------------------------------- epilogue --
    const int q = warp & 3, h = (warp - 2) >> 2;
    int acc[128];
#pragma unroll
    for (int j = 0; j < 128; ++j) acc[j] = 0;
    int buf = 0;
    uint32_t aph[2] = {0, 0};
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      const TileJob jb = jobs.job(tile);
      // a 128-column tile is drained by the warps of the first column half
      // alone (128 columns each, as for a 256-column tile); the others only
      // release the accumulator
      const bool active = jb.tn == TN || h == 0;
      const int row = jb.row + 32 * q + lane;
      const int col = jb.col + 128 * h;
      int chunk = 0;
      for (int d = 0; d < jb.d0; ++d) chunk += mdgi::diag_chunks(d, jb.s, jb.KB);
      for (int d = jb.d0; d < jb.d1; ++d) {
        const int S = mdgi::diag_pairs(d, jb.s) * jb.KB;
        for (int g0 = 0; g0 < S; g0 += mdgi::GROUP_STEPS) {
          // lane 0 waits; the outcome is broadcast so the warp stays
          // converged for the .sync.aligned TMEM loads
          int ok = 1;
          if (lane == 0) ok = mbar_wait(accfull(buf), aph[buf], abort_flag) ? 1 : 0;
          ok = __shfl_sync(0xffffffffu, ok, 0);
          if (!ok) goto epi_done;
          aph[buf] ^= 1;
          fence_after();
          const uint32_t taddr = tmem_base + ((uint32_t)(32 * q) << 16) + buf * TN + 128 * h;
          if (active) drain128(taddr, acc);
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(accempty(buf));
          buf ^= 1;
          const int g1 = g0 + mdgi::GROUP_STEPS;
          if (g1 % mdgi::CHUNK_STEPS == 0 || g1 >= S) {
            if (active) {
              int4 *dst = reinterpret_cast<int4 *>(jb.out + (size_t)chunk * jb.plane_c +
                                                   (size_t)row * jb.Np + col);
#pragma unroll
              for (int v = 0; v < 32; ++v) {
                dst[v] = make_int4(acc[4 * v], acc[4 * v + 1], acc[4 * v + 2], acc[4 * v + 3]);
                acc[4 * v] = acc[4 * v + 1] = acc[4 * v + 2] = acc[4 * v + 3] = 0;
              }
            }
            ++chunk;
          }
        }
      }
    }
  epi_done:;
  }
  __syncwarp();
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TMEM_COLS)
                 : "memory");
  if (threadIdx.x == 0 && *abort_flag) atomicExch(&g_tc_error, 1);
}


__global__ void __launch_bounds__(THREADS, 1)
    diag_gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA,
                        const __grid_constant__ CUtensorMap tmB, int s, int D, int Mp, int Np,
                        int KB, int *__restrict__ out, long long plane_c) {
  tc1_body(SingleJobs{&tmA, &tmB, s, D, Mp, Np, KB, out, plane_c});
}

// Many problems: a table of GroupedProblem in global memory (tensor maps
// included, 64-byte aligned), units numbered problem after problem and,
// within a problem, part after part (all tiles of one diagonal range, then
// the next range).
__device__ __forceinline__ const mdgi::GroupedProblem &grouped_find(
    const mdgi::GroupedProblem *probs, int count, int u) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].unit_begin <= u) lo = mid; else hi = mid - 1;
  }
  return probs[lo];
}

struct GroupedJobs {
  const mdgi::GroupedProblem *probs;
  int count, total;
  __device__ int tiles() const { return total; }
  __device__ TileJob job(int u) const {
    const mdgi::GroupedProblem &g = grouped_find(probs, count, u);
    const int lt = u - g.unit_begin, tiles = g.mt * g.nt;
    const int tile = lt % tiles, part = lt / tiles;
    int d0, d1;
    part_diagonals(g.s, g.D, part, g.parts, d0, d1);
    return TileJob{reinterpret_cast<const CUtensorMap *>(g.tmA),
                   reinterpret_cast<const CUtensorMap *>(g.tmB), g.s, g.D, g.Mp, g.Np, g.KB,
                   (tile % g.mt) * TM, (tile / g.mt) * g.tn, g.tn, g.ktail, d0, d1, g.out,
                   g.plane_c};
  }
};

__global__ void __launch_bounds__(THREADS, 1)
    diag_gemm_tc_grouped_kernel(const mdgi::GroupedProblem *__restrict__ probs, int count,
                                int total) {
  tc1_body(GroupedJobs{probs, count, total});
}

// ------------------------------------------------------------------------
// The same computation on CTA pairs (cta_group::2): a cluster of two CTAs
// owns a 256 x 256 output tile; CTA r holds rows r*128..+127 of the A
// k-block and rows r*128..+127 of the B k-block (the N half), and the pair's
// tensor cores compute M=256 N=256 K=16 per instruction, issued by one thread
// of the even CTA.  Each CTA streams 32 KiB per k-step instead of 48 and its
// tensor core reads 8 KiB of operands per 128-cycle MMA instead of 12, which
// halves the shared-memory traffic that bounds the single-CTA kernel.
// Synchronisation: both CTAs' TMA loads complete on the even CTA's full
// barrier (cp.async.bulk.tensor .cta_group::2); the even CTA's MMA commits
// arrive, multicast, on the empty and accumulator-full barriers of both
// CTAs; the epilogue warps of both CTAs arrive on the even CTA's
// accumulator-empty barrier (16 arrivals).  Each CTA's TMEM holds its 128
// rows of both accumulators.  Warps: 0 producer, 1 MMA issuer (even CTA),
// 2-9 epilogue, 10 the pacer (even CTA; see "Pacing across clusters").
// Work units are tiles, or parts of tiles (ranges of diagonals), taken in
// strips of `raster` column blocks.
constexpr int TN2 = 256, BH = 128;
constexpr int STAGES2 = 6;
constexpr int A2_BYTES = TM * TK * 2;  // 16 KiB
constexpr int B2_BYTES = BH * TK * 2;  // 16 KiB
constexpr int STAGE2_BYTES = A2_BYTES + B2_BYTES;
constexpr int SMEM2_BYTES = STAGES2 * STAGE2_BYTES + 1024 + 256;
constexpr uint32_t IDESC2 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN2 >> 3) << 17) |
                            ((uint32_t)(256 >> 4) << 24);

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ uint32_t map_to_rank0(uint32_t addr) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(r) : "r"(addr));
  return r;
}

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}

__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap *tm, int x, int y,
                                                 uint32_t bar_cluster) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar_cluster)
      : "memory");
}

__device__ __forceinline__ void mma_bf16_pair(uint32_t d_tmem, uint64_t a, uint64_t b,
                                              uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC2), "r"(acc));
}

__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
  const uint16_t mask = 3;
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
      "[%0], %1;" ::"r"(bar),
      "h"(mask)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster)
               : "memory");
}

// Pacing across clusters.  Clusters that keep the same pace read the same
// k-blocks of the same digit planes at about the same time, so each block
// comes from DRAM once and from L2 for the others; left alone they drift
// apart by more than L2 holds and most blocks come from DRAM again.  An
// eleventh warp of the even CTA (the pacer) publishes its producer's
// progress (k-steps issued, tagged with the launch's epoch) to a slot per
// cluster and posts, in shared memory, how far the producer may go: the
// slowest running cluster's progress plus `pace` k-steps.  The producer
// holds before a k-step beyond that.  Only the timing depends on it: a hold
// longer than PACE_WAIT_NS turns the pacing off for the rest of the launch
// in that CTA, so a cluster that is not resident (or a concurrent launch
// using the slots) costs at most that.
constexpr int PACE_EVERY = 32, PACE_SLOTS = 128;
constexpr int PACER_WARP = 2 + EPI_WARPS, THREADS2 = THREADS + 32;
constexpr unsigned long long PACE_WAIT_NS = 50000, PACE_STALE_NS = 2000000000ull;
constexpr uint32_t PACE_DONE = 0xFFFFFFFFu;
// 64 and 128 k-steps ran equally well on quad-double 4096^3 and 8192^3
// (8192^3: 289 ms per GEMM paced, 326 ms unpaced); 32 holds too often
constexpr int kDefaultPace = 64;
// one slot per 128-byte line, so that the clusters' stores and the pacers'
// polling spread over L2 slices instead of contending for a few lines
constexpr int PACE_STRIDE = 16;
constexpr unsigned PACE_POLL_NS = 2000;
__device__ unsigned long long g_pace[PACE_SLOTS * PACE_STRIDE];

__device__ __forceinline__ void pace_publish(int slot, uint32_t epoch, uint32_t steps) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(g_pace + slot * PACE_STRIDE),
               "l"(((unsigned long long)epoch << 32) | steps)
               : "memory");
}

// Published progress of a cluster in this launch (0 before it publishes).
__device__ __forceinline__ uint32_t pace_load(int slot, int ncl, uint32_t epoch) {
  if (slot >= ncl) return PACE_DONE;
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];"
               : "=l"(v)
               : "l"(g_pace + slot * PACE_STRIDE)
               : "memory");
  return (uint32_t)(v >> 32) == epoch ? (uint32_t)v : 0u;
}

// One unit of work of the pair kernel: a 256 x 256 tile of one problem
// (rows row0.., columns col0..) and the diagonals [d0, d1) it computes.
struct PairJob {
  const CUtensorMap *tmA, *tmB;
  int s, D, Mp, Np, KB, row0, col0, d0, d1;
  int *out;
  long long plane_c;
};

// A single problem: units are tiles, or parts of tiles (ranges of
// diagonals whose digit-pair counts add up to about 1/parts of the tile's
// work), taken in strips of `raster` column blocks: tiles run across a strip
// of `raster` column blocks, then down the rows, so that the clusters busy at
// the same time read few distinct A row blocks and B column blocks and share
// them in L2 (raster = 1 walks each column block top to bottom).
struct PairSingle {
  const CUtensorMap *tmA, *tmB;
  int s, D, Mp, Np, KB;
  int *out;
  long long plane_c;
  int parts, raster;
  __device__ int units() const { return (Mp / 256) * (Np / TN2) * parts; }
  __device__ PairJob job(int u) const {
    const int MB = Mp / 256, NB = Np / TN2, tiles = MB * NB;
    const int tile = u % tiles, part = u / tiles;
    int d0, d1;
    part_diagonals(s, D, part, parts, d0, d1);
    const int strip = tile / (MB * raster);
    const int idx = tile - strip * MB * raster;
    const int c0 = strip * raster;
    const int g = NB - c0 < raster ? NB - c0 : raster;
    const int rb = idx / g, cb = c0 + idx - rb * g;
    return PairJob{tmA, tmB, s, D, Mp, Np, KB, rb * 256, cb * TN2, d0, d1, out, plane_c};
  }
};

// Many problems (GroupedProblem table in global memory, tensor maps with
// 128-row boxes for A and B, Mp a multiple of 256): units are 256 x 256
// tiles times diagonal ranges, numbered as for the single-CTA kernel.
struct PairGrouped {
  const mdgi::GroupedProblem *probs;
  int count, total;
  __device__ int units() const { return total; }
  __device__ PairJob job(int u) const {
    const mdgi::GroupedProblem &g = grouped_find(probs, count, u);
    const int lt = u - g.unit_begin, tiles = g.mt * g.nt;
    const int tile = lt % tiles, part = lt / tiles;
    int d0, d1;
    part_diagonals(g.s, g.D, part, g.parts, d0, d1);
    return PairJob{reinterpret_cast<const CUtensorMap *>(g.tmA),
                   reinterpret_cast<const CUtensorMap *>(g.tmB), g.s, g.D, g.Mp, g.Np, g.KB,
                   (tile % g.mt) * 256, (tile / g.mt) * TN2, d0, d1, g.out, g.plane_c};
  }
};

template <class Jobs>
__device__ __forceinline__ void tc2_body(const Jobs &jobs, int pace, uint32_t epoch,
                                         int no_loads) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES2 * STAGE2_BYTES);
  // bars: STAGES2 full, STAGES2 empty, 2 accfull, 2 accempty, 1 drain, then
  // the TMEM address and the abort flag
  static_assert(2 * STAGES2 + 9 <= 32, "barrier area holds 32 words of 8 bytes");
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bars + 2 * STAGES2 + 5);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 2 * STAGES2 + 6);
  // pacing: k-steps issued by the producer (every PACE_EVERY), k-steps it
  // may issue (posted by the pacer warp)
  volatile uint32_t *pace_steps = reinterpret_cast<volatile uint32_t *>(bars + 2 * STAGES2 + 7);
  volatile uint32_t *pace_allowed = reinterpret_cast<volatile uint32_t *>(bars + 2 * STAGES2 + 8);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const bool leader = rank == 0;
  const uint32_t smem_base = smem_u32(smem);
  auto full = [&](int st) { return smem_u32(bars + st); };
  auto empty = [&](int st) { return smem_u32(bars + STAGES2 + st); };
  auto accfull = [&](int b) { return smem_u32(bars + 2 * STAGES2 + b); };
  auto accempty = [&](int b) { return smem_u32(bars + 2 * STAGES2 + 2 + b); };
  const uint32_t drain_bar = smem_u32(bars + 2 * STAGES2 + 4);

  if (threadIdx.x == 0) {
    for (int st = 0; st < STAGES2; ++st) {
      mbar_init(full(st), 1);
      mbar_init(empty(st), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accfull(b), 1);
      mbar_init(accempty(b), 2 * EPI_WARPS);
    }
    mbar_init(drain_bar, 1);
    *abort_flag = 0;
    *pace_steps = 0;
    *pace_allowed = PACE_DONE;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_holder)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  fence_before();
  cluster_sync();
  fence_after();
  const uint32_t tmem_base = *tmem_holder;

  const int units = jobs.units();
  const int cid = blockIdx.x >> 1, ncl = gridDim.x >> 1;
  const bool pacer = leader && pace > 0 && ncl <= PACE_SLOTS;
  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------ producer --
      int st = 0;
      uint32_t ph = 0;
      // per stage: a copy was issued (bit of `issued`), parity of its phase
      // (bit of `last_par`); bit masks so that they stay in registers
      uint32_t issued = 0, last_par = 0;
      bool pacing = pacer;
      uint32_t steps = 0;  // k-steps issued by this cluster
      // no_loads (self-test of the bounded waits): issue no copy, so the
      // MMA thread's wait for data runs out, it raises the abort flag and
      // every role leaves with nothing in flight
      for (int u = no_loads ? units : cid; u < units; u += ncl) {
        const PairJob jb = jobs.job(u);
        const int s = jb.s, KB = jb.KB;
        const int row = jb.row0 + (int)rank * TM;
        const int col = jb.col0 + (int)rank * BH;
        for (int d = jb.d0; d < jb.d1; ++d) {
          const int ilo = d - (s - 1) > 0 ? d - (s - 1) : 0;
          const int S = mdgi::diag_pairs(d, s) * KB;
          for (int t = 0; t < S; ++t) {
            const int i = ilo + t / KB, kb = t - (t / KB) * KB, j = d - i;
            if (pacing && steps > *pace_allowed) {
              const unsigned long long t0 = now_ns();
              while (steps > *pace_allowed) {
                if (*abort_flag) break;
                if (now_ns() - t0 > PACE_WAIT_NS) {
                  pacing = false;
                  break;
                }
              }
            }
            if (!mbar_wait(empty(st), ph ^ 1, abort_flag)) goto producer_done;
            if (leader) mbar_expect_tx(full(st), 2 * STAGE2_BYTES);
            const uint32_t a_dst = smem_base + st * STAGE2_BYTES;
            const uint32_t bar0 = map_to_rank0(full(st));
            tma_load_2d_pair(a_dst, jb.tmA, kb * TK, i * jb.Mp + row, bar0);
            tma_load_2d_pair(a_dst + A2_BYTES, jb.tmB, kb * TK, j * jb.Np + col, bar0);
            last_par = (last_par & ~(1u << st)) | (ph << st);
            issued |= 1u << st;
            if (++st == STAGES2) {
              st = 0;
              ph ^= 1;
            }
            if ((++steps & (PACE_EVERY - 1)) == 0) *pace_steps = steps;
          }
        }
      }
    producer_done:
      *pace_steps = PACE_DONE;
      if (*abort_flag && leader)
        for (int i = 0; i < STAGES2; ++i)
          if ((issued >> i) & 1u) mbar_drain(full(i), (last_par >> i) & 1u);
    }
  } else if (warp == 1) {
    if (lane == 0 && leader) {
      // ---------------------------------------------------- MMA issuer --
      int st = 0, buf = 0;
      uint32_t ph = 0, aph[2] = {0, 0};
      bool any = false;
      for (int u = cid; u < units; u += ncl) {
        const PairJob jb = jobs.job(u);
        for (int d = jb.d0; d < jb.d1; ++d) {
          const int S = mdgi::diag_pairs(d, jb.s) * jb.KB;
          for (int g0 = 0; g0 < S; g0 += mdgi::GROUP_STEPS) {
            if (!mbar_wait(accempty(buf), aph[buf] ^ 1, abort_flag)) goto mma_done;
            fence_after();
            const uint32_t dt = tmem_base + buf * TN2;
            const int g1 = g0 + mdgi::GROUP_STEPS < S ? g0 + mdgi::GROUP_STEPS : S;
            for (int t = g0; t < g1; ++t) {
              if (!mbar_wait(full(st), ph, abort_flag)) goto mma_done;
              fence_after();
              const uint32_t a_addr = smem_base + st * STAGE2_BYTES;
              const uint64_t da = sw128_desc(a_addr), db = sw128_desc(a_addr + A2_BYTES);
#pragma unroll
              for (int kk = 0; kk < TK / 16; ++kk)
                mma_bf16_pair(dt, da + 2 * kk, db + 2 * kk, (t > g0 || kk > 0) ? 1u : 0u);
              mma_commit_pair(empty(st));
              any = true;
              if (++st == STAGES2) {
                st = 0;
                ph ^= 1;
              }
            }
            mma_commit_pair(accfull(buf));
            aph[buf] ^= 1;
            buf ^= 1;
          }
        }
      }
    mma_done:
      if (*abort_flag && any) {
        mma_commit_pair(drain_bar);
        mbar_drain(drain_bar, 0);
      }
    }
  } else if (warp == PACER_WARP) {
    if (pacer) {
      // --------------------------------------------------------- pacer --
      // publishes the producer's progress and posts the number of k-steps
      // it may issue (slowest running cluster + pace) until the producer
      // is done; bounded by PACE_STALE_NS without news from the producer
      uint32_t last = 0;
      unsigned long long t_last = now_ns();
      while (true) {
        const uint32_t mine = __shfl_sync(0xffffffffu, *pace_steps, 0);
        if (mine != last) {
          last = mine;
          t_last = now_ns();
        }
        if (lane == 0) pace_publish(cid, epoch, mine);
        if (mine == PACE_DONE) break;
        uint32_t m = PACE_DONE;
#pragma unroll
        for (int k = 0; k < PACE_SLOTS / 32; ++k) m = min(m, pace_load(lane + 32 * k, ncl, epoch));
        m = __reduce_min_sync(0xffffffffu, m);
        if (lane == 0)
          *pace_allowed = m == PACE_DONE || m > PACE_DONE - (uint32_t)pace ? PACE_DONE
                                                                           : m + (uint32_t)pace;
        int stop = 0;
        if (lane == 0) stop = (*abort_flag || now_ns() - t_last > PACE_STALE_NS) ? 1 : 0;
        if (__shfl_sync(0xffffffffu, stop, 0)) break;
        __nanosleep(PACE_POLL_NS);
      }
      if (lane == 0) {
        *pace_allowed = PACE_DONE;
        pace_publish(cid, epoch, PACE_DONE);
      }
    }
  } else {
    // -------------------------------------------------------- epilogue --
    const int q = warp & 3, h = (warp - 2) >> 2;
    int acc[128];
#pragma unroll
    for (int j = 0; j < 128; ++j) acc[j] = 0;
    int buf = 0;
    uint32_t aph[2] = {0, 0};
    const uint32_t accempty0[2] = {map_to_rank0(accempty(0)), map_to_rank0(accempty(1))};
    for (int u = cid; u < units; u += ncl) {
      const PairJob jb = jobs.job(u);
      const int row = jb.row0 + (int)rank * TM + 32 * q + lane;
      const int col = jb.col0 + 128 * h;
      int chunk = 0;
      for (int d = 0; d < jb.d0; ++d) chunk += mdgi::diag_chunks(d, jb.s, jb.KB);
      for (int d = jb.d0; d < jb.d1; ++d) {
        const int S = mdgi::diag_pairs(d, jb.s) * jb.KB;
        for (int g0 = 0; g0 < S; g0 += mdgi::GROUP_STEPS) {
          int ok = 1;
          if (lane == 0) ok = mbar_wait(accfull(buf), aph[buf], abort_flag) ? 1 : 0;
          ok = __shfl_sync(0xffffffffu, ok, 0);
          if (!ok) goto epi_done;
          aph[buf] ^= 1;
          fence_after();
          const uint32_t taddr = tmem_base + ((uint32_t)(32 * q) << 16) + buf * TN2 + 128 * h;
          drain128(taddr, acc);
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_cluster(accempty0[buf]);
          buf ^= 1;
          const int g1 = g0 + mdgi::GROUP_STEPS;
          if (g1 % mdgi::CHUNK_STEPS == 0 || g1 >= S) {
            int4 *dst = reinterpret_cast<int4 *>(jb.out + (size_t)chunk * jb.plane_c +
                                                 (size_t)row * jb.Np + col);
#pragma unroll
            for (int v = 0; v < 32; ++v) {
              dst[v] = make_int4(acc[4 * v], acc[4 * v + 1], acc[4 * v + 2], acc[4 * v + 3]);
              acc[4 * v] = acc[4 * v + 1] = acc[4 * v + 2] = acc[4 * v + 3] = 0;
            }
            ++chunk;
          }
        }
      }
    }
  epi_done:;
  }
  __syncwarp();
  fence_before();
  cluster_sync();
  fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TMEM_COLS)
                 : "memory");
  if (threadIdx.x == 0 && *abort_flag) atomicExch(&g_tc_error, 1);
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS2, 1)
    diag_gemm_tc2_kernel(const __grid_constant__ CUtensorMap tmA,
                         const __grid_constant__ CUtensorMap tmB, int s, int D, int Mp, int Np,
                         int KB, int *__restrict__ out, long long plane_c, int parts,
                         int raster, int pace, uint32_t epoch, int no_loads) {
  tc2_body(PairSingle{&tmA, &tmB, s, D, Mp, Np, KB, out, plane_c, parts, raster}, pace, epoch,
           no_loads);
}

// The batched plan's grouped GEMM on CTA pairs (no pacing: the clusters work
// on different problems).
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS2, 1)
    diag_gemm_tc2_grouped_kernel(const mdgi::GroupedProblem *__restrict__ probs, int count,
                                 int total) {
  tc2_body(PairGrouped{probs, count, total}, 0, 0, 0);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // looked up once per process; the initialisation of a function-local
  // static is serialised between threads
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return static_cast<PFN_cuTensorMapEncodeTiled_v12000>(nullptr);
  }();
  return fn;
}

// 2-D map over `planes` planes of rows x Kp BF16 (row stride Kp), box
// 64 x box_rows, 128-byte swizzle.
int make_map(CUtensorMap *m, const void *base, int Kp, long long rows_total, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return MDG_ERROR_NOT_SUPPORTED;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows_total};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? MDG_SUCCESS : MDG_ERROR_NOT_SUPPORTED;
}

}  // namespace

namespace mdgi {

int launch_diag_gemm_tc(int s, int D, int Mp, int Np, int Kp, const void *dA, const void *dB,
                        int ld, long long plane_a, long long plane_b, int *chunks,
                        long long plane_c, int single, int parts_opt, int raster_opt,
                        cudaStream_t st, int pace_opt) {
  if (Mp % TM || Np % TN || Kp % TK || ld != Kp) return MDG_ERROR_INVALID_SIZE;
  if (plane_a != (long long)Mp * Kp || plane_b != (long long)Np * Kp) return MDG_ERROR_INVALID_SIZE;
  if ((reinterpret_cast<uintptr_t>(dA) | reinterpret_cast<uintptr_t>(dB)) & 15)
    return MDG_ERROR_INVALID_SIZE;
  // the CTA-pair kernel needs 256-row tiles
  const bool pair = (Mp % 256 == 0) && !single;
  CUtensorMap ma, mb;
  MDG_TRY(make_map(&ma, dA, Kp, (long long)s * Mp, TM));
  MDG_TRY(make_map(&mb, dB, Kp, (long long)s * Np, pair ? BH : TN));
  int dev = 0, sms = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  // per-device attribute, set on every launch (no process-wide record that
  // a second device or a second host thread could find stale)
  if (pair)
    MDG_TRY_CUDA(cudaFuncSetAttribute(diag_gemm_tc2_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2_BYTES));
  else
    MDG_TRY_CUDA(cudaFuncSetAttribute(diag_gemm_tc_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
  MDG_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (pair) {
    const int tiles = (Mp / 256) * (Np / TN2);
    // split tiles into `parts` diagonal ranges when that shrinks the idle
    // part of the last wave of clusters by more than it costs: each extra
    // part makes the work about 4 % slower (fitted to quad-double 4096^3 and
    // 8192^3: 1024 tiles on 76 clusters run best unsplit, 256 tiles best in
    // two parts)
    const int ncl = sms / 2;
    int parts = 1;
    double best = 0.0;
    for (int u = 1; u <= 8 && u <= D; ++u) {
      const long long units = (long long)tiles * u;
      const long long waves = (units + ncl - 1) / ncl;
      const double cost = (double)waves / u * (1.0 + 0.04 * (u - 1));
      if (u == 1 || cost < best) {
        best = cost;
        parts = u;
      }
    }
    if (parts_opt > 0) parts = std::min(8, parts_opt);
    // tile order: strips about sqrt(clusters) column blocks wide, so that
    // the tiles in work at one time span few row and column blocks (the
    // largest power of two not above sqrt(76) = 8.7 on 152 SMs)
    const int NB = Np / TN2;
    int raster = 1;
    while ((raster * 2) * (raster * 2) <= ncl) raster *= 2;
    if (raster_opt > 0) raster = raster_opt;
    raster = std::min(NB, raster);
    const long long units = (long long)tiles * parts;
    const int clusters = units < ncl ? (int)units : ncl;
    // pacing window in k-steps, 0 = off (MDG_TC_PACE overrides); every
    // launch gets its own epoch so that slots left by earlier launches read
    // as "not started"
    // With no more units than clusters every tile is in work at once and
    // the operands of the whole GEMM are read in one sweep: pacing has no
    // drift to correct there and only costs (qd 1024^3: 7 % slower paced), so
    // the default turns it off; an explicit window still applies.
    int pace = units <= ncl ? 0 : kDefaultPace;
    if (const char *e = std::getenv("MDG_TC_PACE")) pace = std::max(0, std::atoi(e));
    if (pace_opt > 0) pace = pace_opt;
    if (pace_opt < 0) pace = 0;
    static std::atomic<uint32_t> epochs{0};
    uint32_t epoch = ++epochs;
    if (epoch == 0) epoch = ++epochs;
    // MDG_TC_SELFTEST_NO_LOADS=1: the producers issue no copies, the waits
    // for data run out after their 2 s limit and mdg_device_status then
    // reports MDG_ERROR_TIMEOUT (a test of the failure path; the result
    // planes are not written)
    const char *nl = std::getenv("MDG_TC_SELFTEST_NO_LOADS");
    const int no_loads = (nl && *nl == '1') ? 1 : 0;
    diag_gemm_tc2_kernel<<<2 * clusters, THREADS2, SMEM2_BYTES, st>>>(
        ma, mb, s, D, Mp, Np, Kp / TK, chunks, plane_c, parts, raster, pace, epoch, no_loads);
  } else {
    const int tiles = (Mp / TM) * (Np / TN);
    const int grid = tiles < sms ? tiles : sms;
    diag_gemm_tc_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(ma, mb, s, D, Mp, Np, Kp / TK, chunks,
                                                           plane_c);
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

int encode_plane_map(void *map128, const void *base, int Kp, long long rows_total, int box_rows) {
  return make_map(reinterpret_cast<CUtensorMap *>(map128), base, Kp, rows_total, box_rows);
}

int launch_diag_gemm_grouped(const GroupedProblem *dev_probs, int count, int total_units,
                             int pair, cudaStream_t st) {
  if (total_units == 0) return MDG_SUCCESS;
  int dev = 0, sms = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  MDG_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (pair) {
    MDG_TRY_CUDA(cudaFuncSetAttribute(diag_gemm_tc2_grouped_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2_BYTES));
    const int ncl = sms / 2;
    const int clusters = total_units < ncl ? total_units : ncl;
    diag_gemm_tc2_grouped_kernel<<<2 * clusters, THREADS2, SMEM2_BYTES, st>>>(dev_probs, count,
                                                                            total_units);
  } else {
    MDG_TRY_CUDA(cudaFuncSetAttribute(diag_gemm_tc_grouped_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    const int grid = total_units < sms ? total_units : sms;
    diag_gemm_tc_grouped_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(dev_probs, count,
                                                                   total_units);
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

int tc_device_status() {
  MDG_TRY_CUDA(cudaDeviceSynchronize());
  int flag = 0, zero = 0;
  MDG_TRY_CUDA(cudaMemcpyFromSymbol(&flag, g_tc_error, sizeof(int)));
  if (flag) {
    MDG_TRY_CUDA(cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)));
    return MDG_ERROR_TIMEOUT;
  }
  return MDG_SUCCESS;
}

}  // namespace mdgi

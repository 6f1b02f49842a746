// Internal interface of the slice-digit form (slice_tc.cu, diag_gemm_tc.cu).
#pragma once

#include <string>

#include <cuda_runtime.h>
#include <stddef.h>

namespace mdgi {

// The diagonal sums are written as int32 "chunk" planes: the products of
// diagonal d (pairs_d digit pairs times Kp/64 k-steps of 64) are cut into
// runs of CHUNK_STEPS k-steps, at most 2032 x 64 = 130048 products of
// |d_i d_j| <= 2^14, so every chunk sum is an exact int32 with |sum| <=
// 2032 x 2^20 = 2130706432 < 2^31.  2032 is the longest run of 16-step
// flush groups that int32 holds: fewer chunk planes to write and to read
// back.  Chunks are numbered diagonal by diagonal.
constexpr int CHUNK_STEPS = 2032;
// k-steps of 64 per FP32 accumulator flush in the tcgen05 engines: 1024
// products of magnitude <= 2^14, so every partial sum is an integer with
// |sum| <= 2^24, exactly representable in FP32.
constexpr int GROUP_STEPS = 16;

__host__ __device__ inline int diag_pairs(int d, int s) {
  const int lo = d - (s - 1) > 0 ? d - (s - 1) : 0, hi = d < s - 1 ? d : s - 1;
  return hi - lo + 1;
}
__host__ __device__ inline int diag_chunks(int d, int s, int KB) {
  return (diag_pairs(d, s) * KB + CHUNK_STEPS - 1) / CHUNK_STEPS;
}
inline int total_chunks(int s, int D, int KB) {
  int c = 0;
  for (int d = 0; d < D; ++d) c += diag_chunks(d, s, KB);
  return c;
}

// Workspace layout of one slice-digit GEMM (byte offsets, 256-aligned).
struct SlicePlan {
  int p, s, D, m, n, k;
  int Mp, Np, Kp;  // padded to 256, 256, 64
  int chunks;
  long long plane_a, plane_b, plane_c;  // elements between digit / chunk planes
  size_t off_rowbits, off_colbits, off_E, off_F, off_dA, off_dB, off_Cd, total;
};

SlicePlan make_slice_plan(int p, int s, int D, int m, int n, int k);
int words_for(int s, int D);

// The FP64-DMMA slice-digit form (digits64.cu): default digits per P
// (19-bit), integer words, workspace layout and the whole GEMM.
struct Digits64Plan {
  int p, s, D, m, n, k;
  size_t off_rowbits, off_colbits, off_E, off_F, off_dA, off_dB, off_Cd, total;
};
int digits64_default(int p);
int words64_for(int s, int D);
Digits64Plan make_digits64_plan(int p, int s, int D, int m, int n, int k);
int run_digits64_gemm(const Digits64Plan &pl, const double *A, int lda, const double *B, int ldb,
                      double *C, int ldc, void *ws, cudaStream_t st);

int launch_scale_exponents(int p, int m, int n, int k, const double *A, int lda,
                           const double *B, int ldb, unsigned long long *rowbits,
                           unsigned long long *colbits, int *E, int *F, cudaStream_t st);
int launch_digits(int p, int s, int rows, int cols, const double *X, int ldx, const int *E,
                  int trans, void *planes, int ld_out, long long plane_stride, int rows_pad,
                  int cols_pad, cudaStream_t st);
// Engines write chunk planes of Mp x Np int32 (row stride Np).
// mma.sync engine (Mp % 128, Np % 64, Kp % 64)
int launch_diag_gemm_v0(int s, int D, int Mp, int Np, int Kp, const void *dA, const void *dB,
                        int ld, long long plane_a, long long plane_b, int *chunks,
                        long long plane_c, cudaStream_t st);
// tcgen05 engine (Mp % 128, Np % 256, Kp % 64, ld == Kp).  single: 1 forces
// 128 x 256 tiles on one CTA, 0 uses CTA pairs when Mp % 256 == 0.  parts:
// diagonal ranges per pair tile, 0 = chosen to fill the last wave.  raster:
// pair tiles run across strips this many 256-column blocks wide (0 = auto).
// pace: cross-cluster pacing window of the pair kernel in k-steps (0 = the
// default, or MDG_TC_PACE when set; -1 = off).
int launch_diag_gemm_tc(int s, int D, int Mp, int Np, int Kp, const void *dA, const void *dB,
                        int ld, long long plane_a, long long plane_b, int *chunks,
                        long long plane_c, int single, int parts, int raster, cudaStream_t st,
                        int pace = 0);
// Renormalisation for P limbs with NW-word integers, V columns per thread
// (instantiated in renorm_p{2,4,8,16}.cu).
template <int P>
int launch_renorm_p(int NW, int V, int s, int D, int KB, int m, int n, const int *chunks,
                    long long plane_c, int ldcd, const int *E, const int *F, double *C, int ldc,
                    cudaStream_t st);
int launch_renorm(int p, int s, int D, int KB, int m, int n, const int *chunks,
                  long long plane_c, int ldcd, const int *E, const int *F, double *C, int ldc,
                  cudaStream_t st);
// One problem of a grouped diagonal GEMM: the single-CTA tcgen05 kernel
// (tiles of 128 rows x tn columns, tn = 256 or 128) or the CTA-pair kernel
// (tiles of 256 x 256; B box of 128 rows, one half per CTA).  Tensor maps of
// its digit planes, sizes, first global work unit, row tiles mt and column
// tiles nt, parts per tile, output chunk planes.  The problem's units are
// its mt x nt tiles times `parts` ranges of diagonals (whose digit-pair
// counts add up to about 1/parts of a tile's pairs each), numbered part
// after part.  ktail: MMAs of K = 16 that reach data in the last 64-deep
// k-block (1..4; single-CTA kernel).  Lives in global memory, 64-byte
// aligned.
struct alignas(64) GroupedProblem {
  unsigned char tmA[128];  // CUtensorMap, A planes, box 64 x 128
  unsigned char tmB[128];  // CUtensorMap, B planes, box 64 x tn (pairs: 64 x 128)
  int s, D, Mp, Np, KB, unit_begin, tn, mt, nt, ktail, parts;
  int *out;
  long long plane_c;
};
int encode_plane_map(void *map128, const void *base, int Kp, long long rows_total, int box_rows);
// The batched plan's entries in the tuning cache (plan.cu), under the
// current device: the tile policy and split mode recorded for a batch key,
// if any (left alone otherwise; a record without a split mode sets only the
// policy), and a new record.
void tune_lookup_batch(const std::string &key, int *policy, int *split);
void tune_record_batch(const std::string &key, int policy, int split, double ms);
// pair: the CTA-pair kernel (Mp of every problem a multiple of 256).
int launch_diag_gemm_grouped(const GroupedProblem *dev_probs, int count, int total_units,
                             int pair, cudaStream_t st);

// Waits for the device; MDG_ERROR_TIMEOUT if a bounded wait of the tcgen05
// engine gave up since the last call (the flag is then cleared).
int tc_device_status();

// engine: 0 = mma.sync, 1 = tcgen05 auto tiles, 2 = tcgen05 single CTA,
// 3 = tcgen05 CTA pairs
int run_slice_gemm(const SlicePlan &pl, const double *A, int lda, const double *B, int ldb,
                   double *C, int ldc, void *ws, int engine, int parts, int raster,
                   cudaStream_t st, int pace = 0);

// run_slice_gemm in two parts, for callers that split A into row panels
// (the pipelined host path): slice_prepare_b computes the column exponents
// and digits of B once; slice_panel then computes rows (<= pl.m) rows of C
// from the matching rows of A.  Every row of C depends only on its row of A
// and on all of B, so panels give the bits of one run_slice_gemm.
int slice_prepare_b(const SlicePlan &pl, const double *B, int ldb, void *ws, cudaStream_t st);
int slice_panel(const SlicePlan &pl, int rows, const double *A, int lda, double *C, int ldc,
                void *ws, int engine, int parts, int raster, cudaStream_t st, int pace = 0);
// slice_panel in two parts, for callers that also split B into column
// strips (each with its own plan and workspace, prepared by
// slice_prepare_b): slice_panel_a computes the exponents and digits of
// rows (<= pla.m) rows of A into wsa; slice_block then computes those rows
// of C against the strip of plb / wsb (plans of equal m, k, s, D).  Every
// column of C depends only on its column of B, so blocks give the bits of
// one run_slice_gemm.
int slice_panel_a(const SlicePlan &pl, int rows, const double *A, int lda, void *ws,
                  cudaStream_t st);
int slice_block(const SlicePlan &pla, const void *wsa, const SlicePlan &plb, void *wsb, int rows,
                double *C, int ldc, int engine, int parts, int raster, cudaStream_t st,
                int pace = 0);

// Which engine mdg_gemm uses for the BF16 form (MDG_SLICE_ENGINE=0/1 overrides).
int default_engine();
// mdg_options.engine -> run_slice_gemm engine code.
int engine_choice(int opt);

}  // namespace mdgi

/*
 * mdgemm.h -- C ABI of the GB300 multi-double GEMM library (libmdgemm.so).
 *
 * Plain C types only: device pointers, sizes, a cudaStream_t passed as
 * void*.  Every entry point returns an mdg_status; none of them exits or
 * throws.  Matrices of P-doubles are row-major with the P limbs of one
 * entry contiguous, most significant first, the layout of the reference
 * (C++/TCcuda.cu:130-131): entry (r, c) limb l of a matrix with leading
 * dimension ld (in entries) is at  ptr[(r * ld + c) * P + l].
 *
 * Each function names the reference interface it replaces.  The reference
 * surface is C++ (C++/TCcuda.h:23-103, C++/floatybits.h:17-97); its
 * std::vector wrappers are provided on top of this ABI by TCcuda.h and
 * floatybits.h in this directory.
 */
#ifndef MDGEMM_H
#define MDGEMM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MDG_SUCCESS = 0,
  MDG_ERROR_INVALID_LIMBS = 1,  /* P not in {2, 4, 8, 16} (or not allowed for this call) */
  MDG_ERROR_INVALID_SIZE = 2,   /* negative size, leading dimension too small, size too large */
  MDG_ERROR_NULL_POINTER = 3,   /* a required pointer is NULL */
  MDG_ERROR_INVALID_FORM = 4,   /* unknown form or option value */
  MDG_ERROR_WORKSPACE = 5,      /* workspace missing or smaller than *_workspace_size */
  MDG_ERROR_CUDA = 6,           /* a CUDA call failed, see mdg_last_cuda_error() */
  MDG_ERROR_NOT_SUPPORTED = 7,  /* valid request the library cannot serve */
  MDG_ERROR_TIMEOUT = 8,        /* a bounded device-side wait gave up */
  MDG_ERROR_ALLOCATION = 9,     /* device or pinned allocation failed */
  MDG_ERROR_TOO_LARGE = 10      /* problem needs more than the fixed scratch of mdg_gemm_slice_static */
} mdg_status;

/* GEMM forms. */
enum {
  /* The plain multi-double GEMM on FP64 CUDA cores: one product and one
   * addition per step with the reference's arithmetic, bit for bit the
   * result of matmul{dd,qd,od,hd}f (TCcuda.cu:320-372) and of matmulTCnt
   * compiled without contraction (TCcuda.cu:248-302). */
  MDG_FORM_PLAIN = 0,
  /* The reference's own split method: every limb cut into 13-bit (or
   * 7-bit) FP64 slices (floatybits.cu:196,303,327), the truncated slice
   * convolution on FP64 DMMA tensor cores (TCtest.cu:21-46 against the
   * block-Toeplitz bigB2, TCcuda.cu:79-95), then the squeeze of the
   * partial sums (TCcuda.cu:876-958). */
  MDG_FORM_FP64_SPLIT = 1,
  /* Slice digits on BF16 tensor cores: exact 8-bit balanced digits per
   * operand with a shared exponent per row of A / column of B, exact
   * diagonal sums (FP32 accumulation flushed into integers before a partial
   * sum can pass 2^24: every 1024 products on tcgen05, every 256 on the
   * mma.sync engine), exact rounding back to P limbs.  No reference counterpart:
   * this is the tensor-core form the reference set out to build. */
  MDG_FORM_SLICE_BF16 = 2,
  /* The same slice-digit scheme on the FP64 tensor cores the reference
   * uses (DMMA, TCtest.cu:21-46): 19-bit balanced digits stored as doubles
   * (quad-double: 12 digits, 78 digit pairs), FP64 sums of at most 65536
   * products (exact), int64 diagonal sums, the same exact rounding.  It
   * reaches the BF16 form's accuracy, so the two tensor-core paths compare
   * at equal error bits.  mdg_options.slices / diagonals set its digits
   * (default mdg_default_fp64_digits). */
  MDG_FORM_FP64_DIGITS = 3
};

/* Options; a NULL pointer or zero fields mean the defaults. */
typedef struct {
  int slices;       /* digit forms: digits per operand (0: default for P) */
  int diagonals;    /* digit forms: diagonals kept, 1..2*slices-1 (0: = slices) */
  int split_kind;   /* FP64 form: 0 split4 (pp=4P), 1 split8 (pp=8P), 2 mixed dd (pp=12) */
  int split_exact;  /* FP64 form: 0 or 1 = exact slices (default), 2 = reference-compatible */
  int engine;       /* BF16 form: 0 auto, 1 tcgen05 128x256 tiles, 2 tcgen05 CTA pairs
                       256x256, 3 mma.sync (legacy tensor path) */
  int parts;        /* BF16 form, CTA pairs: diagonal ranges per tile (0: auto, 1..8) */
  int raster;       /* BF16 form, CTA pairs: tile order runs across strips this many
                       256-column blocks wide (0: auto) */
  int pace;         /* BF16 form, CTA pairs: cross-cluster pacing window in k-steps
                       (0: default 64, off when every tile runs in the first wave of
                       clusters, or MDG_TC_PACE when set; -1: off; at most 65536) */
} mdg_options;

/* One problem of a batched call. */
typedef struct {
  int p, m, n, k;
  const double *A;  /* device, m x k, leading dimension lda */
  const double *B;  /* device, k x n */
  double *C;        /* device, m x n */
  int lda, ldb, ldc;
} mdg_problem;

const char *mdg_status_string(int status);
/* Text of the last CUDA error seen by the calling thread ("" if none). */
const char *mdg_last_cuda_error(void);
int mdg_version(void);

/* Default number of BF16 digits for P limbs. */
int mdg_default_slices(int p);
/* Default number of 19-bit digits of MDG_FORM_FP64_DIGITS for P limbs
 * (6, 12, 24, 47 for P = 2, 4, 8, 16). */
int mdg_default_fp64_digits(int p);

/* ---------------------------------------------------------------- GEMM -- */

/* Bytes of device workspace mdg_gemm needs for this problem (0 for the
 * plain form).  Replaces the cudaMalloc calls inside matmulTCnt and
 * TCtest.cu:73-82, which the reference never frees. */
size_t mdg_gemm_workspace_size(int form, int p, int m, int n, int k,
                               const mdg_options *opt);

/* C = A * B, all device pointers, asynchronous on `stream`.
 * Replaces matmulTCnt (TCcuda.cu:248, form PLAIN) and the split GEMM of
 * TCtest.cu:48-114 (form FP64_SPLIT); any m, n, k >= 0. */
int mdg_gemm(int form, int p, int m, int n, int k, const double *A, int lda,
             const double *B, int ldb, double *C, int ldc,
             const mdg_options *opt, void *workspace, size_t workspace_bytes,
             void *stream);

/* C = op(A) op(B), or C = C (+) op(A) op(B) with accumulate = 1, where
 * op(A) = A (m x k, lda >= k) or, with trans_a = 1, the transpose of A
 * stored k x m (lda >= m); op(B) = B (k x n, ldb >= n) or, with trans_b = 1,
 * the transpose of B stored n x k (ldb >= k); (+) is the reference's
 * P-double addition (ddf_add for P = 2, else baileyAdd_fast,
 * quad_double_functions.cu:216).  The result equals mdg_gemm of the same
 * form on the transposed operands, then the addition; with k = 0 C is
 * cleared (or kept, when accumulating).  Extends the reference's square,
 * overwrite-only call (TCcuda.h:66).  Workspace: mdg_gemm_ex_workspace_size
 * (the inner GEMM's plus transposed copies and the product when needed). */
size_t mdg_gemm_ex_workspace_size(int form, int trans_a, int trans_b, int accumulate,
                                  int p, int m, int n, int k, const mdg_options *opt);
int mdg_gemm_ex(int form, int trans_a, int trans_b, int accumulate, int p, int m, int n,
                int k, const double *A, int lda, const double *B, int ldb, double *C,
                int ldc, const mdg_options *opt, void *workspace,
                size_t workspace_bytes, void *stream);

/* C = A * B with HOST buffers: copies in, computes, copies out, waits.
 * Device memory comes from a cache owned by the library (freed by
 * mdg_release_cache).  This is the call the std::vector wrappers make. */
int mdg_gemm_host(int form, int p, int m, int n, int k, const double *A,
                  const double *B, double *C, const mdg_options *opt);

/* Many independent problems with mixed P and sizes in one persistent
 * launch per stage (plain: one launch in all).  No reference counterpart
 * (the reference runs one square problem per call). */
size_t mdg_gemm_batched_workspace_size(int form, const mdg_problem *problems,
                                       int count, const mdg_options *opt);
int mdg_gemm_batched(int form, const mdg_problem *problems, int count,
                     const mdg_options *opt, void *workspace,
                     size_t workspace_bytes, void *stream);

void mdg_release_cache(void);

/* Page-locked host memory for the buffers of mdg_gemm_host (cudaHostAlloc,
 * portable to every device): copies from it run at the host link's full
 * rate, without the staging a pageable buffer needs.  *out is NULL on a
 * failure (MDG_ERROR_ALLOCATION).  Not in the reference, whose wrappers copy
 * from pageable std::vector storage. */
int mdg_host_alloc(size_t bytes, void **out);
void mdg_host_free(void *ptr);

/* Batched BF16 slice-digit GEMM as a reusable plan.  mdg_batch_create lays
 * out `workspace` (mdg_batch_workspace_size bytes) for these problems
 * (device pointers, P in {2,4,8,16}, m, n, k >= 1, default digits per P),
 * uploads the per-problem tables and tensor maps and returns a handle;
 * it synchronises `stream`.  mdg_batch_run only launches kernels (one for
 * the exponents of every row and column, one for the digits of every
 * operand, one grouped tcgen05 diagonal GEMM over the tiles of every
 * problem, and one renormalisation per limb count present) and may be
 * captured into a CUDA graph; each C equals the single-problem mdg_gemm
 * result bit for bit.  No counterpart in the reference. */
typedef struct mdg_batch_s *mdg_batch;
size_t mdg_batch_workspace_size(const mdg_problem *problems, int count);
int mdg_batch_create(const mdg_problem *problems, int count, void *workspace,
                     size_t workspace_bytes, void *stream, mdg_batch *out);
int mdg_batch_run(mdg_batch batch, void *stream);
void mdg_batch_destroy(mdg_batch batch);

/* Tile policies of the batched plan's diagonal GEMM: single-CTA tiles of
 * 128 rows by 256 columns only, by 128 columns only, or (auto) 128 columns
 * for the problems where that pads fewer columns (n mod 256 in 1..128), else
 * 256; or CTA pairs with 256 x 256 tiles (half the operand bytes per
 * product, rows padded to 256).  Every policy gives the same bits. */
enum {
  MDG_BATCH_TILES_AUTO = 0,
  MDG_BATCH_TILES_256 = 1,
  MDG_BATCH_TILES_128 = 2,
  MDG_BATCH_TILES_PAIR = 3
};
/* Re-deals the plan's tiles under `policy` (uploads the tile table and
 * synchronises `stream`; not during a capture).  mdg_batch_tiles returns
 * the policy in use; a new plan starts with the policy recorded by
 * mdg_batch_tune for its problem shapes, else MDG_BATCH_TILES_256. */
int mdg_batch_set_tiles(mdg_batch batch, int policy, void *stream);
int mdg_batch_tiles(mdg_batch batch);
/* Split mode of the diagonal GEMM's work: 0 = each tile is one unit; 1 =
 * heavy tiles are cut into ranges of diagonals, so that units carry about
 * equal work and the units of one problem run side by side on the GPU
 * (its digit planes then stay in L2 while they are reused).  Same bits
 * either way; uploads the table and synchronises `stream` like
 * mdg_batch_set_tiles.  mdg_batch_split returns the mode in use. */
int mdg_batch_set_split(mdg_batch batch, int split, void *stream);
int mdg_batch_split(mdg_batch batch);
/* Times one mdg_batch_run under each tile policy and split mode (after a
 * warm-up each), keeps the fastest and records it in the tuning cache under
 * the batch's problem shapes; mdg_batch_create starts later plans of the
 * same shapes with the recorded choice.  Synchronises `stream`. */
int mdg_batch_tune(mdg_batch batch, void *stream);

/* C = A * B in the BF16 slice-digit form (default digits) without any
 * device allocation and without a workspace argument, for callers that may
 * not call cudaMalloc: code running inside a stream capture owned by
 * another component, hosts that own every device allocation, real-time
 * integrations that forbid allocation after start-up.  No counterpart in
 * the reference.  The scratch is a fixed array of mdg_static_scratch_bytes()
 * (64 MiB) inside the library, held on every GPU that loads it; a problem
 * whose BF16 workspace (mdg_gemm_workspace_size) is larger gets
 * MDG_ERROR_TOO_LARGE (e.g. quad-double fits up to 512^3, octo-double up to
 * 256^3).  The first call in a CUDA context (the device's primary context,
 * or one the caller made current) looks up the array's device address and
 * should come before any stream capture; a context created later, e.g.
 * after cudaDeviceReset, gets its own lookup.  Calls share the array and it
 * keeps the last call's contents (each call writes every region it reads):
 * calls that overlap on the GPU race, so order them on one stream. */
size_t mdg_static_scratch_bytes(void);
int mdg_gemm_slice_static(int p, int m, int n, int k, const double *A, int lda,
                          const double *B, int ldb, double *C, int ldc,
                          void *stream);

/* ------------------------------------------------- FP64 split stages -- */

/* Slices of `count` P-doubles: kind 0 split4pd (floatybits.cu:196),
 * 1 split8pd (:303), 2 mixsplit2 (:327, P must be 2), 3 the unbalanced
 * split4pd of the CPU convolution driver (TCcudant.cpp:163).  exact = 0
 * gives the reference's slices bit for bit, quirks included (a negative
 * limb gives zero slices, the 53rd significand bit is dropped); exact = 1
 * keeps sign and all bits.  out: count x pp doubles (pp = 4P, 8P, 12, 4P). */
int mdg_split(int kind, int exact, int p, long long count, const double *x,
              double *out, void *stream);

/* The same slices as pp planes: slice j of entry e at planes[j * plane_stride
 * + e], plane_stride >= count.  With kind 3 this is splitp(split4pd(x), 4P)
 * of TCcudant.cpp:163-183 (without splitp's read one element past the end,
 * which shifts every plane after the first by one entry there). */
int mdg_split_planes(int kind, int exact, int p, long long count, const double *x,
                     double *planes, long long plane_stride, void *stream);

/* y_i = sum_j x[i*pp + j] through the P-double inc_d, j in order; y is
 * count x P.  Replaces pllsqueeze_old (TCcuda.cu:908) and its kernels
 * pllsqueeze_{2,4,8,16}_pp_old (TCcuda.cu:876-906); pp >= 1. */
int mdg_squeeze(int p, int pp, long long count, const double *x, double *y,
                void *stream);

/* Truncated slice convolution on FP64 tensor cores:
 * Cq[r][c][i] = sum_k sum_{j<=i} Aq[r][k][j] * Bq[k][c][i-j], Aq m x k x pp,
 * Bq k x n x pp, Cq m x n x pp (the reference's matmul kernel against
 * bigB2, TCtest.cu:21-46, TCcuda.cu:79-95, without forming bigB2). */
size_t mdg_slice_conv_workspace_size(int pp, int m, int n, int k);
int mdg_slice_conv(int pp, int m, int n, int k, const double *Aq,
                   const double *Bq, double *Cq, void *workspace,
                   size_t workspace_bytes, void *stream);

/* The same convolution on slice planes, the layout of the CPU convolution
 * driver: A is pp planes of m x k, B pp planes of k x n, C pp planes of
 * m x n (all row-major, planes contiguous); C_i = sum_{j<=i} A_j B_{i-j}.
 * Replaces manualconvmult (convmult2 + convadd2, TCcudant.cpp:216-250) and
 * directdotconv (TCcudant.cpp:252-276), which compute it in FP64 on one
 * core. */
int mdg_plane_conv(int pp, int m, int n, int k, const double *A,
                   const double *B, double *C, void *stream);

/* ----------------------------------------------- BF16 slice stages -- */

/* Scale exponents: E[r] for the rows of A (m x k), F[c] for the columns
 * of B (k x n); 2^E bounds every entry of the row. */
int mdg_scale_exponents(int p, int m, int n, int k, const double *A, int lda,
                        const double *B, int ldb, int *E, int *F,
                        void *stream);

/* Balanced base-256 digits of a P-double matrix as BF16 planes.
 * trans = 0: X is rows x cols (A), plane i is rows x ld_out row-major.
 * trans = 1: X is cols x rows (B, k x n), plane i is rows(n) x ld_out,
 * i.e. transposed so that both operands are K-major.  Planes are
 * plane_stride elements apart.  Values are the integers d in [-128, 128]. */
int mdg_slice_digits(int p, int s, int rows, int cols, const double *X,
                     int ldx, const int *E, int trans, void *planes,
                     int ld_out, long long plane_stride, void *stream);

/* Number of int32 chunk planes mdg_slice_diagonals writes: the products
 * of diagonal d (its digit pairs times k/64 steps of 64) are cut into runs
 * of 2032 steps, so each chunk holds at most 130048 products of magnitude
 * <= 2^14 and its sum is an exact int32 with |sum| <= 2032 * 2^20 < 2^31.
 * Diagonal d has mdg_slice_chunk_count(s, d + 1, k) -
 * mdg_slice_chunk_count(s, d, k) of them (0 for d = 0), numbered diagonal
 * by diagonal. */
int mdg_slice_chunk_count(int s, int D, int k);

/* Exact diagonal sums on BF16 tensor cores: for d < D the sum over i+j=d
 * and over k of dA_i[r][k] dB_j[c][k], written as chunk planes
 * chunks[q][r][c] (int32, m x n each, chunk q of diagonal d after those of
 * diagonals 0..d-1).  dA: s planes m x ld (plane_a >= m ld apart), dB: s
 * planes n x ld (plane_b >= n ld apart); m % 128 == 0, n % 256 == 0,
 * k % 64 == 0. */
int mdg_slice_diagonals(int s, int D, int m, int n, int k, const void *dA,
                        const void *dB, int ld, long long plane_a,
                        long long plane_b, int *chunks, void *stream);

/* C[r][c] = RN_P( sum_d C_d[r][c] 256^(D-1-d) ) * 2^(E[r]+F[c]-14-8(D-1)),
 * C_d the sum of the chunks of diagonal d (layout of mdg_slice_diagonals
 * for s digits and depth k; chunk planes are plane_c elements apart with
 * row stride ldcd); each limb is rounded to nearest. */
int mdg_renorm_diagonals(int p, int s, int D, int k, int m, int n,
                         const int *chunks, long long plane_c, int ldcd,
                         const int *E, const int *F, double *C, int ldc,
                         void *stream);

/* ------------------------------------------------- plans and tuning -- */

/* A plan for one problem shape: it owns its device workspace and the
 * schedule it runs with.  mdg_plan_tune times the schedules that give the
 * same bits (BF16 form: CTA pairs with diagonal ranges per tile auto / 1 /
 * 2 / 4, tile strips 4 or 16 column blocks wide, pacing windows 32 or 128
 * k-steps or none, and the single-CTA engine) on the caller's operands, keeps the
 * fastest, and records it in the library's tuning cache under the device
 * (GPU name and driver version) and the shape class (form, P, digits,
 * padded m, n, k); plans created later for the same class start from the
 * cached schedule.  Other forms have nothing to tune.  The cache persists
 * as a JSON file through mdg_tune_cache_save / mdg_tune_cache_load. */
typedef struct mdg_plan_s *mdg_plan;
int mdg_plan_create(int form, int p, int m, int n, int k, const mdg_options *opt,
                    mdg_plan *plan);
size_t mdg_plan_workspace_bytes(mdg_plan plan);
/* Runs every candidate once more after a warm-up on `stream` and waits
 * for it; C holds the product afterwards. */
int mdg_plan_tune(mdg_plan plan, const double *A, int lda, const double *B, int ldb,
                  double *C, int ldc, void *stream);
int mdg_plan_run(mdg_plan plan, const double *A, int lda, const double *B, int ldb,
                 double *C, int ldc, void *stream);
/* The options the plan runs with (engine, parts, raster, pace filled in). */
int mdg_plan_schedule(mdg_plan plan, mdg_options *out);
void mdg_plan_destroy(mdg_plan plan);
/* The tuning cache: {"<gpu>|<driver>": {"<form> <p> <s> <D> <Mp> <Np> <Kp>":
 * {"engine": e, "parts": q, "raster": r, "pace": w, "ms": t}, ...}, ...}, and
 * batched plans under "batch <count> <hash>": {"tiles": policy, "ms": t}.  Loading
 * merges into the cache; MDG_ERROR_NOT_SUPPORTED if the file cannot be
 * opened, MDG_ERROR_INVALID_FORM if it is not of that form. */
int mdg_tune_cache_load(const char *path);
int mdg_tune_cache_save(const char *path);
void mdg_tune_cache_clear(void);
int mdg_tune_cache_size(void);

/* ---------------------------------------------------- input generator -- */

/* Distributions of mdg_generate (low two bits of dist), and scale flags
 * that may be OR'ed onto MDG_GEN_UNIFORM or MDG_GEN_NORMAL. */
enum {
  MDG_GEN_UNIFORM = 0,     /* hi limb U[-1, 1); limb i+1 = U[-1, 1) * ulp(limb i) / 2;
                              then a bottom-up and a top-down quick-two-sum sweep */
  MDG_GEN_NORMAL = 1,      /* as UNIFORM with a hi limb of mean 0 and variance 1: the
                              Irwin-Hall sum of 12 uniforms minus 6, rounded once */
  MDG_GEN_REFERENCE = 2,   /* the reference's random_pd family (floatybits.cu:107-120):
                              limb i = f_i 2^(e - 52 i), f_i in [0.5, 1) with 52 fraction
                              bits, the first set; e = e0 + U{0 .. e1 - e0 - 1} (e0 when
                              e1 == e0); e0 >= -1021 + 52 (P - 1), e <= 1023 */
  MDG_GEN_SCALE_ROWS = 4,  /* then multiply row r by 2^U{e0 .. e1}, -64 <= e0 <= e1 <= 64 */
  MDG_GEN_SCALE_COLS = 8   /* then multiply column c by 2^U{e0 .. e1} (both flags: both) */
};

/* Fills the rows x cols P-double matrix X (device, leading dimension ldx
 * in entries) from `seed` with a counter-based generator (splitmix64 of
 * the seed, the entry index r * cols + c and the draw number): every entry
 * depends only on those, so any device, any launch shape and the CPU give
 * the same bits.  Builds inputs on the GPU instead of the host loops of
 * random_pd / mat (floatybits.cu:107-120, TCcuda.cu:14-21), for callers
 * that do not need the rand() sequence (the drop-in mat keeps it). */
int mdg_generate(int dist, int p, int rows, int cols, unsigned long long seed,
                 int e0, int e1, double *X, int ldx, void *stream);

/* Waits for the device and reports MDG_ERROR_TIMEOUT when a bounded wait
 * inside a tensor-core kernel gave up since the previous call (the record
 * is then cleared); MDG_SUCCESS otherwise. */
int mdg_device_status(void);

#ifdef __cplusplus
}
#endif

#endif /* MDGEMM_H */

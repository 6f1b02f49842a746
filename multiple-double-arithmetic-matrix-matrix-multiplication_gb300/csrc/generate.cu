// Counter-based generator of P-double test matrices (mdg_generate).
//
// Every value is made from 64-bit words w = mix(base(seed, entry) + j * G)
// (mix = the splitmix64 finaliser, G its golden-ratio increment, j the draw
// number) by integer arithmetic, exact scalings by powers of two and
// FP64 additions, so the bits depend only on (seed, entry index) and are
// the same on any GPU and on the CPU (this file is compiled with
// -fmad=false; the CPU build with -ffp-contract=off).
//
// * uniform U[-1, 1): k = w >> 11 (53 bits), (k - 2^52) 2^-52, exact.
// * hi limb of MDG_GEN_NORMAL: T = sum of twelve 53-bit k minus 6 2^53
//   (an exact int64), RN(T) 2^-53: the Irwin-Hall approximation of N(0, 1)
//   with one rounding.
// * tail limbs: x_{i+1} = u ulp(x_i) / 2 with ulp(x) = 2^(ilogb(x) - 52)
//   (0 for x = 0), then quick-two-sum sweeps bottom-up and top-down.
// * MDG_GEN_REFERENCE: the distribution of random_pd (floatybits.cu:107-120):
//   limb i = (2^51 + 51 random bits) 2^(e - 52 i - 52), e = e0 + offset.
// * row / column scales: 2^(e0 + w mod (e1 - e0 + 1)) from a separate
//   stream per row or column.
#include "common.cuh"

namespace {

constexpr uint64_t kGolden = 0x9e3779b97f4a7c15ull;

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += kGolden;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Stream bases: entries, row scales, column scales.
__device__ __forceinline__ uint64_t stream_base(uint64_t key, uint64_t index) {
  return mix64(key ^ (index * 0xd1342543de82ef95ull));
}

__device__ __forceinline__ uint64_t draw(uint64_t base, int j) {
  return mix64(base + (uint64_t)(j + 1) * kGolden);
}

__device__ __forceinline__ double uniform_pm1(uint64_t w) {
  const long long k = (long long)(w >> 11) - (1ll << 52);
  return ldexp((double)k, -52);
}

__device__ __forceinline__ double ulp_of(double x) {
  return x == 0.0 ? 0.0 : ldexp(1.0, ilogb(x) - 52);
}

__device__ __forceinline__ int scale_exponent(uint64_t w, int e0, int e1) {
  return e0 + (int)(w % (uint64_t)(e1 - e0 + 1));
}

template <int P>
__global__ void generate_kernel(int dist, int rows, int cols, uint64_t key_e, uint64_t key_r,
                                uint64_t key_c, int e0, int e1, double *__restrict__ X,
                                int ldx) {
  const long long total = (long long)rows * cols;
  const int kind = dist & 3;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / cols), c = (int)(e - (long long)r * cols);
    const uint64_t base = stream_base(key_e, (uint64_t)e);
    double x[P];
    if (kind == MDG_GEN_REFERENCE) {
      int ex = e0;
      if (e1 != e0) ex += (int)(draw(base, 0) % (uint64_t)(e1 - e0));
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const uint64_t frac = (1ull << 51) | (draw(base, 1 + i) >> 13);
        x[i] = ldexp((double)frac, ex - 52 * i - 52);
      }
    } else {
      int j = 0;
      if (kind == MDG_GEN_NORMAL) {
        long long t = -(6ll << 53);
        for (; j < 12; ++j) t += (long long)(draw(base, j) >> 11);
        x[0] = ldexp((double)t, -53);
      } else {
        x[0] = uniform_pm1(draw(base, j++));
      }
#pragma unroll
      for (int i = 1; i < P; ++i)
        x[i] = uniform_pm1(draw(base, j + i - 1)) * ulp_of(x[i - 1]) * 0.5;
#pragma unroll
      for (int i = P - 2; i >= 0; --i) {
        const double s = x[i] + x[i + 1];
        x[i + 1] = x[i + 1] - (s - x[i]);
        x[i] = s;
      }
#pragma unroll
      for (int i = 0; i < P - 1; ++i) {
        const double s = x[i] + x[i + 1];
        x[i + 1] = x[i + 1] - (s - x[i]);
        x[i] = s;
      }
      int sc = 0;
      if (dist & MDG_GEN_SCALE_ROWS)
        sc += scale_exponent(draw(stream_base(key_r, (uint64_t)r), 0), e0, e1);
      if (dist & MDG_GEN_SCALE_COLS)
        sc += scale_exponent(draw(stream_base(key_c, (uint64_t)c), 0), e0, e1);
      if (sc) {
#pragma unroll
        for (int i = 0; i < P; ++i) x[i] = ldexp(x[i], sc);
      }
    }
    double *out = X + ((size_t)r * ldx + c) * P;
#pragma unroll
    for (int i = 0; i < P; ++i) out[i] = x[i];
  }
}

}  // namespace

extern "C" int mdg_generate(int dist, int p, int rows, int cols, unsigned long long seed, int e0,
                            int e1, double *X, int ldx, void *stream) {
  if (!mdgi::valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (rows < 0 || cols < 0 || ldx < (cols > 1 ? cols : 1)) return MDG_ERROR_INVALID_SIZE;
  const int kind = dist & 3, flags = dist & ~3;
  if (kind == 3 || (flags & ~(MDG_GEN_SCALE_ROWS | MDG_GEN_SCALE_COLS)))
    return MDG_ERROR_INVALID_FORM;
  // reference family: every limb a normal double (limb i lies in
  // [2^(e - 52 i - 1), 2^(e - 52 i)) for e in [e0, max(e0, e1 - 1)])
  if (kind == MDG_GEN_REFERENCE &&
      (flags || e1 < e0 || e0 < -1021 + 52 * (p - 1) || (e1 > e0 ? e1 - 1 : e0) > 1023))
    return MDG_ERROR_INVALID_FORM;
  if (flags && (e1 < e0 || e0 < -64 || e1 > 64)) return MDG_ERROR_INVALID_FORM;
  if (rows == 0 || cols == 0) return MDG_SUCCESS;
  if (!X) return MDG_ERROR_NULL_POINTER;
  const uint64_t key = mix64(seed);
  const uint64_t key_e = mix64(key ^ 0x5851f42d4c957f2dull);
  const uint64_t key_r = mix64(key ^ 0xa0761d6478bd642full);
  const uint64_t key_c = mix64(key ^ 0xe7037ed1a0b428dbull);
  const long long total = (long long)rows * cols;
  int dev = 0, sms = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  MDG_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256;
  const long long want = (total + threads - 1) / threads;
  const int grid = (int)(want < 8ll * sms ? want : 8ll * sms);
  cudaStream_t st = mdgi::as_stream(stream);
  switch (p) {
    case 2:
      generate_kernel<2><<<grid, threads, 0, st>>>(dist, rows, cols, key_e, key_r, key_c, e0, e1,
                                                   X, ldx);
      break;
    case 4:
      generate_kernel<4><<<grid, threads, 0, st>>>(dist, rows, cols, key_e, key_r, key_c, e0, e1,
                                                   X, ldx);
      break;
    case 8:
      generate_kernel<8><<<grid, threads, 0, st>>>(dist, rows, cols, key_e, key_r, key_c, e0, e1,
                                                   X, ldx);
      break;
    default:
      generate_kernel<16><<<grid, threads, 0, st>>>(dist, rows, cols, key_e, key_r, key_c, e0,
                                                    e1, X, ldx);
  }
  MDG_TRY_LAUNCH();
  return MDG_SUCCESS;
}

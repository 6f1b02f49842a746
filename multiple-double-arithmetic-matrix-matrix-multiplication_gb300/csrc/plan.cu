// Plans for one problem shape and the schedule tuner (mdg_plan_*,
// mdg_tune_cache_*).
//
// A plan owns its device workspace and the mdg_options it runs with.  For
// the BF16 slice-digit form, mdg_plan_tune times the schedules that return
// the same bits (the CTA-pair engine with 0 = auto, 1, 2 or 4 diagonal ranges
// per tile, tile strips 4 or 16 column blocks wide, pacing windows of 32 and
// 128 k-steps or none, and the single-CTA engine) on the caller's own
// operands and keeps
// the fastest.  Choices live in a process-wide cache keyed by device ("<GPU
// name>|<driver version>") and shape class ("<form> <P> <s> <D> <Mp> <Np>
// <Kp>", the padded sizes the kernels see); mdg_tune_cache_save / _load keep
// it as a small JSON file.  Slice and diagonal counts change the rounding, so
// they stay the caller's options and are part of the key, not tuned.  The
// batched plan (batched.cu) records its tile policy and split mode here
// too, under "batch <count> <hash of the problem shapes>".
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

#include "common.cuh"
#include "slice_tc.cuh"

namespace {

// A single-problem schedule (engine, parts, raster, pace), or for a batched
// plan ("batch ..." keys) its tile policy and split mode (-1: not recorded).
struct TuneEntry {
  int engine = 0, parts = 0, raster = 0, pace = 0, tiles = 0, split = -1;
  double ms = 0.0;
};

std::mutex g_tune_mu;
std::map<std::string, std::map<std::string, TuneEntry>> g_tune;  // device -> shape -> entry

int device_key(std::string *out) {
  int dev = 0, drv = 0;
  MDG_TRY_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  MDG_TRY_CUDA(cudaGetDeviceProperties(&prop, dev));
  MDG_TRY_CUDA(cudaDriverGetVersion(&drv));
  *out = std::string(prop.name) + "|" + std::to_string(drv);
  return MDG_SUCCESS;
}

std::string shape_key(int form, int p, int m, int n, int k, const mdg_options *opt) {
  const int s = (opt && opt->slices) ? opt->slices
                : form == MDG_FORM_FP64_DIGITS ? mdg_default_fp64_digits(p)
                                               : mdg_default_slices(p);
  const int D = (opt && opt->diagonals) ? opt->diagonals : s;
  const mdgi::SlicePlan pl = mdgi::make_slice_plan(p, s, D, m, n, k);
  char buf[160];
  std::snprintf(buf, sizeof(buf), "%d %d %d %d %d %d %d", form, p, s, D, pl.Mp, pl.Np, pl.Kp);
  return buf;
}

// ---- the JSON form of the cache: objects of objects of numbers ----------
struct Json {
  const std::string &t;
  size_t i = 0;
  void ws() {
    while (i < t.size() && std::isspace((unsigned char)t[i])) ++i;
  }
  bool eat(char c) {
    ws();
    if (i < t.size() && t[i] == c) {
      ++i;
      return true;
    }
    return false;
  }
  bool str(std::string *out) {
    ws();
    if (i >= t.size() || t[i] != '"') return false;
    ++i;
    out->clear();
    while (i < t.size() && t[i] != '"') {
      if (t[i] == '\\' && i + 1 < t.size()) ++i;
      out->push_back(t[i++]);
    }
    if (i >= t.size()) return false;
    ++i;
    return true;
  }
  bool num(double *v) {
    ws();
    if (i >= t.size()) return false;
    char *end = nullptr;
    *v = std::strtod(t.c_str() + i, &end);
    const size_t used = (size_t)(end - (t.c_str() + i));
    if (!used) return false;
    i += used;
    return true;
  }
  // { "key": <value>, ... } with each value parsed by f
  template <class F>
  bool object(F f) {
    if (!eat('{')) return false;
    if (eat('}')) return true;
    do {
      std::string key;
      if (!str(&key) || !eat(':') || !f(key)) return false;
    } while (eat(','));
    return eat('}');
  }
};

// v is a whole number in [lo, hi] (NaN and infinities are not)
bool whole_in(double v, int lo, int hi, int *out) {
  if (!(v >= lo && v <= hi) || v != (double)(int)v) return false;
  *out = (int)v;
  return true;
}

std::string quoted(const std::string &s) {
  std::string q = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') q.push_back('\\');
    q.push_back(c);
  }
  return q + "\"";
}

}  // namespace

namespace mdgi {

void tune_lookup_batch(const std::string &key, int *policy, int *split) {
  std::string dev;
  if (device_key(&dev) != MDG_SUCCESS) return;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto d = g_tune.find(dev);
  if (d == g_tune.end()) return;
  auto e = d->second.find(key);
  if (e == d->second.end()) return;
  *policy = e->second.tiles;
  if (e->second.split >= 0) *split = e->second.split;
}

void tune_record_batch(const std::string &key, int policy, int split, double ms) {
  std::string dev;
  if (device_key(&dev) != MDG_SUCCESS) return;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  TuneEntry &t = g_tune[dev][key];
  t.tiles = policy;
  t.split = split;
  t.ms = ms;
}

}  // namespace mdgi

struct mdg_plan_s {
  int form, p, m, n, k;
  mdg_options opt;  // the caller's options, schedule fields filled in
  void *ws = nullptr;
  size_t bytes = 0;
  std::string dev_key, shape_key;
};

extern "C" {

int mdg_plan_create(int form, int p, int m, int n, int k, const mdg_options *opt,
                    mdg_plan *plan) {
  if (!plan) return MDG_ERROR_NULL_POINTER;
  *plan = nullptr;
  if (form < MDG_FORM_PLAIN || form > MDG_FORM_FP64_DIGITS) return MDG_ERROR_INVALID_FORM;
  if (!mdgi::valid_p(p)) return MDG_ERROR_INVALID_LIMBS;
  if (m < 0 || n < 0 || k < 0) return MDG_ERROR_INVALID_SIZE;
  const size_t bytes = mdg_gemm_workspace_size(form, p, m, n, k, opt);
  if (form != MDG_FORM_PLAIN && bytes == 0) return MDG_ERROR_INVALID_FORM;  // options rejected
  if (mdgi::alloc_over_limit(bytes)) return MDG_ERROR_ALLOCATION;
  auto *h = new mdg_plan_s();
  h->form = form;
  h->p = p;
  h->m = m;
  h->n = n;
  h->k = k;
  h->opt = opt ? *opt : mdg_options{};
  h->shape_key = shape_key(form, p, m, n, k, opt);
  int st = device_key(&h->dev_key);
  if (st == MDG_SUCCESS && form == MDG_FORM_SLICE_BF16 && !(opt && opt->engine)) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto d = g_tune.find(h->dev_key);
    if (d != g_tune.end()) {
      auto e = d->second.find(h->shape_key);
      if (e != d->second.end()) {
        h->opt.engine = e->second.engine;
        h->opt.parts = e->second.parts;
        h->opt.raster = e->second.raster;
        h->opt.pace = e->second.pace;
      }
    }
  }
  if (st == MDG_SUCCESS && bytes) {
    cudaError_t e = cudaMalloc(&h->ws, bytes);
    if (e != cudaSuccess) {
      mdgi::set_cuda_error(e);
      st = MDG_ERROR_ALLOCATION;
    }
    h->bytes = bytes;
  }
  if (st != MDG_SUCCESS) {
    delete h;
    return st;
  }
  *plan = h;
  return MDG_SUCCESS;
}

size_t mdg_plan_workspace_bytes(mdg_plan plan) { return plan ? plan->bytes : 0; }

int mdg_plan_run(mdg_plan plan, const double *A, int lda, const double *B, int ldb, double *C,
                 int ldc, void *stream) {
  if (!plan) return MDG_ERROR_NULL_POINTER;
  return mdg_gemm(plan->form, plan->p, plan->m, plan->n, plan->k, A, lda, B, ldb, C, ldc,
                  &plan->opt, plan->ws, plan->bytes, stream);
}

int mdg_plan_tune(mdg_plan plan, const double *A, int lda, const double *B, int ldb, double *C,
                  int ldc, void *stream) {
  if (!plan) return MDG_ERROR_NULL_POINTER;
  if (plan->form != MDG_FORM_SLICE_BF16 || plan->m == 0 || plan->n == 0 || plan->k == 0) {
    MDG_TRY(mdg_plan_run(plan, A, lda, B, ldb, C, ldc, stream));
    MDG_TRY_CUDA(cudaStreamSynchronize(mdgi::as_stream(stream)));
    return MDG_SUCCESS;
  }
  mdgi::NvtxRange range("mdg plan tune");
  // schedules with the same bits: CTA pairs (engine 2) with parts auto / 1 /
  // 2 / 4, tile strips of 4 and 16 column blocks, pacing windows 32, 128 and
  // off, and single CTAs (engine 1): {engine, parts, raster, pace}
  const int cand[10][4] = {{2, 0, 0, 0},  {2, 1, 0, 0},   {2, 2, 0, 0},  {2, 4, 0, 0},
                           {2, 0, 4, 0},  {2, 0, 16, 0},  {2, 0, 0, 32}, {2, 0, 0, 128},
                           {2, 0, 0, -1}, {1, 0, 0, 0}};
  cudaStream_t st = mdgi::as_stream(stream);
  cudaEvent_t e0, e1;
  MDG_TRY_CUDA(cudaEventCreate(&e0));
  MDG_TRY_CUDA(cudaEventCreate(&e1));
  mdg_options best = plan->opt;
  float best_ms = 0.0f;
  int status = MDG_SUCCESS;
  for (const auto &c : cand) {
    mdg_options o = plan->opt;
    o.engine = c[0];
    o.parts = c[1];
    o.raster = c[2];
    o.pace = c[3];
    status = mdg_gemm(plan->form, plan->p, plan->m, plan->n, plan->k, A, lda, B, ldb, C, ldc, &o,
                      plan->ws, plan->bytes, stream);  // warm-up
    if (status != MDG_SUCCESS) break;
    cudaEventRecord(e0, st);
    status = mdg_gemm(plan->form, plan->p, plan->m, plan->n, plan->k, A, lda, B, ldb, C, ldc, &o,
                      plan->ws, plan->bytes, stream);
    cudaEventRecord(e1, st);
    if (status != MDG_SUCCESS) break;
    float ms = 0.0f;
    if (cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      status = MDG_ERROR_CUDA;
      break;
    }
    if (best_ms == 0.0f || ms < best_ms) {
      best_ms = ms;
      best = o;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MDG_TRY(status);
  MDG_TRY(mdg_device_status());  // a bounded wait that gave up fails the tuning
  plan->opt = best;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    TuneEntry &t = g_tune[plan->dev_key][plan->shape_key];
    t.engine = best.engine;
    t.parts = best.parts;
    t.raster = best.raster;
    t.pace = best.pace;
    t.ms = best_ms;
  }
  return MDG_SUCCESS;
}

int mdg_plan_schedule(mdg_plan plan, mdg_options *out) {
  if (!plan || !out) return MDG_ERROR_NULL_POINTER;
  *out = plan->opt;
  return MDG_SUCCESS;
}

void mdg_plan_destroy(mdg_plan plan) {
  if (!plan) return;
  if (plan->ws) cudaFree(plan->ws);
  delete plan;
}

int mdg_tune_cache_load(const char *path) {
  if (!path) return MDG_ERROR_NULL_POINTER;
  FILE *f = std::fopen(path, "rb");
  if (!f) return MDG_ERROR_NOT_SUPPORTED;
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  std::fclose(f);
  std::map<std::string, std::map<std::string, TuneEntry>> parsed;
  Json js{text};
  const bool ok = js.object([&](const std::string &dev) {
    return js.object([&](const std::string &shape) {
      TuneEntry e;
      // schedule fields are whole numbers in the ranges mdg_gemm accepts, so
      // a loaded entry can never make a later plan of that shape fail
      const bool fields = js.object([&](const std::string &field) {
        double v;
        if (!js.num(&v)) return false;
        if (field == "engine") return whole_in(v, 0, 3, &e.engine);
        if (field == "parts") return whole_in(v, 0, 8, &e.parts);
        if (field == "raster") return whole_in(v, 0, 1 << 20, &e.raster);
        if (field == "pace") return whole_in(v, -1, 65536, &e.pace);
        if (field == "tiles") return whole_in(v, 0, 3, &e.tiles);
        if (field == "split") return whole_in(v, 0, 1, &e.split);
        if (field == "ms") {
          if (!(v >= 0.0 && v <= 1e12)) return false;
          e.ms = v;
        }
        return true;
      });
      if (fields) parsed[dev][shape] = e;
      return fields;
    });
  });
  js.ws();
  if (!ok || js.i != text.size()) return MDG_ERROR_INVALID_FORM;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (auto &d : parsed)
    for (auto &e : d.second) g_tune[d.first][e.first] = e.second;
  return MDG_SUCCESS;
}

int mdg_tune_cache_save(const char *path) {
  if (!path) return MDG_ERROR_NULL_POINTER;
  std::string out = "{";
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    bool first_dev = true;
    for (auto &d : g_tune) {
      out += (first_dev ? "\n  " : ",\n  ") + quoted(d.first) + ": {";
      first_dev = false;
      bool first = true;
      for (auto &e : d.second) {
        char buf[160];
        if (e.first.compare(0, 6, "batch ") == 0 && e.second.split >= 0)
          std::snprintf(buf, sizeof(buf), "{\"tiles\": %d, \"split\": %d, \"ms\": %.4f}",
                        e.second.tiles, e.second.split, e.second.ms);
        else if (e.first.compare(0, 6, "batch ") == 0)
          std::snprintf(buf, sizeof(buf), "{\"tiles\": %d, \"ms\": %.4f}", e.second.tiles,
                        e.second.ms);
        else
          std::snprintf(buf, sizeof(buf),
                        "{\"engine\": %d, \"parts\": %d, \"raster\": %d, \"pace\": %d, "
                        "\"ms\": %.4f}",
                        e.second.engine, e.second.parts, e.second.raster, e.second.pace,
                        e.second.ms);
        out += (first ? "\n    " : ",\n    ") + quoted(e.first) + ": " + buf;
        first = false;
      }
      out += "\n  }";
    }
  }
  out += "\n}\n";
  FILE *f = std::fopen(path, "wb");
  if (!f) return MDG_ERROR_NOT_SUPPORTED;
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  std::fclose(f);
  return ok ? MDG_SUCCESS : MDG_ERROR_NOT_SUPPORTED;
}

void mdg_tune_cache_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

int mdg_tune_cache_size(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int c = 0;
  for (auto &d : g_tune) c += (int)d.second.size();
  return c;
}

}  // extern "C"

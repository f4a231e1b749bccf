// selector.cu — GEMM tile configurations, the fixed size-threshold
// selector, the learned (MLP) selector and the exhaustive autotuner.
//
// portBLAS picks its GEMM tile at compile time from size thresholds per
// element type (src/interface/blas3/backend/nvidia_gpu.hpp:116-171) and
// tunes offline with a compile-time sweep (tools/auto_tuner).  Here every
// configuration is compiled in and chosen per call:
//   configs  0..19  FP32 SIMT, CTA tile {128x128, 128x64, 64x128, 64x64} x
//                   split-K {1, 2, 4, 8, 16}
//   configs 20..39  FP32 as 3-term split-BF16 on tcgen05, N tile {128, 64} x
//                   split-K {1, 2, 4, 8, 16} x raster {grouped (16 tile rows
//                   down M, then along N), down M}
//   configs 40..59  FP64 SIMT, CTA tile {128x128, 128x64, 64x128, 64x64} x
//                   split-K {1, 2, 4, 8, 16}
// All FP32 configs are FP32-accurate, so AUTO may pick any of them.  The
// learned selector is one small MLP for both element types (features ->
// 3 x 64 GELU -> predicted log2 of the time relative to the best config, one
// output per config; the element type is a one-hot input, and the pick is
// the best predicted config of the call's element type); its weights are
// trained by the project's own CUDA kernels (mlp.cu) on autotuner timings
// and loaded from a file.  Exhaustive autotuning (time every config of the
// element type) stays available and its winners override the model for the
// shapes it has seen.
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "selector.h"

namespace gb {

struct SgemmConfig {
  int method;  // 0 FP32 SIMT, 1 split-BF16 x6, 2 FP64 SIMT
  int tile_m, tile_n;
  int split;
  int raster_m;
};

static const int kSplits[5] = {1, 2, 4, 8, 16};

static SgemmConfig simt_config(int i, int method) {
  static const int tm[4] = {128, 128, 64, 64}, tn[4] = {128, 64, 128, 64};
  SgemmConfig s{};
  s.method = method;
  s.tile_m = tm[i / 5];
  s.tile_n = tn[i / 5];
  s.split = kSplits[i % 5];
  return s;
}

static SgemmConfig config_of(int c) {
  if (c < 20) return simt_config(c, 0);
  if (c >= kDgemmFirst) return simt_config(c - kDgemmFirst, 2);
  SgemmConfig s{};
  const int i = c - 20;
  s.method = 1;
  s.tile_m = 128;
  s.tile_n = i < 10 ? 128 : 64;
  s.split = kSplits[(i % 10) / 2];
  s.raster_m = i % 2 ? 1 : 2;  // raster codes of launch_gemm_split_bf16_cfg
  return s;
}

static int simt_tile_id(const SgemmConfig& s) {
  return s.tile_m == 128 ? (s.tile_n == 128 ? kSimtTile128x128 : kSimtTile128x64)
                         : (s.tile_n == 128 ? kSimtTile64x128 : kSimtTile64x64);
}

gbblas_status_t launch_sgemm_config(gbblas_handle_t h, const GemmArgs<float>& g, int config) {
  if (config < 0 || config >= kSgemmConfigs) return fail(GBBLAS_STATUS_INVALID_ARG, "sgemm: unknown config");
  const SgemmConfig s = config_of(config);
  if (s.method == 0) return launch_gemm_simt_tiled(h, g, simt_tile_id(s), s.split);
  return launch_gemm_split_bf16_cfg(h, g, 3, s.tile_n, s.split, s.raster_m);
}

gbblas_status_t launch_dgemm_config(gbblas_handle_t h, const GemmArgs<double>& g, int config) {
  if (config < kDgemmFirst || config >= kGemmConfigs) return fail(GBBLAS_STATUS_INVALID_ARG, "dgemm: unknown config");
  const SgemmConfig s = config_of(config);
  return launch_gemm_simt_tiled(h, g, simt_tile_id(s), s.split);
}

// ------------------------------------------------------------- features --
void gemm_features(int64_t m, int64_t n, int64_t k, int ta, int tb, int64_t lda, int64_t ldb, int64_t ldc,
                   int64_t batch, int dtype, float* f) {
  auto lg = [](int64_t v) { return float(std::log2(double(v < 1 ? 1 : v))) / 14.0f; };
  f[0] = lg(m);
  f[1] = lg(n);
  f[2] = lg(k);
  f[3] = float(ta != 0);
  f[4] = float(tb != 0);
  f[5] = float(lda % 16) / 16.0f;
  f[6] = float(ldb % 16) / 16.0f;
  f[7] = float(ldc % 16) / 16.0f;
  f[8] = lg(batch) * 14.0f / 10.0f;
  f[9] = dtype == kSelF32 ? 1.0f : 0.0f;   // element type one-hot: FP32
  f[10] = dtype == kSelF64 ? 1.0f : 0.0f;  //                       FP64
}

// -------------------------------------------------- fixed heuristic selector --
// The size thresholds of portBLAS's NVIDIA backend (batched -> small tile;
// M, N <= 256 -> small; <= 1024 -> medium; <= 2048 -> large; else the
// largest), mapped onto this config space with the tensor-core kernel as the
// largest tier.
int heuristic_config(int64_t m, int64_t n, int64_t batch, int dtype) {
  const int64_t mx = m > n ? m : n;
  if (dtype == kSelF64) {  // SIMT tiles only: 64x64, 128x64, 128x128 by size
    if (batch > 1 || mx <= 256) return kDgemmFirst + 15;
    if (mx <= 1024) return kDgemmFirst + 5;
    return kDgemmFirst;
  }
  if (batch > 1) return 15;                   // SIMT 64x64
  if (mx <= 256) return 15;                   // SIMT 64x64
  if (mx <= 1024) return 5;                   // SIMT 128x64
  if (mx <= 2048) return 0;                   // SIMT 128x128
  return 20;                                  // tcgen05 x6, N tile 128
}

// --------------------------------------------------------- MLP selector --
struct MlpSelector {
  bool loaded = false;
  int in = 0, hid = 0, out = 0;
  std::vector<float> p;  // W1 b1 W2 b2 W3 b3 W4 b4 (row-major out x in)
  std::string path;
};

static MlpSelector& selector() {
  static MlpSelector s;
  return s;
}

static inline float gelu(float x) { return 0.5f * x * (1.0f + std::erf(x * 0.70710678118654752f)); }

// Forward pass on the host (the same math as mlp.cu's kernels) -> the
// config in [lo, hi) with the smallest prediction.
static int mlp_pick(const MlpSelector& s, const float* f, int lo, int hi) {
  std::vector<float> a(f, f + s.in), z;
  const float* w = s.p.data();
  int din = s.in;
  for (int layer = 0; layer < 4; ++layer) {
    const int dout = layer < 3 ? s.hid : s.out;
    z.assign(size_t(dout), 0.f);
    const float* b = w + size_t(dout) * din;
    for (int o = 0; o < dout; ++o) {
      float acc = b[o];
      for (int i = 0; i < din; ++i) acc += w[size_t(o) * din + i] * a[size_t(i)];
      z[size_t(o)] = layer < 3 ? gelu(acc) : acc;
    }
    w = b + dout;
    a = z;
    din = dout;
  }
  int best = lo;
  for (int c = lo + 1; c < hi; ++c)
    if (a[size_t(c)] < a[size_t(best)]) best = c;
  return best;
}

// File format: "GBMLP\0\0\0", int32 in, hidden, out, then the packed FP32
// parameters (little-endian).
static bool load_selector_file(const std::string& path, MlpSelector& s) {
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) return false;
  char magic[8];
  int32_t dims[3];
  bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, "GBMLP\0\0\0", 8) == 0 &&
            std::fread(dims, 4, 3, fp) == 3 && dims[0] == kSgemmFeatures && dims[1] > 0 && dims[1] <= 1024 &&
            dims[2] == kGemmConfigs;
  if (ok) {
    const size_t cnt = size_t(dims[1]) * (dims[0] + 1) + 2 * size_t(dims[1]) * (dims[1] + 1) +
                       size_t(dims[2]) * (dims[1] + 1);
    s.p.resize(cnt);
    ok = std::fread(s.p.data(), 4, cnt, fp) == cnt;
    s.in = dims[0];
    s.hid = dims[1];
    s.out = dims[2];
  }
  std::fclose(fp);
  s.loaded = ok;
  if (ok) s.path = path;
  return ok;
}

// Default weights: $GBBLAS_SGEMM_SELECTOR, else tuning/gemm_selector.bin
// next to the package directory that holds libgbblas.so.
static void load_default_selector() {
  static bool tried = false;
  if (tried) return;
  tried = true;
  if (const char* env = std::getenv("GBBLAS_SGEMM_SELECTOR")) {
    if (std::strcmp(env, "off") == 0) return;
    load_selector_file(env, selector());
    return;
  }
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&heuristic_config), &info) && info.dli_fname) {
    std::string lib(info.dli_fname);
    const size_t slash = lib.rfind('/');
    const std::string dir = slash == std::string::npos ? std::string(".") : lib.substr(0, slash);
    load_selector_file(dir + "/../tuning/gemm_selector.bin", selector());
  }
}

// autotuned winners: key -> config
static std::mutex g_tuned_mu;
static std::unordered_map<std::string, int>& tuned() {
  static std::unordered_map<std::string, int> t;
  return t;
}
template <typename T>
static std::string shape_key(const GemmArgs<T>& g) {
  char buf[168];
  std::snprintf(buf, sizeof buf, "%d:%d%d:%lld:%lld:%lld:%lld:%lld:%lld:%lld", int(sizeof(T)), int(g.ta), int(g.tb),
                (long long)g.m, (long long)g.n, (long long)g.k, (long long)(g.lda % 16), (long long)(g.ldb % 16),
                (long long)(g.ldc % 16), (long long)g.batch);
  return buf;
}

// the network's picks, per shape key (every input of the network is part of
// the key, so a remembered pick is the one the network would make again);
// cleared when it grows past kPickCacheMax entries
static std::unordered_map<std::string, int>& picked() {
  static std::unordered_map<std::string, int> t;
  return t;
}
constexpr size_t kPickCacheMax = 4096;

template <typename T>
static int select_config(const GemmArgs<T>& g) {
  const int dtype = sizeof(T) == 8 ? kSelF64 : kSelF32;
  const std::string key = shape_key(g);
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    auto it = tuned().find(key);
    if (it != tuned().end()) return it->second;
    auto ip = picked().find(key);
    if (ip != picked().end()) return ip->second;
  }
  load_default_selector();
  const MlpSelector& s = selector();
  if (s.loaded) {
    float f[kSgemmFeatures];
    gemm_features(g.m, g.n, g.k, g.ta, g.tb, g.lda, g.ldb, g.ldc, g.batch, dtype, f);
    const int c = dtype == kSelF64 ? mlp_pick(s, f, kDgemmFirst, kGemmConfigs) : mlp_pick(s, f, 0, kSgemmConfigs);
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    if (picked().size() >= kPickCacheMax) picked().clear();
    picked()[key] = c;
    return c;
  }
  return heuristic_config(g.m, g.n, g.batch, dtype);
}

int select_sgemm_config(gbblas_handle_t, const GemmArgs<float>& g) { return select_config(g); }

bool has_tuned_config(const GemmArgs<float>& g) {
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  return tuned().count(shape_key(g)) != 0;
}
int select_dgemm_config(gbblas_handle_t, const GemmArgs<double>& g) { return select_config(g); }

static gbblas_status_t launch_config(gbblas_handle_t h, const GemmArgs<float>& g, int c) {
  return launch_sgemm_config(h, g, c);
}
static gbblas_status_t launch_config(gbblas_handle_t h, const GemmArgs<double>& g, int c) {
  return launch_dgemm_config(h, g, c);
}

// Times every config of the element type on this shape (operands in a
// zero-filled buffer of their own), remembers the winner for AUTO.
template <typename T>
static gbblas_status_t autotune(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k, int64_t lda,
                                int64_t ldb, int64_t ldc, int64_t batch, int reps, int* best_config, float* best_ms) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "autotune: null handle");
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0) return fail(GBBLAS_STATUS_INVALID_ARG, "autotune: bad dimension");
  const bool tra = (ta | 0x20) != 'n', trb = (tb | 0x20) != 'n';
  const int64_t sa = tra ? m * lda : k * lda, sbs = trb ? k * ldb : n * ldb, sc = n * ldc;
  // operands live in their own buffer: the configs themselves use temp memory
  T* buf = nullptr;
  const size_t elems = size_t(sa + sbs + sc) * size_t(batch);
  GB_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&buf), elems * sizeof(T), h->stream));
  GB_CUDA_TRY(cudaMemsetAsync(buf, 0, elems * sizeof(T), h->stream));
  GemmArgs<T> g{tra, trb, m, n, k, T(1), T(0), buf, lda, sa, buf + sa * batch, ldb, sbs,
                buf + (sa + sbs) * batch, ldc, sc, batch};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = -1;
  float bms = 0.f;
  const int lo = sizeof(T) == 8 ? kDgemmFirst : 0, hi = sizeof(T) == 8 ? kGemmConfigs : kSgemmConfigs;
  for (int c = lo; c < hi; ++c) {
    if (launch_config(h, g, c) != GBBLAS_STATUS_SUCCESS) {
      clear_error();
      continue;
    }
    cudaEventRecord(e0, h->stream);
    for (int r = 0; r < (reps > 0 ? reps : 1); ++r) launch_config(h, g, c);
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= float(reps > 0 ? reps : 1);
    if (best < 0 || ms < bms) {
      best = c;
      bms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, h->stream);
  GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (best < 0) return fail(GBBLAS_STATUS_UNSUPPORTED, "autotune: no config ran");
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    tuned()[shape_key(g)] = best;
  }
  if (best_config) *best_config = best;
  if (best_ms) *best_ms = bms;
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
static gbblas_status_t run_config(gbblas_handle_t h, int config, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                  T alpha, const T* a, int64_t lda, int64_t sa, const T* b, int64_t ldb,
                                  int64_t sbs, T beta, T* c, int64_t ldc, int64_t sc, int64_t batch) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "gemm_config: null handle");
  if (m < 0 || n < 0 || k < 0 || batch < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm_config: bad dimension");
  if (m == 0 || n == 0 || batch == 0) return GBBLAS_STATUS_SUCCESS;
  const char la = char(ta | 0x20), lb = char(tb | 0x20);
  if (la != 'n' && la != 't' && la != 'c') return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransA");
  if (lb != 'n' && lb != 't' && lb != 'c') return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransB");
  GemmArgs<T> g{la != 'n', lb != 'n', m, n, k, alpha, beta, a, lda, sa, b, ldb, sbs, c, ldc, sc, batch};
  return launch_config(h, g, config);
}

}  // namespace gb

using namespace gb;

extern "C" {

int gbblas_sgemm_config_count(void) { return kSgemmConfigs; }
int gbblas_gemm_config_count(void) { return kGemmConfigs; }

gbblas_status_t gbblas_sgemm_config_info(int config, int* method, int* tile_m, int* tile_n, int* split,
                                         int* raster_m) {
  if (config < 0 || config >= kGemmConfigs) return fail(GBBLAS_STATUS_INVALID_ARG, "unknown config");
  const SgemmConfig s = config_of(config);
  if (method) *method = s.method;
  if (tile_m) *tile_m = s.tile_m;
  if (tile_n) *tile_n = s.tile_n;
  if (split) *split = s.split;
  if (raster_m) *raster_m = s.raster_m;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_gemm_features(int dtype, int64_t m, int64_t n, int64_t k, char transa, char transb,
                                     int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, float* out) {
  if (!out) return fail(GBBLAS_STATUS_INVALID_ARG, "features: null output");
  if (dtype != GBBLAS_DTYPE_F32 && dtype != GBBLAS_DTYPE_F64)
    return fail(GBBLAS_STATUS_INVALID_ARG, "features: element type must be F32 or F64");
  gemm_features(m, n, k, (transa | 0x20) != 'n', (transb | 0x20) != 'n', lda, ldb, ldc, batch,
                dtype == GBBLAS_DTYPE_F64 ? kSelF64 : kSelF32, out);
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_sgemm_features(int64_t m, int64_t n, int64_t k, char transa, char transb, int64_t lda,
                                      int64_t ldb, int64_t ldc, int64_t batch, float* out) {
  return gbblas_gemm_features(GBBLAS_DTYPE_F32, m, n, k, transa, transb, lda, ldb, ldc, batch, out);
}

int gbblas_sgemm_heuristic_config(int64_t m, int64_t n, int64_t k, int64_t batch) {
  (void)k;
  return heuristic_config(m, n, batch, kSelF32);
}

int gbblas_gemm_heuristic_config(int dtype, int64_t m, int64_t n, int64_t k, int64_t batch) {
  (void)k;
  return heuristic_config(m, n, batch, dtype == GBBLAS_DTYPE_F64 ? kSelF64 : kSelF32);
}

gbblas_status_t gbblas_sgemm_load_selector(const char* path) {
  clear_error();
  MlpSelector s;
  if (!path || !load_selector_file(path, s)) return fail(GBBLAS_STATUS_INVALID_ARG, "selector: cannot load weights");
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  selector() = s;
  picked().clear();  // the new weights pick afresh
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_gemm_selector_pick(int dtype, int64_t m, int64_t n, int64_t k, char transa, char transb,
                                          int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, int* config) {
  clear_error();
  if (!config) return fail(GBBLAS_STATUS_INVALID_ARG, "selector: null output");
  if (dtype != GBBLAS_DTYPE_F32 && dtype != GBBLAS_DTYPE_F64)
    return fail(GBBLAS_STATUS_INVALID_ARG, "selector: element type must be F32 or F64");
  if (dtype == GBBLAS_DTYPE_F64) {
    GemmArgs<double> g{};
    g.ta = (transa | 0x20) != 'n';
    g.tb = (transb | 0x20) != 'n';
    g.m = m, g.n = n, g.k = k, g.lda = lda, g.ldb = ldb, g.ldc = ldc, g.batch = batch;
    *config = select_config(g);
  } else {
    GemmArgs<float> g{};
    g.ta = (transa | 0x20) != 'n';
    g.tb = (transb | 0x20) != 'n';
    g.m = m, g.n = n, g.k = k, g.lda = lda, g.ldb = ldb, g.ldc = ldc, g.batch = batch;
    *config = select_config(g);
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_sgemm_selector_pick(int64_t m, int64_t n, int64_t k, char transa, char transb, int64_t lda,
                                           int64_t ldb, int64_t ldc, int64_t batch, int* config) {
  return gbblas_gemm_selector_pick(GBBLAS_DTYPE_F32, m, n, k, transa, transb, lda, ldb, ldc, batch, config);
}

gbblas_status_t gbblas_sgemm_strided_batched_config(gbblas_handle_t h, int config, char ta, char tb, int64_t m,
                                                    int64_t n, int64_t k, float alpha, const float* a,
                                                    int64_t lda, int64_t sa, const float* b, int64_t ldb,
                                                    int64_t sbs, float beta, float* c, int64_t ldc, int64_t sc,
                                                    int64_t batch) {
  return run_config<float>(h, config, ta, tb, m, n, k, alpha, a, lda, sa, b, ldb, sbs, beta, c, ldc, sc, batch);
}

gbblas_status_t gbblas_dgemm_strided_batched_config(gbblas_handle_t h, int config, char ta, char tb, int64_t m,
                                                    int64_t n, int64_t k, double alpha, const double* a,
                                                    int64_t lda, int64_t sa, const double* b, int64_t ldb,
                                                    int64_t sbs, double beta, double* c, int64_t ldc, int64_t sc,
                                                    int64_t batch) {
  return run_config<double>(h, config, ta, tb, m, n, k, alpha, a, lda, sa, b, ldb, sbs, beta, c, ldc, sc, batch);
}

gbblas_status_t gbblas_sgemm_autotune(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                      int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, int reps,
                                      int* best_config, float* best_ms) {
  clear_error();
  return autotune<float>(h, ta, tb, m, n, k, lda, ldb, ldc, batch, reps, best_config, best_ms);
}

gbblas_status_t gbblas_dgemm_autotune(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                      int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, int reps,
                                      int* best_config, float* best_ms) {
  clear_error();
  return autotune<double>(h, ta, tb, m, n, k, lda, ldb, ldc, batch, reps, best_config, best_ms);
}

}  // extern "C"

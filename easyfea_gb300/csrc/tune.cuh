// Autotuner decision cache shared by the kernels' launch helpers.
//
// A decision (SpMV lanes per node; element-kernel blocks per SM) is keyed by
// the class of the problem -- kind, element or DOF count per node, value
// type, and log2 buckets of the sizes that change the best schedule -- and
// measured with CUDA events by gfea_tune_* (or on first use in mode 2).
#pragma once

#include <atomic>
#include <map>
#include <mutex>

#include "common.cuh"

namespace gfea {

enum TuneKind { kTuneSpmv = 1, kTuneAssemble = 2 };

struct TuneCache {
  std::mutex mu;
  std::map<int64_t, int32_t> best;
  std::atomic<int> mode{1};  // 0: heuristics only, 1: use decisions, 2: also tune on first use
};

inline TuneCache& tune_cache() {
  static TuneCache c;
  return c;
}

inline int tune_log2(double v) {
  int k = 0;
  while (v >= 2.0 && k < 63) {
    v *= 0.5;
    ++k;
  }
  return k;
}

// kind (8 bits) | a (8) | b (8) | c (8) | d (8)
inline int64_t tune_key(int kind, int a, int b, int c, int d) {
  return ((int64_t)(kind & 0xff) << 32) | ((int64_t)(a & 0xff) << 24) | ((int64_t)(b & 0xff) << 16) |
         ((int64_t)(c & 0xff) << 8) | (int64_t)(d & 0xff);
}

inline bool tune_get(int64_t key, int32_t* v) {
  TuneCache& T = tune_cache();
  if (T.mode.load() == 0) return false;
  std::lock_guard<std::mutex> lock(T.mu);
  auto it = T.best.find(key);
  if (it == T.best.end()) return false;
  *v = it->second;
  return true;
}

inline void tune_put(int64_t key, int32_t v) {
  TuneCache& T = tune_cache();
  std::lock_guard<std::mutex> lock(T.mu);
  T.best[key] = v;
}

// Times 'launch' (already warmed up by the caller's first call) with CUDA
// events: average milliseconds of 'reps' launches on stream st.
template <typename F>
int time_launches(F launch, int reps, cudaStream_t st, float* ms) {
  cudaEvent_t e0, e1;
  GFEA_CUDA_TRY(cudaEventCreate(&e0));
  GFEA_CUDA_TRY(cudaEventCreate(&e1));
  int err = launch();
  if (!err) {
    GFEA_CUDA_TRY(cudaEventRecord(e0, st));
    for (int r = 0; r < reps && !err; ++r) err = launch();
    GFEA_CUDA_TRY(cudaEventRecord(e1, st));
    GFEA_CUDA_TRY(cudaEventSynchronize(e1));
    float t = 0;
    GFEA_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return err;
}

}  // namespace gfea

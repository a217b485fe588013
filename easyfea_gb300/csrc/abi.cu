// Version and status strings of the C ABI.
#include "common.cuh"

extern "C" const char* gfea_version(void) { return "gfea 1 (sm_103a)"; }

extern "C" const char* gfea_status_string(int status) {
  switch (status) {
    case GFEA_OK: return "ok";
    case GFEA_ERR_ARG: return "invalid argument";
    case GFEA_ERR_CUDA: return "CUDA runtime error";
    case GFEA_ERR_CAPACITY: return "node neighbour capacity exceeded";
    case GFEA_ERR_SINGULAR: return "singular diagonal block";
    case GFEA_ERR_NOT_CONVERGED: return "PCG did not converge within max_iters";
    case GFEA_ERR_BREAKDOWN: return "PCG breakdown (p.Ap <= 0: operator not SPD on the unknowns)";
    case GFEA_ERR_NAN: return "non-finite value";
    case GFEA_ERR_WORKSPACE: return "workspace too small";
    case GFEA_ERR_TIMEOUT: return "bounded device wait timed out (or a staged tile out of order)";
    default: return "unknown status";
  }
}

// ---- autotuner decisions ----------------------------------------------------
#include "tune.cuh"

extern "C" int gfea_tune_mode(int mode) {
  if (mode < 0 || mode > 2) return GFEA_ERR_ARG;
  gfea::tune_cache().mode.store(mode);
  return GFEA_OK;
}

extern "C" int gfea_tune_clear(void) {
  gfea::TuneCache& T = gfea::tune_cache();
  std::lock_guard<std::mutex> lock(T.mu);
  T.best.clear();
  return GFEA_OK;
}

extern "C" int gfea_tune_export(int64_t* keys_host, int32_t* values_host, int max_entries, int* n_host) {
  if (!n_host || max_entries < 0 || (max_entries > 0 && (!keys_host || !values_host))) return GFEA_ERR_ARG;
  gfea::TuneCache& T = gfea::tune_cache();
  std::lock_guard<std::mutex> lock(T.mu);
  int n = 0;
  for (const auto& kv : T.best) {
    if (n < max_entries) {
      keys_host[n] = kv.first;
      values_host[n] = kv.second;
    }
    ++n;
  }
  *n_host = n;
  return GFEA_OK;
}

extern "C" int gfea_tune_import(const int64_t* keys_host, const int32_t* values_host, int n) {
  if (n < 0 || (n > 0 && (!keys_host || !values_host))) return GFEA_ERR_ARG;
  for (int i = 0; i < n; ++i) gfea::tune_put(keys_host[i], values_host[i]);
  return GFEA_OK;
}

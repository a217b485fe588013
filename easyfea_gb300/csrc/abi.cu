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
    default: return "unknown status";
  }
}

// Post-processing launches of the higher-order triangles TRI10 and TRI15,
// in a translation unit of their own.

#include "results.cuh"

namespace gfea {

int fields_dispatch_ho2d(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                         const double* u, const gfea_fields* f, cudaStream_t s) {
  FieldArgs A;
  PF P;
  if (fields_setup(f, &A, &P)) return GFEA_ERR_ARG;
  if (elem == GFEA_TRI10) return dispatch_fields<GFEA_TRI10>(mass, coord, connect, Ne, u, A, P, s);
  if (elem == GFEA_TRI15) return dispatch_fields<GFEA_TRI15>(mass, coord, connect, Ne, u, A, P, s);
  return GFEA_ERR_ARG;
}

}  // namespace gfea

// HEXA20 / HEXA27 post-processing launches (their 27-point kernels compile
// in a translation unit of their own).

#include "results.cuh"

namespace gfea {

int fields_dispatch_hexq(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                         const double* u, const gfea_fields* f, cudaStream_t s) {
  FieldArgs A;
  PF P;
  if (fields_setup(f, &A, &P)) return GFEA_ERR_ARG;
  if (elem == GFEA_HEXA20) return dispatch_fields<GFEA_HEXA20>(mass, coord, connect, Ne, u, A, P, s);
  if (elem == GFEA_HEXA27) return dispatch_fields<GFEA_HEXA27>(mass, coord, connect, Ne, u, A, P, s);
  return GFEA_ERR_ARG;
}

}  // namespace gfea

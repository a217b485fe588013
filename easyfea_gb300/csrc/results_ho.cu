// Post-processing launches of the prisms PRISM6, PRISM15 and PRISM18 (the
// higher-order triangles TRI10 and TRI15 in results_ho2d.cu), in a
// translation unit of their own.

#include "results.cuh"

namespace gfea {

int fields_dispatch_ho(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                       const double* u, const gfea_fields* f, cudaStream_t s) {
  FieldArgs A;
  PF P;
  if (fields_setup(f, &A, &P)) return GFEA_ERR_ARG;
  switch (elem) {
    case GFEA_TRI10: case GFEA_TRI15: return fields_dispatch_ho2d(elem, mass, coord, connect, Ne, u, f, s);
    case GFEA_PRISM6: return dispatch_fields<GFEA_PRISM6>(mass, coord, connect, Ne, u, A, P, s);
    case GFEA_PRISM15: return dispatch_fields<GFEA_PRISM15>(mass, coord, connect, Ne, u, A, P, s);
    case GFEA_PRISM18: return dispatch_fields<GFEA_PRISM18>(mass, coord, connect, Ne, u, A, P, s);
    default: return GFEA_ERR_ARG;
  }
}

}  // namespace gfea

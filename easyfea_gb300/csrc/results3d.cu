// The 3D elements' post-processing launches (a translation unit of their
// own so that the library's translation units compile in parallel).

#include "results.cuh"

namespace gfea {

int fields_dispatch_3d(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                       const double* u, const gfea_fields* f, cudaStream_t s) {
  FieldArgs A;
  PF P;
  if (fields_setup(f, &A, &P)) return GFEA_ERR_ARG;
  switch (elem) {
    case GFEA_HEXA8: return dispatch_fields<GFEA_HEXA8>(mass, coord, connect, Ne, u, A, P, s);
    case GFEA_TETRA4: return dispatch_fields<GFEA_TETRA4>(mass, coord, connect, Ne, u, A, P, s);
    case GFEA_TETRA10: return dispatch_fields<GFEA_TETRA10>(mass, coord, connect, Ne, u, A, P, s);
    case GFEA_HEXA20: case GFEA_HEXA27: return fields_dispatch_hexq(elem, mass, coord, connect, Ne, u, f, s);
    default: return GFEA_ERR_ARG;
  }
}

}  // namespace gfea

// The 3D elements' phase-field launches (a translation unit of their own so
// that the library's translation units compile in parallel).

#include "phasefield.cuh"

namespace gfea {

int pf_damage_3d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                 const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                 double* H_new, double* Kd, double* Fd, cudaStream_t s) {
  PF P;
  if (to_pf(params, &P) || P.dim != 3) return GFEA_ERR_ARG;
  switch (elem) {
    case GFEA_HEXA8: return launch_damage<GFEA_HEXA8>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
    case GFEA_TETRA4: return launch_damage<GFEA_TETRA4>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
    case GFEA_TETRA10: return launch_damage<GFEA_TETRA10>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
    case GFEA_HEXA20: case GFEA_HEXA27:
      return pf_damage_hexq(elem, coord, connect, Ne, node_ptr, rank, u, params, H_old, H_new, Kd, Fd, s);
    default: return GFEA_ERR_ARG;
  }
}

template <typename T>
int pf_elastic_3d_t(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                    const uint8_t* rank, const double* u, const double* d, const PF& P, T* v, cudaStream_t s) {
  switch (elem) {
    case GFEA_HEXA8: return launch_pfel<GFEA_HEXA8, T>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    case GFEA_TETRA4: return launch_pfel<GFEA_TETRA4, T>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    case GFEA_TETRA10: return launch_pfel<GFEA_TETRA10, T>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    case GFEA_HEXA20: case GFEA_HEXA27: return GFEA_ERR_ARG;  // pf_elastic_hexq
    default: return GFEA_ERR_ARG;
  }
}

int pf_elastic_3d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                  const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                  int value_type, void* values, cudaStream_t s) {
  PF P;
  if (to_pf(params, &P)) return GFEA_ERR_ARG;
  if (elem == GFEA_HEXA20 || elem == GFEA_HEXA27)
    return pf_elastic_hexq(elem, coord, connect, Ne, node_ptr, rank, u, d, params, value_type, values, s);
  if (value_type == GFEA_F64)
    return pf_elastic_3d_t<double>(elem, coord, connect, Ne, node_ptr, rank, u, d, P, static_cast<double*>(values), s);
  if (value_type == GFEA_F32)
    return pf_elastic_3d_t<float>(elem, coord, connect, Ne, node_ptr, rank, u, d, P, static_cast<float*>(values), s);
  return GFEA_ERR_ARG;
}

}  // namespace gfea

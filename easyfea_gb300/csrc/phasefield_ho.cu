// Phase-field launches of the prisms PRISM6, PRISM15 and PRISM18 (the
// higher-order triangles TRI10 and TRI15 in phasefield_ho2d.cu), in a
// translation unit of their own.

#include "phasefield.cuh"

namespace gfea {

int pf_damage_ho(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                 const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                 double* H_new, double* Kd, double* Fd, cudaStream_t s) {
  if (elem == GFEA_TRI10 || elem == GFEA_TRI15)
    return pf_damage_ho2d(elem, coord, connect, Ne, node_ptr, rank, u, params, H_old, H_new, Kd, Fd, s);
  PF P;
  if (to_pf(params, &P) || P.dim != 3) return GFEA_ERR_ARG;
  switch (elem) {
    case GFEA_PRISM6: return launch_damage<GFEA_PRISM6>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
    case GFEA_PRISM15: return launch_damage<GFEA_PRISM15>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
    case GFEA_PRISM18: return launch_damage<GFEA_PRISM18>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
    default: return GFEA_ERR_ARG;
  }
}

template <typename T>
int pf_elastic_ho_t(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                    const uint8_t* rank, const double* u, const double* d, const PF& P, T* v, cudaStream_t s) {
  switch (elem) {
    case GFEA_PRISM6: return launch_pfel<GFEA_PRISM6, T>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    case GFEA_PRISM15: return launch_pfel<GFEA_PRISM15, T>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    case GFEA_PRISM18: return launch_pfel<GFEA_PRISM18, T>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    default: return GFEA_ERR_ARG;
  }
}

int pf_elastic_ho(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                  const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                  int value_type, void* values, cudaStream_t s) {
  if (elem == GFEA_TRI10 || elem == GFEA_TRI15)
    return pf_elastic_ho2d(elem, coord, connect, Ne, node_ptr, rank, u, d, params, value_type, values, s);
  PF P;
  if (to_pf(params, &P)) return GFEA_ERR_ARG;
  if (value_type == GFEA_F64)
    return pf_elastic_ho_t<double>(elem, coord, connect, Ne, node_ptr, rank, u, d, P, static_cast<double*>(values), s);
  if (value_type == GFEA_F32)
    return pf_elastic_ho_t<float>(elem, coord, connect, Ne, node_ptr, rank, u, d, P, static_cast<float*>(values), s);
  return GFEA_ERR_ARG;
}

}  // namespace gfea

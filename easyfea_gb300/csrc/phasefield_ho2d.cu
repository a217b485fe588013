// Phase-field launches of the higher-order triangles TRI10 and TRI15, in a
// translation unit of their own.

#include "phasefield.cuh"

namespace gfea {

int pf_damage_ho2d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                   const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                   double* H_new, double* Kd, double* Fd, cudaStream_t s) {
  PF P;
  if (to_pf(params, &P) || P.dim != 2) return GFEA_ERR_ARG;
  if (elem == GFEA_TRI10) return launch_damage<GFEA_TRI10>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
  if (elem == GFEA_TRI15) return launch_damage<GFEA_TRI15>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd, s);
  return GFEA_ERR_ARG;
}

int pf_elastic_ho2d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                    const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                    int value_type, void* values, cudaStream_t s) {
  PF P;
  if (to_pf(params, &P)) return GFEA_ERR_ARG;
  if (value_type == GFEA_F64) {
    auto* v = static_cast<double*>(values);
    if (elem == GFEA_TRI10) return launch_pfel<GFEA_TRI10, double>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    if (elem == GFEA_TRI15) return launch_pfel<GFEA_TRI15, double>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
  } else if (value_type == GFEA_F32) {
    auto* v = static_cast<float*>(values);
    if (elem == GFEA_TRI10) return launch_pfel<GFEA_TRI10, float>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
    if (elem == GFEA_TRI15) return launch_pfel<GFEA_TRI15, float>(coord, connect, Ne, node_ptr, rank, u, d, P, v, s);
  }
  return GFEA_ERR_ARG;
}

}  // namespace gfea

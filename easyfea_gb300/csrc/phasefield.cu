// Phase-field entry points and the 2D elements' launches (kernels in
// phasefield.cuh, the 3D elements' launches in phasefield3d.cu, the
// higher-order elements' in phasefield_ho.cu).

#include "phasefield.cuh"

using namespace gfea;


extern "C" int gfea_pf_damage(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                              const int32_t* node_ptr, const uint8_t* rank, const double* u,
                              const gfea_pf_params* params_host, const double* H_old, double* H_new,
                              double* Kd_values, double* Fd, void* stream) {
  PF P;
  if (to_pf(params_host, &P)) return GFEA_ERR_ARG;
  if (!coord || !connect || !node_ptr || !rank || !u || !H_new || !Kd_values || !Fd || n_elems < 0) return GFEA_ERR_ARG;
  if (n_elems == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (higher_order_elem(elem))
    return pf_damage_ho(elem, coord, connect, n_elems, node_ptr, rank, u, params_host, H_old, H_new, Kd_values, Fd, s);
  switch (elem) {
    case GFEA_TRI3: if (P.dim != 2) return GFEA_ERR_ARG; return launch_damage<GFEA_TRI3>(coord, connect, n_elems, node_ptr, rank, u, P, H_old, H_new, Kd_values, Fd, s);
    case GFEA_QUAD4: if (P.dim != 2) return GFEA_ERR_ARG; return launch_damage<GFEA_QUAD4>(coord, connect, n_elems, node_ptr, rank, u, P, H_old, H_new, Kd_values, Fd, s);
    case GFEA_QUAD9: if (P.dim != 2) return GFEA_ERR_ARG; return launch_damage<GFEA_QUAD9>(coord, connect, n_elems, node_ptr, rank, u, P, H_old, H_new, Kd_values, Fd, s);
    case GFEA_TRI6: if (P.dim != 2) return GFEA_ERR_ARG; return launch_damage<GFEA_TRI6>(coord, connect, n_elems, node_ptr, rank, u, P, H_old, H_new, Kd_values, Fd, s);
    case GFEA_QUAD8: if (P.dim != 2) return GFEA_ERR_ARG; return launch_damage<GFEA_QUAD8>(coord, connect, n_elems, node_ptr, rank, u, P, H_old, H_new, Kd_values, Fd, s);
    default:
      if (P.dim != 3) return GFEA_ERR_ARG;
      return pf_damage_3d(elem, coord, connect, n_elems, node_ptr, rank, u, params_host, H_old, H_new, Kd_values, Fd,
                          s);
  }
}

extern "C" int gfea_pf_elastic(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                               const int32_t* node_ptr, const uint8_t* rank, const double* u, const double* d,
                               const gfea_pf_params* params_host, int value_type, void* values, void* stream) {
  PF P;
  if (to_pf(params_host, &P)) return GFEA_ERR_ARG;
  if (!coord || !connect || !node_ptr || !rank || !u || !d || !values || n_elems < 0) return GFEA_ERR_ARG;
  if (n_elems == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (higher_order_elem(elem))
    return pf_elastic_ho(elem, coord, connect, n_elems, node_ptr, rank, u, d, params_host, value_type, values, s);
  if (value_type == GFEA_F64) {
    auto* v = static_cast<double*>(values);
    switch (elem) {
      case GFEA_TRI3: return launch_pfel<GFEA_TRI3, double>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_QUAD4: return launch_pfel<GFEA_QUAD4, double>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_QUAD9: return launch_pfel<GFEA_QUAD9, double>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_TRI6: return launch_pfel<GFEA_TRI6, double>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_QUAD8: return launch_pfel<GFEA_QUAD8, double>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      default: return pf_elastic_3d(elem, coord, connect, n_elems, node_ptr, rank, u, d, params_host, value_type,
                                    values, s);
    }
  } else if (value_type == GFEA_F32) {
    auto* v = static_cast<float*>(values);
    switch (elem) {
      case GFEA_TRI3: return launch_pfel<GFEA_TRI3, float>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_QUAD4: return launch_pfel<GFEA_QUAD4, float>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_QUAD9: return launch_pfel<GFEA_QUAD9, float>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_TRI6: return launch_pfel<GFEA_TRI6, float>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      case GFEA_QUAD8: return launch_pfel<GFEA_QUAD8, float>(coord, connect, n_elems, node_ptr, rank, u, d, P, v, s);
      default: return pf_elastic_3d(elem, coord, connect, n_elems, node_ptr, rank, u, d, params_host, value_type,
                                    values, s);
    }
  }
  return GFEA_ERR_ARG;
}

extern "C" int gfea_pf_split(const double* eps, int64_t n_points, const gfea_pf_params* params_host, double* cP,
                             double* cM, double* psiP, double* psiM, void* stream) {
  PF P;
  if (to_pf(params_host, &P)) return GFEA_ERR_ARG;
  if (!eps || n_points < 0) return GFEA_ERR_ARG;
  if (n_points == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = grid_for(n_points, 128);
  if (P.dim == 2)
    pf_anisot(P.split) ? split_kernel<2, true><<<blocks, 128, 0, s>>>(eps, n_points, P, cP, cM, psiP, psiM)
                       : split_kernel<2, false><<<blocks, 128, 0, s>>>(eps, n_points, P, cP, cM, psiP, psiM);
  else
    pf_anisot(P.split) ? split_kernel<3, true><<<blocks, 128, 0, s>>>(eps, n_points, P, cP, cM, psiP, psiM)
                       : split_kernel<3, false><<<blocks, 128, 0, s>>>(eps, n_points, P, cP, cM, psiP, psiM);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

// Entry points of the stiffness, mass and surface-load assembly (the
// kernels are in assemble.cuh; the higher-order elements' launches compile
// in assemble_ho.cu).

#include "assemble.cuh"

namespace gfea {
namespace {

template <typename T>
int dispatch_elastic(int elem, bool tune, const double* coord, const int32_t* connect, int64_t Ne,
                     const int32_t* node_ptr, const uint8_t* rank, const double* C, int cpe, double factor, T* v,
                     int64_t n_values, cudaStream_t s, int32_t* best, float* ms) {
#define GFEA_ELASTIC_CASE(EL)                                                                                   \
  case EL:                                                                                                      \
    return tune ? tune_elastic<EL, T, T>(coord, connect, Ne, node_ptr, rank, C, cpe, factor, v, n_values, s, best, \
                                         ms)                                                                    \
                : launch_elastic<EL, T, T>(coord, connect, Ne, node_ptr, rank, C, cpe, factor, v, s);
  switch (elem) {
    GFEA_ELASTIC_CASE(GFEA_TRI3)
    GFEA_ELASTIC_CASE(GFEA_QUAD4)
    GFEA_ELASTIC_CASE(GFEA_QUAD9)
    GFEA_ELASTIC_CASE(GFEA_HEXA8)
    GFEA_ELASTIC_CASE(GFEA_TETRA4)
    GFEA_ELASTIC_CASE(GFEA_TRI6)
    GFEA_ELASTIC_CASE(GFEA_QUAD8)
    GFEA_ELASTIC_CASE(GFEA_TETRA10)
    GFEA_ELASTIC_CASE(GFEA_HEXA20)
    GFEA_ELASTIC_CASE(GFEA_HEXA27)
    default:
      return elastic_ho(elem, tune, coord, connect, Ne, node_ptr, rank, C, cpe, factor,
                        sizeof(T) == 8 ? GFEA_F64 : GFEA_F32, v, n_values, s, best, ms);
  }
#undef GFEA_ELASTIC_CASE
}

int elem_dim(int elem) {
  switch (elem) {
    case GFEA_SEG2: case GFEA_SEG3: case GFEA_SEG4: case GFEA_SEG5: return 1;
    case GFEA_HEXA8: case GFEA_TETRA4: case GFEA_TETRA10: case GFEA_HEXA20: case GFEA_HEXA27: case GFEA_PRISM6:
    case GFEA_PRISM15: case GFEA_PRISM18: return 3;
    case GFEA_TRI3: case GFEA_QUAD4: case GFEA_QUAD9: case GFEA_TRI6: case GFEA_QUAD8: case GFEA_TRI10:
    case GFEA_TRI15: return 2;
    default: return -1;
  }
}

}  // namespace
}  // namespace gfea

using namespace gfea;

extern "C" int gfea_assemble_elastic(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                                     const int32_t* node_ptr, const uint8_t* rank, const double* C,
                                     int c_per_elem, double factor, int value_type, void* values,
                                     int64_t n_values, int accumulate, void* stream) {
  if (!coord || !connect || !node_ptr || !rank || !C || !values || n_elems < 0) return GFEA_ERR_ARG;
  if (c_per_elem < 0 || c_per_elem > 4) return GFEA_ERR_ARG;
  const int d = elem_dim(elem);
  if (d < 2) return GFEA_ERR_ARG;
  if (value_type != GFEA_F64 && value_type != GFEA_F32) return GFEA_ERR_ARG;
  if (n_elems == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // first assembly of this class in tuning mode: choose the tile schedule
  int32_t tuned = 0;
  float ms = 0;
  const bool tune = !accumulate && n_values > 0 && tune_cache().mode.load() == 2 &&
                    !tune_get(assemble_key(elem, value_type, c_per_elem, n_elems), &tuned);
  if (!accumulate && n_values > 0 && !tune)
    GFEA_CUDA_TRY(cudaMemsetAsync(values, 0, (value_type == GFEA_F64 ? 8 : 4) * (size_t)n_values, s));
  if (value_type == GFEA_F64)
    return dispatch_elastic<double>(elem, tune, coord, connect, n_elems, node_ptr, rank, C, c_per_elem, factor,
                                    static_cast<double*>(values), n_values, s, &tuned, &ms);
  return dispatch_elastic<float>(elem, tune, coord, connect, n_elems, node_ptr, rank, C, c_per_elem, factor,
                                 static_cast<float*>(values), n_values, s, &tuned, &ms);
}

extern "C" int gfea_tune_assemble_elastic(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                                          const int32_t* node_ptr, const uint8_t* rank, const double* C,
                                          int c_per_elem, double factor, int value_type, void* values,
                                          int64_t n_values, int32_t* blocks_per_sm_host, float* ms_host,
                                          void* stream) {
  if (!coord || !connect || !node_ptr || !rank || !C || !values || n_elems <= 0 || n_values <= 0 ||
      !blocks_per_sm_host || !ms_host)
    return GFEA_ERR_ARG;
  if (elem_dim(elem) < 2 || (value_type != GFEA_F64 && value_type != GFEA_F32)) return GFEA_ERR_ARG;
  if (c_per_elem < 0 || c_per_elem > 4) return GFEA_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (value_type == GFEA_F64)
    return dispatch_elastic<double>(elem, true, coord, connect, n_elems, node_ptr, rank, C, c_per_elem, factor,
                                    static_cast<double*>(values), n_values, s, blocks_per_sm_host, ms_host);
  return dispatch_elastic<float>(elem, true, coord, connect, n_elems, node_ptr, rank, C, c_per_elem, factor,
                                 static_cast<float*>(values), n_values, s, blocks_per_sm_host, ms_host);
}

extern "C" int gfea_assemble_mass(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                                  const int32_t* node_ptr, const uint8_t* rank, int dof_n, double rho,
                                  double factor, int value_type, void* values, int64_t n_values,
                                  int accumulate, void* stream) {
  if (!coord || !connect || !node_ptr || !rank || !values || n_elems < 0 || dof_n < 1 || dof_n > 3) return GFEA_ERR_ARG;
  if (n_elems == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!accumulate && n_values > 0)
    GFEA_CUDA_TRY(cudaMemsetAsync(values, 0, (value_type == GFEA_F64 ? 8 : 4) * (size_t)n_values, s));
  if (value_type == GFEA_F64) {
    auto* v = static_cast<double*>(values);
    switch (elem) {
      case GFEA_TRI3: return launch_mass<GFEA_TRI3, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_QUAD4: return launch_mass<GFEA_QUAD4, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_QUAD9: return launch_mass<GFEA_QUAD9, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_HEXA8: return launch_mass<GFEA_HEXA8, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_TETRA4: return launch_mass<GFEA_TETRA4, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_TRI6: return launch_mass<GFEA_TRI6, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_QUAD8: return launch_mass<GFEA_QUAD8, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_TETRA10: return launch_mass<GFEA_TETRA10, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_HEXA20: return launch_mass<GFEA_HEXA20, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_HEXA27: return launch_mass<GFEA_HEXA27, double, double>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      default: return mass_ho(elem, coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, value_type, values, s);
    }
  } else if (value_type == GFEA_F32) {
    auto* v = static_cast<float*>(values);
    switch (elem) {
      case GFEA_TRI3: return launch_mass<GFEA_TRI3, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_QUAD4: return launch_mass<GFEA_QUAD4, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_QUAD9: return launch_mass<GFEA_QUAD9, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_HEXA8: return launch_mass<GFEA_HEXA8, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_TETRA4: return launch_mass<GFEA_TETRA4, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_TRI6: return launch_mass<GFEA_TRI6, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_QUAD8: return launch_mass<GFEA_QUAD8, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_TETRA10: return launch_mass<GFEA_TETRA10, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_HEXA20: return launch_mass<GFEA_HEXA20, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      case GFEA_HEXA27: return launch_mass<GFEA_HEXA27, float, float>(coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, v, s);
      default: return mass_ho(elem, coord, connect, n_elems, node_ptr, rank, dof_n, rho, factor, value_type, values, s);
    }
  }
  return GFEA_ERR_ARG;
}

extern "C" int gfea_surface_load(int belem, const double* coord, const int32_t* bconnect, int64_t n_belems,
                                 const uint8_t* node_mask, int dof_n, int n_unknowns,
                                 const int32_t* unknown_idx_host, const double* values_host, double factor,
                                 double* b, void* stream) {
  if (!coord || !bconnect || !node_mask || !b || n_belems < 0 || n_unknowns < 1 || n_unknowns > 4 ||
      !unknown_idx_host || !values_host)
    return GFEA_ERR_ARG;
  if (n_belems == 0) return GFEA_OK;
  int ui[4] = {0, 0, 0, 0};
  double uv[4] = {0, 0, 0, 0};
  for (int u = 0; u < n_unknowns; ++u) {
    if (unknown_idx_host[u] < 0 || unknown_idx_host[u] >= dof_n) return GFEA_ERR_ARG;
    ui[u] = unknown_idx_host[u];
    uv[u] = values_host[u];
  }
  const int4 uidx = make_int4(ui[0], ui[1], ui[2], ui[3]);
  const Traction4 uval{uv[0], uv[1], uv[2], uv[3]};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = grid_for(n_belems, 128);
  switch (belem) {
    case GFEA_SEG2:
      surface_load_kernel<GFEA_SEG2><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_QUAD4:
      surface_load_kernel<GFEA_QUAD4><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_TRI3:
      surface_load_kernel<GFEA_TRI3><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_SEG3:
      surface_load_kernel<GFEA_SEG3><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_TRI6:
      surface_load_kernel<GFEA_TRI6><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_QUAD8:
      surface_load_kernel<GFEA_QUAD8><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_QUAD9:
      surface_load_kernel<GFEA_QUAD9><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_SEG4:
      surface_load_kernel<GFEA_SEG4><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    case GFEA_SEG5:
      surface_load_kernel<GFEA_SEG5><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n, n_unknowns, uidx, uval, factor, b);
      break;
    default:
      return GFEA_ERR_ARG;
  }
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" int gfea_boundary_gauss_points(int belem, const double* coord, const int32_t* bconnect, int64_t n_belems,
                                          double* xyz, int32_t* npg_host, void* stream) {
  if (!coord || !bconnect || !npg_host || n_belems < 0 || (n_belems > 0 && !xyz)) return GFEA_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = grid_for(n_belems > 0 ? n_belems : 1, 128);
  switch (belem) {
    case GFEA_SEG2:
      *npg_host = RefTables<GFEA_SEG2, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_SEG2><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_QUAD4:
      *npg_host = RefTables<GFEA_QUAD4, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_QUAD4><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_TRI3:
      *npg_host = RefTables<GFEA_TRI3, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_TRI3><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_SEG3:
      *npg_host = RefTables<GFEA_SEG3, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_SEG3><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_TRI6:
      *npg_host = RefTables<GFEA_TRI6, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_TRI6><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_QUAD8:
      *npg_host = RefTables<GFEA_QUAD8, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_QUAD8><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_QUAD9:
      *npg_host = RefTables<GFEA_QUAD9, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_QUAD9><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_SEG4:
      *npg_host = RefTables<GFEA_SEG4, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_SEG4><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    case GFEA_SEG5:
      *npg_host = RefTables<GFEA_SEG5, true>::nPg;
      if (n_belems) boundary_gauss_kernel<GFEA_SEG5><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, xyz);
      break;
    default:
      return GFEA_ERR_ARG;
  }
  if (n_belems) GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" int gfea_surface_load_field(int belem, const double* coord, const int32_t* bconnect, int64_t n_belems,
                                       const uint8_t* node_mask, int dof_n, int unknown_idx, int mode,
                                       const double* values, double factor, double* b, void* stream) {
  if (!coord || !bconnect || !node_mask || !b || !values || n_belems < 0 || unknown_idx < 0 ||
      unknown_idx >= dof_n || (mode != 0 && mode != 1))
    return GFEA_ERR_ARG;
  if (n_belems == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = grid_for(n_belems, 128);
  switch (belem) {
    case GFEA_SEG2:
      surface_load_field_kernel<GFEA_SEG2><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                                   unknown_idx, mode, values, factor, b);
      break;
    case GFEA_QUAD4:
      surface_load_field_kernel<GFEA_QUAD4><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                                    unknown_idx, mode, values, factor, b);
      break;
    case GFEA_TRI3:
      surface_load_field_kernel<GFEA_TRI3><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                                   unknown_idx, mode, values, factor, b);
      break;
    case GFEA_SEG3:
      surface_load_field_kernel<GFEA_SEG3><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                           unknown_idx, mode, values, factor, b);
      break;
    case GFEA_TRI6:
      surface_load_field_kernel<GFEA_TRI6><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                           unknown_idx, mode, values, factor, b);
      break;
    case GFEA_QUAD8:
      surface_load_field_kernel<GFEA_QUAD8><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                           unknown_idx, mode, values, factor, b);
      break;
    case GFEA_QUAD9:
      surface_load_field_kernel<GFEA_QUAD9><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                           unknown_idx, mode, values, factor, b);
      break;
    case GFEA_SEG4:
      surface_load_field_kernel<GFEA_SEG4><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                           unknown_idx, mode, values, factor, b);
      break;
    case GFEA_SEG5:
      surface_load_field_kernel<GFEA_SEG5><<<blocks, 128, 0, s>>>(coord, bconnect, n_belems, node_mask, dof_n,
                                                           unknown_idx, mode, values, factor, b);
      break;
    default:
      return GFEA_ERR_ARG;
  }
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

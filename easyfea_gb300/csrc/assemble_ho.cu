// Stiffness and mass launches of the higher-order elements TRI10, TRI15,
// PRISM6, PRISM15 and PRISM18 (a translation unit of their own so that the
// library's translation units compile in parallel).

#include "assemble.cuh"

namespace gfea {
namespace {

template <typename T>
int elastic_ho_t(int elem, bool tune, const double* coord, const int32_t* connect, int64_t Ne,
                 const int32_t* node_ptr, const uint8_t* rank, const double* C, int cpe, double factor, T* v,
                 int64_t n_values, cudaStream_t s, int32_t* best, float* ms) {
#define GFEA_ELASTIC_CASE(EL)                                                                                   \
  case EL:                                                                                                      \
    return tune ? tune_elastic<EL, T, T>(coord, connect, Ne, node_ptr, rank, C, cpe, factor, v, n_values, s, best, \
                                         ms)                                                                    \
                : launch_elastic<EL, T, T>(coord, connect, Ne, node_ptr, rank, C, cpe, factor, v, s);
  switch (elem) {
    GFEA_ELASTIC_CASE(GFEA_TRI10)
    GFEA_ELASTIC_CASE(GFEA_TRI15)
    GFEA_ELASTIC_CASE(GFEA_PRISM6)
    GFEA_ELASTIC_CASE(GFEA_PRISM15)
    GFEA_ELASTIC_CASE(GFEA_PRISM18)
    default: return GFEA_ERR_ARG;
  }
#undef GFEA_ELASTIC_CASE
}

template <typename T>
int mass_ho_t(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
              const uint8_t* rank, int dof_n, double rho, double factor, T* v, cudaStream_t s) {
  switch (elem) {
    case GFEA_TRI10: return launch_mass<GFEA_TRI10, T, T>(coord, connect, Ne, node_ptr, rank, dof_n, rho, factor, v, s);
    case GFEA_TRI15: return launch_mass<GFEA_TRI15, T, T>(coord, connect, Ne, node_ptr, rank, dof_n, rho, factor, v, s);
    case GFEA_PRISM6: return launch_mass<GFEA_PRISM6, T, T>(coord, connect, Ne, node_ptr, rank, dof_n, rho, factor, v, s);
    case GFEA_PRISM15: return launch_mass<GFEA_PRISM15, T, T>(coord, connect, Ne, node_ptr, rank, dof_n, rho, factor, v, s);
    case GFEA_PRISM18: return launch_mass<GFEA_PRISM18, T, T>(coord, connect, Ne, node_ptr, rank, dof_n, rho, factor, v, s);
    default: return GFEA_ERR_ARG;
  }
}

}  // namespace

int elastic_ho(int elem, bool tune, const double* coord, const int32_t* connect, int64_t Ne,
               const int32_t* node_ptr, const uint8_t* rank, const double* C, int cpe, double factor,
               int value_type, void* values, int64_t n_values, cudaStream_t s, int32_t* best, float* ms) {
  if (value_type == GFEA_F64)
    return elastic_ho_t<double>(elem, tune, coord, connect, Ne, node_ptr, rank, C, cpe, factor,
                                static_cast<double*>(values), n_values, s, best, ms);
  if (value_type == GFEA_F32)
    return elastic_ho_t<float>(elem, tune, coord, connect, Ne, node_ptr, rank, C, cpe, factor,
                               static_cast<float*>(values), n_values, s, best, ms);
  return GFEA_ERR_ARG;
}

int mass_ho(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
            const uint8_t* rank, int dof_n, double rho, double factor, int value_type, void* values,
            cudaStream_t s) {
  if (value_type == GFEA_F64)
    return mass_ho_t<double>(elem, coord, connect, Ne, node_ptr, rank, dof_n, rho, factor,
                             static_cast<double*>(values), s);
  if (value_type == GFEA_F32)
    return mass_ho_t<float>(elem, coord, connect, Ne, node_ptr, rank, dof_n, rho, factor,
                            static_cast<float*>(values), s);
  return GFEA_ERR_ARG;
}

}  // namespace gfea

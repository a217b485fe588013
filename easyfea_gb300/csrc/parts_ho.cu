// Row-owned stiffness launches of the higher-order elements TRI10, TRI15,
// PRISM6, PRISM15 and PRISM18 (a translation unit of their own so that the
// library's translation units compile in parallel).

#include "parts.cuh"

namespace gfea {
namespace {

template <typename T>
int parts_ho_t(int elem, const double* coord, const int32_t* connect, const int32_t* node_ptr, const uint8_t* rank,
               const double* C, int cpe, double factor, const PartArgs& A, int n_parts, int threads, T* vals,
               cudaStream_t s) {
  switch (elem) {
    case GFEA_TRI10: return launch_parts<GFEA_TRI10, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_TRI15: return launch_parts<GFEA_TRI15, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_PRISM6: return launch_parts<GFEA_PRISM6, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_PRISM15: return launch_parts<GFEA_PRISM15, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_PRISM18: return launch_parts<GFEA_PRISM18, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    default: return GFEA_ERR_ARG;
  }
}

}  // namespace

int parts_ho(int elem, const double* coord, const int32_t* connect, const int32_t* node_ptr, const uint8_t* rank,
             const double* C, int cpe, double factor, const PartArgs& A, int n_parts, int threads, int value_type,
             void* vals, cudaStream_t s) {
  if (value_type == GFEA_F64)
    return parts_ho_t<double>(elem, coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads,
                              static_cast<double*>(vals), s);
  if (value_type == GFEA_F32)
    return parts_ho_t<float>(elem, coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads,
                             static_cast<float*>(vals), s);
  return GFEA_ERR_ARG;
}

size_t part_smem_ho(int elem, int value_type, int max_vals, int threads) {
  const bool f32 = value_type == GFEA_F32;
  switch (elem) {
#define GFEA_PART_SMEM(EL) \
  case EL: return f32 ? part_smem<EL, float>(max_vals, threads) : part_smem<EL, double>(max_vals, threads);
    GFEA_PART_SMEM(GFEA_TRI10)
    GFEA_PART_SMEM(GFEA_TRI15)
    GFEA_PART_SMEM(GFEA_PRISM6)
    GFEA_PART_SMEM(GFEA_PRISM15)
    GFEA_PART_SMEM(GFEA_PRISM18)
#undef GFEA_PART_SMEM
    default: return 0;
  }
}

}  // namespace gfea

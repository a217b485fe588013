// Post-processing entry points and the 2D elements' launches; the kernels
// are in results.cuh, the 3D elements' launches in results3d.cu and the
// higher-order elements' in results_ho.cu.

#include "results.cuh"

using namespace gfea;

extern "C" int gfea_element_fields(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                                   const double* u, const gfea_fields* f, void* stream) {
  if (!f || f->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (!coord || !connect || !u || n_elems < 0 || (f->gauss != 0 && f->gauss != 1)) return GFEA_ERR_ARG;
  if (!(f->coef > 0)) return GFEA_ERR_ARG;
  FieldArgs A;
  PF P;
  const int st = fields_setup(f, &A, &P);
  int dim = 0;
  switch (elem) {
    case GFEA_TRI3: case GFEA_QUAD4: case GFEA_QUAD9: case GFEA_TRI6: case GFEA_QUAD8: case GFEA_TRI10:
    case GFEA_TRI15: dim = 2; break;
    case GFEA_HEXA8: case GFEA_TETRA4: case GFEA_TETRA10: case GFEA_HEXA20: case GFEA_HEXA27: case GFEA_PRISM6:
    case GFEA_PRISM15: case GFEA_PRISM18: dim = 3; break;
    default: return GFEA_ERR_ARG;
  }
  if (A.pf) {
    if (st || P.dim != dim || !f->d) return GFEA_ERR_ARG;
  } else {
    if (!f->C || f->c_per_elem < 0 || f->c_per_elem > 4 || f->psiP_e || f->H_old) return GFEA_ERR_ARG;
  }
  if (n_elems == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool mass = f->gauss == 1;
  if (higher_order_elem(elem)) return fields_dispatch_ho(elem, mass, coord, connect, n_elems, u, f, s);
  switch (elem) {
    case GFEA_TRI3: return dispatch_fields<GFEA_TRI3>(mass, coord, connect, n_elems, u, A, P, s);
    case GFEA_QUAD4: return dispatch_fields<GFEA_QUAD4>(mass, coord, connect, n_elems, u, A, P, s);
    case GFEA_QUAD9: return dispatch_fields<GFEA_QUAD9>(mass, coord, connect, n_elems, u, A, P, s);
    case GFEA_TRI6: return dispatch_fields<GFEA_TRI6>(mass, coord, connect, n_elems, u, A, P, s);
    case GFEA_QUAD8: return dispatch_fields<GFEA_QUAD8>(mass, coord, connect, n_elems, u, A, P, s);
    default: return fields_dispatch_3d(elem, mass, coord, connect, n_elems, u, f, s);
  }
}
extern "C" int gfea_node_average(const int32_t* inc_ptr, const int32_t* inc_list, int64_t n_nodes,
                                 const double* values_e, int n_cols, double* values_n, void* stream) {
  if (!inc_ptr || !inc_list || !values_e || !values_n || n_nodes < 0 || n_cols < 1) return GFEA_ERR_ARG;
  if (n_nodes == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int blocks = grid_for(n_nodes * n_cols, 256);
  if (blocks > kSMs * 16) blocks = kSMs * 16;
  node_average_kernel<<<blocks, 256, 0, s>>>(inc_ptr, inc_list, n_nodes, values_e, n_cols, values_n);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

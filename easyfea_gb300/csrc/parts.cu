// Row-owned stiffness assembly: entry points and host-side part plan (the
// kernels are in parts.cuh, the higher-order elements' launches in
// parts_ho.cu).

#include <algorithm>
#include <vector>

#include "parts.cuh"

namespace gfea {
namespace {

template <typename T>
int dispatch_parts(int elem, const double* coord, const int32_t* connect, const int32_t* node_ptr,
                   const uint8_t* rank, const double* C, int cpe, double factor, const PartArgs& A, int n_parts,
                   int threads, T* vals, cudaStream_t s) {
  switch (elem) {
    case GFEA_TRI3: return launch_parts<GFEA_TRI3, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_QUAD4: return launch_parts<GFEA_QUAD4, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_QUAD9: return launch_parts<GFEA_QUAD9, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_HEXA8: return launch_parts<GFEA_HEXA8, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_TETRA4: return launch_parts<GFEA_TETRA4, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_TRI6: return launch_parts<GFEA_TRI6, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_QUAD8: return launch_parts<GFEA_QUAD8, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_TETRA10: return launch_parts<GFEA_TETRA10, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_HEXA20: return launch_parts<GFEA_HEXA20, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    case GFEA_HEXA27: return launch_parts<GFEA_HEXA27, T>(coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads, vals, s);
    default:
      return parts_ho(elem, coord, connect, node_ptr, rank, C, cpe, factor, A, n_parts, threads,
                      sizeof(T) == 4 ? GFEA_F32 : GFEA_F64, vals, s);
  }
}

// Morton key of a point: 21 bits per axis, interleaved (x lowest)
uint64_t spread21(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

}  // namespace
}  // namespace gfea

using namespace gfea;

extern "C" size_t gfea_part_smem_bytes(int elem, int value_type, int32_t max_part_values, int threads) {
  const bool f32 = value_type == GFEA_F32;
  if (threads <= 0) threads = f32 ? part_threads<float>() : part_threads<double>();
  switch (elem) {
#define GFEA_PART_SMEM(EL)                                                                                \
  case EL:                                                                                                \
    return f32 ? part_smem<EL, float>(max_part_values, threads) : part_smem<EL, double>(max_part_values, threads);
    GFEA_PART_SMEM(GFEA_TRI3)
    GFEA_PART_SMEM(GFEA_QUAD4)
    GFEA_PART_SMEM(GFEA_QUAD9)
    GFEA_PART_SMEM(GFEA_HEXA8)
    GFEA_PART_SMEM(GFEA_TETRA4)
    GFEA_PART_SMEM(GFEA_TRI6)
    GFEA_PART_SMEM(GFEA_QUAD8)
    GFEA_PART_SMEM(GFEA_TETRA10)
    GFEA_PART_SMEM(GFEA_HEXA20)
    GFEA_PART_SMEM(GFEA_HEXA27)
#undef GFEA_PART_SMEM
    default: return part_smem_ho(elem, value_type, max_part_values, threads);
  }
}

extern "C" int gfea_part_plan_host(const double* coord_host, const int32_t* connect_host, int64_t n_elems, int nPe,
                                   int64_t n_nodes, const int32_t* node_ptr_host, int dof_n,
                                   int32_t max_part_values, int32_t* node_off_host, int32_t* part_node_ptr_host,
                                   int32_t* part_nodes_host, int32_t* part_nvals_host, int32_t* visit_ptr_host,
                                   int32_t* visit_elem_host, uint32_t* visit_mask_host, int32_t* n_parts_host,
                                   int64_t* n_visits_host) {
  if (!coord_host || !connect_host || !node_ptr_host || !node_off_host || !part_node_ptr_host || !part_nodes_host ||
      !part_nvals_host || !visit_ptr_host || !visit_elem_host || !visit_mask_host || !n_parts_host || !n_visits_host)
    return GFEA_ERR_ARG;
  if (n_elems <= 0 || n_nodes <= 0 || nPe < 1 || nPe > 32 || dof_n < 1 || dof_n > 3 || max_part_values <= 0)
    return GFEA_ERR_ARG;
  if (n_elems * nPe >= ((int64_t)1 << 31) || n_nodes >= ((int64_t)1 << 31) - 1) return GFEA_ERR_ARG;
  const int64_t Nn = n_nodes, Ne = n_elems;
  for (int64_t i = 0; i < Ne * nPe; ++i)
    if (connect_host[i] < 0 || connect_host[i] >= Nn) return GFEA_ERR_ARG;
  // nodes in Morton order of their coordinates (one scale for every axis)
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t a = 0; a < Nn; ++a)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], coord_host[a * 3 + k]);
      hi[k] = std::max(hi[k], coord_host[a * 3 + k]);
    }
  double ext = 0;
  for (int k = 0; k < 3; ++k) ext = std::max(ext, hi[k] - lo[k]);
  const double scale = ext > 0 ? (double)((1 << 21) - 1) / ext : 0.0;
  std::vector<std::pair<uint64_t, int32_t>> key(Nn);
  for (int64_t a = 0; a < Nn; ++a) {
    uint64_t m = 0;
    for (int k = 0; k < 3; ++k) {
      double t = (coord_host[a * 3 + k] - lo[k]) * scale;
      if (!(t >= 0)) t = 0;
      m |= spread21((uint64_t)std::min(t, (double)((1 << 21) - 1))) << k;
    }
    key[a] = {m, (int32_t)a};
  }
  std::sort(key.begin(), key.end());
  // greedy cut into parts of at most max_part_values CSR values
  std::vector<int32_t> part_of(Nn);
  const int dd = dof_n * dof_n;
  int32_t part = 0;
  int64_t fill = 0;
  part_node_ptr_host[0] = 0;
  for (int64_t s = 0; s < Nn; ++s) {
    const int32_t a = key[s].second;
    const int64_t c = (int64_t)dd * (node_ptr_host[a + 1] - node_ptr_host[a]);
    if (c > max_part_values) return GFEA_ERR_CAPACITY;
    if (fill + c > max_part_values) {
      part_nvals_host[part] = (int32_t)fill;
      part_node_ptr_host[++part] = (int32_t)s;
      fill = 0;
    }
    node_off_host[a] = (int32_t)fill;
    part_of[a] = part;
    part_nodes_host[s] = a;
    fill += c;
  }
  part_nvals_host[part] = (int32_t)fill;
  part_node_ptr_host[++part] = (int32_t)Nn;
  const int32_t n_parts = part;
  // visits: one per (element, part owning one of its nodes), element order within a part
  std::vector<int32_t> cnt(n_parts + 1, 0);
  for (int64_t e = 0; e < Ne; ++e) {
    const int32_t* ce = connect_host + e * nPe;
    for (int p = 0; p < nPe; ++p) {
      const int32_t pp = part_of[ce[p]];
      bool first = true;
      for (int q = 0; q < p; ++q) first &= part_of[ce[q]] != pp;
      if (first) ++cnt[pp];
    }
  }
  visit_ptr_host[0] = 0;
  for (int32_t k = 0; k < n_parts; ++k) visit_ptr_host[k + 1] = visit_ptr_host[k] + cnt[k];
  std::vector<int32_t> cur(visit_ptr_host, visit_ptr_host + n_parts);
  for (int64_t e = 0; e < Ne; ++e) {
    const int32_t* ce = connect_host + e * nPe;
    for (int p = 0; p < nPe; ++p) {
      const int32_t pp = part_of[ce[p]];
      bool first = true;
      for (int q = 0; q < p; ++q) first &= part_of[ce[q]] != pp;
      if (!first) continue;
      uint32_t mask = 0;
      for (int q = p; q < nPe; ++q)
        if (part_of[ce[q]] == pp) mask |= 1u << q;
      const int32_t slot = cur[pp]++;
      visit_elem_host[slot] = (int32_t)e;
      visit_mask_host[slot] = mask;
    }
  }
  // within a part, visits by descending number of owned rows (then element):
  // the lane groups of a warp take consecutive visits and run the same
  // number of row blocks
  {
    std::vector<std::pair<int, int32_t>> tmp;
    for (int32_t k = 0; k < n_parts; ++k) {
      const int32_t b = visit_ptr_host[k], n = visit_ptr_host[k + 1] - b;
      tmp.resize(n);
      for (int32_t i = 0; i < n; ++i) tmp[i] = {-__builtin_popcount(visit_mask_host[b + i]), visit_elem_host[b + i]};
      std::vector<uint32_t> mk(visit_mask_host + b, visit_mask_host + b + n);
      std::vector<int32_t> order(n);
      for (int32_t i = 0; i < n; ++i) order[i] = i;
      std::sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return tmp[x] < tmp[y]; });
      for (int32_t i = 0; i < n; ++i) {
        visit_elem_host[b + i] = tmp[order[i]].second;
        visit_mask_host[b + i] = mk[order[i]];
      }
    }
  }
  *n_parts_host = n_parts;
  *n_visits_host = visit_ptr_host[n_parts];
  return GFEA_OK;
}

extern "C" int gfea_assemble_elastic_parts(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                                           const int32_t* node_ptr, const uint8_t* rank, const double* C,
                                           int c_per_elem, double factor, int value_type, void* values,
                                           const gfea_part_plan* plan, void* stream) {
  if (!coord || !connect || !node_ptr || !rank || !C || !values || !plan || n_elems < 0) return GFEA_ERR_ARG;
  if (plan->version != GFEA_ABI_VERSION || plan->n_parts < 0 || plan->max_part_values <= 0) return GFEA_ERR_ARG;
  if (c_per_elem < 0 || c_per_elem > 4) return GFEA_ERR_ARG;
  if (!plan->node_off || !plan->part_node_ptr || !plan->part_nodes || !plan->part_nvals || !plan->visit_ptr ||
      !plan->visit_elem || !plan->visit_mask)
    return GFEA_ERR_ARG;
  if (n_elems == 0 || plan->n_parts == 0) return GFEA_OK;
  PartArgs A;
  A.max_vals = plan->max_part_values;
  A.node_off = plan->node_off;
  A.part_node_ptr = plan->part_node_ptr;
  A.part_nodes = plan->part_nodes;
  A.part_nvals = plan->part_nvals;
  A.visit_ptr = plan->visit_ptr;
  A.visit_elem = plan->visit_elem;
  A.visit_mask = plan->visit_mask;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int threads = plan->threads;
  if (threads == 0) threads = value_type == GFEA_F32 ? part_threads<float>() : part_threads<double>();
  if (threads < 32 || threads > 256 || threads % 32) return GFEA_ERR_ARG;
  if (value_type == GFEA_F64)
    return dispatch_parts<double>(elem, coord, connect, node_ptr, rank, C, c_per_elem, factor, A, plan->n_parts,
                                  threads, static_cast<double*>(values), s);
  if (value_type == GFEA_F32)
    return dispatch_parts<float>(elem, coord, connect, node_ptr, rank, C, c_per_elem, factor, A, plan->n_parts,
                                 threads, static_cast<float*>(values), s);
  return GFEA_ERR_ARG;
}

// Sparsity pattern on the device.
//
// The reference builds its CSR pattern once per mesh by handing every element
// DOF pair to scipy (COO -> canonical CSR) and then maps each element entry to
// its slot with a searchsorted (EasyFEA/Simulations/_simu.py:1062-1102).  That
// pattern is exactly "every pair of DOFs whose nodes share an element", with
// sorted columns.  Here the same pattern is derived from the node graph:
//   node -> incident elements -> sorted unique neighbour nodes,
// and the per-element slot map shrinks to one uint8 rank per node pair.

#include "common.cuh"

namespace gfea {
namespace {

constexpr int kMaxNb = 128;      // neighbour capacity per node (HEXA8 27, QUAD9 25, HEXA27 125)
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

struct GraphWork {
  int32_t* inc_ptr;   // Nn + 1
  int32_t* cursor;    // Nn
  int32_t* inc_list;  // Ne * nPe
  int32_t* nnb;       // Nn + 1
  int32_t* sums;      // scan block sums
  int32_t* flag;      // 1 int: error flag
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t graph_ws(int64_t Nn, int64_t Ne, int nPe, GraphWork* w, char* base) {
  size_t off = 0;
  auto take = [&](int32_t** p, int64_t n) {
    if (base) *p = reinterpret_cast<int32_t*>(base + off);
    off += align256(sizeof(int32_t) * (size_t)n);
  };
  GraphWork tmp;
  if (!w) w = &tmp;
  take(&w->inc_ptr, Nn + 1);
  take(&w->cursor, Nn);
  take(&w->inc_list, Ne * nPe);
  take(&w->nnb, Nn + 1);
  take(&w->sums, ceil_div(Nn + 1, kScanTile) + 1);
  take(&w->flag, 1);
  return off;
}

// ---- exclusive scan of int32[n] into out[n] (out may alias in) -------------

__global__ void scan_reduce(const int32_t* in, int64_t n, int32_t* sums) {
  __shared__ int32_t sh[kScanThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  int32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kScanThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

// single block: exclusive scan of the block sums (any count)
__global__ void scan_sums(int32_t* sums, int nb) {
  __shared__ int32_t sh[kScanThreads];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int c = 0; c < nb; c += kScanThreads) {
    const int i = c + threadIdx.x;
    const int32_t v = i < nb ? sums[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {
      int32_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry += sh[kScanThreads - 1];
    __syncthreads();
  }
}

__global__ void scan_apply(const int32_t* in, int64_t n, const int32_t* sums, int32_t* out) {
  __shared__ int32_t sh[kScanThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    int32_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  int32_t run = sums[blockIdx.x] + sh[threadIdx.x] - s;
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

int exclusive_scan(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, cudaStream_t s) {
  const int nb = (int)ceil_div(n, kScanTile);
  if (nb == 0) return GFEA_OK;
  scan_reduce<<<nb, kScanThreads, 0, s>>>(in, n, sums);
  GFEA_LAUNCH_CHECK();
  scan_sums<<<1, kScanThreads, 0, s>>>(sums, nb);
  GFEA_LAUNCH_CHECK();
  scan_apply<<<nb, kScanThreads, 0, s>>>(in, n, sums, out);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

// ---- incidence ---------------------------------------------------------------

__global__ void inc_count(const int32_t* connect, int64_t n, int64_t Nn, int32_t* cnt, int32_t* flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = connect[i];
    if (a < 0 || a >= Nn) { atomicOr(flag, 1); continue; }
    atomicAdd(&cnt[a], 1);
  }
}

__global__ void inc_fill(const int32_t* connect, int64_t Ne, int nPe, int64_t Nn, int32_t* cursor,
                         int32_t* list) {
  const int64_t n = Ne * nPe;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = connect[i];
    if (a < 0 || a >= Nn) continue;
    const int32_t pos = atomicAdd(&cursor[a], 1);
    list[pos] = (int32_t)(i / nPe);
  }
}

// Sorted unique neighbour nodes of node a, into a local buffer.
__device__ int gather_neighbours(int64_t a, const int32_t* connect, int nPe, const int32_t* inc_ptr,
                                 const int32_t* inc_list, int32_t* buf, bool* overflow) {
  int n = 0;
  for (int32_t k = inc_ptr[a]; k < inc_ptr[a + 1]; ++k) {
    const int64_t e = inc_list[k];
    for (int q = 0; q < nPe; ++q) {
      const int32_t b = connect[e * nPe + q];
      // binary search for the insertion point
      int lo = 0, hi = n;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (buf[mid] < b) lo = mid + 1; else hi = mid;
      }
      if (lo < n && buf[lo] == b) continue;
      if (n == kMaxNb) { *overflow = true; return n; }
      for (int t = n; t > lo; --t) buf[t] = buf[t - 1];
      buf[lo] = b;
      ++n;
    }
  }
  return n;
}

__global__ void nb_count(const int32_t* connect, int nPe, int64_t Nn, const int32_t* inc_ptr,
                         const int32_t* inc_list, int32_t* nnb, int32_t* flag) {
  int32_t buf[kMaxNb];
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x) {
    bool over = false;
    const int n = gather_neighbours(a, connect, nPe, inc_ptr, inc_list, buf, &over);
    if (over) atomicOr(flag, 2);
    nnb[a] = n;
  }
}

__global__ void nb_fill(const int32_t* connect, int nPe, int64_t Nn, const int32_t* inc_ptr,
                        const int32_t* inc_list, const int32_t* node_ptr, int32_t* nbr, int32_t* flag) {
  int32_t buf[kMaxNb];
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x) {
    bool over = false;
    const int n = gather_neighbours(a, connect, nPe, inc_ptr, inc_list, buf, &over);
    if (over || n != node_ptr[a + 1] - node_ptr[a]) { atomicOr(flag, 2); continue; }
    int32_t* dst = nbr + node_ptr[a];
    for (int k = 0; k < n; ++k) dst[k] = buf[k];
  }
}

__global__ void rank_fill(const int32_t* connect, int64_t Ne, int nPe, const int32_t* node_ptr,
                          const int32_t* nbr, uint8_t* rank, int32_t* flag) {
  const int64_t n = Ne * nPe * nPe;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / (nPe * nPe);
    const int p = (int)((i / nPe) % nPe), q = (int)(i % nPe);
    const int32_t a = connect[e * nPe + p], b = connect[e * nPe + q];
    int lo = node_ptr[a], hi = node_ptr[a + 1];
    const int base = lo;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (nbr[mid] < b) lo = mid + 1; else hi = mid;
    }
    if (lo >= node_ptr[a + 1] || nbr[lo] != b || lo - base > 255) { atomicOr(flag, 4); rank[i] = 0; continue; }
    rank[i] = (uint8_t)(lo - base);
  }
}

__global__ void csr_pattern_kernel(const int32_t* node_ptr, const int32_t* nbr, int64_t Nn, int dof_n,
                                   int64_t* indptr, int32_t* indices) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t a = warp; a < Nn; a += nwarps) {
    const int32_t p0 = node_ptr[a];
    const int32_t nb = node_ptr[a + 1] - p0;
    const int64_t w = (int64_t)dof_n * nb;
    for (int i = 0; i < dof_n; ++i) {
      const int64_t row0 = (int64_t)dof_n * dof_n * p0 + i * w;
      if (lane == 0) indptr[a * dof_n + i] = row0;
      for (int64_t t = lane; t < w; t += 32) {
        const int32_t k = (int32_t)(t / dof_n), j = (int32_t)(t % dof_n);
        indices[row0 + t] = nbr[p0 + k] * dof_n + j;
      }
    }
    if (a == Nn - 1 && lane == 0) indptr[Nn * dof_n] = (int64_t)dof_n * dof_n * node_ptr[Nn];
  }
}

// Each node's incident elements in ascending order (insertion sort in place:
// a node of a conforming mesh has a few tens of elements at most).
__global__ void inc_sort(const int32_t* inc_ptr, int64_t Nn, int32_t* list) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x) {
    const int32_t lo = inc_ptr[a], hi = inc_ptr[a + 1];
    for (int32_t i = lo + 1; i < hi; ++i) {
      const int32_t v = list[i];
      int32_t j = i;
      while (j > lo && list[j - 1] > v) {
        list[j] = list[j - 1];
        --j;
      }
      list[j] = v;
    }
  }
}

}  // namespace
}  // namespace gfea

using namespace gfea;

extern "C" int gfea_graph_workspace_size(int64_t n_nodes, int64_t n_elems, int nPe, size_t* bytes_host) {
  if (!bytes_host || n_nodes < 0 || n_elems < 0 || nPe < 1 || nPe > 32) return GFEA_ERR_ARG;
  *bytes_host = graph_ws(n_nodes, n_elems, nPe, nullptr, nullptr);
  return GFEA_OK;
}

extern "C" int gfea_graph_count(const int32_t* connect, int64_t n_elems, int nPe, int64_t n_nodes,
                                int32_t* node_ptr, int64_t* n_pairs_host, void* work, size_t work_bytes,
                                void* stream) {
  if (!connect || !node_ptr || !work || n_nodes <= 0 || n_elems <= 0 || nPe < 1 || nPe > 32) return GFEA_ERR_ARG;
  if (n_elems * nPe >= ((int64_t)1 << 31) || n_nodes >= ((int64_t)1 << 31) - 1) return GFEA_ERR_ARG;
  GraphWork w;
  if (graph_ws(n_nodes, n_elems, nPe, &w, static_cast<char*>(work)) > work_bytes) return GFEA_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GFEA_CUDA_TRY(cudaMemsetAsync(w.inc_ptr, 0, sizeof(int32_t) * (n_nodes + 1), s));
  GFEA_CUDA_TRY(cudaMemsetAsync(w.flag, 0, sizeof(int32_t), s));
  const int64_t nent = n_elems * nPe;
  inc_count<<<grid_for(nent, 256), 256, 0, s>>>(connect, nent, n_nodes, w.inc_ptr, w.flag);
  GFEA_LAUNCH_CHECK();
  int st = exclusive_scan(w.inc_ptr, w.inc_ptr, n_nodes + 1, w.sums, s);
  if (st) return st;
  GFEA_CUDA_TRY(cudaMemcpyAsync(w.cursor, w.inc_ptr, sizeof(int32_t) * n_nodes, cudaMemcpyDeviceToDevice, s));
  inc_fill<<<grid_for(nent, 256), 256, 0, s>>>(connect, n_elems, nPe, n_nodes, w.cursor, w.inc_list);
  GFEA_LAUNCH_CHECK();
  nb_count<<<grid_for(n_nodes, 128), 128, 0, s>>>(connect, nPe, n_nodes, w.inc_ptr, w.inc_list, w.nnb, w.flag);
  GFEA_LAUNCH_CHECK();
  GFEA_CUDA_TRY(cudaMemsetAsync(w.nnb + n_nodes, 0, sizeof(int32_t), s));
  st = exclusive_scan(w.nnb, node_ptr, n_nodes + 1, w.sums, s);
  if (st) return st;
  int32_t host[2];
  GFEA_CUDA_TRY(cudaMemcpyAsync(&host[0], node_ptr + n_nodes, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFEA_CUDA_TRY(cudaMemcpyAsync(&host[1], w.flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFEA_CUDA_TRY(cudaStreamSynchronize(s));
  if (host[1] & 1) return GFEA_ERR_ARG;
  if (host[1] & 2) return GFEA_ERR_CAPACITY;
  if (n_pairs_host) *n_pairs_host = host[0];
  return GFEA_OK;
}

extern "C" int gfea_graph_fill(const int32_t* connect, int64_t n_elems, int nPe, int64_t n_nodes,
                               const int32_t* node_ptr, int32_t* nbr, uint8_t* rank, void* work,
                               size_t work_bytes, void* stream) {
  if (!connect || !node_ptr || !nbr || !rank || !work || n_nodes <= 0 || n_elems <= 0) return GFEA_ERR_ARG;
  GraphWork w;
  if (graph_ws(n_nodes, n_elems, nPe, &w, static_cast<char*>(work)) > work_bytes) return GFEA_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  nb_fill<<<grid_for(n_nodes, 128), 128, 0, s>>>(connect, nPe, n_nodes, w.inc_ptr, w.inc_list, node_ptr, nbr, w.flag);
  GFEA_LAUNCH_CHECK();
  const int64_t nr = n_elems * nPe * nPe;
  rank_fill<<<grid_for(nr, 256), 256, 0, s>>>(connect, n_elems, nPe, node_ptr, nbr, rank, w.flag);
  GFEA_LAUNCH_CHECK();
  int32_t flag = 0;
  GFEA_CUDA_TRY(cudaMemcpyAsync(&flag, w.flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFEA_CUDA_TRY(cudaStreamSynchronize(s));
  if (flag & 2) return GFEA_ERR_CAPACITY;
  if (flag) return GFEA_ERR_ARG;
  return GFEA_OK;
}

extern "C" int gfea_csr_pattern(const int32_t* node_ptr, const int32_t* nbr, int64_t n_nodes, int dof_n,
                                int64_t* indptr, int32_t* indices, void* stream) {
  if (!node_ptr || !nbr || !indptr || !indices || n_nodes <= 0 || dof_n < 1 || dof_n > 3) return GFEA_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  csr_pattern_kernel<<<grid_for(n_nodes * 32, 256), 256, 0, s>>>(node_ptr, nbr, n_nodes, dof_n, indptr, indices);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" int gfea_node_incidence(const int32_t* connect, int64_t n_elems, int nPe, int64_t n_nodes,
                                   int32_t* inc_ptr, int32_t* inc_list, void* work, size_t work_bytes,
                                   void* stream) {
  if (!connect || !inc_ptr || !inc_list || !work || n_nodes <= 0 || n_elems <= 0 || nPe < 1 || nPe > 32)
    return GFEA_ERR_ARG;
  if (n_elems * nPe >= ((int64_t)1 << 31) || n_nodes >= ((int64_t)1 << 31) - 1) return GFEA_ERR_ARG;
  GraphWork w;
  if (graph_ws(n_nodes, n_elems, nPe, &w, static_cast<char*>(work)) > work_bytes) return GFEA_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GFEA_CUDA_TRY(cudaMemsetAsync(inc_ptr, 0, sizeof(int32_t) * (n_nodes + 1), s));
  GFEA_CUDA_TRY(cudaMemsetAsync(w.flag, 0, sizeof(int32_t), s));
  const int64_t nent = n_elems * nPe;
  inc_count<<<grid_for(nent, 256), 256, 0, s>>>(connect, nent, n_nodes, inc_ptr, w.flag);
  GFEA_LAUNCH_CHECK();
  int st = exclusive_scan(inc_ptr, inc_ptr, n_nodes + 1, w.sums, s);
  if (st) return st;
  GFEA_CUDA_TRY(cudaMemcpyAsync(w.cursor, inc_ptr, sizeof(int32_t) * n_nodes, cudaMemcpyDeviceToDevice, s));
  inc_fill<<<grid_for(nent, 256), 256, 0, s>>>(connect, n_elems, nPe, n_nodes, w.cursor, inc_list);
  GFEA_LAUNCH_CHECK();
  inc_sort<<<grid_for(n_nodes, 128), 128, 0, s>>>(inc_ptr, n_nodes, inc_list);
  GFEA_LAUNCH_CHECK();
  int32_t flag = 0;
  GFEA_CUDA_TRY(cudaMemcpyAsync(&flag, w.flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFEA_CUDA_TRY(cudaStreamSynchronize(s));
  return flag ? GFEA_ERR_ARG : GFEA_OK;
}

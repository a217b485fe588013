// Sparse SPD solve: node-block CSR SpMV, nodal block-Jacobi and PCG.
//
// The CSR values keep the reference's scalar CSR layout, but their column
// structure is read from the node graph: a node's dof_n rows share one sorted
// neighbour list, so the SpMV reads 4 bytes of index per dof_n^2 values
// instead of 4 per value.  G lanes of a warp serve one node; within a row
// lane t reads value t, t+G, ... so every load instruction is contiguous.
//
// Dirichlet DOFs are eliminated as in Solvers.__Solver_1 (EasyFEA/Simulations/
// Solvers.py:502-553) but without extracting A_ii: PCG runs on the masked
// operator P A P + (I - P) (P = diag(unknown)); search directions vanish on
// known DOFs, so the product is a plain SpMV with known rows zeroed.
//
// One PCG iteration is two kernels:
//   dir_spmv : p' = z + beta p  (own rows), Ap' (gathered z + beta p), p'.Ap'
//   update   : x += alpha p', r -= alpha Ap', z = D^-1 r, r.z, r.r
// Reductions are per-block partials summed in a fixed order by the last block
// to finish (atomic ticket, no spinning), which also derives the scalar
// recurrences (alpha, beta, convergence) on the device.  Kernels return early
// once the device flag 'done' is set, so a host loop (or a captured graph) may
// run more iterations than needed at no cost.

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.cuh"
#include "rowops.cuh"

namespace gfea {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = kSMs * 8;

struct Scal {
  double rz, rr, pap, alpha, beta, bb, tol2, rr_true, absAx;
  int32_t done, iters, status, max_iters;
  uint32_t ticket1, ticket2, ticket3, pad;
};

// Optional CUDA-event timing of the PCG direction/SpMV kernel (the dominant
// launch of a solve), read back by gfea_profile_read.
struct KernelProfile {
  static constexpr int kPairs = 64;
  bool on = false;
  bool created = false;
  cudaEvent_t ev[2 * kPairs];
  double ms = 0;
  long long n = 0;
};
KernelProfile& prof() {
  static KernelProfile p;
  return p;
}



// Publish NV block partials; returns true in the last block, where out[] holds
// the fixed-order totals (valid in every thread of that block).
template <int NV>
__device__ bool reduce_last(const double (&v)[NV], double* partials, uint32_t* ticket, double (&out)[NV]) {
  __shared__ double sh[32];
  __shared__ bool last;
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k] = block_sum(v[k], sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = s[k];
    __threadfence();
    const uint32_t t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) a += ((volatile double*)partials)[k * gridDim.x + i];
    out[k] = block_sum(a, sh);
    if (threadIdx.x == 0) sh[31] = out[k];
    __syncthreads();
    out[k] = sh[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0;
  return true;
}

// ---------------------------------------------------------------------------
// node-row products
// ---------------------------------------------------------------------------


// y = A x (unmasked)
template <int D, int G, typename T>
__global__ void __launch_bounds__(kThreads) spmv_kernel(SysT<T> S, const T* __restrict__ x, T* __restrict__ y) {
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    T acc[D];
    node_rows<D, G, T, T>(ac, lane, S, [&](int64_t c) { return x[c]; }, acc);
    if (a < Nn && lane < D) {
      T v = acc[0];
#pragma unroll
      for (int i = 1; i < D; ++i) if (lane == i) v = acc[i];
      y[a * D + lane] = v;
    }
  }
}

// FP64 residual of the reduced system: r = P (b - A x); partials r.r,
// ||P (b - A x_c)||^2 (x_c: x on known columns only, the reference norm) and
// ||P |A| |x|||^2 (scale of the rounding floor of r).
template <int D, int G, typename T>
__global__ void __launch_bounds__(kThreads) resid_kernel(SysT<T> S, const double* __restrict__ b,
                                                         const double* __restrict__ x, double* __restrict__ r,
                                                         double* partials, Scal* sc) {
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  double v[3] = {0, 0, 0};
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    double all[D], kn[D], ab[D];
    node_rows<D, G, T, double>(ac, lane, S, [&](int64_t c) { return x[c]; }, all);
    node_rows<D, G, T, double>(ac, lane, S, [&](int64_t c) { return S.known[c] ? x[c] : 0.0; }, kn);
    node_rows<D, G, T, double, true>(ac, lane, S, [&](int64_t c) { return fabs(x[c]); }, ab);
    if (a < Nn && lane == 0) {
#pragma unroll
      for (int i = 0; i < D; ++i) {
        const int64_t dof = a * D + i;
        const bool unk = !S.known[dof];
        const double ri = unk ? b[dof] - all[i] : 0.0;
        const double rci = unk ? b[dof] - kn[i] : 0.0;
        const double ai = unk ? ab[i] + fabs(b[dof]) : 0.0;
        r[dof] = ri;
        v[0] += ri * ri;
        v[1] += rci * rci;
        v[2] += ai * ai;
      }
    }
  }
  double out[3];
  if (reduce_last<3>(v, partials, &sc->ticket3, out) && threadIdx.x == 0) {
    sc->rr_true = out[0];
    sc->bb = out[1];
    sc->absAx = out[2];
  }
}

// Block-Jacobi: invert the (masked) dof_n x dof_n diagonal block of each node.
template <int D, typename T>
__global__ void bjacobi_kernel(SysT<T> S, T* __restrict__ dinv, int32_t* flag) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < S.Nn; a += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p0 = S.node_ptr[a], p1 = S.node_ptr[a + 1];
    int lo = p0, hi = p1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (S.nbr[mid] < a) lo = mid + 1; else hi = mid;
    }
    const bool has = lo < p1 && S.nbr[lo] == a;
    const int32_t W = D * (p1 - p0);
    const int k = lo - p0;
    double M[D][D];
    bool kn[D];
#pragma unroll
    for (int i = 0; i < D; ++i) kn[i] = S.known[a * D + i] != 0;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double v = has ? (double)S.vals[(int64_t)D * D * p0 + (int64_t)i * W + D * k + j] : 0.0;
        if (kn[i] || kn[j]) v = (i == j) ? 1.0 : 0.0;
        M[i][j] = v;
      }
    double iM[D][D];
    const double det = det_inv<D>(M, iM);
    bool bad = !(fabs(det) > 0) || !isfinite(det);
    if (bad) {
      atomicOr(flag, 1);
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) iM[i][j] = (i == j) ? 1.0 : 0.0;
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) dinv[a * D * D + i * D + j] = (T)iM[i][j];
  }
}

// z = D^-1 r, partial r.z and r.r; the last block derives beta and the
// convergence state.  mode 0: PCG iteration (x += alpha p, r -= alpha Ap
// first); mode 1: start (beta = 0); mode 2: residual replaced by a reliable
// update (beta = r.z / previous r.z, the search direction is kept).
template <int D, typename T>
__global__ void __launch_bounds__(kThreads) update_kernel(int64_t Nn, const uint8_t* __restrict__ known,
                                                          const T* __restrict__ dinv, T* __restrict__ x,
                                                          T* __restrict__ r, T* __restrict__ z,
                                                          const T* __restrict__ p, const T* __restrict__ Ap,
                                                          double* partials, Scal* sc, int mode) {
  if (mode == 0 && sc->done) return;
  const double alpha = mode == 0 ? sc->alpha : 0.0;
  double v[2] = {0, 0};
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x) {
    T rl[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const int64_t dof = a * D + i;
      T ri = r[dof];
      if (mode == 0) {
        x[dof] += (T)alpha * p[dof];
        ri -= (T)alpha * Ap[dof];
        r[dof] = ri;
      }
      rl[i] = ri;
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
      T zi = 0;
#pragma unroll
      for (int j = 0; j < D; ++j) zi += dinv[a * D * D + i * D + j] * rl[j];
      if (known[a * D + i]) zi = 0;
      z[a * D + i] = zi;
      v[0] += (double)rl[i] * (double)zi;
      v[1] += (double)rl[i] * (double)rl[i];
    }
  }
  double out[2];
  if (reduce_last<2>(v, partials, &sc->ticket2, out) && threadIdx.x == 0) {
    const double rz_new = out[0], rr = out[1];
    sc->beta = mode == 1 ? 0.0 : rz_new / sc->rz;
    // a replaced residual larger than the iterated one (drift) restarts the direction
    if (mode == 2 && !(sc->beta <= 1.0)) sc->beta = 0.0;
    sc->rz = rz_new;
    sc->rr = rr;
    if (mode != 0) return;  // the host sets the next stopping threshold
    sc->iters += 1;
    if (!isfinite(rr) || !isfinite(rz_new)) {
      sc->status = GFEA_ERR_NAN;
      sc->done = 1;
    } else if (rr <= sc->tol2) {
      sc->status = GFEA_OK;
      sc->done = 1;
    } else if (sc->iters >= sc->max_iters) {
      sc->status = GFEA_ERR_NOT_CONVERGED;
      sc->done = 1;
    }
  }
}

// p' = z + beta p (own rows), Ap' = masked A p'; partial p'.Ap'; last block sets alpha.
template <int D, int G, typename T>
__global__ void __launch_bounds__(kThreads) dir_spmv_kernel(SysT<T> S, const T* __restrict__ z,
                                                            const T* __restrict__ p_old, T* __restrict__ p_new,
                                                            T* __restrict__ Ap, double* partials, Scal* sc) {
  if (sc->done) return;
  const T beta = (T)sc->beta;
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  double v[1] = {0};
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    T acc[D];
    auto dir = [&](int64_t c) { return z[c] + beta * p_old[c]; };
    if (sizeof(T) == 4 && S.diff)
      node_rows<D, G, T, T, false, true>(ac, lane, S, dir, acc);
    else
      node_rows<D, G, T, T>(ac, lane, S, dir, acc);
    if (a < Nn && lane < D) {
      T av = acc[0];
#pragma unroll
      for (int i = 1; i < D; ++i) if (lane == i) av = acc[i];
      const int64_t dof = a * D + lane;
      const T pn = z[dof] + beta * p_old[dof];
      if (S.known[dof]) av = 0;
      p_new[dof] = pn;
      Ap[dof] = av;
      v[0] += (double)pn * (double)av;
    }
  }
  double out[1];
  if (reduce_last<1>(v, partials, &sc->ticket1, out) && threadIdx.x == 0) {
    sc->pap = out[0];
    if (!(out[0] > 0) || !isfinite(out[0])) {
      sc->status = isfinite(out[0]) ? GFEA_ERR_BREAKDOWN : GFEA_ERR_NAN;
      sc->done = 1;
    } else {
      sc->alpha = sc->rz / out[0];
    }
  }
}

template <typename T>
__global__ void cast_kernel(const double* __restrict__ s, T* __restrict__ d, int64_t n) {
  // FP64 -> T copy
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (T)s[i];
}

template <typename T>
__global__ void add_correction_kernel(double* __restrict__ x, const T* __restrict__ dx, const uint8_t* known, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!known[i]) x[i] += (double)dx[i];
}

__global__ void zero_unknown_kernel(double* __restrict__ x, const uint8_t* known, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!known[i]) x[i] = 0.0;
}

// Sets the threshold at which the device stops iterating (the next reliable
// update), keeping the iteration count.
__global__ void set_trigger_kernel(Scal* sc, double tol2, int max_iters) {
  sc->tol2 = tol2;
  sc->max_iters = max_iters;
  sc->status = GFEA_OK;
  if (!isfinite(sc->rr) || !isfinite(sc->rz)) {
    sc->status = GFEA_ERR_NAN;
    sc->done = 1;
  } else {
    sc->done = (sc->rr <= tol2 || sc->iters >= max_iters) ? 1 : 0;
    if (sc->iters >= max_iters) sc->status = GFEA_ERR_NOT_CONVERGED;
  }
}

// reaction / energy
template <int D, int G>
__global__ void __launch_bounds__(kThreads) reaction_kernel(SysT<double> S, const double* __restrict__ x,
                                                            double* __restrict__ Ax, double* partials, Scal* sc) {
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  double v[1] = {0};
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    double acc[D];
    node_rows<D, G, double, double>(ac, lane, S, [&](int64_t c) { return x[c]; }, acc);
    if (a < Nn && lane < D) {
      double av = acc[0];
#pragma unroll
      for (int i = 1; i < D; ++i) if (lane == i) av = acc[i];
      Ax[a * D + lane] = av;
      v[0] += 0.5 * x[a * D + lane] * av;
    }
  }
  double out[1];
  if (reduce_last<1>(v, partials, &sc->ticket1, out) && threadIdx.x == 0) sc->rr_true = out[0];
}

__global__ void gather_sum_kernel(const double* __restrict__ Ax, const int64_t* __restrict__ dofs, int64_t n,
                                  double* partials, Scal* sc) {
  double v[1] = {0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[0] += Ax[dofs[i]];
  double out[1];
  if (reduce_last<1>(v, partials, &sc->ticket2, out) && threadIdx.x == 0) sc->pap = out[0];
}

__global__ void max_abs_diff_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                                    unsigned long long* out) {
  double m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = fabs(a[i] - b[i]);
    m = fmax(m, isnan(d) ? INFINITY : d);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  // non-negative doubles order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int pick_lanes(const gfea_system* s, int requested) {
  if (requested == 4 || requested == 8 || requested == 16 || requested == 32) return requested;
  // values per row W = dof_n * neighbours: small groups for short rows
  const double W = s->n_nodes > 0 ? (double)s->dof_n * (double)s->n_pairs / (double)s->n_nodes : 1.0;
  if (W <= 10) return 4;
  if (W <= 24) return 8;
  if (W <= 56) return 16;
  return 32;
}

int grid_nodes(int64_t Nn, int G) {
  const int64_t groups_per_block = kThreads / G;
  int64_t g = ceil_div(Nn, groups_per_block);
  if (g > kMaxBlocks) g = kMaxBlocks;
  if (g < 1) g = 1;
  return (int)g;
}

int grid_elems(int64_t n) {
  int64_t g = ceil_div(n, kThreads);
  if (g > kMaxBlocks) g = kMaxBlocks;
  if (g < 1) g = 1;
  return (int)g;
}

struct PcgWork {
  void* r; void* z; void* pa; void* pb; void* Ap; void* dinv; void* dx;  // T-typed (inner solve)
  double* r64;                                                         // FP64 residual
  double* partials;
  Scal* sc;
  int32_t* flag;
};

template <typename T>
size_t pcg_layout(int64_t Nn, int D, PcgWork* w, char* base) {
  size_t off = 0;
  const int64_t N = Nn * D;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  PcgWork t;
  if (!w) w = &t;
  w->r = take(sizeof(T) * N);
  w->z = take(sizeof(T) * N);
  w->pa = take(sizeof(T) * N);
  w->pb = take(sizeof(T) * N);
  w->Ap = take(sizeof(T) * N);
  w->dinv = take(sizeof(T) * N * D);
  w->dx = take(sizeof(T) * N);
  w->r64 = reinterpret_cast<double*>(take(sizeof(double) * N));
  w->partials = reinterpret_cast<double*>(take(sizeof(double) * 4 * kMaxBlocks));
  w->sc = reinterpret_cast<Scal*>(take(sizeof(Scal)));
  w->flag = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * 4));
  return off;
}

template <typename T>
SysT<T> sys_t(const gfea_system* s);
template <>
SysT<double> sys_t<double>(const gfea_system* s) {
  return SysT<double>{s->n_nodes, s->node_ptr, s->nbr, s->vals64, s->known, s->translation_invariant};
}
template <>
SysT<float> sys_t<float>(const gfea_system* s) {
  return SysT<float>{s->n_nodes, s->node_ptr, s->nbr, s->vals32, s->known, s->translation_invariant};
}

// Launch helpers dispatching (D, G).
#define GFEA_DG_SWITCH(D, G, CALL)                                   \
  switch (D * 100 + G) {                                             \
    case 104: { constexpr int DD = 1, GG = 4; CALL; } break;          \
    case 108: { constexpr int DD = 1, GG = 8; CALL; } break;          \
    case 116: { constexpr int DD = 1, GG = 16; CALL; } break;         \
    case 132: { constexpr int DD = 1, GG = 32; CALL; } break;         \
    case 204: { constexpr int DD = 2, GG = 4; CALL; } break;          \
    case 208: { constexpr int DD = 2, GG = 8; CALL; } break;          \
    case 216: { constexpr int DD = 2, GG = 16; CALL; } break;         \
    case 232: { constexpr int DD = 2, GG = 32; CALL; } break;         \
    case 304: { constexpr int DD = 3, GG = 4; CALL; } break;          \
    case 308: { constexpr int DD = 3, GG = 8; CALL; } break;          \
    case 316: { constexpr int DD = 3, GG = 16; CALL; } break;         \
    case 332: { constexpr int DD = 3, GG = 32; CALL; } break;         \
    default: return GFEA_ERR_ARG;                                    \
  }

#define GFEA_D_SWITCH(D, CALL)                         \
  switch (D) {                                         \
    case 1: { constexpr int DD = 1; CALL; } break;     \
    case 2: { constexpr int DD = 2; CALL; } break;     \
    case 3: { constexpr int DD = 3; CALL; } break;     \
    default: return GFEA_ERR_ARG;                      \
  }

int launch_resid(const gfea_system* s, int G, const double* b, const double* x, PcgWork& w, cudaStream_t st) {
  const SysT<double> S = sys_t<double>(s);
  const int grid = grid_nodes(s->n_nodes, G);
  GFEA_DG_SWITCH(s->dof_n, G, (resid_kernel<DD, GG, double><<<grid, kThreads, 0, st>>>(S, b, x, w.r64, w.partials, w.sc)));
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <typename T>
int launch_bjacobi(const gfea_system* s, PcgWork& w, cudaStream_t st) {
  const SysT<T> S = sys_t<T>(s);
  GFEA_D_SWITCH(s->dof_n, (bjacobi_kernel<DD, T><<<grid_elems(s->n_nodes), kThreads, 0, st>>>(S, (T*)w.dinv, w.flag)));
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <typename T>
int launch_update(const gfea_system* s, PcgWork& w, T* x, T* p, int mode, cudaStream_t st) {
  const int grid = grid_elems(s->n_nodes);
  GFEA_D_SWITCH(s->dof_n, (update_kernel<DD, T><<<grid, kThreads, 0, st>>>(s->n_nodes, s->known, (const T*)w.dinv, x,
                                                                            (T*)w.r, (T*)w.z, p, (const T*)w.Ap,
                                                                            w.partials + 2 * kMaxBlocks, w.sc, mode)));
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <typename T>
int launch_dir(const gfea_system* s, int G, PcgWork& w, const T* p_old, T* p_new, cudaStream_t st) {
  const SysT<T> S = sys_t<T>(s);
  const int grid = grid_nodes(s->n_nodes, G);
  GFEA_DG_SWITCH(s->dof_n, G, (dir_spmv_kernel<DD, GG, T><<<grid, kThreads, 0, st>>>(S, (const T*)w.z, p_old, p_new, (T*)w.Ap,
                                                                                      w.partials, w.sc)));
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

// Runs PCG iterations until the device flags done; checks every 'check'
// iterations.  pa holds the current search direction on entry and exit.
template <typename T>
int pcg_loop(const gfea_system* s, int G, PcgWork& w, T* x, int check, Scal* host_sc, T*& pa, T*& pb,
             int iters0, cudaStream_t st) {
  // iteration j reads direction buf[j % 2] and writes buf[(j + 1) % 2]; launches
  // after the device set 'done' are no-ops, so the current direction follows
  // from the number of iterations actually performed
  T* buf[2] = {pa, pb};
  KernelProfile& P = prof();
  const bool timed = P.on && check <= KernelProfile::kPairs;
  int before = iters0;
  for (int j = 0;;) {
    for (int it = 0; it < check; ++it, ++j) {
      if (timed) GFEA_CUDA_TRY(cudaEventRecord(P.ev[2 * it], st));
      int e = launch_dir<T>(s, G, w, buf[j & 1], buf[(j + 1) & 1], st);
      if (e) return e;
      if (timed) GFEA_CUDA_TRY(cudaEventRecord(P.ev[2 * it + 1], st));
      e = launch_update<T>(s, w, x, buf[(j + 1) & 1], 0, st);
      if (e) return e;
    }
    GFEA_CUDA_TRY(cudaMemcpyAsync(host_sc, w.sc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
    GFEA_CUDA_TRY(cudaStreamSynchronize(st));
    if (timed) {  // durations of the direction/SpMV launches that did work
      const int performed = host_sc->iters - before;
      for (int it = 0; it < performed && it < check; ++it) {
        float ms = 0;
        GFEA_CUDA_TRY(cudaEventElapsedTime(&ms, P.ev[2 * it], P.ev[2 * it + 1]));
        P.ms += ms;
        P.n += 1;
      }
    }
    before = host_sc->iters;
    if (host_sc->done) break;
  }
  const int performed = host_sc->iters - iters0;
  pa = buf[performed & 1];
  pb = buf[(performed + 1) & 1];
  return GFEA_OK;
}

int fetch(Scal* h, PcgWork& w, cudaStream_t st) {
  GFEA_CUDA_TRY(cudaMemcpyAsync(h, w.sc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
  GFEA_CUDA_TRY(cudaStreamSynchronize(st));
  return GFEA_OK;
}

// PCG in T precision with reliable updates (FP64 residual replacement):
//   the iteration runs on T values and vectors with FP64 dots and scalar
//   recurrences, accumulating its correction in dx; whenever the iterated
//   residual has dropped by delta^2 since the last update, dx is added to the
//   FP64 solution, r = P(b - A x) is recomputed with the FP64 operator and
//   replaces the iterated residual, and the iteration continues along the same
//   search direction.  It stops when the FP64 residual satisfies
//   ||r|| <= max(rtol ||P(b - A x_c)||, floor), floor = 32 eps64 ||P(|A||x| + |b|)||
//   (the rounding level of an FP64 residual).
template <typename T>
int refine_solve(const gfea_system* s, const double* b, double* x, const gfea_pcg_opts* o, void* work,
                 size_t work_bytes, gfea_pcg_result* res, cudaStream_t st) {
  PcgWork w;
  if (pcg_layout<T>(s->n_nodes, s->dof_n, &w, static_cast<char*>(work)) > work_bytes) return GFEA_ERR_WORKSPACE;
  const int G = pick_lanes(s, o->lanes);
  const int64_t N = s->n_nodes * s->dof_n;
  const int check = o->check_every > 0 ? o->check_every : 32;
  const bool fp64 = sizeof(T) == 8;
  const double eps64 = 2.220446049250313e-16;
  // reliable update after the iterated residual fell by delta: inner_rtol
  // (default 0.1) in FP32, whose recursive residual drifts from the true one
  // by ~eps32 * condition; 1000x in FP64
  const double dlt = (o->inner_rtol > 0 && o->inner_rtol < 1) ? o->inner_rtol : 0.1;
  const double delta2 = fp64 ? 1e-6 : dlt * dlt;
  Scal hs;
  GFEA_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(Scal), st));
  GFEA_CUDA_TRY(cudaMemsetAsync(w.flag, 0, sizeof(int32_t) * 4, st));
  int e = launch_bjacobi<T>(s, w, st);
  if (e) return e;
  e = launch_resid(s, G, b, x, w, st);
  if (e) return e;
  int32_t flag = 0;
  GFEA_CUDA_TRY(cudaMemcpyAsync(&flag, w.flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  e = fetch(&hs, w, st);
  if (e) return e;
  if (flag) { res->status = GFEA_ERR_SINGULAR; return GFEA_ERR_SINGULAR; }
  const double bb = hs.bb;
  if (!(bb == bb) || !isfinite(hs.rr_true)) { res->status = GFEA_ERR_NAN; return GFEA_ERR_NAN; }
  if (bb == 0) {  // b_i - A_ic x_c = 0: the unknowns are zero
    zero_unknown_kernel<<<grid_elems(N), kThreads, 0, st>>>(x, s->known, N);
    GFEA_LAUNCH_CHECK();
    GFEA_CUDA_TRY(cudaStreamSynchronize(st));
    res->status = GFEA_OK;
    return GFEA_OK;
  }
  double rr = hs.rr_true, rr_best = rr;
  double floor2 = (32 * eps64) * (32 * eps64) * hs.absAx;
  double tol2 = fmax(o->rtol * o->rtol * bb, floor2);
  res->rel_residual = sqrt(rr / bb);
  res->floor_rel = sqrt(floor2 / bb);
  if (rr <= tol2) { res->status = GFEA_OK; return GFEA_OK; }
  const int max_upd = o->max_refine > 0 ? o->max_refine : 200;
  T* pa = (T*)w.pa;
  T* pb = (T*)w.pb;
  // start: r (T) = r64, dx = 0, p = 0, z = D^-1 r
  cast_kernel<T><<<grid_elems(N), kThreads, 0, st>>>(w.r64, (T*)w.r, N);
  GFEA_LAUNCH_CHECK();
  GFEA_CUDA_TRY(cudaMemsetAsync(w.dx, 0, sizeof(T) * N, st));
  GFEA_CUDA_TRY(cudaMemsetAsync(pa, 0, sizeof(T) * N, st));
  e = launch_update<T>(s, w, (T*)w.dx, pa, 1, st);
  if (e) return e;
  set_trigger_kernel<<<1, 1, 0, st>>>(w.sc, fmax(delta2 * rr, 0.25 * tol2), o->max_iters);
  GFEA_LAUNCH_CHECK();
  res->status = GFEA_ERR_NOT_CONVERGED;
  int stall = 0;
  int iters0 = 0;
  for (int upd = 0;; ++upd) {
    e = pcg_loop<T>(s, G, w, (T*)w.dx, check, &hs, pa, pb, iters0, st);
    if (e) return e;
    res->iterations = hs.iters;
    const int st_inner = hs.status;
    // reliable update: x += dx (FP64), r = P(b - A x) in FP64
    add_correction_kernel<T><<<grid_elems(N), kThreads, 0, st>>>(x, (const T*)w.dx, s->known, N);
    GFEA_LAUNCH_CHECK();
    GFEA_CUDA_TRY(cudaMemsetAsync(w.dx, 0, sizeof(T) * N, st));
    e = launch_resid(s, G, b, x, w, st);
    if (e) return e;
    e = fetch(&hs, w, st);
    if (e) return e;
    rr = hs.rr_true;
    if (getenv("GFEA_DEBUG"))
      fprintf(stderr, "[gfea pcg%d] update %d: iterations %d, inner status %d, rel residual %.3e\n",
              fp64 ? 64 : 32, upd + 1, hs.iters, st_inner, sqrt(rr / bb));
    iters0 = hs.iters;
    res->refinements = upd + 1;
    floor2 = (32 * eps64) * (32 * eps64) * hs.absAx;
    tol2 = fmax(o->rtol * o->rtol * bb, floor2);
    res->rel_residual = sqrt(rr / bb);
    res->floor_rel = sqrt(floor2 / bb);
    if (!isfinite(rr)) { res->status = GFEA_ERR_NAN; break; }
    if (rr <= tol2) { res->status = GFEA_OK; break; }
    if (st_inner == GFEA_ERR_NAN || st_inner == GFEA_ERR_BREAKDOWN || st_inner == GFEA_ERR_NOT_CONVERGED) {
      res->status = st_inner;
      break;
    }
    stall = rr > 0.9 * rr_best ? stall + 1 : 0;
    if (rr < rr_best) rr_best = rr;
    if (stall >= 8 || upd + 1 >= max_upd) break;
    // continue on the replaced residual along the same direction
    cast_kernel<T><<<grid_elems(N), kThreads, 0, st>>>(w.r64, (T*)w.r, N);
    GFEA_LAUNCH_CHECK();
    e = launch_update<T>(s, w, (T*)w.dx, pa, 2, st);
    if (e) return e;
    set_trigger_kernel<<<1, 1, 0, st>>>(w.sc, fmax(delta2 * rr, 0.25 * tol2), o->max_iters);
    GFEA_LAUNCH_CHECK();
  }
  return res->status;
}

}  // namespace
}  // namespace gfea

using namespace gfea;

extern "C" int gfea_spmv(const gfea_system* s, int value_type, const void* x, void* y, void* stream) {
  if (!s || s->version != GFEA_ABI_VERSION || !x || !y || s->n_nodes <= 0) return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int G = pick_lanes(s, 0);
  const int grid = grid_nodes(s->n_nodes, G);
  if (value_type == GFEA_F64) {
    if (!s->vals64) return GFEA_ERR_ARG;
    const SysT<double> S = sys_t<double>(s);
    GFEA_DG_SWITCH(s->dof_n, G, (spmv_kernel<DD, GG, double><<<grid, kThreads, 0, st>>>(S, (const double*)x, (double*)y)));
  } else if (value_type == GFEA_F32) {
    if (!s->vals32) return GFEA_ERR_ARG;
    const SysT<float> S = sys_t<float>(s);
    GFEA_DG_SWITCH(s->dof_n, G, (spmv_kernel<DD, GG, float><<<grid, kThreads, 0, st>>>(S, (const float*)x, (float*)y)));
  } else {
    return GFEA_ERR_ARG;
  }
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" int gfea_pcg_workspace_size(const gfea_system* s, const gfea_pcg_opts* o, size_t* bytes) {
  if (!s || !o || !bytes || s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3) return GFEA_ERR_ARG;
  if (o->precision == GFEA_F64)
    *bytes = pcg_layout<double>(s->n_nodes, s->dof_n, nullptr, nullptr);
  else
    *bytes = pcg_layout<float>(s->n_nodes, s->dof_n, nullptr, nullptr);
  return GFEA_OK;
}

extern "C" int gfea_pcg_solve(const gfea_system* s, const double* b, double* x, const gfea_pcg_opts* o, void* work,
                              size_t work_bytes, gfea_pcg_result* res, void* stream) {
  if (!s || !o || !b || !x || !work || !res) return GFEA_ERR_ARG;
  if (s->version != GFEA_ABI_VERSION || o->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3 || !s->node_ptr || !s->nbr || !s->known || !s->vals64)
    return GFEA_ERR_ARG;
  if (o->max_iters < 1 || !(o->rtol > 0)) return GFEA_ERR_ARG;
  res->status = GFEA_OK;
  res->iterations = 0;
  res->refinements = 0;
  res->rel_residual = 0;
  res->floor_rel = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (o->precision == GFEA_F64) return refine_solve<double>(s, b, x, o, work, work_bytes, res, st);
  if (o->precision == GFEA_F32) {
    if (!s->vals32) return GFEA_ERR_ARG;
    return refine_solve<float>(s, b, x, o, work, work_bytes, res, st);
  }
  return GFEA_ERR_ARG;
}

extern "C" size_t gfea_reduce_workspace_size(void) { return sizeof(double) * 4 * kMaxBlocks + 256; }

extern "C" int gfea_reaction_energy(const gfea_system* s, const double* x, const int64_t* dofs, int64_t n_dofs,
                                    double* Ax, double* out_host, void* work, void* stream) {
  if (!s || !x || !Ax || !out_host || !work || s->n_nodes <= 0 || !s->vals64) return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partials = static_cast<double*>(work);
  Scal* sc = reinterpret_cast<Scal*>(partials + 4 * kMaxBlocks);
  GFEA_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(Scal), st));
  const int G = pick_lanes(s, 0);
  const SysT<double> S = sys_t<double>(s);
  const int grid = grid_nodes(s->n_nodes, G);
  GFEA_DG_SWITCH(s->dof_n, G, (reaction_kernel<DD, GG><<<grid, kThreads, 0, st>>>(S, x, Ax, partials, sc)));
  GFEA_LAUNCH_CHECK();
  if (n_dofs > 0 && dofs) {
    gather_sum_kernel<<<grid_elems(n_dofs), kThreads, 0, st>>>(Ax, dofs, n_dofs, partials + 2 * kMaxBlocks, sc);
    GFEA_LAUNCH_CHECK();
  }
  Scal hs;
  GFEA_CUDA_TRY(cudaMemcpyAsync(&hs, sc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
  GFEA_CUDA_TRY(cudaStreamSynchronize(st));
  out_host[0] = (n_dofs > 0 && dofs) ? hs.pap : 0.0;
  out_host[1] = hs.rr_true;
  return GFEA_OK;
}

extern "C" int gfea_max_abs_diff(const double* a, const double* b, int64_t n, double* out_host, void* work,
                                 void* stream) {
  if (!a || !b || !out_host || !work || n < 0) return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto* o = static_cast<unsigned long long*>(work);
  GFEA_CUDA_TRY(cudaMemsetAsync(o, 0, sizeof(unsigned long long), st));
  if (n > 0) {
    max_abs_diff_kernel<<<grid_elems(n), kThreads, 0, st>>>(a, b, n, o);
    GFEA_LAUNCH_CHECK();
  }
  unsigned long long h = 0;
  GFEA_CUDA_TRY(cudaMemcpyAsync(&h, o, sizeof(h), cudaMemcpyDeviceToHost, st));
  GFEA_CUDA_TRY(cudaStreamSynchronize(st));
  double v;
  memcpy(&v, &h, sizeof(v));
  *out_host = v;
  return GFEA_OK;
}

extern "C" int gfea_cast_f64_f32(const double* src, float* dst, int64_t n, void* stream) {
  if (!src || !dst || n < 0) return GFEA_ERR_ARG;
  if (n == 0) return GFEA_OK;
  cast_kernel<float><<<grid_elems(n), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(src, dst, n);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" long long gfea_launch_count(void) { return gfea::launch_counter().load(); }

extern "C" int gfea_profile_enable(int on) {
  gfea::KernelProfile& P = gfea::prof();
  if (on && !P.created) {
    for (int i = 0; i < 2 * gfea::KernelProfile::kPairs; ++i) GFEA_CUDA_TRY(cudaEventCreate(&P.ev[i]));
    P.created = true;
  }
  P.on = on != 0;
  return GFEA_OK;
}

extern "C" int gfea_profile_read(double* ms_host, long long* launches_host) {
  if (!ms_host || !launches_host) return GFEA_ERR_ARG;
  gfea::KernelProfile& P = gfea::prof();
  *ms_host = P.ms;
  *launches_host = P.n;
  P.ms = 0;
  P.n = 0;
  return GFEA_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free PCG.
//
// For callers that cannot allocate device memory themselves: a solver embedded
// in a host application whose device memory is owned by another allocator or
// pre-reserved pool, or a latency-critical loop where allocation (and the
// synchronisation it can imply) is not allowed.  The scratch of the solve
// lives in the file-scope array below, which every GPU that loads this library
// holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace gfea {
namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of g_static_scratch on the current device (looked up once per
// device; the array's name in host code is only a host-side stand-in).
int static_scratch(void** out) {
  int dev = 0;
  GFEA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return GFEA_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    GFEA_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GFEA_OK;
}

}  // namespace
}  // namespace gfea

extern "C" int gfea_pcg_solve_noalloc(const gfea_system* s, const double* b, double* x, const gfea_pcg_opts* o,
                                      gfea_pcg_result* res, void* stream) {
  if (!s || !o || !b || !x || !res) return GFEA_ERR_ARG;
  if (s->version != GFEA_ABI_VERSION || o->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3 || !s->node_ptr || !s->nbr || !s->known || !s->vals64)
    return GFEA_ERR_ARG;
  if (o->max_iters < 1 || !(o->rtol > 0)) return GFEA_ERR_ARG;
  if (o->precision != GFEA_F64 && (o->precision != GFEA_F32 || !s->vals32)) return GFEA_ERR_ARG;
  // reject problems whose scratch exceeds the static array, before any device work
  const size_t need = o->precision == GFEA_F64 ? pcg_layout<double>(s->n_nodes, s->dof_n, nullptr, nullptr)
                                               : pcg_layout<float>(s->n_nodes, s->dof_n, nullptr, nullptr);
  if (need > kStaticScratchBytes) return GFEA_ERR_WORKSPACE;
  void* scratch = nullptr;
  const int e = static_scratch(&scratch);
  if (e) return e;
  res->status = GFEA_OK;
  res->iterations = 0;
  res->refinements = 0;
  res->rel_residual = 0;
  res->floor_rel = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (o->precision == GFEA_F64) return refine_solve<double>(s, b, x, o, scratch, kStaticScratchBytes, res, st);
  return refine_solve<float>(s, b, x, o, scratch, kStaticScratchBytes, res, st);
}

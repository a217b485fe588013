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
// One PCG iteration is three kernels (block-Jacobi) or five (two-level):
//   dir      : p' = z + beta p
//   apply    : Ap' (masked SpMV), p'.Ap', alpha
//   update   : x += alpha p', r -= alpha Ap', z = D^-1 r, r.z, r.r, beta
// with the coarse level, update is split into update_r (x, r, restriction),
// coarse_gemv and finish_z (z = D^-1 r + prolonged correction, dots, beta).
// Reductions are per-block partials summed in a fixed order by the last block
// to finish (atomic ticket, no spinning), which also derives the scalar
// recurrences (alpha, beta, convergence) on the device.  Kernels return early
// once the device flag 'done' is set, so a host loop (or a captured graph) may
// run more iterations than needed at no cost.

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <mutex>
#include <vector>

#include "coarse.cuh"
#include "common.cuh"
#include "rowops.cuh"
#include "stage.cuh"
#include "tune.cuh"

namespace gfea {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = kSMs * 8;

struct Scal {
  double rz, rr, pap, alpha, beta, bb, tol2, rr_true, absAx;
  int32_t done, iters, status, max_iters;
  uint32_t ticket1, ticket2, ticket3, pad;
};

// Optional CUDA-event timing of the launches of the PCG iterations, per
// kernel kind; gfea_profile_read returns the SpMV kernel's (the dominant
// launch of a solve).  Events are recorded after each launch of a chunk of
// iterations and attributed once the chunk's performed iterations are known.
enum ProfTag { kTagDir, kTagApply, kTagUpdate, kTagRestrict, kTagGemv, kTagFinish, kNumTags };
const char* const kTagNames[kNumTags] = {"direction", "spmv", "update", "update+restrict", "coarse gemv",
                                         "finish z"};

// Solves may run concurrently from several host threads (one stream each):
// the events of a chunk are per thread, the totals are shared under a mutex.
struct KernelProfile {
  std::atomic<bool> on{false};
  std::mutex mu;
  double ms[kNumTags] = {};
  long long n[kNumTags] = {};
};
KernelProfile& prof() {
  static KernelProfile p;
  return p;
}

struct ChunkEvents {
  static constexpr int kEvents = 512;
  bool created = false;
  bool active = false;  // inside a timed chunk
  cudaEvent_t ev[kEvents];
  int tag[kEvents];
  int cur = 0;
};
ChunkEvents& chunk_events() {
  thread_local ChunkEvents c;
  return c;
}

// Event after a launch of kind 'tag' (tag < 0: iteration start).
int prof_mark(cudaStream_t st, int tag) {
  ChunkEvents& E = chunk_events();
  if (!E.active || E.cur >= ChunkEvents::kEvents) return GFEA_OK;
  GFEA_CUDA_TRY(cudaEventRecord(E.ev[E.cur], st));
  E.tag[E.cur++] = tag;
  return GFEA_OK;
}



// The last block to finish (atomic ticket, no waiting) sums the NV block
// partials in a fixed order; out[] holds the totals in every thread of it.
template <int NV>
__device__ bool reduce_last_tail(double* partials, uint32_t* ticket, double (&out)[NV], double* sh, bool& last) {
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
  return reduce_last_tail<NV>(partials, ticket, out, sh, last);
}

// reduce_last for dot accumulators: warp sums by warp_sum_acc (FP32 pairs
// stay in FP32), then the warps' doubles in a fixed order.
template <int NV, typename T>
__device__ bool reduce_last_acc(const DotAcc<T> (&acc)[NV], double* partials, uint32_t* ticket, double (&out)[NV]) {
  __shared__ double sh[32];
  __shared__ double shw[NV][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double v = warp_sum_acc(acc[k]);
    if (lane == 0) shw[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += shw[k][i];
      partials[k * gridDim.x + blockIdx.x] = t;
    }
    __threadfence();
    const uint32_t t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  return reduce_last_tail<NV>(partials, ticket, out, sh, last);
}

// ---------------------------------------------------------------------------
// node-row products
// ---------------------------------------------------------------------------


// y = A x (unmasked); DIFF: the difference form of the PCG's FP32 products
// (used to time the same loads and arithmetic when tuning)
template <int D, int G, typename T, bool DIFF = false>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 8 : 6) spmv_kernel(SysT<T> S, const T* __restrict__ x,
                                                                             T* __restrict__ y) {
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    const T v = node_rows_t<D, G, T, T, false, DIFF>(ac, lane, S, [x](int64_t c) { return __ldg(x + c); });
    int r = -1;
#pragma unroll
    for (int i = 0; i < D; ++i) if (lane == row_lane<D, G>(i)) r = i;
    if (a < Nn && r >= 0) y[a * D + r] = v;
  }
}

// FP64 residual of the reduced system: r = P (b - A x); partials r.r,
// ||P (b - A x_c)||^2 (x_c: x on known columns only, the reference norm) and
// ||P |A| |x|||^2 (scale of the rounding floor of r).
// The three products share one pass over the values; KN = false skips the
// known-column product (b - A x_c does not change between reliable updates).
// AB32: the |A||x| product (only a floor estimate, 1e-6 accuracy is plenty)
// from the FP32 values and an FP32 copy of x, on the FP32 pipe; the residual
// itself stays FP64.
template <int D, int G, typename T, bool KN, bool AB32>
__global__ void __launch_bounds__(kThreads) resid_kernel(SysT<T> S, const float* __restrict__ v32,
                                                         const float* __restrict__ x32,
                                                         const double* __restrict__ b,
                                                         const double* __restrict__ x, double* __restrict__ r,
                                                         double* partials, Scal* sc) {
  constexpr int LA = G - G % D;
  constexpr int NPP = LA / D;
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  const int j = lane % D;
  double v[3] = {0, 0, 0};
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    double all[D], kn[D], ab[D];
    float ab32[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      all[i] = kn[i] = ab[i] = 0;
      ab32[i] = 0.f;
    }
    if (lane < LA) {
      const int32_t p0 = S.node_ptr[ac], nb = S.node_ptr[ac + 1] - p0;
      const int32_t W = D * nb;
      const T* base = S.vals + (int64_t)D * D * p0;
      const float* base32 = AB32 ? v32 + (int64_t)D * D * p0 : nullptr;
      for (int32_t k = lane / D, t = lane; k < nb; k += NPP, t += LA) {
        const int64_t col = (int64_t)__ldg(S.nbr + p0 + k) * D + j;
        const double xv = __ldg(x + col);
        const double xk = (KN && S.known[col]) ? xv : 0.0;
        const float xa32 = AB32 ? fabsf(__ldg(x32 + col)) : 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) {
          const double w = (double)__ldg(base + (int64_t)i * W + t);
          all[i] += w * xv;
          if (KN) kn[i] += w * xk;
          if (AB32)
            ab32[i] += fabsf(__ldg(base32 + (int64_t)i * W + t)) * xa32;
          else
            ab[i] += fabs(w) * fabs(xv);
        }
      }
    }
    // row i's three sums land in lane row_lane(i)
    const double s_all = group_sum_rows<D, G, double>(all, lane);
    const double s_kn = KN ? group_sum_rows<D, G, double>(kn, lane) : 0.0;
    const double s_ab = AB32 ? (double)group_sum_rows<D, G, float>(ab32, lane) : group_sum_rows<D, G, double>(ab, lane);
    int ri_row = -1;
#pragma unroll
    for (int i = 0; i < D; ++i) if (lane == row_lane<D, G>(i)) ri_row = i;
    if (a < Nn && ri_row >= 0) {
      const int64_t dof = a * D + ri_row;
      const bool unk = !S.known[dof];
      const double ri = unk ? b[dof] - s_all : 0.0;
      const double rci = unk ? b[dof] - s_kn : 0.0;
      const double ai = unk ? s_ab + fabs(b[dof]) : 0.0;
      r[dof] = ri;
      v[0] += ri * ri;
      v[1] += rci * rci;
      v[2] += ai * ai;
    }
  }
  double out[3];
  if (reduce_last<3>(v, partials, &sc->ticket3, out) && threadIdx.x == 0) {
    sc->rr_true = out[0];
    if (KN) sc->bb = out[1];
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
  DotAcc<T> rz, rr;
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
      rz.add_prod(rl[i], zi);
      rr.add_prod(rl[i], rl[i]);
    }
  }
  const DotAcc<T> v[2] = {rz, rr};
  double out[2];
  if (reduce_last_acc<2, T>(v, partials, &sc->ticket2, out) && threadIdx.x == 0) {
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

// ---------------------------------------------------------------------------
// Two-level preconditioner: M^-1 r = D^-1 r + P A_c^-1 P^T r.  P maps each
// aggregate (a cell of a regular grid over the bounding box) to the rigid-body
// modes of its nodes -- translations and rotations about the cell centre
// (constants for a scalar field) -- with known DOFs masked out; A_c = P^T A P
// is assembled from the CSR values of the iteration's precision (sums in
// FP64) and inverted densely (FP64 Gauss-Jordan) once per solve.  Per iteration: restriction fused into the
// residual update, one dense coarse GEMV, prolongation fused into z.
// ---------------------------------------------------------------------------

constexpr int kCoarseMax = 1536;  // largest coarse dimension nr * n_agg

// Aggregation kept at the start of the coarse workspace, so that a later
// solve on the same mesh can reuse it.
struct CoarseHdr {
  int32_t n_agg, nc, nr, valid;
  int64_t Nn;
};

// The restriction's FP64 atomics go to kRcCopies copies of the coarse vector
// (block b adds into copy b % kRcCopies): one copy held them all on a few L2
// slices, where they serialised.  Below kRcCopyMinNodes nodes the atomics
// are few and an iteration is launch-latency bound: one copy (rc itself,
// cleared by finish_z) and no summing launch.
constexpr int kRcCopies = 16;
constexpr int64_t kRcCopyMinNodes = 100000;

struct CoarseDev {
  int nr = 0, n_agg = 0, nc = 0;
  int ncopies = 1;         // 1: restriction into rc; kRcCopies: into rcp, summed by rc_sum_kernel
  CoarseHdr* hdr = nullptr;
  int32_t* agg = nullptr;  // node -> aggregate
  float4* off = nullptr;   // node offset from its cell centre / largest cell size
  double* Ac = nullptr;    // nc x nc, inverted in place
  // working storage of the inversion: float-float pairs (hi, lo)
  float* Ahi = nullptr;    // nc x nc
  float* Alo = nullptr;
  float* rowph = nullptr;  // kGJB x nc: row panel of the pivot block
  float* rowpl = nullptr;
  float* colph = nullptr;  // nc x kGJB: column panel of the pivot block
  float* colpl = nullptr;
  float* pinvh = nullptr;  // kGJB x kGJB: inverse of the pivot block
  float* pinvl = nullptr;
  double* rc = nullptr;    // nc: restriction R^T r (summed from the copies)
  double* rcp = nullptr;   // kRcCopies x nc: restriction accumulators, one per group of blocks
  double* ec = nullptr;    // nc: coarse correction
  float* ecf = nullptr;    // nc: its FP32 copy (read by the FP32 prolongation)
};

__global__ void bbox_kernel(const double* __restrict__ coord, int64_t Nn, double* partials) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      lo[k] = fmin(lo[k], coord[a * 3 + k]);
      hi[k] = fmax(hi[k], coord[a * 3 + k]);
    }
  __shared__ double s[6][kThreads];
  for (int k = 0; k < 3; ++k) {
    s[k][threadIdx.x] = lo[k];
    s[3 + k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; ++k) {
        s[k][threadIdx.x] = fmin(s[k][threadIdx.x], s[k][threadIdx.x + o]);
        s[3 + k][threadIdx.x] = fmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + o]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) partials[blockIdx.x * 6 + k] = s[k][0];
}

// Cell of each node (the longest extent varies slowest, which keeps the
// coarse matrix banded) and its offset from the cell centre, scaled by hinv.
__global__ void aggregate_kernel(const double* __restrict__ coord, int64_t Nn, double3 lo, double3 h, int3 cells,
                                 int3 order, double hinv, int32_t* agg, float4* off) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x) {
    const double x = coord[a * 3], y = coord[a * 3 + 1], z = coord[a * 3 + 2];
    int ix = (int)floor((x - lo.x) / h.x), iy = (int)floor((y - lo.y) / h.y), iz = (int)floor((z - lo.z) / h.z);
    ix = ix < 0 ? 0 : (ix >= cells.x ? cells.x - 1 : ix);
    iy = iy < 0 ? 0 : (iy >= cells.y ? cells.y - 1 : iy);
    iz = iz < 0 ? 0 : (iz >= cells.z ? cells.z - 1 : iz);
    const int idx[3] = {ix, iy, iz}, n[3] = {cells.x, cells.y, cells.z};
    // order.x varies fastest, order.z slowest
    agg[a] = idx[order.x] + n[order.x] * (idx[order.y] + n[order.y] * idx[order.z]);
    off[a] = make_float4((float)((x - (lo.x + (ix + 0.5) * h.x)) * hinv),
                         (float)((y - (lo.y + (iy + 0.5) * h.y)) * hinv),
                         (float)((z - (lo.z + (iz + 0.5) * h.z)) * hinv), 0.f);
  }
}

// A_c += R_a^T K_ab R_b, summed per node over neighbours sharing an aggregate
// (T: the iteration's value type -- the FP32 operator of the mixed path gives
// a coarse matrix accurate to ~1e-6, plenty for a preconditioner, on the FP32
// pipe; sums go to A_c in FP64).
template <int D, typename T>
__device__ __forceinline__ void coarse_assemble_body(const SysT<T>& S, const CoarseDev& C, int64_t bx, int64_t gx) {
  constexpr int nr = Modes<D>::nr;
  constexpr int kSlots = 8;
  for (int64_t a = bx * (int64_t)blockDim.x + threadIdx.x; a < S.Nn; a += gx * blockDim.x) {
    const int ga = C.agg[a];
    T Ra[D][nr];
    node_modes<D, T>(C.off[a], S.known + a * D, Ra);
    int sid[kSlots];
    T acc[kSlots][nr][nr];
    int ns = 0;
    const int32_t p0 = S.node_ptr[a], nb = S.node_ptr[a + 1] - p0;
    const int32_t W = D * nb;
    for (int k = 0; k < nb; ++k) {
      const int32_t b = S.nbr[p0 + k];
      const int gb = C.agg[b];
      T Rb[D][nr];
      node_modes<D, T>(C.off[b], S.known + (int64_t)b * D, Rb);
      // K_ab R_b (D x nr)
      T KR[D][nr];
      for (int i = 0; i < D; ++i)
        for (int m = 0; m < nr; ++m) {
          T v = 0;
          for (int j = 0; j < D; ++j) v += S.vals[(int64_t)D * D * p0 + (int64_t)i * W + D * k + j] * Rb[j][m];
          KR[i][m] = v;
        }
      int slot = -1;
      for (int q = 0; q < ns; ++q)
        if (sid[q] == gb) slot = q;
      if (slot < 0) {
        if (ns == kSlots) {  // flush (rare: more distinct neighbour aggregates than slots)
          for (int q = 0; q < ns; ++q)
            for (int m = 0; m < nr; ++m)
              for (int l = 0; l < nr; ++l)
                atomicAdd(&C.Ac[(int64_t)(ga * nr + m) * C.nc + sid[q] * nr + l], (double)acc[q][m][l]);
          ns = 0;
        }
        slot = ns++;
        sid[slot] = gb;
        for (int m = 0; m < nr; ++m)
          for (int l = 0; l < nr; ++l) acc[slot][m][l] = 0;
      }
      for (int m = 0; m < nr; ++m)
        for (int l = 0; l < nr; ++l) {
          T v = 0;
          for (int i = 0; i < D; ++i) v += Ra[i][m] * KR[i][l];
          acc[slot][m][l] += v;
        }
    }
    for (int q = 0; q < ns; ++q)
      for (int m = 0; m < nr; ++m)
        for (int l = 0; l < nr; ++l)
          atomicAdd(&C.Ac[(int64_t)(ga * nr + m) * C.nc + sid[q] * nr + l], (double)acc[q][m][l]);
  }
}

template <int D, typename T>
__global__ void coarse_assemble_kernel(SysT<T> S, CoarseDev C) {
  coarse_assemble_body<D, T>(S, C, blockIdx.x, gridDim.x);
}

// Unit diagonal for empty or fully constrained coarse DOFs, a 1e-10 relative
// shift elsewhere (rotation modes of degenerate aggregates), identity in inv.
// (zero_tol, shift): (1e-14, 1e-10) for a coarse matrix built in FP64,
// (1e-6, 1e-6) for one built from FP32 values, whose rounding can reach the
// 1e-6 level in nearly degenerate modes.
__device__ __forceinline__ void coarse_regularize_body(const CoarseDev& C, double zero_tol, double shift) {
  __shared__ double smax[256];
  double m = 0;
  for (int i = threadIdx.x; i < C.nc; i += blockDim.x) m = fmax(m, fabs(C.Ac[(int64_t)i * C.nc + i]));
  smax[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
    __syncthreads();
  }
  const double dmax = smax[0] > 0 ? smax[0] : 1.0;
  for (int i = threadIdx.x; i < C.nc; i += blockDim.x) {
    double& d = C.Ac[(int64_t)i * C.nc + i];
    d = d > zero_tol * dmax ? d + shift * dmax : dmax;
  }
}

__global__ void coarse_regularize_kernel(CoarseDev C, double zero_tol, double shift) {
  coarse_regularize_body(C, zero_tol, shift);
}

// In-place blocked Gauss-Jordan inversion of the SPD coarse matrix (no
// pivoting: every pivot block of an SPD matrix is SPD).  For the pivot block
// K = [k0, k0 + b) of A = [[A11, A12], [A21, A22]]:
//   A11 <- A11^-1,  A12 <- A11^-1 A12,  A21 <- -A21 A11^-1,
//   A22 <- A22 - A21 A11^-1 A12,
// two launches per block: gj_panel saves the row panel A11^-1 A1* (rowp),
// the old column panel A*1 (colp) and A11^-1 (pinv); gj_update applies the
// rank-b update to every element (each read and written by one thread).
constexpr int kGJB = 16;

// Float-float arithmetic of the inversion's trailing updates: a value is an
// unevaluated pair hi + lo of floats (~2^-44 relative), products by the exact
// FMA split, sums by TwoSum (Knuth); GB300 runs FP32 at 64x its FP64 rate, so
// the n^3 update FMAs cost less than in FP64 even at ~12 FP32 operations each.
__device__ __forceinline__ void ff_split(double d, float& hi, float& lo) {
  hi = (float)d;
  lo = (float)(d - (double)hi);
}

// (sh, sl) += (ah, al) (bh, bl); the al bl term is below the pair's precision
__device__ __forceinline__ void ff_fma_acc(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  const float e = fmaf(ah, bh, -p) + fmaf(ah, bl, al * bh);
  const float t = sh + p;
  const float bp = t - sh;
  sl += ((sh - (t - bp)) + (p - bp)) + e;
  sh = t;
}

// (ah, al) - (sh, sl), normalised
__device__ __forceinline__ void ff_sub(float ah, float al, float sh, float sl, float& hi, float& lo) {
  const float t = ah - sh;
  const float bp = t - ah;
  const float err = (ah - (t - bp)) + (-sh - bp);
  const float l = err + (al - sl);
  hi = t + l;
  lo = l - (hi - t);
}

__global__ void ff_split_kernel(const double* __restrict__ a, float* __restrict__ hi, float* __restrict__ lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    ff_split(a[i], hi[i], lo[i]);
}

__global__ void ff_merge_kernel(double* __restrict__ a, const float* __restrict__ hi, const float* __restrict__ lo,
                                int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (double)hi[i] + (double)lo[i];
}

// block (bx, l): row l of the transformed row panel for columns bx * 128 ..;
// every block inverts the b x b pivot block itself (b steps in shared
// memory, FP64), so the panel's work spreads over n / 128 x b blocks
__device__ __forceinline__ void gj_panel_body(const CoarseDev& C, int k0, int b, int bx, int l) {
  const int n = C.nc;
  __shared__ double M[kGJB][kGJB + 1], M2[kGJB][kGJB + 1];
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
    const int64_t q = (int64_t)(k0 + t / b) * n + k0 + t % b;
    M[t / b][t % b] = (double)C.Ahi[q] + (double)C.Alo[q];
  }
  __syncthreads();
  for (int p = 0; p < b; ++p) {  // Gauss-Jordan of the pivot block in shared memory
    const double ip = 1.0 / M[p][p];
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
      const int i = t / b, j = t % b;
      M2[i][j] = i == p ? (j == p ? ip : M[p][j] * ip) : (j == p ? -M[i][p] * ip : M[i][j] - M[i][p] * (M[p][j] * ip));
    }
    __syncthreads();
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) M[t / b][t % b] = M2[t / b][t % b];
    __syncthreads();
  }
  if (bx == 0 && l == 0)
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) ff_split(M[t / b][t % b], C.pinvh[t], C.pinvl[t]);
  const int j = bx * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double s = 0;
#pragma unroll
  for (int m = 0; m < kGJB; ++m)
    if (m < b) {
      const int64_t q = (int64_t)(k0 + m) * n + j;
      s += M[l][m] * ((double)C.Ahi[q] + (double)C.Alo[q]);
    }
  ff_split(s, C.rowph[(int64_t)l * n + j], C.rowpl[(int64_t)l * n + j]);
  if (l == 0) {
#pragma unroll
    for (int q = 0; q < kGJB; ++q) {
      const int64_t src = (int64_t)j * n + k0 + q;
      C.colph[(int64_t)j * kGJB + q] = q < b ? C.Ahi[src] : 0.f;
      C.colpl[(int64_t)j * kGJB + q] = q < b ? C.Alo[src] : 0.f;
    }
  }
}

__global__ void __launch_bounds__(128) gj_panel_kernel(CoarseDev C, int k0, int b) {
  gj_panel_body(C, k0, b, blockIdx.x, blockIdx.y);
}

// Block (bx, by) owns column j = bx * blockDim + tid and rows by, by + gridDim.y, ...
__device__ __forceinline__ void gj_update_body(const CoarseDev& C, int k0, int b, int bx, int by, int gy) {
  const int n = C.nc;
  const int j = bx * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const bool jk = j >= k0 && j < k0 + b;
  float rh[kGJB], rl[kGJB];
#pragma unroll
  for (int l = 0; l < kGJB; ++l) {
    const int64_t q = jk ? (int64_t)l * b + (j - k0) : (int64_t)l * n + j;
    rh[l] = l < b ? (jk ? C.pinvh[q] : C.rowph[q]) : 0.f;
    rl[l] = l < b ? (jk ? C.pinvl[q] : C.rowpl[q]) : 0.f;
  }
  for (int i = by; i < n; i += gy) {
    const int64_t q = (int64_t)i * n + j;
    float vh, vl;
    if (i >= k0 && i < k0 + b) {
      const int64_t r = jk ? (int64_t)(i - k0) * b + (j - k0) : (int64_t)(i - k0) * n + j;
      vh = jk ? C.pinvh[r] : C.rowph[r];
      vl = jk ? C.pinvl[r] : C.rowpl[r];
    } else {
      const float* ch = C.colph + (int64_t)i * kGJB;
      const float* cl = C.colpl + (int64_t)i * kGJB;
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int l = 0; l < kGJB; ++l) ff_fma_acc(sh, sl, __ldg(ch + l), __ldg(cl + l), rh[l], rl[l]);
      ff_sub(jk ? 0.f : C.Ahi[q], jk ? 0.f : C.Alo[q], sh, sl, vh, vl);
    }
    C.Ahi[q] = vh;
    C.Alo[q] = vl;
  }
}

__global__ void __launch_bounds__(128) gj_update_kernel(CoarseDev C, int k0, int b) {
  gj_update_body(C, k0, b, blockIdx.x, blockIdx.y, gridDim.y);
}

template <int nr, typename T>
__device__ __forceinline__ void restrict_add(double* rc, int g, T (&v)[nr]) {
  const int lane = threadIdx.x & 31;
  const int gp = __shfl_up_sync(0xffffffffu, g, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || g != gp);
  const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));  // first lane of this lane's run
  const int gn = __shfl_down_sync(0xffffffffu, g, 1);
  const bool tail = lane == 31 || gn != g;
#pragma unroll
  for (int m = 0; m < nr; ++m) {
    T s = v[m];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const T t = __shfl_up_sync(0xffffffffu, s, d);
      if (lane - d >= start) s += t;
    }
    if (tail && g >= 0 && s != 0) atomicAdd(&rc[g * nr + m], (double)s);
  }
}

// x, r update (mode 0) and restriction rc += R_a^T r_a.  The node loop runs
// whole warps (stride a multiple of 32) for the warp-level pre-reduction.
template <int D, typename T>
__global__ void __launch_bounds__(kThreads) update_r_kernel(int64_t Nn, const uint8_t* __restrict__ known,
                                                            T* __restrict__ x,
                                                            T* __restrict__ r, const T* __restrict__ p,
                                                            const T* __restrict__ Ap, Scal* sc, CoarseDev C,
                                                            int mode) {
  if (mode == 0 && sc->done) return;
  constexpr int nr = Modes<D>::nr;
  const double alpha = mode == 0 ? sc->alpha : 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a - (threadIdx.x & 31) < Nn; a += stride) {
    T v[nr];
#pragma unroll
    for (int m = 0; m < nr; ++m) v[m] = 0;
    int g = -1;
    if (a < Nn) {
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
      g = C.agg[a];
      T R[D][nr];
      node_modes<D, T>(C.off[a], known + a * D, R);
#pragma unroll
      for (int m = 0; m < nr; ++m)
#pragma unroll
        for (int i = 0; i < D; ++i) v[m] += R[i][m] * rl[i];
    }
    restrict_add<nr, T>(C.ncopies > 1 ? C.rcp + (int64_t)(blockIdx.x % kRcCopies) * C.nc : C.rc, g, v);
  }
}

// rc = sum of the restriction copies, which are cleared for the next
// iteration (fixed summation order).
__global__ void __launch_bounds__(kThreads) rc_sum_kernel(CoarseDev C, const Scal* sc, int mode) {
  if (mode == 0 && sc->done) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < C.nc; j += gridDim.x * blockDim.x) {
    double t = 0;
#pragma unroll
    for (int k = 0; k < kRcCopies; ++k) {
      double* q = C.rcp + (int64_t)k * C.nc + j;
      t += *q;
      *q = 0;
    }
    C.rc[j] = t;
  }
}

// ec = A_c^-1 rc: one block of kGemvThreads per coarse row (enough warps in
// flight to stream the L2-resident inverse), fixed-order block reduction.
constexpr int kGemvThreads = 128;

__global__ void __launch_bounds__(kGemvThreads) coarse_gemv_kernel(CoarseDev C, const Scal* sc, int mode) {
  if (mode == 0 && sc->done) return;
  __shared__ double sh[kGemvThreads / 32];
  for (int i = blockIdx.x; i < C.nc; i += gridDim.x) {
    const double* row = C.Ac + (int64_t)i * C.nc;
    double v = 0;
    for (int j = threadIdx.x; j < C.nc; j += kGemvThreads) v += row[j] * C.rc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
#pragma unroll
      for (int w = 0; w < kGemvThreads / 32; ++w) t += sh[w];
      C.ec[i] = t;
      C.ecf[i] = (float)t;
    }
    __syncthreads();
  }
}

// z = D^-1 r + R_a ec (masked), partial r.z and r.r, rc reset; the last block
// derives beta and the convergence state exactly as update_kernel does.
template <int D, typename T>
__global__ void __launch_bounds__(kThreads) finish_z_kernel(int64_t Nn, const uint8_t* __restrict__ known,
                                                            const T* __restrict__ dinv, const T* __restrict__ r,
                                                            T* __restrict__ z, double* partials, Scal* sc,
                                                            CoarseDev C, int mode) {
  if (mode == 0 && sc->done) return;
  constexpr int nr = Modes<D>::nr;
  DotAcc<T> rz, rr;
  const T* ec = sizeof(T) == 4 ? (const T*)C.ecf : (const T*)C.ec;
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x) {
    T rl[D];
#pragma unroll
    for (int i = 0; i < D; ++i) rl[i] = r[a * D + i];
    const int g = C.agg[a];
    T R[D][nr];
    node_modes<D, T>(C.off[a], known + a * D, R);
    T e[nr];
#pragma unroll
    for (int m = 0; m < nr; ++m) e[m] = ec[g * nr + m];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      T zi = 0;
#pragma unroll
      for (int j = 0; j < D; ++j) zi += dinv[a * D * D + i * D + j] * rl[j];
#pragma unroll
      for (int m = 0; m < nr; ++m) zi += R[i][m] * e[m];
      if (known[a * D + i]) zi = 0;
      z[a * D + i] = zi;
      rz.add_prod(rl[i], zi);
      rr.add_prod(rl[i], rl[i]);
    }
  }
  if (C.ncopies == 1)  // single copy: clear rc (read by this iteration's GEMV) for the next restriction
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C.nc; i += gridDim.x * blockDim.x) C.rc[i] = 0;
  const DotAcc<T> v[2] = {rz, rr};
  double out[2];
  if (reduce_last_acc<2, T>(v, partials, &sc->ticket2, out) && threadIdx.x == 0) {
    const double rz_new = out[0], rr = out[1];
    sc->beta = mode == 1 ? 0.0 : rz_new / sc->rz;
    if (mode == 2 && !(sc->beta <= 1.0)) sc->beta = 0.0;
    sc->rz = rz_new;
    sc->rr = rr;
    if (mode != 0) return;
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

// p' = z + beta p (streaming; p' vanishes on known DOFs with z and p).
template <typename T>
__global__ void __launch_bounds__(kThreads) dir_kernel(int64_t n, const T* __restrict__ z,
                                                       const T* __restrict__ p_old, T* __restrict__ p_new,
                                                       const Scal* sc) {
  if (sc->done) return;
  const T beta = (T)sc->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p_new[i] = z[i] + beta * p_old[i];
}

// Ap = masked A p; partial p.Ap; the last block sets alpha.  DIR: the
// search direction is formed on the fly, p = z + beta p_old (beta from the
// scalar record), read for every neighbour from z and p_old and written for
// the block's own rows into p_new -- the direction update of dir_kernel
// fused into the SpMV ('p' is then p_old).
template <int D, int G, typename T, bool DIFF, bool DIR = false>
__global__ void __launch_bounds__(kThreads, (sizeof(T) == 4 && D > 1) ? 8 : 6) apply_kernel(SysT<T> S, const T* __restrict__ p,
                                                                              T* __restrict__ Ap,
                                                         double* partials, Scal* sc,
                                                         const T* __restrict__ z = nullptr,
                                                         T* __restrict__ p_new = nullptr) {
  if (sc->done) return;
  const T beta = DIR ? (T)sc->beta : (T)0;
  const int lane = threadIdx.x % G;
  const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t Nn = S.Nn;
  DotAcc<T> pap;
  for (int64_t a0 = grp - (grp % (32 / G)); a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + (grp % (32 / G));
    const int64_t ac = a < Nn ? a : Nn - 1;
    auto pv = [p, z, beta](int64_t c) { return DIR ? __ldg(z + c) + beta * __ldg(p + c) : __ldg(p + c); };
    T av = node_rows_t<D, G, T, T, false, DIFF>(ac, lane, S, pv);
    int r = -1;
#pragma unroll
    for (int i = 0; i < D; ++i) if (lane == row_lane<D, G>(i)) r = i;
    if (a < Nn && r >= 0) {
      const int64_t dof = a * D + r;
      const T pn = DIR ? pv(dof) : p[dof];  // the value the neighbours' rows used
      if (DIR) p_new[dof] = pn;
      if (S.known[dof]) av = 0;
      Ap[dof] = av;
      pap.add_prod(pn, av);
    }
  }
  const DotAcc<T> v[1] = {pap};
  double out[1];
  if (reduce_last_acc<1, T>(v, partials, &sc->ticket1, out) && threadIdx.x == 0) {
    sc->pap = out[0];
    if (!(out[0] > 0) || !isfinite(out[0])) {
      sc->status = isfinite(out[0]) ? GFEA_ERR_BREAKDOWN : GFEA_ERR_NAN;
      sc->done = 1;
    } else {
      sc->alpha = sc->rz / out[0];
    }
  }
}

// apply_kernel with the operator streamed through shared memory.  Nodes are
// cut into tiles of nt = 32 / D consecutive nodes (one node component per
// lane of a warp).  Once per solve, pack_tiles_kernel lays each tile out as
// one contiguous block of the workspace,
//   [node offsets (nt + 1, relative) | neighbour indices | CSR values],
// so that a producer warp moves a whole tile by ONE bulk asynchronous copy
// (cp.async.bulk, completing on the stage's 'full' mbarrier) into a ring of
// shared-memory stages: the copy engine has a fixed cost per copy that made
// separate copies of the three short ranges the bound.  Each block takes a
// contiguous range of tiles (consecutive tiles share neighbourhoods, so their
// gathers of p hit the SM's L1); tile i of a block goes to consumer warp
// i % 8, which owns stage i % stages alone (stages is a multiple of 8).  A
// lane owns one component j of one node: it gathers p at component j of each
// neighbour once and accumulates its share of all D rows; the D lanes of the
// node then exchange partial rows (D - 1 shuffles).  A tile with more
// neighbour slots than a stage holds is not packed and is read from global
// memory by the same lanes.  Every wait is bounded (2 s): on expiry the
// kernel sets GFEA_ERR_TIMEOUT, waits (bounded) for its copies in flight and
// returns.
struct StageGeom {
  int64_t ntiles;
  int32_t nt;          // nodes per tile
  int32_t cap_slots;   // neighbour slots a packed tile holds
  int32_t stages;      // ring depth (a multiple of the consumer warps, <= kMaxStages)
  uint32_t hdr_bytes;  // node offsets region
  uint32_t tile_bytes; // packed tile stride = shared-memory stage size
};

constexpr int kMaxStages = 32;
constexpr int kStagedThreads = kThreads + 32;  // consumer warps + the producer warp
constexpr int kConsumerWarps = kThreads / 32;

__host__ __device__ inline uint32_t align16u(uint64_t b) { return (uint32_t)((b + 15) & ~uint64_t(15)); }

// Bytes of packed tile k's used part (node offsets, indices, values).
template <int D, typename T>
__device__ __forceinline__ uint32_t packed_used(const StageGeom& g, int64_t slots) {
  return g.hdr_bytes + align16u(4 * slots) + align16u((uint64_t)slots * D * D * sizeof(T));
}

// Packs tile k (one warp per tile): node offsets relative to the tile's
// first slot, its neighbour indices and its CSR values (row (a, i) of the
// tile's node a keeps the CSR order: D^2 q0 + i D nb + D k + j from the tile
// start, q0 = a's relative offset).  Tiles over capacity are skipped.
template <int D, typename T>
__global__ void __launch_bounds__(kThreads) pack_tiles_kernel(SysT<T> S, StageGeom g, unsigned char* __restrict__ packed) {
  const int wl = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = w0; k < g.ntiles; k += nw) {
    const int64_t a0 = k * g.nt, a1 = min(a0 + g.nt, S.Nn);
    const int64_t s0 = S.node_ptr[a0], slots = S.node_ptr[a1] - s0;
    if (slots > g.cap_slots) continue;
    unsigned char* base = packed + k * (int64_t)g.tile_bytes;
    int32_t* __restrict__ P = reinterpret_cast<int32_t*>(base);
    int32_t* __restrict__ Nb = reinterpret_cast<int32_t*>(base + g.hdr_bytes);
    T* __restrict__ V = reinterpret_cast<T*>(base + g.hdr_bytes + align16u(4 * slots));
    for (int t = wl; t <= (int)(a1 - a0); t += 32) P[t] = (int32_t)(__ldg(S.node_ptr + a0 + t) - s0);
    const int32_t* __restrict__ nsrc = S.nbr + s0;
    for (int q = wl; q < (int)slots; q += 32) Nb[q] = __ldg(nsrc + q);
    // four loads in flight per lane
    const T* __restrict__ src = S.vals + (int64_t)D * D * s0;
    const int n = (int)slots * D * D;
    for (int e = wl; e < n; e += 128) {
      T v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = e + 32 * u < n ? __ldcs(src + e + 32 * u) : (T)0;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (e + 32 * u < n) V[e + 32 * u] = v[u];
    }
  }
}

// Row j of the node from the partial rows of its D component lanes: in step
// s the lane of component j' offers its partial of row (j' - s) mod D, and
// the lane of component j takes the offer of lane j + s (mod D).
template <int D, typename T>
__device__ __forceinline__ T node_rows_exchange(const T (&acc)[D], int j, int lane) {
  T row = acc[0];
#pragma unroll
  for (int i = 1; i < D; ++i) row = (j == i) ? acc[i] : row;
#pragma unroll
  for (int st = 1; st < D; ++st) {
    const int oi = j >= st ? j - st : j - st + D;  // (j - st) mod D
    const int sj = j + st < D ? j + st : j + st - D;  // (j + st) mod D
    T offer = acc[0];
#pragma unroll
    for (int i = 1; i < D; ++i) offer = (oi == i) ? acc[i] : offer;
    row += __shfl_sync(0xffffffffu, offer, lane - j + sj);
  }
  return row;
}

// Partial rows (all D rows, component j) of node a over its nb neighbours:
// the lane gathers p at component j of every neighbour once and accumulates
// vrow(i W + D k + j) x (W = D nb) into row i; nrow(k) are the neighbour
// indices.
// The gathers of a chunk of kGatherChunk neighbours are all issued before
// their products, so that a chunk costs one trip to L2 for the gathers that
// miss L1 (neighbours in other planes of the mesh live on other SMs).
constexpr int kGatherChunk = 27;

template <int D, typename T, bool DIFF, typename VR, typename NR>
__device__ __forceinline__ void node_component_partials(VR vrow, NR nrow, int nb, int64_t a, int j,
                                                        const T* __restrict__ p, T (&acc)[D]) {
  const int W = D * nb;
  const T self = DIFF ? __ldg(p + a * D + j) : (T)0;
#pragma unroll
  for (int i = 0; i < D; ++i) acc[i] = 0;
  for (int k0 = 0; k0 < nb; k0 += kGatherChunk) {
    T x[kGatherChunk];
#pragma unroll
    for (int m = 0; m < kGatherChunk; ++m) {
      const int k = k0 + m;
      x[m] = k < nb ? __ldg(p + ((uint32_t)nrow(k) * D + j)) : (T)0;
    }
#pragma unroll
    for (int m = 0; m < kGatherChunk; ++m) {
      const int k = k0 + m;
      if (k < nb) {
        const T xv = DIFF ? x[m] - self : x[m];
#pragma unroll
        for (int i = 0; i < D; ++i) acc[i] += vrow(i * W + D * k + j) * xv;
      }
    }
  }
}

template <int D, typename T, bool DIFF>
__global__ void __launch_bounds__(kStagedThreads, 2) apply_staged_kernel(SysT<T> S, StageGeom g,
                                                                         const unsigned char* __restrict__ packed,
                                                                         const T* __restrict__ p, T* __restrict__ Ap,
                                                                         double* partials, Scal* sc) {
  if (sc->done) return;
  extern __shared__ __align__(128) unsigned char stage_mem[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages];
  __shared__ int64_t tile_of[kMaxStages];  // tile held by each stage (-1 - k: read directly)
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, wl = threadIdx.x & 31;
  if (g.stages % kConsumerWarps || g.stages > kMaxStages) {  // the stage -> warp ownership needs this
    if (threadIdx.x == 0) {
      sc->status = GFEA_ERR_ARG;
      sc->done = 1;
    }
    return;
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < g.stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
      tile_of[s] = INT64_MIN;
    }
    abort_flag = 0;
  }
  __syncthreads();
  const int64_t Nn = S.Nn;
  // each block takes a contiguous range of tiles, so that the gathers of p
  // by consecutive tiles (overlapping neighbourhoods) hit the SM's L1
  const int64_t per_block = ceil_div(g.ntiles, gridDim.x);
  const int64_t t_begin = blockIdx.x * per_block;
  const int64_t t_end = min(t_begin + per_block, g.ntiles);
  DotAcc<T> pap;
  if (warp == kConsumerWarps) {
    // producer (lane 0); the tiles' slot counts come from node_ptr at the
    // tile boundaries, loaded 32 tiles at a time, one tile per lane
    const uint64_t pol = l2_evict_first();
    int i = 0;
    int64_t sl = 0;
    for (int64_t k = t_begin; k < t_end; ++k, ++i) {
      const int m = i & 31;
      if (m == 0) {
        const int64_t kl = k + wl;
        if (kl < t_end) sl = __ldg(S.node_ptr + min((kl + 1) * g.nt, Nn)) - __ldg(S.node_ptr + kl * g.nt);
      }
      const int64_t slots = __shfl_sync(0xffffffffu, sl, m);
      const int s = i % g.stages;
      // warp-uniform outcome of the bounded wait (the lanes leave together)
      if (i >= g.stages &&
          !__all_sync(0xffffffffu, mbar_wait(&empty[s], ((i / g.stages) - 1) & 1, &abort_flag))) {
        sc->status = GFEA_ERR_TIMEOUT;  // the last block ends the solve
        *(volatile int*)&abort_flag = 1;
        break;
      }
      if (wl == 0) {
        const bool dir = slots > g.cap_slots;
        tile_of[s] = dir ? -1 - k : k;
        if (dir) {
          mbar_arrive(&full[s]);
        } else {
          const uint32_t bytes = packed_used<D, T>(g, slots);
          mbar_expect_tx(&full[s], bytes);
          bulk_g2s(stage_mem + (size_t)s * g.tile_bytes, packed + k * (int64_t)g.tile_bytes, bytes, &full[s], pol);
          mbar_arrive(&full[s]);
        }
      }
      __syncwarp();
    }
    // the copies of the last tiles issued land before the block may exit
    if (wl == 0)
      for (int j = i > g.stages ? i - g.stages : 0; j < i; ++j) mbar_wait(&full[j % g.stages], (j / g.stages) & 1);
    __syncwarp();
  } else {
    // consumer warp 'warp' takes tiles warp, warp + 8, ... of the block
    int i = warp;
    for (int64_t k = t_begin + warp; k < t_end; k += kConsumerWarps, i += kConsumerWarps) {
      const int s = i % g.stages;
      if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (i / g.stages) & 1, &abort_flag))) {
        sc->status = GFEA_ERR_TIMEOUT;
        *(volatile int*)&abort_flag = 1;
        break;
      }
      const int64_t held = tile_of[s];
      if (held != k && held != -1 - k) {  // a stage filled for another tile: never read it
        sc->status = GFEA_ERR_TIMEOUT;
        *(volatile int*)&abort_flag = 1;
        break;
      }
      const int64_t a0 = k * g.nt, a1 = min(a0 + g.nt, Nn);
      // lane D n + j: node a0 + n, component j; lanes past the tile only
      // take part in the exchange
      const bool live = wl < D * g.nt && a0 + wl / D < a1;
      const int64_t a = live ? a0 + wl / D : a1 - 1;
      const int j = live ? wl % D : 0;
      T acc[D];
#pragma unroll
      for (int q = 0; q < D; ++q) acc[q] = 0;
      if (!live) {
      } else if (held < 0) {
        const int32_t q0 = __ldg(S.node_ptr + a), q1 = __ldg(S.node_ptr + a + 1);
        const T* vr = S.vals + (int64_t)D * D * q0;
        const int32_t* nr = S.nbr + q0;
        node_component_partials<D, T, DIFF>([vr](int t) { return __ldg(vr + t); },
                                            [nr](int t) { return __ldg(nr + t); }, q1 - q0, a, j, p, acc);
      } else {
        const unsigned char* base = stage_mem + (size_t)s * g.tile_bytes;
        const int32_t* P = reinterpret_cast<const int32_t*>(base);
        const int32_t* Nb = reinterpret_cast<const int32_t*>(base + g.hdr_bytes);
        const T* V = reinterpret_cast<const T*>(base + g.hdr_bytes + align16u(4 * (int64_t)P[a1 - a0]));
        const int32_t q0 = P[a - a0], q1 = P[a + 1 - a0];
        const T* vr = V + D * D * q0;
        const int32_t* nr = Nb + q0;
        node_component_partials<D, T, DIFF>([vr](int t) { return vr[t]; }, [nr](int t) { return nr[t]; }, q1 - q0,
                                            a, j, p, acc);
      }
      // lanes of a node are consecutive: the exchange's sources stay inside it
      T av = node_rows_exchange<D, T>(acc, j, live ? wl : wl - wl % D);
      if (live) {
        const int64_t dof = a * D + j;
        if (S.known[dof]) av = 0;
        Ap[dof] = av;
        pap.add_prod(__ldg(p + dof), av);
      }
      __syncwarp();
      if (wl == 0) mbar_arrive(&empty[s]);
    }
  }
  const DotAcc<T> v[1] = {pap};
  double out[1];
  if (reduce_last_acc<1, T>(v, partials, &sc->ticket1, out) && threadIdx.x == 0) {
    sc->pap = out[0];
    if (sc->status == GFEA_ERR_TIMEOUT) {
      sc->done = 1;
    } else if (!(out[0] > 0) || !isfinite(out[0])) {
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

int64_t spmv_key(const gfea_system* s, int value_type) {
  const double W = s->n_nodes > 0 ? (double)s->dof_n * (double)s->n_pairs / (double)s->n_nodes : 1.0;
  return tune_key(kTuneSpmv, s->dof_n, value_type, tune_log2(4 * W), tune_log2((double)s->n_nodes));
}

// values per row W = dof_n * neighbours: small groups for short rows
int lanes_rule(const gfea_system* s) {
  const double W = s->n_nodes > 0 ? (double)s->dof_n * (double)s->n_pairs / (double)s->n_nodes : 1.0;
  if (W <= 10) return 4;
  if (W <= 24) return 8;
  if (W <= 56) return 16;
  return 32;
}

// Lanes per node of the node-row products: the request, else the autotuner's
// decision for this problem class, else a rule on the row length.
int pick_lanes(const gfea_system* s, int requested, int value_type) {
  if (requested == 4 || requested == 8 || requested == 16 || requested == 32) return requested;
  int32_t tuned = 0;
  if (tune_get(spmv_key(s, value_type), &tuned)) return tuned;
  return lanes_rule(s);
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
  bool coarse = false;
  bool is_f32 = false;  // T-typed buffers hold floats
  CoarseDev C;
  unsigned char* packed = nullptr;  // tiles of the staged SpMV (nullptr: apply_kernel)
  StageGeom geom{};
  // CUDA graphs of kGraphIters PCG iterations, one per direction-buffer order
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  long long gkernels = 0;
  bool graphs_ok = true;
  // direct kernel launches only: no graph capture, no events, no tuning (the
  // allocation-free entry point, which must create no driver resources)
  bool direct_only = false;
  PcgWork() = default;
  PcgWork(const PcgWork&) = delete;
  PcgWork& operator=(const PcgWork&) = delete;
  ~PcgWork() {
    for (int i = 0; i < 2; ++i)
      if (gexec[i]) cudaGraphExecDestroy(gexec[i]);
  }
};

int coarse_nr(int D) { return D == 1 ? 1 : (D == 2 ? 3 : 6); }

// Number of aggregates of the coarse level (0: block-Jacobi only).
// Automatic: k Nn^0.43 (k = 0.6 for 3D elasticity, 1.5 otherwise), which
// balances the coarse inverse (~ nc^3) against the iterations it saves
// (~ (H/h) ~ (Nn / n_agg)^(1/dim)) per node-row product (~ Nn).
int coarse_target(const gfea_system* s, const gfea_pcg_opts* o) {
  if (!o || o->coarse == 0 || !s->coord) return 0;
  const int64_t cap = kCoarseMax / coarse_nr(s->dof_n);
  int64_t t = o->coarse > 0 ? o->coarse
                            : (int64_t)((s->dof_n == 3 ? 0.6 : 1.5) * pow((double)s->n_nodes, 0.43));
  if (t > cap) t = cap;
  if (t < 1) t = 1;
  return (int)t;
}

template <typename T>
size_t pcg_layout(int64_t Nn, int D, int n_agg_max, PcgWork* w, char* base, size_t packed = 0) {
  size_t off = 0;
  const int64_t N = Nn * D;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  PcgWork t;
  if (!w) w = &t;
  w->is_f32 = sizeof(T) == 4;
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
  w->coarse = n_agg_max > 0;
  if (w->coarse) {
    const int64_t nc = (int64_t)n_agg_max * coarse_nr(D);
    w->C.hdr = reinterpret_cast<CoarseHdr*>(take(sizeof(CoarseHdr)));
    w->C.agg = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * Nn));
    w->C.off = reinterpret_cast<float4*>(take(sizeof(float4) * Nn));
    w->C.Ac = reinterpret_cast<double*>(take(sizeof(double) * nc * nc));
    w->C.Ahi = reinterpret_cast<float*>(take(sizeof(float) * nc * nc));
    w->C.Alo = reinterpret_cast<float*>(take(sizeof(float) * nc * nc));
    w->C.rowph = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
    w->C.rowpl = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
    w->C.colph = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
    w->C.colpl = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
    w->C.pinvh = reinterpret_cast<float*>(take(sizeof(float) * kGJB * kGJB));
    w->C.pinvl = reinterpret_cast<float*>(take(sizeof(float) * kGJB * kGJB));
    w->C.rc = reinterpret_cast<double*>(take(sizeof(double) * nc));
    w->C.rcp = reinterpret_cast<double*>(take(sizeof(double) * nc * kRcCopies));
    w->C.ncopies = Nn >= kRcCopyMinNodes ? kRcCopies : 1;
    w->C.ec = reinterpret_cast<double*>(take(sizeof(double) * nc));
    w->C.ecf = reinterpret_cast<float*>(take(sizeof(float) * nc));
  }
  w->packed = packed ? reinterpret_cast<unsigned char*>(take(packed)) : nullptr;
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

int launch_resid(const gfea_system* s, int G, const double* b, const double* x, PcgWork& w, bool kn,
                 cudaStream_t st) {
  const SysT<double> S = sys_t<double>(s);
  const int grid = grid_nodes(s->n_nodes, G);
  const int64_t N = s->n_nodes * s->dof_n;
  const float* v32 = s->vals32;
  float* x32 = nullptr;
  if (v32 && w.is_f32) {  // FP32 copy of x for the floor product (the A.p buffer is free here)
    x32 = static_cast<float*>(w.Ap);
    cast_kernel<float><<<grid_elems(N), kThreads, 0, st>>>(x, x32, N);
    GFEA_LAUNCH_CHECK();
  }
#define GFEA_RESID(KN_, AB_)                                                                                   \
  GFEA_DG_SWITCH(s->dof_n, G, (resid_kernel<DD, GG, double, KN_, AB_><<<grid, kThreads, 0, st>>>(               \
                                  S, v32, x32, b, x, w.r64, w.partials, w.sc)))
  if (kn) {
    if (x32) { GFEA_RESID(true, true); } else { GFEA_RESID(true, false); }
  } else {
    if (x32) { GFEA_RESID(false, true); } else { GFEA_RESID(false, false); }
  }
#undef GFEA_RESID
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
  return prof_mark(st, kTagUpdate);
}

// Shared memory of the staged apply: one packed tile per stage, one stage
// per consumer warp (a deeper ring at one block per SM measured slower than
// this at two blocks per SM: twice the warps gathering p).
constexpr size_t kSmemMax = 220 * 1024;  // dynamic part (the opt-in limit is 227 KB with the static part)

// Tiles of apply_staged_kernel for this operator; false when it cannot be
// staged (no nodes or values, arrays not 4-byte aligned, tiles too large).
// A packed tile holds 15 % more neighbour slots than an average tile; larger
// tiles are read directly by the kernel.
template <typename T>
bool stage_geom(const gfea_system* s, const T* vals, StageGeom* g) {
  if (s->n_nodes <= 0 || !vals || s->n_pairs <= 0) return false;
  if (((uintptr_t)vals % sizeof(T)) | ((uintptr_t)s->nbr & 3) | ((uintptr_t)s->node_ptr & 3)) return false;
  const int D = s->dof_n;
  const double avg = (double)s->n_pairs / (double)s->n_nodes;
  const int nt = 32 / D;
  g->nt = nt;
  g->cap_slots = (int32_t)ceil(1.15 * avg * nt) + 8;
  g->hdr_bytes = align16u(4 * (uint64_t)(nt + 1));
  g->tile_bytes = g->hdr_bytes + align16u(4 * (uint64_t)g->cap_slots) +
                  align16u((uint64_t)g->cap_slots * D * D * sizeof(T));
  g->ntiles = ceil_div(s->n_nodes, nt);
  g->stages = kConsumerWarps;
  return (size_t)g->stages * g->tile_bytes <= kSmemMax;
}

// Operators whose packed tiles fit in half of the 129 MB L2 stay unstaged:
// the lane-group kernel then reads values that stay L2-resident across
// iterations, whereas the staged path adds a packing pass per solve and
// streams its tiles with an evict-first policy, so an L2-sized operator
// gains nothing from it (served small solves: 291 solves/s staged against
// 299 unstaged).
constexpr size_t kStageMinBytes = size_t(64) << 20;

// Workspace bytes of the packed tiles (0: not staged).  'query': sizes only
// (the arrays may not exist yet; a solve checks them again).
template <typename T>
size_t packed_bytes(const gfea_system* s, bool query = false) {
  StageGeom g;
  const T* vals = sizeof(T) == 4 ? (const T*)s->vals32 : (const T*)s->vals64;
  gfea_system q = *s;
  if (query) {  // stand-in aligned addresses for the checks on pointers
    vals = reinterpret_cast<const T*>(alignof(double));
    q.nbr = q.node_ptr = reinterpret_cast<const int32_t*>(alignof(double));
  }
  if (!stage_geom<T>(&q, vals, &g)) return 0;
  const size_t bytes = (size_t)g.ntiles * g.tile_bytes;
  size_t min_bytes = kStageMinBytes;  // GFEA_STAGE_MIN_BYTES overrides (0: stage every operator)
  if (const char* e = getenv("GFEA_STAGE_MIN_BYTES")) min_bytes = strtoull(e, nullptr, 10);
  return bytes < min_bytes ? 0 : bytes;
}

template <typename T>
int launch_pack(const gfea_system* s, PcgWork& w, cudaStream_t st) {
  const SysT<T> S = sys_t<T>(s);
  GFEA_D_SWITCH(s->dof_n, (pack_tiles_kernel<DD, T><<<kSMs * 8, kThreads, 0, st>>>(S, w.geom, w.packed)));
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

// Persistent grid of the staged apply: as many blocks as fit on the SMs.
template <int D, typename T, bool DIFF>
int launch_apply_staged(const SysT<T>& S, const StageGeom& g, const unsigned char* packed, const T* p, T* Ap,
                        double* partials, Scal* sc, cudaStream_t st) {
  auto kern = apply_staged_kernel<D, T, DIFF>;
  const size_t smem = (size_t)g.stages * g.tile_bytes;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [&] { attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax); });
  GFEA_CUDA_TRY(attr);
  static std::atomic<int64_t> occ{0};  // (smem << 8) | blocks per SM of the last query
  int64_t o = occ.load(std::memory_order_relaxed);
  int per_sm = (int)(o & 255);
  if ((o >> 8) != (int64_t)smem || per_sm == 0) {
    GFEA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kStagedThreads, smem));
    if (per_sm < 1) return GFEA_ERR_ARG;
    occ.store(((int64_t)smem << 8) | per_sm, std::memory_order_relaxed);
  }
  int64_t grid = (int64_t)kSMs * per_sm;
  if (grid > g.ntiles) grid = g.ntiles;
  if (grid > kMaxBlocks) grid = kMaxBlocks;
  if (grid < 1) grid = 1;
  kern<<<(int)grid, kStagedThreads, smem, st>>>(S, g, packed, p, Ap, partials, sc);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

// Masked SpMV with p.Ap and alpha: the staged kernel over the packed tiles
// when the workspace holds them, else apply_kernel (with z given and no
// packed tiles: the direction p_new = z + beta p formed inside it).
template <typename T>
int launch_apply(const gfea_system* s, int G, PcgWork& w, const T* p, cudaStream_t st, const T* z = nullptr,
                 T* p_new = nullptr) {
  const SysT<T> S = sys_t<T>(s);
  const bool diff = sizeof(T) == 4 && s->translation_invariant;
  if (w.packed) {
    int e = GFEA_OK;
    if (diff) {
      GFEA_D_SWITCH(s->dof_n, (e = launch_apply_staged<DD, T, true>(S, w.geom, w.packed, p, (T*)w.Ap, w.partials,
                                                                    w.sc, st)));
    } else {
      GFEA_D_SWITCH(s->dof_n, (e = launch_apply_staged<DD, T, false>(S, w.geom, w.packed, p, (T*)w.Ap,
                                                                     w.partials, w.sc, st)));
    }
    return e;
  }
  const int grid = grid_nodes(s->n_nodes, G);
  if (z && diff) {
    GFEA_DG_SWITCH(s->dof_n, G, (apply_kernel<DD, GG, T, true, true><<<grid, kThreads, 0, st>>>(
                                    S, p, (T*)w.Ap, w.partials, w.sc, z, p_new)));
  } else if (z) {
    GFEA_DG_SWITCH(s->dof_n, G, (apply_kernel<DD, GG, T, false, true><<<grid, kThreads, 0, st>>>(
                                    S, p, (T*)w.Ap, w.partials, w.sc, z, p_new)));
  } else if (diff) {
    GFEA_DG_SWITCH(s->dof_n, G, (apply_kernel<DD, GG, T, true><<<grid, kThreads, 0, st>>>(S, p, (T*)w.Ap,
                                                                                         w.partials, w.sc)));
  } else {
    GFEA_DG_SWITCH(s->dof_n, G, (apply_kernel<DD, GG, T, false><<<grid, kThreads, 0, st>>>(S, p, (T*)w.Ap,
                                                                                          w.partials, w.sc)));
  }
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <typename T>
int launch_dir(const gfea_system* s, int G, PcgWork& w, const T* p_old, T* p_new, cudaStream_t st) {
  if (!w.packed) {  // one kernel: the direction formed inside the SpMV
    const int e = launch_apply<T>(s, G, w, p_old, st, (const T*)w.z, p_new);
    if (e) return e;
    return prof_mark(st, kTagApply);
  }
  const int64_t N = s->n_nodes * s->dof_n;
  dir_kernel<T><<<grid_elems(N), kThreads, 0, st>>>(N, (const T*)w.z, p_old, p_new, w.sc);
  GFEA_LAUNCH_CHECK();
  int e = prof_mark(st, kTagDir);
  if (e) return e;
  e = launch_apply<T>(s, G, w, p_new, st);
  if (e) return e;
  return prof_mark(st, kTagApply);
}

// z = M^-1 r (with the x, r update in mode 0): update_kernel alone, or the
// restriction / coarse solve / prolongation sequence of the two-level
// preconditioner.
template <typename T>
int launch_precond(const gfea_system* s, PcgWork& w, T* x, T* p, int mode, cudaStream_t st) {
  if (!w.coarse) return launch_update<T>(s, w, x, p, mode, st);
  const int grid = grid_elems(s->n_nodes);
  GFEA_D_SWITCH(s->dof_n, (update_r_kernel<DD, T><<<grid, kThreads, 0, st>>>(s->n_nodes, s->known, x,
                                                                              (T*)w.r, p, (const T*)w.Ap, w.sc, w.C,
                                                                              mode)));
  GFEA_LAUNCH_CHECK();
  int e = prof_mark(st, kTagRestrict);
  if (e) return e;
  if (w.C.ncopies > 1) {
    rc_sum_kernel<<<(int)ceil_div(w.C.nc, kThreads), kThreads, 0, st>>>(w.C, w.sc, mode);
    GFEA_LAUNCH_CHECK();
  }
  coarse_gemv_kernel<<<std::min(w.C.nc, 8 * kSMs), kGemvThreads, 0, st>>>(w.C, w.sc, mode);
  GFEA_LAUNCH_CHECK();
  e = prof_mark(st, kTagGemv);
  if (e) return e;
  GFEA_D_SWITCH(s->dof_n, (finish_z_kernel<DD, T><<<grid, kThreads, 0, st>>>(s->n_nodes, s->known,
                                                                              (const T*)w.dinv, (const T*)w.r,
                                                                              (T*)w.z, w.partials + 2 * kMaxBlocks,
                                                                              w.sc, w.C, mode)));
  GFEA_LAUNCH_CHECK();
  return prof_mark(st, kTagFinish);
}

// Coarse level of the two-level preconditioner: aggregates = cells of a grid
// of about 'target' cells over the bounding box of the nodes (degenerate
// extents get one cell), A_c = R^T A R from the FP64 values, inverted in place.
constexpr int32_t kHdrValid = 0x5eed;

int coarse_aggregate(const gfea_system* s, int target, PcgWork& w, cudaStream_t st) {
  CoarseDev& C = w.C;
  const int64_t Nn = s->n_nodes;
  const int D = s->dof_n;
  bbox_kernel<<<kSMs, kThreads, 0, st>>>(s->coord, Nn, w.partials);
  GFEA_LAUNCH_CHECK();
  double hb[6 * kSMs];
  GFEA_CUDA_TRY(cudaMemcpyAsync(hb, w.partials, sizeof(hb), cudaMemcpyDeviceToHost, st));
  GFEA_CUDA_TRY(cudaStreamSynchronize(st));
  double lo[3], ext[3], emax = 0;
  for (int k = 0; k < 3; ++k) {
    double l = INFINITY, h = -INFINITY;
    for (int b = 0; b < kSMs; ++b) {
      l = fmin(l, hb[b * 6 + k]);
      h = fmax(h, hb[b * 6 + 3 + k]);
    }
    if (!isfinite(l) || !isfinite(h)) return GFEA_ERR_NAN;
    lo[k] = l;
    ext[k] = h - l;
    emax = fmax(emax, ext[k]);
  }
  bool act[3];
  int n_act = 0;
  double vol = 1;
  for (int k = 0; k < 3; ++k) {
    act[k] = ext[k] > 1e-9 * emax;
    if (act[k]) { ++n_act; vol *= ext[k]; }
  }
  int cells[3] = {1, 1, 1};
  if (n_act > 0) {
    const double h = pow(vol / target, 1.0 / n_act);
    for (int k = 0; k < 3; ++k)
      if (act[k]) cells[k] = (int)fmax(1.0, floor(ext[k] / h));
    auto prod = [&]() { return (int64_t)cells[0] * cells[1] * cells[2]; };
    while (prod() > target) {  // too many: coarsen the finest direction
      int kb = 0;
      for (int k = 1; k < 3; ++k) if (cells[k] > cells[kb]) kb = k;
      cells[kb] -= 1;
    }
    for (;;) {  // room left: refine the direction with the longest cells that still fits
      int kb = -1;
      for (int k = 0; k < 3; ++k)
        if (act[k] && prod() / cells[k] * (cells[k] + 1) <= target &&
            (kb < 0 || ext[k] / cells[k] > ext[kb] / cells[kb]))
          kb = k;
      if (kb < 0) break;
      cells[kb] += 1;
    }
  }
  double hk[3], hmax = 0;
  for (int k = 0; k < 3; ++k) {
    hk[k] = act[k] ? ext[k] / cells[k] : 1.0;
    if (act[k]) hmax = fmax(hmax, hk[k]);
  }
  int order[3] = {0, 1, 2};  // by number of cells, ascending (stable)
  for (int i = 1; i < 3; ++i)
    for (int j = i; j > 0 && cells[order[j]] < cells[order[j - 1]]; --j) {
      const int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
    }
  C.nr = coarse_nr(D);
  C.n_agg = cells[0] * cells[1] * cells[2];
  C.nc = C.nr * C.n_agg;
  aggregate_kernel<<<grid_elems(Nn), kThreads, 0, st>>>(
      s->coord, Nn, make_double3(lo[0], lo[1], lo[2]), make_double3(hk[0], hk[1], hk[2]),
      make_int3(cells[0], cells[1], cells[2]), make_int3(order[0], order[1], order[2]),
      hmax > 0 ? 1.0 / hmax : 1.0, C.agg, C.off);
  GFEA_LAUNCH_CHECK();
  CoarseHdr h{C.n_agg, C.nc, C.nr, kHdrValid, Nn};
  GFEA_CUDA_TRY(cudaMemcpyAsync(C.hdr, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  GFEA_CUDA_TRY(cudaStreamSynchronize(st));  // h leaves scope
  return GFEA_OK;
}

// Coarse level of the two-level preconditioner: aggregates = cells of a grid
// of about 'target' cells over the bounding box of the nodes (degenerate
// extents get one cell), A_c = R^T A R from the FP64 values, inverted in place.
// With 'reuse', an aggregation left in the workspace by an earlier call on the
// same node count and target is kept.
// A_c = R^T A R from the T-typed values, regularised and inverted in place
// (the aggregation in C is given).
template <typename T>
int coarse_matrix(const gfea_system* s, CoarseDev& C, cudaStream_t st, cudaEvent_t mark) {
  const int64_t Nn = s->n_nodes;
  const int D = s->dof_n;
  GFEA_CUDA_TRY(cudaMemsetAsync(C.Ac, 0, sizeof(double) * C.nc * C.nc, st));
  const SysT<T> S = sys_t<T>(s);
  GFEA_D_SWITCH(D, (coarse_assemble_kernel<DD, T><<<grid_elems(Nn), kThreads, 0, st>>>(S, C)));
  GFEA_LAUNCH_CHECK();
  if (sizeof(T) == 4)
    coarse_regularize_kernel<<<1, 256, 0, st>>>(C, 1e-6, 1e-6);
  else
    coarse_regularize_kernel<<<1, 256, 0, st>>>(C, 1e-14, 1e-10);
  GFEA_LAUNCH_CHECK();
  if (mark) GFEA_CUDA_TRY(cudaEventRecord(mark, st));
  const int64_t n2 = (int64_t)C.nc * C.nc;
  ff_split_kernel<<<grid_elems(n2), kThreads, 0, st>>>(C.Ac, C.Ahi, C.Alo, n2);
  GFEA_LAUNCH_CHECK();
  const int gx = (int)ceil_div(C.nc, 128);
  const int gy = (int)std::min<int64_t>(C.nc, ceil_div(2 * kMaxBlocks, gx));
  for (int k0 = 0; k0 < C.nc; k0 += kGJB) {
    const int b = std::min(kGJB, C.nc - k0);
    gj_panel_kernel<<<dim3(gx, b), 128, 0, st>>>(C, k0, b);
    GFEA_LAUNCH_CHECK();
    gj_update_kernel<<<dim3(gx, gy), 128, 0, st>>>(C, k0, b);
    GFEA_LAUNCH_CHECK();
  }
  ff_merge_kernel<<<grid_elems(n2), kThreads, 0, st>>>(C.Ac, C.Ahi, C.Alo, n2);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <typename T>
int coarse_setup(const gfea_system* s, int target, bool reuse, PcgWork& w, cudaStream_t st, cudaEvent_t mark) {
  CoarseDev& C = w.C;
  const int64_t Nn = s->n_nodes;
  const int D = s->dof_n;
  bool have = false;
  if (reuse) {
    CoarseHdr h;
    GFEA_CUDA_TRY(cudaMemcpyAsync(&h, C.hdr, sizeof(h), cudaMemcpyDeviceToHost, st));
    GFEA_CUDA_TRY(cudaStreamSynchronize(st));
    have = h.valid == kHdrValid && h.Nn == Nn && h.nr == coarse_nr(D) && h.n_agg >= 1 && h.n_agg <= target &&
           h.nc == h.nr * h.n_agg;
    if (have) {
      C.nr = h.nr;
      C.n_agg = h.n_agg;
      C.nc = h.nc;
    }
  }
  if (!have) {
    const int e = coarse_aggregate(s, target, w, st);
    if (e) return e;
  }
  const int e = coarse_matrix<T>(s, C, st, mark);
  if (e) return e;
  GFEA_CUDA_TRY(cudaMemsetAsync(C.rc, 0, sizeof(double) * C.nc, st));
  GFEA_CUDA_TRY(cudaMemsetAsync(C.rcp, 0, sizeof(double) * C.nc * kRcCopies, st));
  return GFEA_OK;
}

// SpMV row-block schedule: times the node-row product with 4, 8, 16 and 32
// lanes per node (CUDA events, 5 launches each after a warm-up) and records
// the fastest for this problem class.
template <typename T>
int tune_spmv_impl(const gfea_system* s, const T* x, T* y, cudaStream_t st, int32_t* best, float* best_ms) {
  const SysT<T> S = sys_t<T>(s);
  const bool diff = sizeof(T) == 4 && s->translation_invariant;
  const int vt = sizeof(T) == 4 ? GFEA_F32 : GFEA_F64;
  const int cand[4] = {4, 8, 16, 32};
  const int rule = lanes_rule(s);
  float bm = INFINITY, t_rule = INFINITY;
  int bg = 0;
  for (int c = 0; c < 4; ++c) {
    const int G = cand[c];
    if (G < s->dof_n) continue;
    const int grid = grid_nodes(s->n_nodes, G);
    float ms = 0;
    const int e = time_launches(
        [&]() -> int {
          if (diff) {
            GFEA_DG_SWITCH(s->dof_n, G, (spmv_kernel<DD, GG, T, true><<<grid, kThreads, 0, st>>>(S, x, y)));
          } else {
            GFEA_DG_SWITCH(s->dof_n, G, (spmv_kernel<DD, GG, T, false><<<grid, kThreads, 0, st>>>(S, x, y)));
          }
          GFEA_LAUNCH_CHECK();
          return GFEA_OK;
        },
        5, st, &ms);
    if (e) return e;
    if (G == rule) t_rule = ms;
    if (ms < bm) {
      bm = ms;
      bg = G;
    }
  }
  if (bg == 0) return GFEA_ERR_ARG;
  if (!(bm < 0.95f * t_rule)) {  // keep the rule unless clearly beaten
    bg = rule;
    bm = t_rule;
  }
  tune_put(spmv_key(s, vt), bg);
  *best = bg;
  *best_ms = bm;
  return GFEA_OK;
}

// Row-block schedule chosen on the PCG's own masked SpMV (apply_kernel, with
// the p.Ap reduction): each candidate is timed twice (5 launches after a
// warm-up) and the faster round counts; the rule's choice is kept unless a
// candidate beats it by more than 5 %.  p = w.pa must hold a direction with
// p.Ap > 0 on the unknowns.
template <typename T>
int tune_apply_impl(const gfea_system* s, PcgWork& w, cudaStream_t st, int* G_out) {
  const int vt = sizeof(T) == 4 ? GFEA_F32 : GFEA_F64;
  const int rule = lanes_rule(s);
  const int cand[4] = {4, 8, 16, 32};
  float t_rule = INFINITY, bm = INFINITY;
  int bg = rule;
  for (int c = 0; c < 4; ++c) {
    const int G = cand[c];
    if (G < s->dof_n) continue;
    float best = INFINITY;
    for (int round = 0; round < 2; ++round) {
      GFEA_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(Scal), st));
      float ms = 0;
      const int e = time_launches([&]() -> int { return launch_apply<T>(s, G, w, (const T*)w.pa, st); }, 5, st, &ms);
      if (e) return e;
      best = fminf(best, ms);
    }
    if (G == rule) t_rule = best;
    if (best < bm) {
      bm = best;
      bg = G;
    }
  }
  const int choice = (bm < 0.95f * t_rule) ? bg : rule;
  tune_put(spmv_key(s, vt), choice);
  *G_out = choice;
  return GFEA_OK;
}

// A chunk of PCG iterations is launched as CUDA graphs of kGraphIters
// iterations (captured once per solve on a private stream of the calling
// thread, so that the caller's stream may be the legacy default stream):
// one graph launch replaces 4 x (3 or 5) kernel launches, which dominate the
// iteration time of small systems.
constexpr int kGraphIters = 4;

// Solves in flight in this process (several host threads may solve at once).
// Concurrent solves hide each other's launch latency, while graph
// instantiation serialises them, so a solve that starts its iterations while
// others run launches its kernels directly.
std::atomic<int>& active_solves() {
  static std::atomic<int> n{0};
  return n;
}

struct ActiveSolve {
  ActiveSolve() { active_solves().fetch_add(1); }
  ~ActiveSolve() { active_solves().fetch_sub(1); }
};

// CUDA graphs instantiated by the library in this process (instrumentation).
std::atomic<long long>& graph_counter() {
  static std::atomic<long long> n{0};
  return n;
}

cudaStream_t capture_stream() {
  thread_local cudaStream_t cs = nullptr;
  if (!cs && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) cs = nullptr;
  return cs;
}

template <typename T>
int capture_iterations(const gfea_system* s, int G, PcgWork& w, T* x, T* p0, T* p1, cudaGraphExec_t* out) {
  cudaStream_t cs = capture_stream();
  if (!cs) return GFEA_ERR_CUDA;
  GFEA_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  T* buf[2] = {p0, p1};
  int e = GFEA_OK;
  for (int j = 0; j < kGraphIters && !e; ++j) {
    e = launch_dir<T>(s, G, w, buf[j & 1], buf[(j + 1) & 1], cs);
    if (!e) e = launch_precond<T>(s, w, x, buf[(j + 1) & 1], 0, cs);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(cs, &g);
  // kernels per iteration: direction + SpMV (one kernel without packed
  // tiles), then update (block-Jacobi) or
  // update/restrict + restriction sum (with restriction copies) + coarse
  // GEMV + finish (two-level); counted when the graph runs, not when it is
  // captured
  w.gkernels = (long long)kGraphIters * ((w.packed ? 2 : 1) + (w.coarse ? (w.C.ncopies > 1 ? 4 : 3) : 1));
  launch_counter().fetch_sub(w.gkernels);
  if (e || ce != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return e ? e : GFEA_ERR_CUDA;
  }
  const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    *out = nullptr;
    cudaGetLastError();
    return GFEA_ERR_CUDA;
  }
  graph_counter().fetch_add(1);
  return GFEA_OK;
}

// Runs PCG iterations until the device flags done, checking after chunks of
// 'check' iterations.  With 'grow' set, a chunk that did not finish is
// followed by one sized from the iterated residual's decay since the start
// of the call (rr0 at iters0): the iterations its log still needs to reach
// the trigger at the mean rate so far, plus 15 % and two (doubling when the
// residual has not decreased).  Iterations launched after the device set
// 'done' are no-op kernels that still cost their launch, so sizing the chunk
// to the expected remainder, rather than doubling it, keeps those few.  pa
// holds the current search direction on entry and exit.
template <typename T>
int pcg_loop(const gfea_system* s, int G, PcgWork& w, T* x, int check, bool grow, Scal* host_sc, T*& pa,
             T*& pb, int iters0, double rr0, cudaStream_t st) {
  // iteration j reads direction buf[j % 2] and writes buf[(j + 1) % 2]; launches
  // after the device set 'done' are no-ops, so the current direction follows
  // from the number of iterations actually performed
  T* buf[2] = {pa, pb};
  KernelProfile& P = prof();
  ChunkEvents& E = chunk_events();
  const int cap = P.on.load() ? 64 : 256;  // events of a timed chunk: 64 iterations at most
  if (grow && check > cap) check = cap;
  const bool timed = !w.direct_only && P.on.load() && check <= 64;
  if (timed && !E.created) {
    for (int i = 0; i < ChunkEvents::kEvents; ++i) GFEA_CUDA_TRY(cudaEventCreate(&E.ev[i]));
    E.created = true;
  }
  int before = iters0;
  // graphs are used outside timed chunks (their events need direct launches)
  const int order = pa == (T*)w.pa ? 0 : 1;
  static const bool graphs_env = [] {
    const char* v = getenv("GFEA_PCG_GRAPHS");  // "0": direct launches only
    return !(v && v[0] == '0');
  }();
  if (!graphs_env || w.direct_only || (!w.gexec[0] && !w.gexec[1] && active_solves().load() > 1))
    w.graphs_ok = false;
  if (!timed && w.graphs_ok && !w.gexec[order] &&
      capture_iterations<T>(s, G, w, x, buf[0], buf[1], &w.gexec[order]) != GFEA_OK)
    w.graphs_ok = false;  // direct launches from here on
  const bool graphs = !timed && w.graphs_ok && w.gexec[order];
  for (int j = 0;;) {
    E.active = timed;
    E.cur = 0;
    if (graphs) {  // an even number of iterations per graph keeps the buffer order
      for (int it = 0; it < check; it += kGraphIters, j += kGraphIters) {
        GFEA_CUDA_TRY(cudaGraphLaunch(w.gexec[order], st));
        launch_counter().fetch_add(w.gkernels);
      }
    } else {
      for (int it = 0; it < check; ++it, ++j) {
        int e = prof_mark(st, -1);
        if (e) return e;
        e = launch_dir<T>(s, G, w, buf[j & 1], buf[(j + 1) & 1], st);
        if (e) return e;
        e = launch_precond<T>(s, w, x, buf[(j + 1) & 1], 0, st);
        if (e) return e;
      }
    }
    E.active = false;
    GFEA_CUDA_TRY(cudaMemcpyAsync(host_sc, w.sc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
    GFEA_CUDA_TRY(cudaStreamSynchronize(st));
    if (timed) {  // attribute the launches of the iterations that did work
      const int performed = host_sc->iters - before;
      double ms_t[kNumTags] = {};
      long long n_t[kNumTags] = {};
      int itn = -1;
      for (int k = 0; k < E.cur; ++k) {
        if (E.tag[k] < 0) {
          if (++itn >= performed) break;
          continue;
        }
        float ms = 0;
        GFEA_CUDA_TRY(cudaEventElapsedTime(&ms, E.ev[k - 1], E.ev[k]));
        ms_t[E.tag[k]] += ms;
        n_t[E.tag[k]] += 1;
      }
      std::lock_guard<std::mutex> lock(P.mu);
      for (int t = 0; t < kNumTags; ++t) {
        P.ms[t] += ms_t[t];
        P.n[t] += n_t[t];
      }
    }
    before = host_sc->iters;
    if (host_sc->done) break;
    if (grow) {
      int next = check * 2;
      const int di = host_sc->iters - iters0;
      if (di > 0 && rr0 > 0 && host_sc->rr > 0 && host_sc->tol2 > 0) {
        const double lr = log(host_sc->rr);
        const double rate = (lr - log(rr0)) / di;  // log-residual change per iteration
        if (rate < 0 && isfinite(rate)) {
          const double rem = (log(host_sc->tol2) - lr) / rate;
          if (rem < 1e6) next = (int)ceil(1.15 * rem) + 2;
        }
      }
      next = (next + kGraphIters - 1) / kGraphIters * kGraphIters;  // whole graph launches
      check = next < kGraphIters ? kGraphIters : (next > cap ? cap : next);
    }
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
                 size_t work_bytes, gfea_pcg_result* res, cudaStream_t st, bool direct_only = false) {
  const auto t_start = std::chrono::steady_clock::now();
  const ActiveSolve active;
  PcgWork w;
  w.direct_only = direct_only;
  const int target = coarse_target(s, o);
  // the packed tiles of the staged SpMV when the workspace has room for them
  size_t pk = packed_bytes<T>(s);
  if (const char* e = getenv("GFEA_APPLY_STAGED")) if (e[0] == '0') pk = 0;  // the unstaged kernel (A/B runs)
  if (pk && pcg_layout<T>(s->n_nodes, s->dof_n, target, nullptr, nullptr, pk) > work_bytes) pk = 0;
  if (pcg_layout<T>(s->n_nodes, s->dof_n, target, &w, static_cast<char*>(work), pk) > work_bytes)
    return GFEA_ERR_WORKSPACE;
  if (pk) {
    stage_geom<T>(s, sys_t<T>(s).vals, &w.geom);
    const int ep = launch_pack<T>(s, w, st);
    if (ep) return ep;
  }
  const int vt = sizeof(T) == 4 ? GFEA_F32 : GFEA_F64;
  const int64_t N = s->n_nodes * s->dof_n;
  // host checks: every check_every iterations, or (check_every <= 0) after a
  // first chunk sized from the previous reliable-update cycle, then doubling
  const bool adaptive = o->check_every <= 0;
  int check = adaptive ? 16 : o->check_every;
  const bool fp64 = sizeof(T) == 8;
  const double eps64 = 2.220446049250313e-16;
  // reliable update after the iterated residual fell by delta: inner_rtol
  // (default 0.1) in FP32, whose recursive residual drifts from the true one
  // by ~eps32 * condition; 1000x in FP64
  // default: 0.1 with block-Jacobi alone, 0.01 with the coarse level (its
  // better conditioned FP32 iteration drifts less between updates)
  const double dlt = (o->inner_rtol > 0 && o->inner_rtol < 1) ? o->inner_rtol : (w.coarse ? 0.01 : 0.1);
  const double delta2 = fp64 ? 1e-6 : dlt * dlt;
  Scal hs;
  GFEA_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(Scal), st));
  GFEA_CUDA_TRY(cudaMemsetAsync(w.flag, 0, sizeof(int32_t) * 4, st));
  int e = launch_bjacobi<T>(s, w, st);
  if (e) return e;
  int G = pick_lanes(s, o->lanes, vt);
  if (w.coarse) {
    const bool dbg = !direct_only && getenv("GFEA_DEBUG") != nullptr;
    cudaEvent_t ev[3];
    if (dbg) {
      for (int i = 0; i < 3; ++i) GFEA_CUDA_TRY(cudaEventCreate(&ev[i]));
      GFEA_CUDA_TRY(cudaEventRecord(ev[0], st));
    }
    e = coarse_setup<T>(s, target, o->coarse_reuse != 0, w, st, dbg ? ev[1] : nullptr);
    if (e) return e;
    if (dbg) {
      GFEA_CUDA_TRY(cudaEventRecord(ev[2], st));
      GFEA_CUDA_TRY(cudaStreamSynchronize(st));
      float t1 = 0, t2 = 0;
      GFEA_CUDA_TRY(cudaEventElapsedTime(&t1, ev[0], ev[1]));
      GFEA_CUDA_TRY(cudaEventElapsedTime(&t2, ev[1], ev[2]));
      fprintf(stderr, "[gfea pcg] coarse level: %d aggregates, dimension %d; setup %.3f ms + inverse %.3f ms\n",
              w.C.n_agg, w.C.nc, t1, t2);
      for (int i = 0; i < 3; ++i) cudaEventDestroy(ev[i]);
    }
  }
  e = launch_resid(s, G, b, x, w, true, st);
  if (e) return e;
  int32_t flag = 0;
  GFEA_CUDA_TRY(cudaMemcpyAsync(&flag, w.flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  e = fetch(&hs, w, st);
  if (e) return e;
  if (flag) { res->status = GFEA_ERR_SINGULAR; return GFEA_ERR_SINGULAR; }
  int32_t tuned = 0;
  if (!direct_only && o->lanes == 0 && tune_cache().mode.load() == 2 && !tune_get(spmv_key(s, vt), &tuned) &&
      hs.rr_true > 0) {
    // first solve of this problem class: time the PCG's own SpMV kernel on the
    // initial residual, then reset the scalar record it wrote
    cast_kernel<T><<<grid_elems(N), kThreads, 0, st>>>(w.r64, (T*)w.pa, N);
    GFEA_LAUNCH_CHECK();
    e = tune_apply_impl<T>(s, w, st, &G);
    if (e) return e;
    GFEA_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(Scal), st));
  }
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
  e = launch_precond<T>(s, w, (T*)w.dx, pa, 1, st);
  if (e) return e;
  set_trigger_kernel<<<1, 1, 0, st>>>(w.sc, fmax(delta2 * rr, 0.25 * tol2), o->max_iters);
  GFEA_LAUNCH_CHECK();
  res->status = GFEA_ERR_NOT_CONVERGED;
  int stall = 0;
  int iters0 = 0;
  for (int upd = 0;; ++upd) {
    e = pcg_loop<T>(s, G, w, (T*)w.dx, check, adaptive, &hs, pa, pb, iters0, rr, st);
    if (adaptive) {
      const int cycle = hs.iters - iters0;
      check = cycle + 2 < 4 ? 4 : (cycle + 2 > 64 ? 64 : cycle + 2);
    }
    if (e) return e;
    res->iterations = hs.iters;
    const int st_inner = hs.status;
    // reliable update: x += dx (FP64), r = P(b - A x) in FP64
    add_correction_kernel<T><<<grid_elems(N), kThreads, 0, st>>>(x, (const T*)w.dx, s->known, N);
    GFEA_LAUNCH_CHECK();
    GFEA_CUDA_TRY(cudaMemsetAsync(w.dx, 0, sizeof(T) * N, st));
    e = launch_resid(s, G, b, x, w, false, st);
    if (e) return e;
    e = fetch(&hs, w, st);
    if (e) return e;
    rr = hs.rr_true;
    if (getenv("GFEA_DEBUG"))
      fprintf(stderr, "[gfea pcg%d] update %d: iterations %d, inner status %d, rel residual %.3e, %.2f ms\n",
              fp64 ? 64 : 32, upd + 1, hs.iters, st_inner, sqrt(rr / bb),
              std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count());
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
    e = launch_precond<T>(s, w, (T*)w.dx, pa, 2, st);
    if (e) return e;
    set_trigger_kernel<<<1, 1, 0, st>>>(w.sc, fmax(delta2 * rr, 0.25 * tol2), o->max_iters);
    GFEA_LAUNCH_CHECK();
  }
  return res->status;
}

// Self-test of the bounded mbarrier wait the staged SpMV relies on: thread 0
// initialises a barrier of one arrival, arrives or not, and waits on its
// first phase with the given limit; the outcome goes to selftest_status.
__device__ int32_t selftest_status;

__global__ void wait_selftest_kernel(uint64_t limit_ns, int arrive) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    abort_flag = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (arrive) mbar_arrive(&bar);
    selftest_status = mbar_wait(&bar, 0, &abort_flag, limit_ns) ? GFEA_OK : GFEA_ERR_TIMEOUT;
  }
}

}  // namespace
}  // namespace gfea

using namespace gfea;

extern "C" int gfea_selftest_wait(int32_t limit_us, int32_t arrive, int32_t* status_host, void* stream) {
  if (!status_host || limit_us < 1 || limit_us > 1000000) return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int32_t unset = -1;
  GFEA_CUDA_TRY(cudaMemcpyToSymbolAsync(selftest_status, &unset, sizeof(int32_t), 0, cudaMemcpyHostToDevice, st));
  wait_selftest_kernel<<<1, 32, 0, st>>>((uint64_t)limit_us * 1000ull, arrive != 0);
  GFEA_LAUNCH_CHECK();
  GFEA_CUDA_TRY(cudaMemcpyFromSymbolAsync(status_host, selftest_status, sizeof(int32_t), 0, cudaMemcpyDeviceToHost,
                                          st));
  GFEA_CUDA_TRY(cudaStreamSynchronize(st));
  return GFEA_OK;
}

extern "C" int gfea_spmv(const gfea_system* s, int value_type, const void* x, void* y, void* stream) {
  if (!s || s->version != GFEA_ABI_VERSION || !x || !y || s->n_nodes <= 0) return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int G = pick_lanes(s, 0, value_type);
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

extern "C" int gfea_tune_spmv(const gfea_system* s, int value_type, const void* x, void* y, int32_t* lanes_host,
                              float* ms_host, void* stream) {
  if (!s || s->version != GFEA_ABI_VERSION || !x || !y || !lanes_host || !ms_host || s->n_nodes <= 0 ||
      s->dof_n < 1 || s->dof_n > 3)
    return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (value_type == GFEA_F64) {
    if (!s->vals64) return GFEA_ERR_ARG;
    return tune_spmv_impl<double>(s, (const double*)x, (double*)y, st, lanes_host, ms_host);
  }
  if (value_type == GFEA_F32) {
    if (!s->vals32) return GFEA_ERR_ARG;
    return tune_spmv_impl<float>(s, (const float*)x, (float*)y, st, lanes_host, ms_host);
  }
  return GFEA_ERR_ARG;
}

extern "C" int gfea_pcg_workspace_size(const gfea_system* s, const gfea_pcg_opts* o, size_t* bytes) {
  if (!s || !o || !bytes || s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3) return GFEA_ERR_ARG;
  const int target = coarse_target(s, o);
  if (o->precision == GFEA_F64)
    *bytes = pcg_layout<double>(s->n_nodes, s->dof_n, target, nullptr, nullptr, packed_bytes<double>(s, true));
  else
    *bytes = pcg_layout<float>(s->n_nodes, s->dof_n, target, nullptr, nullptr, packed_bytes<float>(s, true));
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

// ---------------------------------------------------------------------------
// Coarse level for the batched PCG (gfea_batch_pcg): the same aggregation,
// coarse matrix and inverse as the single-system two-level preconditioner,
// built into a caller workspace, plus the nodes of each aggregate in
// ascending order (the batched restriction gathers them in a fixed order) and
// an FP32 copy of the inverse (the FP32 iteration's coarse GEMV).
// ---------------------------------------------------------------------------

// Coarse dimension cap of the batched solve: the whole inverse is read once
// per iteration by the one cluster that owns the system.
constexpr int kBatchCoarseMax = 512;

struct CoarseLevelWork {
  CoarseDev C;
  double* partials = nullptr;
  int32_t* agg_ptr = nullptr;
  int32_t* agg_nodes = nullptr;
  int32_t* counts = nullptr;
  float* inv32 = nullptr;
};

int batch_coarse_target(const gfea_system* s, const gfea_pcg_opts* o) {
  const int t = coarse_target(s, o);
  const int cap = kBatchCoarseMax / coarse_nr(s->dof_n);
  return t > cap ? cap : t;
}

size_t coarse_level_layout(int64_t Nn, int D, int n_agg_max, CoarseLevelWork* w, char* base) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  CoarseLevelWork t;
  if (!w) w = &t;
  const int64_t nc = (int64_t)n_agg_max * coarse_nr(D);
  CoarseDev& C = w->C;
  w->partials = reinterpret_cast<double*>(take(sizeof(double) * 4 * kMaxBlocks));
  C.hdr = reinterpret_cast<CoarseHdr*>(take(sizeof(CoarseHdr)));
  C.agg = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * Nn));
  C.off = reinterpret_cast<float4*>(take(sizeof(float4) * Nn));
  C.Ac = reinterpret_cast<double*>(take(sizeof(double) * nc * nc));
  C.Ahi = reinterpret_cast<float*>(take(sizeof(float) * nc * nc));
  C.Alo = reinterpret_cast<float*>(take(sizeof(float) * nc * nc));
  C.rowph = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
  C.rowpl = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
  C.colph = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
  C.colpl = reinterpret_cast<float*>(take(sizeof(float) * kGJB * nc));
  C.pinvh = reinterpret_cast<float*>(take(sizeof(float) * kGJB * kGJB));
  C.pinvl = reinterpret_cast<float*>(take(sizeof(float) * kGJB * kGJB));
  C.rc = reinterpret_cast<double*>(take(sizeof(double) * nc));
  C.ec = reinterpret_cast<double*>(take(sizeof(double) * nc));
  C.ecf = reinterpret_cast<float*>(take(sizeof(float) * nc));
  w->agg_ptr = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * (n_agg_max + 1)));
  w->counts = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * (n_agg_max + 1)));
  w->agg_nodes = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * Nn));
  w->inv32 = reinterpret_cast<float*>(take(sizeof(float) * nc * nc));
  return off;
}

__global__ void agg_count_kernel(const int32_t* __restrict__ agg, int64_t Nn, int32_t* counts) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < Nn; a += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&counts[agg[a]], 1);
}

// ptr = exclusive scan of counts (one block; n_agg <= kBatchCoarseMax)
__global__ void agg_scan_kernel(const int32_t* __restrict__ counts, int n, int32_t* ptr) {
  if (threadIdx.x == 0) {
    int32_t s = 0;
    for (int g = 0; g < n; ++g) {
      ptr[g] = s;
      s += counts[g];
    }
    ptr[n] = s;
  }
}

// Nodes of aggregate g in ascending order: warp g scans the node range in
// order, placing its matches with a ballot prefix (no atomics, deterministic).
__global__ void agg_fill_kernel(const int32_t* __restrict__ agg, int64_t Nn, int n_agg,
                                const int32_t* __restrict__ ptr, int32_t* __restrict__ nodes) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = warp; g < n_agg; g += nwarps) {
    int32_t pos = ptr[g];
    for (int64_t base = 0; base < Nn; base += 32) {
      const int64_t a = base + lane;
      const bool hit = a < Nn && agg[a] == (int32_t)g;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (hit) nodes[pos + __popc(m & ((1u << lane) - 1u))] = (int32_t)a;
      pos += __popc(m);
    }
  }
}

extern "C" int gfea_coarse_workspace_size(const gfea_system* s, const gfea_pcg_opts* o, size_t* bytes) {
  if (!s || !o || !bytes || s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3) return GFEA_ERR_ARG;
  const int target = batch_coarse_target(s, o);
  *bytes = target > 0 ? coarse_level_layout(s->n_nodes, s->dof_n, target, nullptr, nullptr) : 0;
  return GFEA_OK;
}

extern "C" int gfea_coarse_setup(const gfea_system* s, const gfea_pcg_opts* o, int keep_aggregation, void* work,
                                 size_t work_bytes, gfea_coarse_level* level, void* stream) {
  if (!s || !o || !work || !level) return GFEA_ERR_ARG;
  if (s->version != GFEA_ABI_VERSION || o->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3 || !s->node_ptr || !s->nbr || !s->known || !s->coord)
    return GFEA_ERR_ARG;
  const bool f32 = o->precision == GFEA_F32;
  if (!(f32 ? (const void*)s->vals32 : (const void*)s->vals64)) return GFEA_ERR_ARG;
  const int target = batch_coarse_target(s, o);
  if (target <= 0) return GFEA_ERR_ARG;
  if (coarse_level_layout(s->n_nodes, s->dof_n, target, nullptr, nullptr) > work_bytes) return GFEA_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CoarseLevelWork cw;
  coarse_level_layout(s->n_nodes, s->dof_n, target, &cw, static_cast<char*>(work));
  CoarseDev& C = cw.C;
  C.ncopies = 1;
  const int64_t Nn = s->n_nodes;
  if (keep_aggregation) {
    // the aggregation of an earlier call on this mesh and workspace
    if (level->n_agg < 1 || level->n_agg > target || level->nr != coarse_nr(s->dof_n) ||
        level->nc != level->nr * level->n_agg || level->agg != C.agg)
      return GFEA_ERR_ARG;
    C.nr = level->nr;
    C.n_agg = level->n_agg;
    C.nc = level->nc;
  } else {
    PcgWork w;
    w.partials = cw.partials;
    w.C = C;
    const int e = coarse_aggregate(s, target, w, st);
    if (e) return e;
    C = w.C;
    GFEA_CUDA_TRY(cudaMemsetAsync(cw.counts, 0, sizeof(int32_t) * (C.n_agg + 1), st));
    agg_count_kernel<<<grid_elems(Nn), kThreads, 0, st>>>(C.agg, Nn, cw.counts);
    GFEA_LAUNCH_CHECK();
    agg_scan_kernel<<<1, 32, 0, st>>>(cw.counts, C.n_agg, cw.agg_ptr);
    GFEA_LAUNCH_CHECK();
    const int warps_per_block = kThreads / 32;
    agg_fill_kernel<<<(int)ceil_div(C.n_agg, warps_per_block), kThreads, 0, st>>>(C.agg, Nn, C.n_agg, cw.agg_ptr,
                                                                                   cw.agg_nodes);
    GFEA_LAUNCH_CHECK();
  }
  const int e = f32 ? coarse_matrix<float>(s, C, st, nullptr) : coarse_matrix<double>(s, C, st, nullptr);
  if (e) return e;
  const int64_t n2 = (int64_t)C.nc * C.nc;
  cast_kernel<float><<<grid_elems(n2), kThreads, 0, st>>>(C.Ac, cw.inv32, n2);
  GFEA_LAUNCH_CHECK();
  level->n_agg = C.n_agg;
  level->nr = C.nr;
  level->nc = C.nc;
  level->pad = 0;
  level->agg = C.agg;
  level->off = reinterpret_cast<const float*>(C.off);
  level->agg_ptr = cw.agg_ptr;
  level->agg_nodes = cw.agg_nodes;
  level->inv = C.Ac;
  level->inv32 = cw.inv32;
  level->rc = C.rc;
  level->ec = C.ec;
  return GFEA_OK;
}

// ---------------------------------------------------------------------------
// Coarse matrices and inverses of a whole batch with one launch per stage:
// the single-system stages above, with blockIdx.y (elementwise and assembly
// stages) or blockIdx.z (Gauss-Jordan panels) selecting the system.  A batch
// of 256 systems otherwise records ~15,000 launches, each a few microseconds.
// ---------------------------------------------------------------------------

struct CoarseJob {
  CoarseDev C;
  int64_t Nn;
  const int32_t* node_ptr;
  const int32_t* nbr;
  const void* vals;  // the iteration's value type
  const uint8_t* known;
  float* inv32;
  int32_t dof_n;
  int32_t diff;
};

__global__ void cb_zero_kernel(const CoarseJob* __restrict__ jobs) {
  const CoarseDev C = jobs[blockIdx.y].C;
  const int64_t n2 = (int64_t)C.nc * C.nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
    C.Ac[i] = 0.0;
}

template <int D, typename T>
__global__ void cb_assemble_kernel(const CoarseJob* __restrict__ jobs, int first) {
  const CoarseJob& J = jobs[first + blockIdx.y];
  if (J.dof_n != D) return;
  const SysT<T> S{J.Nn, J.node_ptr, J.nbr, static_cast<const T*>(J.vals), J.known, J.diff};
  coarse_assemble_body<D, T>(S, J.C, blockIdx.x, gridDim.x);
}

__global__ void cb_regularize_kernel(const CoarseJob* __restrict__ jobs, double zero_tol, double shift) {
  coarse_regularize_body(jobs[blockIdx.x].C, zero_tol, shift);
}

__global__ void cb_split_kernel(const CoarseJob* __restrict__ jobs) {
  const CoarseDev C = jobs[blockIdx.y].C;
  const int64_t n2 = (int64_t)C.nc * C.nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
    ff_split(C.Ac[i], C.Ahi[i], C.Alo[i]);
}

// merge the float-float pairs back into A_c^-1 and write its FP32 copy
__global__ void cb_merge_kernel(const CoarseJob* __restrict__ jobs) {
  const CoarseJob& J = jobs[blockIdx.y];
  const CoarseDev C = J.C;
  const int64_t n2 = (int64_t)C.nc * C.nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)C.Ahi[i] + (double)C.Alo[i];
    C.Ac[i] = v;
    J.inv32[i] = (float)v;
  }
}

__global__ void __launch_bounds__(128) cb_gj_panel_kernel(const CoarseJob* __restrict__ jobs, int k0) {
  const CoarseDev C = jobs[blockIdx.z].C;
  if (k0 >= C.nc) return;
  const int b = C.nc - k0 < kGJB ? C.nc - k0 : kGJB;
  if ((int)blockIdx.y >= b || (int)(blockIdx.x * blockDim.x) >= C.nc) return;
  gj_panel_body(C, k0, b, blockIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(128) cb_gj_update_kernel(const CoarseJob* __restrict__ jobs, int k0) {
  const CoarseDev C = jobs[blockIdx.z].C;
  if (k0 >= C.nc) return;
  const int b = C.nc - k0 < kGJB ? C.nc - k0 : kGJB;
  gj_update_body(C, k0, b, blockIdx.x, blockIdx.y, gridDim.y);
}

extern "C" size_t gfea_coarse_batch_scratch_size(int n) {
  return n < 0 ? 0 : align256(sizeof(CoarseJob) * (size_t)(n > 0 ? n : 1));
}

extern "C" int gfea_coarse_batch_prepare(const gfea_system* systems, const gfea_pcg_opts* o, int n,
                                         void* const* works, const gfea_coarse_level* levels, void* scratch,
                                         size_t scratch_bytes, void* stream) {
  if (!systems || !o || n < 0 || (n > 0 && (!works || !levels)) || !scratch) return GFEA_ERR_ARG;
  if (o->version != GFEA_ABI_VERSION || (o->precision != GFEA_F32 && o->precision != GFEA_F64)) return GFEA_ERR_ARG;
  if (scratch_bytes < gfea_coarse_batch_scratch_size(n)) return GFEA_ERR_WORKSPACE;
  if (n == 0) return GFEA_OK;
  const bool f32 = o->precision == GFEA_F32;
  std::vector<CoarseJob> jobs((size_t)n);
  // systems of one dof_n are contiguous (the assembly stage runs per dof_n)
  for (int i = 0; i < n; ++i) {
    const gfea_system* s = &systems[i];
    const gfea_coarse_level& L = levels[i];
    if (s->version != GFEA_ABI_VERSION || s->n_nodes <= 0 || s->dof_n < 1 || s->dof_n > 3 || !works[i])
      return GFEA_ERR_ARG;
    if (i > 0 && s->dof_n < systems[i - 1].dof_n) return GFEA_ERR_ARG;
    if (!(f32 ? (const void*)s->vals32 : (const void*)s->vals64)) return GFEA_ERR_ARG;
    const int target = batch_coarse_target(s, o);
    CoarseLevelWork cw;
    coarse_level_layout(s->n_nodes, s->dof_n, target, &cw, static_cast<char*>(works[i]));
    // the aggregation a gfea_coarse_setup call left in this workspace
    if (target <= 0 || L.n_agg < 1 || L.n_agg > target || L.nr != coarse_nr(s->dof_n) || L.nc != L.nr * L.n_agg ||
        L.agg != cw.C.agg)
      return GFEA_ERR_ARG;
    CoarseJob& J = jobs[(size_t)i];
    J.C = cw.C;
    J.C.nr = L.nr;
    J.C.n_agg = L.n_agg;
    J.C.nc = L.nc;
    J.C.ncopies = 1;
    J.Nn = s->n_nodes;
    J.node_ptr = s->node_ptr;
    J.nbr = s->nbr;
    J.vals = f32 ? (const void*)s->vals32 : (const void*)s->vals64;
    J.known = s->known;
    J.inv32 = cw.inv32;
    J.dof_n = s->dof_n;
    J.diff = s->translation_invariant;
  }
  GFEA_CUDA_TRY(cudaMemcpyAsync(scratch, jobs.data(), sizeof(CoarseJob) * (size_t)n, cudaMemcpyHostToDevice,
                                static_cast<cudaStream_t>(stream)));
  GFEA_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));  // jobs leaves scope
  return GFEA_OK;
}

extern "C" int gfea_coarse_batch_build(const void* scratch, int n, const int32_t* dof_n_first_host, int max_nc,
                                       int precision, void* stream) {
  if (!scratch || n < 0 || !dof_n_first_host || max_nc < 0 || max_nc > kBatchCoarseMax) return GFEA_ERR_ARG;
  if (precision != GFEA_F32 && precision != GFEA_F64) return GFEA_ERR_ARG;
  if (n == 0 || max_nc == 0) return GFEA_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const auto* jobs = static_cast<const CoarseJob*>(scratch);
  const int64_t n2 = (int64_t)max_nc * max_nc;
  const int ge = (int)std::min<int64_t>(ceil_div(n2, kThreads), 64);
  cb_zero_kernel<<<dim3(ge, n), kThreads, 0, st>>>(jobs);
  GFEA_LAUNCH_CHECK();
  // dof_n_first_host[d - 1] = first system with dof_n = d (n if none), d = 1..3; [3] = n
  for (int d = 1; d <= 3; ++d) {
    const int first = dof_n_first_host[d - 1], last = dof_n_first_host[d];
    if (first < 0 || last > n || first > last) return GFEA_ERR_ARG;
    if (first == last) continue;
    const dim3 grid(kSMs, last - first);
    if (precision == GFEA_F32) {
      GFEA_D_SWITCH(d, (cb_assemble_kernel<DD, float><<<grid, kThreads, 0, st>>>(jobs, first)));
    } else {
      GFEA_D_SWITCH(d, (cb_assemble_kernel<DD, double><<<grid, kThreads, 0, st>>>(jobs, first)));
    }
    GFEA_LAUNCH_CHECK();
  }
  if (precision == GFEA_F32)
    cb_regularize_kernel<<<n, 256, 0, st>>>(jobs, 1e-6, 1e-6);
  else
    cb_regularize_kernel<<<n, 256, 0, st>>>(jobs, 1e-14, 1e-10);
  GFEA_LAUNCH_CHECK();
  cb_split_kernel<<<dim3(ge, n), kThreads, 0, st>>>(jobs);
  GFEA_LAUNCH_CHECK();
  const int gx = (int)ceil_div(max_nc, 128);
  const int gy = (int)std::min<int64_t>(max_nc, 16);
  for (int k0 = 0; k0 < max_nc; k0 += kGJB) {
    cb_gj_panel_kernel<<<dim3(gx, kGJB, n), 128, 0, st>>>(jobs, k0);
    GFEA_LAUNCH_CHECK();
    cb_gj_update_kernel<<<dim3(gx, gy, n), 128, 0, st>>>(jobs, k0);
    GFEA_LAUNCH_CHECK();
  }
  cb_merge_kernel<<<dim3(ge, n), kThreads, 0, st>>>(jobs);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" size_t gfea_reduce_workspace_size(void) { return sizeof(double) * 4 * kMaxBlocks + 256; }

extern "C" int gfea_reaction_energy(const gfea_system* s, const double* x, const int64_t* dofs, int64_t n_dofs,
                                    double* Ax, double* out_host, void* work, void* stream) {
  if (!s || !x || !Ax || !out_host || !work || s->n_nodes <= 0 || !s->vals64) return GFEA_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partials = static_cast<double*>(work);
  Scal* sc = reinterpret_cast<Scal*>(partials + 4 * kMaxBlocks);
  GFEA_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(Scal), st));
  const int G = pick_lanes(s, 0, GFEA_F64);
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

extern "C" long long gfea_cuda_graph_count(void) { return gfea::graph_counter().load(); }

extern "C" int gfea_profile_enable(int on) {
  gfea::prof().on = on != 0;
  return GFEA_OK;
}

extern "C" int gfea_profile_read(double* ms_host, long long* launches_host) {
  if (!ms_host || !launches_host) return GFEA_ERR_ARG;
  gfea::KernelProfile& P = gfea::prof();
  std::lock_guard<std::mutex> lock(P.mu);
  *ms_host = P.ms[gfea::kTagApply];
  *launches_host = P.n[gfea::kTagApply];
  if (getenv("GFEA_DEBUG"))
    for (int t = 0; t < gfea::kNumTags; ++t)
      if (P.n[t] > 0)
        fprintf(stderr, "[gfea profile] %-16s %7lld launches, %.4f ms per launch\n", gfea::kTagNames[t], P.n[t],
                P.ms[t] / P.n[t]);
  for (int t = 0; t < gfea::kNumTags; ++t) {
    P.ms[t] = 0;
    P.n[t] = 0;
  }
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

namespace gfea {
namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch in the current device's context.  The
// array's name in host code is only a host-side stand-in; the lookup is cheap
// and is repeated on every call, so the address stays valid across device
// switches and context re-creation (cudaDeviceReset).
int static_scratch(void** out) {
  void* p = nullptr;
  GFEA_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
  *out = p;
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
  const int target = coarse_target(s, o);
  const size_t need = o->precision == GFEA_F64
                          ? pcg_layout<double>(s->n_nodes, s->dof_n, target, nullptr, nullptr)
                          : pcg_layout<float>(s->n_nodes, s->dof_n, target, nullptr, nullptr);
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
  // the array keeps whatever the last call (on any mesh) left in it, so a
  // coarse aggregation is never reused from it
  gfea_pcg_opts oo = *o;
  oo.coarse_reuse = 0;
  // direct launches only: no graph, stream or event is created
  if (o->precision == GFEA_F64) return refine_solve<double>(s, b, x, &oo, scratch, kStaticScratchBytes, res, st, true);
  return refine_solve<float>(s, b, x, &oo, scratch, kStaticScratchBytes, res, st, true);
}

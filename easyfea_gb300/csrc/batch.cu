// Cluster-resident batched PCG: many independent systems in one persistent launch.
//
// Each thread-block cluster (kCL CTAs) takes one system at a time from a work
// counter and runs its whole solve without returning to the host: the node
// loops are spread over the cluster's CTAs, every reduction is a block
// reduction followed by one hardware cluster barrier and a fixed-order sum of
// the kCL block partials read through distributed shared memory (so every
// thread of the cluster obtains the same value, control flow stays uniform,
// and a system's result does not depend on which other systems share the
// launch).  Iterations are FP32 (values, vectors, block-Jacobi) with FP64 dot
// products, scalars and reliable-update residuals, or FP64 throughout.
//
// Cross-CTA reads of vectors written inside the launch use L2-only loads
// (ld.global.cg), so no stale L1 line is ever consulted; the cluster barrier
// orders the writes (release/acquire at cluster scope).

#include <cooperative_groups.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "coarse.cuh"
#include "common.cuh"
#include "rowops.cuh"

namespace cg = cooperative_groups;

namespace gfea {
namespace {

constexpr int kCL = 8;    // CTAs per cluster (portable cluster size)
constexpr int kBT = 256;  // threads per CTA

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
struct BatchBuf {
  T *r, *z, *pa, *pb, *Ap, *dinv, *dx;
  double* r64;
};

template <typename T>
__host__ __device__ size_t batch_layout(int64_t Nn, int D, BatchBuf<T>* w, char* base) {
  const size_t N = (size_t)Nn * D;
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  BatchBuf<T> t;
  if (!w) w = &t;
  w->r = (T*)take(sizeof(T) * N);
  w->z = (T*)take(sizeof(T) * N);
  w->pa = (T*)take(sizeof(T) * N);
  w->pb = (T*)take(sizeof(T) * N);
  w->Ap = (T*)take(sizeof(T) * N);
  w->dinv = (T*)take(sizeof(T) * N * D);
  w->dx = (T*)take(sizeof(T) * N);
  w->r64 = (double*)take(sizeof(double) * N);
  return off;
}

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) {
  return __ldcg(p);
}

struct Ctx {
  cg::cluster_group cl;
  unsigned rank;
  double* slots;  // this CTA's 2 x 4 reduction slots
  double* sh;     // block_sum scratch
  int phase;
};

// Cluster-wide sum of NV values; every thread of every CTA gets the same result.
template <int NV>
__device__ void csum(Ctx& c, const double (&v)[NV], double (&out)[NV]) {
  double* slot = c.slots + (c.phase & 1) * 4;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double s = block_sum(v[k], c.sh);
    if (threadIdx.x == 0) slot[k] = s;
  }
  c.cl.sync();
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = 0;
  for (unsigned r = 0; r < (unsigned)kCL; ++r) {
    const double* rs = c.cl.map_shared_rank(slot, r);
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] += rs[k];
  }
  ++c.phase;
}

// FP64 residual r64 = P(b - A64 x) over the cluster; partials r.r, ||P(b - A x_c)||^2,
// ||P(|A||x| + |b|)||^2 accumulated into v[0..2].
template <int D, int G>
__device__ void resid64(const SysT<double>& S, const double* b, const double* x, double* r64, int64_t grp,
                        int64_t ngrp, int lane, double (&v)[4]) {
  const int64_t Nn = S.Nn;
  const int64_t sub = grp % (32 / G);
  for (int64_t a0 = grp - sub; a0 < Nn; a0 += ngrp) {
    const int64_t a = a0 + sub;
    const int64_t ac = a < Nn ? a : Nn - 1;
    double all[D], kn[D], ab[D];
    node_rows<D, G, double, double>(ac, lane, S, [&](int64_t cc) { return ldcg(x + cc); }, all);
    node_rows<D, G, double, double>(ac, lane, S,
                                    [&](int64_t cc) { return S.known[cc] ? ldcg(x + cc) : 0.0; }, kn);
    node_rows<D, G, double, double, true>(ac, lane, S, [&](int64_t cc) { return fabs(ldcg(x + cc)); }, ab);
    if (a < Nn && lane == 0) {
#pragma unroll
      for (int i = 0; i < D; ++i) {
        const int64_t dof = a * D + i;
        const bool unk = !S.known[dof];
        const double bi = __ldg(b + dof);
        const double ri = unk ? bi - all[i] : 0.0;
        const double rci = unk ? bi - kn[i] : 0.0;
        const double ai = unk ? ab[i] + fabs(bi) : 0.0;
        r64[dof] = ri;
        v[0] += ri * ri;
        v[1] += rci * rci;
        v[2] += ai * ai;
      }
    }
  }
}

// r = (T) r64, z = D^-1 r (masked) for the nodes of this thread; partials r.z, r.r.
template <int D, typename T>
__device__ void restart_rz(const gfea_batch_instance& I, const BatchBuf<T>& w, int64_t gtid, int64_t nthr,
                           double (&v)[2]) {
  for (int64_t a = gtid; a < I.n_nodes; a += nthr) {
    T rl[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const int64_t dof = a * D + i;
      rl[i] = (T)ldcg(w.r64 + dof);
      w.r[dof] = rl[i];
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
      T zi = 0;
#pragma unroll
      for (int j = 0; j < D; ++j) zi += w.dinv[a * D * D + i * D + j] * rl[j];
      if (I.known[a * D + i]) zi = 0;
      w.z[a * D + i] = zi;
      v[0] += (double)rl[i] * (double)zi;
      v[1] += (double)rl[i] * (double)rl[i];
    }
  }
}

// node_rows for R nodes at once (one G-lane group): the index, value and
// gathered-vector loads of the R rows in a pass are independent and issued
// together.  A cluster runs 16 warps per SM, too few to hide the three
// dependent L2 round trips of a row (row pointer, neighbour index, gather)
// one row at a time.
template <int D, int G, typename T, bool DIFF, int R, typename XF>
__device__ __forceinline__ void node_rows_multi(const int64_t (&a)[R], int lane, const SysT<T>& S, XF xf,
                                                T (&acc)[R][D]) {
  constexpr int LA = G - G % D;
  constexpr int NPP = LA / D;
  const int j = lane % D;
  int32_t p0[R], nb[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    p0[r] = S.node_ptr[a[r]];
    nb[r] = S.node_ptr[a[r] + 1] - p0[r];
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int i = 0; i < D; ++i) acc[r][i] = 0;
  if (lane < LA) {
    T self[R];
#pragma unroll
    for (int r = 0; r < R; ++r) self[r] = DIFF ? xf(a[r] * D + j) : (T)0;
    int32_t maxnb = nb[0];
#pragma unroll
    for (int r = 1; r < R; ++r) maxnb = nb[r] > maxnb ? nb[r] : maxnb;
    for (int32_t k = lane / D, t = lane; k < maxnb; k += NPP, t += LA) {
      int32_t c[R];
#pragma unroll
      for (int r = 0; r < R; ++r) c[r] = k < nb[r] ? __ldg(S.nbr + p0[r] + k) : -1;
      T v[R][D];
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int i = 0; i < D; ++i)
          v[r][i] = c[r] >= 0 ? __ldg(S.vals + (int64_t)D * D * p0[r] + (int64_t)i * D * nb[r] + t) : (T)0;
      T xv[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T x = c[r] >= 0 ? xf((int64_t)c[r] * D + j) : (T)0;
        xv[r] = DIFF && c[r] >= 0 ? x - self[r] : x;
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int i = 0; i < D; ++i) acc[r][i] += v[r][i] * xv[r];
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int i = 0; i < D; ++i) acc[r][i] = group_sum<G, T>(acc[r][i]);
}

// Coarse correction of the two-level preconditioner, cluster-wide:
// rc = R^T r (one warp per aggregate, its nodes in ascending order, fixed
// butterfly), ec = A_c^-1 rc (one warp per row; FP32 inverse for the FP32
// iteration).  Every thread of the cluster calls it; r must be written.
template <int D, typename T>
__device__ void coarse_correct(Ctx& c, const gfea_batch_instance& I, const T* r, int64_t gtid, int64_t nthr) {
  constexpr int nr = Modes<D>::nr;
  const gfea_coarse_level& L = I.coarse;
  const int lane = threadIdx.x & 31;
  const int64_t gw = gtid >> 5, nw = nthr >> 5;
  const float4* off = reinterpret_cast<const float4*>(L.off);
  c.cl.sync();  // r of every node written
  for (int64_t g = gw; g < L.n_agg; g += nw) {
    T v[nr];
#pragma unroll
    for (int m = 0; m < nr; ++m) v[m] = 0;
    const int32_t k1 = L.agg_ptr[g + 1];
    for (int32_t k = L.agg_ptr[g] + lane; k < k1; k += 32) {
      const int64_t a = L.agg_nodes[k];
      T R[D][nr];
      node_modes<D, T>(off[a], I.known + a * D, R);
#pragma unroll
      for (int i = 0; i < D; ++i) {
        const T ri = ldcg(r + a * D + i);
#pragma unroll
        for (int m = 0; m < nr; ++m) v[m] += R[i][m] * ri;
      }
    }
#pragma unroll
    for (int m = 0; m < nr; ++m) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[m] += __shfl_xor_sync(0xffffffffu, v[m], o);
      if (lane == 0) L.rc[g * nr + m] = (double)v[m];
    }
  }
  c.cl.sync();  // rc complete
  const int nc = L.nc;
  for (int64_t i = gw; i < nc; i += nw) {
    T acc = 0;
    if (sizeof(T) == 4) {
      const float* row = L.inv32 + i * nc;
      for (int j = lane; j < nc; j += 32) acc += (T)__ldg(row + j) * (T)ldcg(L.rc + j);
    } else {
      const double* row = L.inv + i * nc;
      for (int j = lane; j < nc; j += 32) acc += (T)(__ldg(row + j) * ldcg(L.rc + j));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) L.ec[i] = (double)acc;
  }
  c.cl.sync();  // ec complete
}

// z = D^-1 r + R ec[agg] (masked) for the nodes of this thread; partials r.z, r.r.
template <int D, typename T>
__device__ void z_two_level(const gfea_batch_instance& I, const BatchBuf<T>& w, int64_t gtid, int64_t nthr,
                            DotAcc<T>& rz, DotAcc<T>& rr) {
  constexpr int nr = Modes<D>::nr;
  const gfea_coarse_level& L = I.coarse;
  const float4* off = reinterpret_cast<const float4*>(L.off);
  for (int64_t a = gtid; a < I.n_nodes; a += nthr) {
    T rl[D];
#pragma unroll
    for (int i = 0; i < D; ++i) rl[i] = ldcg(w.r + a * D + i);
    const int g = L.agg[a];
    T R[D][nr];
    node_modes<D, T>(off[a], I.known + a * D, R);
    T e[nr];
#pragma unroll
    for (int m = 0; m < nr; ++m) e[m] = (T)ldcg(L.ec + g * nr + m);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      T zi = 0;
#pragma unroll
      for (int j = 0; j < D; ++j) zi += w.dinv[a * D * D + i * D + j] * rl[j];
#pragma unroll
      for (int m = 0; m < nr; ++m) zi += R[i][m] * e[m];
      if (I.known[a * D + i]) zi = 0;
      w.z[a * D + i] = zi;
      rz.add_prod(rl[i], zi);
      rr.add_prod(rl[i], rl[i]);
    }
  }
}

// restart_rz with the coarse level: r = (T) r64, coarse correction, z.
template <int D, typename T>
__device__ void restart_rz_two_level(Ctx& c, const gfea_batch_instance& I, const BatchBuf<T>& w, int64_t gtid,
                                     int64_t nthr, double (&v)[2]) {
  for (int64_t a = gtid; a < I.n_nodes; a += nthr)
#pragma unroll
    for (int i = 0; i < D; ++i) w.r[a * D + i] = (T)ldcg(w.r64 + a * D + i);
  coarse_correct<D, T>(c, I, w.r, gtid, nthr);
  DotAcc<T> rz, rr;
  z_two_level<D, T>(I, w, gtid, nthr, rz, rr);
  v[0] = rz.value();
  v[1] = rr.value();
}

template <int D, int G, typename T>
__device__ void solve_instance(Ctx& c, const gfea_batch_instance& I, double delta2) {
  const int64_t Nn = I.n_nodes;
  BatchBuf<T> w;
  batch_layout<T>(Nn, D, &w, static_cast<char*>(I.work));
  const T* vals = sizeof(T) == 4 ? reinterpret_cast<const T*>(I.vals32) : reinterpret_cast<const T*>(I.vals64);
  const SysT<T> S{Nn, I.node_ptr, I.nbr, vals, I.known, I.translation_invariant};
  const SysT<double> S64{Nn, I.node_ptr, I.nbr, I.vals64, I.known, 0};
  const int tid = threadIdx.x;
  const int64_t gtid = (int64_t)c.rank * kBT + tid;
  const int64_t nthr = (int64_t)kCL * kBT;
  const int lane = tid % G;
  const int64_t grp = gtid / G, ngrp = nthr / G;
  const int64_t sub = grp % (32 / G);
  const double eps64 = 2.220446049250313e-16;
  const bool two_level = I.coarse.n_agg > 0;

  // block-Jacobi inverses (thread per node)
  double bad = 0;
  for (int64_t a = gtid; a < Nn; a += nthr) {
    const int32_t p0 = S.node_ptr[a], p1 = S.node_ptr[a + 1];
    int lo = p0, hi = p1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (S.nbr[mid] < a) lo = mid + 1; else hi = mid;
    }
    const bool has = lo < p1 && S.nbr[lo] == a;
    const int32_t W = D * (p1 - p0);
    double M[D][D], iM[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double v = has ? (double)vals[(int64_t)D * D * p0 + (int64_t)i * W + D * (lo - p0) + j] : 0.0;
        if (S.known[a * D + i] || S.known[a * D + j]) v = (i == j) ? 1.0 : 0.0;
        M[i][j] = v;
      }
    const double det = det_inv<D>(M, iM);
    if (!(fabs(det) > 0) || !isfinite(det)) {
      bad += 1;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) iM[i][j] = (i == j) ? 1.0 : 0.0;
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) w.dinv[a * D * D + i * D + j] = (T)iM[i][j];
  }

  // FP64 residual of the start
  double v4[4] = {0, 0, 0, bad}, o4[4];
  resid64<D, G>(S64, I.b, I.x, w.r64, grp, ngrp, lane, v4);
  csum<4>(c, v4, o4);
  double rr_true = o4[0];
  const double bb = o4[1];
  double floor2 = (32 * eps64) * (32 * eps64) * o4[2];
  double tol2 = fmax(I.rtol * I.rtol * bb, floor2);
  int status = GFEA_ERR_NOT_CONVERGED, iters = 0, updates = 0;
  bool finished = false;
  if (o4[3] > 0) {
    status = GFEA_ERR_SINGULAR;
    finished = true;
  } else if (!isfinite(rr_true) || !(bb == bb)) {
    status = GFEA_ERR_NAN;
    finished = true;
  } else if (bb == 0) {  // b_i - A_ic x_c = 0: the unknowns are zero
    for (int64_t a = gtid; a < Nn; a += nthr)
#pragma unroll
      for (int i = 0; i < D; ++i)
        if (!I.known[a * D + i]) I.x[a * D + i] = 0.0;
    status = GFEA_OK;
    finished = true;
  } else if (rr_true <= tol2) {
    status = GFEA_OK;
    finished = true;
  }

  if (!finished) {
    // start: r = r64, dx = 0, p = 0, z = D^-1 r
    for (int64_t a = gtid; a < Nn; a += nthr)
#pragma unroll
      for (int i = 0; i < D; ++i) {
        w.dx[a * D + i] = 0;
        w.pa[a * D + i] = 0;
      }
    double v2[2] = {0, 0}, o2[2];
    if (two_level)
      restart_rz_two_level<D, T>(c, I, w, gtid, nthr, v2);
    else
      restart_rz<D, T>(I, w, gtid, nthr, v2);
    csum<2>(c, v2, o2);
    double rz = o2[0];
    double beta = 0;
    double trigger = fmax(delta2 * rr_true, 0.25 * tol2);
    double rr_best = rr_true;
    int stall = 0;
    T* pa = w.pa;
    T* pb = w.pb;
    const bool diff = sizeof(T) == 4 && S.diff;
    for (;;) {
      // direction p' = z + beta p and Ap' (masked SpMV); partial p'.Ap'
      double va[1] = {0}, oa[1];
      DotAcc<T> pap_acc;
      const T bt = (T)beta;
      constexpr int R = 4;  // rows per group per round
      for (int64_t a0 = grp - sub; a0 < Nn; a0 += (int64_t)R * ngrp) {
        int64_t an[R], ac[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          an[r] = a0 + sub + (int64_t)r * ngrp;
          ac[r] = an[r] < Nn ? an[r] : Nn - 1;
        }
        T acc[R][D];
        auto dir = [&](int64_t cc) { return ldcg(w.z + cc) + bt * ldcg(pa + cc); };
        if (diff)
          node_rows_multi<D, G, T, true, R>(ac, lane, S, dir, acc);
        else
          node_rows_multi<D, G, T, false, R>(ac, lane, S, dir, acc);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (an[r] < Nn && lane < D) {
            T av = acc[r][0];
#pragma unroll
            for (int i = 1; i < D; ++i)
              if (lane == i) av = acc[r][i];
            const int64_t dof = an[r] * D + lane;
            const T pn = ldcg(w.z + dof) + bt * ldcg(pa + dof);
            if (S.known[dof]) av = 0;
            pb[dof] = pn;
            w.Ap[dof] = av;
            pap_acc.add_prod(pn, av);
          }
        }
      }
      va[0] = pap_acc.value();
      csum<1>(c, va, oa);
      const double pap = oa[0];
      if (!(pap > 0) || !isfinite(pap)) {
        status = isfinite(pap) ? GFEA_ERR_BREAKDOWN : GFEA_ERR_NAN;
        break;
      }
      const double alpha = rz / pap;
      // x, r, z update; partials r.z, r.r
      double vb[2] = {0, 0}, ob[2];
      DotAcc<T> rz_acc, rr_acc;
      const T al = (T)alpha;
      if (two_level) {  // x, r; then the coarse correction; then z
        for (int64_t a = gtid; a < Nn; a += nthr)
#pragma unroll
          for (int i = 0; i < D; ++i) {
            const int64_t dof = a * D + i;
            w.dx[dof] = ldcg(w.dx + dof) + al * ldcg(pb + dof);
            w.r[dof] = ldcg(w.r + dof) - al * ldcg(w.Ap + dof);
          }
        coarse_correct<D, T>(c, I, w.r, gtid, nthr);
        z_two_level<D, T>(I, w, gtid, nthr, rz_acc, rr_acc);
      } else
      for (int64_t a = gtid; a < Nn; a += nthr) {
        T rl[D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          const int64_t dof = a * D + i;
          w.dx[dof] = ldcg(w.dx + dof) + al * ldcg(pb + dof);
          rl[i] = ldcg(w.r + dof) - al * ldcg(w.Ap + dof);
          w.r[dof] = rl[i];
        }
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T zi = 0;
#pragma unroll
          for (int j = 0; j < D; ++j) zi += w.dinv[a * D * D + i * D + j] * rl[j];
          if (I.known[a * D + i]) zi = 0;
          w.z[a * D + i] = zi;
          rz_acc.add_prod(rl[i], zi);
          rr_acc.add_prod(rl[i], rl[i]);
        }
      }
      vb[0] = rz_acc.value();
      vb[1] = rr_acc.value();
      csum<2>(c, vb, ob);
      beta = ob[0] / rz;
      rz = ob[0];
      const double rr_it = ob[1];
      ++iters;
      T* t = pa;
      pa = pb;
      pb = t;
      if (!isfinite(rr_it)) {
        status = GFEA_ERR_NAN;
        break;
      }
      if (rr_it > trigger && iters < I.max_iters) continue;
      // reliable update: x += dx in FP64, then the FP64 residual replaces r
      for (int64_t a = gtid; a < Nn; a += nthr)
#pragma unroll
        for (int i = 0; i < D; ++i) {
          const int64_t dof = a * D + i;
          if (!I.known[dof]) I.x[dof] = ldcg(I.x + dof) + (double)ldcg(w.dx + dof);
          w.dx[dof] = 0;
        }
      c.cl.sync();  // the updated x of every node is visible before the residual reads neighbours
      double vr[4] = {0, 0, 0, 0}, orr[4];
      resid64<D, G>(S64, I.b, I.x, w.r64, grp, ngrp, lane, vr);
      csum<4>(c, vr, orr);
      rr_true = orr[0];
      ++updates;
      floor2 = (32 * eps64) * (32 * eps64) * orr[2];
      tol2 = fmax(I.rtol * I.rtol * bb, floor2);
      if (!isfinite(rr_true)) {
        status = GFEA_ERR_NAN;
        break;
      }
      if (rr_true <= tol2) {
        status = GFEA_OK;
        break;
      }
      if (iters >= I.max_iters) break;
      stall = rr_true > 0.9 * rr_best ? stall + 1 : 0;
      rr_best = fmin(rr_best, rr_true);
      if (stall >= 8) break;
      double vz[2] = {0, 0}, oz[2];
      if (two_level)
        restart_rz_two_level<D, T>(c, I, w, gtid, nthr, vz);
      else
        restart_rz<D, T>(I, w, gtid, nthr, vz);
      csum<2>(c, vz, oz);
      beta = oz[0] / rz;
      if (!(beta <= 1.0)) beta = 0;  // a replaced residual above the iterated one restarts
      rz = oz[0];
      trigger = fmax(delta2 * rr_true, 0.25 * tol2);
    }
  }
  if (c.rank == 0 && tid == 0) {
    gfea_pcg_result* R = I.result;
    R->status = status;
    R->iterations = iters;
    R->refinements = updates;
    R->pad = 0;
    R->rel_residual = bb > 0 ? sqrt(rr_true / bb) : 0.0;
    R->floor_rel = bb > 0 ? sqrt(floor2 / bb) : 0.0;
  }
}

template <typename T>
__device__ void dispatch(Ctx& c, const gfea_batch_instance& I, double delta2) {
  switch (I.dof_n) {
    case 1: solve_instance<1, 8, T>(c, I, delta2); break;
    case 2: solve_instance<2, 8, T>(c, I, delta2); break;
    default: solve_instance<3, 32, T>(c, I, delta2); break;
  }
}

__global__ void __cluster_dims__(kCL, 1, 1) __launch_bounds__(kBT, 2)
    batch_pcg_kernel(const gfea_batch_instance* __restrict__ insts, int n, int* next, int fp64, double delta2) {
  __shared__ double slots[8];
  __shared__ double sh[32];
  __shared__ int s_idx;
  Ctx c{cg::this_cluster(), 0, slots, sh, 0};
  c.rank = c.cl.block_rank();
  for (;;) {
    if (c.rank == 0 && threadIdx.x == 0) s_idx = atomicAdd(next, 1);
    c.cl.sync();
    const int idx = *c.cl.map_shared_rank(&s_idx, 0);
    c.cl.sync();  // rank 0's slot is read by all before it changes
    if (idx >= n) break;
    const gfea_batch_instance I = insts[idx];
    if (fp64)
      dispatch<double>(c, I, 1e-6);
    else
      dispatch<float>(c, I, delta2);
  }
}

}  // namespace
}  // namespace gfea

using namespace gfea;

extern "C" size_t gfea_batch_workspace_size(int64_t n_nodes, int dof_n, int precision) {
  if (n_nodes <= 0 || dof_n < 1 || dof_n > 3) return 0;
  return precision == GFEA_F64 ? batch_layout<double>(n_nodes, dof_n, nullptr, nullptr)
                               : batch_layout<float>(n_nodes, dof_n, nullptr, nullptr);
}

extern "C" size_t gfea_batch_scratch_size(int n_instances) {
  if (n_instances < 0) return 0;
  return a256(sizeof(int)) + a256(sizeof(gfea_batch_instance) * (size_t)n_instances);
}

extern "C" int gfea_batch_prepare(const gfea_batch_instance* inst_host, int n, void* scratch, size_t scratch_bytes,
                                  const gfea_pcg_opts* opts_host, void* stream) {
  if (!inst_host || n < 0 || !scratch || !opts_host || opts_host->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (scratch_bytes < gfea_batch_scratch_size(n)) return GFEA_ERR_WORKSPACE;
  const int prec = opts_host->precision;
  if (prec != GFEA_F64 && prec != GFEA_F32) return GFEA_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    const gfea_batch_instance& I = inst_host[i];
    if (I.version != GFEA_ABI_VERSION || I.dof_n < 1 || I.dof_n > 3 || I.n_nodes <= 0 || !I.node_ptr || !I.nbr ||
        !I.vals64 || !I.known || !I.b || !I.x || !I.work || !I.result || I.max_iters < 1 || !(I.rtol > 0))
      return GFEA_ERR_ARG;
    if (prec == GFEA_F32 && !I.vals32) return GFEA_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(I.work) & 255) != 0) return GFEA_ERR_ARG;
    const gfea_coarse_level& L = I.coarse;
    if (L.n_agg < 0) return GFEA_ERR_ARG;
    if (L.n_agg > 0) {
      const int nr = I.dof_n == 1 ? 1 : (I.dof_n == 2 ? 3 : 6);
      if (L.nr != nr || L.nc != nr * L.n_agg || L.nc > 512 || !L.agg || !L.off || !L.agg_ptr || !L.agg_nodes ||
          !L.inv || !L.inv32 || !L.rc || !L.ec)
        return GFEA_ERR_ARG;
    }
  }
  if (n == 0) return GFEA_OK;
  // largest systems first (longest-processing-time order over the clusters)
  std::vector<gfea_batch_instance> order(inst_host, inst_host + n);
  std::stable_sort(order.begin(), order.end(), [](const gfea_batch_instance& a, const gfea_batch_instance& b) {
    return a.n_pairs * a.dof_n * a.dof_n > b.n_pairs * b.dof_n * b.dof_n;
  });
  auto* desc = reinterpret_cast<gfea_batch_instance*>(static_cast<char*>(scratch) + a256(sizeof(int)));
  GFEA_CUDA_TRY(cudaMemcpyAsync(desc, order.data(), sizeof(gfea_batch_instance) * (size_t)n, cudaMemcpyHostToDevice,
                                static_cast<cudaStream_t>(stream)));
  // (a copy from pageable host memory has been staged when cudaMemcpyAsync
  // returns, so the local descriptor array may go out of scope)
  return GFEA_OK;
}

extern "C" int gfea_batch_launch(void* scratch, int n, const gfea_pcg_opts* opts_host, void* stream) {
  if (!scratch || n < 0 || !opts_host || opts_host->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  const int prec = opts_host->precision;
  if (prec != GFEA_F64 && prec != GFEA_F32) return GFEA_ERR_ARG;
  if (n == 0) return GFEA_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* next = static_cast<int*>(scratch);
  auto* desc = reinterpret_cast<gfea_batch_instance*>(static_cast<char*>(scratch) + a256(sizeof(int)));
  GFEA_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(int), s));
  // persistent clusters: enough to fill the GPU, never more than the systems
  int clusters = std::min(n, 2 * kSMs / kCL);
  if (clusters < 1) clusters = 1;
  const double d = (opts_host->inner_rtol > 0 && opts_host->inner_rtol < 1) ? opts_host->inner_rtol : 0.1;
  batch_pcg_kernel<<<clusters * kCL, kBT, 0, s>>>(desc, n, next, prec == GFEA_F64 ? 1 : 0, d * d);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

extern "C" int gfea_batch_pcg(const gfea_batch_instance* inst_host, int n, void* scratch, size_t scratch_bytes,
                              const gfea_pcg_opts* opts_host, void* stream) {
  int e = gfea_batch_prepare(inst_host, n, scratch, scratch_bytes, opts_host, stream);
  if (e) return e;
  return gfea_batch_launch(scratch, n, opts_host, stream);
}

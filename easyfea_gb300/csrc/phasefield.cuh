// Phase-field kernels: History field, damage system and degraded
// displacement stiffness, each fused with its CSR scatter; the split itself
// is in split.cuh.  phasefield.cu launches them for the 2D elements,
// phasefield3d.cu for the 3D ones.

#pragma once

#include <math.h>

#include "split.cuh"

namespace gfea {
namespace {


template <int ELEM, bool ANI>
__global__ void __launch_bounds__(128) damage_kernel(const double* __restrict__ coord, const int32_t* __restrict__ connect,
                                                     int64_t Ne, const int32_t* __restrict__ node_ptr,
                                                     const uint8_t* __restrict__ rank, const double* __restrict__ u,
                                                     PF P, const double* __restrict__ H_old, double* __restrict__ H_new,
                                                     double* __restrict__ Kd, double* __restrict__ Fd) {
  using E = Elem<ELEM>;
  constexpr int nPe = E::nPe, D = E::dim, G = NextPow2<nPe>::value, EPW = 32 / G;
  constexpr int nPgM = E::nPg_mass;
  __shared__ RefTables<ELEM, true> refm;
  __shared__ RefTables<ELEM, false> refr;
  refm.fill();
  refr.fill();
  __syncthreads();
  const int lane = threadIdx.x % G;
  const int sub = (threadIdx.x & 31) / G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool node_lane = lane < nPe;
  const double k = P.regu == GFEA_AT1 ? 3.0 / 4 * P.Gc * P.l0 : P.Gc * P.l0;
  for (int64_t e0 = warp * EPW; e0 < Ne; e0 += nwarp * EPW) {
    const int64_t e = e0 + sub;
    const bool valid = e < Ne;
    const int64_t ec = valid ? e : Ne - 1;
    const int32_t a = node_lane ? connect[ec * nPe + lane] : 0;
    double X[D], ul[D];
#pragma unroll
    for (int kk = 0; kk < D; ++kk) {
      X[kk] = node_lane ? coord[(int64_t)a * 3 + kk] : 0.0;
      ul[kk] = node_lane ? u[(int64_t)a * D + kk] : 0.0;
    }
    double acc[nPe], fp = 0;
#pragma unroll
    for (int q = 0; q < nPe; ++q) acc[q] = 0;
    for (int g = 0; g < nPgM; ++g) {
      double grad[D];
      const double wJ = lane_geo<ELEM, true, G>(refm, g, lane, node_lane, X, grad);
      double eps[D == 2 ? 3 : 6];
      group_strain<ELEM, G>(grad, ul, node_lane, eps);
      double psi = psi_plus<D, ANI>(P, eps);
      if (H_old) {
        const double ho = H_old[ec * nPgM + g];
        if (psi - ho < 0) psi = ho;
      }
      if (valid && lane == 0) H_new[ec * nPgM + g] = psi;
      double r, f;
      if (P.regu == GFEA_AT1) {
        r = 2 * psi;
        f = 2 * psi - (3 * P.Gc) / (8 * P.l0);
        f = (f + fabs(f)) / 2;
      } else {
        r = 2 * psi + P.Gc / P.l0;
        f = 2 * psi;
      }
      const double np = node_lane ? refm.N[g][lane] : 0.0;
#pragma unroll
      for (int q = 0; q < nPe; ++q) acc[q] += r * wJ * np * refm.N[g][q];
      fp += f * wJ * np;
    }
    for (int g = 0; g < RefTables<ELEM, false>::nPg; ++g) {
      double grad[D];
      const double wJ = lane_geo<ELEM, false, G>(refr, g, lane, node_lane, X, grad);
      double Ag[D];
#pragma unroll
      for (int i = 0; i < D; ++i) {
        Ag[i] = 0;
#pragma unroll
        for (int j = 0; j < D; ++j) Ag[i] += P.A[i * D + j] * grad[j];
      }
#pragma unroll
      for (int q = 0; q < nPe; ++q) {
        double s = 0;
#pragma unroll
        for (int i = 0; i < D; ++i) s += group_bcast<G, double>(grad[i], q) * Ag[i];
        acc[q] += k * wJ * s;
      }
    }
    if (valid && node_lane) {
      const int32_t p0 = node_ptr[a];
      const uint8_t* rk = rank + (ec * nPe + lane) * nPe;
#pragma unroll
      for (int q = 0; q < nPe; ++q) atomicAdd(Kd + p0 + rk[q], P.thickness * acc[q]);
      atomicAdd(Fd + a, P.thickness * fp);
    }
  }
}

template <int ELEM, typename T, bool ANI>
__global__ void __launch_bounds__(128) pf_elastic_kernel(const double* __restrict__ coord,
                                                         const int32_t* __restrict__ connect, int64_t Ne,
                                                         const int32_t* __restrict__ node_ptr,
                                                         const uint8_t* __restrict__ rank, const double* __restrict__ u,
                                                         const double* __restrict__ dmg, PF P, T* __restrict__ vals) {
  using E = Elem<ELEM>;
  constexpr int nPe = E::nPe, D = E::dim, G = NextPow2<nPe>::value, EPW = 32 / G, NS = D == 2 ? 3 : 6;
  __shared__ RefTables<ELEM, false> ref;
  ref.fill();
  __syncthreads();
  const int lane = threadIdx.x % G;
  const int sub = (threadIdx.x & 31) / G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool node_lane = lane < nPe;
  const double cK = 1.0 / kSqrt2;
  for (int64_t e0 = warp * EPW; e0 < Ne; e0 += nwarp * EPW) {
    const int64_t e = e0 + sub;
    const bool valid = e < Ne;
    const int64_t ec = valid ? e : Ne - 1;
    const int32_t a = node_lane ? connect[ec * nPe + lane] : 0;
    double X[D], ul[D];
#pragma unroll
    for (int kk = 0; kk < D; ++kk) {
      X[kk] = node_lane ? coord[(int64_t)a * 3 + kk] : 0.0;
      ul[kk] = node_lane ? u[(int64_t)a * D + kk] : 0.0;
    }
    const double dl = node_lane ? dmg[a] : 0.0;
    double acc[nPe][D][D];
#pragma unroll
    for (int q = 0; q < nPe; ++q)
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) acc[q][i][j] = 0;
    for (int g = 0; g < RefTables<ELEM, false>::nPg; ++g) {
      double grad[D];
      const double wJ = lane_geo<ELEM, false, G>(ref, g, lane, node_lane, X, grad);
      double eps[NS];
      group_strain<ELEM, G>(grad, ul, node_lane, eps);
      const double dpg = group_sum<G, double>(node_lane ? ref.N[g][lane] * dl : 0.0);
      const double gd = (1 - dpg) * (1 - dpg) + P.k_res;
      double c[NS * NS];
      split_c<D, ANI>(P, eps, gd, c, nullptr, nullptr);
      // BtC and accumulation as in the elastic kernel (KM B of _group_elem.py:1242-1312)
      double BtC[D][NS];
      if constexpr (D == 2) {
        for (int s = 0; s < 3; ++s) {
          BtC[0][s] = wJ * (grad[0] * c[0 * 3 + s] + cK * grad[1] * c[2 * 3 + s]);
          BtC[1][s] = wJ * (grad[1] * c[1 * 3 + s] + cK * grad[0] * c[2 * 3 + s]);
        }
      } else {
        for (int s = 0; s < 6; ++s) {
          BtC[0][s] = wJ * (grad[0] * c[0 * 6 + s] + cK * (grad[2] * c[4 * 6 + s] + grad[1] * c[5 * 6 + s]));
          BtC[1][s] = wJ * (grad[1] * c[1 * 6 + s] + cK * (grad[2] * c[3 * 6 + s] + grad[0] * c[5 * 6 + s]));
          BtC[2][s] = wJ * (grad[2] * c[2 * 6 + s] + cK * (grad[1] * c[3 * 6 + s] + grad[0] * c[4 * 6 + s]));
        }
      }
#pragma unroll
      for (int q = 0; q < nPe; ++q) {
        double h[D];
#pragma unroll
        for (int kk = 0; kk < D; ++kk) h[kk] = group_bcast<G, double>(grad[kk], q);
        if constexpr (D == 2) {
          const double chx = cK * h[0], chy = cK * h[1];
          for (int i = 0; i < 2; ++i) {
            acc[q][i][0] += BtC[i][0] * h[0] + BtC[i][2] * chy;
            acc[q][i][1] += BtC[i][1] * h[1] + BtC[i][2] * chx;
          }
        } else {
          const double chx = cK * h[0], chy = cK * h[1], chz = cK * h[2];
          for (int i = 0; i < 3; ++i) {
            acc[q][i][0] += BtC[i][0] * h[0] + BtC[i][4] * chz + BtC[i][5] * chy;
            acc[q][i][1] += BtC[i][1] * h[1] + BtC[i][3] * chz + BtC[i][5] * chx;
            acc[q][i][2] += BtC[i][2] * h[2] + BtC[i][3] * chy + BtC[i][4] * chx;
          }
        }
      }
    }
    if (valid && node_lane) {
      const int32_t p0 = node_ptr[a];
      const int32_t nb = node_ptr[a + 1] - p0;
      const uint8_t* rk = rank + (ec * nPe + lane) * nPe;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        T* row = vals + (int64_t)D * D * p0 + (int64_t)i * D * nb;
#pragma unroll
        for (int q = 0; q < nPe; ++q) {
          const int r = rk[q];
#pragma unroll
          for (int j = 0; j < D; ++j) atomicAdd(row + D * r + j, (T)(P.thickness * acc[q][i][j]));
        }
      }
    }
  }
}

template <int D, bool ANI>
__global__ void split_kernel(const double* __restrict__ eps, int64_t n, PF P, double* cP, double* cM, double* psiP,
                             double* psiM) {
  constexpr int ns = D == 2 ? 3 : 6;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double e[ns], c[ns * ns], p[ns * ns], m[ns * ns];
    for (int k = 0; k < ns; ++k) e[k] = eps[i * ns + k];
    split_c<D, ANI>(P, e, 1.0, c, p, m);
    double sp = 0, sm = 0;
    for (int a = 0; a < ns; ++a) {
      double tp = 0, tm = 0;
      for (int b = 0; b < ns; ++b) {
        tp += p[a * ns + b] * e[b];
        tm += m[a * ns + b] * e[b];
      }
      sp += 0.5 * e[a] * tp;
      sm += 0.5 * e[a] * tm;
    }
    if (cP) for (int k = 0; k < ns * ns; ++k) cP[i * ns * ns + k] = p[k];
    if (cM) for (int k = 0; k < ns * ns; ++k) cM[i * ns * ns + k] = m[k];
    if (psiP) psiP[i] = sp;
    if (psiM) psiM[i] = sm;
  }
}

int to_pf(const gfea_pf_params* p, PF* o) {
  if (!p || p->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (p->dim != 2 && p->dim != 3) return GFEA_ERR_ARG;
  if (p->split < GFEA_SPLIT_BOURDIN || p->split > GFEA_SPLIT_ANISOT_STRESS_NOCROSS) return GFEA_ERR_ARG;
  if (p->regularization != GFEA_AT1 && p->regularization != GFEA_AT2) return GFEA_ERR_ARG;
  o->split = p->split;
  o->plane_stress = p->plane_stress;
  o->regu = p->regularization;
  o->dim = p->dim;
  o->lambda = p->lambda_;
  o->mu = p->mu;
  o->Gc = p->Gc;
  o->l0 = p->l0;
  o->thickness = p->thickness;
  o->k_res = p->k_res;
  for (int i = 0; i < 9; ++i) o->A[i] = p->A[i];
  for (int i = 0; i < 36; ++i) o->C[i] = p->C[i];
  for (int i = 0; i < 36; ++i) o->S[i] = p->S[i];
  return GFEA_OK;
}

template <int ELEM>
int launch_damage(const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                  const uint8_t* rank, const double* u, const PF& P, const double* H_old, double* H_new, double* Kd,
                  double* Fd, cudaStream_t s) {
  constexpr int G = NextPow2<Elem<ELEM>::nPe>::value;
  int blocks = grid_for(ceil_div(Ne, 32 / G) * 32, 128);
  if (blocks > kSMs * 64) blocks = kSMs * 64;
  if (pf_anisot(P.split))
    damage_kernel<ELEM, true><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd);
  else
    damage_kernel<ELEM, false><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, u, P, H_old, H_new, Kd, Fd);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <int ELEM, typename T>
int launch_pfel(const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr, const uint8_t* rank,
                const double* u, const double* d, const PF& P, T* vals, cudaStream_t s) {
  constexpr int G = NextPow2<Elem<ELEM>::nPe>::value;
  int blocks = grid_for(ceil_div(Ne, 32 / G) * 32, 128);
  if (blocks > kSMs * 64) blocks = kSMs * 64;
  if (pf_anisot(P.split))
    pf_elastic_kernel<ELEM, T, true><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, u, d, P, vals);
  else
    pf_elastic_kernel<ELEM, T, false><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, u, d, P, vals);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

}  // namespace

// the 3D elements' launches (phasefield3d.cu)
int pf_damage_3d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                 const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                 double* H_new, double* Kd, double* Fd, cudaStream_t s);
int pf_elastic_3d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                  const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                  int value_type, void* values, cudaStream_t s);
// TRI10, TRI15 (through phasefield_ho2d.cu), PRISM6, PRISM15 and PRISM18 (phasefield_ho.cu)
int pf_damage_ho(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                 const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                 double* H_new, double* Kd, double* Fd, cudaStream_t s);
int pf_elastic_ho(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                  const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                  int value_type, void* values, cudaStream_t s);
// TRI10 and TRI15 (phasefield_ho2d.cu)
int pf_damage_ho2d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                   const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                   double* H_new, double* Kd, double* Fd, cudaStream_t s);
int pf_elastic_ho2d(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                    const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                    int value_type, void* values, cudaStream_t s);
// HEXA20 and HEXA27 (phasefield_hexq.cu)
int pf_damage_hexq(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                   const uint8_t* rank, const double* u, const gfea_pf_params* params, const double* H_old,
                   double* H_new, double* Kd, double* Fd, cudaStream_t s);
int pf_elastic_hexq(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                    const uint8_t* rank, const double* u, const double* d, const gfea_pf_params* params,
                    int value_type, void* values, cudaStream_t s);

}  // namespace gfea

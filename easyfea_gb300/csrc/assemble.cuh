// Element kernels of the stiffness and mass assembly, their launch
// templates and the surface loads, shared by assemble.cu and assemble_ho.cu.
//
// Element operators at Gauss points fused with the CSR scatter.
//
// One group of G = next_pow2(nPe) lanes per element; lane p owns local node p:
// it loads that node's coordinates, contributes dN_p (x) X_p to the Jacobian
// (reduced across the group with shuffles), computes its physical gradient
// invF.dN_p, and accumulates the blocks K_pq of half of the element matrix
// (q = p .. p + nPe/2 mod nPe; gradients of the other nodes arrive by
// shuffle).  Each block is scattered into row p and, transposed, into row q,
// with one atomic add per entry at slot
//   dof_n^2 node_ptr[a] + i dof_n nnb(a) + dof_n rank[e,p,q] + j.
// Element matrices never touch global memory.
#pragma once

#include "common.cuh"
#include "element.cuh"
#include "tune.cuh"

namespace gfea {
namespace {

// Per-lane geometry at one Gauss point: Jacobian reduced across the group,
// wJ and the physical gradient of this lane's shape function.
// Reciprocal by Newton-Raphson iteration on f(r) = 1/r - x (r <- r + r (1 - x r))
// from an FP32 seed (relative error ~2^-23): two steps reach double precision
// with four FP64 FMAs; the full division where the seed is out of FP32 range.
__device__ __forceinline__ double recip_newton(double x) {
  const float s = 1.0f / (float)x;
  if (!(fabsf(s) > 0.f) || isinf(s)) return 1.0 / x;
  double r = (double)s;
  r = fma(r, fma(-x, r, 1.0), r);
  r = fma(r, fma(-x, r, 1.0), r);
  return r;
}

// Sum of nine per-lane values over a group of 8 lanes (the 3x3 Jacobian of a
// HEXA8): a reduce-scatter in three exchange steps -- each lane keeps the
// values owned by its half (value v owned by lane v, value 8 by lane 0) and
// adds the partner's copies -- then broadcasts from the owners: 10 FP64 adds
// instead of the butterfly's 27 (FP64 adds, not lanes, cost time on GB300).
__device__ __forceinline__ void group8_sum9(const double (&v)[9], double (&F)[9], int lane) {
  const bool b = lane & 4, c = lane & 2, e = lane & 1;
  double k1[5], k2[3], k3[2];
  {
    const double L[5] = {v[0], v[1], v[2], v[3], v[8]}, U[5] = {v[4], v[5], v[6], v[7], 0.0};
#pragma unroll
    for (int m = 0; m < 5; ++m) k1[m] = (b ? U[m] : L[m]) + __shfl_xor_sync(0xffffffffu, b ? L[m] : U[m], 4, 8);
  }
  {
    const double L[3] = {k1[0], k1[1], k1[4]}, U[3] = {k1[2], k1[3], 0.0};
#pragma unroll
    for (int m = 0; m < 3; ++m) k2[m] = (c ? U[m] : L[m]) + __shfl_xor_sync(0xffffffffu, c ? L[m] : U[m], 2, 8);
  }
  {
    const double L[2] = {k2[0], k2[2]}, U[2] = {k2[1], 0.0};
#pragma unroll
    for (int m = 0; m < 2; ++m) k3[m] = (e ? U[m] : L[m]) + __shfl_xor_sync(0xffffffffu, e ? L[m] : U[m], 1, 8);
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) F[i] = __shfl_sync(0xffffffffu, k3[0], i, 8);
  F[8] = __shfl_sync(0xffffffffu, k3[1], 0, 8);
}

// FP32 values: the whole geometry on the FP32 pipe, from coordinates taken
// relative to the element's first node (so the Jacobian's entries keep
// FP32 precision however far the element is from the origin): F by group
// sums of dN_p (x) X_p, det and adjugate in FP32, one FP32 division.
template <int D, int G>
__device__ __forceinline__ float lane_geometry_f32(const float (&dn)[D], const float (&X)[D], float w,
                                                   float (&grad)[D]) {
  float F[D][D];
#pragma unroll
  for (int d = 0; d < D; ++d)
#pragma unroll
    for (int k = 0; k < D; ++k) F[d][k] = group_sum<G, float>(dn[d] * X[k]);
  if constexpr (D == 2) {
    const float det = F[0][0] * F[1][1] - F[1][0] * F[0][1];
    const float id = 1.0f / det;
    grad[0] = id * (F[1][1] * dn[0] - F[0][1] * dn[1]);
    grad[1] = id * (-F[1][0] * dn[0] + F[0][0] * dn[1]);
    return fabsf(det) * w;
  } else {
    const float a11 = F[0][0], a12 = F[0][1], a13 = F[0][2], a21 = F[1][0], a22 = F[1][1], a23 = F[1][2],
                a31 = F[2][0], a32 = F[2][1], a33 = F[2][2];
    const float c11 = a22 * a33 - a32 * a23, c21 = -(a21 * a33 - a31 * a23), c31 = a21 * a32 - a31 * a22;
    const float det = a11 * c11 + a12 * c21 + a13 * c31;
    const float id = 1.0f / det;
    const float adj[3][3] = {{c11, -(a12 * a33 - a32 * a13), a12 * a23 - a22 * a13},
                             {c21, a11 * a33 - a31 * a13, -(a11 * a23 - a21 * a13)},
                             {c31, -(a11 * a32 - a31 * a12), a11 * a22 - a21 * a12}};
#pragma unroll
    for (int i = 0; i < 3; ++i) grad[i] = id * (adj[i][0] * dn[0] + adj[i][1] * dn[1] + adj[i][2] * dn[2]);
    return fabsf(det) * w;
  }
}

template <int ELEM, bool MASS, int G, typename R>
__device__ __forceinline__ R lane_geometry(const RefTables<ELEM, MASS>& ref, int g, int lane, bool node_lane,
                                           const R (&X)[Elem<ELEM>::dim], R (&grad)[Elem<ELEM>::dim]) {
  constexpr int D = Elem<ELEM>::dim;
  if constexpr (sizeof(R) == 4 && D >= 2) {
    float dn[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dn[d] = node_lane ? (float)ref.dN[g][d][lane] : 0.f;
    float Xf[D];
#pragma unroll
    for (int k = 0; k < D; ++k) Xf[k] = (float)X[k];
    float gf[D];
    const float wJ = lane_geometry_f32<D, G>(dn, Xf, (float)ref.w[g], gf);
#pragma unroll
    for (int k = 0; k < D; ++k) grad[k] = (R)gf[k];
    return (R)wJ;
  } else if constexpr (D == 3 && G == 8) {
    // F[d][k] = sum_p dN_d(p) X_p[k]; grad = F^-1 dN = adj(F) dN / det(F)
    double dn[3], v[9], F[9];
#pragma unroll
    for (int d = 0; d < 3; ++d) dn[d] = node_lane ? (double)ref.dN[g][d][lane] : 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int k = 0; k < 3; ++k) v[d * 3 + k] = dn[d] * (double)X[k];
    group8_sum9(v, F, lane);
    const double a11 = F[0], a12 = F[1], a13 = F[2], a21 = F[3], a22 = F[4], a23 = F[5], a31 = F[6], a32 = F[7],
                 a33 = F[8];
    const double c11 = a22 * a33 - a32 * a23, c21 = -(a21 * a33 - a31 * a23), c31 = a21 * a32 - a31 * a22;
    const double det = a11 * c11 + a12 * c21 + a13 * c31;
    const double id = recip_newton(det);
    const double adj[3][3] = {{c11, -(a12 * a33 - a32 * a13), a12 * a23 - a22 * a13},
                              {c21, a11 * a33 - a31 * a13, -(a11 * a23 - a21 * a13)},
                              {c31, -(a11 * a32 - a31 * a12), a11 * a22 - a21 * a12}};
#pragma unroll
    for (int i = 0; i < 3; ++i) grad[i] = (R)(id * (adj[i][0] * dn[0] + adj[i][1] * dn[1] + adj[i][2] * dn[2]));
    return (R)(fabs(det) * ref.w[g]);
  } else {
    double F[D][D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const R dn = node_lane ? (R)ref.dN[g][d][lane] : (R)0;
#pragma unroll
      for (int k = 0; k < D; ++k) F[d][k] = (double)group_sum<G, R>(dn * X[k]);
    }
    double iF[D][D];
    const double det = det_inv<D>(F, iF);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double v = 0;
#pragma unroll
      for (int d = 0; d < D; ++d) v += iF[i][d] * (node_lane ? ref.dN[g][d][lane] : 0.0);
      grad[i] = (R)v;
    }
    return (R)(fabs(det) * ref.w[g]);
  }
}

template <int ELEM, typename T, typename R, int CMODE>
__global__ void __launch_bounds__(128) elastic_kernel(const double* __restrict__ coord,
                                                      const int32_t* __restrict__ connect, int64_t Ne,
                                                      const int32_t* __restrict__ node_ptr,
                                                      const uint8_t* __restrict__ rank,
                                                      const double* __restrict__ Cglob, double factor,
                                                      T* __restrict__ vals) {
  using E = Elem<ELEM>;
  constexpr int nPe = E::nPe, D = E::dim, G = NextPow2<nPe>::value, NS = D == 2 ? 3 : 6;
  constexpr int EPW = 32 / G;  // elements per warp
  // modes 3, 4: isotropic law given by (lambda, mu): K_pq = lambda M + mu M^T
  // + mu tr(M) I with M = sum_g wJ grad N_p (x) grad N_q -- the same matrix as
  // B^T C B for C = lambda 1 (x) 1 + 2 mu I (Kelvin-Mandel), with D^2 FMAs per
  // block and Gauss point instead of B^T C (D x NS x 3) plus B^T C B
  constexpr bool ISO = CMODE == 3 || CMODE == 4;
  __shared__ RefTables<ELEM, false> ref;
  __shared__ R Csh[NS * NS];
  ref.fill();
  if (CMODE == 0 || CMODE == 2)  // homogeneous C, or the reference C of mode 2
    for (int i = threadIdx.x; i < NS * NS; i += blockDim.x) Csh[i] = (R)Cglob[i];
  __syncthreads();
  const R lam = ISO ? (R)Cglob[0] : (R)0, mu = ISO ? (R)Cglob[1] : (R)0;

  const int lane = threadIdx.x % G;
  const int sub = (threadIdx.x & 31) / G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool node_lane = lane < nPe;

  for (int64_t e0 = warp * EPW; e0 < Ne; e0 += nwarp * EPW) {
    const int64_t e = e0 + sub;
    const bool valid = e < Ne;
    const int64_t ec = valid ? e : Ne - 1;
    const bool act = valid && node_lane;
    const int32_t a = node_lane ? connect[ec * nPe + lane] : 0;
    R X[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const double xa = node_lane ? coord[(int64_t)a * 3 + k] : 0.0;
      // FP32 values: coordinates relative to the element's first node
      const double x0 = sizeof(R) == 4 ? group_bcast<G, double>(xa, 0) : 0.0;
      X[k] = node_lane ? (R)(xa - x0) : (R)0;
    }
    R Cl[NS * NS];
    const R* C = Csh;
    if (CMODE == 1) {
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) Cl[i] = (R)__ldg(Cglob + ec * NS * NS + i);
      C = Cl;
    }
    // K_e is symmetric: lane p computes the blocks K_pq for q = p + d (mod nPe),
    // d = 0 .. nPe/2 (the opposite pair of an even nPe only on lanes p < nPe/2),
    // which covers every unordered pair once; each block is scattered into
    // row p and, transposed, into row q
    constexpr int NB = nPe / 2 + 1;
    const bool extra = (nPe % 2 == 1) || lane < nPe / 2;  // lane owns d = nPe/2 (odd nPe: always)
    R acc[NB][D][D];
#pragma unroll
    for (int d = 0; d < NB; ++d)
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) acc[d][i][j] = 0;

    for (int g = 0; g < RefTables<ELEM, false>::nPg; ++g) {
      R grad[D];
      const R wJ = lane_geometry<ELEM, false, G, R>(ref, g, lane, node_lane, X, grad);
      if constexpr (ISO) {
        R wa[D];
#pragma unroll
        for (int k = 0; k < D; ++k) wa[k] = wJ * grad[k];
#pragma unroll
        for (int d = 0; d < NB; ++d) {
          const int q = node_lane ? (lane + d) % nPe : 0;
          R h[D];
#pragma unroll
          for (int k = 0; k < D; ++k) h[k] = group_bcast<G, R>(grad[k], q);
          if (d < NB - 1 || extra) {
#pragma unroll
            for (int i = 0; i < D; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) acc[d][i][j] += wa[i] * h[j];
          }
        }
      } else {
        R BtC[D][NS];
        btc<D, R>(grad, C, wJ, BtC);
#pragma unroll
        for (int d = 0; d < NB; ++d) {
          const int q = node_lane ? (lane + d) % nPe : 0;
          R h[D];
#pragma unroll
          for (int k = 0; k < D; ++k) h[k] = group_bcast<G, R>(grad[k], q);
          if (d < NB - 1 || extra) btcb<D, R>(BtC, h, acc[d]);
        }
      }
    }
    if constexpr (ISO) {
#pragma unroll
      for (int d = 0; d < NB; ++d) {
        R tr = 0;
#pragma unroll
        for (int i = 0; i < D; ++i) tr += acc[d][i][i];
        R K[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) K[i][j] = lam * acc[d][i][j] + mu * acc[d][j][i] + (i == j ? mu * tr : (R)0);
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) acc[d][i][j] = K[i][j];
      }
    }
    if (act) {
      // modes 2, 4: per-element factor of the reference law (e.g. a per-element Young's modulus)
      const double f = CMODE == 2   ? factor * __ldg(Cglob + NS * NS + ec)
                       : CMODE == 4 ? factor * __ldg(Cglob + 2 + ec)
                                    : factor;
      const int32_t* ce = connect + ec * nPe;
      const uint8_t* rke = rank + ec * nPe * nPe;
      const int32_t pa0 = node_ptr[a];
      const int32_t nba = node_ptr[a + 1] - pa0;
#pragma unroll
      for (int d = 0; d < NB; ++d) {
        if (d == NB - 1 && !extra) continue;
        const int q = (lane + d) % nPe;
        // row p (node a), block q
        const int r_pq = rke[lane * nPe + q];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T* row = vals + (int64_t)D * D * pa0 + (int64_t)i * D * nba + D * r_pq;
#pragma unroll
          for (int j = 0; j < D; ++j) atomic_add_t<T>(row + j, (T)(f * (double)acc[d][i][j]));
        }
        if (d == 0) continue;
        // row q (node b), block p: the transpose
        const int32_t b = ce[q];
        const int32_t pb0 = node_ptr[b];
        const int32_t nbb = node_ptr[b + 1] - pb0;
        const int r_qp = rke[q * nPe + lane];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T* row = vals + (int64_t)D * D * pb0 + (int64_t)i * D * nbb + D * r_qp;
#pragma unroll
          for (int j = 0; j < D; ++j) atomic_add_t<T>(row + j, (T)(f * (double)acc[d][j][i]));
        }
      }
    }
  }
}

template <int ELEM, typename T, typename R>
__global__ void __launch_bounds__(128) mass_kernel(const double* __restrict__ coord,
                                                   const int32_t* __restrict__ connect, int64_t Ne,
                                                   const int32_t* __restrict__ node_ptr,
                                                   const uint8_t* __restrict__ rank, int dof_n, double rho,
                                                   double factor, T* __restrict__ vals) {
  using E = Elem<ELEM>;
  constexpr int nPe = E::nPe, D = E::dim, G = NextPow2<nPe>::value;
  constexpr int EPW = 32 / G;
  __shared__ RefTables<ELEM, true> ref;
  ref.fill();
  __syncthreads();
  const int lane = threadIdx.x % G;
  const int sub = (threadIdx.x & 31) / G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool node_lane = lane < nPe;
  for (int64_t e0 = warp * EPW; e0 < Ne; e0 += nwarp * EPW) {
    const int64_t e = e0 + sub;
    const bool valid = e < Ne;
    const int64_t ec = valid ? e : Ne - 1;
    const int32_t a = node_lane ? connect[ec * nPe + lane] : 0;
    R X[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const double xa = node_lane ? coord[(int64_t)a * 3 + k] : 0.0;
      // FP32 values: coordinates relative to the element's first node
      const double x0 = sizeof(R) == 4 ? group_bcast<G, double>(xa, 0) : 0.0;
      X[k] = node_lane ? (R)(xa - x0) : (R)0;
    }
    R acc[nPe];
#pragma unroll
    for (int q = 0; q < nPe; ++q) acc[q] = 0;
    for (int g = 0; g < RefTables<ELEM, true>::nPg; ++g) {
      R grad[D];
      const R wJ = lane_geometry<ELEM, true, G, R>(ref, g, lane, node_lane, X, grad);
      const R np = node_lane ? (R)ref.N[g][lane] : (R)0;
#pragma unroll
      for (int q = 0; q < nPe; ++q) acc[q] += wJ * np * (R)ref.N[g][q];
    }
    if (valid && node_lane) {
      const int32_t p0 = node_ptr[a];
      const int32_t nb = node_ptr[a + 1] - p0;
      const uint8_t* rk = rank + (ec * nPe + lane) * nPe;
      for (int i = 0; i < dof_n; ++i) {
        T* row = vals + (int64_t)dof_n * dof_n * p0 + (int64_t)i * dof_n * nb;
#pragma unroll
        for (int q = 0; q < nPe; ++q) atomic_add_t<T>(row + dof_n * rk[q] + i, (T)(factor * rho * (double)acc[q]));
      }
    }
  }
}

// Up to four traction components, passed by value to the surface kernel.
struct Traction4 {
  double x, y, z, w;
};

// Boundary (line / face) integration of constant tractions.
template <int BELEM>
__global__ void surface_load_kernel(const double* __restrict__ coord, const int32_t* __restrict__ bconnect,
                                    int64_t Nbe, const uint8_t* __restrict__ mask, int dof_n, int nu,
                                    int4 uidx, Traction4 uval, double factor, double* __restrict__ b) {
  using E = Elem<BELEM>;
  constexpr int nPe = E::nPe, BD = E::dim;
  __shared__ RefTables<BELEM, true> ref;
  ref.fill();
  __syncthreads();
  const int ui[4] = {uidx.x, uidx.y, uidx.z, uidx.w};
  const double uv[4] = {uval.x, uval.y, uval.z, uval.w};
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < Nbe; e += (int64_t)gridDim.x * blockDim.x) {
    int32_t nd[nPe];
    bool all = true;
    for (int p = 0; p < nPe; ++p) {
      nd[p] = bconnect[e * nPe + p];
      all = all && mask[nd[p]];
    }
    if (!all) continue;
    double Nw[nPe];
    for (int p = 0; p < nPe; ++p) Nw[p] = 0;
    for (int g = 0; g < RefTables<BELEM, true>::nPg; ++g) {
      double T[BD][3];
      for (int d = 0; d < BD; ++d)
        for (int k = 0; k < 3; ++k) {
          double s = 0;
          for (int n = 0; n < nPe; ++n) s += ref.dN[g][d][n] * coord[(int64_t)nd[n] * 3 + k];
          T[d][k] = s;
        }
      double J;
      if (BD == 1) {
        J = sqrt(T[0][0] * T[0][0] + T[0][1] * T[0][1] + T[0][2] * T[0][2]);
      } else {
        const double cx = T[0][1] * T[BD - 1][2] - T[0][2] * T[BD - 1][1];
        const double cy = T[0][2] * T[BD - 1][0] - T[0][0] * T[BD - 1][2];
        const double cz = T[0][0] * T[BD - 1][1] - T[0][1] * T[BD - 1][0];
        J = sqrt(cx * cx + cy * cy + cz * cz);
      }
      const double wJ = J * ref.w[g];
      for (int p = 0; p < nPe; ++p) Nw[p] += wJ * ref.N[g][p];
    }
    for (int u = 0; u < nu; ++u)
      for (int p = 0; p < nPe; ++p) atomicAdd(&b[(int64_t)nd[p] * dof_n + ui[u]], factor * uv[u] * Nw[p]);
  }
}

// Jacobian measure of a boundary element at Gauss point g (length of the
// tangent in 1D, norm of the cross product of the two tangents in 2D).
template <int BELEM>
__device__ double boundary_wj(const RefTables<BELEM, true>& ref, const double* __restrict__ coord,
                              const int32_t (&nd)[Elem<BELEM>::nPe], int g) {
  constexpr int nPe = Elem<BELEM>::nPe, BD = Elem<BELEM>::dim;
  double T[BD][3];
  for (int d = 0; d < BD; ++d)
    for (int k = 0; k < 3; ++k) {
      double s = 0;
      for (int n = 0; n < nPe; ++n) s += ref.dN[g][d][n] * coord[(int64_t)nd[n] * 3 + k];
      T[d][k] = s;
    }
  double J;
  if (BD == 1) {
    J = sqrt(T[0][0] * T[0][0] + T[0][1] * T[0][1] + T[0][2] * T[0][2]);
  } else {
    const double cx = T[0][1] * T[BD - 1][2] - T[0][2] * T[BD - 1][1];
    const double cy = T[0][2] * T[BD - 1][0] - T[0][0] * T[BD - 1][2];
    const double cz = T[0][0] * T[BD - 1][1] - T[0][1] * T[BD - 1][0];
    J = sqrt(cx * cx + cy * cy + cz * cz);
  }
  return J * ref.w[g];
}

// Coordinates of the mass Gauss points of boundary elements: xyz[(e nPg + g) 3 + k].
template <int BELEM>
__global__ void boundary_gauss_kernel(const double* __restrict__ coord, const int32_t* __restrict__ bconnect,
                                      int64_t Nbe, double* __restrict__ xyz) {
  using E = Elem<BELEM>;
  constexpr int nPe = E::nPe;
  constexpr int nPg = RefTables<BELEM, true>::nPg;
  __shared__ RefTables<BELEM, true> ref;
  ref.fill();
  __syncthreads();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < Nbe; e += (int64_t)gridDim.x * blockDim.x) {
    int32_t nd[nPe];
    for (int p = 0; p < nPe; ++p) nd[p] = bconnect[e * nPe + p];
    for (int g = 0; g < nPg; ++g)
      for (int k = 0; k < 3; ++k) {
        double s = 0;
        for (int n = 0; n < nPe; ++n) s += ref.N[g][n] * coord[(int64_t)nd[n] * 3 + k];
        xyz[((int64_t)e * nPg + g) * 3 + k] = s;
      }
  }
}

// Neumann load of one unknown with values varying over the boundary, on the
// elements whose every node has mask set: mode 0, values at the mass Gauss
// points (values[e nPg + g]): b_p += factor sum_g wJ f_g N_p(g); mode 1,
// values per node: b_p += factor f_p sum_g wJ N_p(g).
template <int BELEM>
__global__ void surface_load_field_kernel(const double* __restrict__ coord, const int32_t* __restrict__ bconnect,
                                          int64_t Nbe, const uint8_t* __restrict__ mask, int dof_n, int ui, int mode,
                                          const double* __restrict__ vals, double factor, double* __restrict__ b) {
  using E = Elem<BELEM>;
  constexpr int nPe = E::nPe;
  constexpr int nPg = RefTables<BELEM, true>::nPg;
  __shared__ RefTables<BELEM, true> ref;
  ref.fill();
  __syncthreads();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < Nbe; e += (int64_t)gridDim.x * blockDim.x) {
    int32_t nd[nPe];
    bool all = true;
    for (int p = 0; p < nPe; ++p) {
      nd[p] = bconnect[e * nPe + p];
      all = all && mask[nd[p]];
    }
    if (!all) continue;
    double acc[nPe];
    for (int p = 0; p < nPe; ++p) acc[p] = 0;
    for (int g = 0; g < nPg; ++g) {
      const double wJ = boundary_wj<BELEM>(ref, coord, nd, g);
      const double fg = mode == 0 ? vals[e * nPg + g] : 1.0;
      for (int p = 0; p < nPe; ++p) acc[p] += wJ * fg * ref.N[g][p];
    }
    for (int p = 0; p < nPe; ++p) {
      const double f = mode == 0 ? 1.0 : vals[nd[p]];
      atomicAdd(&b[(int64_t)nd[p] * dof_n + ui], factor * f * acc[p]);
    }
  }
}

int64_t assemble_key(int elem, int value_type, int cpe, int64_t Ne) {
  return tune_key(kTuneAssemble, elem, value_type, cpe, tune_log2((double)Ne));
}

// Element tile schedule: the grid is capped at per_sm blocks of 128 threads
// per SM (each block then strides over its elements); per_sm = 0 takes the
// autotuner's decision for this class, else 64.
template <int ELEM, typename T, typename R>
int launch_elastic(const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                   const uint8_t* rank, const double* C, int cpe, double factor, T* vals, cudaStream_t s,
                   int per_sm = 0) {
  constexpr int G = NextPow2<Elem<ELEM>::nPe>::value;
  if (per_sm <= 0) {
    int32_t tuned = 0;
    per_sm = tune_get(assemble_key(ELEM, sizeof(T) == 4 ? GFEA_F32 : GFEA_F64, cpe, Ne), &tuned) ? tuned : 64;
  }
  const int64_t warps = ceil_div(Ne, 32 / G);
  int blocks = grid_for(warps * 32, 128);
  if (blocks > kSMs * per_sm) blocks = kSMs * per_sm;
  switch (cpe) {
    case 1: elastic_kernel<ELEM, T, R, 1><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, C, factor, vals); break;
    case 2: elastic_kernel<ELEM, T, R, 2><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, C, factor, vals); break;
    case 3: elastic_kernel<ELEM, T, R, 3><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, C, factor, vals); break;
    case 4: elastic_kernel<ELEM, T, R, 4><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, C, factor, vals); break;
    default: elastic_kernel<ELEM, T, R, 0><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, C, factor, vals); break;
  }
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <int ELEM, typename T, typename R>
int launch_mass(const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                const uint8_t* rank, int dof_n, double rho, double factor, T* vals, cudaStream_t s) {
  constexpr int G = NextPow2<Elem<ELEM>::nPe>::value;
  const int64_t warps = ceil_div(Ne, 32 / G);
  int blocks = grid_for(warps * 32, 128);
  if (blocks > kSMs * 64) blocks = kSMs * 64;
  mass_kernel<ELEM, T, R><<<blocks, 128, 0, s>>>(coord, connect, Ne, node_ptr, rank, dof_n, rho, factor, vals);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

// Times the element kernel with 4 .. 64 blocks per SM (values zeroed before
// each candidate), records the fastest and leaves the values assembled by it.
template <int ELEM, typename T, typename R>
int tune_elastic(const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
                 const uint8_t* rank, const double* C, int cpe, double factor, T* vals, int64_t n_values,
                 cudaStream_t s, int32_t* best, float* best_ms) {
  const int cand[5] = {4, 8, 16, 32, 64};
  float bm = INFINITY, t_def = INFINITY;
  int bc = 64;
  for (int c = 0; c < 5; ++c) {
    GFEA_CUDA_TRY(cudaMemsetAsync(vals, 0, sizeof(T) * (size_t)n_values, s));
    float ms = 0;
    const int e = time_launches(
        [&]() { return launch_elastic<ELEM, T, R>(coord, connect, Ne, node_ptr, rank, C, cpe, factor, vals, s, cand[c]); },
        2, s, &ms);
    if (e) return e;
    if (cand[c] == 64) t_def = ms;
    if (ms < bm) {
      bm = ms;
      bc = cand[c];
    }
  }
  if (!(bm < 0.95f * t_def)) {  // keep the default unless clearly beaten
    bc = 64;
    bm = t_def;
  }
  tune_put(assemble_key(ELEM, sizeof(T) == 4 ? GFEA_F32 : GFEA_F64, cpe, Ne), bc);
  GFEA_CUDA_TRY(cudaMemsetAsync(vals, 0, sizeof(T) * (size_t)n_values, s));
  *best = bc;
  *best_ms = bm;
  return launch_elastic<ELEM, T, R>(coord, connect, Ne, node_ptr, rank, C, cpe, factor, vals, s, bc);
}

}  // namespace

// the higher-order elements (TRI10, TRI15, PRISM6, PRISM15, PRISM18;
// assemble_ho.cu): value_type GFEA_F64 or GFEA_F32, values of that type
int elastic_ho(int elem, bool tune, const double* coord, const int32_t* connect, int64_t Ne,
               const int32_t* node_ptr, const uint8_t* rank, const double* C, int cpe, double factor,
               int value_type, void* values, int64_t n_values, cudaStream_t s, int32_t* best, float* ms);
int mass_ho(int elem, const double* coord, const int32_t* connect, int64_t Ne, const int32_t* node_ptr,
            const uint8_t* rank, int dof_n, double rho, double factor, int value_type, void* values,
            cudaStream_t s);

}  // namespace gfea

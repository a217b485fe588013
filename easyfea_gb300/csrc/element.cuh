// Element-matrix building blocks shared by the assembly kernels: the
// Kelvin-Mandel B_p^T C product and its contraction with B_q.
#pragma once

#include "common.cuh"

namespace gfea {
namespace {

constexpr double kInvSqrt2 = 0.70710678118654752440;

template <typename T>
__device__ __forceinline__ void atomic_add_t(T* p, T v) { atomicAdd(p, v); }

// B_p^T C scaled by wJ: BtC[i][s] = wJ * sum_r B_p[r][i] C[r][s]
// (Kelvin-Mandel B of EasyFEA/FEM/_group_elem.py:1242-1312)
template <int D, typename R>
__device__ __forceinline__ void btc(const R (&g)[D], const R* C, R wJ, R (&out)[D][D == 2 ? 3 : 6]) {
  const R c = (R)kInvSqrt2;
  if constexpr (D == 2) {
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      out[0][s] = wJ * (g[0] * C[0 * 3 + s] + c * g[1] * C[2 * 3 + s]);
      out[1][s] = wJ * (g[1] * C[1 * 3 + s] + c * g[0] * C[2 * 3 + s]);
    }
  } else {
#pragma unroll
    for (int s = 0; s < 6; ++s) {
      out[0][s] = wJ * (g[0] * C[0 * 6 + s] + c * (g[2] * C[4 * 6 + s] + g[1] * C[5 * 6 + s]));
      out[1][s] = wJ * (g[1] * C[1 * 6 + s] + c * (g[2] * C[3 * 6 + s] + g[0] * C[5 * 6 + s]));
      out[2][s] = wJ * (g[2] * C[2 * 6 + s] + c * (g[1] * C[3 * 6 + s] + g[0] * C[4 * 6 + s]));
    }
  }
}

// acc[i][j] += sum_s BtC[i][s] B_q[s][j]
template <int D, typename R>
__device__ __forceinline__ void btcb(const R (&BtC)[D][D == 2 ? 3 : 6], const R (&h)[D], R (&acc)[D][D]) {
  const R c = (R)kInvSqrt2;
  if constexpr (D == 2) {
    const R chx = c * h[0], chy = c * h[1];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      acc[i][0] += BtC[i][0] * h[0] + BtC[i][2] * chy;
      acc[i][1] += BtC[i][1] * h[1] + BtC[i][2] * chx;
    }
  } else {
    const R chx = c * h[0], chy = c * h[1], chz = c * h[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      acc[i][0] += BtC[i][0] * h[0] + BtC[i][4] * chz + BtC[i][5] * chy;
      acc[i][1] += BtC[i][1] * h[1] + BtC[i][3] * chz + BtC[i][5] * chx;
      acc[i][2] += BtC[i][2] * h[2] + BtC[i][3] * chy + BtC[i][4] * chx;
    }
  }
}

}  // namespace
}  // namespace gfea

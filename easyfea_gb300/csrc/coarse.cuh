// Rigid-body modes of the two-level preconditioner's coarse space, shared by
// the single-system PCG (solver.cu) and the batched PCG (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gfea {

template <int D>
struct Modes {
  static constexpr int nr = D == 1 ? 1 : (D == 2 ? 3 : 6);
};

// Rigid-body modes at one node (D x nr), rows of known DOFs zeroed.
// R holds exactly representable products of the float offsets, so the FP32
// and FP64 iterations apply the same modes.
template <int D, typename T = double>
__device__ __forceinline__ void node_modes(float4 o, const uint8_t* kn, T (&R)[D][Modes<D>::nr]) {
  if constexpr (D == 1) {
    R[0][0] = kn[0] ? T(0) : T(1);
  } else if constexpr (D == 2) {
    const T dx = o.x, dy = o.y;
    const T r0[3] = {1, 0, -dy}, r1[3] = {0, 1, dx};
    const bool k0 = kn[0], k1 = kn[1];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      R[0][m] = k0 ? T(0) : r0[m];
      R[1][m] = k1 ? T(0) : r1[m];
    }
  } else {
    const T dx = o.x, dy = o.y, dz = o.z;
    const T r0[6] = {1, 0, 0, 0, dz, -dy}, r1[6] = {0, 1, 0, -dz, 0, dx}, r2[6] = {0, 0, 1, dy, -dx, 0};
    const bool k0 = kn[0], k1 = kn[1], k2 = kn[2];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      R[0][m] = k0 ? T(0) : r0[m];
      R[1][m] = k1 ? T(0) : r1[m];
      R[2][m] = k2 ? T(0) : r2[m];
    }
  }
}

}  // namespace gfea

// Node-row products and block reductions shared by the PCG kernels
// (multi-kernel solver and cluster-resident batched solver).
#pragma once

#include "common.cuh"

namespace gfea {

template <typename T>
struct SysT {
  int64_t Nn;
  const int32_t* node_ptr;
  const int32_t* nbr;
  const T* vals;
  const uint8_t* known;
  int diff;  // difference form sum_b K_ab (x_b - x_a) (translation-invariant operators)
};

// warp then block reduction with a fixed tree (deterministic); result valid in thread 0
__device__ __forceinline__ double block_sum(double v, double* sh) {
  // warp then block reduction with a fixed tree (deterministic)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0;
  if (w == 0) {
    t = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

// acc[i] = sum over row (a,i) of vals * xf(col) (|vals| * xf with ABS);
// reduced across the G lanes.
//
// With DIFF the product is evaluated as sum_b K_ab (x_b - x_a): identical for an
// operator whose node block rows sum to zero (rigid translations), but its
// rounding then scales with the local differences of x rather than with |x|
// (used by the FP32 products of elastic stiffness matrices).
//
// Lane l of the G-lane group owns component j = l % D of neighbours
// k = l / D, l / D + G/D, ... (the first G - G % D lanes are active): its slot
// t = D k + j advances by G - G % D, so the value loads of a row stay
// contiguous across lanes, and the component, the own-node value of the
// difference form and the slot stride are fixed per lane.
template <int D, int G, typename T, typename A, bool ABS = false, bool DIFF = false, typename XF>
__device__ __forceinline__ void node_rows(int64_t a, int lane, const SysT<T>& S, XF xf, A (&acc)[D]) {
  constexpr int LA = G - G % D;  // active lanes
  constexpr int NPP = LA / D;    // neighbours per pass
  const int32_t p0 = S.node_ptr[a];
  const int32_t nb = S.node_ptr[a + 1] - p0;
  const int32_t W = D * nb;
  const T* base = S.vals + (int64_t)D * D * p0;
  const int j = lane % D;
#pragma unroll
  for (int i = 0; i < D; ++i) acc[i] = 0;
  if (lane < LA) {
    const A self = DIFF ? xf(a * D + j) : (A)0;
    for (int32_t k = lane / D, t = lane; k < nb; k += NPP, t += LA) {
      const int64_t col = (int64_t)__ldg(S.nbr + p0 + k) * D + j;
      const A xv = DIFF ? xf(col) - self : xf(col);
#pragma unroll
      for (int i = 0; i < D; ++i) {
        const A v = (A)__ldg(base + (int64_t)i * W + t);
        acc[i] += (ABS ? (v < 0 ? -v : v) : v) * xv;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < D; ++i) acc[i] = group_sum<G, A>(acc[i]);
}

}  // namespace gfea

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

// Per-thread accumulator of dot-product terms.  For FP32 operands the sum is
// kept as an unevaluated pair s + c of floats: each product is split exactly
// (p = a b, e = fma(a, b, -p)) and added with TwoSum (Knuth), so the pair
// carries the sum of the exact products to ~2^-48 relative -- FP64-class
// accuracy without FP64 instructions, which on GB300 run at 1/64 of the FP32
// rate and were the bound of the FP32 PCG kernels.  value() returns the
// double to reduce across threads in FP64.
template <typename T>
struct DotAcc {
  double v = 0;
  __device__ __forceinline__ void add_prod(T a, T b) { v += (double)a * (double)b; }
  __device__ __forceinline__ double value() const { return v; }
};

template <>
struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float t = s + p;
    const float bp = t - s;
    const float err = (s - (t - bp)) + (p - bp);
    s = t;
    c += err + e;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Warp sum of dot accumulators (every lane receives it).  FP32 pairs are
// combined with TwoSum at each butterfly step, so the sum keeps the pairs'
// accuracy with one FP64 conversion per lane instead of FP64 shuffles and
// adds (GB300's FP64 pipe made those a visible share of short kernels).
__device__ __forceinline__ double warp_sum_acc(const DotAcc<double>& a) {
  double v = a.v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_acc(const DotAcc<float>& a) {
  float s = a.s, c = a.c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, s, o), c2 = __shfl_xor_sync(0xffffffffu, c, o);
    const float t = s + s2;
    const float bp = t - s;
    const float err = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = (c + c2) + err;
  }
  return (double)s + (double)c;
}

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

// Sum of D per-lane values over a G-lane group with a transposing butterfly:
// the first log2(V) exchange steps (V = D rounded up to a power of two) swap
// half of the remaining values with the partner lane instead of adding all of
// them, so D sums cost log2(G) + V - 2 shuffles instead of D log2(G).
// Returns row r's sum in lanes r * (G / V) .. (the other lanes hold the
// other rows' sums or padding); row_lane<D, G>(r) gives the lane.
template <int D, int G>
__host__ __device__ constexpr int row_lane(int r) {
  return r * (G / (D == 1 ? 1 : (D == 2 ? 2 : 4)));
}

template <int D, int G, typename A>
__device__ __forceinline__ A group_sum_rows(const A (&v)[D], int lane) {
  if constexpr (D == 1) {
    return group_sum<G, A>(v[0]);
  } else if constexpr (D == 2) {
    const bool hi = lane & (G / 2);
    const A send = hi ? v[0] : v[1];
    A keep = hi ? v[1] : v[0];
    keep += __shfl_xor_sync(0xffffffffu, send, G / 2, G);
#pragma unroll
    for (int o = G / 4; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o, G);
    return keep;
  } else {
    static_assert(D == 3 && G >= 4, "three rows need at least four lanes");
    const A w3 = 0;
    const bool b1 = lane & (G / 2);
    // step 1: keep {0, 1} (low half) or {2, 3} (high half), send the other pair
    A k0 = b1 ? v[2] : v[0], k1 = b1 ? w3 : v[1];
    const A s0 = b1 ? v[0] : v[2], s1 = b1 ? v[1] : w3;
    k0 += __shfl_xor_sync(0xffffffffu, s0, G / 2, G);
    k1 += __shfl_xor_sync(0xffffffffu, s1, G / 2, G);
    // step 2: keep one of the pair
    const bool b2 = lane & (G / 4);
    A keep = b2 ? k1 : k0;
    keep += __shfl_xor_sync(0xffffffffu, b2 ? k0 : k1, G / 4, G);
#pragma unroll
    for (int o = G / 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o, G);
    return keep;
  }
}

// node_rows with the transposing reduction: the returned value is row r's
// sum in lane row_lane<D, G>(r) (r < D) of the group.
template <int D, int G, typename T, typename A, bool ABS = false, bool DIFF = false, typename XF>
__device__ __forceinline__ A node_rows_t(int64_t a, int lane, const SysT<T>& S, XF xf) {
  constexpr int LA = G - G % D;
  constexpr int NPP = LA / D;
  const int32_t p0 = S.node_ptr[a];
  const int32_t nb = S.node_ptr[a + 1] - p0;
  const int32_t W = D * nb;
  const T* base = S.vals + (int64_t)D * D * p0;
  const int j = lane % D;
  A acc[D];
#pragma unroll
  for (int i = 0; i < D; ++i) acc[i] = 0;
  if (lane < LA) {
    const A self = DIFF ? xf(a * D + j) : (A)0;
    // PF passes at a time with every load issued before the arithmetic: the
    // index -> gather chains of the passes overlap (the product is bound by
    // memory latency, not bandwidth, at one pass at a time)
    constexpr int PF = 3;
    for (int32_t k0 = lane / D, t0 = lane; k0 < nb; k0 += PF * NPP, t0 += PF * LA) {
      int32_t c[PF];
      T v[PF][D];
#pragma unroll
      for (int m = 0; m < PF; ++m) {
        const bool in = k0 + m * NPP < nb;
        c[m] = in ? __ldg(S.nbr + p0 + k0 + m * NPP) : -1;
#pragma unroll
        for (int i = 0; i < D; ++i) v[m][i] = in ? __ldcs(base + (int64_t)i * W + t0 + m * LA) : (T)0;
      }
#pragma unroll
      for (int m = 0; m < PF; ++m) {
        const A xv = c[m] < 0 ? (A)0 : (DIFF ? xf((int64_t)c[m] * D + j) - self : xf((int64_t)c[m] * D + j));
#pragma unroll
        for (int i = 0; i < D; ++i) {
          const A w = (A)v[m][i];
          acc[i] += (ABS ? (w < 0 ? -w : w) : w) * xv;
        }
      }
    }
  }
  return group_sum_rows<D, G, A>(acc, lane);
}

// node_rows_t over a node whose rows were staged in shared memory: 'vrow'
// holds its D rows of W = D nb values, 'nrow' its nb neighbour indices.  The
// gathers of x for PF passes are issued before their products.
template <int D, int G, typename T, typename A, bool DIFF, typename XF>
__device__ __forceinline__ A node_rows_s(const T* vrow, const int32_t* nrow, int nb, int64_t a, int lane, XF xf) {
  constexpr int LA = G - G % D;
  constexpr int NPP = LA / D;
  constexpr int PF = 3;
  const int W = D * nb;
  const int j = lane % D;
  A acc[D];
#pragma unroll
  for (int i = 0; i < D; ++i) acc[i] = 0;
  if (lane < LA) {
    const A self = DIFF ? xf(a * D + j) : (A)0;
    for (int k0 = lane / D, t0 = lane; k0 < nb; k0 += PF * NPP, t0 += PF * LA) {
      A xv[PF];
#pragma unroll
      for (int m = 0; m < PF; ++m) {
        const int k = k0 + m * NPP;
        xv[m] = k < nb ? (DIFF ? xf((int64_t)nrow[k] * D + j) - self : xf((int64_t)nrow[k] * D + j)) : (A)0;
      }
#pragma unroll
      for (int m = 0; m < PF; ++m) {
        if (k0 + m * NPP < nb) {
#pragma unroll
          for (int i = 0; i < D; ++i) acc[i] += (A)vrow[i * W + t0 + m * LA] * xv[m];
        }
      }
    }
  }
  return group_sum_rows<D, G, A>(acc, lane);
}

}  // namespace gfea

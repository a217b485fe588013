// Kernels and launch templates of the row-owned stiffness assembly, shared
// by parts.cu and parts_ho.cu.
//
// Row-owned stiffness assembly: no global atomics.
//
// The element kernel of assemble.cu scatters every element block into the
// CSR values with global atomic adds (each value is hit by every element
// sharing its two nodes: up to 8 for HEXA8), so its DRAM traffic is about
// three times the values' size and its FP32 form is bound by the atomic
// units, not by HBM.  Here the nodes are cut into parts whose CSR rows fit in
// shared memory; one block per part zeroes the part's rows in shared memory,
// visits every element touching one of its nodes, adds the element blocks
// K_pq of its own rows p with shared-memory atomics, and writes the rows out
// once, coalesced.  Parts are compact in space (nodes taken in Morton order
// of their coordinates), so an element is visited by ~1.2-1.9 parts and each
// block K_pq is computed exactly once (by the part owning node p).
//
// Per visit, G lanes (G = next_pow2(nPe)) work on one element: lane g
// computes the Jacobian, its inverse and every node's gradient at Gauss point
// g into the group's shared scratch; lane q then accumulates, for each owned
// row p of the element, the block K_pq from the gradients of p and q at all
// Gauss points (isotropic laws: M = sum wJ grad N_p (x) grad N_q and
// K_pq = lambda M + mu M^T + mu tr(M) I; other laws: B_p^T C B_q).
//
// The plan (parts, node offsets, visit lists) is built once per mesh on the
// host by gfea_part_plan_host.
#pragma once

#include "common.cuh"
#include "element.cuh"

namespace gfea {

// the device arrays of a part plan (gfea_part_plan), passed to the kernel by value
struct PartArgs {
  int32_t max_vals;
  const int32_t* node_off;
  const int32_t* part_node_ptr;
  const int32_t* part_nodes;
  const int32_t* part_nvals;
  const int32_t* visit_ptr;
  const int32_t* visit_elem;
  const uint32_t* visit_mask;
};

namespace {

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// Rigidity Gauss weights and reference gradients in the compute type (the
// FP32 kernel must not convert FP64 table entries in its inner loops: the
// conversions run on the FP64 pipe)
template <int ELEM, typename R>
struct RefGrad {
  using E = Elem<ELEM>;
  static constexpr int nPg = E::nPg_rigi;
  R w[nPg];
  R dN[nPg][E::dim][E::nPe];
  __device__ void fill() {
    for (int i = threadIdx.x; i < nPg * E::nPe; i += blockDim.x) {
      const int g = i / E::nPe, n = i % E::nPe;
      double xi[3], wg;
      E::gauss(false, g, xi, &wg);
      for (int d = 0; d < E::dim; ++d) dN[g][d][n] = (R)E::dN(xi, d, n);
      if (n == 0) w[g] = (R)wg;
    }
  }
};

template <int ELEM>
struct PartShape {
  using E = Elem<ELEM>;
  static constexpr int nPe = E::nPe, D = E::dim, nPg = E::nPg_rigi, G = NextPow2<nPe>::value;
  // gradients of Gauss point g at g * GS (odd stride: lane g's writes hit distinct banks)
  static constexpr int GS = nPe * D + 1;
  // the coordinates' block, rounded up to an even count so that the
  // gradients after it start on an 8-byte boundary in FP32 (the paired
  // layout reads them as 64-bit words; PRISM15 has nPe D = 45)
  static constexpr int XS = (nPe * D + 1) / 2 * 2;
  // per lane group: X, gradients, wJ; the groups of a warp start 24 banks
  // apart with 4 groups (G = 8) so that the 32 lanes' gradient reads and
  // writes fall in 32 distinct banks, one bank apart otherwise
  static constexpr int SCR0 = XS + nPg * GS + nPg;
  static constexpr int SHIFT = G == 8 ? 24 : 2;  // even: the paired layout reads 8-byte words
  static constexpr int SCR = SCR0 + ((SHIFT - SCR0 % 32) + 32) % 32;
  // per lane group: each node's row offset in the part and neighbour count
  // (int32), the element's slot ranks (bytes, padded to 4)
  static constexpr int ISCR = 2 * nPe + (nPe * nPe + 3) / 4;
};

template <int ELEM, typename T>
size_t part_smem(int max_vals, int threads) {
  using S = PartShape<ELEM>;
  const int gpb = threads / S::G;
  return align16((size_t)max_vals * sizeof(T)) + align16((size_t)gpb * S::SCR * sizeof(T)) +
         (size_t)gpb * S::ISCR * 4;
}

// Two FP32 FMAs in one instruction (fma.rn.f32x2, sm_100 and later): the
// operands are pairs of floats packed in 64-bit registers.
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__device__ __forceinline__ float pair_sum(unsigned long long v) {
  return __uint_as_float((unsigned)(v & 0xffffffffu)) + __uint_as_float((unsigned)(v >> 32));
}

template <int ELEM, typename T, int CMODE>
__global__ void __launch_bounds__(256, 3) parts_elastic_kernel(const double* __restrict__ coord, const int32_t* __restrict__ connect,
                                     const int32_t* __restrict__ node_ptr, const uint8_t* __restrict__ rank,
                                     const double* __restrict__ Cglob, double factor, PartArgs P,
                                     T* __restrict__ vals) {
  using S = PartShape<ELEM>;
  using E = Elem<ELEM>;
  constexpr int nPe = S::nPe, D = S::D, nPg = S::nPg, G = S::G, NS = D == 2 ? 3 : 6;
  constexpr bool ISO = CMODE == 3 || CMODE == 4;
  // FP32 isotropic blocks: Gauss points taken two at a time by paired FMAs,
  // on gradients scaled by sqrt(wJ) stored as (g, g + 1) pairs
  constexpr bool PAIR = sizeof(T) == 4 && ISO && nPg % 2 == 0;
  using R = T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ RefGrad<ELEM, R> ref;
  __shared__ R Csh[NS * NS];
  T* acc = reinterpret_cast<T*>(smem_raw);
  const int grp = threadIdx.x / G, lane = threadIdx.x % G;
  const int gpb = blockDim.x / G;
  unsigned char* scr = smem_raw + align16((size_t)P.max_vals * sizeof(T));
  R* sX = reinterpret_cast<R*>(scr) + grp * S::SCR;
  R* sG = sX + S::XS;
  // 64-bit pair reads: the group's scratch and its gradients start on 8-byte boundaries
  static_assert(S::SCR % 2 == 0 && S::XS % 2 == 0, "paired FP32 gradients need 8-byte alignment");
  R* sW = sG + nPg * S::GS;
  int32_t* sOff = reinterpret_cast<int32_t*>(scr + align16((size_t)gpb * S::SCR * sizeof(R))) + grp * S::ISCR;
  int32_t* sNb = sOff + nPe;
  uint8_t* sRk = reinterpret_cast<uint8_t*>(sNb + nPe);
  // the lanes of this group within the warp
  const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));

  ref.fill();
  if (CMODE == 0 || CMODE == 2)
    for (int i = threadIdx.x; i < NS * NS; i += blockDim.x) Csh[i] = (R)Cglob[i];
  const int part = blockIdx.x;
  const int nv = P.part_nvals[part];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) acc[i] = (T)0;
  // where the part's rows go: loaded now, used after the visits
  constexpr int kWo = 256;  // the largest block
  __shared__ int32_t wo_src[kWo], wo_p0[kWo], wo_nb[kWo];
  const int k0 = P.part_node_ptr[part], nn = P.part_node_ptr[part + 1] - k0;
  if (threadIdx.x < nn && threadIdx.x < kWo) {
    const int32_t a = P.part_nodes[k0 + threadIdx.x];
    wo_src[threadIdx.x] = P.node_off[a];
    wo_p0[threadIdx.x] = node_ptr[a];
    wo_nb[threadIdx.x] = node_ptr[a + 1] - node_ptr[a];
  }
  __syncthreads();
  const R lam = ISO ? (R)Cglob[0] : (R)0, mu = ISO ? (R)Cglob[1] : (R)0;

  const int v1 = P.visit_ptr[part + 1];
  // the next visit's element, mask and node coordinates are loaded while the
  // current one is computed
  int64_t e_n = 0;
  uint32_t m_n = 0;
  double f_n = factor;
  R x_n[D];
  int32_t off_n = 0, nb_n = 0;
  constexpr int NW = (nPe + 3) / 4;
  uint32_t rk_n[NW];  // lane p: the ranks of row p, four to a word
  auto fetch = [&](int vv) {
    e_n = P.visit_elem[vv];
    m_n = P.visit_mask[vv];
    if (CMODE == 2) f_n = factor * __ldg(Cglob + NS * NS + e_n);
    if (CMODE == 4) f_n = factor * __ldg(Cglob + 2 + e_n);
    if (lane < nPe) {
      const int32_t a = connect[e_n * nPe + lane];
      const int32_t a0 = connect[e_n * nPe];
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const double x = coord[(int64_t)a * 3 + k];
        x_n[k] = sizeof(R) == 4 ? (R)(x - coord[(int64_t)a0 * 3 + k]) : (R)x;
      }
      off_n = P.node_off[a];
      nb_n = node_ptr[a + 1] - node_ptr[a];
      const uint8_t* rr = rank + (e_n * nPe + lane) * nPe;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        uint32_t word = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if (4 * w + b < nPe) word |= (uint32_t)rr[4 * w + b] << (8 * b);
        rk_n[w] = word;
      }
    }
  };
  int v = P.visit_ptr[part] + grp;
  if (v < v1) fetch(v);
  for (; v < v1; v += gpb) {
    const int64_t e = e_n;
    const uint32_t mask = m_n;
    const R f = (R)f_n;
    // coordinates into the group's scratch (FP32: relative to the element's
    // first node, taken in FP64, so the Jacobian keeps FP32 precision far
    // from the origin), with the nodes' row offsets and the element's slot
    // ranks
    if (lane < nPe) {
#pragma unroll
      for (int k = 0; k < D; ++k) sX[lane * D + k] = x_n[k];
      sOff[lane] = off_n;
      sNb[lane] = nb_n;
#pragma unroll
      for (int q = 0; q < nPe; ++q) sRk[lane * nPe + q] = (uint8_t)(rk_n[q / 4] >> (8 * (q % 4)));
    }
    if (v + gpb < v1) fetch(v + gpb);
    __syncwarp(gmask);
    // geometry: lane g owns Gauss point g
    for (int g = lane; g < nPg; g += G) {
      // this Gauss point's reference gradients and the element's coordinates in registers
      R dn[D][nPe], xs[nPe][D];
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int n = 0; n < nPe; ++n) dn[d][n] = ref.dN[g][d][n];
#pragma unroll
      for (int n = 0; n < nPe; ++n)
#pragma unroll
        for (int k = 0; k < D; ++k) xs[n][k] = sX[n * D + k];
      R F[D][D];
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int k = 0; k < D; ++k) {
          R s = 0;
#pragma unroll
          for (int n = 0; n < nPe; ++n) s += dn[d][n] * xs[n][k];
          F[d][k] = s;
        }
      R iF[D][D], det;
      if constexpr (D == 2) {
        det = F[0][0] * F[1][1] - F[1][0] * F[0][1];
        const R id = (R)1 / det;
        iF[0][0] = id * F[1][1];
        iF[0][1] = -id * F[0][1];
        iF[1][0] = -id * F[1][0];
        iF[1][1] = id * F[0][0];
      } else {
        const R c11 = F[1][1] * F[2][2] - F[2][1] * F[1][2], c21 = -(F[1][0] * F[2][2] - F[2][0] * F[1][2]),
                c31 = F[1][0] * F[2][1] - F[2][0] * F[1][1];
        det = F[0][0] * c11 + F[0][1] * c21 + F[0][2] * c31;
        const R id = (R)1 / det;
        iF[0][0] = id * c11;
        iF[0][1] = -id * (F[0][1] * F[2][2] - F[2][1] * F[0][2]);
        iF[0][2] = id * (F[0][1] * F[1][2] - F[1][1] * F[0][2]);
        iF[1][0] = id * c21;
        iF[1][1] = id * (F[0][0] * F[2][2] - F[2][0] * F[0][2]);
        iF[1][2] = -id * (F[0][0] * F[1][2] - F[1][0] * F[0][2]);
        iF[2][0] = id * c31;
        iF[2][1] = -id * (F[0][0] * F[2][1] - F[2][0] * F[0][1]);
        iF[2][2] = id * (F[0][0] * F[1][1] - F[1][0] * F[0][1]);
      }
      const R wJ = (det < 0 ? -det : det) * ref.w[g];
      const R sc = PAIR ? (R)sqrtf((float)wJ) : (R)1;
#pragma unroll
      for (int n = 0; n < nPe; ++n)
#pragma unroll
        for (int i = 0; i < D; ++i) {
          R s = 0;
#pragma unroll
          for (int d = 0; d < D; ++d) s += iF[i][d] * dn[d][n];
          if constexpr (PAIR)
            sG[(g >> 1) * 2 * S::GS + (n * D + i) * 2 + (g & 1)] = sc * s;
          else
            sG[g * S::GS + n * D + i] = s;
        }
      sW[g] = wJ;
    }
    __syncwarp(gmask);
    if constexpr (PAIR) {
      if (lane < nPe) {
        // lane q: its own scaled gradients as (g, g + 1) pairs, then one block per owned row p
        const unsigned long long* sG2 = reinterpret_cast<const unsigned long long*>(sG);
        unsigned long long gq2[nPg / 2][D];
#pragma unroll
        for (int h = 0; h < nPg / 2; ++h)
#pragma unroll
          for (int j = 0; j < D; ++j) gq2[h][j] = sG2[h * S::GS + lane * D + j];
        for (uint32_t m = mask; m; m &= m - 1) {
          const int p = __ffs(m) - 1;
          unsigned long long a2[D][D];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) a2[i][j] = 0ull;
#pragma unroll
          for (int h = 0; h < nPg / 2; ++h) {
            unsigned long long gp2[D];
#pragma unroll
            for (int i = 0; i < D; ++i) gp2[i] = sG2[h * S::GS + p * D + i];
#pragma unroll
            for (int i = 0; i < D; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) a2[i][j] = ffma2(gp2[i], gq2[h][j], a2[i][j]);
          }
          R M[D][D];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) M[i][j] = pair_sum(a2[i][j]);
          R tr = 0;
#pragma unroll
          for (int i = 0; i < D; ++i) tr += M[i][i];
          const int32_t nb = sNb[p];
          T* row = acc + sOff[p] + D * (int)sRk[p * nPe + lane];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j)
              atomicAdd(row + i * D * nb + j, f * (lam * M[i][j] + mu * M[j][i] + (i == j ? mu * tr : (R)0)));
        }
      }
    } else if (lane < nPe) {
      // lane q: its own gradients at every Gauss point, then one block per owned row p
      R gq[nPg][D], wq[nPg];
#pragma unroll
      for (int g = 0; g < nPg; ++g) {
        wq[g] = sW[g];
#pragma unroll
        for (int i = 0; i < D; ++i) gq[g][i] = sG[g * S::GS + lane * D + i];
      }
      R Cl[NS * NS];
      const R* C = Csh;
      if (CMODE == 1) {
#pragma unroll
        for (int i = 0; i < NS * NS; ++i) Cl[i] = (R)__ldg(Cglob + e * NS * NS + i);
        C = Cl;
      }
      for (uint32_t m = mask; m; m &= m - 1) {
        const int p = __ffs(m) - 1;
        R K[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) K[i][j] = 0;
#pragma unroll
        for (int g = 0; g < nPg; ++g) {
          R gp[D];
#pragma unroll
          for (int i = 0; i < D; ++i) gp[i] = sG[g * S::GS + p * D + i];
          if constexpr (ISO) {
#pragma unroll
            for (int i = 0; i < D; ++i) {
              const R wp = wq[g] * gp[i];
#pragma unroll
              for (int j = 0; j < D; ++j) K[i][j] += wp * gq[g][j];
            }
          } else {
            R BtC[D][NS];
            btc<D, R>(gp, C, wq[g], BtC);
            btcb<D, R>(BtC, gq[g], K);
          }
        }
        if constexpr (ISO) {
          R tr = 0;
#pragma unroll
          for (int i = 0; i < D; ++i) tr += K[i][i];
          R Kt[D][D];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) Kt[i][j] = lam * K[i][j] + mu * K[j][i] + (i == j ? mu * tr : (R)0);
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) K[i][j] = Kt[i][j];
        }
        const int32_t nb = sNb[p];
        T* row = acc + sOff[p] + D * (int)sRk[p * nPe + lane];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) atomicAdd(row + i * D * nb + j, (T)(f * K[i][j]));
      }
    }
    __syncwarp(gmask);
  }
  __syncthreads();
  // the part's rows, one warp per node, coalesced
  const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int k = warp; k < nn; k += nw) {
    int32_t off, p0, nb;
    if (k < kWo && k < (int)blockDim.x) {  // the entries loaded before the visits
      off = wo_src[k];
      p0 = wo_p0[k];
      nb = wo_nb[k];
    } else {
      const int32_t a = P.part_nodes[k0 + k];
      off = P.node_off[a];
      p0 = node_ptr[a];
      nb = node_ptr[a + 1] - p0;
    }
    const int cnt = D * D * nb;
    const T* src = acc + off;
    T* dst = vals + (int64_t)D * D * p0;
    for (int t = l32; t < cnt; t += 32) dst[t] = src[t];
  }
}

template <typename T>
constexpr int part_threads() { return sizeof(T) == 4 ? 256 : 128; }

template <int ELEM, typename T, int CMODE>
int launch_parts_mode(const double* coord, const int32_t* connect, const int32_t* node_ptr, const uint8_t* rank,
                      const double* C, double factor, const PartArgs& A, int n_parts, int threads, T* vals,
                      cudaStream_t s) {
  const size_t smem = part_smem<ELEM, T>(A.max_vals, threads);
  if (smem > 200 * 1024) return GFEA_ERR_ARG;
  auto kern = parts_elastic_kernel<ELEM, T, CMODE>;
  GFEA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  GFEA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared));
  kern<<<n_parts, threads, smem, s>>>(coord, connect, node_ptr, rank, C, factor, A, vals);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <int ELEM, typename T>
int launch_parts(const double* coord, const int32_t* connect, const int32_t* node_ptr, const uint8_t* rank,
                 const double* C, int cpe, double factor, const PartArgs& A, int n_parts, int threads, T* vals,
                 cudaStream_t s) {
  switch (cpe) {
    case 0: return launch_parts_mode<ELEM, T, 0>(coord, connect, node_ptr, rank, C, factor, A, n_parts, threads, vals, s);
    case 1: return launch_parts_mode<ELEM, T, 1>(coord, connect, node_ptr, rank, C, factor, A, n_parts, threads, vals, s);
    case 2: return launch_parts_mode<ELEM, T, 2>(coord, connect, node_ptr, rank, C, factor, A, n_parts, threads, vals, s);
    case 3: return launch_parts_mode<ELEM, T, 3>(coord, connect, node_ptr, rank, C, factor, A, n_parts, threads, vals, s);
    default: return launch_parts_mode<ELEM, T, 4>(coord, connect, node_ptr, rank, C, factor, A, n_parts, threads, vals, s);
  }
}

}  // namespace

// the higher-order elements (TRI10, TRI15, PRISM6, PRISM15, PRISM18; parts_ho.cu)
int parts_ho(int elem, const double* coord, const int32_t* connect, const int32_t* node_ptr, const uint8_t* rank,
             const double* C, int cpe, double factor, const PartArgs& A, int n_parts, int threads, int value_type,
             void* vals, cudaStream_t s);
size_t part_smem_ho(int elem, int value_type, int max_vals, int threads);

}  // namespace gfea

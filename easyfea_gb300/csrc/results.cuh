// Post-processing on the device: per-element strain and stress results, their
// von Mises equivalents, the strain energy (plain and ZZ1-smoothed), the
// phase-field psi+ result, and the element -> node average.
//
// Restates the strain / stress branch of Elastic.Result (EasyFEA/Simulations/
// _elastic.py:296-320) through Result_strain_or_stress_field_e and
// __Result_in_Strain_or_Stress_field (EasyFEA/Models/_utils.py:302-430):
// per Gauss point eps = B u_e and sigma = C eps in Kelvin-Mandel form, the
// shear components times 1/coef, the von Mises equivalent of those components
// (2D sqrt(xx^2 + yy^2 - xx yy + 3 xy^2), 3D the six-component form), then the
// mean over the Gauss points.  Elastic._Calc_Psi_Elas (_elastic.py:322-395)
// integrates 1/2 sigma . eps with thickness * wJ; with smoothing the stress is
// the node-averaged element mean interpolated back with N (the ZZ1 estimator,
// :397-418).  The phase-field stress is g(d) cP eps + cM eps with g = (1 -
// N d_e)^2 + k_res (EasyFEA/Simulations/_phasefield.py:868-915,
// Models/_phasefield.py:295-317) and psiP the History-max'ed psi+ at the mass
// Gauss points (_phasefield.py:494-530, :706-714).
//
// One lane group of G lanes per element: lane p stages node p's coordinates
// and displacement in shared memory, lane g then computes Gauss point g
// (Jacobian, gradients, strain, stress and its results; FP64, the FP64 work
// done once per point), the group sums the points' contributions and lane 0
// writes the element's results.

#pragma once

#include "split.cuh"

namespace gfea {
namespace {

struct FieldArgs {
  double coef_inv, thickness;
  const double* C;
  int cmode, pf;
  const double* d;
  const double* H_old;
  const double* sigma_n;
  double* strain_e;
  double* stress_e;
  double* vm_e;
  double* energy_e;
  double* psiP_e;
};

// von Mises equivalent of the scaled components (tensor xy, not sqrt(2) xy)
template <int D>
__device__ __forceinline__ double von_mises(const double* t) {
  if constexpr (D == 2) {
    return sqrt(t[0] * t[0] + t[1] * t[1] - t[0] * t[1] + 3 * t[2] * t[2]);
  } else {
    const double a = t[0] - t[1], b = t[1] - t[2], c = t[2] - t[0];
    return sqrt(0.5 * (a * a + b * b + c * c + 6 * (t[5] * t[5] + t[3] * t[3] + t[4] * t[4])));
  }
}

template <int ELEM, bool MASS, bool PFM, bool ANI>
__global__ void __launch_bounds__(128) fields_kernel(const double* __restrict__ coord,
                                                     const int32_t* __restrict__ connect, int64_t Ne,
                                                     const double* __restrict__ u, FieldArgs A, PF P) {
  using E = Elem<ELEM>;
  constexpr int nPe = E::nPe, D = E::dim, G = NextPow2<nPe>::value, EPW = 32 / G, NS = D == 2 ? 3 : 6;
  using Ref = RefTables<ELEM, MASS>;
  constexpr int nPg = Ref::nPg;
  constexpr int GPB = 128 / G;                      // lane groups per block
  constexpr int SC = 2 * nPe * D + nPe + nPe * NS;  // per group: X, u, d, nodal stress
  __shared__ Ref ref;
  __shared__ double scr[GPB][SC];
  ref.fill();
  __syncthreads();
  const int lane = threadIdx.x % G;
  const int sub = (threadIdx.x & 31) / G;
  double* sX = scr[threadIdx.x / G];
  double* sU = sX + nPe * D;
  double* sD = sU + nPe * D;
  double* sS = sD + nPe;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool iso = A.cmode == 3 || A.cmode == 4;

  for (int64_t e0 = warp * EPW; e0 < Ne; e0 += nwarp * EPW) {
    const int64_t e = e0 + sub;
    const bool valid = e < Ne;
    const int64_t ec = valid ? e : Ne - 1;
    // the element's nodes into the group's scratch
    if (lane < nPe) {
      const int32_t a = connect[ec * nPe + lane];
#pragma unroll
      for (int k = 0; k < D; ++k) {
        sX[lane * D + k] = coord[(int64_t)a * 3 + k];
        sU[lane * D + k] = u[(int64_t)a * D + k];
      }
      if (PFM) sD[lane] = A.d[a];
      if (A.sigma_n)
#pragma unroll
        for (int i = 0; i < NS; ++i) sS[lane * NS + i] = A.sigma_n[(int64_t)a * NS + i];
    }
    __syncwarp();
    // the element's elastic law
    double C[NS * NS];
    double lam = 0, mu = 0;
    if (!PFM) {
      if (iso) {
        const double f = A.cmode == 4 ? A.C[2 + ec] : 1.0;
        lam = f * A.C[0];
        mu = f * A.C[1];
      } else {
        const double* src = A.cmode == 1 ? A.C + ec * NS * NS : A.C;
        const double f = A.cmode == 2 ? A.C[NS * NS + ec] : 1.0;
#pragma unroll
        for (int i = 0; i < NS * NS; ++i) C[i] = f * src[i];
      }
    }
    double se[NS], ss[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) se[i] = ss[i] = 0;
    double vme = 0, vms = 0, W = 0, pp = 0;
    // lane g: Gauss point g (and g + G, ...)
    for (int g = lane; g < nPg; g += G) {
      double F[D][D];
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int k = 0; k < D; ++k) {
          double t = 0;
#pragma unroll
          for (int n = 0; n < nPe; ++n) t += ref.dN[g][d][n] * sX[n * D + k];
          F[d][k] = t;
        }
      double iF[D][D];
      const double det = det_inv<D>(F, iF);
      const double wJ = fabs(det) * ref.w[g];
      double eps[NS], sig[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) eps[i] = 0;
#pragma unroll
      for (int n = 0; n < nPe; ++n) {
        double gr[D], un[D], en[NS];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          double t = 0;
#pragma unroll
          for (int d = 0; d < D; ++d) t += iF[i][d] * ref.dN[g][d][n];
          gr[i] = t;
          un[i] = sU[n * D + i];
        }
        node_strain<D>(gr, un, en);
#pragma unroll
        for (int i = 0; i < NS; ++i) eps[i] += en[i];
      }
      if constexpr (PFM) {
        double dg = 0;
#pragma unroll
        for (int n = 0; n < nPe; ++n) dg += ref.N[g][n] * sD[n];
        const double gd = (1 - dg) * (1 - dg) + P.k_res;
        double c[NS * NS];
        split_c<D, ANI>(P, eps, gd, c, nullptr, nullptr);
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          double t = 0;
#pragma unroll
          for (int j = 0; j < NS; ++j) t += c[i * NS + j] * eps[j];
          sig[i] = t;
        }
        if (A.psiP_e) {
          double psi = psi_plus<D, ANI>(P, eps);
          if (A.H_old) {
            const double ho = A.H_old[ec * nPg + g];
            if (psi - ho < 0) psi = ho;
          }
          pp += psi;
        }
      } else if (iso) {
        const double tr = D == 2 ? eps[0] + eps[1] : eps[0] + eps[1] + eps[2];
#pragma unroll
        for (int i = 0; i < NS; ++i) sig[i] = (i < D ? lam * tr : 0.0) + 2 * mu * eps[i];
      } else {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          double t = 0;
#pragma unroll
          for (int j = 0; j < NS; ++j) t += C[i * NS + j] * eps[j];
          sig[i] = t;
        }
      }
      // results of this Gauss point: scaled components and von Mises
      double te[NS], ts[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        te[i] = i < D ? eps[i] : eps[i] * A.coef_inv;
        ts[i] = i < D ? sig[i] : sig[i] * A.coef_inv;
        se[i] += te[i];
        ss[i] += ts[i];
      }
      if (A.vm_e) {
        vme += von_mises<D>(te);
        vms += von_mises<D>(ts);
      }
      // energy density 1/2 sigma . eps, sigma either C eps or the smoothed nodal stress
      double psi = 0;
      if (A.sigma_n) {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          double sn = 0;
#pragma unroll
          for (int n = 0; n < nPe; ++n) sn += ref.N[g][n] * sS[n * NS + i];
          psi += sn * eps[i];
        }
      } else {
#pragma unroll
        for (int i = 0; i < NS; ++i) psi += sig[i] * eps[i];
      }
      W += A.thickness * wJ * (0.5 * psi);
    }
    // sums over the Gauss points (each lane holds its own points' share)
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      se[i] = group_sum<G, double>(se[i]);
      ss[i] = group_sum<G, double>(ss[i]);
    }
    vme = group_sum<G, double>(vme);
    vms = group_sum<G, double>(vms);
    W = group_sum<G, double>(W);
    pp = group_sum<G, double>(pp);
    if (valid && lane == 0) {
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        if (A.strain_e) A.strain_e[e * NS + i] = se[i] / nPg;
        if (A.stress_e) A.stress_e[e * NS + i] = ss[i] / nPg;
      }
      if (A.vm_e) {
        A.vm_e[e * 2] = vme / nPg;
        A.vm_e[e * 2 + 1] = vms / nPg;
      }
      if (A.energy_e) A.energy_e[e] = W;
      if (A.psiP_e) A.psiP_e[e] = pp / nPg;
    }
    __syncwarp();  // the scratch is overwritten by the next element
  }
}

__global__ void node_average_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc_list,
                                    int64_t Nn, const double* __restrict__ ve, int nc, double* __restrict__ vn) {
  const int64_t n = Nn * nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i / nc;
    const int c = (int)(i % nc);
    const int32_t k0 = inc_ptr[a], k1 = inc_ptr[a + 1];
    double s = 0;
    for (int32_t k = k0; k < k1; ++k) s += ve[(int64_t)inc_list[k] * nc + c];
    vn[i] = s / (double)(k1 - k0);  // 0/0 = NaN for a node of no element, as the reference
  }
}

template <int ELEM, bool MASS, bool PFM, bool ANI>
int launch_fields(const double* coord, const int32_t* connect, int64_t Ne, const double* u, const FieldArgs& A,
                  const PF& P, cudaStream_t s) {
  constexpr int G = NextPow2<Elem<ELEM>::nPe>::value;
  int blocks = grid_for(ceil_div(Ne, 32 / G) * 32, 128);
  if (blocks > kSMs * 32) blocks = kSMs * 32;
  fields_kernel<ELEM, MASS, PFM, ANI><<<blocks, 128, 0, s>>>(coord, connect, Ne, u, A, P);
  GFEA_LAUNCH_CHECK();
  return GFEA_OK;
}

template <int ELEM>
int dispatch_fields(bool mass, const double* coord, const int32_t* connect, int64_t Ne, const double* u,
                    const FieldArgs& A, const PF& P, cudaStream_t s) {
  if (A.pf && pf_anisot(P.split))
    return mass ? launch_fields<ELEM, true, true, true>(coord, connect, Ne, u, A, P, s)
                : launch_fields<ELEM, false, true, true>(coord, connect, Ne, u, A, P, s);
  if (A.pf)
    return mass ? launch_fields<ELEM, true, true, false>(coord, connect, Ne, u, A, P, s)
                : launch_fields<ELEM, false, true, false>(coord, connect, Ne, u, A, P, s);
  return mass ? launch_fields<ELEM, true, false, false>(coord, connect, Ne, u, A, P, s)
              : launch_fields<ELEM, false, false, false>(coord, connect, Ne, u, A, P, s);
}

int to_pf_params(const gfea_pf_params* p, PF* o) {
  if (!p || p->version != GFEA_ABI_VERSION) return GFEA_ERR_ARG;
  if (p->dim != 2 && p->dim != 3) return GFEA_ERR_ARG;
  if (p->split < GFEA_SPLIT_BOURDIN || p->split > GFEA_SPLIT_ANISOT_STRESS_NOCROSS) return GFEA_ERR_ARG;
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

// FieldArgs and PF of a gfea_fields (after the entry point's checks)
inline int fields_setup(const gfea_fields* f, FieldArgs* A, PF* P) {
  A->coef_inv = 1.0 / f->coef;
  A->thickness = f->thickness;
  A->C = f->C;
  A->cmode = f->c_per_elem;
  A->pf = f->pf != nullptr;
  A->d = f->d;
  A->H_old = f->H_old;
  A->sigma_n = f->sigma_n;
  A->strain_e = f->strain_e;
  A->stress_e = f->stress_e;
  A->vm_e = f->vm_e;
  A->energy_e = f->energy_e;
  A->psiP_e = f->psiP_e;
  *P = PF{};
  return A->pf ? to_pf_params(f->pf, P) : GFEA_OK;
}

}  // namespace

// the 3D elements' launches, compiled in their own translation unit
int fields_dispatch_3d(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                       const double* u, const gfea_fields* f, cudaStream_t s);
// TRI10, TRI15 (through results_ho2d.cu), PRISM6, PRISM15 and PRISM18 (results_ho.cu)
int fields_dispatch_ho(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                       const double* u, const gfea_fields* f, cudaStream_t s);
// TRI10 and TRI15 (results_ho2d.cu)
int fields_dispatch_ho2d(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                         const double* u, const gfea_fields* f, cudaStream_t s);
// HEXA20 and HEXA27 (results_hexq.cu)
int fields_dispatch_hexq(int elem, bool mass, const double* coord, const int32_t* connect, int64_t Ne,
                         const double* u, const gfea_fields* f, cudaStream_t s);

}  // namespace gfea

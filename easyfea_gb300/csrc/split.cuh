// Gauss-point strain and the phase-field strain-energy split, shared by the
// phase-field kernels and the post-processing kernels.
//
// The split restates Models.PhaseField.Calc_C (EasyFEA/Models/_phasefield.py:
// 396-571) in FP64 registers: Bourdin, Amor (:451-483) and Miehe with the
// closed-form eigenprojectors of :751-1041 (2D :777-807, 3D Q.-C. He form with
// the Lode-angle cases :809-948) and the projector assembly of :1043-1243.
// The reference picks its repeated-eigenvalue branches with exact equality
// tests (v1 == v2, g == 0, theta == 0 or pi/3).  Those tests depend on the
// last bit of the computed invariants: with fused multiply-adds, or a 1-ulp
// difference in pow, a repeated eigenvalue comes out as a gap of 1e-16 and
// the distinct-eigenvalue formulas then divide rounding noise by rounding
// noise (the reference itself returns NaN at some of these points, when the
// arccos argument rounds past +-1).  Here the branches are chosen with small
// relative tolerances instead (kEigTol*): identical to the reference wherever
// its branch choice is exact or its formulas are well conditioned, accurate
// in the band of eigenvalue gaps below ~1e-7 where they are not.

#pragma once

#include <math.h>

#include "common.cuh"

namespace gfea {
namespace {

constexpr double kSqrt2 = 1.41421356237309504880;
// repeated-eigenvalue tolerances: 2D discriminant and 3D invariant g relative to
// the squared Frobenius norm; 3D arccos argument distance to +-1
constexpr double kEigTolSq = 1e-14;
constexpr double kEigTolArg = 1e-12;
// eigenvalues within kEigTolZero * ||eps|| of zero are zero (Heaviside(0) = 1/2)
constexpr double kEigTolZero = 1e-12;

// anisotropic splits (compiled into the ANI instantiations only)
__host__ __device__ inline bool pf_anisot(int split) {
  return split >= GFEA_SPLIT_ANISOT_STRAIN && split <= GFEA_SPLIT_ANISOT_STRESS_NOCROSS;
}

struct PF {
  int split, regu, dim, plane_stress;
  double lambda, mu, Gc, l0, thickness, k_res;
  double A[9];
  double C[36];
  double S[36];
};

__host__ __device__ __forceinline__ double heav(double v) { return v > 0 ? 1.0 : (v == 0 ? 0.5 : 0.0); }
__host__ __device__ __forceinline__ double sgn(double v) { return v > 0 ? 1.0 : (v < 0 ? -1.0 : 0.0); }

// Spectral projector P+ of a second-order tensor given as a Kelvin-Mandel
// vector (the strain for Miehe, the stress for the stress-based splits, the
// transformed strain of He): its positive part is P+ : vec and P- = I - P+
// (Models/_phasefield.py:751-1243).
template <int D>
__host__ __device__ void spectral_proj(const double* vec, double* projP) {
  if constexpr (D == 2) {
    // eigenvalues m -+ rad with m = tr/2 and rad^2 = ((M00 - M11)/2)^2 + M01^2,
    // i.e. the reference's (tr -+ sqrt(tr^2 - 4 det))/2 without its cancellation
    const double M00 = vec[0], M11 = vec[1], M01 = vec[2] / kSqrt2;
    const double trM = M00 + M11;
    const double h = (M00 - M11) / 2;
    double rad2 = h * h + M01 * M01;
    const bool repeated = rad2 <= 0.25 * kEigTolSq * (M00 * M00 + M11 * M11 + 2 * M01 * M01);
    if (repeated) rad2 = 0;
    const double rad = sqrt(rad2);
    const double zero_tol = kEigTolZero * sqrt(M00 * M00 + M11 * M11 + 2 * M01 * M01);
    double v1 = trM / 2 - rad, v2 = trM / 2 + rad;
    if (fabs(v1) <= zero_tol) v1 = 0;
    if (fabs(v2) <= zero_tol) v2 = 0;
    double A00 = 1, A11 = 0, A01 = 0;  // M1 = (M - v2 I) / (v1 - v2)
    if (!repeated) {
      A00 = (rad - h) / (2 * rad);
      A11 = (rad + h) / (2 * rad);
      A01 = -M01 / (2 * rad);
    }
    const double m1[3] = {A00, A11, A01 * kSqrt2};
    const double m2[3] = {1 - A00, 1 - A11, -A01 * kSqrt2};
    const double vp1 = (v1 + fabs(v1)) / 2, vp2 = (v2 + fabs(v2)) / 2;
    double d12 = v1 - v2;
    if (d12 == 0) d12 = 1;
    const double beta = (vp1 - vp2) / d12;
    const double g1 = heav(v1) - beta, g2 = heav(v2) - beta;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        projP[i * 3 + j] = (i == j ? beta : 0.0) + g1 * m1[i] * m1[j] + g2 * m2[i] * m2[j];
  } else {
    double M[3][3];
    M[0][0] = vec[0]; M[1][1] = vec[1]; M[2][2] = vec[2];
    M[1][2] = M[2][1] = vec[3] / kSqrt2;
    M[0][2] = M[2][0] = vec[4] / kSqrt2;
    M[0][1] = M[1][0] = vec[5] / kSqrt2;
    // Invariants of the deviator s = M - I1/3 I: g = I1^2 - 3 I2 = 3/2 tr(s^2)
    // and 2 I1^3 - 9 I1 I2 + 27 I3 = 27 det(s), the reference's quantities
    // without their cancellation when the eigenvalues cluster.
    const double I1 = M[0][0] + M[1][1] + M[2][2];
    double trMM = 0;
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) trMM += M[i][k] * M[k][i];
    double S[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] = M[i][j] - (i == j ? I1 / 3 : 0.0);
    double trSS = 0;
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) trSS += S[i][k] * S[k][i];
    const double detS = S[0][0] * ((S[1][1] * S[2][2]) - (S[2][1] * S[1][2])) -
                        S[0][1] * ((S[1][0] * S[2][2]) - (S[2][0] * S[1][2])) +
                        S[0][2] * ((S[1][0] * S[2][1]) - (S[2][0] * S[1][1]));
    double g = 1.5 * trSS;
    if (g <= kEigTolSq * trMM) g = 0;  // three equal eigenvalues
    const double sg = sqrt(g);
    double arg = 0.0;
    if (g != 0) arg = 13.5 * detS / (g * sg);
    if (arg > 1) arg = 1;
    if (arg < -1) arg = -1;
    double v[3] = {I1 / 3, I1 / 3, I1 / 3};
    double M1[3][3] = {{1, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double M3[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 1}};
    if (g != 0) {
      // M - ((I1 - sg)/3) I = S + sg/3 I
      const double gm = 1.0 / sg;
      if (arg <= -1 + kEigTolArg) {  // theta = pi/3: e1 < e2 = e3
        v[0] += -2.0 / 3 * sg; v[1] += 1.0 / 3 * sg; v[2] += 1.0 / 3 * sg;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M1[i][j] = -gm * (S[i][j] + (i == j ? sg / 3 : 0.0));
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M3[i][j] = 0.5 * ((i == j ? 1.0 : 0.0) - M1[i][j]);
      } else if (arg >= 1 - kEigTolArg) {  // theta = 0: e1 = e2 < e3
        v[0] += -1.0 / 3 * sg; v[1] += -1.0 / 3 * sg; v[2] += 2.0 / 3 * sg;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M3[i][j] = gm * (S[i][j] + (i == j ? sg / 3 : 0.0));
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M1[i][j] = 0.5 * ((i == j ? 1.0 : 0.0) - M3[i][j]);
      } else {
        const double theta = acos(arg) / 3;
        const double twopi3 = 2 * M_PI / 3;
        // deviatoric eigenvalues sk; v = I1/3 + sk
        const double sk[3] = {2.0 / 3 * (sg * cos(twopi3 + theta)), 2.0 / 3 * (sg * cos(twopi3 - theta)),
                              2.0 / 3 * (sg * cos(theta))};
        v[0] += sk[0];
        v[1] += sk[1];
        v[2] += sk[2];
        double P2[3][3], P3[3][3], Q1[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            P2[i][j] = S[i][j] - (i == j ? sk[1] : 0.0);
            P3[i][j] = S[i][j] - (i == j ? sk[2] : 0.0);
            Q1[i][j] = S[i][j] - (i == j ? sk[0] : 0.0);
          }
        const double den1 = (sk[0] - sk[1]) * (sk[0] - sk[2]);
        const double den3 = (sk[2] - sk[0]) * (sk[2] - sk[1]);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double a = 0, b = 0;
            for (int k = 0; k < 3; ++k) {
              a += P2[i][k] * P3[k][j];
              b += Q1[i][k] * P2[k][j];
            }
            M1[i][j] = a / den1;
            M3[i][j] = b / den3;
          }
      }
    }
    const double zero_tol = kEigTolZero * sqrt(trMM);
    for (int k = 0; k < 3; ++k)
      if (fabs(v[k]) <= zero_tol) v[k] = 0;
    double n1 = 0, n3 = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        n1 += M1[i][j] * M1[i][j];
        n3 += M3[i][j] * M3[i][j];
      }
    n1 = sqrt(n1);
    n3 = sqrt(n3);
    double Ms[3][3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Ms[0][i][j] = M1[i][j] / n1;
        Ms[2][i][j] = M3[i][j] / n3;
        Ms[1][i][j] = (i == j ? 1.0 : 0.0) - (Ms[0][i][j] + Ms[2][i][j]);
      }
    double vp[3], dv[3], mv[3][6];
    for (int k = 0; k < 3; ++k) {
      vp[k] = (v[k] + fabs(v[k])) / 2;
      dv[k] = heav(v[k]);
      mv[k][0] = Ms[k][0][0]; mv[k][1] = Ms[k][1][1]; mv[k][2] = Ms[k][2][2];
      mv[k][3] = Ms[k][1][2] * kSqrt2; mv[k][4] = Ms[k][0][2] * kSqrt2; mv[k][5] = Ms[k][0][1] * kSqrt2;
    }
    double d12 = v[0] - v[1], d13 = v[0] - v[2], d23 = v[1] - v[2];
    if (d12 == 0) d12 = 1;
    if (d13 == 0) d13 = 1;
    if (d23 == 0) d23 = 1;
    const double th[3] = {(vp[0] - vp[1]) / (2 * d12), (vp[0] - vp[2]) / (2 * d13), (vp[1] - vp[2]) / (2 * d23)};
    const int rI[6] = {0, 1, 2, 1, 0, 0};
    const int rJ[6] = {0, 1, 2, 2, 2, 1};
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    for (int I = 0; I < 6; ++I)
      for (int K = 0; K < 6; ++K) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += dv[k] * mv[k][I] * mv[k][K];
        const double sc = (I < 3) == (K < 3) ? (I < 3 ? 1.0 : 2.0) : kSqrt2;
        const int iI = rI[I], jI = rJ[I], iK = rI[K], jK = rJ[K];
        double gs = 0;
        for (int t = 0; t < 3; ++t) {
          const double (&A)[3][3] = Ms[pa[t]];
          const double (&B)[3][3] = Ms[pb[t]];
          const double G = (A[iI][iK] * B[jI][jK] + A[iI][jK] * B[iK][jI] + B[iI][iK] * A[jI][jK] +
                            B[iI][jK] * A[iK][jI]) * sc;
          gs += th[t] * G;
        }
        projP[I * 6 + K] = s + gs;
      }
  }
}

// Anisotropic splits (Models/_phasefield.py:541-567, 646-676): with the
// projectors P+- of eps (strain) or of sigma = C eps (stress),
//   strain: Cab = Pa^T C Pb;   stress: Cab = (Pa C)^T S (Pb C)
// and cP / cM from the four blocks by variant (full: cP = Cpp + Cpm + Cmp;
// PM: Cpp + Cpm; MP: Cpp + Cmp; NoCross: Cpp; cM takes the rest).  Compiled
// only into the kernels instantiated for them (split_c's ANI): its 6x6
// temporaries would otherwise weigh on the registers of every split.
template <int D>
__host__ __device__ __forceinline__ void split_anisot(const PF& P, const double* eps, double gP, double* c, double* cPo,
                                                   double* cMo) {
  constexpr int n = D == 2 ? 3 : 6;

    const double* C = P.C;
    const bool strain = P.split <= GFEA_SPLIT_ANISOT_STRAIN_NOCROSS;
    const int variant = (P.split - GFEA_SPLIT_ANISOT_STRAIN) % 4;
    double pp[n * n], ap[n * n], am[n * n], bp[n * n], bm[n * n];
    if (strain) {
      spectral_proj<D>(eps, pp);
      // ap = C P+, am = C P-; blocks Cab = Pa^T (C Pb): bp/bm are P+^T, P-^T
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double t = 0;
          for (int k = 0; k < n; ++k) t += C[i * n + k] * pp[k * n + j];
          ap[i * n + j] = t;
          am[i * n + j] = C[i * n + j] - t;
          bp[i * n + j] = pp[j * n + i];
          bm[i * n + j] = (i == j ? 1.0 : 0.0) - pp[j * n + i];
        }
    } else {
      double sig[n];
      for (int i = 0; i < n; ++i) {
        double t = 0;
        for (int j = 0; j < n; ++j) t += C[i * n + j] * eps[j];
        sig[i] = t;
      }
      spectral_proj<D>(sig, pp);
      // Cp = P+ C, Cm = C - Cp; ap = S Cp, am = S Cm; bp = Cp^T, bm = Cm^T
      double cpm[n * n];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double t = 0;
          for (int k = 0; k < n; ++k) t += pp[i * n + k] * C[k * n + j];
          cpm[i * n + j] = t;
        }
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double tp = 0, tm = 0;
          for (int k = 0; k < n; ++k) {
            tp += P.S[i * n + k] * cpm[k * n + j];
            tm += P.S[i * n + k] * (C[k * n + j] - cpm[k * n + j]);
          }
          ap[i * n + j] = tp;
          am[i * n + j] = tm;
          bp[i * n + j] = cpm[j * n + i];
          bm[i * n + j] = C[j * n + i] - cpm[j * n + i];
        }
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double cpp = 0, cpmm = 0, cmp = 0, cmm = 0;  // Cpp, Cpm, Cmp, Cmm
        for (int k = 0; k < n; ++k) {
          cpp += bp[i * n + k] * ap[k * n + j];
          cpmm += bp[i * n + k] * am[k * n + j];
          cmp += bm[i * n + k] * ap[k * n + j];
          cmm += bm[i * n + k] * am[k * n + j];
        }
        double cp, cm;
        switch (variant) {
          case 0: cp = cpp + cpmm + cmp; cm = cmm; break;
          case 1: cp = cpp + cpmm; cm = cmm + cmp; break;
          case 2: cp = cpp + cmp; cm = cmm + cpmm; break;
          default: cp = cpp; cm = cmm + cpmm + cmp; break;
        }
        c[i * n + j] = gP * cp + cm;
        if (cPo) cPo[i * n + j] = cp;
        if (cMo) cMo[i * n + j] = cm;
      }
}

// c = gP * cP + cM  (n x n, row-major); gP = 1 gives cP + cM.
// With want_parts, cP and cM are also returned separately.
template <int D, bool ANI = false>
__host__ __device__ void split_c(const PF& P, const double* eps, double gP, double* c, double* cPo, double* cMo) {
  constexpr int n = D == 2 ? 3 : 6;
  const double tr = D == 2 ? eps[0] + eps[1] : eps[0] + eps[1] + eps[2];
  const double Rp = (1 + sgn(tr)) / 2, Rm = (1 + sgn(-tr)) / 2;
  auto IxI = [](int i, int j) { return (i < D && j < D) ? 1.0 : 0.0; };
  if (P.split == GFEA_SPLIT_BOURDIN) {
    for (int i = 0; i < n * n; ++i) {
      c[i] = gP * P.C[i];
      if (cPo) cPo[i] = P.C[i];
      if (cMo) cMo[i] = 0.0;
    }
    return;
  }
  if (P.split == GFEA_SPLIT_AMOR) {
    const double bulk = P.lambda + 2 * P.mu / D;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double cp = bulk * (Rp * IxI(i, j)) + 2 * P.mu * ((i == j ? 1.0 : 0.0) - 1.0 / D * IxI(i, j));
        const double cm = bulk * (Rm * IxI(i, j));
        c[i * n + j] = gP * cp + cm;
        if (cPo) cPo[i * n + j] = cp;
        if (cMo) cMo[i * n + j] = cm;
      }
    return;
  }
  if constexpr (ANI) {
    split_anisot<D>(P, eps, gP, c, cPo, cMo);
    return;
  }
  if (P.split == GFEA_SPLIT_ZHANG || P.split == GFEA_SPLIT_STRESS || P.split == GFEA_SPLIT_HE) {
    // stress-based splits (Models/_phasefield.py:573-687): projectors of
    // sigma = C eps; He (:689-749): projectors of C^1/2 eps mapped back with
    // C^-1/2 (.) C^1/2, where C^1/2 of the isotropic law is
    // sqrt(2 mu) (I - Pv) + sqrt(D lambda + 2 mu) Pv, Pv = IxI / D
    const double* C = P.C;
    double pp[n * n], cp[n * n], cm[n * n];
    if (P.split == GFEA_SPLIT_HE) {
      const double a = sqrt(2 * P.mu), b = sqrt(D * P.lambda + 2 * P.mu);
      double sq[n * n], si[n * n];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          const double pv = IxI(i, j) / D, id = i == j ? 1.0 : 0.0;
          sq[i * n + j] = a * (id - pv) + b * pv;
          si[i * n + j] = (id - pv) / a + pv / b;
        }
      double et[n];
      for (int i = 0; i < n; ++i) {
        double t = 0;
        for (int j = 0; j < n; ++j) t += sq[i * n + j] * eps[j];
        et[i] = t;
      }
      double ppt[n * n];
      spectral_proj<D>(et, ppt);
      // P+ = S^1/2 Pt+ C^1/2, P- = S^1/2 (I - Pt+) C^1/2 = I - P+
      double tmp[n * n];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double t = 0;
          for (int k = 0; k < n; ++k) t += ppt[i * n + k] * sq[k * n + j];
          tmp[i * n + j] = t;
        }
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double t = 0;
          for (int k = 0; k < n; ++k) t += si[i * n + k] * tmp[k * n + j];
          pp[i * n + j] = t;
        }
      // cP = C P+, cM = C P-
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double tp = 0, tm = 0;
          for (int k = 0; k < n; ++k) {
            tp += C[i * n + k] * pp[k * n + j];
            tm += C[i * n + k] * ((k == j ? 1.0 : 0.0) - pp[k * n + j]);
          }
          cp[i * n + j] = tp;
          cm[i * n + j] = tm;
        }
    } else {
      double sig[n];
      for (int i = 0; i < n; ++i) {
        double t = 0;
        for (int j = 0; j < n; ++j) t += C[i * n + j] * eps[j];
        sig[i] = t;
      }
      spectral_proj<D>(sig, pp);
      if (P.split == GFEA_SPLIT_ZHANG) {  // cP = P+ C, cM = P- C
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            double tp = 0, tm = 0;
            for (int k = 0; k < n; ++k) {
              tp += pp[i * n + k] * C[k * n + j];
              tm += ((i == k ? 1.0 : 0.0) - pp[i * n + k]) * C[k * n + j];
            }
            cp[i * n + j] = tp;
            cm[i * n + j] = tm;
          }
      } else {  // Stress: s+- = a1 P+- - a2 R+- IxI (isotropic compliance), c+- = C s+- C
        const double trs = D == 2 ? sig[0] + sig[1] : sig[0] + sig[1] + sig[2];
        const double Rps = (1 + sgn(trs)) / 2, Rms = (1 + sgn(-trs)) / 2;
        const double nu = P.plane_stress ? P.lambda / (P.lambda + 2 * P.mu) : P.lambda / (2 * (P.lambda + P.mu));
        const double E = 2 * P.mu * (1 + nu);
        const double a1 = D == 2 ? (1 + nu) / E : 1 / (2 * P.mu);
        const double a2 = D == 2 ? (P.plane_stress ? nu / E : nu * (1 + nu) / E) : nu / E;
        double sp[n * n], sm[n * n];
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            const double id = i == j ? 1.0 : 0.0;
            sp[i * n + j] = a1 * pp[i * n + j] - a2 * Rps * IxI(i, j);
            sm[i * n + j] = a1 * (id - pp[i * n + j]) - a2 * Rms * IxI(i, j);
          }
        double tp[n * n], tm[n * n];
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            double a = 0, b = 0;
            for (int k = 0; k < n; ++k) {
              a += C[k * n + i] * sp[k * n + j];  // C^T s
              b += C[k * n + i] * sm[k * n + j];
            }
            tp[i * n + j] = a;
            tm[i * n + j] = b;
          }
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            double a = 0, b = 0;
            for (int k = 0; k < n; ++k) {
              a += tp[i * n + k] * C[k * n + j];
              b += tm[i * n + k] * C[k * n + j];
            }
            cp[i * n + j] = a;
            cm[i * n + j] = b;
          }
      }
    }
    for (int i = 0; i < n * n; ++i) {
      c[i] = gP * cp[i] + cm[i];
      if (cPo) cPo[i] = cp[i];
      if (cMo) cMo[i] = cm[i];
    }
    return;
  }
  // Miehe: projP from the eigen decomposition of the strain tensor
  double projP[n * n];
  spectral_proj<D>(eps, projP);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double pp = projP[i * n + j];
      const double pm = (i == j ? 1.0 : 0.0) - pp;
      const double cp = P.lambda * (Rp * IxI(i, j)) + 2 * P.mu * pp;
      const double cm = P.lambda * (Rm * IxI(i, j)) + 2 * P.mu * pm;
      c[i * n + j] = gP * cp + cm;
      if (cPo) cPo[i * n + j] = cp;
      if (cMo) cMo[i * n + j] = cm;
    }
}

template <int D, bool ANI = false>
__device__ double psi_plus(const PF& P, const double* eps) {
  constexpr int n = D == 2 ? 3 : 6;
  double c[n * n], cP[n * n];
  split_c<D, ANI>(P, eps, 1.0, c, cP, nullptr);
  double s = 0;
  for (int i = 0; i < n; ++i) {
    double sig = 0;
    for (int j = 0; j < n; ++j) sig += cP[i * n + j] * eps[j];
    s += 0.5 * eps[i] * sig;
  }
  return s;
}

// strain contribution B_p u_p of one node (KM), dim D
template <int D>
__device__ __forceinline__ void node_strain(const double (&g)[D], const double (&u)[D], double* e) {
  const double c = 1.0 / kSqrt2;
  if constexpr (D == 2) {
    e[0] = g[0] * u[0];
    e[1] = g[1] * u[1];
    e[2] = c * g[1] * u[0] + c * g[0] * u[1];
  } else {
    e[0] = g[0] * u[0];
    e[1] = g[1] * u[1];
    e[2] = g[2] * u[2];
    e[3] = c * g[2] * u[1] + c * g[1] * u[2];
    e[4] = c * g[2] * u[0] + c * g[0] * u[2];
    e[5] = c * g[1] * u[0] + c * g[0] * u[1];
  }
}

template <int ELEM, bool MASS, int G>
__device__ __forceinline__ double lane_geo(const RefTables<ELEM, MASS>& ref, int g, int lane, bool node_lane,
                                           const double (&X)[Elem<ELEM>::dim], double (&grad)[Elem<ELEM>::dim]) {
  constexpr int D = Elem<ELEM>::dim;
  double F[D][D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double dn = node_lane ? ref.dN[g][d][lane] : 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) F[d][k] = group_sum<G, double>(dn * X[k]);
  }
  double iF[D][D];
  const double det = det_inv<D>(F, iF);
#pragma unroll
  for (int i = 0; i < D; ++i) {
    double v = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) v += iF[i][d] * (node_lane ? ref.dN[g][d][lane] : 0.0);
    grad[i] = v;
  }
  return fabs(det) * ref.w[g];
}

template <int ELEM, int G>
__device__ __forceinline__ void group_strain(const double (&grad)[Elem<ELEM>::dim], const double (&u)[Elem<ELEM>::dim],
                                             bool node_lane, double* eps) {
  constexpr int D = Elem<ELEM>::dim, n = D == 2 ? 3 : 6;
  double e[n];
  node_strain<D>(grad, u, e);
#pragma unroll
  for (int i = 0; i < n; ++i) eps[i] = group_sum<G, double>(node_lane ? e[i] : 0.0);
}

}  // namespace
}  // namespace gfea

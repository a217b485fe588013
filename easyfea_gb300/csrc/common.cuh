// Internal helpers shared by the gfea kernels: element reference data,
// lane-group reductions and status plumbing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>

#include "../../include/gfea.h"

// A failed CUDA runtime call returns GFEA_ERR_CUDA; with GFEA_DEBUG set the
// call and the runtime's error string go to stderr.
#define GFEA_CUDA_TRY(expr)                                                                      \
  do {                                                                                           \
    cudaError_t _e = (expr);                                                                     \
    if (_e != cudaSuccess) {                                                                     \
      if (getenv("GFEA_DEBUG"))                                                                  \
        fprintf(stderr, "gfea: %s:%d %s: %s\n", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return GFEA_ERR_CUDA;                                                                      \
    }                                                                                            \
  } while (0)

namespace gfea {
// number of kernels this library has launched (process lifetime)
inline std::atomic<long long>& launch_counter() {
  static std::atomic<long long> n{0};
  return n;
}
}  // namespace gfea

#define GFEA_LAUNCH_CHECK()                 \
  do {                                      \
    gfea::launch_counter().fetch_add(1);    \
    GFEA_CUDA_TRY(cudaGetLastError());      \
  } while (0)

namespace gfea {

constexpr int kSMs = 152;  // GB300 streaming multiprocessors (two dies x 76)

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// Element reference data.  Gauss tables follow EasyFEA/FEM/_gauss.py:364-480
// and the shape functions EasyFEA/FEM/Elems/{_seg,_tri,_quad,_hexa,_tetra,_prism}.py; they
// are evaluated on the device into shared memory by each kernel's prologue.
// ---------------------------------------------------------------------------

template <int ELEM> struct Elem;

// The higher-order elements whose launches compile in the *_ho.cu
// translation units, and the dimension of every element code (-1: unknown).
inline bool higher_order_elem(int elem) {
  return elem == GFEA_TRI10 || elem == GFEA_TRI15 || elem == GFEA_PRISM6 || elem == GFEA_PRISM15 ||
         elem == GFEA_PRISM18;
}

template <> struct Elem<GFEA_SEG2> {
  static constexpr int nPe = 2, dim = 1, nPg_rigi = 1, nPg_mass = 2;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) {
    if (!mass) { xi[0] = 0.0; *w = 2.0; return; }
    const double a = 1.0 / sqrt(3.0);
    xi[0] = g == 0 ? -a : a;
    *w = 1.0;
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0];
    return n == 0 ? -(r - 1) / 2 : (r + 1) / 2;
  }
  __device__ static double dN(const double*, int, int n) { return n == 0 ? -0.5 : 0.5; }
};

template <> struct Elem<GFEA_TRI3> {
  static constexpr int nPe = 3, dim = 2, nPg_rigi = 1, nPg_mass = 3;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) {
    if (!mass) { xi[0] = 1.0 / 3; xi[1] = 1.0 / 3; *w = 0.5; return; }
    const double xs[3] = {1.0 / 6, 2.0 / 3, 1.0 / 6};
    const double ys[3] = {1.0 / 6, 1.0 / 6, 2.0 / 3};
    xi[0] = xs[g]; xi[1] = ys[g]; *w = 1.0 / 6;
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1];
    return n == 0 ? -r - s + 1 : (n == 1 ? r : s);
  }
  __device__ static double dN(const double*, int d, int n) {
    if (n == 0) return -1.0;
    return (n == 1) == (d == 0) ? 1.0 : 0.0;
  }
};

template <> struct Elem<GFEA_QUAD4> {
  static constexpr int nPe = 4, dim = 2, nPg_rigi = 4, nPg_mass = 4;
  __device__ static void gauss(bool, int g, double* xi, double* w) {
    const double a = 1.0 / sqrt(3.0);
    const double xs[4] = {-a, a, a, -a};
    const double ys[4] = {-a, -a, a, a};
    xi[0] = xs[g]; xi[1] = ys[g]; *w = 1.0;
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1];
    switch (n) {
      case 0: return (r - 1) * (s - 1) / 4;
      case 1: return -(r + 1) * (s - 1) / 4;
      case 2: return (r + 1) * (s + 1) / 4;
      default: return -(r - 1) * (s + 1) / 4;
    }
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double r = p[0], s = p[1];
    if (d == 0) {
      switch (n) {
        case 0: return s / 4 - 1.0 / 4;
        case 1: return 1.0 / 4 - s / 4;
        case 2: return s / 4 + 1.0 / 4;
        default: return -s / 4 - 1.0 / 4;
      }
    }
    switch (n) {
      case 0: return r / 4 - 1.0 / 4;
      case 1: return -r / 4 - 1.0 / 4;
      case 2: return r / 4 + 1.0 / 4;
      default: return 1.0 / 4 - r / 4;
    }
  }
};

template <> struct Elem<GFEA_QUAD9> {
  static constexpr int nPe = 9, dim = 2, nPg_rigi = 9, nPg_mass = 9;
  __device__ static void gauss(bool, int g, double* xi, double* w) {
    const double a = 0.774596669241483;  // literal of EasyFEA/FEM/_gauss.py:125
    const double xs[9] = {-a, a, a, -a, 0.0, a, 0.0, -a, 0.0};
    const double ys[9] = {-a, -a, a, a, -a, 0.0, a, 0.0, 0.0};
    xi[0] = xs[g]; xi[1] = ys[g];
    *w = g < 4 ? 25.0 / 81 : (g < 8 ? 40.0 / 81 : 64.0 / 81);
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1];
    switch (n) {
      case 0: return r * s * (r - 1) * (s - 1) / 4;
      case 1: return r * s * (r + 1) * (s - 1) / 4;
      case 2: return r * s * (r + 1) * (s + 1) / 4;
      case 3: return r * s * (r - 1) * (s + 1) / 4;
      case 4: return -s * (r - 1) * (r + 1) * (s - 1) / 2;
      case 5: return -r * (r + 1) * (s - 1) * (s + 1) / 2;
      case 6: return -s * (r - 1) * (r + 1) * (s + 1) / 2;
      case 7: return -r * (r - 1) * (s - 1) * (s + 1) / 2;
      default: return (r - 1) * (r + 1) * (s - 1) * (s + 1);
    }
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double r = p[0], s = p[1];
    if (d == 0) {
      switch (n) {
        case 0: return r * s * (s - 1) / 4 + s * (r - 1) * (s - 1) / 4;
        case 1: return r * s * (s - 1) / 4 + s * (r + 1) * (s - 1) / 4;
        case 2: return r * s * (s + 1) / 4 + s * (r + 1) * (s + 1) / 4;
        case 3: return r * s * (s + 1) / 4 + s * (r - 1) * (s + 1) / 4;
        case 4: return -s * (r - 1) * (s - 1) / 2 - s * (r + 1) * (s - 1) / 2;
        case 5: return -r * (s - 1) * (s + 1) / 2 - (r + 1) * (s - 1) * (s + 1) / 2;
        case 6: return -s * (r - 1) * (s + 1) / 2 - s * (r + 1) * (s + 1) / 2;
        case 7: return -r * (s - 1) * (s + 1) / 2 - (r - 1) * (s - 1) * (s + 1) / 2;
        default: return (r - 1) * (s - 1) * (s + 1) + (r + 1) * (s - 1) * (s + 1);
      }
    }
    switch (n) {
      case 0: return r * s * (r - 1) / 4 + r * (r - 1) * (s - 1) / 4;
      case 1: return r * s * (r + 1) / 4 + r * (r + 1) * (s - 1) / 4;
      case 2: return r * s * (r + 1) / 4 + r * (r + 1) * (s + 1) / 4;
      case 3: return r * s * (r - 1) / 4 + r * (r - 1) * (s + 1) / 4;
      case 4: return -s * (r - 1) * (r + 1) / 2 - (r - 1) * (r + 1) * (s - 1) / 2;
      case 5: return -r * (r + 1) * (s - 1) / 2 - r * (r + 1) * (s + 1) / 2;
      case 6: return -s * (r - 1) * (r + 1) / 2 - (r - 1) * (r + 1) * (s + 1) / 2;
      case 7: return -r * (r - 1) * (s - 1) / 2 - r * (r - 1) * (s + 1) / 2;
      default: return (r - 1) * (r + 1) * (s - 1) + (r - 1) * (r + 1) * (s + 1);
    }
  }
};

template <> struct Elem<GFEA_HEXA8> {
  static constexpr int nPe = 8, dim = 3, nPg_rigi = 8, nPg_mass = 8;
  __device__ static void gauss(bool, int g, double* xi, double* w) {
    const double a = 1.0 / sqrt(3.0);
    // x = [-a]*4 + [a]*4, y = [-a,-a,a,a]*2, z = [-a,a]*4 (EasyFEA/FEM/_gauss.py:207-212)
    xi[0] = g < 4 ? -a : a;
    xi[1] = (g & 2) ? a : -a;
    xi[2] = (g & 1) ? a : -a;
    *w = 1.0;
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1], t = p[2];
    switch (n) {
      case 0: return -(r - 1) * (s - 1) * (t - 1) / 8;
      case 1: return (r + 1) * (s - 1) * (t - 1) / 8;
      case 2: return -(r + 1) * (s + 1) * (t - 1) / 8;
      case 3: return (r - 1) * (s + 1) * (t - 1) / 8;
      case 4: return (r - 1) * (s - 1) * (t + 1) / 8;
      case 5: return -(r + 1) * (s - 1) * (t + 1) / 8;
      case 6: return (r + 1) * (s + 1) * (t + 1) / 8;
      default: return -(r - 1) * (s + 1) * (t + 1) / 8;
    }
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double r = p[0], s = p[1], t = p[2];
    // node signs (sr, ss, st) of the reference element corners
    const double sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
    const double ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    const double st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    const double a = sr[n], b = ss[n], c = st[n];
    // N_n = (1 + a r)(1 + b s)(1 + c t) / 8
    if (d == 0) return a * (1 + b * s) * (1 + c * t) / 8;
    if (d == 1) return b * (1 + a * r) * (1 + c * t) / 8;
    return c * (1 + a * r) * (1 + b * s) / 8;
  }
};

template <> struct Elem<GFEA_TETRA4> {
  static constexpr int nPe = 4, dim = 3, nPg_rigi = 1, nPg_mass = 4;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) {
    if (!mass) { xi[0] = xi[1] = xi[2] = 0.25; *w = 1.0 / 6; return; }
    // EasyFEA/FEM/_gauss.py:155-163: a = (5 - sqrt 5)/20, b = (5 + 3 sqrt 5)/20,
    // x = [a, a, a, b], y = [a, a, b, a], z = [a, b, a, a], weights 1/24
    const double a = (5 - sqrt(5.0)) / 20, b = (5 + 3 * sqrt(5.0)) / 20;
    xi[0] = g == 3 ? b : a;
    xi[1] = g == 2 ? b : a;
    xi[2] = g == 1 ? b : a;
    *w = 1.0 / 24;
  }
  __device__ static double N(const double* p, int n) {
    return n == 0 ? 1 - p[0] - p[1] - p[2] : p[n - 1];
  }
  __device__ static double dN(const double*, int d, int n) {
    if (n == 0) return -1.0;
    return d == n - 1 ? 1.0 : 0.0;
  }
};

// Quadratic elements (EasyFEA/FEM/Elems/_seg.py SEG3, _tri.py TRI6, _quad.py
// QUAD8, _tetra.py TETRA10; Gauss rules of EasyFEA/FEM/_gauss.py:55-108 and
// :364-480: SEG3 1 / 3 points, TRI6 3 / 6, QUAD8 4 / 9, TETRA10 4 / 4).
template <> struct Elem<GFEA_SEG3> {
  static constexpr int nPe = 3, dim = 1, nPg_rigi = 1, nPg_mass = 3;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) {
    if (!mass) { xi[0] = 0.0; *w = 2.0; return; }
    const double a = sqrt(3.0 / 5.0);
    xi[0] = g == 0 ? -a : (g == 1 ? 0.0 : a);
    *w = g == 1 ? 8.0 / 9 : 5.0 / 9;
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0];
    return n == 0 ? r * (r - 1) / 2 : (n == 1 ? r * (r + 1) / 2 : -(r - 1) * (r + 1));
  }
  __device__ static double dN(const double* p, int, int n) {
    const double r = p[0];
    return n == 0 ? r - 0.5 : (n == 1 ? r + 0.5 : -2 * r);
  }
};

template <> struct Elem<GFEA_TRI6> {
  static constexpr int nPe = 6, dim = 2, nPg_rigi = 3, nPg_mass = 6;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) {
    if (!mass) {
      const double xs[3] = {1.0 / 6, 2.0 / 3, 1.0 / 6};
      const double ys[3] = {1.0 / 6, 1.0 / 6, 2.0 / 3};
      xi[0] = xs[g]; xi[1] = ys[g]; *w = 1.0 / 6;
      return;
    }
    // literals of EasyFEA/FEM/_gauss.py:71-74
    const double a = 0.445948490915965, b = 0.091576213509771;
    const double p1 = 0.11169079483905, p2 = 0.0549758718227661;
    const double xs[6] = {b, 1 - 2 * b, b, a, a, 1 - 2 * a};
    const double ys[6] = {b, b, 1 - 2 * b, 1 - 2 * a, a, a};
    xi[0] = xs[g]; xi[1] = ys[g]; *w = g < 3 ? p2 : p1;
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1];
    switch (n) {
      case 0: return (r + s - 1) * (2 * r + 2 * s - 1);
      case 1: return r * (2 * r - 1);
      case 2: return s * (2 * s - 1);
      case 3: return -4 * r * (r + s - 1);
      case 4: return 4 * r * s;
      default: return -4 * s * (r + s - 1);
    }
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double r = p[0], s = p[1];
    switch (n) {
      case 0: return 4 * r + 4 * s - 3;
      case 1: return d == 0 ? 4 * r - 1 : 0.0;
      case 2: return d == 0 ? 0.0 : 4 * s - 1;
      case 3: return d == 0 ? -8 * r - 4 * s + 4 : -4 * r;
      case 4: return d == 0 ? 4 * s : 4 * r;
      default: return d == 0 ? -4 * s : -4 * r - 8 * s + 4;
    }
  }
};

template <> struct Elem<GFEA_QUAD8> {
  static constexpr int nPe = 8, dim = 2, nPg_rigi = 4, nPg_mass = 9;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) {
    if (mass) { Elem<GFEA_QUAD9>::gauss(true, g, xi, w); return; }
    Elem<GFEA_QUAD4>::gauss(false, g, xi, w);
  }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1];
    switch (n) {
      case 0: return -(r - 1) * (s - 1) * (r + s + 1) / 4;
      case 1: return -(r + 1) * (s - 1) * (r - s - 1) / 4;
      case 2: return (r + 1) * (s + 1) * (r + s - 1) / 4;
      case 3: return (r - 1) * (s + 1) * (r - s + 1) / 4;
      case 4: return (r - 1) * (r + 1) * (s - 1) / 2;
      case 5: return -(r + 1) * (s - 1) * (s + 1) / 2;
      case 6: return -(r - 1) * (r + 1) * (s + 1) / 2;
      default: return (r - 1) * (s - 1) * (s + 1) / 2;
    }
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double r = p[0], s = p[1];
    if (d == 0) {
      switch (n) {
        case 0: return -(r - 1) * (s - 1) / 4 - (s - 1) * (r + s + 1) / 4;
        case 1: return -(r + 1) * (s - 1) / 4 - (s - 1) * (r - s - 1) / 4;
        case 2: return (r + 1) * (s + 1) / 4 + (s + 1) * (r + s - 1) / 4;
        case 3: return (r - 1) * (s + 1) / 4 + (s + 1) * (r - s + 1) / 4;
        case 4: return (r - 1) * (s - 1) / 2 + (r + 1) * (s - 1) / 2;
        case 5: return -(s - 1) * (s + 1) / 2;
        case 6: return -(r - 1) * (s + 1) / 2 - (r + 1) * (s + 1) / 2;
        default: return (s - 1) * (s + 1) / 2;
      }
    }
    switch (n) {
      case 0: return -(r - 1) * (s - 1) / 4 - (r - 1) * (r + s + 1) / 4;
      case 1: return (r + 1) * (s - 1) / 4 - (r + 1) * (r - s - 1) / 4;
      case 2: return (r + 1) * (s + 1) / 4 + (r + 1) * (r + s - 1) / 4;
      case 3: return -(r - 1) * (s + 1) / 4 + (r - 1) * (r - s + 1) / 4;
      case 4: return (r - 1) * (r + 1) / 2;
      case 5: return -(r + 1) * (s - 1) / 2 - (r + 1) * (s + 1) / 2;
      case 6: return -(r - 1) * (r + 1) / 2;
      default: return (r - 1) * (s - 1) / 2 + (r - 1) * (s + 1) / 2;
    }
  }
};

template <> struct Elem<GFEA_TETRA10> {
  static constexpr int nPe = 10, dim = 3, nPg_rigi = 4, nPg_mass = 4;
  __device__ static void gauss(bool, int g, double* xi, double* w) { Elem<GFEA_TETRA4>::gauss(true, g, xi, w); }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1], t = p[2];
    switch (n) {
      case 0: return (r + s + t - 1) * (2 * r + 2 * s + 2 * t - 1);
      case 1: return r * (2 * r - 1);
      case 2: return s * (2 * s - 1);
      case 3: return t * (2 * t - 1);
      case 4: return -4 * r * (r + s + t - 1);
      case 5: return 4 * r * s;
      case 6: return -4 * s * (r + s + t - 1);
      case 7: return -4 * t * (r + s + t - 1);
      case 8: return 4 * s * t;
      default: return 4 * r * t;
    }
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double r = p[0], s = p[1], t = p[2];
    switch (n) {
      case 0: return 4 * r + 4 * s + 4 * t - 3;
      case 1: return d == 0 ? 4 * r - 1 : 0.0;
      case 2: return d == 1 ? 4 * s - 1 : 0.0;
      case 3: return d == 2 ? 4 * t - 1 : 0.0;
      case 4: return d == 0 ? -8 * r - 4 * s - 4 * t + 4 : -4 * r;
      case 5: return d == 0 ? 4 * s : (d == 1 ? 4 * r : 0.0);
      case 6: return d == 1 ? -4 * r - 8 * s - 4 * t + 4 : -4 * s;
      case 7: return d == 2 ? -4 * r - 4 * s - 8 * t + 4 : -4 * t;
      case 8: return d == 0 ? 0.0 : (d == 1 ? 4 * t : 4 * s);
      default: return d == 0 ? 4 * t : (d == 1 ? 0.0 : 4 * r);
    }
  }
};

// Quadratic hexahedra (EasyFEA/FEM/Elems/_hexa.py HEXA20, HEXA27): the
// reference's node order, given by each node's local coordinates (corners,
// then edge middles, then -- HEXA27 -- face centres and the centre); 27
// Gauss points for both families (_gauss.py:216-261: a = sqrt(3/5), x
// slowest, weights 5/9 and 8/9 per axis).  Shape functions: HEXA20 the
// serendipity ones, corner (1+r ri)(1+s si)(1+t ti)(r ri+s si+t ti-2)/8 and
// edge (1-r^2)(1+s si)(1+t ti)/4 (and permutations); HEXA27 the products of
// the 1D quadratic Lagrange polynomials x(x-1)/2, 1-x^2, x(x+1)/2.
static __device__ __constant__ const signed char kHexaLocal[27][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1},
    {0, -1, -1},  {-1, 0, -1}, {-1, -1, 0}, {1, 0, -1}, {1, -1, 0}, {0, 1, -1}, {1, 1, 0}, {-1, 1, 0},
    {0, -1, 1},   {-1, 0, 1},  {1, 0, 1},   {0, 1, 1},  {0, 0, -1}, {0, -1, 0}, {-1, 0, 0}, {1, 0, 0},
    {0, 1, 0},    {0, 0, 1},   {0, 0, 0}};

__device__ inline void hexa27_gauss(int g, double* xi, double* w) {
  const double a = sqrt(3.0 / 5.0), c1 = 5.0 / 9, c2 = 8.0 / 9;
  const int i = g / 9, j = (g / 3) % 3, k = g % 3;
  const double x[3] = {-a, 0.0, a};
  xi[0] = x[i]; xi[1] = x[j]; xi[2] = x[k];
  const int n0 = (i == 1) + (j == 1) + (k == 1);  // coordinates at the centre
  *w = n0 == 0 ? c1 * c1 * c1 : (n0 == 1 ? c1 * c1 * c2 : (n0 == 2 ? c1 * c2 * c2 : c2 * c2 * c2));
}

// 1D quadratic Lagrange polynomial of the node at xa in {-1, 0, 1}, and its derivative
__device__ inline double lag2(double x, int xa) { return xa == 0 ? 1 - x * x : x * (x + xa) / 2; }
__device__ inline double dlag2(double x, int xa) { return xa == 0 ? -2 * x : x + xa * 0.5; }

template <> struct Elem<GFEA_HEXA20> {
  static constexpr int nPe = 20, dim = 3, nPg_rigi = 27, nPg_mass = 27;
  __device__ static void gauss(bool, int g, double* xi, double* w) { hexa27_gauss(g, xi, w); }
  __device__ static double N(const double* p, int n) {
    const double r = p[0], s = p[1], t = p[2];
    const int ra = kHexaLocal[n][0], sa = kHexaLocal[n][1], ta = kHexaLocal[n][2];
    if (n < 8) return (1 + r * ra) * (1 + s * sa) * (1 + t * ta) * (r * ra + s * sa + t * ta - 2) / 8;
    if (ra == 0) return (1 - r * r) * (1 + s * sa) * (1 + t * ta) / 4;
    if (sa == 0) return (1 + r * ra) * (1 - s * s) * (1 + t * ta) / 4;
    return (1 + r * ra) * (1 + s * sa) * (1 - t * t) / 4;
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double x[3] = {p[0], p[1], p[2]};
    const int c[3] = {kHexaLocal[n][0], kHexaLocal[n][1], kHexaLocal[n][2]};
    const int e = (d + 1) % 3, f = (d + 2) % 3;  // the other two axes
    if (n < 8)
      return c[d] * (1 + x[e] * c[e]) * (1 + x[f] * c[f]) * (2 * x[d] * c[d] + x[e] * c[e] + x[f] * c[f] - 1) / 8;
    if (c[d] == 0) return -2 * x[d] * (1 + x[e] * c[e]) * (1 + x[f] * c[f]) / 4;
    // the zero coordinate is along e or f
    const int z = c[e] == 0 ? e : f, o = c[e] == 0 ? f : e;
    return c[d] * (1 - x[z] * x[z]) * (1 + x[o] * c[o]) / 4;
  }
};

template <> struct Elem<GFEA_HEXA27> {
  static constexpr int nPe = 27, dim = 3, nPg_rigi = 27, nPg_mass = 27;
  __device__ static void gauss(bool, int g, double* xi, double* w) { hexa27_gauss(g, xi, w); }
  __device__ static double N(const double* p, int n) {
    return lag2(p[0], kHexaLocal[n][0]) * lag2(p[1], kHexaLocal[n][1]) * lag2(p[2], kHexaLocal[n][2]);
  }
  __device__ static double dN(const double* p, int d, int n) {
    double v = 1;
    for (int k = 0; k < 3; ++k) v *= k == d ? dlag2(p[k], kHexaLocal[n][k]) : lag2(p[k], kHexaLocal[n][k]);
    return v;
  }
};

// ---------------------------------------------------------------------------
// Higher-order segments and triangles (EasyFEA/FEM/Elems/_seg.py SEG4, SEG5;
// _tri.py TRI10, TRI15): the Lagrange interpolants of their nodes, written
// from the nodes' positions rather than as expanded polynomials.
//
// Segment of order p: node n sits at x = -1 + 2 k/p, k = kSegK[p][n] (the end
// nodes first, then the inner ones from the first end); with v = p (x + 1) / 2,
// N = prod_{q != k} (v - q) / (k - q).
// Triangle of order p: node n has barycentric indices (i0, i1, i2), i1 = p r,
// i2 = p s, i0 = p - i1 - i2 (corners, then p - 1 nodes on each edge 01, 12,
// 20 in that direction, then the inner nodes); with the barycentric
// coordinates L0 = 1 - r - s, L1 = r, L2 = s,
// N = phi_i0(p L0) phi_i1(p L1) phi_i2(p L2), phi_i(v) = prod_{q < i} (v - q) / (i - q).
// ---------------------------------------------------------------------------
static __device__ __constant__ const signed char kSegK[6][5] = {
    {0}, {0}, {0}, {0, 3, 1, 2}, {0, 4, 1, 2, 3}, {0}};

template <int P>
__device__ inline double seg_lagrange(double x, int n) {
  const double v = P * (x + 1) / 2;
  const int k = kSegK[P][n];
  double r = 1;
#pragma unroll
  for (int q = 0; q <= P; ++q)
    if (q != k) r *= (v - q) / (k - q);
  return r;
}

template <int P>
__device__ inline double seg_lagrange_d(double x, int n) {
  const double v = P * (x + 1) / 2;
  const int k = kSegK[P][n];
  double sum = 0;
#pragma unroll
  for (int j = 0; j <= P; ++j) {
    if (j == k) continue;
    double r = 1.0 / (k - j);
#pragma unroll
    for (int q = 0; q <= P; ++q)
      if (q != k && q != j) r *= (v - q) / (k - q);
    sum += r;
  }
  return sum * P / 2;  // dv/dx = p / 2
}

// phi_i(v) and its derivative
__device__ inline double tri_phi(int i, double v) {
  double r = 1;
  for (int q = 0; q < i; ++q) r *= (v - q) / (i - q);
  return r;
}
__device__ inline double tri_phi_d(int i, double v) {
  double sum = 0;
  for (int j = 0; j < i; ++j) {
    double r = 1.0 / (i - j);
    for (int q = 0; q < i; ++q)
      if (q != j) r *= (v - q) / (i - q);
    sum += r;
  }
  return sum;
}

// (i1, i2) of the TRI10 and TRI15 nodes in the reference's order
static __device__ __constant__ const signed char kTri10I[10][2] = {
    {0, 0}, {3, 0}, {0, 3}, {1, 0}, {2, 0}, {2, 1}, {1, 2}, {0, 2}, {0, 1}, {1, 1}};
static __device__ __constant__ const signed char kTri15I[15][2] = {
    {0, 0}, {4, 0}, {0, 4}, {1, 0}, {2, 0}, {3, 0}, {3, 1}, {2, 2}, {1, 3}, {0, 3}, {0, 2}, {0, 1},
    {1, 1}, {2, 1}, {1, 2}};

template <int P>
__device__ inline double tri_lagrange(const double* p, int i1, int i2) {
  const double L[3] = {1 - p[0] - p[1], p[0], p[1]};
  const int ii[3] = {P - i1 - i2, i1, i2};
  return tri_phi(ii[0], P * L[0]) * tri_phi(ii[1], P * L[1]) * tri_phi(ii[2], P * L[2]);
}

// d/dr (d = 0) or d/ds (d = 1): dL0 = -1, dL1 / dr = 1, dL2 / ds = 1
template <int P>
__device__ inline double tri_lagrange_d(const double* p, int d, int i1, int i2) {
  const double L[3] = {1 - p[0] - p[1], p[0], p[1]};
  const int ii[3] = {P - i1 - i2, i1, i2};
  const double f[3] = {tri_phi(ii[0], P * L[0]), tri_phi(ii[1], P * L[1]), tri_phi(ii[2], P * L[2])};
  const int b = d == 0 ? 1 : 2;  // the coordinate that grows with the derivative's variable
  return P * (tri_phi_d(ii[b], P * L[b]) * f[0] - tri_phi_d(ii[0], P * L[0]) * f[b]) * f[3 - b];
}

// Gauss-Legendre rules of 2, 4 and 5 points (ascending abscissae, as
// numpy.polynomial.legendre.leggauss, which EasyFEA/FEM/_gauss.py:395-420 calls)
__device__ inline void legendre_gauss(int n, int g, double* x, double* w) {
  if (n == 2) {
    const double a = 1 / sqrt(3.0);
    *x = g == 0 ? -a : a;
    *w = 1.0;
  } else if (n == 4) {
    const double t = 2.0 / 7.0 * sqrt(6.0 / 5.0);
    const double xo = sqrt(3.0 / 7.0 + t), xi = sqrt(3.0 / 7.0 - t);
    const double wo = (18.0 - sqrt(30.0)) / 36.0, wi = (18.0 + sqrt(30.0)) / 36.0;
    const double xs[4] = {-xo, -xi, xi, xo}, ws[4] = {wo, wi, wi, wo};
    *x = xs[g];
    *w = ws[g];
  } else {  // 5
    const double t = 2.0 * sqrt(10.0 / 7.0);
    const double xo = sqrt(5.0 + t) / 3.0, xi = sqrt(5.0 - t) / 3.0;
    const double wo = (322.0 - 13.0 * sqrt(70.0)) / 900.0, wi = (322.0 + 13.0 * sqrt(70.0)) / 900.0;
    const double xs[5] = {-xo, -xi, 0.0, xi, xo}, ws[5] = {wo, wi, 128.0 / 225.0, wi, wo};
    *x = xs[g];
    *w = ws[g];
  }
}

template <> struct Elem<GFEA_SEG4> {
  static constexpr int nPe = 4, dim = 1, nPg_rigi = 2, nPg_mass = 4;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) { legendre_gauss(mass ? 4 : 2, g, xi, w); }
  __device__ static double N(const double* p, int n) { return seg_lagrange<3>(p[0], n); }
  __device__ static double dN(const double* p, int, int n) { return seg_lagrange_d<3>(p[0], n); }
};

template <> struct Elem<GFEA_SEG5> {
  static constexpr int nPe = 5, dim = 1, nPg_rigi = 4, nPg_mass = 5;
  __device__ static void gauss(bool mass, int g, double* xi, double* w) { legendre_gauss(mass ? 5 : 4, g, xi, w); }
  __device__ static double N(const double* p, int n) { return seg_lagrange<4>(p[0], n); }
  __device__ static double dN(const double* p, int, int n) { return seg_lagrange_d<4>(p[0], n); }
};

template <> struct Elem<GFEA_TRI10> {
  static constexpr int nPe = 10, dim = 2, nPg_rigi = 6, nPg_mass = 6;  // _gauss.py: 6 points for both
  __device__ static void gauss(bool, int g, double* xi, double* w) { Elem<GFEA_TRI6>::gauss(true, g, xi, w); }
  __device__ static double N(const double* p, int n) { return tri_lagrange<3>(p, kTri10I[n][0], kTri10I[n][1]); }
  __device__ static double dN(const double* p, int d, int n) {
    return tri_lagrange_d<3>(p, d, kTri10I[n][0], kTri10I[n][1]);
  }
};

template <> struct Elem<GFEA_TRI15> {
  static constexpr int nPe = 15, dim = 2, nPg_rigi = 12, nPg_mass = 12;  // 12 points for both
  __device__ static void gauss(bool, int g, double* xi, double* w) {
    // the 12-point rule of degree 6 with the literals of EasyFEA/FEM/_gauss.py:92-104
    const double a = 0.063089014491502, b = 0.249286745170910, c = 0.310352451033785, d = 0.053145049844816;
    const double p1 = 0.025422453185103, p2 = 0.058393137863189, p3 = 0.041425537809187;
    const double xs[12] = {a, 1 - 2 * a, a, b, 1 - 2 * b, b, c, d, 1 - c - d, 1 - c - d, c, d};
    const double ys[12] = {a, a, 1 - 2 * a, b, b, 1 - 2 * b, d, c, c, d, 1 - c - d, 1 - c - d};
    xi[0] = xs[g];
    xi[1] = ys[g];
    *w = g < 3 ? p1 : (g < 6 ? p2 : p3);
  }
  __device__ static double N(const double* p, int n) { return tri_lagrange<4>(p, kTri15I[n][0], kTri15I[n][1]); }
  __device__ static double dN(const double* p, int d, int n) {
    return tri_lagrange_d<4>(p, d, kTri15I[n][0], kTri15I[n][1]);
  }
};

// ---------------------------------------------------------------------------
// Prisms (EasyFEA/FEM/Elems/_prism.py PRISM6, PRISM15, PRISM18): a triangle
// (r, s) times a segment t in [-1, 1].  Node n has local coordinates
// (r, s, t) = (kPrismLocal[n][0] / 2, kPrismLocal[n][1] / 2, kPrismLocal[n][2])
// in the reference's order: the corners of the t = -1 and t = 1 triangles,
// the edge middles (01, 02, 03 vertical, 12, 14 vertical, 25 vertical, 34, 35,
// 45), then -- PRISM18 -- the centres of the three quadrangular faces.
//   PRISM6:  the triangle's L_a (a = the corner) times (1 + t tn) / 2.
//   PRISM15 (serendipity): corner L_a (1 + t tn) (2 L_a + t tn - 2) / 2,
//            triangle-edge middle 2 L_a L_b (1 + t tn), vertical-edge middle L_a (1 - t^2).
//   PRISM18: the TRI6 function of (r, s) times the quadratic Lagrange
//            polynomial of t (lag2).
// Gauss points (_gauss.py:268-360; base triangle coordinates r, s, axis t):
// 6 points (r, s) in {(1/2, 1/2), (0, 1/2), (1/2, 0)} at t = -+1/sqrt(3),
// weight 1/6; 21 points: the 7-point triangle rule (closed-form
// coordinates) at t = -sqrt(3/5), 0, sqrt(3/5) with weights 5/9, 8/9, 5/9.
// ---------------------------------------------------------------------------
static __device__ __constant__ const signed char kPrismLocal[18][3] = {
    {0, 0, -1}, {2, 0, -1}, {0, 2, -1}, {0, 0, 1}, {2, 0, 1}, {0, 2, 1},
    {1, 0, -1}, {0, 1, -1}, {0, 0, 0},  {1, 1, -1}, {2, 0, 0}, {0, 2, 0},
    {1, 0, 1},  {0, 1, 1},  {1, 1, 1},  {1, 0, 0},  {0, 1, 0}, {1, 1, 0}};

__device__ inline void prism_gauss(int npg, int g, double* xi, double* w) {
  if (npg == 6) {
    const double a = 1 / sqrt(3.0);
    const double rs[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};
    xi[0] = rs[g % 3][0];
    xi[1] = rs[g % 3][1];
    xi[2] = g < 3 ? -a : a;
    *w = 1.0 / 6;
    return;
  }
  const double al = sqrt(3.0 / 5.0), c1 = 5.0 / 9, c2 = 8.0 / 9;
  const double a = (6 + sqrt(15.0)) / 21, b = (6 - sqrt(15.0)) / 21;
  const double cp = (155 + sqrt(15.0)) / 2400, cm = (155 - sqrt(15.0)) / 2400;
  const int l = g / 7, k = g % 7;
  const double r[7] = {1.0 / 3, a, 1 - 2 * a, a, b, 1 - 2 * b, b};
  const double s[7] = {1.0 / 3, a, a, 1 - 2 * a, b, b, 1 - 2 * b};
  const double wt[7] = {9.0 / 80, cp, cp, cp, cm, cm, cm};
  xi[0] = r[k];
  xi[1] = s[k];
  xi[2] = l == 0 ? -al : (l == 1 ? 0.0 : al);
  *w = (l == 1 ? c2 : c1) * wt[k];
}

// the corner a in {0, 1, 2} of the base triangle at doubled (r, s) = (2, 0) etc.
__device__ inline int prism_corner(int r2, int s2) { return r2 == 2 ? 1 : (s2 == 2 ? 2 : 0); }
// the corners (e0, e1) of the base-triangle edge whose middle is at doubled
// (r, s) = (1, 0): 0-1, (0, 1): 0-2, (1, 1): 1-2
__device__ inline void prism_edge(int r2, int s2, int* e0, int* e1) {
  *e0 = r2 == 1 && s2 == 1 ? 1 : 0;
  *e1 = s2 == 0 ? 1 : 2;
}

template <> struct Elem<GFEA_PRISM6> {
  static constexpr int nPe = 6, dim = 3, nPg_rigi = 6, nPg_mass = 6;
  __device__ static void gauss(bool, int g, double* xi, double* w) { prism_gauss(6, g, xi, w); }
  __device__ static double N(const double* p, int n) {
    const double L[3] = {1 - p[0] - p[1], p[0], p[1]};
    return L[n % 3] * (1 + p[2] * kPrismLocal[n][2]) / 2;
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double L[3] = {1 - p[0] - p[1], p[0], p[1]};
    const int a = n % 3, tn = kPrismLocal[n][2];
    if (d == 2) return L[a] * tn / 2;
    const double dL = a == 0 ? -1.0 : (a == d + 1 ? 1.0 : 0.0);
    return dL * (1 + p[2] * tn) / 2;
  }
};

template <> struct Elem<GFEA_PRISM15> {
  static constexpr int nPe = 15, dim = 3, nPg_rigi = 6, nPg_mass = 6;
  __device__ static void gauss(bool, int g, double* xi, double* w) { prism_gauss(6, g, xi, w); }
  // dL_a / d(r or s)
  __device__ static double dL(int a, int d) { return a == 0 ? -1.0 : (a == d + 1 ? 1.0 : 0.0); }
  __device__ static double N(const double* p, int n) {
    const double L[3] = {1 - p[0] - p[1], p[0], p[1]}, t = p[2];
    const int r2 = kPrismLocal[n][0], s2 = kPrismLocal[n][1], tn = kPrismLocal[n][2];
    if (n < 6) {
      const int a = n % 3;
      return L[a] * (1 + t * tn) * (2 * L[a] + t * tn - 2) / 2;
    }
    if (tn == 0) return L[prism_corner(r2, s2)] * (1 - t * t);
    int e0, e1;
    prism_edge(r2, s2, &e0, &e1);
    return 2 * L[e0] * L[e1] * (1 + t * tn);
  }
  __device__ static double dN(const double* p, int d, int n) {
    const double L[3] = {1 - p[0] - p[1], p[0], p[1]}, t = p[2];
    const int r2 = kPrismLocal[n][0], s2 = kPrismLocal[n][1], tn = kPrismLocal[n][2];
    if (n < 6) {
      const int a = n % 3;
      const double ft = 1 + t * tn, q = 2 * L[a] + t * tn - 2;
      if (d == 2) return L[a] * tn * (q + ft) / 2;
      return dL(a, d) * ft * (q + 2 * L[a]) / 2;
    }
    if (tn == 0) {
      const int a = prism_corner(r2, s2);
      return d == 2 ? -2 * t * L[a] : dL(a, d) * (1 - t * t);
    }
    int e0, e1;
    prism_edge(r2, s2, &e0, &e1);
    if (d == 2) return 2 * L[e0] * L[e1] * tn;
    return 2 * (dL(e0, d) * L[e1] + L[e0] * dL(e1, d)) * (1 + t * tn);
  }
};

template <> struct Elem<GFEA_PRISM18> {
  static constexpr int nPe = 18, dim = 3, nPg_rigi = 21, nPg_mass = 21;
  __device__ static void gauss(bool, int g, double* xi, double* w) { prism_gauss(21, g, xi, w); }
  __device__ static double N(const double* p, int n) {
    return tri_lagrange<2>(p, kPrismLocal[n][0], kPrismLocal[n][1]) * lag2(p[2], kPrismLocal[n][2]);
  }
  __device__ static double dN(const double* p, int d, int n) {
    const int i1 = kPrismLocal[n][0], i2 = kPrismLocal[n][1], tn = kPrismLocal[n][2];
    if (d == 2) return tri_lagrange<2>(p, i1, i2) * dlag2(p[2], tn);
    return tri_lagrange_d<2>(p, d, i1, i2) * lag2(p[2], tn);
  }
};

// Shared-memory reference tables of one element type and Gauss family.
template <int ELEM, bool MASS>
struct RefTables {
  using E = Elem<ELEM>;
  static constexpr int nPg = MASS ? E::nPg_mass : E::nPg_rigi;
  double w[nPg];
  double N[nPg][E::nPe];
  double dN[nPg][E::dim][E::nPe];

  __device__ void fill() {
    for (int i = threadIdx.x; i < nPg * E::nPe; i += blockDim.x) {
      const int g = i / E::nPe, n = i % E::nPe;
      double xi[3], wg;
      E::gauss(MASS, g, xi, &wg);
      N[g][n] = E::N(xi, n);
      for (int d = 0; d < E::dim; ++d) dN[g][d][n] = E::dN(xi, d, n);
      if (n == 0) w[g] = wg;
    }
  }
};

// ---------------------------------------------------------------------------
// Lane groups: G consecutive lanes of a warp cooperate on one element/node.
// ---------------------------------------------------------------------------
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
  return v;
}

template <int G, typename T>
__device__ __forceinline__ T group_bcast(T v, int src) {
  return __shfl_sync(0xffffffffu, v, src, G);
}

template <int n> struct NextPow2 {
  static constexpr int value = n <= 1 ? 1 : (n <= 2 ? 2 : (n <= 4 ? 4 : (n <= 8 ? 8 : (n <= 16 ? 16 : 32))));
};

// ---------------------------------------------------------------------------
// Jacobian helpers (closed forms of EasyFEA/FEM/_linalg.py:533-656)
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ double det_inv(const double (&F)[D][D], double (&iF)[D][D]) {
  if constexpr (D == 1) {
    iF[0][0] = 1.0 / F[0][0];
    return F[0][0];
  } else if constexpr (D == 2) {
    const double det = F[0][0] * F[1][1] - F[1][0] * F[0][1];
    const double id = 1.0 / det;
    iF[0][0] = id * F[1][1];
    iF[0][1] = id * -F[0][1];
    iF[1][0] = id * -F[1][0];
    iF[1][1] = id * F[0][0];
    return det;
  } else {
    const double a11 = F[0][0], a12 = F[0][1], a13 = F[0][2];
    const double a21 = F[1][0], a22 = F[1][1], a23 = F[1][2];
    const double a31 = F[2][0], a32 = F[2][1], a33 = F[2][2];
    const double det = a11 * ((a22 * a33) - (a32 * a23)) - a12 * ((a21 * a33) - (a31 * a23)) +
                       a13 * ((a21 * a32) - (a31 * a22));
    const double id = 1.0 / det;
    iF[0][0] = id * (a22 * a33 - a32 * a23);
    iF[0][1] = id * -(a12 * a33 - a32 * a13);
    iF[0][2] = id * (a12 * a23 - a22 * a13);
    iF[1][0] = id * -(a21 * a33 - a31 * a23);
    iF[1][1] = id * (a11 * a33 - a31 * a13);
    iF[1][2] = id * -(a11 * a23 - a21 * a13);
    iF[2][0] = id * (a21 * a32 - a31 * a22);
    iF[2][1] = id * -(a11 * a32 - a31 * a12);
    iF[2][2] = id * (a11 * a22 - a21 * a12);
    return det;
  }
}

// Launch configuration helpers.
inline int grid_for(int64_t n_items, int per_block) {
  int64_t g = ceil_div(n_items, per_block);
  if (g < 1) g = 1;
  if (g > (int64_t)1 << 30) g = (int64_t)1 << 30;
  return (int)g;
}

}  // namespace gfea

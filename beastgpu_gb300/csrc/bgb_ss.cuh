// Sauter-Schwab helpers shared by the FP64 and double-float singular kernels: the
// shared-vertex permutation of the reference, the chart maps, and the region maps.
#pragma once

#include "bgb_common.cuh"

namespace bgb {

struct Chart {
  double cv[3][2];
  double ct[2][2];
};

// Shared-vertex permutation of pulledback_integrand_gpu.jl (CF :22-58, CE :60-102, CV :117-155).
__device__ inline void ss_permutation(int cls, const Geo64& A, const Geo64& B, int I[3], int J[3]) {
  const double tol = 1e3 * 2.220446049250313e-16;
  I[0] = I[1] = I[2] = 0;
  J[0] = J[1] = J[2] = 0;
  int cap = (cls == BGB_CLASS_CE) ? 3 : 2;
  int e = 1;
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 3; ++j) {
      double R = 0.0;
      for (int c = 0; c < 3; ++c) {
        double d = __dsub_rn(A.v[i - 1][c], B.v[j - 1][c]);
        R = __dadd_rn(R, __dmul_rn(d, d));
      }
      if (__dsqrt_rn(R) < tol) {
        if (cls == BGB_CLASS_CF) {
          J[i - 1] = j;
        } else if (e <= cap) {
          J[e - 1] = j;
          I[e - 1] = i;
          e += 1;
        }
      }
    }
  if (cls == BGB_CLASS_CF) {
    I[0] = 1;
    I[1] = 2;
    I[2] = 3;
    return;
  }
  for (int k = 0; k < 2; ++k) {
    int* a = k ? I : J;
    bool e1 = (e == 1), e2 = (e == 2);
    a[0] = e1 ? 1 : a[0];
    a[1] = e1 ? 2 : (e2 ? (a[0] == 1 ? 2 : 1) : a[1]);
    a[2] = 6 - a[0] - a[1];
    if (cls == BGB_CLASS_CE) {
      int t = a[0];
      a[0] = a[1];
      a[1] = a[2];
      a[2] = t;
    }
  }
}

__device__ inline void make_chart(const int P[3], Chart& C) {
  const double V[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {0.0, 0.0}};
  for (int u = 0; u < 3; ++u) {
    int p = P[u] - 1;
    p = p < 0 ? 0 : (p > 2 ? 2 : p);
    C.cv[u][0] = V[p][0];
    C.cv[u][1] = V[p][1];
  }
  for (int u = 0; u < 2; ++u) {
    C.ct[u][0] = C.cv[u][0] - C.cv[2][0];
    C.ct[u][1] = C.cv[u][1] - C.cv[2][1];
  }
}


// Region maps of the Sauter-Schwab rules (SauterSchwab.jl:265-297): test/trial chart
// parameters (u1, u2), (v1, v2) and the weight of region r at the 4-D point (h1, h2, h3, xi).
__host__ __device__ __forceinline__ void ss_region(int cls, int r, double h1, double h2, double h3, double xi, double wt,
                                          double& u1, double& u2, double& v1, double& v2, double& mul) {
  const double xi3 = xi * xi * xi;
  if (cls == BGB_CLASS_CV) {
    const double xh1 = xi * h1, xh2 = xi * h2;
    mul = wt * xi3 * h2;
    double a1 = 1 - xi, a2 = xh1, b1 = 1 - xh2, b2 = xh2 * h3;
    if (r == 0) { u1 = a1; u2 = a2; v1 = b1; v2 = b2; }
    else { u1 = b1; u2 = b2; v1 = a1; v2 = a2; }
  } else if (cls == BGB_CLASS_CE) {
    const double xh1 = xi * h1, h12 = h1 * h2, h23 = h2 * h3, h123 = h12 * h3;
    mul = wt * xi3 * (h1 * h1) * h2;
    switch (r) {
      case 0: u1 = 1 - xi; u2 = xh1; v1 = 1 - xi * (1 - h123); v2 = xh1 * h2 * (1 - h3); break;
      case 1: u1 = 1 - xi * (1 - h12); u2 = xh1 * (1 - h2); v1 = 1 - xi; v2 = xh1 * h23; break;
      case 2: u1 = 1 - xi * (1 - h123); u2 = xh1 * h2 * (1 - h3); v1 = 1 - xi; v2 = xh1; break;
      case 3: u1 = 1 - xi * (1 - h123); u2 = xh1 * (1 - h23); v1 = 1 - xi; v2 = xh1 * h2; break;
      default:
        mul = wt * xi3 * (h1 * h1);
        u1 = 1 - xi; u2 = xh1 * h3; v1 = 1 - xi * (1 - h12); v2 = xh1 * (1 - h2);
    }
  } else {
    mul = wt * xi3 * (h1 * h1) * h2;
    const double a = (xi - xi * h1) + xi * h1 * h2, b = 1 - (xi - xi * h1 * h2 * h3), c = xi - xi * h1;
    const double d = xi * h1 * ((1 - h2) + h2 * h3), e = 1 - (xi - xi * h1 * h2), f = xi * h1 * (1 - h2);
    const double g = xi * h1 * (1 - h2 * h3);
    switch (r) {
      case 0: u1 = 1 - xi; u2 = a; v1 = b; v2 = c; break;
      case 1: u1 = b; u2 = c; v1 = 1 - xi; v2 = a; break;
      case 2: u1 = 1 - xi; u2 = d; v1 = e; v2 = f; break;
      case 3: u1 = e; u2 = f; v1 = 1 - xi; v2 = d; break;
      case 4: u1 = b; u2 = g; v1 = 1 - xi; v2 = f; break;
      default: u1 = 1 - xi; u2 = f; v1 = b; v2 = g;
    }
  }
}

// The same permutation from the coincident-vertex mask recorded by the classifier (bit
// (i-1) * 3 + (j-1) set when test vertex i and trial vertex j coincide): pure integer logic.
__host__ __device__ inline void ss_permutation_mask(int cls, int mask, int I[3], int J[3]) {
  I[0] = I[1] = I[2] = 0;
  J[0] = J[1] = J[2] = 0;
  const int cap = (cls == BGB_CLASS_CE) ? 3 : 2;
  int e = 1;
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 3; ++j)
      if ((mask >> ((i - 1) * 3 + (j - 1))) & 1) {
        if (cls == BGB_CLASS_CF) {
          J[i - 1] = j;
        } else if (e <= cap) {
          J[e - 1] = j;
          I[e - 1] = i;
          e += 1;
        }
      }
  if (cls == BGB_CLASS_CF) {
    I[0] = 1;
    I[1] = 2;
    I[2] = 3;
    return;
  }
  for (int k = 0; k < 2; ++k) {
    int* a = k ? I : J;
    const bool e1 = (e == 1), e2 = (e == 2);
    a[0] = e1 ? 1 : a[0];
    a[1] = e1 ? 2 : (e2 ? (a[0] == 1 ? 2 : 1) : a[1]);
    a[2] = 6 - a[0] - a[1];
    if (cls == BGB_CLASS_CE) {
      const int t = a[0];
      a[0] = a[1];
      a[1] = a[2];
      a[2] = t;
    }
  }
}

}  // namespace bgb

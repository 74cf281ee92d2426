// Real solid harmonics for the survey estimator's multipoles (used by survey.cu and by the weighted z pass
// in bin.cu): the 2l+1 real harmonic polynomials h_lm of degree l, and the weight h_lm(r^) of a cell whose
// corner is the offset (px, py, pz) from the observer.
#pragma once
#include <cuda_runtime.h>

// Real harmonic polynomials of degree l (m = 0 .. 2l), with L_l(n.u) = sum_m c_lm h_lm(n) h_lm(u) for unit
// n and u (the factors c_lm are harm_coef in survey.cu).
template <typename R>
__device__ __forceinline__ R harm(int l, int m, R x, R y, R z) {
  const R x2 = x * x, y2 = y * y, z2 = z * z;
  switch (l) {
    case 1:
      return m == 0 ? x : (m == 1 ? y : z);
    case 2:
      switch (m) {
        case 0: return x * y;
        case 1: return y * z;
        case 2: return x * z;
        case 3: return x2 - y2;
        default: return (R)2 * z2 - x2 - y2;
      }
    case 3:
      switch (m) {
        case 0: return x * (x2 - (R)3 * y2);
        case 1: return y * ((R)3 * x2 - y2);
        case 2: return z * (x2 - y2);
        case 3: return x * y * z;
        case 4: return x * ((R)4 * z2 - x2 - y2);
        case 5: return y * ((R)4 * z2 - x2 - y2);
        default: return z * ((R)2 * z2 - (R)3 * x2 - (R)3 * y2);
      }
    default: {
      const R p = x2 + y2;
      switch (m) {
        case 0: return x * y * (x2 - y2);
        case 1: return x2 * x2 - (R)6 * x2 * y2 + y2 * y2;
        case 2: return y * z * ((R)3 * x2 - y2);
        case 3: return x * z * (x2 - (R)3 * y2);
        case 4: return x * y * ((R)6 * z2 - p);
        case 5: return (x2 - y2) * ((R)6 * z2 - p);
        case 6: return y * z * ((R)4 * z2 - (R)3 * p);
        case 7: return x * z * ((R)4 * z2 - (R)3 * p);
        default: return (R)8 * z2 * z2 - (R)24 * z2 * p + (R)3 * p * p;
      }
    }
  }
}

__device__ __forceinline__ float sv_rsqrt(float a) { return rsqrtf(a); }
__device__ __forceinline__ double sv_rsqrt(double a) { return rsqrt(a); }
// h_lm(r^) of a cell, r^ the unit vector from the observer to the cell corner (px, py, pz) (pxy = px^2 +
// py^2). A corner at the observer (r2 == 0) gets r2 = 1, as in the reference, so its harmonics vanish.
template <typename R>
__device__ __forceinline__ R sv_cell_weight(int l, int m, R px, R py, R pxy, R pz) {
  R r2 = pxy + pz * pz;
  if (r2 == (R)0) r2 = (R)1;
  const R inv = sv_rsqrt(r2);
  return harm<R>(l, m, px * inv, py * inv, pz * inv);
}


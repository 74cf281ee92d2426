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

// harm<R>(l, m, x, y, z) as a polynomial in z: c[0] + c[1] z + ... + c[L] z^L, its coefficients from x and y
// (the same polynomials as above, collected by powers of z).
template <int L>
__device__ __forceinline__ void harm_zpoly(int m, float x, float y, float *c) {
  const float x2 = x * x, y2 = y * y, p = x2 + y2;
#pragma unroll
  for (int k = 0; k <= L; k++) c[k] = 0.0f;
  if (L == 1) {
    if (m == 0) c[0] = x;
    else if (m == 1) c[0] = y;
    else c[1] = 1.0f;
  } else if (L == 2) {
    switch (m) {
      case 0: c[0] = x * y; break;
      case 1: c[1] = y; break;
      case 2: c[1] = x; break;
      case 3: c[0] = x2 - y2; break;
      default: c[0] = -p; c[2] = 2.0f; break;
    }
  } else if (L == 3) {
    switch (m) {
      case 0: c[0] = x * (x2 - 3.0f * y2); break;
      case 1: c[0] = y * (3.0f * x2 - y2); break;
      case 2: c[1] = x2 - y2; break;
      case 3: c[1] = x * y; break;
      case 4: c[0] = -x * p; c[2] = 4.0f * x; break;
      case 5: c[0] = -y * p; c[2] = 4.0f * y; break;
      default: c[1] = -3.0f * p; c[3] = 2.0f; break;
    }
  } else {
    switch (m) {
      case 0: c[0] = x * y * (x2 - y2); break;
      case 1: c[0] = x2 * x2 - 6.0f * x2 * y2 + y2 * y2; break;
      case 2: c[1] = y * (3.0f * x2 - y2); break;
      case 3: c[1] = x * (x2 - 3.0f * y2); break;
      case 4: c[0] = -x * y * p; c[2] = 6.0f * x * y; break;
      case 5: c[0] = -(x2 - y2) * p; c[2] = 6.0f * (x2 - y2); break;
      case 6: c[1] = -3.0f * y * p; c[3] = 4.0f * y; break;
      case 7: c[1] = -3.0f * x * p; c[3] = 4.0f * x; break;
      default: c[0] = 3.0f * p * p; c[2] = -24.0f * p; c[4] = 8.0f; break;
    }
  }
}

// The weights of one row of cells (corner offsets px, py fixed, pz varying) for the set (L, m): harm is
// homogeneous of degree L, so h_lm(r^) = P(px, py, pz) / r^L with P = harm_zpoly's polynomial in pz. A
// corner at the observer (r2 == 0) gets r2 = 1, as in sv_cell_weight, where P = 0 for L >= 1.
template <int L>
struct HarmRow {
  float c[L + 1];
  float pxy;
  __device__ __forceinline__ HarmRow(int m, float px, float py) : pxy(px * px + py * py) {
    harm_zpoly<L>(m, px, py, c);
  }
  __device__ __forceinline__ float at(float pz) const {
    float r2 = pxy + pz * pz;
    if (r2 == 0.0f) r2 = 1.0f;
    const float inv = rsqrtf(r2);
    float poly = c[L];
#pragma unroll
    for (int k = L - 1; k >= 0; k--) poly = poly * pz + c[k];
    float invl = inv;
#pragma unroll
    for (int k = 1; k < L; k++) invl *= inv;
    return poly * invl;
  }
};

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


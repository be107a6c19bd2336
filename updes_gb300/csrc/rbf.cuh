// Radial basis functions, monomials and their closed-form derivatives (FP64).
//
// Kernels: updes/utils.py:30-69.  The reference differentiates them with
// jax.grad / jax.jacfwd(jax.grad) and applies nan_to_num
// (updes/operators.py:34-85): at r = 0 every derivative is 0/0 -> NaN -> 0,
// so derivatives are returned as 0 there, while the value keeps phi(0)
// (nan_to_num(log 0 * 0) = 0 for the thin plate spline).
//
// For r > 0, with f = f(r), g1 = f'(r)/r and g2 = (f'' - f'/r)/r^2:
//   grad phi = g1 * s,  d2phi/dx2 = g1 + g2 dx^2,  d2phi/dy2 = g1 + g2 dy^2,
// where s = (dx, dy) = x - center.
#pragma once

#include "common.cuh"

struct RbfG {
  double phi, g1, g2;
};

__device__ __forceinline__ double ipow(double x, int e) {
  double r = 1.0;
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

// r2 = dx^2 + dy^2 > 0 is assumed; the caller handles r2 == 0.
template <int KIND>
__device__ __forceinline__ RbfG rbf_g(double r2, double param, int ip) {
  RbfG o;
  if constexpr (KIND == UPDES_RBF_POLYHARMONIC) {
    // r^k, k = 2a+1 = ip: g1 = k r^(k-2), g2 = k (k-2) r^(k-4)
    const double rinv = rsqrt(r2);
    const double r = r2 * rinv;
    const int a = (ip - 1) / 2;
    const double rk2 = r * ipow(r2, a - 1);  // r^(2a-1) = r^(k-2)
    o.phi = rk2 * r2;
    o.g1 = double(ip) * rk2;
    o.g2 = double(ip) * double(ip - 2) * rk2 * (rinv * rinv);
  } else if constexpr (KIND == UPDES_RBF_GAUSSIAN) {
    const double e2 = param * param;
    const double f = exp(-e2 * r2);
    o.phi = f;
    o.g1 = -2.0 * e2 * f;
    o.g2 = 4.0 * e2 * e2 * f;
  } else if constexpr (KIND == UPDES_RBF_MULTIQUADRIC) {
    const double e2 = param * param;
    const double qi = rsqrt(1.0 + e2 * r2);
    const double q = (1.0 + e2 * r2) * qi;
    o.phi = q;
    o.g1 = e2 * qi;
    o.g2 = -e2 * e2 * qi * qi * qi;
  } else if constexpr (KIND == UPDES_RBF_INVERSE_MULTIQUADRIC) {
    const double e2 = param * param;
    const double qi = rsqrt(1.0 + e2 * r2);
    const double qi3 = qi * qi * qi;
    o.phi = qi;
    o.g1 = -e2 * qi3;
    o.g2 = 3.0 * e2 * e2 * qi3 * qi * qi;
  } else {  // thin plate: r^(2a) log r, a = ip
    const int a = ip;
    const double lr2 = log(r2);  // 2 log r
    const double p1 = ipow(r2, a - 1);
    o.phi = 0.5 * lr2 * p1 * r2;
    o.g1 = p1 * (double(a) * lr2 + 1.0);
    o.g2 = p1 * (double(a) * double(2 * a - 2) * lr2 + double(4 * a - 2)) / r2;
  }
  return o;
}

template <int KIND>
__device__ __forceinline__ double rbf_phi0() {
  return (KIND == UPDES_RBF_POLYHARMONIC || KIND == UPDES_RBF_THIN_PLATE) ? 0.0 : 1.0;
}

// Value of the kernel alone (value rows, Phi block of A, field evaluation).
template <int KIND>
__device__ __forceinline__ double rbf_value(double dx, double dy, double param, int ip) {
  const double r2 = dx * dx + dy * dy;
  if (r2 == 0.0) return rbf_phi0<KIND>();
  if constexpr (KIND == UPDES_RBF_POLYHARMONIC) {
    const double r = sqrt(r2);
    const int a = (ip - 1) / 2;
    return r * ipow(r2, a);
  } else {
    return rbf_g<KIND>(r2, param, ip).phi;
  }
}

// Monomial exponents by id (updes/utils.py:103-132).
__device__ __constant__ int8_t kMonoPx[15] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0, 4, 3, 2, 1, 0};
__device__ __constant__ int8_t kMonoPy[15] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4};

struct MonoT {
  double m, mx, my, mxx, myy;
};

__device__ __forceinline__ MonoT monomial_terms(int k, double x, double y) {
  const int px = kMonoPx[k], py = kMonoPy[k];
  MonoT t;
  const double xp = ipow(x, px), yp = ipow(y, py);
  t.m = xp * yp;
  t.mx = px > 0 ? double(px) * ipow(x, px - 1) * yp : 0.0;
  t.my = py > 0 ? double(py) * xp * ipow(y, py - 1) : 0.0;
  t.mxx = px > 1 ? double(px * (px - 1)) * ipow(x, px - 2) * yp : 0.0;
  t.myy = py > 1 ? double(py * (py - 1)) * xp * ipow(y, py - 2) : 0.0;
  return t;
}

// sin(pi x) (and cos(pi x)) for the element kernels' analytic loads, table-driven.
#pragma once
#include <cstdint>

#include "pxg_sinpi_table.h"

namespace pxg
{
// sin(pi x) and cos(pi x) by the table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point arithmetic", ACM
// TOMS 15 (1989), here for sine and cosine): x = k/64 + d with k = rint(64 x) and
// |d| <= 1/128 (d exact: x and k/64 are within a factor 2 of each other, or k = 0),
// sin(pi x) = S_k cos(pi d) + C_k sin(pi d), cos(pi x) = C_k cos(pi d) - S_k sin(pi d),
// with S_k, C_k the doubles nearest to sin, cos(pi k/64) (k mod 128, from
// pxg_sinpi_table.h) and the series of sin t to t^7 and cos t to t^6 in t = pi d
// (|t| <= pi/128: truncation below 1e-20 and 4e-18).  Near a zero of sin(pi x), k is a
// multiple of 64 and S_k is exactly 0, so no cancellation occurs.  |x| >= 2^40 (tested
// on the exponent bits) and non-finite x: CUDA's sincospi, out of line.
__device__ __noinline__ inline void sinCosPiWide(double x, double * s, double * c) { sincospi(x, s, c); }
__device__ __forceinline__ void sinCosPiTab(double x, double & s, double & c)
{
  if (((uint32_t)__double2hiint(x) & 0x7ff00000u) >= ((1023u + 40u) << 20))
  {
    sinCosPiWide(x, &s, &c);
    return;
  }
  double const kd = rint(64.0 * x);
  double const d = fma(kd, -1.0 / 64.0, x);
  double2 const sc = __ldg(reinterpret_cast<double2 const *>(kSinCosPi64[(long long)kd & 127]));
  double const t = d * 3.141592653589793;
  double const t2 = t * t;
  double const st = fma(t * t2, fma(t2, fma(t2, -1.0 / 5040., 1.0 / 120.), -1.0 / 6.), t);
  double const ct = fma(t2, fma(t2, fma(t2, -1.0 / 720., 1.0 / 24.), -0.5), 1.0);
  s = fma(sc.x, ct, sc.y * st);
  c = fma(sc.y, ct, -(sc.x * st));
}

// sin(pi x) alone, by the same reduction and series
__device__ __forceinline__ double sinPiTab(double x)
{
  if (((uint32_t)__double2hiint(x) & 0x7ff00000u) >= ((1023u + 40u) << 20))
  {
    double s, c;
    sinCosPiWide(x, &s, &c);
    return s;
  }
  double const kd = rint(64.0 * x);
  double const d = fma(kd, -1.0 / 64.0, x);
  double2 const sc = __ldg(reinterpret_cast<double2 const *>(kSinCosPi64[(long long)kd & 127]));
  double const t = d * 3.141592653589793;
  double const t2 = t * t;
  double const st = fma(t * t2, fma(t2, fma(t2, -1.0 / 5040., 1.0 / 120.), -1.0 / 6.), t);
  double const ct = fma(t2, fma(t2, fma(t2, -1.0 / 720., 1.0 / 24.), -0.5), 1.0);
  return fma(sc.x, ct, sc.y * st);
}
} // namespace pxg

// Double-float ("dfl") arithmetic on the FP32 pipe.
//
// GB300 runs FP64 at ~1/64 of its FP32 rate (ncu: FP32:FP64 = 64:1; measured 600 GFMA/s
// FP64 vs 35 TFMA/s FP32).  A value is kept as an unevaluated sum h + l of two floats
// (|l| <= ulp(h)), which carries ~48 significant bits.  The building blocks are the
// classical error-free transformations, written here from their published definitions:
//   - TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + e = a + b exactly, 6 flops;
//   - FastTwoSum (Dekker 1971), valid for |a| >= |b|: 3 flops;
//   - TwoProd with an FMA: p + e = a * b exactly, 2 flops;
// combined into the double-word addition ("sloppy" variant) and multiplication of
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic", ACM TOMS 44(2), 2017 (algorithms 4 and 12).
// Error: a product has relative error <= ~5 * 2^-48; a sum has absolute error
// <= ~2^-47 (|a| + |b|), which is the normwise bound the assembled matrices need
// (agreement with the FP64 reference to 1e-12 of the largest entry).
//
// The intrinsics __fadd_rn / __fmul_rn keep the compiler from contracting or
// reordering the operations of the transformations.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace pxg
{

// the dfl overloads below must not hide the double ones
using ::fabs;
using ::fma;

struct __align__(8) dfl
{
  float h, l;
};

__device__ __forceinline__ dfl dflTwoSum(float a, float b)
{
  float const s = __fadd_rn(a, b);
  float const bb = __fsub_rn(s, a);
  float const e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ dfl dflFastTwoSum(float a, float b)
{
  float const s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b)
{
  dfl const s = dflTwoSum(a.h, b.h);
  return dflFastTwoSum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b)
{
  float const p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return dflFastTwoSum(p, e);
}
__device__ __forceinline__ dfl & operator+=(dfl & a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl & operator-=(dfl & a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl fma(dfl a, dfl b, dfl c) { return a * b + c; }
__device__ __forceinline__ dfl fabs(dfl a) { return a.h < 0.f ? -a : a; }
__device__ __forceinline__ bool operator<(dfl a, float b) { return a.h < b; }

// Fused expressions: the products are formed exactly with FMAs (TwoProd), the high
// parts summed with TwoSum, and everything of order 2^-24 (product errors, cross terms
// a.h * b.l, the low parts) gathered in one float before a single renormalisation.
// Same accuracy class as the chained operations (relative ~2^-47 of the sum of the
// magnitudes), fewer instructions: a*b + c*d 19 instead of 25, the 3-term dot product
// 31 instead of 43 (the compensated dot product of Ogita, Rump and Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26(6), 2005, on double-word inputs).
__device__ __forceinline__ dfl dot2(dfl a, dfl b, dfl c, dfl d)
{
  float const p1 = __fmul_rn(a.h, b.h), p2 = __fmul_rn(c.h, d.h);
  float lo = __fadd_rn(__fmaf_rn(a.h, b.h, -p1), __fmaf_rn(c.h, d.h, -p2));
  dfl const s = dflTwoSum(p1, p2);
  lo = __fadd_rn(lo, s.l);
  lo = __fmaf_rn(a.h, b.l, lo);
  lo = __fmaf_rn(a.l, b.h, lo);
  lo = __fmaf_rn(c.h, d.l, lo);
  lo = __fmaf_rn(c.l, d.h, lo);
  return dflFastTwoSum(s.h, lo);
}
__device__ __forceinline__ dfl dot3(dfl a, dfl b, dfl c, dfl d, dfl e, dfl f)
{
  float const p1 = __fmul_rn(a.h, b.h), p2 = __fmul_rn(c.h, d.h), p3 = __fmul_rn(e.h, f.h);
  float lo = __fadd_rn(__fadd_rn(__fmaf_rn(a.h, b.h, -p1), __fmaf_rn(c.h, d.h, -p2)), __fmaf_rn(e.h, f.h, -p3));
  dfl const s1 = dflTwoSum(p1, p2);
  dfl const s2 = dflTwoSum(s1.h, p3);
  lo = __fadd_rn(lo, __fadd_rn(s1.l, s2.l));
  lo = __fmaf_rn(a.h, b.l, lo);
  lo = __fmaf_rn(a.l, b.h, lo);
  lo = __fmaf_rn(c.h, d.l, lo);
  lo = __fmaf_rn(c.l, d.h, lo);
  lo = __fmaf_rn(e.h, f.l, lo);
  lo = __fmaf_rn(e.l, f.h, lo);
  return dflFastTwoSum(s2.h, lo);
}
__device__ __forceinline__ double dot2(double a, double b, double c, double d) { return a * b + c * d; }
__device__ __forceinline__ double dot3(double a, double b, double c, double d, double e, double f)
{
  return a * b + c * d + e * f;
}

// Running sum of double-float terms: TwoSum on the high parts, the errors and the low
// parts in one float (8 instructions a term instead of 11), one renormalisation at the end.
struct DflSum
{
  float s, c;
};
__device__ __forceinline__ DflSum sumStart(dfl t) { return DflSum{t.h, t.l}; }
__device__ __forceinline__ void sumAdd(DflSum & a, dfl t)
{
  dfl const s = dflTwoSum(a.s, t.h);
  a.s = s.h;
  a.c = __fadd_rn(a.c, __fadd_rn(s.l, t.l));
}
__device__ __forceinline__ dfl sumEnd(DflSum a) { return dflFastTwoSum(a.s, a.c); }
__device__ __forceinline__ double sumStart(double t) { return t; }
__device__ __forceinline__ void sumAdd(double & a, double t) { a += t; }
__device__ __forceinline__ double sumEnd(double a) { return a; }

// The same with a sign on each term, given as the bits of the float +1 or -1: the
// products with +-1 are exact, so that the FMAs below round like the additions of
// sumAdd on the negated term, and the sign costs no instruction.
__device__ __forceinline__ DflSum sumStartS(dfl t, uint32_t sg)
{
  float const f = __uint_as_float(sg);
  return DflSum{__fmul_rn(f, t.h), __fmul_rn(f, t.l)};
}
__device__ __forceinline__ void sumAddS(DflSum & a, dfl t, uint32_t sg)
{
  float const f = __uint_as_float(sg);
  float const s = __fmaf_rn(f, t.h, a.s);
  float const bb = __fsub_rn(s, a.s);
  float const e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fmaf_rn(f, t.h, -bb));
  a.s = s;
  a.c = __fadd_rn(a.c, __fmaf_rn(f, t.l, e));
}
__device__ __forceinline__ double sumStartS(double t, uint32_t sg) { return (sg >> 31) ? -t : t; }
__device__ __forceinline__ void sumAddS(double & a, double t, uint32_t sg) { a += (sg >> 31) ? -t : t; }

// 1/a: float reciprocal refined by one Newton step in double-float
__device__ __forceinline__ dfl rcp(dfl a)
{
  float const r0 = __frcp_rn(a.h);
  dfl const one{1.f, 0.f};
  dfl const e = one - a * dfl{r0, 0.f};
  return dfl{r0, 0.f} + dfl{r0, 0.f} * e;
}
__device__ __forceinline__ double rcp(double a) { return 1.0 / a; }

// ---------------------------------------------------------------- conversions
// Compile-time constants: split a double into its nearest float and the remainder.
template <typename T>
__host__ __device__ constexpr T cst(double x);
template <>
__host__ __device__ constexpr double cst<double>(double x)
{
  return x;
}
template <>
__host__ __device__ constexpr dfl cst<dfl>(double x)
{
  return dfl{(float)x, (float)(x - (double)(float)x)};
}

// Rare path of toDfl (magnitudes outside 2^-74 .. 2^127): kept out of line, so that
// the compiler does not predicate its FP64-pipe conversions into every call.
static __device__ __noinline__ dfl toDflSlow(double x)
{
  float const h = __double2float_rn(x);
  return dfl{h, __double2float_rn(x - (double)h)};
}

// Run-time double -> dfl with integer operations only (the FP64 pipe, which also
// executes F2F conversions on GB300, stays free): the high float takes the top 24
// significant bits (truncated), the low float the remaining 29 bits times 2^(e-52).
// Exact to 2^-47 relative for normal doubles of magnitude 2^-74 .. 2^127; zero and
// subnormals give zero, other values outside that range take toDflSlow.
__device__ __forceinline__ dfl toDfl(double x)
{
  unsigned long long const b = (unsigned long long)__double_as_longlong(x);
  unsigned const hi = (unsigned)(b >> 32), lo = (unsigned)b;
  int const e = (int)((hi >> 20) & 0x7ffu);
  if (e != 0 && (e < 949 || e > 1150))
    return toDflSlow(x);
  unsigned const sign = hi & 0x80000000u;
  float const h = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
  float const scale = __uint_as_float((unsigned)(e - 1075 + 127) << 23);
  float const l = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu), scale);
  return e == 0 ? dfl{0.f, 0.f} : dfl{h, sign ? -l : l};
}

// float -> double by integer operations, branch-free (exact; subnormal floats become
// zero, infinities and NaNs keep their class)
__device__ __forceinline__ double f2dExact(float f)
{
  unsigned const u = __float_as_uint(f);
  unsigned const a = u & 0x7fffffffu;
  unsigned hi = (a >> 3) + 0x38000000u; // exponent rebased by 1023 - 127
  hi = a >= 0x7f800000u ? ((a >> 3) | 0x7ff00000u) : hi;
  hi = a < 0x00800000u ? 0u : hi;
  unsigned const lo = a < 0x00800000u ? 0u : u << 29;
  return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}

// dfl -> double: exact conversions of both parts, one FP64 addition
__device__ __forceinline__ double toDouble(dfl a) { return f2dExact(a.h) + f2dExact(a.l); }

// float -> double for the low part of a double-float value, by integer operations: the
// exponent rebased by 1023 - 127 and the significand shifted into place.  Exact for
// normal floats; +-0 stays +-0.  A subnormal low part (|l| < 2^-126) comes out wrong by
// less than 2^-126 in absolute terms, which the FP64 sum with the high part absorbs
// unless that is itself below ~2^-73.  The low part is finite whenever the high part
// is, and a non-finite high part makes the sum non-finite.
__device__ __forceinline__ double f2dLow(float f)
{
  unsigned const u = __float_as_uint(f);
  // the arithmetic shift leaves the sign in bit 31 and copies it into bits 30..28,
  // which the mask clears
  unsigned hi = ((unsigned)((int)u >> 3) & 0x8fffffffu) + 0x38000000u;
  hi = (u << 1) == 0u ? (u & 0x80000000u) : hi;
  return __hiloint2double((int)hi, (int)(u << 29));
}

// dfl -> double with the high part by the hardware conversion (exact for every float,
// on the FP64 pipe) and the low part by f2dLow: fewer integer operations than toDouble,
// one more FP64-pipe instruction.  Measured per kernel (128^3 Q1: 2.18 -> 2.14 ms with it
// for the entries; P1 tetrahedra 0.78 -> 0.80 ms, so the others keep toDouble).
__device__ __forceinline__ double toDoubleMixed(dfl a) { return (double)a.h + f2dLow(a.l); }
__device__ __forceinline__ double toDoubleMixed(double a) { return a; }
__device__ __forceinline__ double toDouble(double a) { return a; }

template <typename T>
__device__ __forceinline__ T fromDouble(double x);
template <>
__device__ __forceinline__ double fromDouble<double>(double x)
{
  return x;
}
template <>
__device__ __forceinline__ dfl fromDouble<dfl>(double x)
{
  return toDfl(x);
}

} // namespace pxg

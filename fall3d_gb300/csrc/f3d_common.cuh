// f3d_common.cuh -- device helpers shared by the transport kernels.
//
// Semantics that the reference leaves to the Fortran processor are fixed
// here exactly as in the CPU oracle:
//  * MAX/MIN follow gfortran 4.8 (the compiler of the reference build):
//    mvar = a; if (b .op. mvar .or. isnan(mvar)) mvar = b.  They return the
//    non-NaN operand and keep the first operand on ties (so MAX(0,-0) = +0).
//  * SIGN(1,b) is copysign(1,b), with a NaN b counted as positive (the CUDA
//    and aarch64 default NaN is positive).
// The binary64 kernels are compiled with --fmad=false so that every
// expression is rounded operation by operation, as the Fortran is.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define F3D_HD __host__ __device__ __forceinline__

template <class T>
F3D_HD T fmax2(T a, T b) { return (b > a || isnan(a)) ? b : a; }
template <class T>
F3D_HD T fmin2(T a, T b) { return (b < a || isnan(a)) ? b : a; }
template <class T>
F3D_HD T sign1(T b) { return isnan(b) ? T(1) : (signbit(b) ? T(-1) : T(1)); }
template <class T>
F3D_HD T fabs_t(T x) { return x < T(0) ? -x : (x == T(0) ? T(0) : x); }

// |x| and x > 0 of binary64 values on the bit patterns (integer operations;
// the binary64 pipe is the plain form's bottleneck): clearing the sign bit
// is fabs, NaN included; x > 0 holds exactly for the patterns of positive
// finite values and +inf, 1 .. 0x7ff0000000000000 as signed integers.
__device__ __forceinline__ double absd(double x) {
  return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ float absd(float x) { return fabsf(x); }
__device__ __forceinline__ bool gt0(double x) {
  const long long b = __double_as_longlong(x);
  return b > 0 && b <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool gt0(float x) { return x > 0.0f; }

// RN(a/b) from y = RN(1/b) without a division (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J.
// Res. Develop. 34(1), 1990): q0 = RN(a*y) is within 1.5 ulp of a/b;
// q1 = RN(q0 + RN(a - b*q0)*y) is within 1 ulp; and when y is within half
// an ulp of 1/b and q1 within one ulp of a/b, the residual a - b*q1 is
// exact and RN(q1 + (a - b*q1)*y) = RN(a/b).  A zero a gives a*y (the
// signed zero of a/b).  Operands outside [2^-900, 2^900] in
// magnitude (where a residual could leave the normal range), or
// non-finite, take the IEEE division: the result is RN(a/b) for all inputs.
// the rare paths out of line, so that they cost the callers no registers
static __device__ __noinline__ double div_ieee(double a, double b) { return a / b; }
static __device__ __noinline__ double minmod_div_ieee(double a, double b, double dx) {
  const double dr = a / dx, dl = b / dx;
  return 0.5 * (sign1(dr) + sign1(dl)) * fmin2(fabs(dr), fabs(dl));
}
__device__ __forceinline__ bool div_in_range(double x) {
  const unsigned long long m = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  return m - 0x07b0000000000000ULL <= 0x7080000000000000ULL;  // 2^-900 <= |x| <= 2^900
}
__device__ __forceinline__ double div_rn_recip(double a, double b, double y) {
  if (!div_in_range(b)) return div_ieee(a, b);  // y may be inexact, infinite or zero
  const double q0 = a * y;
  if ((__double_as_longlong(a) & 0x7fffffffffffffffLL) == 0) return q0;
  if (!(div_in_range(a) && div_in_range(q0))) return div_ieee(a, b);
  const double q1 = fma(fma(-q0, b, a), y, q0);
  return fma(fma(-q1, b, a), y, q1);
}

// The slope limiter of advctx.f90:34-40 (and advcty), with
// deltar = a/dx, deltal = b/dx:
//   sigma = 0.5*(SIGN(1,deltar)+SIGN(1,deltal))*MIN(|deltar|,|deltal|).
// For dx > 0, x -> RN(x/dx) is monotonic and keeps the sign of x (zeros and
// underflows included), so SIGN(1,RN(a/dx)) = SIGN(1,a) and
// MIN(|RN(a/dx)|,|RN(b/dx)|) = RN(m/dx) with m = MIN(|a|,|b|) under the same
// MIN rule (NaN operands included): one division instead of two, the same
// bits.  Other dx take the reference's two divisions.
template <class T>
__device__ __forceinline__ T minmod_div(T a, T b, T dx, T rdx) {
  (void)rdx;
  if (!(dx > T(0))) {
    const T dr = a / dx, dl = b / dx;
    return T(0.5) * (sign1(dr) + sign1(dl)) * fmin2(absd(dr), absd(dl));
  }
  return T(0.5) * (sign1(a) + sign1(b)) * (fmin2(absd(a), absd(b)) / dx);
}

// The limiter 0.5*(SIGN(1,dr)+SIGN(1,dl))*MIN(|dr|,|dl|) (advctzc.f90:44).
template <class T>
__device__ __forceinline__ T minmod_ref(T dr, T dl) {
  return T(0.5) * (sign1(dr) + sign1(dl)) * fmin2(absd(dr), absd(dl));
}

// binary64 forms of both limiters on the bit patterns.  GB300 issues
// binary64 arithmetic at 1/64 of the binary32 rate while integer operations
// run at full rate, so the sign and minimum logic moves to integers.  For
// finite operands (the others take the formula):
//  * 0.5*(s_r + s_l) is +-1 when the sign bits agree (SIGN(1,-0) = -1), and
//    +0 when they differ, where +0 * (a finite m >= 0) = +0;
//  * |x| of finite binary64 values orders like the integers of their bit
//    patterns with the sign cleared, and MIN keeps the first operand on
//    ties, which has the same bits as the second;
//  * (+-1) * m is m with the sign bit of the first operand.
// The results are the formula's bits.
__device__ __forceinline__ double minmod_ref(double dr, double dl) {
  const long long br = __double_as_longlong(dr), bl = __double_as_longlong(dl);
  const long long mr = br & 0x7fffffffffffffffLL, ml = bl & 0x7fffffffffffffffLL;
  if (mr >= 0x7ff0000000000000LL || ml >= 0x7ff0000000000000LL)
    return 0.5 * (sign1(dr) + sign1(dl)) * fmin2(fabs(dr), fabs(dl));
  if ((br ^ bl) < 0) return 0.0;
  return __longlong_as_double((ml < mr ? ml : mr) | (br & (long long)0x8000000000000000ULL));
}
// rdx = RN(1/dx): the division by dx goes through div_rn_recip.
__device__ __forceinline__ double minmod_div(double a, double b, double dx, double rdx) {
  const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b);
  const long long ma = ba & 0x7fffffffffffffffLL, mb = bb & 0x7fffffffffffffffLL;
  if (!(dx > 0.0) || ma >= 0x7ff0000000000000LL || mb >= 0x7ff0000000000000LL)
    return minmod_div_ieee(a, b, dx);
  const double q = div_rn_recip(__longlong_as_double(mb < ma ? mb : ma), dx, rdx);  // >= 0, +inf on overflow
  if ((ba ^ bb) < 0) return isinf(q) ? 0.0 * q : 0.0;             // 0 * q
  return __longlong_as_double(__double_as_longlong(q) | (ba & (long long)0x8000000000000000ULL));
}

// Grid geometry of one scenario (interior nx, ny, nz; halo arrays are
// (nx+2)(ny+2)(nz+2), x fastest).
struct Dims {
  int nx, ny, nz;
  F3D_HD long long C(int i, int j, int k) const {
    return (long long)i + (long long)(nx + 2) * ((long long)j + (long long)(ny + 2) * k);
  }
  F3D_HD long long M(int i, int j, int k) const {
    return (long long)(i - 1) + (long long)nx * ((long long)(j - 1) + (long long)ny * (k - 1));
  }
  F3D_HD long long P(int i, int j) const { return (long long)(i - 1) + (long long)nx * (j - 1); }
  F3D_HD long long halo() const { return (long long)(nx + 2) * (ny + 2) * (nz + 2); }
  F3D_HD long long cells() const { return (long long)nx * ny * nz; }
  F3D_HD long long plane() const { return (long long)nx * ny; }
};

// Double-double accumulator (Knuth TwoSum): sums that are exact to well
// below one binary64 ulp, and independent of the reduction order up to the
// final rounding.  Used for the mass budgets.
struct DD {
  double hi, lo;
};
F3D_HD DD dd_zero() { return DD{0.0, 0.0}; }
F3D_HD DD dd_add_d(DD a, double b) {
  double s = a.hi + b;
  double bb = s - a.hi;
  double err = (a.hi - (s - bb)) + (b - bb);
  double lo = a.lo + err;
  double hi = s + lo;
  lo = lo - (hi - s);
  return DD{hi, lo};
}
F3D_HD DD dd_add(DD a, DD b) {
  double s = a.hi + b.hi;
  double bb = s - a.hi;
  double err = (a.hi - (s - bb)) + (b.hi - bb);
  double lo = a.lo + b.lo + err;
  double hi = s + lo;
  lo = lo - (hi - s);
  return DD{hi, lo};
}
__device__ __forceinline__ DD dd_shfl_down(DD v, int off) {
  return DD{__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off)};
}

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

__device__ __forceinline__ double absd(double x) { return fabs(x); }
__device__ __forceinline__ float absd(float x) { return fabsf(x); }

// The slope limiter of advctx.f90:34-40 (and advcty), with
// deltar = a/dx, deltal = b/dx:
//   sigma = 0.5*(SIGN(1,deltar)+SIGN(1,deltal))*MIN(|deltar|,|deltal|).
// For dx > 0, x -> RN(x/dx) is monotonic and keeps the sign of x (zeros and
// underflows included), so SIGN(1,RN(a/dx)) = SIGN(1,a) and
// MIN(|RN(a/dx)|,|RN(b/dx)|) = RN(m/dx) with m = MIN(|a|,|b|) under the same
// MIN rule (NaN operands included): one division instead of two, the same
// bits.  Other dx take the reference's two divisions.
template <class T>
__device__ __forceinline__ T minmod_div(T a, T b, T dx) {
  if (!(dx > T(0))) {
    const T dr = a / dx, dl = b / dx;
    return T(0.5) * (sign1(dr) + sign1(dl)) * fmin2(absd(dr), absd(dl));
  }
  return T(0.5) * (sign1(a) + sign1(b)) * (fmin2(absd(a), absd(b)) / dx);
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

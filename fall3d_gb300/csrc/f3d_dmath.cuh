// f3d_dmath.cuh -- table-driven binary64 logarithm and exponential for the
// settling-velocity iteration (vsettl), whose cost on GB300 is the number of
// binary64 operations per drag iteration.
//
// Methods (published):
//  * exp: P. T. P. Tang, "Table-driven implementation of the exponential
//    function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989.
//    a = (64 m + j) ln2/64 + r with |r| <= ln2/128, exp(a) = 2^m 2^(j/64) e^r,
//    2^(j/64) from a 64-entry table, e^r - 1 by its Taylor series to r^6.
//  * log: P. T. P. Tang, "Table-driven implementation of the logarithm
//    function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990.
//    x = 2^k z, z in [1, 2); the top seven fraction bits of z pick the
//    breakpoint c = 1 + (j + 1/2)/128, r = z/c - 1 (one fused multiply-add
//    with the tabulated reciprocal), |r| <= 2^-8, and
//    log x = k ln2 - log(1/c) + log1p(r), log1p by its Taylor series to r^7.
//
// Accuracy: the truncated series are below 2^-64; the results are within
// a few units in the last place (the tests bound both against a
// high-precision evaluation).  Arguments outside the reduced ranges (log of
// a non-normal or huge value, exp beyond +-700) fall back to CUDA's log/exp.
#pragma once

namespace f3d {

struct DMathTab {
  double invc[128];  // RN(1 / (1 + (j + 1/2)/128))
  double logc[128];  // RN(-log(invc[j]))
  double e2[64];     // RN(2^(j/64))
};

// Fills the tables with all threads of the block (the caller synchronises).
__device__ __forceinline__ void dmath_tab_init(DMathTab& t) {
  for (int j = threadIdx.x; j < 128; j += blockDim.x) {
    const double ic = 1.0 / (1.0 + (j + 0.5) / 128.0);
    t.invc[j] = ic;
    t.logc[j] = -log(ic);
  }
  for (int j = threadIdx.x; j < 64; j += blockDim.x) t.e2[j] = exp2(j / 64.0);
}

__device__ __forceinline__ double dm_log(const DMathTab& t, double x) {
  const long long ix = __double_as_longlong(x);
  // 2^-1000 <= x <= 2^1000 (positive, normal, finite), as one unsigned compare
  if ((unsigned long long)(ix - 0x0170000000000000LL) > 0x7d00000000000000ULL) return log(x);
  const int k = (int)(ix >> 52) - 1023;
  const int j = (int)((ix >> 45) & 127);
  const double z = __longlong_as_double((ix & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const double r = fma(z, t.invc[j], -1.0);
  double q = fma(r, 1.0 / 7.0, -1.0 / 6.0);
  q = fma(q, r, 1.0 / 5.0);
  q = fma(q, r, -1.0 / 4.0);
  q = fma(q, r, 1.0 / 3.0);
  q = fma(q, r, -1.0 / 2.0);
  const double p = fma(q, r * r, r);  // log1p(r)
  const double kd = (double)k;
  const double hi = fma(kd, 0x1.62e42fefa3800p-1, t.logc[j]);  // kd * ln2_hi is exact
  const double lo = fma(kd, 0x1.ef35793c76730p-45, p);
  return hi + lo;
}

__device__ __forceinline__ double dm_exp(const DMathTab& t, double a) {
  // |a| <= 700 (NaN excluded), as one integer compare on the magnitude bits
  if ((__double_as_longlong(a) & 0x7fffffffffffffffLL) > 0x4085e00000000000LL) return exp(a);
  const double shift = 0x1.8p52;                        // rounds a*64/ln2 to an integer
  const double kd = fma(a, 0x1.71547652b82fep+6, shift);
  const long long n = __double_as_longlong(kd) - __double_as_longlong(shift);
  const double kn = kd - shift;
  double r = fma(kn, -0x1.62e42fefa0000p-7, a);        // kn * (ln2/64)_hi is exact
  r = fma(kn, -0x1.cf79abc9e3b3ap-46, r);
  double q = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  q = fma(q, r, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  const double em1 = fma(q, r * r, r);  // e^r - 1
  const long long m52 = (long long)((unsigned long long)(n >> 6) << 52);  // 2^m in the exponent field
  const double s = __longlong_as_double(__double_as_longlong(t.e2[n & 63]) + m52);
  return fma(s, em1, s);
}

}  // namespace f3d

// f3d_budget.cu -- mass budgets, CFL step and output fields.
//
// The reference accumulates its budgets sequentially in binary64
// (Sources/cmass2d.f90:42-104, Sources/cmass3d.f90:29-47).  Here each sum is
// a deterministic two-level reduction in double-double (TwoSum), i.e. the
// exact sum rounded once; it differs from the reference's sequential
// rounding by at most (N-1)*u*sum|terms| (all cmass2d/cmass3d terms are >= 0
// after the clip, so that bound is relative to the result).  The grid shape
// depends only on the problem size, so results are reproducible run to run.
#include <algorithm>

#include "f3d_internal.h"

namespace f3d {

namespace {
constexpr int RB = 256;   // threads per reduction block
constexpr int RMAXB = 1024;  // reduction blocks

int reduce_blocks(long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + RB - 1) / RB, RMAXB));
}

template <int NS>
__device__ void block_store_dd(DD (&v)[NS], DD* partial) {
  __shared__ DD sh[RB / 32][NS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < NS; ++s)
    for (int off = 16; off > 0; off >>= 1) v[s] = dd_add(v[s], dd_shfl_down(v[s], off));
  if (lane == 0)
#pragma unroll
    for (int s = 0; s < NS; ++s) sh[wid][s] = v[s];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      DD a = sh[0][s];
      for (int w = 1; w < RB / 32; ++w) a = dd_add(a, sh[w][s]);
      partial[(long long)blockIdx.x * NS + s] = a;
    }
  }
}

// Sums nblk partials of NS sums; out[s] = (hi(sum_s) * f0) * f1, or with
// accum, out[s] = out[s] + hi(sum_s) (outmass = outmass + sum(mymass),
// cmass2d.f90:104).
template <int NS>
__global__ void k_reduce_finish(const DD* partial, int nblk, double f0, double f1, double* out,
                                int accum) {
  DD v[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) v[s] = dd_zero();
  for (int b = threadIdx.x; b < nblk; b += RB)
#pragma unroll
    for (int s = 0; s < NS; ++s) v[s] = dd_add(v[s], partial[(long long)b * NS + s]);
  __shared__ DD sh[RB / 32][NS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < NS; ++s)
    for (int off = 16; off > 0; off >>= 1) v[s] = dd_add(v[s], dd_shfl_down(v[s], off));
  if (lane == 0)
#pragma unroll
    for (int s = 0; s < NS; ++s) sh[wid][s] = v[s];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      DD a = sh[0][s];
      for (int w = 1; w < RB / 32; ++w) a = dd_add(a, sh[w][s]);
      if (accum)
        out[s] = out[s] + a.hi;
      else
        out[s] = a.hi * f0 * f1;
    }
  }
}
}  // namespace

size_t reduce_scratch_bytes(long long nterms, int nsums) {
  return sizeof(DD) * (size_t)reduce_blocks(nterms) * nsums + 256;
}

// ----------------------------------------------------------- cmass2d
// Terms of Sources/cmass2d.f90:42-102: x faces (ic, j, k, left/right),
// y faces (ic, i, k, down/up), top (ic, i, j).  The work is split by face
// cell ("item"): an item computes its class-independent factor
// (dt*area)*velo (faces) or dt*area (top) once and walks the classes, so
// each term is still ((dt*area)*velo)*conc rounded as the reference writes
// it.  A zero concentration (inflow faces, cells the plume has not
// reached) gives an exact zero term, which leaves the sum unchanged and is
// skipped.  Items: [0, nT) top (i fastest), then x faces (j fastest, left
// half first), then y faces (i fastest, down half first).
struct Cm2Items {
  int nT, nX, nY;  // top items, x-face items, y-face items
};
__host__ __device__ inline Cm2Items cm2_items(const Dims& d, int iz_loc, int nz_loc) {
  Cm2Items r;
  r.nT = (iz_loc + nz_loc - 1 == d.nz) ? d.nx * d.ny : 0;
  r.nX = 2 * d.ny * nz_loc;
  r.nY = 2 * d.nx * nz_loc;
  return r;
}

// Cascaded TwoSum (Ogita, Rump and Oishi, "Accurate sum and dot product",
// SIAM J. Sci. Comput. 26 (2005), Algorithm 4.4): s carries the running
// binary64 sum, e the exact rounding errors of its additions summed in
// binary64; s + e is as accurate as a sum in twice the working precision.
struct DS {
  double s, e;
};
__device__ __forceinline__ void ds_add(DS& a, double b) {
  const double s = a.s + b;
  const double bb = s - a.s;
  a.e = a.e + ((a.s - (s - bb)) + (b - bb));
  a.s = s;
}
__device__ __forceinline__ DD ds_dd(DS a) {
  const double hi = a.s + a.e;
  return DD{hi, a.e - (hi - a.s)};
}

// the terms of one side-face cell, classes in order: +-(w*conc)
template <class T>
__device__ __forceinline__ void face_terms(const T* cc, long long hb, int nc_loc, double w, int side,
                                           DS& acc) {
  for (int q0 = 0; q0 < nc_loc; q0 += 4) {
    T cv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) cv[u] = q0 + u < nc_loc ? cc[(q0 + u) * hb] : T(0);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (cv[u] == T(0)) continue;
      const double t = w * (double)cv[u];
      ds_add(acc, side ? t : -t);
    }
  }
}

// Block sum of the threads' accumulators into partial[blockIdx.x]; a warp
// whose accumulators are all zero contributes an exact zero without the
// binary64 shuffle reduction.
__device__ void block_store_ds(DS a, DD* partial) {
  __shared__ DD sh[RB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  DD v = dd_zero();
  if (__any_sync(0xffffffffu, a.s != 0.0 || a.e != 0.0)) {
    v = ds_dd(a);
    for (int off = 16; off > 0; off >>= 1) v = dd_add(v, dd_shfl_down(v, off));
  }
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    DD r = sh[0];
    for (int w = 1; w < RB / 32; ++w) r = dd_add(r, sh[w]);
    partial[blockIdx.x] = r;
  }
}

template <class T>
__device__ __forceinline__ void cmass2d_item(int u, const Cm2Items& it, const T* c, const double* vx,
                                             const double* vy, const double* vz, const double* vset,
                                             const Dims& d, int ic_loc, int nc_loc, int iz_loc,
                                             int nz_loc, double dx, double dy, const double* dz,
                                             double dt, DS& acc) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long hb = d.halo(), s3 = d.cells();
  const T* c0 = c + (long long)(ic_loc - 1) * hb;
  if (u < it.nT) {
    const int i = u % nx + 1, j = u / nx + 1;
    double faty = 1.0;
    if (j == 1 || j == ny) faty = 0.5;
    double fatx = 1.0;
    if (i == 1 || i == nx) fatx = 0.5;
    const double area = fatx * faty * dx * dy;
    const double da = dt * area;
    const long long m = d.M(i, j, nz);
    const double w = vz[m];
    const double* vs = vset + (long long)(ic_loc - 1) * s3 + m;
    const T* cc = c0 + d.C(i, j, nz + 1);
    for (int q0 = 0; q0 < nc_loc; q0 += 4) {
      T cv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) cv[u] = q0 + u < nc_loc ? cc[(q0 + u) * hb] : T(0);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (cv[u] == T(0)) continue;  // an exact zero term (finite velocities)
        const double velo = w + vs[(q0 + u) * s3];
        ds_add(acc, da * velo * (double)cv[u]);
      }
    }
    return;
  }
  u -= it.nT;
  if (u < it.nX) {
    const int half = it.nX / 2, side = u >= half;
    const int v = side ? u - half : u;
    const int j = v % ny + 1, k = v / ny + iz_loc;
    double faty = 1.0;
    if (j == 1 || j == ny) faty = 0.5;
    const double area = faty * dy * 0.5 * (dz[k] + dz[k - 1]);
    const double w = dt * area * vx[d.M(side ? nx : 1, j, k)];
    const T* cc = c0 + d.C(side ? nx + 1 : 0, j, k);
    face_terms<T>(cc, hb, nc_loc, w, side, acc);
    return;
  }
  u -= it.nX;
  const int half = it.nY / 2, side = u >= half;
  const int v = side ? u - half : u;
  const int i = v % nx + 1, k = v / nx + iz_loc;
  double fatx = 1.0;
  if (i == 1 || i == nx) fatx = 0.5;
  const double area = fatx * dx * 0.5 * (dz[k] + dz[k - 1]);
  const double w = dt * area * vy[d.M(i, side ? ny : 1, k)];
  const T* cc = c0 + d.C(i, side ? ny + 1 : 0, k);
  face_terms<T>(cc, hb, nc_loc, w, side, acc);
}

template <class T>
__global__ void k_cmass2d(const T* c, const double* vx, const double* vy, const double* vz,
                          const double* vset, Dims d, int ic_loc, int nc_loc, int iz_loc,
                          int nz_loc, double dx, double dy, const double* dz, double dt,
                          DD* partial) {
  const Cm2Items it = cm2_items(d, iz_loc, nz_loc);
  const int ntot = it.nT + it.nX + it.nY;
  DS acc{0.0, 0.0};
  for (int u = blockIdx.x * RB + threadIdx.x; u < ntot; u += gridDim.x * RB)
    cmass2d_item<T>(u, it, c, vx, vy, vz, vset, d, ic_loc, nc_loc, iz_loc, nz_loc, dx, dy, dz, dt,
                    acc);
  block_store_ds(acc, partial);
}

// Batched form: scenario blockIdx.y, its outflow summed over gridDim.x
// blocks; the step's result is in the buffer the fused kernel wrote
// (bstep even: c_b, odd: c_a).
__global__ void k_cmass2d_batch(const BatchAux* tab, const int* bstep, DD* partial) {
  const BatchAux& b = tab[blockIdx.y];
  const float* c = (bstep[blockIdx.y] & 1) ? b.c_a : b.c_b;
  const Dims d = b.d;
  const Cm2Items it = cm2_items(d, 1, d.nz);
  const int ntot = it.nT + it.nX + it.nY;
  DS acc{0.0, 0.0};
  for (int u = blockIdx.x * RB + threadIdx.x; u < ntot; u += gridDim.x * RB)
    cmass2d_item<float>(u, it, c, b.vx, b.vy, b.vz, b.vset, d, 1, b.nc, 1, d.nz, b.dX1, b.dX2, b.dz,
                        b.dt, acc);
  block_store_ds(acc, partial + (long long)blockIdx.y * gridDim.x);
}

// outmass = outmass + sum (cmass2d.f90:104), one block per scenario
__global__ void k_cmass2d_batch_finish(const BatchAux* tab, const DD* partial, int nblk) {
  const DD* p = partial + (long long)blockIdx.x * nblk;
  DD v[1] = {dd_zero()};
  for (int b = threadIdx.x; b < nblk; b += RB) v[0] = dd_add(v[0], p[b]);
  __shared__ DD sh[RB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) v[0] = dd_add(v[0], dd_shfl_down(v[0], off));
  if (lane == 0) sh[wid] = v[0];
  __syncthreads();
  if (threadIdx.x == 0) {
    DD a = sh[0];
    for (int w = 1; w < RB / 32; ++w) a = dd_add(a, sh[w]);
    double* out = tab[blockIdx.x].outmass;
    *out = *out + a.hi;
  }
}

size_t cmass2d_scratch_bytes(Dims d, int iz_loc, int nz_loc) {
  const Cm2Items it = cm2_items(d, iz_loc, nz_loc);
  return reduce_scratch_bytes((long long)it.nT + it.nX + it.nY, 1);
}

template <class T>
void launch_cmass2d(const T* c, const double* vx, const double* vy, const double* vz,
                    const double* vset, Dims d, int ic_loc, int nc_loc, int iz_loc, int nz_loc,
                    double dx, double dy, const double* dz, double dt, void* scratch,
                    double* out, cudaStream_t s) {
  const Cm2Items it = cm2_items(d, iz_loc, nz_loc);
  const int nb = reduce_blocks((long long)it.nT + it.nX + it.nY);
  DD* partial = reinterpret_cast<DD*>(scratch);
  k_cmass2d<T><<<nb, RB, 0, s>>>(c, vx, vy, vz, vset, d, ic_loc, nc_loc, iz_loc, nz_loc, dx, dy, dz,
                                 dt, partial);
  k_reduce_finish<1><<<1, RB, 0, s>>>(partial, nb, 1.0, 1.0, out, 1);
  count_launch(2);
}

// ----------------------------------------------------------- cmass3d
// Sources/cmass3d.f90:29-53: per (i,j,ic) the column trapezoid zmass is
// accumulated sequentially in k exactly as the reference does; the sums
// over (i,j,ic) are the reductions.
template <class T>
__global__ void k_cmass3d(const T* c, const double* cload, const double* cdry, const double* cwet,
                          Dims d, int nc, const double* dz, DD* partial) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long hb = d.halo(), pl = d.plane();
  DD acc[4] = {dd_zero(), dd_zero(), dd_zero(), dd_zero()};
  const long long ntot = pl * nc;
  for (long long t = blockIdx.x * (long long)RB + threadIdx.x; t < ntot;
       t += (long long)gridDim.x * RB) {
    const long long p = t % pl;
    const int ic = (int)(t / pl) + 1;
    const int i = (int)(p % nx) + 1, j = (int)(p / nx) + 1;
    double fatx = 1.0;
    if (i == 1 || i == nx) fatx = 0.5;
    double faty = 1.0;
    if (j == 1 || j == ny) faty = 0.5;
    const T* cc = c + (long long)(ic - 1) * hb;
    double zmass = 0.0;
    double ck = (double)cc[d.C(i, j, 1)];
    for (int k = 1; k <= nz - 1; ++k) {
      const double ck1 = (double)cc[d.C(i, j, k + 1)];
      zmass = zmass + 0.5 * dz[k] * (ck + ck1);
      ck = ck1;
    }
    acc[0] = dd_add_d(acc[0], fatx * faty * zmass);
    if (ic == 1) {
      acc[1] = dd_add_d(acc[1], fatx * faty * cload[p]);
      acc[2] = dd_add_d(acc[2], fatx * faty * cdry[p]);
      acc[3] = dd_add_d(acc[3], fatx * faty * cwet[p]);
    }
  }
  block_store_dd<4>(acc, partial);
}

template <class T>
void launch_cmass3d(const T* c, const double* cload, const double* cdry, const double* cwet,
                    Dims d, int nc, double dx, double dy, const double* dz, void* scratch,
                    double* out, cudaStream_t s) {
  const long long n = d.plane() * nc;
  const int nb = reduce_blocks(n);
  DD* partial = reinterpret_cast<DD*>(scratch);
  k_cmass3d<T><<<nb, RB, 0, s>>>(c, cload, cdry, cwet, d, nc, dz, partial);
  k_reduce_finish<4><<<1, RB, 0, s>>>(partial, nb, dx, dy, out, 0);
  count_launch(2);
}

// ------------------------------------------------------------- getc0
// Sources/endstep.f90:94-104 then cload = cdry + cwet (endstep.f90:35,60).
__global__ void k_getc0(double* cdry, double* cwet, double* cload, Dims d, int nc, int np) {
  const long long pl = d.plane();
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= pl) return;
  double sd = 0.0, sw = 0.0;
  for (int ic = 1; ic <= np; ++ic) {
    sd = sd + cdry[ic * pl + p];
    sw = sw + cwet[ic * pl + p];
  }
  cdry[p] = sd;
  cwet[p] = sw;
  for (int ic = 0; ic <= nc; ++ic) cload[ic * pl + p] = cdry[ic * pl + p] + cwet[ic * pl + p];
}

void launch_getc0(double* cdry, double* cwet, double* cload, Dims d, int nc, int np,
                  cudaStream_t s) {
  const long long pl = d.plane();
  k_getc0<<<(unsigned)((pl + 255) / 256), 256, 0, s>>>(cdry, cwet, cload, d, nc, np);
  count_launch();
}

// ------------------------------------------------------------ finddt
// Sources/finddt.f90:26-57.  MAX is exact and order independent, so the
// largest dtcni is found with a bitwise atomicMax on the (non-negative)
// binary64 patterns; NaN terms are skipped as MAX(dtcn,NaN) keeps dtcn.
// Every division has a divisor known per launch or per level, so each is
// formed from that divisor's reciprocal (div_rn_recip: the same quotient).
__global__ void k_finddt(Dims d, int nc, double dX1, double dX2, const double* dz,
                         const double* vx, const double* vy, const double* vz,
                         const double* vset, const double* rkh1, const double* rkhor,
                         const double* rkver, unsigned long long* dtcn_bits) {
  extern __shared__ double lvl[];  // per level k (index k-1): 1/ddz, 1/ddz^2, 1/den
  const int nx = d.nx, nz = d.nz;
  const long long s3 = d.cells();
  for (int k = threadIdx.x + 1; k <= nz; k += blockDim.x) {
    const double ddz = fmin2(dz[k - 1], dz[k]);
    const double den = k == 1 ? dz[1] : (k == nz ? dz[nz - 1] : dz[k] + dz[k - 1]);
    lvl[k - 1] = 1.0 / ddz;
    lvl[nz + k - 1] = 1.0 / (ddz * ddz);
    lvl[2 * nz + k - 1] = 1.0 / den;
  }
  __syncthreads();
  const double x2 = dX1 * dX1, y2 = dX2 * dX2;
  const double rx2 = 1.0 / x2, rx = 1.0 / dX1, ry2 = 1.0 / y2, ry = 1.0 / dX2;
  double best = 0.0;
  // one thread per cell: the five class-independent terms are summed once
  // (the reference's left-to-right order keeps them as a prefix), then the
  // two settling terms of every class are added to that prefix
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < s3;
       m += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(m % nx) + 1;
    const long long r = m / nx;
    const int j = (int)(r % d.ny) + 1, k = (int)(r / d.ny) + 1;
    const double ddz = fmin2(dz[k - 1], dz[k]);
    const double rz = lvl[k - 1], rzz = lvl[nz + k - 1], rden = lvl[2 * nz + k - 1];
    const double pre = div_rn_recip(2.0 * rkh1[m], x2, rx2) + div_rn_recip(absd(vx[m]), dX1, rx) +
                       div_rn_recip(2.0 * rkhor[m], y2, ry2) + div_rn_recip(absd(vy[m]), dX2, ry) +
                       div_rn_recip(2.0 * rkver[m], ddz * ddz, rzz);
    long long mlo, mhi;
    double den;
    if (k == 1) {
      mlo = d.M(i, j, 1);
      mhi = d.M(i, j, 2);
      den = dz[1];
    } else if (k == nz) {
      mlo = d.M(i, j, nz - 1);
      mhi = d.M(i, j, nz);
      den = dz[nz - 1];
    } else {
      mlo = d.M(i, j, k - 1);
      mhi = d.M(i, j, k + 1);
      den = dz[k] + dz[k - 1];
    }
    const double vzm = vz[m];
    for (int ic = 0; ic < nc; ++ic) {
      const double* vs = vset + (long long)ic * s3;
      const double dvsetdz = div_rn_recip(vs[mhi] - vs[mlo], den, rden);
      const double dtcni = pre + div_rn_recip(absd(vzm + vs[m]), ddz, rz) + absd(dvsetdz);
      // MAX(best, dtcni) of non-negative values (a NaN dtcni is skipped):
      // their bit patterns order as signed integers
      const long long db = __double_as_longlong(dtcni);
      if (db <= 0x7ff0000000000000LL && db > __double_as_longlong(best)) best = dtcni;
    }
  }
  for (int off = 16; off > 0; off >>= 1) best = fmax2(best, __shfl_down_sync(0xffffffffu, best, off));
  if ((threadIdx.x & 31) == 0 && best > 0.0)
    atomicMax(dtcn_bits, (unsigned long long)__double_as_longlong(best));
}

void launch_finddt(Dims d, int nc, double dX1, double dX2, const double* dz, const double* vx,
                   const double* vy, const double* vz, const double* vset, const double* rkh1,
                   const double* rkhor, const double* rkver, unsigned long long* dtcn_bits,
                   cudaStream_t s) {
  const long long n = d.cells();
  const int nb = (int)std::min<long long>((n + 255) / 256, 152LL * 8);
  k_finddt<<<nb, 256, 3 * sizeof(double) * (size_t)d.nz, s>>>(d, nc, dX1, dX2, dz, vx, vy, vz, vset, rkh1,
                                                              rkhor, rkver, dtcn_bits);
  count_launch();
}

size_t cmass2d_batch_scratch_bytes(int nscen) { return sizeof(DD) * (size_t)nscen * 64 + 256; }

void launch_cmass2d_batch(const BatchAux* tab, const int* bstep, int nscen, void* scratch,
                          cudaStream_t s) {
  if (nscen <= 0) return;
  DD* partial = reinterpret_cast<DD*>(scratch);
  k_cmass2d_batch<<<dim3(64, nscen), RB, 0, s>>>(tab, bstep, partial);
  k_cmass2d_batch_finish<<<nscen, RB, 0, s>>>(tab, partial, 64);
  count_launch(2);
}

// ------------------------------------------------ non-finite values
// Adds to *count the number of NaN or infinite values among a[0..n): the
// exponent field all ones, tested on the bit pattern.  A grid-stride loop of
// 8 blocks per SM, one atomic add per warp that found any.
__device__ __forceinline__ bool nonfinite_bits(float v) {
  return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u;
}
__device__ __forceinline__ bool nonfinite_bits(double v) {
  return ((unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}
template <class T>
__global__ void k_count_nonfinite(const T* __restrict__ a, long long n, unsigned long long* count) {
  unsigned long long k = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    k += nonfinite_bits(a[i]) ? 1ull : 0ull;
  for (int o = 16; o > 0; o >>= 1) k += __shfl_down_sync(0xffffffffu, k, o);
  if ((threadIdx.x & 31) == 0 && k) atomicAdd(count, k);
}

template <class T>
void launch_count_nonfinite(const T* a, long long n, unsigned long long* count, cudaStream_t s) {
  if (n <= 0) return;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n + 255) / 256;
  const int blocks = (int)std::min<long long>(want, 8LL * std::max(sms, 1));
  k_count_nonfinite<T><<<blocks, 256, 0, s>>>(a, n, count);
  count_launch();
}
template void launch_count_nonfinite<float>(const float*, long long, unsigned long long*, cudaStream_t);
template void launch_count_nonfinite<double>(const double*, long long, unsigned long long*, cudaStream_t);

template void launch_cmass2d<double>(const double*, const double*, const double*, const double*,
                                     const double*, Dims, int, int, int, int, double, double,
                                     const double*, double, void*, double*, cudaStream_t);
template void launch_cmass2d<float>(const float*, const double*, const double*, const double*,
                                    const double*, Dims, int, int, int, int, double, double,
                                    const double*, double, void*, double*, cudaStream_t);
template void launch_cmass3d<double>(const double*, const double*, const double*, const double*,
                                     Dims, int, double, double, const double*, void*, double*,
                                     cudaStream_t);
template void launch_cmass3d<float>(const float*, const double*, const double*, const double*,
                                    Dims, int, double, double, const double*, void*, double*,
                                    cudaStream_t);

}  // namespace f3d

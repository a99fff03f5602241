// f3d_internal.h -- launchers shared by the C-ABI layer and the kernels.
// All pointers are device pointers; every launcher enqueues on `s` and
// returns without synchronising.  Class-batched launchers process classes
// 0..ncls-1 whose blocks are `cstride` (concentration), `vstride` (vset)
// and `dstride` (vdep) elements apart.
#pragma once

#include <cuda_runtime.h>

#include <unordered_map>
#include <vector>

#include "f3d_common.cuh"

namespace f3d {

// Incremented by every launcher (diagnostic count of kernel launches).
void count_launch(int n = 1);

template <class T>
void launch_setbcc(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vx,
                   const T* vy, const T* vz, const T* vset, long long vstride, const T* vdep,
                   long long dstride, const T* rkver, const T* dz, int ncls, cudaStream_t s);
template <class T>
void launch_advctzc(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vz,
                    const T* vset, long long vstride, const T* dz, T dt, int ncls,
                    cudaStream_t s);
template <class T>
void launch_advctx(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vx, T dx,
                   T dt, int ncls, cudaStream_t s);
template <class T>
void launch_advcty(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vy, T dy,
                   T dt, int ncls, cudaStream_t s);
template <class T>
// rksz, lrz: the face coefficients and 1/rho precomputed
// (launch_diff_coeffs) or NULL.
void launch_diffz(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* dz, T dt,
                  const T* rkver, const T* rho, const T* rksz, const T* lrz, int ncls, cudaStream_t s);
// lr, pk: 1/rho and rkh*rho precomputed (launch_diff_coeffs), or NULL to
// form them from rho and rkh in the sweep.
template <class T>
void launch_diffx(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, T dx, T dt,
                  const T* rkh, const T* rho, const T* lr, const T* pk, int ncls, cudaStream_t s);
template <class T>
void launch_diffy(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, T dy, T dt,
                  const T* rkh, const T* rho, const T* lr, const T* pk, int ncls, cudaStream_t s);
void launch_diff_coeffs(Dims d, const double* rho, const double* rkh1, const double* rkhor,
                        const double* rkver, double* lr, double* pkx, double* pky, double* rksz,
                        cudaStream_t s);
// wetdep for classes ic0..ic0+ncls-1 (0-based, all particle classes);
// cwet points at cwet(1,1,0) and is binary64 in every form.  lam2d: the
// scavenging coefficient of the current dt (launch_wet_lambda) or NULL.
template <class T>
void launch_wetdep(T* c, long long cstride, double* cwet, int ic0, Dims d, int nz_loc, int iz_loc,
                   double dt, const double* diam, const double* zlayer, const double* dz,
                   const double* zi, const double* prate, const double* lam2d, int ncls, cudaStream_t s);
// accum in binary64 (vset/vdep binary64, c widened).
template <class T>
void launch_accum(const T* c, long long cstride, double* cdry, int ic0, Dims d, int iz_loc,
                  double dt, const double* vset, long long vstride, const double* vdep,
                  long long dstride, int ncls, cudaStream_t s);
template <class T>
void launch_clip(T* c, long long n, cudaStream_t s);
// setsrc.f90:20-35 adds the sources in file order; only sources in one
// cell need that order.  source_links gives link[0..n) = the next source in
// the same cell (-1: none) and link[n..2n) = 1 for the first source of its
// cell, so that one thread per first source walks its cell's chain; sources
// with k outside 1..nz are in no chain (the reference skips them).
inline std::vector<int> source_links(int n, const int* isrc, const int* jsrc, const int* ksrc,
                                     int nz) {
  std::vector<int> link(2 * (size_t)n, 0);
  std::unordered_map<long long, int> last;  // cell -> last source seen in it
  for (int s = 0; s < n; ++s) {
    link[s] = -1;
    if (ksrc[s] < 1 || ksrc[s] > nz) continue;
    const long long key = ((long long)ksrc[s] << 42) | ((long long)jsrc[s] << 21) | isrc[s];
    auto it = last.find(key);
    if (it == last.end()) {
      link[n + s] = 1;
      last.emplace(key, s);
    } else {
      link[it->second] = s;
      it->second = s;
    }
  }
  return link;
}
template <class T>
void launch_setsrc(T* c, long long cstride, Dims d, int nc, int nsou, const int* isrc,
                   const int* jsrc, const int* ksrc, const int* link, const double* tmrat,
                   const double* dz, const double* zlayer, const double* Hm1, double dX1, double dX2,
                   double dt, cudaStream_t s);

// Batched form: per scenario of a batch, the arguments of setsrc and cmass2d
// (global memory, one entry per scenario in batch order).  c_a / c_b are
// the scenario's two binary32 state buffers: after an even number of batch
// steps the state is in c_a, after an odd number in c_b.
struct BatchAux {
  float* c_a;
  float* c_b;
  long long cstride;
  Dims d;
  int nc;
  double dt;
  // setsrc.f90:20-35
  int nsou;
  const int *isrc, *jsrc, *ksrc, *link;
  const double* tmrat;
  const double *dz, *zlayer, *Hm1;
  double dX1, dX2;
  // cmass2d.f90:42-104 (binary64 velocities, device outmass)
  const double *vx, *vy, *vz, *vset;
  double* outmass;
};
void launch_setsrc_batch(const BatchAux* tab, const int* bstep, int nscen, int max_nc, int max_nsou,
                         cudaStream_t s);
size_t cmass2d_batch_scratch_bytes(int nscen);
void launch_cmass2d_batch(const BatchAux* tab, const int* bstep, int nscen, void* scratch,
                          cudaStream_t s);
void launch_batch_advance(int* bstep, int nscen, cudaStream_t s);

// Budget reductions.  `scratch` holds at least reduce_scratch_bytes(...)
// bytes; results are written as binary64 to device memory `out`.
size_t reduce_scratch_bytes(long long nterms, int nsums);
// Scratch bytes launch_cmass2d needs: its block count follows the number of
// face cells (class independent), so size it from the grid, not the classes.
size_t cmass2d_scratch_bytes(Dims d, int iz_loc, int nz_loc);
// Outflow of one step: *out = *out + sum of the terms of cmass2d.f90:42-102
// (out is the device copy of outmass).
template <class T>
void launch_cmass2d(const T* c, const double* vx, const double* vy, const double* vz,
                    const double* vset, Dims d, int ic_loc, int nc_loc, int iz_loc, int nz_loc,
                    double dx, double dy, const double* dz, double dt, void* scratch,
                    double* out, cudaStream_t s);
// out[0..3] = massvol, massdep, massdry, masswet of cmass3d.f90:29-58.
template <class T>
void launch_cmass3d(const T* c, const double* cload, const double* cdry, const double* cwet,
                    Dims d, int nc, double dx, double dy, const double* dz, void* scratch,
                    double* out, cudaStream_t s);
void launch_getc0(double* cdry, double* cwet, double* cload, Dims d, int nc, int np,
                  cudaStream_t s);
// *count += the number of NaN or infinite values among a[0..n).
template <class T>
void launch_count_nonfinite(const T* a, long long n, unsigned long long* count, cudaStream_t s);
// Largest dtcni of finddt.f90:26-57 as a binary64 bit pattern in *dtcn_bits
// (which must hold +0.0 on entry).
void launch_finddt(Dims d, int nc, double dX1, double dX2, const double* dz, const double* vx,
                   const double* vy, const double* vz, const double* vset, const double* rkh1,
                   const double* rkhor, const double* rkver, unsigned long long* dtcn_bits,
                   cudaStream_t s);

// Coefficient chain (binary64).
void launch_kappa3(Dims d, int modkv, int modkh, int coord_sys, double rkv0, double rkh0,
                   double Csh, double dX1, double dX2, double dx, double dy, const double* dz,
                   const double* zlayer, const double* Hm1, const double* vx, const double* vy,
                   const double* vptemp, const double* ustar, const double* zi, const double* rl,
                   double* rkver, double* rkhor, cudaStream_t s);
void launch_setvdrydep(Dims d, int nc, const double* diam, const double* zlayer,
                       const double* ldu, const double* rl, const double* znt,
                       const double* ustar, const double* tempe, const double* rho,
                       double* vdep, cudaStream_t s);
void launch_meteo_scale(Dims d, int coord_sys, double dX1, double dX2, const double* dz,
                        const double* Hm1, const double* topg, double* vx, double* vy,
                        double* vz, double* rho, const double* rkhor, double* rkh1,
                        double* divu, cudaStream_t s);
// Sources/setdivu.f90: divu of the scaled velocities
void launch_setdivu(Dims d, double dX1, double dX2, const double* dz, const double* Hm1,
                    const double* vx, const double* vy, const double* vz, double* divu,
                    cudaStream_t s);
void launch_reamet_fix(Dims d, int wetdep, double* vz, double* prate, cudaStream_t s);

// setvset with the cd chain.  Work buffers come from setvset_scratch_bytes.
size_t setvset_scratch_bytes(Dims d, int np);
// Returns non-zero through *status (device int): 1 = vsettl/get_gama did not
// converge.  cd_state is a device double (entry value in, exit value out).
// beside_step != 0: the chain runs as one 64-thread block per SM, sized to
// fit next to a resident step-kernel block (a look-ahead update on a second
// stream); the results do not depend on it.
void launch_setvset(Dims d, int nc, int np, int modv, const double* diam, const double* rhop,
                    const double* psi, const double* sphe, const double* tempe,
                    const double* rho, int aggregate, double vset_factor, double* vset,
                    int* iters, double* cd_state, void* scratch, int* status, cudaStream_t s,
                    int beside_step = 0);
// The drag iteration's table-driven log (op 0) and exp (op 1) on n values.
void launch_dmath_eval(int op, long long n, const double* x, double* y, cudaStream_t s);

// Conversions for the FP32 form.
void launch_d2f(float* dst, const double* src, long long n, cudaStream_t s);
void launch_f2d(double* dst, const float* src, long long n, cudaStream_t s);

}  // namespace f3d

// f3d_fused.h -- arguments of the precision form's fused step kernel.
#pragma once

#include <cuda.h>  // CUtensorMap (types only; the encoder is reached through the runtime)

#include "f3d_internal.h"

namespace f3d {

struct FusedArgs {
  const float* c_in;  // class blocks of (nx+2)(ny+2)(nz+2), after setsrc
  float* c_out;       // same layout; receives the step's result incl. ghosts
  long long cstride;
  Dims d;
  int ncls;
  int xfirst;  // iiter even: x before y (sizloop.f90:42-48)
  float dt;
  double dt64;
  // binary32 coefficients (scaled fields of meteo.f90:108-112)
  const float *vx, *vy, *vz;
  const float* vk;  // vz + vset, class blocks of nx*ny*nz
  long long vstride;
  const float* vdep;  // class blocks of nx*ny
  long long dstride;
  const float* rkver1;  // rkver(:,:,1) (setbcc bottom)
  const float* lrho;    // 1/rho
  const float *pkx, *pky, *pkz;  // rkh1*rho, rkhor*rho, rkver*rho
  const float* dz;      // dz(0:nz)
  float auxvx, auxvy, inv_dx, inv_dy, dtdx2, dtdy2;
  // binary64 deposits
  const unsigned char* wet_class;  // per class: wet deposition applies (or NULL)
  const double* lambda2d;          // min(dt*a*prate^b,1) per column
  const double* zi;
  const double* zlayer;
  const double* dz64;
  double* cwet;  // (nx,ny,0:nc)
  double* cdry;
  const double* vset64;  // class blocks, vstride apart
  const double* vdep64;  // class blocks of nx*ny
  // the same binary32 fields in the halo layout of c, ghost entries zero, but
  // with the row pitch hpitch = nx+2 rounded up to a multiple of 4 (padding
  // zero), so that a tensor copy can stage them: used by the
  // two-columns-per-lane kernel (tile shape 3)
  const float *vxh, *vyh, *lrhoh, *pkxh, *pkyh, *pkzh;
  const float* vkh;  // class blocks of hstride values
  int hpitch;
  long long hstride;  // hpitch * (ny+2) * (nz+2)
  int pair_aligned;  // nx even: every even column starts an 8-byte pair
  int* status;       // device status word: F3D_STEP_STAGING_TIMEOUT is or-ed into it
};

// a staging wait of the step kernel gave up (a tensor copy did not arrive)
#define F3D_STEP_STAGING_TIMEOUT 0x100

// Tensor maps of the met fields for the shape-3 step kernel's tensor copies:
// boxes of 68 x 32 x 1 values (x, rows, planes) of the padded halo layout.
struct F2Maps {
  enum { VK = 0, VX, VY, L, PZ, PX, PY, N };
  CUtensorMap m[N];
};
// 0 on success
int make_fused2_maps(const FusedArgs& a, F2Maps* out);
// the largest nz the shape-3 kernel's shared memory holds
int fused2_max_nz();
inline int halo_pitch(int nx) { return (nx + 2 + 3) & ~3; }

// tile region (x by y) / threads: 0 = 32x32 / 256 (default), 1 = 32x64 / 512,
// 2 = 32x32 / 512, 3 = 64x32 / 512 with two columns per lane.
void launch_step_fused(const FusedArgs& a, int shape, cudaStream_t s);
// beside != 0: the 112-register build, which leaves room for a look-ahead
// meteo update's settling chain on the same SMs (same results)
void launch_step_fused2(const FusedArgs& a, const F2Maps& maps, cudaStream_t s, int beside = 0);
// met fields (nx,ny,nz) -> halo layout of row pitch hp (ghost entries untouched)
void launch_to_halo(Dims d, int hp, int nfield, const float* const* src, float* const* dst, cudaStream_t s);
// tiles of one class of an nx x ny grid for a tile shape
int fused_tiles(int nx, int ny, int shape);

// Batched form: the arguments of up to F3D_BATCH_MAX scenarios in constant
// memory (c_in / c_out are the scenario's two buffers), then one persistent
// launch over the work items of all of them.
#define F3D_BATCH_MAX 128
int upload_batch_args(const FusedArgs* h, int n, cudaStream_t s);
int upload_batch_args2(const FusedArgs* h, int n, cudaStream_t s);  // the shape-3 kernel's table
int fused2_batch_grid(int max_nz);
// items [0, split) belong to scenarios with an even nx (two counters)
// maps: the scenarios' tensor maps (device array in batch order)
// fork: when both parts exist, the odd-nx part runs on fork->s2 as a
// parallel branch (fork->a recorded on s, fork->b on s2, s waits for it), so
// that its blocks fill the SMs the even-nx part's last blocks leave free
struct BatchFork {
  cudaStream_t s2 = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
};
void launch_step_fused2_batch(int grid, const int* item_off, int nscen, int split, int total, int* counter,
                              const int* bstep, const int* iiter0, int commit, int max_nz, const F2Maps* maps,
                              cudaStream_t s, const BatchFork* fork = nullptr);
// sets the kernel's shared-memory limit and returns its persistent grid (-1 on error)
int fused_batch_grid(int shape, int max_nz);
// counter: two ints; split / total: see launch_step_fused2_batch (shape 3)
void launch_step_fused_batch(int shape, int grid, const int* item_off, int nscen, int split, int total,
                             int* counter, const int* bstep, const int* iiter0, int commit, int max_nz,
                             const F2Maps* maps, cudaStream_t s, const BatchFork* fork = nullptr);
void launch_vk32(long long n, int nc, const float* vz, const float* vset, float* vk, cudaStream_t s);
void launch_wet_lambda(long long n, double dt, const double* prate, double* lam, cudaStream_t s);
void launch_fp32_coeffs(long long n, const double* rho, const double* rkh1, const double* rkhor,
                        const double* rkver, float* lrho, float* pkx, float* pky, float* pkz,
                        cudaStream_t s);

}  // namespace f3d

// f3d_ctx.cu -- the coarse context API: one scenario resident in HBM.
//
// Device layout of one context (all sizes in elements):
//   c        nc * (nx+2)(ny+2)(nz+2)  binary64 (plain form) or binary32
//   cdry, cwet, cload   (nc+1) * nx*ny binary64 (ground deposit, all forms)
//   met      vx vy vz tempe vptemp rho rkhor rkh1 rkver divu: nx*ny*nz each
//   vset     nc * nx*ny*nz, vdep nc * nx*ny          binary64
//   2-D      ustar zi rl znt prate ldu                binary64
//   FP32 form: binary32 copies of vx vy vz rho rkhor rkh1 rkver vset vdep dz
//   scratch  reduction partials, setvset chain buffers, small results.
// Everything of one step is enqueued on the context's stream without a host
// synchronisation; the host keeps only the scalars of the time loop.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <utility>
#include <string>
#include <vector>

#include "f3d_ctx_impl.h"

namespace f3d {
int ctx_error(int code, const char* msg);
}
using namespace f3d;


namespace {

#define CK(call)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);                   \
      return f3d::ctx_error(F3D_ERR_CUDA, m_.c_str());                                       \
    }                                                                                        \
  } while (0)

double* small_outmass(f3d_ctx* x) { return x->small; }
double* small_budget(f3d_ctx* x) { return x->small + 1; }
double* small_cd(f3d_ctx* x) { return x->small + 8; }
double* small_cd_prev(f3d_ctx* x) { return x->small + 9; }  // cd before the latest meteo update
unsigned long long* small_dtcn(f3d_ctx* x) {
  return reinterpret_cast<unsigned long long*>(x->small + 16);
}
int* small_status(f3d_ctx* x) { return reinterpret_cast<int*>(x->small + 24); }
int* small_step_status(f3d_ctx* x) { return reinterpret_cast<int*>(x->small + 26); }  // F3D_STEP_* bits
// the look-ahead meteo update's chain state, CFL maximum and status
double* small_pref_cd(f3d_ctx* x) { return x->small + 32; }
unsigned long long* small_pref_dtcn(f3d_ctx* x) { return reinterpret_cast<unsigned long long*>(x->small + 33); }
int* small_pref_status(f3d_ctx* x) { return reinterpret_cast<int*>(x->small + 34); }
// the non-finite counts of f3d_count_nonfinite: in c, in cdry + cwet
unsigned long long* small_nonfinite(f3d_ctx* x) { return reinterpret_cast<unsigned long long*>(x->small + 40); }

template <class T>
int dalloc(f3d_ctx* x, T** p, size_t n) {
  if (n == 0) n = 1;
  void* q = nullptr;
  if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return f3d::ctx_error(F3D_ERR_OOM, "device allocation failed");
  }
  x->allocs.push_back(q);
  if (cudaMemsetAsync(q, 0, n * sizeof(T), x->stream) != cudaSuccess)
    return f3d::ctx_error(F3D_ERR_CUDA, "cudaMemsetAsync failed");
  *p = reinterpret_cast<T*>(q);
  return F3D_OK;
}

// Device buffers of one met set (f3d_met_set) for the context's grid and
// precision; the members a precision does not use stay null.
int met_set_alloc(f3d_ctx* x, f3d_met_set* m) {
  const Dims d = x->d;
  const size_t s3 = (size_t)d.cells(), pl = (size_t)d.plane(), nc = (size_t)x->g.nc;
  const size_t hsz = (size_t)f3d::halo_pitch(d.nx) * (d.ny + 2) * (d.nz + 2);
  int rc = 0;
#define A(p, n) \
  if (!rc) rc = dalloc(x, &m->p, (n))
  A(vx, s3);
  A(vy, s3);
  A(vz, s3);
  A(tempe, s3);
  A(vptemp, s3);
  A(rho, s3);
  A(rkhor, s3);
  A(rkh1, s3);
  A(rkver, s3);
  A(divu, s3);
  A(vset, s3 * nc);
  A(vdep, pl * nc);
  A(ustar, pl);
  A(zi, pl);
  A(rl, pl);
  A(znt, pl);
  A(prate, pl);
  A(iters, s3 * nc);
  if (x->prec == F3D_PREC_FP64) {
    A(lrho64, s3);
    A(pkx64, s3);
    A(pky64, s3);
    A(rksz64, s3);
  } else {
    A(vx32, s3);
    A(vy32, s3);
    A(vz32, s3);
    A(rho32, s3);
    A(rkhor32, s3);
    A(rkh132, s3);
    A(rkver32, s3);
    A(vset32, s3 * nc);
    A(vdep32, pl * nc);
    A(lrho32, s3);
    A(pkx32, s3);
    A(pky32, s3);
    A(pkz32, s3);
    A(vk32, s3 * nc);
    A(vxh, hsz);
    A(vyh, hsz);
    A(lrhoh, hsz);
    A(pkxh, hsz);
    A(pkyh, hsz);
    A(pkzh, hsz);
    A(vkh, hsz * nc);
  }
#undef A
  return rc;
}

// Exchanges the context's current met set with *m (pointers only).
void met_set_swap(f3d_ctx* x, f3d_met_set* m) {
#define F3D_X(T, n) std::swap(x->n, m->n);
  F3D_MET_SET_D(F3D_X)
  F3D_MET_SET_F(F3D_X)
#undef F3D_X
  std::swap(x->maps2, m->maps2);
}

}  // namespace

namespace f3d {
int ctx_alloc(f3d_ctx* x, void** p, size_t bytes) {
  unsigned char* q = nullptr;
  const int rc = dalloc(x, &q, bytes);
  *p = q;
  return rc;
}

void refresh_fp32_class(f3d_ctx* x, int ic) {
  const Dims d = x->d;
  const size_t s3 = (size_t)d.cells();
  cudaStream_t s = x->stream;
  launch_d2f(x->vset32 + ic * s3, x->vset + ic * s3, (long long)s3, s);
  launch_vk32((long long)s3, 1, x->vz32, x->vset32 + ic * s3, x->vk32 + ic * s3, s);
  const float* vs = x->vk32 + ic * s3;
  const int hp = halo_pitch(d.nx);
  float* vd = x->vkh + (size_t)ic * (size_t)hp * (d.ny + 2) * (d.nz + 2);
  launch_to_halo(d, hp, 1, &vs, &vd, s);
}
}  // namespace f3d

namespace {

int is_dev(const void* p) {
  if (!p) return 0;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? 1 : 0;
}

int upload_on(double* dst, const double* src, size_t n, cudaStream_t s) {
  CK(cudaMemcpyAsync(dst, src, n * sizeof(double),
                     is_dev(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  return F3D_OK;
}

int upload(f3d_ctx* x, double* dst, const double* src, size_t n) { return upload_on(dst, src, n, x->stream); }

long long footprint_bytes(const f3d_grid* g) {
  const long long nx = g->nx, ny = g->ny, nz = g->nz, nc = g->nc;
  const long long s3 = nx * ny * nz, pl = nx * ny, halo = (nx + 2) * (ny + 2) * (nz + 2);
  long long b = 0;
  b += 8LL * (nz + 1 + nz + 2 * pl + 4 * nc);  // static
  b += 8LL * 10 * s3;                          // met + coefficients
  b += 8LL * (s3 * nc + pl * nc + 6 * pl);     // vset, vdep, 2-D
  b += 4LL * s3 * nc;                          // vsettl iteration counts
  b += 8LL * 3 * pl * (nc + 1);                // cdry cwet cload
  if (g->precision == F3D_PREC_FP32) {
    b += 2 * 4LL * halo * nc;
    b += 4LL * (11 * s3 + s3 * nc + pl * nc + nz + 1) + 8LL * pl + nc;
    b += 4LL * (6 + nc) * f3d::halo_pitch(g->nx) * (ny + 2) * (nz + 2);  // padded halo-layout met fields
  } else {
    b += 8LL * halo * nc;
    b += 8LL * 4 * s3 + 8LL * pl;  // 1/rho, rkh1*rho, rkhor*rho, diffz face coefficients; lambda
  }
  b += (long long)f3d::reduce_scratch_bytes(2LL * nc * (nx + ny) * nz + nc * pl, 4);
  b += (long long)f3d::setvset_scratch_bytes(Dims{g->nx, g->ny, g->nz}, g->np);
  b += 4096;
  return b;
}

// Brackets one launch with events when profiling is on.
struct ProfScope {
  f3d_ctx* x;
  int kind = -1;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEvent_t take() {
    if (!x->prof_pool.empty()) {
      cudaEvent_t e = x->prof_pool.back();
      x->prof_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  ProfScope(f3d_ctx* xx, const char* name) : x(xx) {
    if (!x->prof) return;
    for (size_t i = 0; i < x->prof_names.size(); ++i)
      if (x->prof_names[i] == name) kind = (int)i;
    if (kind < 0) {
      kind = (int)x->prof_names.size();
      x->prof_names.push_back(name);
      x->prof_count.push_back(0);
      x->prof_ms.push_back(0.0);
    }
    a = take();
    b = take();
    cudaEventRecord(a, x->stream);
  }
  ~ProfScope() {
    if (!x->prof) return;
    cudaEventRecord(b, x->stream);
    x->prof_pending.push_back({kind, a, b});
  }
};

void prof_drain(f3d_ctx* x) {
  if (x->prof_pending.empty()) return;
  cudaStreamSynchronize(x->stream);
  for (auto& r : x->prof_pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    x->prof_ms[r.kind] += ms;
    x->prof_count[r.kind] += 1;
    x->prof_pool.push_back(r.a);
    x->prof_pool.push_back(r.b);
  }
  x->prof_pending.clear();
}

template <class T>
struct Fields;  // per-precision views of the stencil inputs

template <>
struct Fields<double> {
  static double* c(f3d_ctx* x) { return x->c64; }
  static const double* vx(f3d_ctx* x) { return x->vx; }
  static const double* vy(f3d_ctx* x) { return x->vy; }
  static const double* vz(f3d_ctx* x) { return x->vz; }
  static const double* rho(f3d_ctx* x) { return x->rho; }
  static const double* rkhor(f3d_ctx* x) { return x->rkhor; }
  static const double* rkh1(f3d_ctx* x) { return x->rkh1; }
  static const double* rkver(f3d_ctx* x) { return x->rkver; }
  static const double* vset(f3d_ctx* x) { return x->vset; }
  static const double* vdep(f3d_ctx* x) { return x->vdep; }
  static const double* dz(f3d_ctx* x) { return x->dz; }
  static const double* lrho(f3d_ctx* x) { return x->lrho64; }
  static const double* pkx(f3d_ctx* x) { return x->pkx64; }
  static const double* pky(f3d_ctx* x) { return x->pky64; }
  static const double* rksz(f3d_ctx* x) { return x->rksz64; }
};
template <>
struct Fields<float> {
  static float* c(f3d_ctx* x) { return x->c32; }
  static const float* vx(f3d_ctx* x) { return x->vx32; }
  static const float* vy(f3d_ctx* x) { return x->vy32; }
  static const float* vz(f3d_ctx* x) { return x->vz32; }
  static const float* rho(f3d_ctx* x) { return x->rho32; }
  static const float* rkhor(f3d_ctx* x) { return x->rkhor32; }
  static const float* rkh1(f3d_ctx* x) { return x->rkh132; }
  static const float* rkver(f3d_ctx* x) { return x->rkver32; }
  static const float* vset(f3d_ctx* x) { return x->vset32; }
  static const float* vdep(f3d_ctx* x) { return x->vdep32; }
  static const float* dz(f3d_ctx* x) { return x->dz32; }
  // the per-routine binary32 sweeps divide in binary32 themselves
  static const float* lrho(f3d_ctx*) { return nullptr; }
  static const float* pkx(f3d_ctx*) { return nullptr; }
  static const float* pky(f3d_ctx*) { return nullptr; }
  static const float* rksz(f3d_ctx*) { return nullptr; }
};

// Sources/sizloop.f90:31-83 for all classes, class-batched sweeps.
template <class T>
void sizloop(f3d_ctx* x) {
  using F = Fields<T>;
  const Dims d = x->d;
  const int nz = d.nz, nc = x->g.nc, np = x->g.np;
  const long long hb = d.halo(), s3 = d.cells(), pl = d.plane();
  cudaStream_t s = x->stream;
  T* c = F::c(x);
  const T dt = (T)x->dt;
  const T dX1 = (T)x->g.dX1, dX2 = (T)x->g.dX2;
  auto advx = [&] {
    ProfScope ps(x, "advctx");
    launch_advctx<T>(c, hb, d, nz, 1, F::vx(x), dX1, dt, nc, s);
  };
  auto advy = [&] {
    ProfScope ps(x, "advcty");
    launch_advcty<T>(c, hb, d, nz, 1, F::vy(x), dX2, dt, nc, s);
  };
  auto difx = [&] {
    ProfScope ps(x, "diffx");
    launch_diffx<T>(c, hb, d, nz, 1, dX1, dt, F::rkh1(x), F::rho(x), F::lrho(x), F::pkx(x), nc, s);
  };
  auto dify = [&] {
    ProfScope ps(x, "diffy");
    launch_diffy<T>(c, hb, d, nz, 1, dX2, dt, F::rkhor(x), F::rho(x), F::lrho(x), F::pky(x), nc, s);
  };
  {
    ProfScope ps(x, "setbcc");
    launch_setbcc<T>(c, hb, d, nz, 1, F::vx(x), F::vy(x), F::vz(x), F::vset(x), s3, F::vdep(x), pl,
                     F::rkver(x), F::dz(x), nc, s);
  }
  {
    ProfScope ps(x, "advctzc");
    launch_advctzc<T>(c, hb, d, nz, 1, F::vz(x), F::vset(x), s3, F::dz(x), dt, nc, s);
  }
  // sizloop.f90:42-48: x/y order alternates with the parity of iiter
  if (x->iiter % 2 == 0) {
    advx();
    advy();
  } else {
    advy();
    advx();
  }
  {
    ProfScope ps(x, "diffz");
    launch_diffz<T>(c, hb, d, nz, 1, F::dz(x), dt, F::rkver(x), F::rho(x), F::rksz(x), F::lrho(x), nc, s);
  }
  if (x->iiter % 2 == 0) {
    difx();
    dify();
  } else {
    dify();
    difx();
  }
  if (x->g.wetdep && np > 0) {
    ProfScope ps(x, "wetdep");
    launch_wetdep<T>(c, hb, x->cwet, 0, d, nz, 1, x->dt, x->diam, x->zlayer, x->dz, x->zi, x->prate,
                     x->lambda2d, np, s);
  }
  {
    ProfScope ps(x, "accum");
    launch_accum<T>(c, hb, x->cdry, 0, d, 1, x->dt, x->vset, s3, x->vdep, pl, nc, s);
  }
  {
    ProfScope ps(x, "clip");
    launch_clip<T>(c, hb * nc, s);
  }
  {
    ProfScope ps(x, "cmass2d");
    launch_cmass2d<T>(c, x->vx, x->vy, x->vz, x->vset, d, 1, nc, 1, nz, x->g.dX1, x->g.dX2, x->dz,
                      x->dt, x->red_scratch, small_outmass(x), s);
  }
}


// The precision form's step as one fused kernel (f3d_fused.cu), then the
// clipped state's boundary outflow (cmass2d) in binary64.
void sizloop_fused(f3d_ctx* x) {
  const Dims d = x->d;
  const int nc = x->g.nc;
  cudaStream_t s = x->stream;
  const FusedArgs a = f3d::ctx_fused_args(x);
  {
    ProfScope ps(x, "step_fused");
    if (x->opt_tile == 3)  // the 112-register build while a look-ahead update runs beside it
      launch_step_fused2(a, x->maps2, s, x->pref_ready && cudaEventQuery(x->ev_pref) == cudaErrorNotReady);
    else
      launch_step_fused(a, x->opt_tile, s);
  }
  std::swap(x->c32, x->c32b);
  {
    ProfScope ps(x, "cmass2d");
    launch_cmass2d<float>(x->c32, x->vx, x->vy, x->vz, x->vset, d, 1, nc, 1, d.nz, x->g.dX1,
                          x->g.dX2, x->dz, x->dt, x->red_scratch, small_outmass(x), s);
  }
}

}  // namespace

namespace f3d {
FusedArgs ctx_fused_args(f3d_ctx* x) {
  const Dims d = x->d;
  const long long hb = d.halo(), s3 = d.cells(), pl = d.plane();
  FusedArgs a{};
  a.c_in = x->c32;
  a.c_out = x->c32b;
  a.cstride = hb;
  a.d = d;
  a.ncls = x->g.nc;
  a.xfirst = (x->iiter % 2 == 0) ? 1 : 0;
  a.dt = (float)x->dt;
  a.dt64 = x->dt;
  a.vx = x->vx32;
  a.vy = x->vy32;
  a.vz = x->vz32;
  a.vk = x->vk32;
  a.vstride = s3;
  a.vdep = x->vdep32;
  a.dstride = pl;
  a.rkver1 = x->rkver32;
  a.lrho = x->lrho32;
  a.pkx = x->pkx32;
  a.pky = x->pky32;
  a.pkz = x->pkz32;
  a.dz = x->dz32;
  a.auxvx = (float)(x->dt / x->g.dX1);
  a.auxvy = (float)(x->dt / x->g.dX2);
  a.inv_dx = (float)(1.0 / x->g.dX1);
  a.inv_dy = (float)(1.0 / x->g.dX2);
  a.dtdx2 = (float)(x->dt / (x->g.dX1 * x->g.dX1));
  a.dtdy2 = (float)(x->dt / (x->g.dX2 * x->g.dX2));
  a.wet_class = x->g.wetdep ? x->wet_class : nullptr;
  a.lambda2d = x->lambda2d;
  a.zi = x->zi;
  a.zlayer = x->zlayer;
  a.dz64 = x->dz;
  a.cwet = x->cwet;
  a.cdry = x->cdry;
  a.vset64 = x->vset;
  a.vdep64 = x->vdep;
  a.vxh = x->vxh;
  a.vyh = x->vyh;
  a.lrhoh = x->lrhoh;
  a.pkxh = x->pkxh;
  a.pkyh = x->pkyh;
  a.pkzh = x->pkzh;
  a.vkh = x->vkh;
  a.hpitch = halo_pitch(d.nx);
  a.hstride = (long long)a.hpitch * (d.ny + 2) * (d.nz + 2);
  a.status = small_step_status(x);
  a.pair_aligned = (d.nx % 2 == 0) ? 1 : 0;
  return a;
}
}  // namespace f3d

namespace f3d {
int ctx_error(int code, const char* msg);
}

namespace {

// The kernels of one meteo update on stream s (Sources/meteo.f90:27-149 with
// reamet.f90's fixes), writing the context's current met set: the raw
// fields are copied in (from host or device memory), the settling-velocity
// chain continues from *cd_state (setvset.f90:89), finddt's CFL maximum goes
// to *dtcn and a non-convergence to *status.  beside_step: the chain runs
// next to the step kernel (a look-ahead update on the second stream).
int meteo_enqueue(f3d_ctx* x, cudaStream_t s, const double* u, const double* v, const double* w,
                  const double* t, const double* tp, const double* rho, const double* ust,
                  const double* pblh, const double* rmol, const double* znt, const double* prate,
                  const double* ldu, double* cd_state, unsigned long long* dtcn, int* status,
                  int beside_step) {
  const Dims d = x->d;
  const size_t s3 = (size_t)d.cells(), pl = (size_t)d.plane();
  int rc = 0;
  // reamet.f90:20-153
  if (!rc) rc = upload_on(x->vx, u, s3, s);
  if (!rc) rc = upload_on(x->vy, v, s3, s);
  if (!rc) rc = upload_on(x->vz, w, s3, s);
  if (!rc) rc = upload_on(x->tempe, t, s3, s);
  if (!rc) rc = upload_on(x->vptemp, tp, s3, s);
  if (!rc) rc = upload_on(x->rho, rho, s3, s);
  if (!rc) rc = upload_on(x->ustar, ust, pl, s);
  if (!rc) rc = upload_on(x->zi, pblh, pl, s);
  if (!rc) rc = upload_on(x->rl, rmol, pl, s);
  if (!rc) rc = upload_on(x->znt, znt, pl, s);
  if (!rc && ldu) rc = upload_on(x->ldu, ldu, pl, s);
  if (!rc && x->g.wetdep) rc = upload_on(x->prate, prate, pl, s);
  if (rc) return rc;
  const f3d_grid& g = x->g;
  launch_reamet_fix(d, g.wetdep, x->vz, x->prate, s);
  // meteo.f90:27 kappa3 (unscaled vx, vy)
  launch_kappa3(d, g.modkv, g.modkh, g.coord_sys, g.rkv0, g.rkh0, g.Csh, g.dX1, g.dX2, g.dx, g.dy,
                x->dz, x->zlayer, x->Hm1, x->vx, x->vy, x->vptemp, x->ustar, x->zi, x->rl, x->rkver,
                x->rkhor, s);
  // meteo.f90:81 setvset (unscaled rho), continuing the cd chain
  launch_setvset(d, g.nc, g.np, g.modv, x->diam, x->rhop, x->psi, x->sphe, x->tempe, x->rho,
                 g.aggregate, g.vset_factor, x->vset, x->iters, cd_state, x->vset_scratch, status, s,
                 beside_step);
  // meteo.f90:100 setvdrydep (tempe(:,:,1), unscaled rho(:,:,1))
  launch_setvdrydep(d, g.nc, x->diam, x->zlayer, x->ldu, x->rl, x->znt, x->ustar, x->tempe, x->rho,
                    x->vdep, s);
  // meteo.f90:108-135 scaling and corvver, :140 addradialwind, :145 setdivu
  launch_meteo_scale(d, g.coord_sys, g.dX1, g.dX2, x->dz, x->Hm1, x->topg, x->vx, x->vy, x->vz,
                     x->rho, x->rkhor, x->rkh1, nullptr, s);
  if (x->gc_on) {  // the context's stream only: no look-ahead with the gravity current
    if (int r = f3d::gc_addradialwind(x)) return r;
  }
  launch_setdivu(d, g.dX1, g.dX2, x->dz, x->Hm1, x->vx, x->vy, x->vz, x->divu, s);
  // meteo.f90:149 finddt
  CK(cudaMemsetAsync(dtcn, 0, sizeof(unsigned long long), s));
  launch_finddt(d, g.nc, g.dX1, g.dX2, x->dz, x->vx, x->vy, x->vz, x->vset, x->rkh1, x->rkhor,
                x->rkver, dtcn, s);
  if (x->prec == F3D_PREC_FP64)
    launch_diff_coeffs(d, x->rho, x->rkh1, x->rkhor, x->rkver, x->lrho64, x->pkx64, x->pky64, x->rksz64, s);
  if (x->prec == F3D_PREC_FP32) {
    launch_d2f(x->vx32, x->vx, (long long)s3, s);
    launch_d2f(x->vy32, x->vy, (long long)s3, s);
    launch_d2f(x->vz32, x->vz, (long long)s3, s);
    launch_d2f(x->rho32, x->rho, (long long)s3, s);
    launch_d2f(x->rkhor32, x->rkhor, (long long)s3, s);
    launch_d2f(x->rkh132, x->rkh1, (long long)s3, s);
    launch_d2f(x->rkver32, x->rkver, (long long)s3, s);
    launch_d2f(x->vset32, x->vset, (long long)(s3 * g.nc), s);
    launch_d2f(x->vdep32, x->vdep, (long long)(pl * g.nc), s);
    launch_fp32_coeffs((long long)s3, x->rho, x->rkh1, x->rkhor, x->rkver, x->lrho32, x->pkx32,
                       x->pky32, x->pkz32, s);
    launch_vk32((long long)s3, g.nc, x->vz32, x->vset32, x->vk32, s);
    {  // halo-layout copies for the two-columns-per-lane kernel
      const float* src[6] = {x->vx32, x->vy32, x->lrho32, x->pkx32, x->pky32, x->pkz32};
      float* dst[6] = {x->vxh, x->vyh, x->lrhoh, x->pkxh, x->pkyh, x->pkzh};
      const int hp = halo_pitch(d.nx);
      launch_to_halo(d, hp, 6, src, dst, s);
      for (int c = 0; c < g.nc; ++c) {
        const float* vs = x->vk32 + (size_t)c * s3;
        float* vd = x->vkh + (size_t)c * (size_t)hp * (d.ny + 2) * (d.nz + 2);
        launch_to_halo(d, hp, 1, &vs, &vd, s);
      }
    }
  }
  CK(cudaGetLastError());
  return F3D_OK;
}

// What follows an update on the host: finddt.f90:58-66 from the CFL
// maximum, the wet-scavenging rate of the new dt (wetdep.f90:31), the
// aggregation flags (Fall3d.f90:94-96).
int meteo_finish(f3d_ctx* x, unsigned long long dtcn_bits, int status) {
  if (status) return f3d::ctx_error(F3D_ERR_NOCONV, "No convergence in vsettl routine");
  double dtcn;
  memcpy(&dtcn, &dtcn_bits, sizeof dtcn);
  dtcn = fmax2(dtcn, 1e-13);
  x->dtc = 1.0 / dtcn;
  x->dt = x->g.safety_factor * x->dtc;
  if (x->g.wetdep) {
    launch_wet_lambda((long long)x->d.plane(), x->dt, x->prate, x->lambda2d, x->stream);
    CK(cudaGetLastError());
  }
  x->have_met = 1;
  if (x->agr_on) {
    x->agr_due = 1;
    x->agr_npar = 0;
  }
  return F3D_OK;
}

// The second met set, the staging buffer of the next snapshot's raw fields,
// the second stream (lowest priority) and its events, made on first use.
int prefetch_setup(f3d_ctx* x) {
  if (x->pref_alloc) return F3D_OK;
  f3d_met_set m;
  if (int rc = met_set_alloc(x, &m)) return rc;
  if (x->prec == F3D_PREC_FP32 && x->fused_ok) {  // tensor maps of the second set's fields
    met_set_swap(x, &m);
    const int r2 = f3d::make_fused2_maps(f3d::ctx_fused_args(x), &x->maps2);
    met_set_swap(x, &m);
    if (r2) return f3d::ctx_error(F3D_ERR_CUDA, "cuTensorMapEncodeTiled failed for the second met set");
  }
  x->shadow = m;
  const size_t s3 = (size_t)x->d.cells(), pl = (size_t)x->d.plane();
  if (int rc = dalloc(x, &x->pref_stage, 6 * s3 + 5 * pl)) return rc;
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  CK(cudaStreamCreateWithPriority(&x->side, cudaStreamNonBlocking, least));
  CK(cudaEventCreateWithFlags(&x->ev_pref, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&x->ev_free, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&x->ev_staged, cudaEventDisableTiming));
  CK(cudaMallocHost((void**)&x->pref_host, 2 * sizeof(unsigned long long)));
  CK(cudaStreamSynchronize(x->stream));  // the zero fills of the new buffers
  x->pref_alloc = 1;
  return F3D_OK;
}

// Enqueues the meteo update of snapshot itime of the series on the second
// stream, into the second met set.  Its raw fields are staged first; the
// update itself waits for the steps enqueued so far (they read the set it
// overwrites).  Its chain starts from the committed chain state and writes
// its own slot, so a dropped look-ahead leaves the run as it was.
int prefetch_start(f3d_ctx* x, const f3d_met_series* met, int itime) {
  if (!x->opt_prefetch || x->pref_failed || x->gc_on || x->agr_on) return F3D_OK;
  if (x->g.wetdep && !met->prate) return F3D_OK;
  if (prefetch_setup(x)) {  // no room for a second set: the updates stay where they are due
    cudaGetLastError();
    x->pref_failed = 1;
    return F3D_OK;
  }
  const size_t s3 = (size_t)x->d.cells(), pl = (size_t)x->d.plane();
  const size_t o3 = (size_t)itime * s3, o2 = (size_t)itime * pl;
  cudaStream_t s = x->side;
  double* st = x->pref_stage;
  const double* src3[6] = {met->u + o3, met->v + o3, met->w + o3, met->t + o3, met->tp + o3, met->rho + o3};
  const double* src2[5] = {met->ust + o2, met->pblh + o2, met->rmol + o2, met->znt + o2,
                           met->prate ? met->prate + o2 : nullptr};
  double* f3[6];
  double* f2[5];
  for (int q = 0; q < 6; ++q) {
    f3[q] = st + q * s3;
    if (int rc = upload_on(f3[q], src3[q], s3, s)) return rc;
  }
  for (int q = 0; q < 5; ++q) {
    f2[q] = st + 6 * s3 + q * pl;
    if (src2[q])
      if (int rc = upload_on(f2[q], src2[q], pl, s)) return rc;
  }
  CK(cudaEventRecord(x->ev_staged, s));  // f3d_run returns only after these reads of the series
  CK(cudaEventRecord(x->ev_free, x->stream));
  CK(cudaStreamWaitEvent(s, x->ev_free, 0));
  CK(cudaMemcpyAsync(small_pref_cd(x), small_cd(x), sizeof(double), cudaMemcpyDeviceToDevice, s));
  met_set_swap(x, &x->shadow);
  const int rc = meteo_enqueue(x, s, f3[0], f3[1], f3[2], f3[3], f3[4], f3[5], f2[0], f2[1], f2[2], f2[3],
                               src2[4] ? f2[4] : nullptr, nullptr, small_pref_cd(x), small_pref_dtcn(x),
                               small_pref_status(x), 1);
  met_set_swap(x, &x->shadow);
  if (rc) return rc;
  CK(cudaMemcpyAsync(x->pref_host, small_pref_dtcn(x), sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(x->pref_host + 1, small_pref_status(x), sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(x->ev_pref, s));
  x->pref_ready = 1;
  x->pref_itime = itime;
  return F3D_OK;
}

// The look-ahead update becomes the current one: the two met sets are
// exchanged, its chain state is committed (the state before it kept for a
// checkpoint) and the host finishes the update as f3d_meteo does.
int prefetch_commit(f3d_ctx* x) {
  CK(cudaEventSynchronize(x->ev_pref));
  const unsigned long long bits = x->pref_host[0];
  int status = 0;
  memcpy(&status, x->pref_host + 1, sizeof status);
  CK(cudaStreamWaitEvent(x->stream, x->ev_pref, 0));
  met_set_swap(x, &x->shadow);
  x->pref_ready = 0;
  CK(cudaMemcpyAsync(small_cd_prev(x), small_cd(x), sizeof(double), cudaMemcpyDeviceToDevice, x->stream));
  CK(cudaMemcpyAsync(small_cd(x), small_pref_cd(x), sizeof(double), cudaMemcpyDeviceToDevice, x->stream));
  return meteo_finish(x, bits, status);
}

}  // namespace

namespace f3d {
void ctx_prefetch_drop(f3d_ctx* x) {
  if (!x->pref_ready) return;
  cudaEventSynchronize(x->ev_pref);
  x->pref_ready = 0;
}
}  // namespace f3d

extern "C" {

int f3d_ctx_footprint(const f3d_grid* g, long long* bytes) {
  if (!g || !bytes) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  *bytes = footprint_bytes(g);
  return F3D_OK;
}

int f3d_ctx_destroy(f3d_ctx* x) {
  if (!x) return F3D_OK;
  f3d::ctx_prefetch_drop(x);
  if (x->side) cudaStreamSynchronize(x->side);
  if (x->stream) cudaStreamSynchronize(x->stream);
  if (x->ev_pref) cudaEventDestroy(x->ev_pref);
  if (x->ev_free) cudaEventDestroy(x->ev_free);
  if (x->ev_staged) cudaEventDestroy(x->ev_staged);
  if (x->pref_host) cudaFreeHost(x->pref_host);
  if (x->side) cudaStreamDestroy(x->side);
  for (auto& r : x->prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : x->prof_pool) cudaEventDestroy(e);
  for (void* p : x->allocs) cudaFree(p);
  if (x->stream) cudaStreamDestroy(x->stream);
  delete x;
  return F3D_OK;
}

int f3d_ctx_create(const f3d_grid* g, f3d_ctx** out) {
  if (!g || !out) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (g->nx < 3 || g->ny < 3 || g->nz < 3) return f3d::ctx_error(F3D_ERR_ARG, "nx, ny, nz must be >= 3");
  if (g->nc < 1 || g->np < 0 || g->np > g->nc) return f3d::ctx_error(F3D_ERR_ARG, "invalid nc/np");
  if (g->precision != F3D_PREC_FP64 && g->precision != F3D_PREC_FP32)
    return f3d::ctx_error(F3D_ERR_ARG, "precision must be 64 or 32");
  if (g->modv < 1 || g->modv > 4 || g->modkv < 0 || g->modkv > 2 || g->modkh < 0 || g->modkh > 2)
    return f3d::ctx_error(F3D_ERR_ARG, "invalid model selector");
  if (!g->dz || !g->zlayer || !g->Hm1 || !g->topg || !g->diam || !g->rhop || !g->psi || !g->sphe)
    return f3d::ctx_error(F3D_ERR_ARG, "NULL grid array");
  f3d_ctx* x = new f3d_ctx();
  x->g = *g;
  x->g.dz = x->g.zlayer = x->g.Hm1 = x->g.topg = nullptr;
  x->g.diam = x->g.rhop = x->g.psi = x->g.sphe = nullptr;
  x->d = Dims{g->nx, g->ny, g->nz};
  x->prec = g->precision;
  x->h_diam.assign(g->diam, g->diam + g->nc);
  x->h_rhop.assign(g->rhop, g->rhop + g->nc);
  x->h_zlayer.assign(g->zlayer, g->zlayer + g->nz);
  x->hm11 = g->Hm1[0];
  for (int k = 1; k < g->nz; ++k)
    if (!(g->zlayer[k] >= g->zlayer[k - 1])) x->fused_ok = 0;
  if (x->d.halo() >= (1LL << 31) || x->d.cells() >= (1LL << 31)) x->fused_ok = 0;
  if ((long long)f3d::halo_pitch(g->nx) * (g->ny + 2) * (g->nz + 2) >= (1LL << 31)) x->fused_ok = 0;
  if (g->nz > f3d::fused2_max_nz()) x->fused_ok = 0;  // the shape-3 kernel's per-level table
  // the highest priority: a look-ahead meteo update on the context's second
  // stream (lowest priority) runs in what the steps leave free
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (cudaStreamCreateWithPriority(&x->stream, cudaStreamNonBlocking, prio_greatest) != cudaSuccess) {
    delete x;
    return f3d::ctx_error(F3D_ERR_CUDA, "cudaStreamCreate failed");
  }
  const Dims d = x->d;
  const size_t s3 = (size_t)d.cells(), pl = (size_t)d.plane(), hb = (size_t)d.halo();
  const size_t nc = (size_t)g->nc, nz = (size_t)g->nz;
  int rc = 0;
#define A(p, n) \
  if (!rc) rc = dalloc(x, &x->p, (n))
  A(dz, nz + 1);
  A(zlayer, nz);
  A(Hm1, pl);
  A(topg, pl);
  A(diam, nc);
  A(rhop, nc);
  A(psi, nc);
  A(sphe, nc);
  A(ldu, pl);
  A(cdry, pl * (nc + 1));
  A(cwet, pl * (nc + 1));
  A(cload, pl * (nc + 1));
  A(small, 64);
  if (x->prec == F3D_PREC_FP32) {
    A(c32, hb * nc);
    A(dz32, nz + 1);
    A(c32b, hb * nc);
    A(wet_class, nc);
  } else {
    A(c64, hb * nc);
  }
  A(lambda2d, pl);
#undef A
  if (!rc) {  // the met set (f3d_met_set) the meteo updates fill
    f3d_met_set m;
    rc = met_set_alloc(x, &m);
    if (!rc) met_set_swap(x, &m);
  }
  if (!rc) {
    unsigned char* p = nullptr;
    rc = dalloc(x, &p, f3d::reduce_scratch_bytes(2LL * g->nc * (g->nx + g->ny) * g->nz +
                                                      (long long)g->nc * g->nx * g->ny, 4));
    x->red_scratch = p;
  }
  if (!rc) {
    unsigned char* p = nullptr;
    rc = dalloc(x, &p, f3d::setvset_scratch_bytes(d, g->np));
    x->vset_scratch = p;
  }
  if (rc) {
    f3d_ctx_destroy(x);
    return rc;
  }
  // static fields
  if (!rc) rc = upload(x, x->dz, g->dz, nz + 1);
  if (!rc) rc = upload(x, x->zlayer, g->zlayer, nz);
  if (!rc) rc = upload(x, x->Hm1, g->Hm1, pl);
  if (!rc) rc = upload(x, x->topg, g->topg, pl);
  if (!rc) rc = upload(x, x->diam, g->diam, nc);
  if (!rc) rc = upload(x, x->rhop, g->rhop, nc);
  if (!rc) rc = upload(x, x->psi, g->psi, nc);
  if (!rc) rc = upload(x, x->sphe, g->sphe, nc);
  const double cd0 = 1.0;  // setvset.f90:89
  if (!rc && cudaMemcpyAsync(small_cd(x), &cd0, sizeof cd0, cudaMemcpyHostToDevice, x->stream) != cudaSuccess)
    rc = f3d::ctx_error(F3D_ERR_CUDA, "upload failed");
  if (!rc && cudaMemcpyAsync(small_cd_prev(x), &cd0, sizeof cd0, cudaMemcpyHostToDevice, x->stream) != cudaSuccess)
    rc = f3d::ctx_error(F3D_ERR_CUDA, "upload failed");
  // LDU defaults to -99 (Master.f90:176)
  if (!rc) {
    std::vector<double> l(pl, -99.0);
    rc = upload(x, x->ldu, l.data(), pl);
    if (!rc && cudaStreamSynchronize(x->stream) != cudaSuccess) rc = f3d::ctx_error(F3D_ERR_CUDA, "sync failed");
  }
  if (!rc && x->prec == F3D_PREC_FP32) {
    // wetdep.f90:28-30 and sizloop.f90:65: particles of at most 100 um
    std::vector<unsigned char> wc(nc, 0);
    double diam_max = 100.0;
    diam_max = diam_max * 1e-6;
    for (size_t ic = 0; ic < nc; ++ic)
      wc[ic] = (g->wetdep && (int)ic < g->np && !(g->diam[ic] > diam_max)) ? 1 : 0;
    if (cudaMemcpyAsync(x->wet_class, wc.data(), nc, cudaMemcpyHostToDevice, x->stream) != cudaSuccess)
      rc = f3d::ctx_error(F3D_ERR_CUDA, "upload failed");
    launch_d2f(x->dz32, x->dz, (long long)nz + 1, x->stream);
    if (cudaStreamSynchronize(x->stream) != cudaSuccess) rc = f3d::ctx_error(F3D_ERR_CUDA, "sync failed");
    // the tensor maps of the shape-3 step kernel: the fields stay at these addresses
    if (!rc && x->fused_ok && f3d::make_fused2_maps(f3d::ctx_fused_args(x), &x->maps2) != 0)
      rc = f3d::ctx_error(F3D_ERR_CUDA, "cuTensorMapEncodeTiled failed for the step kernel's met fields");
  }
  if (rc) {
    f3d_ctx_destroy(x);
    return rc;
  }
  *out = x;
  return F3D_OK;
}

int f3d_meteo(f3d_ctx* x, const double* u, const double* v, const double* w, const double* t,
              const double* tp, const double* rho, const double* ust, const double* pblh,
              const double* rmol, const double* znt, const double* prate, const double* ldu) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  if (!u || !v || !w || !t || !tp || !rho || !ust || !pblh || !rmol || !znt)
    return f3d::ctx_error(F3D_ERR_ARG, "NULL meteorological field");
  if (x->g.wetdep && !prate) return f3d::ctx_error(F3D_ERR_ARG, "PRATE required with wet deposition");
  f3d::ctx_prefetch_drop(x);
  cudaStream_t s = x->stream;
  // the chain state this update starts from (a checkpoint replays the update)
  CK(cudaMemcpyAsync(small_cd_prev(x), small_cd(x), sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (int rc = meteo_enqueue(x, s, u, v, w, t, tp, rho, ust, pblh, rmol, znt, prate, ldu, small_cd(x),
                             small_dtcn(x), small_status(x), 0))
    return rc;
  struct {
    unsigned long long dtcn;
    int status;
  } h{};
  CK(cudaMemcpyAsync(&h.dtcn, small_dtcn(x), sizeof h.dtcn, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&h.status, small_status(x), sizeof h.status, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return meteo_finish(x, h.dtcn, h.status);
}

int f3d_source(f3d_ctx* x, int nsou, const int* isrc, const int* jsrc, const int* ksrc,
               const double* tmrat) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  if (nsou < 0) return f3d::ctx_error(F3D_ERR_ARG, "nsou < 0");
  const int nc = x->g.nc, nx = x->g.nx, ny = x->g.ny, nz = x->g.nz;
  // host copies (reasrc.f90:76-80 checks, source.f90:136-185 sums and scaling)
  std::vector<int> hi(nsou), hj(nsou), hk(nsou);
  std::vector<double> ht((size_t)nsou * nc);
  if (nsou > 0) {
    const cudaMemcpyKind k = is_dev(isrc) ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    CK(cudaMemcpy(hi.data(), isrc, sizeof(int) * nsou, k));
    CK(cudaMemcpy(hj.data(), jsrc, sizeof(int) * nsou, k));
    CK(cudaMemcpy(hk.data(), ksrc, sizeof(int) * nsou, k));
    CK(cudaMemcpy(ht.data(), tmrat, sizeof(double) * nsou * nc,
                  is_dev(tmrat) ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
  }
  for (int s = 0; s < nsou; ++s)
    if (hi[s] < 1 || hi[s] > nx || hj[s] < 1 || hj[s] > ny || hk[s] > nz) {
      char m[160];
      snprintf(m, sizeof m, "Inconsistence between dbs and src files: source %d at (%d,%d,%d)", s + 1,
               hi[s], hj[s], hk[s]);
      return f3d::ctx_error(F3D_ERR_RANGE, m);
    }
  double fr = 0.0;  // SUM(tmrat(1:nsou,1:nc)) in element order
  for (int ic = 0; ic < nc; ++ic)
    for (int s = 0; s < nsou; ++s) fr = fr + ht[(size_t)s + (size_t)nsou * ic];
  x->flowrate = fr;
  // tmrat(isou,:) = tmrat(isou,:)*Hm1(isrc,jsrc): Hm1 lives on the device;
  // the host needs only the 2-D plane values at the source cells.
  std::vector<double> hm(nsou);
  for (int s = 0; s < nsou; ++s)
    CK(cudaMemcpy(&hm[s], x->Hm1 + (size_t)(hi[s] - 1) + (size_t)nx * (hj[s] - 1), sizeof(double),
                  cudaMemcpyDeviceToHost));
  for (int s = 0; s < nsou; ++s)
    for (int ic = 0; ic < nc; ++ic) ht[(size_t)s + (size_t)nsou * ic] *= hm[s];
  double mfr = 0.0;  // SUM of the scaled tmrat in element order (addradialwind.f90:61)
  for (int ic = 0; ic < nc; ++ic)
    for (int s = 0; s < nsou; ++s) mfr = mfr + ht[(size_t)s + (size_t)nsou * ic];
  x->mfr_scaled = mfr;
  if (nsou > x->src_cap) {
    int cap = nsou;
    int rc = dalloc(x, &x->isrc, cap);
    if (!rc) rc = dalloc(x, &x->jsrc, cap);
    if (!rc) rc = dalloc(x, &x->ksrc, cap);
    if (!rc) rc = dalloc(x, &x->slink, 2 * (size_t)cap);
    if (!rc) rc = dalloc(x, &x->tmrat, (size_t)cap * nc);
    if (rc) return rc;
    x->src_cap = cap;
  }
  x->nsou = nsou;
  if (nsou > 0) {
    const std::vector<int> link = f3d::source_links(nsou, hi.data(), hj.data(), hk.data(), nz);
    CK(cudaMemcpyAsync(x->slink, link.data(), sizeof(int) * 2 * nsou, cudaMemcpyHostToDevice, x->stream));
    CK(cudaMemcpyAsync(x->isrc, hi.data(), sizeof(int) * nsou, cudaMemcpyHostToDevice, x->stream));
    CK(cudaMemcpyAsync(x->jsrc, hj.data(), sizeof(int) * nsou, cudaMemcpyHostToDevice, x->stream));
    CK(cudaMemcpyAsync(x->ksrc, hk.data(), sizeof(int) * nsou, cudaMemcpyHostToDevice, x->stream));
    CK(cudaMemcpyAsync(x->tmrat, ht.data(), sizeof(double) * nsou * nc, cudaMemcpyHostToDevice,
                       x->stream));
    CK(cudaStreamSynchronize(x->stream));  // host vectors go out of scope
  }
  if (x->agr_on) x->agr_due = 1;  // Fall3d.f90:84-86
  return F3D_OK;
}

int f3d_step(f3d_ctx* x) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  if (!x->have_met) return f3d::ctx_error(F3D_ERR_STATE, "f3d_step before f3d_meteo");
  if (x->agr_on && x->agr_due) {  // Fall3d.f90:101-110: agrpar after this step's updates
    const int rc = x->agr_replay > 0 ? f3d::agg_restore_vset(x, x->agr_replay) : f3d::agg_agrpar(x);
    if (rc) return rc;
    x->agr_due = 0;
    x->agr_replay = 0;
  }
  f3d::ctx_advance(x);
  const Dims d = x->d;
  // setsrc.f90:20-35
  if (x->prof) prof_drain(x);  // bounded event backlog: resolve the previous step
  if (x->prec == F3D_PREC_FP32) {
    ProfScope ps(x, "setsrc");
    launch_setsrc<float>(x->c32, d.halo(), d, x->g.nc, x->nsou, x->isrc, x->jsrc, x->ksrc, x->slink,
                         x->tmrat, x->dz, x->zlayer, x->Hm1, x->g.dX1, x->g.dX2, x->dt, x->stream);
  } else {
    ProfScope ps(x, "setsrc");
    launch_setsrc<double>(x->c64, d.halo(), d, x->g.nc, x->nsou, x->isrc, x->jsrc, x->ksrc, x->slink,
                          x->tmrat, x->dz, x->zlayer, x->Hm1, x->g.dX1, x->g.dX2, x->dt, x->stream);
  }
  if (x->agr_on) {  // setsrc.f90:37-76
    if (int rc = f3d::agg_setsrc(x)) return rc;
  }
  if (x->prec == F3D_PREC_FP32 && x->opt_fused && x->fused_ok)
    sizloop_fused(x);
  else if (x->prec == F3D_PREC_FP32)
    sizloop<float>(x);
  else
    sizloop<double>(x);
  CK(cudaGetLastError());
  return F3D_OK;
}

int f3d_sync(f3d_ctx* x) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  CK(cudaStreamSynchronize(x->stream));
  return f3d::ctx_check_step_status(x);
}

int f3d_budget(f3d_ctx* x, double* massvol, double* massdep, double* massdry, double* masswet) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  const Dims d = x->d;
  launch_getc0(x->cdry, x->cwet, x->cload, d, x->g.nc, x->g.np, x->stream);
  if (x->prec == F3D_PREC_FP32)
    launch_cmass3d<float>(x->c32, x->cload, x->cdry, x->cwet, d, x->g.nc, x->g.dX1, x->g.dX2, x->dz,
                          x->red_scratch, small_budget(x), x->stream);
  else
    launch_cmass3d<double>(x->c64, x->cload, x->cdry, x->cwet, d, x->g.nc, x->g.dX1, x->g.dX2, x->dz,
                           x->red_scratch, small_budget(x), x->stream);
  double h[4];
  CK(cudaMemcpyAsync(h, small_budget(x), sizeof h, cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  if (massvol) *massvol = h[0];
  if (massdep) *massdep = h[1];
  if (massdry) *massdry = h[2];
  if (masswet) *masswet = h[3];
  return F3D_OK;
}

int f3d_count_nonfinite(f3d_ctx* x, long long* in_c, long long* in_deposits) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  const Dims d = x->d;
  const long long hb = (long long)d.halo() * x->g.nc, dep = (long long)d.plane() * (x->g.nc + 1);
  unsigned long long* cnt = small_nonfinite(x);
  CK(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), x->stream));
  if (x->prec == F3D_PREC_FP32)
    launch_count_nonfinite<float>(x->c32, hb, cnt, x->stream);
  else
    launch_count_nonfinite<double>(x->c64, hb, cnt, x->stream);
  launch_count_nonfinite<double>(x->cdry, dep, cnt + 1, x->stream);
  launch_count_nonfinite<double>(x->cwet, dep, cnt + 1, x->stream);
  unsigned long long h[2];
  CK(cudaMemcpyAsync(h, cnt, sizeof h, cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  if (in_c) *in_c = (long long)h[0];
  if (in_deposits) *in_deposits = (long long)h[1];
  return F3D_OK;
}

int f3d_get_state(const f3d_ctx* cx, int* iiter, double* time, double* dt, double* dtc,
                  double* erumass, double* outmass, double* flowrate) {
  f3d_ctx* x = const_cast<f3d_ctx*>(cx);
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  if (outmass) {
    CK(cudaMemcpyAsync(outmass, small_outmass(x), sizeof(double), cudaMemcpyDeviceToHost, x->stream));
    CK(cudaStreamSynchronize(x->stream));
  }
  if (iiter) *iiter = x->iiter;
  if (time) *time = x->time;
  if (dt) *dt = x->dt;
  if (dtc) *dtc = x->dtc;
  if (erumass) *erumass = x->erumass;
  if (flowrate) *flowrate = x->flowrate;
  return F3D_OK;
}

int f3d_get_cd(const f3d_ctx* cx, double* cd) {
  f3d_ctx* x = const_cast<f3d_ctx*>(cx);
  if (!x || !cd) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  CK(cudaMemcpyAsync(cd, small_cd(x), sizeof(double), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  return F3D_OK;
}

int f3d_set_time(f3d_ctx* x, double time, int iiter) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  x->time = time;
  x->iiter = iiter;
  return F3D_OK;
}

int f3d_download(f3d_ctx* x, double* c, double* cdry, double* cwet, double* vset, double* vdep) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  const Dims d = x->d;
  const size_t hb = (size_t)d.halo() * x->g.nc, pl = (size_t)d.plane(), nc = (size_t)x->g.nc;
  cudaStream_t s = x->stream;
  auto kind = [](const void* p) { return is_dev(p) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost; };
  if (c) {
    if (x->prec == F3D_PREC_FP32) {
      if (is_dev(c)) {
        launch_f2d(c, x->c32, (long long)hb, s);
      } else {
        double* tmp = nullptr;
        CK(cudaMallocAsync((void**)&tmp, hb * sizeof(double), s));
        launch_f2d(tmp, x->c32, (long long)hb, s);
        CK(cudaMemcpyAsync(c, tmp, hb * sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaFreeAsync(tmp, s));
      }
    } else {
      CK(cudaMemcpyAsync(c, x->c64, hb * sizeof(double), kind(c), s));
    }
  }
  if (cdry) CK(cudaMemcpyAsync(cdry, x->cdry, pl * (nc + 1) * sizeof(double), kind(cdry), s));
  if (cwet) CK(cudaMemcpyAsync(cwet, x->cwet, pl * (nc + 1) * sizeof(double), kind(cwet), s));
  if (vset) CK(cudaMemcpyAsync(vset, x->vset, (size_t)d.cells() * nc * sizeof(double), kind(vset), s));
  if (vdep) CK(cudaMemcpyAsync(vdep, x->vdep, pl * nc * sizeof(double), kind(vdep), s));
  CK(cudaStreamSynchronize(s));
  return F3D_OK;
}

int f3d_upload_state(f3d_ctx* x, const double* c, const double* cdry, const double* cwet,
                     double erumass, double outmass, double cd) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  const Dims d = x->d;
  const size_t hb = (size_t)d.halo() * x->g.nc, pl = (size_t)d.plane(), nc = (size_t)x->g.nc;
  cudaStream_t s = x->stream;
  int rc = 0;
  if (c) {
    if (x->prec == F3D_PREC_FP32) {
      double* tmp = nullptr;
      CK(cudaMallocAsync((void**)&tmp, hb * sizeof(double), s));
      rc = upload(x, tmp, c, hb);
      launch_d2f(x->c32, tmp, (long long)hb, s);
      CK(cudaFreeAsync(tmp, s));
    } else {
      rc = upload(x, x->c64, c, hb);
    }
  }
  if (!rc && cdry) rc = upload(x, x->cdry, cdry, pl * (nc + 1));
  if (!rc && cwet) rc = upload(x, x->cwet, cwet, pl * (nc + 1));
  if (rc) return rc;
  x->erumass = erumass;
  CK(cudaMemcpyAsync(small_outmass(x), &outmass, sizeof outmass, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(small_cd(x), &cd, sizeof cd, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  return F3D_OK;
}

// ---------------------------------------------------------------- checkpoint
// A lossless checkpoint of the state a run carries from step to step (the
// reference's restart, wrirst.f90 / rearst.f90, keeps only c and cload in
// binary32 and the two mass scalars).  The coefficients are not stored: the
// restored run replays the meteo and source updates of the current
// intervals from the drag-coefficient chain state they started from, which
// rebuilds them bit for bit, so a restored run continues exactly as the
// uninterrupted one.
namespace {
struct CkptHeader {
  char magic[8];
  int version, nx, ny, nz, nc, precision, iiter, pad;
  double time, erumass, outmass, cd_prev;
};
const char kCkptMagic[8] = {'F', '3', 'D', 'C', 'K', 'P', 'T', '1'};
const long long kCkptAggr = 0x5247474146334446LL;  // the optional aggregation section
}  // namespace

int f3d_ctx_save(f3d_ctx* x, const char* path) {
  if (!x || !path) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  const Dims d = x->d;
  const size_t hb = (size_t)d.halo() * x->g.nc, pl2 = (size_t)d.plane() * (x->g.nc + 1);
  const size_t esz = x->prec == F3D_PREC_FP32 ? sizeof(float) : sizeof(double);
  CkptHeader h{};
  memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.nx = d.nx;
  h.ny = d.ny;
  h.nz = d.nz;
  h.nc = x->g.nc;
  h.precision = x->prec;
  h.iiter = x->iiter;
  h.time = x->time;
  h.erumass = x->erumass;
  std::vector<unsigned char> c(hb * esz);
  // aggregation: Maggr and the coefficients of the last agrpar
  const size_t s3 = (size_t)d.cells();
  std::vector<double> cdry(pl2), cwet(pl2), agf(x->agr_on ? 5 * s3 : 0);
  cudaStream_t s = x->stream;
  if (x->agr_on) {
    const double* src[5] = {x->agr_maggr, x->agr_al, x->agr_ab, x->agr_as, x->agr_ad};
    for (int q = 0; q < 5; ++q)
      CK(cudaMemcpyAsync(agf.data() + q * s3, src[q], s3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaMemcpyAsync(&h.outmass, small_outmass(x), sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&h.cd_prev, small_cd_prev(x), sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(c.data(), x->prec == F3D_PREC_FP32 ? (const void*)x->c32 : (const void*)x->c64, hb * esz,
                     cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(cdry.data(), x->cdry, pl2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(cwet.data(), x->cwet, pl2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  FILE* f = fopen(path, "wb");
  if (!f) return f3d::ctx_error(F3D_ERR_ARG, "cannot open the checkpoint file for writing");
  bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(c.data(), 1, c.size(), f) == c.size() &&
            fwrite(cdry.data(), sizeof(double), pl2, f) == pl2 && fwrite(cwet.data(), sizeof(double), pl2, f) == pl2;
  if (ok && x->agr_on) {  // aggregation: the agrsrc step counter, agrpar calls since the meteo update,
                          // Maggr and Alagr, Abagr, Asagr, Adagr
    const long long agg[3] = {kCkptAggr, x->agr_ipass, x->agr_npar};
    ok = fwrite(agg, sizeof agg, 1, f) == 1 && fwrite(agf.data(), sizeof(double), agf.size(), f) == agf.size();
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) return f3d::ctx_error(F3D_ERR_ARG, "checkpoint write failed");
  return F3D_OK;
}

int f3d_ctx_restore(f3d_ctx* x, const char* path) {
  if (!x || !path) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  FILE* f = fopen(path, "rb");
  if (!f) return f3d::ctx_error(F3D_ERR_ARG, "cannot open the checkpoint file");
  CkptHeader h{};
  const Dims d = x->d;
  bool ok = fread(&h, sizeof h, 1, f) == 1 && memcmp(h.magic, kCkptMagic, 8) == 0 && h.version == 1;
  if (!ok) {
    fclose(f);
    return f3d::ctx_error(F3D_ERR_ARG, "not a checkpoint of this library");
  }
  if (h.nx != d.nx || h.ny != d.ny || h.nz != d.nz || h.nc != x->g.nc || h.precision != x->prec) {
    fclose(f);
    return f3d::ctx_error(F3D_ERR_ARG, "checkpoint of a different grid, class count or precision");
  }
  const size_t hb = (size_t)d.halo() * x->g.nc, pl2 = (size_t)d.plane() * (x->g.nc + 1);
  const size_t esz = x->prec == F3D_PREC_FP32 ? sizeof(float) : sizeof(double);
  std::vector<unsigned char> c(hb * esz);
  std::vector<double> cdry(pl2), cwet(pl2);
  ok = fread(c.data(), 1, c.size(), f) == c.size() && fread(cdry.data(), sizeof(double), pl2, f) == pl2 &&
       fread(cwet.data(), sizeof(double), pl2, f) == pl2;
  long long agg[3] = {0, 0, 0};
  const bool has_agg = ok && fread(agg, sizeof agg, 1, f) == 1 && agg[0] == kCkptAggr;
  const size_t s3 = (size_t)d.cells();
  std::vector<double> agf(has_agg ? 5 * s3 : 0);
  if (has_agg) ok = fread(agf.data(), sizeof(double), agf.size(), f) == agf.size();
  fclose(f);
  if (!ok) return f3d::ctx_error(F3D_ERR_ARG, "truncated checkpoint file");
  if (has_agg != (x->agr_on != 0))
    return f3d::ctx_error(F3D_ERR_ARG, "aggregation is on in only one of the checkpoint and the context");
  f3d::ctx_prefetch_drop(x);
  cudaStream_t s = x->stream;
  CK(cudaMemcpyAsync(x->prec == F3D_PREC_FP32 ? (void*)x->c32 : (void*)x->c64, c.data(), hb * esz,
                     cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(x->cdry, cdry.data(), pl2 * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(x->cwet, cwet.data(), pl2 * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(small_outmass(x), &h.outmass, sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(small_cd(x), &h.cd_prev, sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(small_cd_prev(x), &h.cd_prev, sizeof(double), cudaMemcpyHostToDevice, s));
  if (has_agg) {
    double* dst[5] = {x->agr_maggr, x->agr_al, x->agr_ab, x->agr_as, x->agr_ad};
    for (int q = 0; q < 5; ++q)
      CK(cudaMemcpyAsync(dst[q], agf.data() + q * s3, s3 * sizeof(double), cudaMemcpyHostToDevice, s));
    x->agr_ipass = (int)agg[1];
    x->agr_replay = (int)agg[2];  // vset scalings owed after the replayed updates (0: none made yet)
  }
  CK(cudaStreamSynchronize(s));
  x->time = h.time;
  x->iiter = h.iiter;
  x->erumass = h.erumass;
  // the next f3d_run replays the updates of the current meteo and source
  // intervals (Fall3d.f90:83-101 select them from the time)
  x->run_started = 1;
  x->meteo_time = h.time;
  x->source_time = h.time;
  x->meteotime = 1;
  x->sourcetime = 1;
  x->have_met = 0;
  return F3D_OK;
}

int f3d_download_coeffs(f3d_ctx* x, double* vx, double* vy, double* vz, double* rho, double* rkhor,
                        double* rkh1, double* rkver) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  const size_t b = (size_t)x->d.cells() * sizeof(double);
  cudaStream_t s = x->stream;
  auto cp = [&](double* dst, const double* src) -> int {
    if (!dst) return F3D_OK;
    CK(cudaMemcpyAsync(dst, src, b, is_dev(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    return F3D_OK;
  };
  int rc = cp(vx, x->vx);
  if (!rc) rc = cp(vy, x->vy);
  if (!rc) rc = cp(vz, x->vz);
  if (!rc) rc = cp(rho, x->rho);
  if (!rc) rc = cp(rkhor, x->rkhor);
  if (!rc) rc = cp(rkh1, x->rkh1);
  if (!rc) rc = cp(rkver, x->rkver);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s));
  return F3D_OK;
}

// vsettl iteration counts of the last f3d_meteo (nx*ny*nz*nc int32).
int f3d_download_iters(f3d_ctx* x, int* iters) {
  if (!x || !iters) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  CK(cudaMemcpyAsync(iters, x->iters, (size_t)x->d.cells() * x->g.nc * sizeof(int),
                     is_dev(iters) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  return F3D_OK;
}

int f3d_outputs(f3d_ctx* x, double* load, double* col_mass, double* c_grnd) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  int rc = F3D_OK;
  if (load) rc = f3d_output(x, F3D_OUT_LOAD, 0, 0, load, F3D_OUT_BINARY64);
  if (!rc && col_mass) rc = f3d_output(x, F3D_OUT_COL_MASS, 0, 0, col_mass, F3D_OUT_BINARY64);
  if (!rc && c_grnd) rc = f3d_output(x, F3D_OUT_C_GRND, 0, 0, c_grnd, F3D_OUT_BINARY64);
  return rc;
}

int f3d_set_option(f3d_ctx* x, int key, int value) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  if (key == F3D_OPT_FUSED) {
    x->opt_fused = value ? 1 : 0;
  } else if (key == F3D_OPT_TILE) {
    if (value < 0 || value > 3) return f3d::ctx_error(F3D_ERR_ARG, "tile shape must be 0..3");
    x->opt_tile = value;
  } else if (key == F3D_OPT_PREFETCH) {
    if (!value) f3d::ctx_prefetch_drop(x);
    x->opt_prefetch = value ? 1 : 0;
    if (value && !x->gc_on && !x->agr_on) {  // the second set now rather than at the first use
      if (int rc = prefetch_setup(x)) {
        x->pref_failed = 1;
        return rc;
      }
    }
  } else {
    return f3d::ctx_error(F3D_ERR_ARG, "unknown option");
  }
  return F3D_OK;
}

int f3d_get_option(const f3d_ctx* x, int key, int* value) {
  if (!x || !value) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  if (key == F3D_OPT_FUSED)
    *value = x->opt_fused;
  else if (key == F3D_OPT_TILE)
    *value = x->opt_tile;
  else if (key == F3D_OPT_PREFETCH)
    *value = x->opt_prefetch;
  else
    return f3d::ctx_error(F3D_ERR_ARG, "unknown option");
  return F3D_OK;
}

int f3d_ctx_stream(f3d_ctx* x, void** stream) {
  if (!x || !stream) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  *stream = (void*)x->stream;
  return F3D_OK;
}

int f3d_profile_enable(f3d_ctx* x, int enable) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  prof_drain(x);
  x->prof = enable ? 1 : 0;
  for (auto& v : x->prof_ms) v = 0.0;
  for (auto& v : x->prof_count) v = 0;
  return F3D_OK;
}

int f3d_profile_read(f3d_ctx* x, int cap, char* names, int name_len, long long* launches,
                     double* total_ms, int* nkinds) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  prof_drain(x);
  const int n = (int)x->prof_names.size();
  if (nkinds) *nkinds = n;
  for (int i = 0; i < n && i < cap; ++i) {
    if (names && name_len > 0) {
      strncpy(names + (size_t)i * name_len, x->prof_names[i].c_str(), (size_t)name_len - 1);
      names[(size_t)i * name_len + name_len - 1] = 0;
    }
    if (launches) launches[i] = x->prof_count[i];
    if (total_ms) total_ms[i] = x->prof_ms[i];
  }
  return F3D_OK;
}

int f3d_run_reset(f3d_ctx* x) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  f3d::ctx_prefetch_drop(x);
  x->run_started = 0;
  return F3D_OK;
}

}  // extern "C"

namespace f3d {
// Sources/Fall3d.f90:83-101 with the interval selection of
// libMaster/get_dbs_value_plane.f90:100-114 and get_source_nsrc.f90:41-59.
int ctx_run_prepare(f3d_ctx* x, const f3d_met_series* met, const f3d_src_series* src, double end_time,
                    int lookahead) {
  const size_t s3 = (size_t)x->d.cells(), pl = (size_t)x->d.plane();
  const int nc = x->g.nc;
  if (x->source_time <= x->time) {
    if (x->sourcetime) {
      const int ts = (int)x->time;
      int found = -1;
      size_t off = 0, off_found = 0, roff = 0, roff_found = 0;
      for (int it = 0; it < src->nint; ++it) {
        if (found < 0 && ts >= src->t1[it] && ts < src->t2[it]) {
          found = it;
          off_found = off;
          roff_found = roff;
        }
        off += (size_t)src->nsou[it];
        roff += (size_t)src->nsou[it] * nc;
      }
      if (found < 0) {
        char m[128];
        snprintf(m, sizeof m, "get_source_nsrc: no source interval at time %d", ts);
        return f3d::ctx_error(F3D_ERR_RANGE, m);
      }
      const int rc = f3d_source(x, src->nsou[found], src->isrc + off_found, src->jsrc + off_found,
                                src->ksrc + off_found, src->tmrat + roff_found);
      if (rc) return rc;
      if (x->agr_on && src->nplume) {  // settemplume at the end of source (source.f90:82)
        size_t po = 0;
        for (int it = 0; it < found; ++it) po += (size_t)src->nplume[it];
        const int r2 = f3d_aggregation_plume(x, src->nplume[found], src->pix + po, src->piy + po, src->piz + po,
                                             src->ptemp + po, src->pwater ? src->pwater + po : nullptr);
        if (r2) return r2;
      }
      x->source_time = (double)src->t2[found];
    }
    if (x->source_time >= end_time) x->sourcetime = 0;
  }
  if (x->meteo_time <= x->time) {
    if (x->meteotime) {
      const int ts = (int)(met->time_lag + x->time);
      const int nt = met->nt;
      if (ts < met->times[0] || ts > met->times[nt - 1]) {
        char m[128];
        snprintf(m, sizeof m, "get_dbs_value_plane: time %d outside the DBS interval", ts);
        return f3d::ctx_error(F3D_ERR_RANGE, m);
      }
      int itime = nt - 1, endsec = met->times[nt - 1];
      for (int it = 0; it < nt - 1; ++it)
        if (ts >= met->times[it] && ts < met->times[it + 1]) {
          itime = it;
          endsec = met->times[it + 1];
        }
      const size_t o3 = (size_t)itime * s3, o2 = (size_t)itime * pl;
      int rc;
      if (lookahead && x->pref_ready && x->pref_itime == itime) {
        rc = prefetch_commit(x);  // computed while the previous interval stepped
      } else {
        if (x->agr_on && met->qv && met->p) {
          if (int r2 = f3d_aggregation_met(x, met->qv + o3, met->p + o3)) return r2;
        }
        rc = f3d_meteo(x, met->u + o3, met->v + o3, met->w + o3, met->t + o3, met->tp + o3, met->rho + o3,
                       met->ust + o2, met->pblh + o2, met->rmol + o2, met->znt + o2,
                       met->prate ? met->prate + o2 : nullptr, met->ldu);
      }
      if (rc) return rc;
      x->meteo_time = (double)endsec - met->time_lag;
      // the next snapshot's update while this interval steps: the update due
      // at meteo_time reads snapshot itime + 1 (the steps are shorter than
      // a DBS interval; otherwise it is dropped and made when due)
      if (lookahead && x->meteo_time < end_time && itime + 1 < nt)
        if (int r3 = prefetch_start(x, met, itime + 1)) return r3;
    }
    if (x->meteo_time >= end_time) x->meteotime = 0;
  }
  return F3D_OK;
}

void ctx_advance(f3d_ctx* x) {  // Fall3d.f90:112-114
  x->time = x->time + x->dt;
  x->iiter = x->iiter + 1;
  x->erumass = x->erumass + x->flowrate * x->dt;
}

// After the stream has drained: a staging wait of the step kernel that gave
// up is an error (the status word is cleared for the next run).
int ctx_check_step_status(f3d_ctx* x) {
  int st = 0;
  CK(cudaMemcpyAsync(&st, small_step_status(x), sizeof st, cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  if (st & F3D_STEP_STAGING_TIMEOUT) {
    CK(cudaMemsetAsync(small_step_status(x), 0, sizeof st, x->stream));
    return f3d::ctx_error(F3D_ERR_CUDA, "step kernel: a staging copy did not arrive in time");
  }
  return F3D_OK;
}

int ctx_log(f3d_ctx* x, f3d_log_record* log, int log_cap, int* nlog) {
  // endstep.f90:51: mass budget every 10 minutes of simulated time
  if (x->iiter == 1 || std::fmod(x->time, 600.0) <= x->dt) {
    const bool rec = log && nlog && *nlog < log_cap;
    if (rec || x->gc_on) {
      double b[4], outmass = 0.0;
      int r2 = f3d_budget(x, &b[0], &b[1], &b[2], &b[3]);
      if (!r2) r2 = f3d_get_state(x, nullptr, nullptr, nullptr, nullptr, nullptr, &outmass, nullptr);
      if (r2) return r2;
      if (rec) {
        f3d_log_record& r = log[(*nlog)++];
        r.iiter = x->iiter;
        r.time = x->time;
        r.dt = x->dt;
        r.dtc = x->dtc;
        r.massvol = b[0];
        r.massdep = b[1];
        r.massdry = b[2];
        r.masswet = b[3];
        r.outmass = outmass;
        r.erumass = x->erumass;
      }
      // endstep.f90:71: after writim
      if (x->gc_on) {
        if (int r3 = gc_divcorr(x, b[0], b[1], outmass)) return r3;
      }
    }
  }
  return F3D_OK;
}
}  // namespace f3d

extern "C" {

// Sources/Fall3d.f90:73-121.
int f3d_run(f3d_ctx* x, const f3d_met_series* met, const f3d_src_series* src, double beg_time,
            double end_time, int max_steps, f3d_log_record* log, int log_cap, int* nlog) {
  if (!x || !met || !src) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  if (met->nt < 1) return f3d::ctx_error(F3D_ERR_ARG, "no meteorological snapshot");
  if (nlog) *nlog = 0;
  bool go_on = true;  // the reference's do-while runs at least one step
  if (!x->run_started) {
    x->time = beg_time;
    x->meteo_time = beg_time;
    x->source_time = beg_time;
    x->iiter = 0;
    x->meteotime = 1;
    x->sourcetime = 1;
    x->run_started = 1;
  } else {
    go_on = x->time < end_time;
    // a later end time than the last call's: the updates that call switched
    // off at its end (Fall3d.f90 stops them once their next time is past
    // the end) are due again
    if (x->meteo_time < end_time) x->meteotime = 1;
    if (x->source_time < end_time) x->sourcetime = 1;
  }
  int steps = 0;
  while (go_on) {
    if (int rc = f3d::ctx_run_prepare(x, met, src, end_time, x->opt_prefetch)) return rc;
    const int rc = f3d_step(x);
    if (rc) return rc;
    ++steps;
    if (int r2 = f3d::ctx_log(x, log, log_cap, nlog)) return r2;
    if (x->time >= end_time) go_on = false;
    if (max_steps > 0 && steps >= max_steps) go_on = false;
  }
  // a look-ahead update still in flight has copied what it reads of the
  // caller's series before the series may change
  if (x->pref_ready && cudaEventSynchronize(x->ev_staged) != cudaSuccess)
    return f3d::ctx_error(F3D_ERR_CUDA, "look-ahead meteo update failed");
  return f3d::ctx_check_step_status(x);
}

}  // extern "C"

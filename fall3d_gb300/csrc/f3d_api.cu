// f3d_api.cu -- the C ABI of include/fall3d_gpu.h.
//
// Fine-grained entry points marshal their array arguments: device pointers
// are used in place, host pointers are staged through device buffers and
// copied back (the Fortran driver's Master arrays live on the host).  Scalars
// passed by reference are always host memory.  Every call is synchronous.
//
// The coarse context keeps one scenario resident in HBM and enqueues all of
// its work on one CUDA stream; f3d_step does not synchronise.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fall3d_gpu.h"
#include "f3d_internal.h"

namespace {

thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define F3D_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return set_error(F3D_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),      \
                       __FILE__, __LINE__);                                                  \
  } while (0)

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(F3D_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return F3D_OK;
}

int check_dims(int nx, int ny, int nz) {
  if (nx < 3 || ny < 3 || nz < 3)
    return set_error(F3D_ERR_ARG, "grid must have nx, ny, nz >= 3 (got %d, %d, %d)", nx, ny, nz);
  return F3D_OK;
}

int check_zrange(int nz, int nz_loc, int iz_loc) {
  if (iz_loc < 1 || nz_loc < 2 || iz_loc + nz_loc - 1 > nz)
    return set_error(F3D_ERR_ARG,
                     "z range iz_loc=%d nz_loc=%d outside 1..%d (the reference needs nz_loc >= 2, "
                     "Domain.f90:37)",
                     iz_loc, nz_loc, nz);
  return F3D_OK;
}

// 1 = device (or managed), 0 = host, -1 = NULL
int ptr_kind(const void* p) {
  if (!p) return -1;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? 1 : 0;
}

// Stages the array arguments of one fine-grained call.
class Marshal {
 public:
  ~Marshal() {
    for (auto& a : args_)
      if (a.owned) cudaFree(a.dev);
  }
  // Registers an array of n elements; returns its device address (or NULL).
  template <class T>
  T* arr(const T* p, size_t n, bool out) {
    if (err_) return nullptr;
    if (!p) return nullptr;
    const int k = ptr_kind(p);
    if (kind_ < 0) kind_ = k;
    if (k != kind_) {
      err_ = set_error(F3D_ERR_ARG, "array arguments mix host and device pointers");
      return nullptr;
    }
    if (k == 1) return const_cast<T*>(p);
    Arg a{nullptr, (void*)p, n * sizeof(T), out, true};
    if (n == 0) n = 1;
    if (cudaMalloc(&a.dev, n * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      err_ = set_error(F3D_ERR_OOM, "cudaMalloc of %zu bytes failed", n * sizeof(T));
      return nullptr;
    }
    if (cudaMemcpy(a.dev, p, a.bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      err_ = set_error(F3D_ERR_CUDA, "host-to-device copy failed");
      cudaFree(a.dev);
      return nullptr;
    }
    args_.push_back(a);
    return reinterpret_cast<T*>(a.dev);
  }
  int error() const { return err_; }
  // Waits for the kernels and copies outputs back.
  int finish() {
    if (err_) return err_;
    F3D_CUDA(cudaGetLastError());
    F3D_CUDA(cudaDeviceSynchronize());
    for (auto& a : args_)
      if (a.out) F3D_CUDA(cudaMemcpy(a.host, a.dev, a.bytes, cudaMemcpyDeviceToHost));
    return F3D_OK;
  }

 private:
  struct Arg {
    void* dev;
    void* host;
    size_t bytes;
    bool out, owned;
  };
  std::vector<Arg> args_;
  int kind_ = -1;
  int err_ = 0;
};

// Scratch owned by the library for fine-grained calls that need work space.
struct TmpBuf {
  void* p = nullptr;
  ~TmpBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t bytes) {
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return set_error(F3D_ERR_OOM, "cudaMalloc of %zu bytes failed", bytes);
    }
    return F3D_OK;
  }
};

Dims dims(int nx, int ny, int nz) { return Dims{nx, ny, nz}; }

}  // namespace

namespace f3d {
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int ctx_error(int code, const char* msg) { return set_error(code, "%s", msg); }
}  // namespace f3d

using namespace f3d;

extern "C" {

int f3d_last_error(char* buf, int len) {
  const int n = (int)g_last_error.size();
  if (buf && len > 0) {
    const int m = n < len - 1 ? n : len - 1;
    memcpy(buf, g_last_error.data(), (size_t)m);
    buf[m] = 0;
  }
  return n;
}

const char* f3d_version(void) { return "fall3d_gb300 1.0 (sm_103a)"; }

long long f3d_kernel_launches(void) { return g_launches.load(); }

/* ================================================================== */
/* Fine-grained entry points                                          */
/* ================================================================== */

int f3d_setbcc(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
               const int* iz_loc, const double* vx, const double* vy, const double* vz,
               const double* vset, const double* vdep, const double* rkver, const double* dz) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* dvx = m.arr(vx, (size_t)d.cells(), false);
  const double* dvy = m.arr(vy, (size_t)d.cells(), false);
  const double* dvz = m.arr(vz, (size_t)d.cells(), false);
  const double* dvs = m.arr(vset, (size_t)d.cells(), false);
  const double* dvd = m.arr(vdep, (size_t)d.plane(), false);
  const double* drk = m.arr(rkver, (size_t)d.cells(), false);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  if (m.error()) return m.error();
  launch_setbcc<double>(dc, 0, d, *nz_loc, *iz_loc, dvx, dvy, dvz, dvs, 0, dvd, 0, drk, ddz, 1, 0);
  return m.finish();
}

int f3d_advctzc(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
                const int* iz_loc, const double* vz, const double* vset, const double* dz,
                const double* dt, const int* lmeth) {
  (void)lmeth;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* dvz = m.arr(vz, (size_t)d.cells(), false);
  const double* dvs = m.arr(vset, (size_t)d.cells(), false);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  if (m.error()) return m.error();
  launch_advctzc<double>(dc, 0, d, *nz_loc, *iz_loc, dvz, dvs, 0, ddz, *dt, 1, 0);
  return m.finish();
}

int f3d_advctx(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
               const int* iz_loc, const double* vx, const double* dx, const double* dt,
               double* work, const int* lmeth) {
  (void)work;
  (void)lmeth;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* dv = m.arr(vx, (size_t)d.cells(), false);
  if (m.error()) return m.error();
  launch_advctx<double>(dc, 0, d, *nz_loc, *iz_loc, dv, *dx, *dt, 1, 0);
  return m.finish();
}

int f3d_advcty(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
               const int* iz_loc, const double* vy, const double* dy, const double* dt,
               double* work, const int* lmeth) {
  (void)work;
  (void)lmeth;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* dv = m.arr(vy, (size_t)d.cells(), false);
  if (m.error()) return m.error();
  launch_advcty<double>(dc, 0, d, *nz_loc, *iz_loc, dv, *dy, *dt, 1, 0);
  return m.finish();
}

int f3d_diffz(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
              const int* iz_loc, const double* dz, const double* dt, const double* rkver,
              const double* rho, double* work) {
  (void)work;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  const double* drk = m.arr(rkver, (size_t)d.cells(), false);
  const double* drho = m.arr(rho, (size_t)d.cells(), false);
  if (m.error()) return m.error();
  launch_diffz<double>(dc, 0, d, *nz_loc, *iz_loc, ddz, *dt, drk, drho, nullptr, nullptr, 1, 0);
  return m.finish();
}

int f3d_diffx(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
              const int* iz_loc, const double* dx, const double* dt, const double* rkhor,
              const double* rho, double* work) {
  (void)work;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* drk = m.arr(rkhor, (size_t)d.cells(), false);
  const double* drho = m.arr(rho, (size_t)d.cells(), false);
  if (m.error()) return m.error();
  launch_diffx<double>(dc, 0, d, *nz_loc, *iz_loc, *dx, *dt, drk, drho, nullptr, nullptr, 1, 0);
  return m.finish();
}

int f3d_diffy(double* c, const int* nx, const int* ny, const int* nz, const int* nz_loc,
              const int* iz_loc, const double* dy, const double* dt, const double* rkhor,
              const double* rho, double* work) {
  (void)work;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  const double* drk = m.arr(rkhor, (size_t)d.cells(), false);
  const double* drho = m.arr(rho, (size_t)d.cells(), false);
  if (m.error()) return m.error();
  launch_diffy<double>(dc, 0, d, *nz_loc, *iz_loc, *dy, *dt, drk, drho, nullptr, nullptr, 1, 0);
  return m.finish();
}

int f3d_wetdep(double* c, double* cwet, const int* ic, const int* nx, const int* ny,
               const int* nz, const int* nz_loc, const int* iz_loc, const double* dt,
               const double* diam, const double* zlayer, const double* dz, const double* zi,
               const double* prate) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  if (*ic < 1) return set_error(F3D_ERR_ARG, "ic must be >= 1");
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), true);
  double* dcw = m.arr(cwet, (size_t)d.plane() * (*ic + 1), true);
  const double* ddiam = m.arr(diam, (size_t)*ic, false);
  const double* dzl = m.arr(zlayer, (size_t)*nz, false);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  const double* dzi = m.arr(zi, (size_t)d.plane(), false);
  const double* dpr = m.arr(prate, (size_t)d.plane(), false);
  if (m.error()) return m.error();
  launch_wetdep<double>(dc, 0, dcw, *ic - 1, d, *nz_loc, *iz_loc, *dt, ddiam, dzl, ddz, dzi, dpr, nullptr, 1,
                        0);
  return m.finish();
}

int f3d_accum(double* c, double* cdry, const int* ic, const int* nx, const int* ny,
              const int* nz, const int* nz_loc, const int* iz_loc, const double* vz,
              const double* dt, const double* vset, const double* vdep) {
  (void)vz;
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  if (*ic < 1) return set_error(F3D_ERR_ARG, "ic must be >= 1");
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo(), false);
  double* dcd = m.arr(cdry, (size_t)d.plane() * (*ic + 1), true);
  const double* dvs = m.arr(vset, (size_t)d.cells(), false);
  const double* dvd = m.arr(vdep, (size_t)d.plane(), false);
  if (m.error()) return m.error();
  launch_accum<double>(dc, 0, dcd, *ic - 1, d, *iz_loc, *dt, dvs, 0, dvd, 0, 1, 0);
  return m.finish();
}

int f3d_clip(double* c, const int* nx, const int* ny, const int* nz, const int* nc,
             const int* ic_loc, const int* nc_loc) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (*ic_loc < 1 || *nc_loc < 0 || *ic_loc + *nc_loc - 1 > *nc)
    return set_error(F3D_ERR_ARG, "class range outside 1..nc");
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo() * *nc, true);
  if (m.error()) return m.error();
  launch_clip<double>(dc + (long long)(*ic_loc - 1) * d.halo(), d.halo() * *nc_loc, 0);
  return m.finish();
}

int f3d_cmass2d(const double* c, const double* vx, const double* vy, const double* vz,
                const double* vset, const int* nx, const int* ny, const int* nz, const int* nc,
                const int* ic_loc, const int* nc_loc, const int* iz_loc, const int* nz_loc,
                const double* dx, const double* dy, const double* dz, const double* dt,
                double* outmass) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  if (*ic_loc < 1 || *nc_loc < 0 || *ic_loc + *nc_loc - 1 > *nc)
    return set_error(F3D_ERR_ARG, "class range outside 1..nc");
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  const double* dc = m.arr(c, (size_t)d.halo() * *nc, false);
  const double* dvx = m.arr(vx, (size_t)d.cells(), false);
  const double* dvy = m.arr(vy, (size_t)d.cells(), false);
  const double* dvz = m.arr(vz, (size_t)d.cells(), false);
  const double* dvs = m.arr(vset, (size_t)d.cells() * *nc, false);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  if (m.error()) return m.error();
  const size_t part = cmass2d_scratch_bytes(d, *iz_loc, *nz_loc);
  TmpBuf tmp;
  if (int r = tmp.alloc(part + 64)) return r;
  double* dout = reinterpret_cast<double*>(reinterpret_cast<char*>(tmp.p) + part);
  F3D_CUDA(cudaMemcpy(dout, outmass, sizeof(double), cudaMemcpyHostToDevice));
  launch_cmass2d<double>(dc, dvx, dvy, dvz, dvs, d, *ic_loc, *nc_loc, *iz_loc, *nz_loc, *dx, *dy,
                         ddz, *dt, tmp.p, dout, 0);
  if (int r = m.finish()) return r;
  F3D_CUDA(cudaMemcpy(outmass, dout, sizeof(double), cudaMemcpyDeviceToHost));
  return F3D_OK;
}

// ------------------------------------------------------------------------
// cmass2d without allocation.  The block partials of the reduction and the
// device copy of outmass live in one file-scope device array instead of a
// cudaMalloc'd buffer.  Nothing in it has to start at zero: every block
// writes its partial before the finishing kernel reads it, and outmass is
// copied in before the launch.  The array is shared by every call on the
// device, so calls must not overlap (one host thread at a time per device).
static __device__ __align__(256) unsigned char f3d_noalloc_scratch[F3D_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::atomic<void*> g_noalloc_ptr[kMaxDevices];

// Address of the scratch array on the current device: looked up once per
// device (the first call on a device does this set-up), then cached.
int noalloc_scratch(void** out) {
  int dev = -1;
  F3D_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(F3D_ERR_ARG, "device ordinal %d out of range", dev);
  void* p = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    F3D_CUDA(cudaGetSymbolAddress(&p, f3d_noalloc_scratch));
    g_noalloc_ptr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return F3D_OK;
}

int require_device(const void* p, const char* name) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return set_error(F3D_ERR_ARG, "%s: not a CUDA pointer", name);
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return set_error(F3D_ERR_ARG, "%s must be device (or managed) memory", name);
  return F3D_OK;
}
}  // namespace

int f3d_cmass2d_noalloc(const double* c, const double* vx, const double* vy, const double* vz,
                        const double* vset, const int* nx, const int* ny, const int* nz,
                        const int* nc, const int* ic_loc, const int* nc_loc, const int* iz_loc,
                        const int* nz_loc, const double* dx, const double* dy, const double* dz,
                        const double* dt, double* outmass) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (int r = check_zrange(*nz, *nz_loc, *iz_loc)) return r;
  if (*ic_loc < 1 || *nc_loc < 0 || *ic_loc + *nc_loc - 1 > *nc)
    return set_error(F3D_ERR_ARG, "class range outside 1..nc");
  const void* arrs[] = {c, vx, vy, vz, vset, dz};
  const char* names[] = {"c", "vx", "vy", "vz", "vset", "dz"};
  for (int q = 0; q < 6; ++q)
    if (int r = require_device(arrs[q], names[q])) return r;
  const Dims d = dims(*nx, *ny, *nz);
  const size_t part = cmass2d_scratch_bytes(d, *iz_loc, *nz_loc);
  if (part + sizeof(double) > (size_t)F3D_NOALLOC_SCRATCH_BYTES)
    return set_error(F3D_ERR_RANGE, "f3d_cmass2d_noalloc needs %zu scratch bytes, more than the %d available",
                     part + sizeof(double), F3D_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  if (int r = noalloc_scratch(&scratch)) return r;
  double* dout = reinterpret_cast<double*>(reinterpret_cast<char*>(scratch) + part);
  F3D_CUDA(cudaMemcpy(dout, outmass, sizeof(double), cudaMemcpyDefault));
  launch_cmass2d<double>(c, vx, vy, vz, vset, d, *ic_loc, *nc_loc, *iz_loc, *nz_loc, *dx, *dy, dz, *dt,
                         scratch, dout, 0);
  F3D_CUDA(cudaGetLastError());
  F3D_CUDA(cudaMemcpy(outmass, dout, sizeof(double), cudaMemcpyDefault));
  return F3D_OK;
}

int f3d_cmass3d(const double* c, const double* cload, const double* cdry, const double* cwet,
                const int* nx, const int* ny, const int* nz, const int* nc, const double* dx,
                const double* dy, const double* dz, double* massvol, double* massdep,
                double* massdry, double* masswet) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  const double* dc = m.arr(c, (size_t)d.halo() * *nc, false);
  const double* dcl = m.arr(cload, (size_t)d.plane(), false);
  const double* dcd = m.arr(cdry, (size_t)d.plane(), false);
  const double* dcw = m.arr(cwet, (size_t)d.plane(), false);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  if (m.error()) return m.error();
  const long long nterms = d.plane() * *nc;
  TmpBuf tmp;
  if (int r = tmp.alloc(reduce_scratch_bytes(nterms, 4) + 64)) return r;
  double* dout = reinterpret_cast<double*>(reinterpret_cast<char*>(tmp.p) + reduce_scratch_bytes(nterms, 4));
  launch_cmass3d<double>(dc, dcl, dcd, dcw, d, *nc, *dx, *dy, ddz, tmp.p, dout, 0);
  if (int r = m.finish()) return r;
  double h[4];
  F3D_CUDA(cudaMemcpy(h, dout, sizeof h, cudaMemcpyDeviceToHost));
  *massvol = h[0];
  *massdep = h[1];
  *massdry = h[2];
  *masswet = h[3];
  return F3D_OK;
}

int f3d_getc0(double* cdry, double* cwet, double* cload, const int* nx, const int* ny,
              const int* nc, const int* np) {
  if (*nx < 1 || *ny < 1 || *nc < 0 || *np < 0 || *np > *nc)
    return set_error(F3D_ERR_ARG, "invalid sizes");
  const Dims d = dims(*nx, *ny, 1);
  const size_t n = (size_t)d.plane() * (*nc + 1);
  Marshal m;
  double* dd = m.arr(cdry, n, true);
  double* dw = m.arr(cwet, n, true);
  double* dl = m.arr(cload, n, true);
  if (m.error()) return m.error();
  launch_getc0(dd, dw, dl, d, *nc, *np, 0);
  return m.finish();
}

int f3d_setsrc(double* c, const int* nx, const int* ny, const int* nz, const int* nc,
               const int* nsou, const int* isrc, const int* jsrc, const int* ksrc,
               const double* tmrat, const double* dz, const double* zlayer, const double* Hm1,
               const double* dX1, const double* dX2, const double* dt) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  const int n = *nsou;
  if (n < 0) return set_error(F3D_ERR_ARG, "nsou < 0");
  // validate indices on the host (reasrc.f90:76-80)
  std::vector<int> hi(n), hj(n), hk(n);
  if (n > 0) {
    const int kind = ptr_kind(isrc);
    const cudaMemcpyKind dir = kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    F3D_CUDA(cudaMemcpy(hi.data(), isrc, sizeof(int) * n, dir));
    F3D_CUDA(cudaMemcpy(hj.data(), jsrc, sizeof(int) * n, dir));
    F3D_CUDA(cudaMemcpy(hk.data(), ksrc, sizeof(int) * n, dir));
  }
  for (int s = 0; s < n; ++s)
    if (hi[s] < 1 || hi[s] > *nx || hj[s] < 1 || hj[s] > *ny || hk[s] > *nz)
      return set_error(F3D_ERR_RANGE, "source %d at (%d,%d,%d) outside the grid", s + 1, hi[s], hj[s],
                       hk[s]);
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  double* dc = m.arr(c, (size_t)d.halo() * *nc, true);
  const int* di = m.arr(isrc, (size_t)n, false);
  const int* dj = m.arr(jsrc, (size_t)n, false);
  const int* dk = m.arr(ksrc, (size_t)n, false);
  const std::vector<int> link = source_links(n, hi.data(), hj.data(), hk.data(), *nz);
  const int* dln = m.arr(link.data(), link.size(), false);
  const double* dtm = m.arr(tmrat, (size_t)n * *nc, false);
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  const double* dzl = m.arr(zlayer, (size_t)*nz, false);
  const double* dh = m.arr(Hm1, (size_t)d.plane(), false);
  if (m.error()) return m.error();
  launch_setsrc<double>(dc, d.halo(), d, *nc, n, di, dj, dk, dln, dtm, ddz, dzl, dh, *dX1, *dX2, *dt, 0);
  return m.finish();
}

int f3d_finddt(const int* nx, const int* ny, const int* nz, const int* nc, const double* dX1,
               const double* dX2, const double* dz, const double* vx, const double* vy,
               const double* vz, const double* vset, const double* rkh1, const double* rkhor,
               const double* rkver, const double* safety_factor, double* dt, double* dtc) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  const double* dvx = m.arr(vx, (size_t)d.cells(), false);
  const double* dvy = m.arr(vy, (size_t)d.cells(), false);
  const double* dvz = m.arr(vz, (size_t)d.cells(), false);
  const double* dvs = m.arr(vset, (size_t)d.cells() * *nc, false);
  const double* dk1 = m.arr(rkh1, (size_t)d.cells(), false);
  const double* dkh = m.arr(rkhor, (size_t)d.cells(), false);
  const double* dkv = m.arr(rkver, (size_t)d.cells(), false);
  if (m.error()) return m.error();
  TmpBuf tmp;
  if (int r = tmp.alloc(sizeof(unsigned long long))) return r;
  F3D_CUDA(cudaMemset(tmp.p, 0, sizeof(unsigned long long)));
  launch_finddt(d, *nc, *dX1, *dX2, ddz, dvx, dvy, dvz, dvs, dk1, dkh, dkv,
                reinterpret_cast<unsigned long long*>(tmp.p), 0);
  if (int r = m.finish()) return r;
  double dtcn;
  F3D_CUDA(cudaMemcpy(&dtcn, tmp.p, sizeof dtcn, cudaMemcpyDeviceToHost));
  dtcn = fmax2(dtcn, 1e-13);  // finddt.f90:58-66
  *dtc = 1.0 / dtcn;
  *dt = *safety_factor * *dtc;
  return F3D_OK;
}

int f3d_kappa3(const int* nx, const int* ny, const int* nz, const int* modkv, const int* modkh,
               const int* coord_sys, const double* rkv0, const double* rkh0, const double* Csh,
               const double* dX1, const double* dX2, const double* dx, const double* dy,
               const double* dz, const double* zlayer, const double* Hm1, const double* vx,
               const double* vy, const double* vptemp, const double* ustar, const double* zi,
               const double* rl, double* rkver, double* rkhor) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  const double* dzl = m.arr(zlayer, (size_t)*nz, false);
  const double* dh = m.arr(Hm1, (size_t)d.plane(), false);
  const double* dvx = m.arr(vx, (size_t)d.cells(), false);
  const double* dvy = m.arr(vy, (size_t)d.cells(), false);
  const double* dvp = m.arr(vptemp, (size_t)d.cells(), false);
  const double* dus = m.arr(ustar, (size_t)d.plane(), false);
  const double* dzi = m.arr(zi, (size_t)d.plane(), false);
  const double* drl = m.arr(rl, (size_t)d.plane(), false);
  double* dkv = m.arr(rkver, (size_t)d.cells(), true);
  double* dkh = m.arr(rkhor, (size_t)d.cells(), true);
  if (m.error()) return m.error();
  launch_kappa3(d, *modkv, *modkh, *coord_sys, *rkv0, *rkh0, *Csh, *dX1, *dX2, *dx, *dy, ddz, dzl,
                dh, dvx, dvy, dvp, dus, dzi, drl, dkv, dkh, 0);
  return m.finish();
}

int f3d_setvset(const int* nx, const int* ny, const int* nz, const int* nc, const int* np,
                const int* modv, const double* diam, const double* rhop, const double* psi,
                const double* sphe, const double* tempe, const double* rho, const int* aggregate,
                const double* vset_factor, double* vset, double* cd) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  if (*np < 0 || *np > *nc) return set_error(F3D_ERR_ARG, "np outside 0..nc");
  if (*modv < 1 || *modv > 4) return set_error(F3D_ERR_ARG, "modv must be 1..4");
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  const double* ddi = m.arr(diam, (size_t)*nc, false);
  const double* drp = m.arr(rhop, (size_t)*nc, false);
  const double* dps = m.arr(psi, (size_t)*nc, false);
  const double* dsp = m.arr(sphe, (size_t)*nc, false);
  const double* dte = m.arr(tempe, (size_t)d.cells(), false);
  const double* drh = m.arr(rho, (size_t)d.cells(), false);
  double* dvs = m.arr(vset, (size_t)d.cells() * *nc, true);
  if (m.error()) return m.error();
  TmpBuf tmp;
  const size_t sb = setvset_scratch_bytes(d, *np);
  if (int r = tmp.alloc(sb + 256)) return r;
  char* small = reinterpret_cast<char*>(tmp.p) + sb;
  double* dcd = reinterpret_cast<double*>(small);
  int* dst = reinterpret_cast<int*>(small + 64);
  F3D_CUDA(cudaMemcpy(dcd, cd, sizeof(double), cudaMemcpyHostToDevice));
  launch_setvset(d, *nc, *np, *modv, ddi, drp, dps, dsp, dte, drh, *aggregate, *vset_factor, dvs,
                 nullptr, dcd, tmp.p, dst, 0);
  if (int r = m.finish()) return r;
  int status = 0;
  F3D_CUDA(cudaMemcpy(&status, dst, sizeof(int), cudaMemcpyDeviceToHost));
  F3D_CUDA(cudaMemcpy(cd, dcd, sizeof(double), cudaMemcpyDeviceToHost));
  if (status) return set_error(F3D_ERR_NOCONV, "No convergence in vsettl routine");
  return F3D_OK;
}

int f3d_dmath_eval(int op, long long n, const double* x, double* y) {
  if (op < 0 || op > 2 || n < 0) return set_error(F3D_ERR_ARG, "op must be 0 (log), 1 (exp) or 2 (quotient), n >= 0");
  if (n > 0 && (!x || !y)) return set_error(F3D_ERR_ARG, "NULL argument");
  Marshal m;
  const double* dx = m.arr(x, (size_t)n * (op == 2 ? 2 : 1), false);
  double* dy = m.arr(y, (size_t)n, true);
  if (m.error()) return m.error();
  launch_dmath_eval(op, n, dx, dy, 0);
  return m.finish();
}

int f3d_setvdrydep(const int* nx, const int* ny, const int* nc, const double* diam,
                   const double* zlayer, const double* ldu, const double* rl, const double* znt,
                   const double* ustar, const double* tempe, const double* rho, double* vdep) {
  if (*nx < 1 || *ny < 1 || *nc < 0) return set_error(F3D_ERR_ARG, "invalid sizes");
  const Dims d = dims(*nx, *ny, 1);
  Marshal m;
  const double* ddi = m.arr(diam, (size_t)*nc, false);
  const double* dzl = m.arr(zlayer, (size_t)1, false);
  const double* dld = m.arr(ldu, (size_t)d.plane(), false);
  const double* drl = m.arr(rl, (size_t)d.plane(), false);
  const double* dzn = m.arr(znt, (size_t)d.plane(), false);
  const double* dus = m.arr(ustar, (size_t)d.plane(), false);
  const double* dte = m.arr(tempe, (size_t)d.plane(), false);
  const double* drh = m.arr(rho, (size_t)d.plane(), false);
  double* dvd = m.arr(vdep, (size_t)d.plane() * *nc, true);
  if (m.error()) return m.error();
  launch_setvdrydep(d, *nc, ddi, dzl, dld, drl, dzn, dus, dte, drh, dvd, 0);
  return m.finish();
}

int f3d_meteo_scale(const int* nx, const int* ny, const int* nz, const int* coord_sys,
                    const double* dX1, const double* dX2, const double* dz, const double* Hm1,
                    const double* topg, double* vx, double* vy, double* vz, double* rho,
                    const double* rkhor, double* rkh1, double* divu) {
  if (int r = check_dims(*nx, *ny, *nz)) return r;
  const Dims d = dims(*nx, *ny, *nz);
  Marshal m;
  const double* ddz = m.arr(dz, (size_t)(*nz + 1), false);
  const double* dh = m.arr(Hm1, (size_t)d.plane(), false);
  const double* dtp = m.arr(topg, (size_t)d.plane(), false);
  double* dvx = m.arr(vx, (size_t)d.cells(), true);
  double* dvy = m.arr(vy, (size_t)d.cells(), true);
  double* dvz = m.arr(vz, (size_t)d.cells(), true);
  double* drh = m.arr(rho, (size_t)d.cells(), true);
  const double* dkh = m.arr(rkhor, (size_t)d.cells(), false);
  double* dk1 = m.arr(rkh1, (size_t)d.cells(), true);
  double* ddv = m.arr(divu, (size_t)d.cells(), true);
  if (m.error()) return m.error();
  launch_meteo_scale(d, *coord_sys, *dX1, *dX2, ddz, dh, dtp, dvx, dvy, dvz, drh, dkh, dk1, ddv, 0);
  return m.finish();
}

}  // extern "C"

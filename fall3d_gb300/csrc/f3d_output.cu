// f3d_output.cu -- the output variables of Sources/printres_nc.f90 computed
// on the device, so that a results record leaves the GPU as a few (nx,ny)
// planes (binary64, or binary32 as the reference's netCDF variables are
// NF90_FLOAT, printres_nc.f90:805-841) instead of the whole state.
//
// Every variable is evaluated in binary64 in the reference's order of
// operations (--fmad=false): a sum over classes is accumulated from 0 in
// class order and divided by Hm1 afterwards, the column trapezoid runs
// upwards from the first layer, and the final unit factor multiplies the
// sum.  In the precision form the binary32 state is widened first.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "f3d_ctx_impl.h"

namespace f3d {
namespace {

constexpr int OB = 128;  // threads per block: one column (i, j) each

// sum over the listed classes of c(i,j,k,ic) (0 + c1 + c2 + ...)
template <class T>
__device__ __forceinline__ double class_sum(const T* c, long long hb, long long q, const int* cls,
                                            int ncls) {
  double s = 0.0;
  for (int n = 0; n < ncls; ++n) s = s + (double)c[(long long)cls[n] * hb + q];
  return s;
}

// z-cumulative concentration, g/m2 (printres_nc.f90:216-246 particles and
// gases, :281-387 PM05/PM10/PM20): w(k) = (sum over the classes)/Hm1,
// work2d = sum_{k<nz} dz(k)*0.5*(w(k)+w(k+1)), times 1e3.
template <class T>
__global__ void k_out_column(const T* c, Dims d, const int* cls, int ncls, const double* dz,
                             const double* Hm1, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  if (p >= d.plane()) return;
  const int i = (int)(p % d.nx) + 1, j = (int)(p / d.nx) + 1;
  const long long hb = d.halo();
  const double h = Hm1[p];
  double acc = 0.0;
  double wp = class_sum<T>(c, hb, d.C(i, j, 1), cls, ncls) / h;
  for (int k = 1; k <= d.nz - 1; ++k) {
    const double wn = class_sum<T>(c, hb, d.C(i, j, k + 1), cls, ncls) / h;
    acc = acc + dz[k] * 0.5 * (wp + wn);
    wp = wn;
  }
  out[p] = 1e3 * acc;
}

// concentration at the first layer, g/m3 (printres_nc.f90:389-493):
// 1e3*(sum over the classes of c(i,j,1,ic))/Hm1.
template <class T>
__global__ void k_out_ground(const T* c, Dims d, const int* cls, int ncls, const double* Hm1,
                             double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  if (p >= d.plane()) return;
  const int i = (int)(p % d.nx) + 1, j = (int)(p / d.nx) + 1;
  const double s = class_sum<T>(c, d.halo(), d.C(i, j, 1), cls, ncls);
  out[p] = 1e3 * s / Hm1[p];
}

// aerosol optical thickness (printres_nc.f90:495-540): for each aerosol
// class in class order and each layer upwards,
// work2d += dz(k)*0.5*(w(k)+w(k+1))*0.75*Qeff(ieff)/(rhop(ic)*reff(ieff))
// with w = c(ic)/Hm1; qeff[n] and den[n] = rhop*reff belong to cls[n].
template <class T>
__global__ void k_out_aot(const T* c, Dims d, const int* cls, const double* qeff, const double* den,
                          int ncls, const double* dz, const double* Hm1, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  if (p >= d.plane()) return;
  const int i = (int)(p % d.nx) + 1, j = (int)(p / d.nx) + 1;
  const long long hb = d.halo();
  const double h = Hm1[p];
  double acc = 0.0;
  for (int n = 0; n < ncls; ++n) {
    const T* cc = c + (long long)cls[n] * hb;
    const double q = qeff[n], r = den[n];
    double wp = (double)cc[d.C(i, j, 1)] / h;
    for (int k = 1; k <= d.nz - 1; ++k) {
      const double wn = (double)cc[d.C(i, j, k + 1)] / h;
      acc = acc + dz[k] * 0.5 * (wp + wn) * 0.75 * q / r;
      wp = wn;
    }
  }
  out[p] = acc;
}

// deposit plane (printres_nc.f90:105-189): field(:,:,ic)/Hm1 of cload or cwet
__global__ void k_out_plane(const double* f, long long n, const double* Hm1, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  if (p < n) out[p] = f[p] / Hm1[p];
}

// deposit thickness, cm (printres_nc.f90:191-214): 1e2*(sum over particle
// classes of cload(ic)/rhop(ic))/Hm1.
__global__ void k_out_thick(const double* cload, long long pl, int np, const double* rhop,
                            const double* Hm1, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  if (p >= pl) return;
  double s = 0.0;
  for (int ic = 1; ic <= np; ++ic) s = s + cload[(long long)ic * pl + p] / rhop[ic - 1];
  out[p] = 1e2 * s / Hm1[p];
}

// concentration at a flight level, g/m3 (printres_nc.f90:542-573 and
// Sources/setcut.f90:1-54): the particle concentration w = (sum c)/Hm1
// interpolated linearly in pressure between the two layers whose
// pressures bracket pnom (p(k) >= pnom > p(k+1)), 0 below the first layer
// or when no pair of layers brackets it; times 1e3.
template <class T>
__global__ void k_out_fl(const T* c, Dims d, const int* cls, int ncls, const double* pres,
                         double pnom, const double* Hm1, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  const long long pl = d.plane();
  if (p >= pl) return;
  const int i = (int)(p % d.nx) + 1, j = (int)(p / d.nx) + 1;
  double v = 0.0;
  if (!(pnom > pres[p])) {
    for (int k = 1; k <= d.nz - 1; ++k) {
      const double pk = pres[(long long)(k - 1) * pl + p], pk1 = pres[(long long)k * pl + p];
      if (pnom <= pk && pnom > pk1) {
        const double s = (pnom - pk) / (pk1 - pk);
        const double h = Hm1[p];
        const long long hb = d.halo();
        const double wk = class_sum<T>(c, hb, d.C(i, j, k), cls, ncls) / h;
        const double wk1 = class_sum<T>(c, hb, d.C(i, j, k + 1), cls, ncls) / h;
        v = wk * (1.0 - s) + wk1 * s;
        break;
      }
    }
  }
  out[p] = 1e3 * v;
}

// 3-D concentration, g/m3 (printres_nc.f90:575-601 all particles,
// :646-671 one class): 1e3*((sum over the classes)/Hm1) on the model
// levels, or with `asl` moved to heights above sea level by
// Sources/ter2asl.f90:1-55 (linear in height between the terrain-following
// levels that bracket zlayer(k) above max(0,topg); 0 below the first level
// and above the last).
template <class T>
__global__ void k_out_con(const T* c, Dims d, const int* cls, int ncls, const double* Hm1,
                          const double* zlayer, const double* topg, int asl, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  const long long pl = d.plane();
  if (p >= pl) return;
  const int i = (int)(p % d.nx) + 1, j = (int)(p / d.nx) + 1;
  const long long hb = d.halo();
  const double h = Hm1[p];
  auto val = [&](int k) { return 1e3 * (class_sum<T>(c, hb, d.C(i, j, k), cls, ncls) / h); };
  if (!asl) {
    for (int k = 1; k <= d.nz; ++k) out[(long long)(k - 1) * pl + p] = val(k);
    return;
  }
  const double zo = fmax2(0.0, topg[p]);
  for (int k = 1; k <= d.nz; ++k) {
    const double zasl = zlayer[k - 1];
    double v = 0.0;
    if (!(zasl < zo + zlayer[0])) {
      for (int kk = 1; kk <= d.nz - 1; ++kk) {
        if (zasl >= zo + zlayer[kk - 1] && zasl <= zo + zlayer[kk]) {
          const double s = (zo + zlayer[kk] - zasl) / (zlayer[kk] - zlayer[kk - 1]);
          v = s * val(kk) + (1.0 - s) * val(kk + 1);
          break;
        }
      }
    }
    out[(long long)(k - 1) * pl + p] = v;
  }
}

// a binary64 3-D field (x fastest) times Hm1 or not, with `asl` moved to
// heights above sea level by ter2asl: the gravity-current winds
// (printres_nc.f90:603-644: vx*Hm1, vy*Hm1) and Maggr (:673-690)
__global__ void k_out_field(const double* f, int times_hm1, Dims d, const double* Hm1,
                            const double* zlayer, const double* topg, int asl, double* out) {
  const long long p = blockIdx.x * (long long)OB + threadIdx.x;
  const long long pl = d.plane();
  if (p >= pl) return;
  const double h = Hm1[p];
  auto val = [&](int k) {
    const double v = f[(long long)(k - 1) * pl + p];
    return times_hm1 ? v * h : v;
  };
  if (!asl) {
    for (int k = 1; k <= d.nz; ++k) out[(long long)(k - 1) * pl + p] = val(k);
    return;
  }
  const double zo = fmax2(0.0, topg[p]);
  for (int k = 1; k <= d.nz; ++k) {
    const double zasl = zlayer[k - 1];
    double v = 0.0;
    if (!(zasl < zo + zlayer[0])) {
      for (int kk = 1; kk <= d.nz - 1; ++kk) {
        if (zasl >= zo + zlayer[kk - 1] && zasl <= zo + zlayer[kk]) {
          const double s = (zo + zlayer[kk] - zasl) / (zlayer[kk] - zlayer[kk - 1]);
          v = s * val(kk) + (1.0 - s) * val(kk + 1);
          break;
        }
      }
    }
    out[(long long)(k - 1) * pl + p] = v;
  }
}

// Tracking points (Sources/writps.f90, writps_air.f90): one thread per
// point, bilinear weights of the cell (ip, jp) at (s, t) in (-1,1)^2.
// out per point: [0..6] load, thickness, ground concentration, PM05, PM10,
// PM20, column mass (writps.f90:64-148); then nz concentrations, nz
// extinctions, nz number concentrations and the AOD (writps_air.f90:
// 64-109); then np class loads (writps.f90:215-222, writps_end).
struct TrackClass {
  double diam, rhop;
  int aer;         // an aerosol class of get_AOT_prop's range
  double q, r;     // Qeff(ieff), reff(ieff)
};
template <class T>
__global__ void k_track(const T* c, const double* cload, Dims d, int np, const int* ip, const int* jp,
                        const double* sp, const double* tp, int npts, const TrackClass* cls,
                        const double* dz, const double* Hm1, double* out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= npts) return;
  const int nz = d.nz;
  const long long pl = d.plane(), hb = d.halo();
  const int stride = 7 + 3 * nz + 1 + np;
  double* o = out + (long long)n * stride;
  const int i = ip[n], j = jp[n];
  const double s = sp[n], t = tp[n], st = s * t;
  const double v1 = (1.0 - t - s + st) * 0.25, v2 = (1.0 - t + s - st) * 0.25;
  const double v3 = (1.0 + t + s + st) * 0.25, v4 = (1.0 + t - s - st) * 0.25;
  const long long p1 = d.P(i, j), p2 = d.P(i + 1, j), p3 = d.P(i + 1, j + 1), p4 = d.P(i, j + 1);
  const double h1 = Hm1[p1], h2 = Hm1[p2], h3 = Hm1[p3], h4 = Hm1[p4];
  auto pl4 = [&](const double* f) {  // v1*(f1/h1) + ... of a 2-D field
    return v1 * (f[p1] / h1) + v2 * (f[p2] / h2) + v3 * (f[p3] / h3) + v4 * (f[p4] / h4);
  };
  auto c4 = [&](int ic, int k) {  // the same of c(:,:,k,ic)
    const T* cc = c + (long long)(ic - 1) * hb;
    return v1 * ((double)cc[d.C(i, j, k)] / h1) + v2 * ((double)cc[d.C(i + 1, j, k)] / h2) +
           v3 * ((double)cc[d.C(i + 1, j + 1, k)] / h3) + v4 * ((double)cc[d.C(i, j + 1, k)] / h4);
  };
  o[0] = pl4(cload);
  double thick = 0.0;
  for (int ic = 1; ic <= np; ++ic) {
    const double* f = cload + (long long)ic * pl;
    const double rp = cls[ic - 1].rhop;
    thick = thick + v1 * (f[p1] / h1 / rp) + v2 * (f[p2] / h2 / rp) + v3 * (f[p3] / h3 / rp) + v4 * (f[p4] / h4 / rp);
  }
  o[1] = 1e2 * thick;
  auto acc4 = [&](double a, int ic, int k) {  // a + v1*(c1/h1) + ... term by term
    const T* cc = c + (long long)(ic - 1) * hb;
    return a + v1 * ((double)cc[d.C(i, j, k)] / h1) + v2 * ((double)cc[d.C(i + 1, j, k)] / h2) +
           v3 * ((double)cc[d.C(i + 1, j + 1, k)] / h3) + v4 * ((double)cc[d.C(i, j + 1, k)] / h4);
  };
  double cg = 0.0, pm5 = 0.0, pm10 = 0.0, pm20 = 0.0;
  for (int ic = 1; ic <= np; ++ic) cg = acc4(cg, ic, 1);
  for (int ic = 1; ic <= np; ++ic)
    if (cls[ic - 1].diam <= 5e-6) pm5 = acc4(pm5, ic, 1);
  for (int ic = 1; ic <= np; ++ic)
    if (cls[ic - 1].diam <= 1e-5) pm10 = acc4(pm10, ic, 1);
  for (int ic = 1; ic <= np; ++ic)
    if (cls[ic - 1].diam <= 2e-5) pm20 = acc4(pm20, ic, 1);
  o[2] = cg * 1e3;
  o[3] = pm5 * 1e3;
  o[4] = pm10 * 1e3;
  o[5] = pm20 * 1e3;
  double cummc = 0.0;
  for (int ic = 1; ic <= np; ++ic)
    for (int k = 1; k <= nz - 1; ++k) {
      const double cp1 = c4(ic, k), cp2 = c4(ic, k + 1);
      cummc = cummc + dz[k] * 0.5 * (cp1 + cp2);
    }
  o[6] = 1e3 * cummc;
  double* cz = o + 7;
  double* ext = cz + nz;
  double* nco = ext + nz;
  double aod = 0.0;
  const double pi = 3.14159265358979323846;
  for (int k = 1; k <= nz; ++k) {
    double a = 0.0, e = 0.0, q = 0.0;
    for (int ic = 1; ic <= np; ++ic) {
      const double cc = c4(ic, k);
      a = a + cc;
      const TrackClass& k1 = cls[ic - 1];
      if (k1.aer) {
        e = e + (cc * 0.75 * k1.q) / (k1.rhop * k1.r);
        aod = aod + (dz[k] * cc * 0.75 * k1.q) / (k1.rhop * k1.r);
      }
      if (0.5 * k1.diam <= 32e-6) q = q + (6.0 * cc) / (k1.rhop * pi * k1.diam * k1.diam * k1.diam);
    }
    cz[k - 1] = a * 1e3;
    ext[k - 1] = e * 1e6;
    nco[k - 1] = q * 1e-6;
  }
  o[7 + 3 * nz] = aod;
  for (int ic = 1; ic <= np; ++ic) o[8 + 3 * nz + ic - 1] = pl4(cload + (long long)ic * pl);
}

__global__ void k_out_to_f32(const double* a, long long n, float* b) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    b[q] = (float)a[q];
}

unsigned blocks(long long n) { return (unsigned)((n + OB - 1) / OB); }

// Sources/printres_nc.f90:2066-2123 (get_AOT_prop): effective radii in
// micrometres and extinction efficiencies of the 20 aerosol bins.
const double kReffUm[20] = {0.014, 0.020, 0.028, 0.040, 0.056, 0.079, 0.112, 0.158, 0.224, 0.316,
                            0.447, 0.631, 0.891, 1.259, 1.778, 2.512, 3.548, 5.012, 7.079, 10.000};
const double kQeff[20] = {0.00213, 0.00386, 0.00864, 0.02324, 0.06674, 0.18285, 0.44613,
                          0.93225, 1.63000, 2.35760, 2.83130, 2.90880, 2.72340, 2.50530,
                          2.35970, 2.27100, 2.21020, 2.16410, 2.12830, 2.10050};

}  // namespace
}  // namespace f3d

using namespace f3d;

namespace {

#define OK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) return f3d::ctx_error(F3D_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// Pressure at a flight level of the ICAO standard atmosphere
// (Sources/setcut.f90:60-107, standard_atm): three layers up to 32 km.
double standard_pressure(double z) {
  const double goo = 9.80665, Roo = 8.31432, Moo = 0.0289644;
  const double zoo = 0.0, Too = 288.15, poo = 101325.0, Loo = -0.0065;
  const double zo1 = 11000.0, To1 = 216.65, po1 = 22632.0;
  const double zo2 = 20000.0, To2 = 216.65, po2 = 5474.0, Lo2 = 0.001;
  if (z < zo1) {
    const double T = Too + Loo * (z - zoo);
    return poo * std::pow(Too / T, goo * Moo / (Roo * Loo));
  } else if (z < zo2) {
    return po1 * std::exp(-(goo * Moo * (z - zo1) / (Roo * To1)));
  }
  const double T = To2 + Lo2 * (z - zo2);
  return po2 * std::pow(To2 / T, goo * Moo / (Roo * Lo2));
}

// One device scratch block of the call: the (nx,ny[,nz]) binary64 result,
// its binary32 copy and the class tables.
struct Scratch {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
};

int finish(f3d_ctx* x, double* res, long long n, void* dst, int dst_type, Scratch& sc) {
  cudaStream_t s = x->stream;
  if (dst_type == F3D_OUT_BINARY32) {
    float* f = reinterpret_cast<float*>(res + n);
    k_out_to_f32<<<(unsigned)std::min<long long>((n + 255) / 256, 152LL * 8), 256, 0, s>>>(res, n, f);
    count_launch();
    OK(cudaMemcpyAsync(dst, f, sizeof(float) * n, cudaMemcpyDefault, s));
  } else {
    OK(cudaMemcpyAsync(dst, res, sizeof(double) * n, cudaMemcpyDefault, s));
  }
  OK(cudaGetLastError());
  OK(cudaStreamSynchronize(s));
  (void)sc;
  return F3D_OK;
}

// classes of printres_nc.f90's selections (0-based)
std::vector<int> particle_classes(const f3d_ctx* x) {
  std::vector<int> v;
  for (int ic = 0; ic < x->g.np; ++ic) v.push_back(ic);
  return v;
}

}  // namespace

extern "C" {

int f3d_output(f3d_ctx* x, int var, int index, int asl, void* dst, int dst_type) {
  if (!x || !dst) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  if (dst_type != F3D_OUT_BINARY64 && dst_type != F3D_OUT_BINARY32)
    return f3d::ctx_error(F3D_ERR_ARG, "dst_type must be F3D_OUT_BINARY64 or F3D_OUT_BINARY32");
  const Dims d = x->d;
  const int nc = x->g.nc, np = x->g.np;
  const long long pl = d.plane();
  long long n = pl;  // values in the result
  std::vector<int> cls;
  std::vector<double> q, r;
  switch (var) {
    case F3D_OUT_LOAD:
    case F3D_OUT_WET:
      if (index < 0 || index > np) return f3d::ctx_error(F3D_ERR_ARG, "class index outside 0..np");
      break;
    case F3D_OUT_THICK:
      break;
    case F3D_OUT_COL_MASS:
      if (index == 0) {
        cls = particle_classes(x);
      } else {
        if (index < 1 || np + index > nc) return f3d::ctx_error(F3D_ERR_ARG, "gas index outside 1..nc-np");
        cls.push_back(np + index - 1);
      }
      break;
    case F3D_OUT_PM_COL:
    case F3D_OUT_PM_GRND: {
      double thr;
      if (index == 5)
        thr = 5e-6;
      else if (index == 10)
        thr = 1e-5;
      else if (index == 20)
        thr = 2e-5;
      else
        return f3d::ctx_error(F3D_ERR_ARG, "PM size must be 5, 10 or 20 (micrometres)");
      for (int ic = 0; ic < np; ++ic)
        if (x->h_diam[ic] <= thr) cls.push_back(ic);
      break;
    }
    case F3D_OUT_C_GRND:
      cls = particle_classes(x);
      break;
    case F3D_OUT_AOT05: {
      double reff[20];
      for (int b = 0; b < 20; ++b) reff[b] = kReffUm[b] * 1e-6;
      for (int ic = 0; ic < np; ++ic) {
        const double rad = 0.5 * x->h_diam[ic];
        if (!(rad >= reff[0] && rad <= reff[19])) continue;
        int ieff = 0;
        for (int b = 0; b < 19; ++b)
          if (rad >= reff[b] && rad <= reff[b + 1]) ieff = b + 1;
        cls.push_back(ic);
        q.push_back(kQeff[ieff]);
        r.push_back(x->h_rhop[ic] * reff[ieff]);
      }
      break;
    }
    case F3D_OUT_CON:
      if (index < 0 || index > nc) return f3d::ctx_error(F3D_ERR_ARG, "class index outside 0..nc");
      if (index == 0)
        cls = particle_classes(x);
      else
        cls.push_back(index - 1);
      n = d.cells();
      break;
    case F3D_OUT_WIND:
      if (index != 1 && index != 2) return f3d::ctx_error(F3D_ERR_ARG, "wind component must be 1 (u) or 2 (v)");
      n = d.cells();
      break;
    case F3D_OUT_MAGGR:
      if (!x->agr_on) return f3d::ctx_error(F3D_ERR_STATE, "aggregation is off");
      n = d.cells();
      break;
    default:
      return f3d::ctx_error(F3D_ERR_ARG, "unknown output variable");
  }
  cudaStream_t s = x->stream;
  Scratch sc;
  sc.s = s;
  const size_t tab = 3 * sizeof(double) * (cls.size() + 1);
  OK(cudaMallocAsync(&sc.p, sizeof(double) * n + sizeof(float) * n + tab + 64, s));
  double* res = reinterpret_cast<double*>(sc.p);
  unsigned char* t = reinterpret_cast<unsigned char*>(sc.p) + ((sizeof(double) * n + sizeof(float) * n + 15) & ~size_t(15));
  int* dcls = reinterpret_cast<int*>(t);
  double* dq = reinterpret_cast<double*>(t + sizeof(double) * (cls.size() + 1));
  double* dr = dq + cls.size() + 1;
  if (!cls.empty()) OK(cudaMemcpyAsync(dcls, cls.data(), sizeof(int) * cls.size(), cudaMemcpyHostToDevice, s));
  if (!q.empty()) {
    OK(cudaMemcpyAsync(dq, q.data(), sizeof(double) * q.size(), cudaMemcpyHostToDevice, s));
    OK(cudaMemcpyAsync(dr, r.data(), sizeof(double) * r.size(), cudaMemcpyHostToDevice, s));
  }
  const int ncls = (int)cls.size();
  const bool f32 = x->prec == F3D_PREC_FP32;
  switch (var) {
    case F3D_OUT_LOAD:
    case F3D_OUT_WET:
    case F3D_OUT_THICK:
      launch_getc0(x->cdry, x->cwet, x->cload, d, nc, np, s);
      if (var == F3D_OUT_THICK)
        k_out_thick<<<blocks(pl), OB, 0, s>>>(x->cload, pl, np, x->rhop, x->Hm1, res);
      else
        k_out_plane<<<blocks(pl), OB, 0, s>>>((var == F3D_OUT_LOAD ? x->cload : x->cwet) + index * pl, pl,
                                              x->Hm1, res);
      break;
    case F3D_OUT_COL_MASS:
    case F3D_OUT_PM_COL:
      if (f32)
        k_out_column<float><<<blocks(pl), OB, 0, s>>>(x->c32, d, dcls, ncls, x->dz, x->Hm1, res);
      else
        k_out_column<double><<<blocks(pl), OB, 0, s>>>(x->c64, d, dcls, ncls, x->dz, x->Hm1, res);
      break;
    case F3D_OUT_C_GRND:
    case F3D_OUT_PM_GRND:
      if (f32)
        k_out_ground<float><<<blocks(pl), OB, 0, s>>>(x->c32, d, dcls, ncls, x->Hm1, res);
      else
        k_out_ground<double><<<blocks(pl), OB, 0, s>>>(x->c64, d, dcls, ncls, x->Hm1, res);
      break;
    case F3D_OUT_AOT05:
      if (f32)
        k_out_aot<float><<<blocks(pl), OB, 0, s>>>(x->c32, d, dcls, dq, dr, ncls, x->dz, x->Hm1, res);
      else
        k_out_aot<double><<<blocks(pl), OB, 0, s>>>(x->c64, d, dcls, dq, dr, ncls, x->dz, x->Hm1, res);
      break;
    case F3D_OUT_WIND:
    case F3D_OUT_MAGGR:
      k_out_field<<<blocks(pl), OB, 0, s>>>(var == F3D_OUT_MAGGR ? x->agr_maggr : (index == 1 ? x->vx : x->vy),
                                            var == F3D_OUT_WIND, d, x->Hm1, x->zlayer, x->topg, asl, res);
      break;
    case F3D_OUT_CON:
      if (f32)
        k_out_con<float><<<blocks(pl), OB, 0, s>>>(x->c32, d, dcls, ncls, x->Hm1, x->zlayer, x->topg, asl,
                                                   res);
      else
        k_out_con<double><<<blocks(pl), OB, 0, s>>>(x->c64, d, dcls, ncls, x->Hm1, x->zlayer, x->topg,
                                                    asl, res);
      break;
  }
  count_launch();
  return finish(x, res, n, dst, dst_type, sc);
}

int f3d_track_points(f3d_ctx* x, int npts, const double* xpts, const double* ypts, double xo, double yo,
                     double* out) {
  if (!x || (npts > 0 && (!xpts || !ypts || !out))) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  if (npts <= 0) return F3D_OK;
  const Dims d = x->d;
  const int np = x->g.np, nz = d.nz;
  // get_pts_st (Sources/reaout.f90:180-224): the cell and (s,t) of each point
  std::vector<int> ip(npts), jp(npts);
  std::vector<double> sp(npts), tp(npts);
  const double dxo = x->g.dx, dyo = x->g.dy;
  for (int n = 0; n < npts; ++n) {
    bool found = false;
    for (int ix = 1; ix <= d.nx - 1; ++ix) {
      const double xx = xo + (ix - 1) * dxo;
      if (xpts[n] >= xx && xpts[n] <= xx + dxo) {
        ip[n] = ix;
        sp[n] = (xpts[n] - xx) / dxo;
        sp[n] = 2.0 * sp[n] - 1.0;
        found = true;
      }
    }
    if (!found) return f3d::ctx_error(F3D_ERR_RANGE, "get_pts_st: value not found");
    found = false;
    for (int iy = 1; iy <= d.ny - 1; ++iy) {
      const double yy = yo + (iy - 1) * dyo;
      if (ypts[n] >= yy && ypts[n] <= yy + dyo) {
        jp[n] = iy;
        tp[n] = (ypts[n] - yy) / dyo;
        tp[n] = 2.0 * tp[n] - 1.0;
        found = true;
      }
    }
    if (!found) return f3d::ctx_error(F3D_ERR_RANGE, "get_pts_st: value not found");
  }
  std::vector<TrackClass> cls(np > 0 ? np : 1);
  double reff[20];
  for (int b = 0; b < 20; ++b) reff[b] = kReffUm[b] * 1e-6;
  for (int ic = 0; ic < np; ++ic) {
    TrackClass& k = cls[ic];
    k.diam = x->h_diam[ic];
    k.rhop = x->h_rhop[ic];
    k.aer = 0;
    k.q = k.r = 0.0;
    const double rad = (double)0.5f * k.diam;
    if (rad >= reff[0] && rad <= reff[19]) {
      int ieff = 0;
      for (int b = 0; b < 19; ++b)
        if (rad >= reff[b] && rad <= reff[b + 1]) ieff = b + 1;
      k.aer = 1;
      k.q = kQeff[ieff];
      k.r = reff[ieff];
    }
  }
  const int stride = 7 + 3 * nz + 1 + np;
  cudaStream_t s = x->stream;
  Scratch sc;
  sc.s = s;
  const size_t bo = sizeof(double) * (size_t)npts * stride;
  const size_t bi = (sizeof(int) * 2 + sizeof(double) * 2) * (size_t)npts;
  OK(cudaMallocAsync(&sc.p, bo + bi + sizeof(TrackClass) * cls.size() + 256, s));
  unsigned char* b = reinterpret_cast<unsigned char*>(sc.p);
  double* res = reinterpret_cast<double*>(b);
  double* dsp = reinterpret_cast<double*>(b + bo);
  double* dtp = dsp + npts;
  int* dip = reinterpret_cast<int*>(dtp + npts);
  int* djp = dip + npts;
  TrackClass* dcls = reinterpret_cast<TrackClass*>(b + ((bo + bi + 15) & ~size_t(15)));
  OK(cudaMemcpyAsync(dsp, sp.data(), sizeof(double) * npts, cudaMemcpyHostToDevice, s));
  OK(cudaMemcpyAsync(dtp, tp.data(), sizeof(double) * npts, cudaMemcpyHostToDevice, s));
  OK(cudaMemcpyAsync(dip, ip.data(), sizeof(int) * npts, cudaMemcpyHostToDevice, s));
  OK(cudaMemcpyAsync(djp, jp.data(), sizeof(int) * npts, cudaMemcpyHostToDevice, s));
  OK(cudaMemcpyAsync(dcls, cls.data(), sizeof(TrackClass) * cls.size(), cudaMemcpyHostToDevice, s));
  launch_getc0(x->cdry, x->cwet, x->cload, d, x->g.nc, np, s);
  const unsigned nb = (unsigned)((npts + 63) / 64);
  if (x->prec == F3D_PREC_FP32)
    k_track<float><<<nb, 64, 0, s>>>(x->c32, x->cload, d, np, dip, djp, dsp, dtp, npts, dcls, x->dz, x->Hm1, res);
  else
    k_track<double><<<nb, 64, 0, s>>>(x->c64, x->cload, d, np, dip, djp, dsp, dtp, npts, dcls, x->dz, x->Hm1, res);
  count_launch();
  OK(cudaMemcpyAsync(out, res, bo, cudaMemcpyDefault, s));
  OK(cudaGetLastError());
  OK(cudaStreamSynchronize(s));
  return F3D_OK;
}

int f3d_output_fl(f3d_ctx* x, double flight_level, const double* p, void* dst, int dst_type) {
  if (!x || !p || !dst) return f3d::ctx_error(F3D_ERR_ARG, "NULL argument");
  if (dst_type != F3D_OUT_BINARY64 && dst_type != F3D_OUT_BINARY32)
    return f3d::ctx_error(F3D_ERR_ARG, "dst_type must be F3D_OUT_BINARY64 or F3D_OUT_BINARY32");
  const Dims d = x->d;
  const long long pl = d.plane(), s3 = d.cells();
  const double pnom = standard_pressure(flight_level * 30.48);  // printres_nc.f90:559
  const std::vector<int> cls = particle_classes(x);
  cudaStream_t s = x->stream;
  Scratch sc;
  sc.s = s;
  const size_t head = (sizeof(double) * pl + sizeof(float) * pl + 15) & ~size_t(15);
  OK(cudaMallocAsync(&sc.p, head + sizeof(double) * s3 + sizeof(int) * (cls.size() + 1) + 64, s));
  double* res = reinterpret_cast<double*>(sc.p);
  double* dp = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(sc.p) + head);
  int* dcls = reinterpret_cast<int*>(dp + s3);
  OK(cudaMemcpyAsync(dp, p, sizeof(double) * s3, cudaMemcpyDefault, s));
  if (!cls.empty()) OK(cudaMemcpyAsync(dcls, cls.data(), sizeof(int) * cls.size(), cudaMemcpyHostToDevice, s));
  if (x->prec == F3D_PREC_FP32)
    k_out_fl<float><<<blocks(pl), OB, 0, s>>>(x->c32, d, dcls, (int)cls.size(), dp, pnom, x->Hm1, res);
  else
    k_out_fl<double><<<blocks(pl), OB, 0, s>>>(x->c64, d, dcls, (int)cls.size(), dp, pnom, x->Hm1, res);
  count_launch();
  return finish(x, res, pl, dst, dst_type, sc);
}

}  // extern "C"

// f3d_gravity.cu -- the gravity current of the umbrella cloud (Costa and
// Macedonio; GRAVITY_CURRENT = YES, Sources/readat.f90:150-213):
//
//  * addradialwind (Sources/addradialwind.f90), called by meteo.f90:140
//    after the scaling and corvver and before setdivu/finddt: a radial wind
//    of the spreading front is added to vx (scaled) and vy between the
//    levels nearest hmin and hmax, outside a minimum radius of 1.5 cell
//    diagonals and inside the passive-transport radius;
//  * divcorr (Sources/divcorr.f90), called by endstep.f90:71 at the
//    mass-budget log steps after writim: c is rescaled by the relative
//    mass-balance error (clamped to +-0.05) where |divu*dt| >= 0.005.
//
// The scalar set-up of addradialwind is evaluated on the host in binary64
// with the host C library (it reads two wind values back from the device);
// the per-column and per-cell updates run on the device (--fmad=false).
#include <cmath>
#include <cstring>

#include "f3d_ctx_impl.h"

namespace f3d {
namespace {

// addradialwind.f90:150-166, one thread per column (i, j)
__global__ void k_addradialwind(Dims d, double dX1, double dX2, double dx, double dy, double xorigr,
                                double yorigr, double cx, double cy, double min_radius,
                                double max_radius, double c_grav_factor, double radius_grav,
                                int kmin, int kmax, const double* Hm1, double* vx, double* vy) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long pl = d.plane();
  if (p >= pl) return;
  const int i = (int)(p % d.nx) + 1, j = (int)(p / d.nx) + 1;
  const double h = Hm1[p];
  const double deltax = dX1 * h * ((xorigr + (double)i * dx) - cx) / dx;
  const double deltay = dX2 * ((yorigr + (double)j * dy) - cy) / dy;
  const double radius = sqrt(deltax * deltax + deltay * deltay);
  if (fabs(radius) <= min_radius) return;
  if (fabs(radius) > max_radius) return;
  const double rvel = c_grav_factor / radius * (1.0 + radius * radius / (3.0 * (radius_grav * radius_grav)));
  for (int k = kmin; k <= kmax; ++k) {
    const long long m = p + (long long)(k - 1) * pl;
    vx[m] = vx[m] + rvel * deltax / radius / h;
    vy[m] = vy[m] + rvel * deltay / radius;
  }
}

// divcorr.f90:28-38 over all classes
template <class T>
__global__ void k_divcorr(T* c, long long hb, Dims d, int nc, const double* divu, double dt,
                          double corrdiv) {
  const long long s3 = d.cells();
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < s3;
       m += (long long)gridDim.x * blockDim.x) {
    const double dive = divu[m];
    if (!(fabs(dive * dt) >= 0.005)) continue;
    const int i = (int)(m % d.nx) + 1, j = (int)((m / d.nx) % d.ny) + 1, k = (int)(m / d.plane()) + 1;
    const long long q = d.C(i, j, k);
    for (int ic = 0; ic < nc; ++ic) {
      T& v = c[(long long)ic * hb + q];
      v = (T)((double)v * (1.0 + corrdiv));
    }
  }
}

// gfortran MAX/MIN of two reals: the first operand unless the second
// compares greater (smaller) or the first is a NaN.
double fmaxg(double a, double b) { return (b > a || std::isnan(a)) ? b : a; }
double fming(double a, double b) { return (b < a || std::isnan(a)) ? b : a; }

// the level whose height is nearest to h (the last one on ties), from `first`
int nearest_level(const std::vector<double>& zl, double h, int first) {
  int kk = first;
  double store = zl.back();
  for (int k = 1; k <= (int)zl.size(); ++k) {
    const double dist = std::fabs(zl[k - 1] - h);
    if (dist <= store) {
      kk = k;
      store = dist;
    }
  }
  return kk;
}

}  // namespace

// addradialwind.f90:46-166 for the context's current sources and winds.
int gc_addradialwind(f3d_ctx* x) {
  const f3d_gravity_current& gc = x->gc;
  const f3d_grid& g = x->g;
  const Dims d = x->d;
  const double pi = 3.14159265358979323846;  // Numeric.f90 pi
  const double min_radius = (double)1.5f * std::sqrt(x->hm11 * g.dX1 * x->hm11 * g.dX1 + g.dX2 * g.dX2);
  const double time_eruption = x->time - gc.beg_time;
  const double mass_flow_rate = x->mfr_scaled;  // sum(tmrat(1:nsou,1:nc)), scaled rates
  if (mass_flow_rate <= (double)0.1f) return F3D_OK;
  const double vol_flow_rate = gc.c_flow_rate * std::sqrt(gc.k_entrain) * std::pow(mass_flow_rate, 0.75) /
                               std::pow(gc.brunt_vaisala, 0.625);
  const double c_gravr = 3.0 * gc.lambda_grav * gc.brunt_vaisala * vol_flow_rate / (2.0 * pi);
  double radius_grav = std::pow(c_gravr * (time_eruption * time_eruption), 0.33333);
  radius_grav = fmaxg(radius_grav, min_radius);
  const double c_gravu = std::sqrt(2.0 * gc.lambda_grav * gc.brunt_vaisala * vol_flow_rate / (3.0 * pi));
  const double c_grav_factor = 0.75 * c_gravu * std::sqrt(radius_grav);
  const double th_grav = c_gravu / (std::sqrt(radius_grav) * gc.lambda_grav * gc.brunt_vaisala);
  const double h_tot = gc.h_tot;
  const double h_umbr = h_tot / 1.32;
  const double hmin = fmaxg(h_umbr - 0.5 * th_grav, 0.5 * h_tot);
  const double hmax = fming(h_umbr + 0.5 * th_grav, h_tot);
  int i_wind = (int)((gc.center_x - gc.xorigr) / g.dx);
  int j_wind = (int)((gc.center_y - gc.yorigr) / g.dy);
  i_wind = i_wind > 1 ? i_wind : 1;
  j_wind = j_wind > 1 ? j_wind : 1;
  if (i_wind > d.nx || j_wind > d.ny)
    return ctx_error(F3D_ERR_RANGE, "gravity current centre outside the grid");
  const int k_wind = nearest_level(x->h_zlayer, h_umbr, 1);
  // wind at the NBL above the crater (scaled vx, as the reference reads it)
  double w[2];
  const long long m = (long long)(i_wind - 1) + (long long)d.nx * (j_wind - 1) + d.plane() * (k_wind - 1);
  if (cudaMemcpyAsync(&w[0], x->vx + m, sizeof(double), cudaMemcpyDeviceToHost, x->stream) != cudaSuccess ||
      cudaMemcpyAsync(&w[1], x->vy + m, sizeof(double), cudaMemcpyDeviceToHost, x->stream) != cudaSuccess ||
      cudaStreamSynchronize(x->stream) != cudaSuccess)
    return ctx_error(F3D_ERR_CUDA, "gravity current: wind read-back failed");
  const double v_wind = std::sqrt(w[0] * w[0] + w[1] * w[1]);
  const double max_radius = 1.7777 * c_gravr / fmaxg(v_wind * v_wind, 0.1);
  const int kmin = nearest_level(x->h_zlayer, hmin, 1);
  const int kmax = nearest_level(x->h_zlayer, hmax, d.nz);
  k_addradialwind<<<(unsigned)((d.plane() + 127) / 128), 128, 0, x->stream>>>(
      d, g.dX1, g.dX2, g.dx, g.dy, gc.xorigr, gc.yorigr, gc.center_x, gc.center_y, min_radius, max_radius,
      c_grav_factor, radius_grav, kmin, kmax, x->Hm1, x->vx, x->vy);
  count_launch();
  return cudaGetLastError() == cudaSuccess ? F3D_OK : ctx_error(F3D_ERR_CUDA, "addradialwind launch failed");
}

// divcorr.f90:21-38 with the budget of the log step
int gc_divcorr(f3d_ctx* x, double massvol, double massdep, double outmass) {
  const double compmass = massvol + massdep + outmass;
  const double eps = 0.005, eps1 = 10.0 * eps;
  const double corrdiv = fmaxg(fming((x->erumass - compmass) / x->erumass, eps1), -eps1);
  const Dims d = x->d;
  const unsigned nb = (unsigned)std::min<long long>((d.cells() + 255) / 256, 152LL * 16);
  (void)eps;
  if (x->prec == F3D_PREC_FP32)
    k_divcorr<float><<<nb, 256, 0, x->stream>>>(x->c32, d.halo(), d, x->g.nc, x->divu, x->dt, corrdiv);
  else
    k_divcorr<double><<<nb, 256, 0, x->stream>>>(x->c64, d.halo(), d, x->g.nc, x->divu, x->dt, corrdiv);
  count_launch();
  return cudaGetLastError() == cudaSuccess ? F3D_OK : ctx_error(F3D_ERR_CUDA, "divcorr launch failed");
}

}  // namespace f3d

extern "C" int f3d_set_gravity_current(f3d_ctx* x, const f3d_gravity_current* gc) {
  if (!x) return f3d::ctx_error(F3D_ERR_ARG, "NULL context");
  f3d::ctx_prefetch_drop(x);  // a look-ahead meteo update does not add the radial wind
  if (!gc) {
    x->gc_on = 0;
    return F3D_OK;
  }
  if (!(gc->brunt_vaisala > 0.0) || !(gc->lambda_grav > 0.0) || !(x->g.dx > 0.0) || !(x->g.dy > 0.0))
    return f3d::ctx_error(F3D_ERR_ARG, "gravity current: brunt_vaisala, lambda_grav, dx, dy must be > 0");
  x->gc = *gc;
  x->gc_on = 1;
  return F3D_OK;
}

// f3d_coeff.cu -- the per-meteo-update coefficient chain of
// Sources/meteo.f90:19-149 on the device (binary64, --fmad=false).
//
// Transcendentals (pow, log, log10, exp, atan, acos, tan) are CUDA's; the
// reference uses the host libm, so these fields agree to a few ulp, not
// bitwise.  Everything else is rounded operation by operation as written.
//
// setvset: vsettl keeps its drag coefficient cd between calls
// (Sources/setvset.f90:89, SAVE), so the reference evaluates one sequential
// chain over (ic, i, j, k) with k fastest, continued across meteo updates.
// The chain is split into segments; each segment starts from a guess after a
// warm-up over the cells that precede it, and is accepted only if its entry
// cd equals, bit for bit, the exit cd of the previous segment (from then on
// the computation is identical to the sequential one).  The iteration
// contracts, so the warm-up reaches the exact chain value within a few to a
// few tens of cells; any segment that fails the check is recomputed in order
// from the verified exit of its predecessor.
//
// The drag iteration is binary64-pipe bound on GB300, so its Ganser form is
// restated with one division, one reciprocal square root and a table-driven
// log/exp per iteration (f3d_dmath.cuh) in place of the reference's four
// divisions, square root and pow: the same iteration and stopping test on
// values that differ from the reference's by a few ulp.
#include <algorithm>

#include "f3d_dmath.cuh"
#include "f3d_internal.h"

namespace f3d {

// ------------------------------------------------------------- kappa3
// Sources/kappa3.f90:50-236, one thread per cell.
__device__ void k3_similarity_grad(Dims d, int i, int j, int k, const double* dz,
                                   const double* vx, const double* vy, const double* vptemp,
                                   double& dvdz2, double& rich) {
  const double gi = 9.81;
  const double dzs = dz[k] + dz[k - 1];
  const double gx = (vx[d.M(i, j, k + 1)] - vx[d.M(i, j, k - 1)]) / dzs;
  const double gy = (vy[d.M(i, j, k + 1)] - vy[d.M(i, j, k - 1)]) / dzs;
  dvdz2 = gx * gx + gy * gy;
  dvdz2 = fmax2(dvdz2, 1e-10);
  rich = gi * ((vptemp[d.M(i, j, k + 1)] - vptemp[d.M(i, j, k - 1)]) / (dz[k] + dz[k - 1])) /
         (vptemp[d.M(i, j, k)] * dvdz2);
}

__global__ void k_kappa3(Dims d, int modkv, int modkh, int coord_sys, double rkv0, double rkh0,
                         double Csh, double dX1, double dX2, double dx, double dy,
                         const double* dz, const double* zlayer, const double* Hm1,
                         const double* vx, const double* vy, const double* vptemp,
                         const double* ustar, const double* zi, const double* rl,
                         double* rkver, double* rkhor) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long s3 = d.cells();
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= s3) return;
  const int i = (int)(m % nx) + 1;
  const int j = (int)((m / nx) % ny) + 1;
  const int k = (int)(m / ((long long)nx * ny)) + 1;
  const long long p = d.P(i, j);
  const double vkarm = 0.4, beta1 = 9.2, beta2 = 13.0, rlamb = 30.0, rkhmin = 1e2, rkvmin = 1.0;
  const double hinf = 5.0, hsup = 5e3, alfa = 0.28, Khf = 8000.0;
  // vertical
  if (modkv == 0) {
    rkver[m] = rkv0;
  } else if (modkv == 1) {
    if (k >= 2) {
      double dvdz2, rich;
      // at k = nz the reference reuses the values of the last point computed
      // at k = nz-1, i.e. (nx, ny, nz-1) (kappa3.f90:64-71)
      if (k < nz)
        k3_similarity_grad(d, i, j, k, dz, vx, vy, vptemp, dvdz2, rich);
      else
        k3_similarity_grad(d, nx, ny, nz - 1, dz, vx, vy, vptemp, dvdz2, rich);
      const double h = fmin2(fmax2(zi[p], hinf), hsup);
      const double zl = zlayer[k - 1];
      const double zeta = zl / h;
      double kv;
      if (zeta < 1.0) {
        if (rl[p] >= 0.0)
          kv = vkarm * ustar[p] * zl * (1.0 - zeta) / (1.0 + beta1 * zl * rl[p]);
        else
          kv = vkarm * ustar[p] * zl * (1.0 - zeta) * sqrt(1.0 - beta2 * zl * rl[p]);
      } else {
        const double lc = 1.0 / ((1.0 / (vkarm * zl)) + (1.0 / rlamb));
        if (rich >= 0.0) {
          kv = lc * lc * sqrt(dvdz2) / (1.0 + 10.0 * rich * (1.0 + 8.0 * rich));
          kv = fmax2(kv, rkvmin);
        } else {
          kv = lc * lc * sqrt(dvdz2) * sqrt(1.0 - 18.0 * rich);
          kv = fmax2(kv, rkvmin);
        }
      }
      rkver[m] = kv;
    }
  } else if (modkv == 2) {
    const double gh = 11.6, betah = 7.8, prt = 0.95;
    const double zl = zlayer[k - 1], us = ustar[p];
    double zeta = zl * rl[p];
    double kv;
    if (zeta < 0.0)
      kv = vkarm * us * zl * sqrt(1.0 - gh * zeta) / prt;
    else if (zeta > 0.0)
      kv = vkarm * us * zl / (prt + betah * zeta);
    else
      kv = vkarm * us * zl / prt;
    const double h = fmin2(fmax2(zi[p], hinf), hsup);
    zeta = zl / h;
    if (zeta > 1.0) zeta = 1.0;
    rkver[m] = kv * (1.0 - zeta);
  }
  // horizontal
  if (modkh == 0) {
    rkhor[m] = rkh0;
  } else if (modkh == 1 || modkh == 2) {
    const double dXX = Hm1[p] * dX1;
    double dvxdx, dvydx, dvxdy, dvydy;
    if (i == 1) {
      dvxdx = (vx[d.M(2, j, k)] - vx[d.M(1, j, k)]) / dXX;
      dvydx = (vy[d.M(2, j, k)] - vy[d.M(1, j, k)]) / dXX;
    } else if (i == nx) {
      dvxdx = (vx[d.M(nx, j, k)] - vx[d.M(nx - 1, j, k)]) / dXX;
      dvydx = (vy[d.M(nx, j, k)] - vy[d.M(nx - 1, j, k)]) / dXX;
    } else {
      dvxdx = (vx[d.M(i + 1, j, k)] - vx[d.M(i - 1, j, k)]) / (2.0 * dXX);
      dvydx = (vy[d.M(i + 1, j, k)] - vy[d.M(i - 1, j, k)]) / (2.0 * dXX);
    }
    if (j == 1) {
      dvxdy = (vx[d.M(i, 2, k)] - vx[d.M(i, 1, k)]) / dX2;
      dvydy = (vy[d.M(i, 2, k)] - vy[d.M(i, 1, k)]) / dX2;
    } else if (j == ny) {
      dvxdy = (vx[d.M(i, ny, k)] - vx[d.M(i, ny - 1, k)]) / dX2;
      dvydy = (vy[d.M(i, ny, k)] - vy[d.M(i, ny - 1, k)]) / dX2;
    } else {
      dvxdy = (vx[d.M(i, j + 1, k)] - vx[d.M(i, j - 1, k)]) / (2.0 * dX2);
      dvydy = (vy[d.M(i, j + 1, k)] - vy[d.M(i, j - 1, k)]) / (2.0 * dX2);
    }
    double kh;
    if (modkh == 1) {
      const double Kmh = 0.075 * pow(dXX * dX2, 2.0 / 3.0);
      const double s1 = dvxdy + dvydx;
      kh = Csh * Csh * dXX * dX2 * sqrt(s1 * s1 + 2.0 * (dvxdx * dvxdx + dvydy * dvydy));
      kh = 1.0 * fmax2(kh, Kmh);
      kh = fmax2(kh, rkhmin);
    } else {
      const double Khn0 = (coord_sys == 0) ? 3.6e-2 : 4000.0;
      const double s1 = dvxdx - dvydy, s2 = dvydx + dvxdy;
      const double Kht = alfa * alfa * dXX * dX2 * sqrt(s1 * s1 + s2 * s2);
      const double Khn = Khf * (Khn0 / Hm1[p] / dx) * (Khn0 / dy);
      kh = (1.0 / Kht) + (1.0 / Khn);
      kh = fmax2(1.0 / kh, rkhmin);
    }
    rkhor[m] = kh;
  }
}

void launch_kappa3(Dims d, int modkv, int modkh, int coord_sys, double rkv0, double rkh0,
                   double Csh, double dX1, double dX2, double dx, double dy, const double* dz,
                   const double* zlayer, const double* Hm1, const double* vx, const double* vy,
                   const double* vptemp, const double* ustar, const double* zi, const double* rl,
                   double* rkver, double* rkhor, cudaStream_t s) {
  const long long n = d.cells();
  k_kappa3<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(d, modkv, modkh, coord_sys, rkv0, rkh0, Csh,
                                                      dX1, dX2, dx, dy, dz, zlayer, Hm1, vx, vy,
                                                      vptemp, ustar, zi, rl, rkver, rkhor);
  count_launch();
}

// --------------------------------------------------------- setvdrydep
// Sources/setvdrydep.f90:74-264; the Feng (2008) coefficient tables of
// setvdrydep.f90:79-129 indexed [land use - 1][mode - 1].
__constant__ double c_feng_a[6][4] = {
    {0.0048, 0.0315, 1.2891, 1.0338}, {0.0037, 0.0120, 1.3977, 1.0707},
    {0.0042, 0.2928, 1.3970, 0.9155}, {0.0032, 0.1201, 1.1838, 1.0096},
    {0.0043, 0.1337, 1.2834, 1.1595}, {0.0045, 0.0925, 1.2654, 1.0891}};
__constant__ double c_feng_b[6][4] = {
    {1.0, 2.7925, 2.6878, 1.2644}, {1.0, 2.2413, 2.5838, 1.3247}, {1.0, 3.8581, 2.5580, 1.0364},
    {1.0, 3.4407, 2.8033, 1.2069}, {1.0, 3.5456, 2.7157, 1.4863}, {1.0, 3.2920, 2.7227, 1.4240}};
// USGS 24-category land use -> Feng land class (setvdrydep.f90:165-215).
__constant__ int c_usgs_feng[25] = {6, 1, 6, 6, 6, 6, 6, 6, 6, 6, 3, 6, 6, 6,
                                    6, 6, 5, 6, 6, 3, 2, 2, 2, 2, 4};

__device__ __forceinline__ int drydep_mode(double dm) {
  if (dm > 100e-6) return 0;
  if (dm > 10e-6) return 4;
  if (dm > 2.5e-6) return 3;
  if (dm > 0.1e-6) return 2;
  return 1;
}

__global__ void k_setvdrydep(Dims d, int nc, const double* diam, const double* zlayer,
                             const double* ldu, const double* rl, const double* znt,
                             const double* ustar, const double* tempe, const double* rho,
                             double* vdep) {
  const long long pl = d.plane();
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= pl) return;
  bool have_to_work = false;
  for (int ic = 0; ic < nc; ++ic) have_to_work |= drydep_mode(diam[ic]) > 0;
  if (!have_to_work) return;
  const double vkarm = 0.4, visc0 = 1.827e-5, Tair0 = 291.15;
  const double lv = ldu[p];
  int iland = 6;
  if (lv > -1.0 && lv < 25.0) {
    const int code = (int)lv;
    if (code >= 1 && code <= 24) iland = c_usgs_feng[code];
  }
  const double zeta = rl[p] * zlayer[0];
  const double zeta0 = rl[p] * znt[p];
  double ra;
  if (ustar[p] > 0.0) {
    ra = log(zlayer[0] / znt[p]);
    if (zeta > 0) {
      ra = ra + 4.7 * (zeta - zeta0);
    } else if (zeta < 0) {
      const double eta = pow(1.0 - 15.0 * zeta, 0.25);
      const double eta0 = pow(1.0 - 15.0 * zeta0, 0.25);
      ra = ra + log((eta0 * eta0 + 1) * ((eta0 + 1) * (eta0 + 1)) /
                    ((eta * eta + 1) * ((eta + 1) * (eta + 1))));
      ra = ra + 2 * (atan(eta) - atan(eta0));
    }
    ra = ra / (ustar[p] * vkarm);
  } else {
    ra = 1e20;
  }
  const double T = tempe[p];
  const double visc = visc0 * ((Tair0 + 120.0) / (T + 120.0)) * pow(T / Tair0, 1.5);
  double Re = ustar[p] * znt[p] * rho[p] / visc;
  if (Re > 40300.0) Re = 40300.0;
  double Vd1 = -0.5 * ((Re - 40300.0) / 15330.0) * ((Re - 40300.0) / 15330.0);
  Vd1 = 0.0226 * ustar[p] * exp(Vd1);
  for (int ic = 0; ic < nc; ++ic) {
    const int mode = drydep_mode(diam[ic]);
    if (mode > 0) {
      double Vd = Vd1 + c_feng_a[iland - 1][mode - 1] * pow(ustar[p], c_feng_b[iland - 1][mode - 1]);
      Vd = ra + 1.0 / Vd;
      vdep[(long long)ic * pl + p] = -1.0 / Vd;
    }
  }
}

void launch_setvdrydep(Dims d, int nc, const double* diam, const double* zlayer,
                       const double* ldu, const double* rl, const double* znt,
                       const double* ustar, const double* tempe, const double* rho,
                       double* vdep, cudaStream_t s) {
  const long long pl = d.plane();
  k_setvdrydep<<<(unsigned)((pl + 127) / 128), 128, 0, s>>>(d, nc, diam, zlayer, ldu, rl, znt, ustar,
                                                           tempe, rho, vdep);
  count_launch();
}

// ------------------------------------------ scaling, corvver, setdivu
// Sources/meteo.f90:108-112 (scaling), Sources/corvver.f90:21-34,
// Sources/setdivu.f90:16-30.
__global__ void k_scale_corvver(Dims d, int coord_sys, double dX1, double dX2, const double* Hm1,
                                const double* topg, double* vx, const double* vy, double* vz,
                                double* rho, const double* rkhor, double* rkh1) {
  const int nx = d.nx, ny = d.ny;
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= d.cells()) return;
  const int ix = (int)(m % nx) + 1;
  const int iy = (int)((m / nx) % ny) + 1;
  const long long p = d.P(ix, iy);
  const double h = Hm1[p];
  const double vxs = vx[m] / h;
  vx[m] = vxs;
  rho[m] = rho[m] * h;
  rkh1[m] = rkhor[m] / (h * h);
  if (coord_sys == 0) {
    const double dyinv = 1.0 / dX2;
    const double dxinv = 1.0 / (h * dX1);
    const double zx = dxinv * (topg[d.P(ix + 1 <= nx ? ix + 1 : nx, iy)] - topg[p]);
    const double zy = dyinv * (topg[d.P(ix, iy + 1 <= ny ? iy + 1 : ny)] - topg[p]);
    const double vs = zx * vxs + zy * vy[m];
    vz[m] = vz[m] - vs;
  }
}

__global__ void k_setdivu(Dims d, double dX1, double dX2, const double* dz, const double* Hm1,
                          const double* vx, const double* vy, const double* vz, double* divu) {
  const int nx = d.nx, ny = d.ny;
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= d.cells()) return;
  const int i = (int)(m % nx) + 1;
  const int j = (int)((m / nx) % ny) + 1;
  const int k = (int)(m / ((long long)nx * ny)) + 1;
  const double vi = vx[m], vi_1 = vx[d.M(i > 1 ? i - 1 : 1, j, k)];
  const double vj = vy[m], vj_1 = vy[d.M(i, j > 1 ? j - 1 : 1, k)];
  const double vk = vz[m], vk_1 = vz[d.M(i, j, k > 1 ? k - 1 : 1)];
  divu[m] = (vi - vi_1) / (Hm1[d.P(i, j)] * dX1) + (vj - vj_1) / dX2 + (vk - vk_1) / dz[k];
}

void launch_meteo_scale(Dims d, int coord_sys, double dX1, double dX2, const double* dz,
                        const double* Hm1, const double* topg, double* vx, double* vy,
                        double* vz, double* rho, const double* rkhor, double* rkh1,
                        double* divu, cudaStream_t s) {
  const long long n = d.cells();
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_scale_corvver<<<nb, 256, 0, s>>>(d, coord_sys, dX1, dX2, Hm1, topg, vx, vy, vz, rho, rkhor, rkh1);
  count_launch();
  if (divu) {
    k_setdivu<<<nb, 256, 0, s>>>(d, dX1, dX2, dz, Hm1, vx, vy, vz, divu);
    count_launch();
  }
}

void launch_setdivu(Dims d, double dX1, double dX2, const double* dz, const double* Hm1,
                    const double* vx, const double* vy, const double* vz, double* divu,
                    cudaStream_t s) {
  const long long n = d.cells();
  k_setdivu<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, dX1, dX2, dz, Hm1, vx, vy, vz, divu);
  count_launch();
}

// reamet.f90:146 (PRATE mm/s -> mm/h when wet deposition is on) and
// reamet.f90:153 (vz(:,:,1) = 0).
__global__ void k_reamet_fix(Dims d, int wetdep, double* vz, double* prate) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= d.plane()) return;
  vz[p] = 0.0;
  if (wetdep) prate[p] = prate[p] * 3600.0;
}

void launch_reamet_fix(Dims d, int wetdep, double* vz, double* prate, cudaStream_t s) {
  k_reamet_fix<<<(unsigned)((d.plane() + 255) / 256), 256, 0, s>>>(d, wetdep, vz, prate);
  count_launch();
}

// ------------------------------------------------------------ setvset
struct ClassConst {
  double diam, rhop, psi;
  double num;       // 4*gi*diam*rhop, the numerator of setvset.f90:104
  double rk1, rk2;  // Ganser shape factors (setvset.f90:127-128)
  double rk12;      // rk1 * rk2
  double sqnum;     // sqrt(num)
  double drk12;     // diam * rk1 * rk2
  double cd100;     // Wilson
  int ok;           // get_gama converged
};

// Sources/setpsi.f90:65-127
__device__ int get_gama_dev(double diam, double sphe, double& gama) {
  const double d = diam * 1e3;
  const double toler = 1e-8;
  double gmin = 1e-3, gmax = 1.0;
  const double pi = 4.0 * atan(1.0);
  const double h = 0.5 * d;
  const double Vp = 4.0 * pi * (h * h * h) / 3.0;
  const double Ap = pow(pi, 1.0 / 3.0) * pow(6.0 * Vp, 2.0 / 3.0) / sphe;
  gama = 0.0;
  for (int it = 1; it <= 1000; ++it) {
    gama = 0.5 * (gmin + gmax);
    const double e = acos(gama);
    const double Ao = 0.5 * pi * d * d * pow(gama, -4.0 / 3.0) * (gama * gama + (e / tan(e)));
    if (Ao < Ap)
      gmax = gama;
    else
      gmin = gama;
    if ((it > 1) && (fabs(Ao - Ap) < toler)) return it;
  }
  return -1;
}

__global__ void k_class_consts(int np, int modv, const double* diam, const double* rhop,
                               const double* psi, const double* sphe, ClassConst* cc) {
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= np) return;
  const double gi = 9.81;
  ClassConst k;
  k.diam = diam[ic];
  k.rhop = rhop[ic];
  k.psi = psi[ic];
  k.num = 4.0 * gi * k.diam * k.rhop;
  k.rk1 = k.rk2 = k.rk12 = k.sqnum = k.drk12 = k.cd100 = 0.0;
  k.ok = 1;
  if (modv == 2) {
    double gama;
    if (get_gama_dev(k.diam, sphe[ic], gama) < 0) k.ok = 0;
    // gama**(-2.0/3.0): binary32 exponent (setvset.f90:120)
    const double dnd = 0.5 * (1.0 + gama) * pow(gama, (double)(-2.0f / 3.0f));
    k.rk1 = 1.0 / (dnd / 3.0 + 2.0 / (3.0 * sqrt(k.psi)));
    k.rk2 = pow(10.0, 1.8148 * pow(-log10(k.psi), 0.5743));
    k.rk12 = k.rk1 * k.rk2;
    k.sqnum = sqrt(k.num);
    k.drk12 = k.diam * k.rk12;
  } else if (modv == 3) {
    k.cd100 = 0.24 * pow(k.psi, -0.828) + 2.0 * sqrt(1.0 - k.psi);
  }
  cc[ic] = k;
}

// Sources/setvset.f90:65-181 for one call; returns iterations (0 for the
// closed-form Dellino model) or -1 when maxit is reached.
//
// Ganser (setvset.f90:117-136): with R = rey*rk1*rk2 = G*v,
// G = (rhoa/visc)*(diam*rk1*rk2), and v = T/sqrt(cd),
// T = sqrt(4*gi*diam*rhop)*sqrt(1/(3*rhoa)),
//   cd = 24/(rey*rk1)*(1 + 0.1118*R^0.6567) + 0.4305*rk2/(1 + 3305/R)
//      = rk2*((24*(R + 3305) + 0.4305*R^2)/(R*(R + 3305)) + 24*0.1118*R^(0.6567-1)).
// The cell factors sqrt(1/(3*rhoa)) and rhoa/visc come from k_visc
// (shared by all classes): cf.x, cf.y.
__device__ int vsettl_dev(const ClassConst& k, int model, double rhoa, double visc, double2 cf,
                          double& cd, double& vset, const DMathTab& tab) {
  const double eps = 1e-3;
  double vold = 1e5, v = 0.0;
  if (model == 2) {
    const double T = k.sqnum * cf.x;
    const double G = cf.y * k.drk12;
    for (int it = 1; it <= 100; ++it) {
      v = T * rsqrt(cd);
      const double R = G * v;
      const double L = dm_log(tab, R);
      const double P = dm_exp(tab, fma(0.6567, L, -L));  // R^0.6567 / R
      const double Q = R + 3305.0;
      const double N = fma(0.4305 * R, R, 24.0 * Q);
      cd = k.rk2 * fma(24.0 * 0.1118, P, N / (R * Q));
      // |v - vold| <= eps on the magnitude bits (the same order for
      // non-negative values; a NaN difference is above eps as in binary64)
      const long long dvb = __double_as_longlong(v - vold) & 0x7fffffffffffffffLL;
      if (it > 1 && dvb <= __double_as_longlong(eps)) {
        vset = T * rsqrt(cd);
        return it;
      }
      vold = v;
    }
    vset = v;
    return -1;
  }
  if (model == 4) {
    const double gi = 9.81, diam = k.diam;
    v = pow((diam * diam * diam * gi * (k.rhop - rhoa) * rhoa * pow(k.psi, 1.6)) / (visc * visc),
            0.5206);
    vset = (1.2065 * visc * v) / (diam * rhoa);
    return 0;
  }
  for (int it = 1; it <= 100; ++it) {
    v = sqrt(k.num / (3.0 * cd * rhoa));
    const double rey = rhoa * v * k.diam / visc;
    if (model == 1) {
      if (rey <= 988.947)
        cd = 24.0 / rey * (1.0 + 0.15 * pow(rey, 0.687));
      else
        cd = 0.44;
    } else {  // model 3
      if (rey <= 100.0) {
        cd = 24.0 / rey * pow(k.psi, -0.828) + 2.0 * sqrt(1.0 - k.psi);
      } else if (rey > 100.0 && rey < 1000.0) {
        const double a = (1.0 - k.cd100) / 900.0;
        const double b = 1.0 - 1000.0 * a;
        cd = a * rey + b;
      } else {
        cd = 1.0;
      }
    }
    if (it > 1 && fabs(v - vold) <= eps) {
      vset = sqrt(k.num / (3.0 * cd * rhoa));
      return it;
    }
    vold = v;
  }
  vset = v;
  return -1;
}

struct ChainGeom {
  Dims d;
  long long L;    // np * nx * ny * nz
  long long S;    // segment length
  long long W;    // warm-up length
  long long nseg;
};

// chain position q -> (ic, i, j, k) with k fastest (setvset.f90:25-33)
__device__ __forceinline__ void chain_cell(const ChainGeom& g, long long q, int& ic, long long& m) {
  const int nz = g.d.nz, ny = g.d.ny, nx = g.d.nx;
  const int k = (int)(q % nz) + 1;
  long long r = q / nz;
  const int j = (int)(r % ny) + 1;
  r /= ny;
  const int i = (int)(r % nx) + 1;
  ic = (int)(r / nx);
  m = g.d.M(i, j, k);
}

__device__ __forceinline__ double sutherland(double T) {
  const double visc0 = 1.827e-5;
  const double Tair0 = (double)291.15f;  // default-real literal (setvset.f90:23)
  return visc0 * ((Tair0 + 120.0) / (T + 120.0)) * pow(T / Tair0, 1.5);
}

// The air viscosity of every cell, shared by all classes (setvset.f90:95-97),
// and the Ganser iteration's cell factors sqrt(1/(3*rho)), rho/visc.
__global__ void k_visc(long long s3, const double* tempe, const double* rho, double* visc, double2* cf) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < s3;
       m += (long long)gridDim.x * blockDim.x) {
    const double vs = sutherland(tempe[m]), r = rho[m];
    visc[m] = vs;
    cf[m] = make_double2(sqrt(1.0 / (3.0 * r)), r / vs);
  }
}

// Runs chain cells [q0, q1) from cd; writes outputs when `write`.
__device__ void chain_run(const ChainGeom& g, long long q0, long long q1, int modv,
                          const ClassConst* cc, const double* viscs, const double2* cf, const double* rho,
                          double* vset, int* iters, double& cd, bool write, int& nonconv,
                          const DMathTab& tab) {
  const long long s3 = g.d.cells();
  for (long long q = q0; q < q1; ++q) {
    int ic;
    long long m;
    chain_cell(g, q, ic, m);
    const double visc = viscs[m];
    double v;
    const int it = vsettl_dev(cc[ic], modv, rho[m], visc, cf[m], cd, v, tab);
    if (write) {
      vset[(long long)ic * s3 + m] = v;
      if (iters) iters[(long long)ic * s3 + m] = it;
      if (it < 0 || !cc[ic].ok) nonconv = 1;
    }
  }
}

// Segment s of the chain: its entry cd (the chain's state for the first
// segment, else the value a warm-up of W cells from cd = 1 reaches), its
// cells and its exit cd.
__device__ __forceinline__ void chain_segment(const ChainGeom& g, long long s, int modv, const ClassConst* cc,
                                              const double* visc, const double2* cf, const double* rho,
                                              double* vset, int* iters, const double* cd_state, double* entry,
                                              double* exitv, int* nonconv, const DMathTab& tab) {
  const long long q0 = s * g.S, q1 = min(g.L, q0 + g.S);
  double cd;
  int nc_flag = 0, dummy = 0;
  if (s == 0) {
    cd = *cd_state;
  } else {
    cd = 1.0;
    chain_run(g, max(0LL, q0 - g.W), q0, modv, cc, visc, cf, rho, vset, iters, cd, false, dummy, tab);
  }
  entry[s] = cd;
  chain_run(g, q0, q1, modv, cc, visc, cf, rho, vset, iters, cd, true, nc_flag, tab);
  exitv[s] = cd;
  nonconv[s] = nc_flag;
}

// One segment per thread; a segment's result does not depend on the thread
// or block that computes it.
__global__ void __launch_bounds__(64, 16)
    k_chain_segments(ChainGeom g, int modv, const ClassConst* cc, const double* visc, const double2* cf,
                     const double* rho, double* vset, int* iters, const double* cd_state, double* entry,
                     double* exitv, int* nonconv) {
  __shared__ DMathTab tab;
  dmath_tab_init(tab);
  __syncthreads();
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= g.nseg) return;
  chain_segment(g, s, modv, cc, visc, cf, rho, vset, iters, cd_state, entry, exitv, nonconv, tab);
}

// The same segments computed beside the step kernel (a look-ahead meteo
// update on a second stream): blocks of four warps, one per SM sub-partition,
// at most 64 registers and 2.5 KB of shared memory, which is what a resident
// step-kernel block (four 112-register warps per sub-partition, 222 KB)
// leaves free.  Only the first block that starts on an SM works (claim[smid]);
// later ones on the same SM return at once, so that an SM idle at launch
// time does not fill up with chain blocks and shut the steps out.  The
// working blocks take segments from a counter until none is left.
__global__ void __launch_bounds__(128, 8)
    k_chain_beside(ChainGeom g, int modv, const ClassConst* cc, const double* visc, const double2* cf,
                   const double* rho, double* vset, int* iters, const double* cd_state, double* entry,
                   double* exitv, int* nonconv, int* claim, unsigned long long* next) {
  __shared__ DMathTab tab;
  __shared__ int mine;
  if (threadIdx.x == 0) {
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    mine = atomicCAS(claim + (smid & 255u), 0, 1) == 0;
  }
  dmath_tab_init(tab);
  __syncthreads();
  if (!mine) return;
  for (;;) {
    const unsigned long long s = atomicAdd(next, 1ULL);
    if (s >= (unsigned long long)g.nseg) break;
    chain_segment(g, (long long)s, modv, cc, visc, cf, rho, vset, iters, cd_state, entry, exitv, nonconv, tab);
  }
}

// Collects segments whose speculative entry differs from the predecessor's exit.
__global__ void k_chain_check(ChainGeom g, const double* entry, const double* exitv, int* bad,
                              int* nbad, int cap) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s < 1 || s >= g.nseg) return;
  if (__double_as_longlong(entry[s]) != __double_as_longlong(exitv[s - 1])) {
    const int slot = atomicAdd(nbad, 1);
    if (slot < cap) bad[slot] = (int)s;
  }
}

// Sequential repair in chain order (single thread).  Segments verified above
// stay; a recomputed segment may change its exit, so its successor is
// re-checked until the chain agrees again.  cap overflow -> full scan.
__global__ void k_chain_fix(ChainGeom g, int modv, const ClassConst* cc, const double* visc,
                            const double2* cf, const double* rho, double* vset, int* iters, double* entry,
                            double* exitv, int* nonconv, int* bad, const int* nbad, int cap,
                            double* cd_state) {
  __shared__ DMathTab tab;
  dmath_tab_init(tab);
  __syncthreads();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int nb = *nbad;
  if (nb > 0) {
    const bool full = nb > cap;
    int cnt = full ? 0 : nb;
    // insertion sort of the (few) bad segment ids
    for (int a = 1; a < cnt; ++a) {
      const int v = bad[a];
      int b = a - 1;
      while (b >= 0 && bad[b] > v) {
        bad[b + 1] = bad[b];
        --b;
      }
      bad[b + 1] = v;
    }
    long long s = full ? 1 : bad[0];
    int next = 1;  // index into bad[] of the next listed segment after s
    while (s < g.nseg) {
      const double expect = exitv[s - 1];
      if (__double_as_longlong(entry[s]) != __double_as_longlong(expect)) {
        double cd = expect;
        int nc_flag = 0;
        entry[s] = cd;
        const long long q0 = s * g.S, q1 = min(g.L, q0 + g.S);
        chain_run(g, q0, q1, modv, cc, visc, cf, rho, vset, iters, cd, true, nc_flag, tab);
        exitv[s] = cd;
        nonconv[s] = nc_flag;
        ++s;  // the successor must be re-checked
        continue;
      }
      if (full) {
        ++s;
        continue;
      }
      while (next < cnt && bad[next] <= s) ++next;
      if (next >= cnt) break;
      s = bad[next];
    }
  }
  *cd_state = exitv[g.nseg - 1];
}

__global__ void k_chain_status(ChainGeom g, const int* nonconv, int* status) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s < g.nseg && nonconv[s]) atomicOr(status, 1);
}

__global__ void k_dmath_eval(int op, long long n, const double* x, double* y) {
  __shared__ DMathTab tab;
  dmath_tab_init(tab);
  __syncthreads();
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    y[q] = op == 0 ? dm_log(tab, x[q]) : op == 1 ? dm_exp(tab, x[q]) : div_rn_recip(x[2 * q], x[2 * q + 1], 1.0 / x[2 * q + 1]);
}

void launch_dmath_eval(int op, long long n, const double* x, double* y, cudaStream_t s) {
  if (n <= 0) return;
  k_dmath_eval<<<(unsigned)std::min<long long>((n + 255) / 256, 152LL * 8), 256, 0, s>>>(op, n, x, y);
  count_launch();
}

// setvset.f90:48-60: the aggregate loop touches class np+1 (a gas class with
// vset = 0 when nc > np), then vset = -vset over all classes.
__global__ void k_vset_finish(long long s3, int nc, int np, int aggregate, double vset_factor,
                              double* vset) {
  const long long n = s3 * nc;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int ic = (int)(q / s3);
    // gas classes keep their previous value (zero of alternating sign, as the
    // reference negates the whole array at every update)
    double v = vset[q];
    if (aggregate && ic == np) v = vset_factor * v;
    vset[q] = -v;
  }
}

// Threads of k_chain_segments the device holds at once (blocks of 64).
static long long chain_capacity() {
  static long long cap = 0;
  if (cap == 0) {
    int dev = 0, nsm = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chain_segments, 64, 0);
    cap = (long long)std::max(1, nsm) * std::max(1, per_sm) * 64;
  }
  return cap;
}

static ChainGeom chain_geom(Dims d, int np) {
  ChainGeom g;
  g.d = d;
  g.L = d.cells() * np;
  // The segments are the threads of one launch: half as many as the device
  // holds at once when the chain is long enough (measured on cfg1: the
  // binary64 pipe stays as busy with half the threads resident, and the
  // warm-up of W cells recomputed from the preceding segment, enough for
  // the cd iteration to forget its guess, halves relative to the work;
  // a quarter is slower again), else fewer, longer segments.
  const long long cap = chain_capacity() / 2;
  long long S = (g.L + cap - 1) / cap;
  S = std::max<long long>(256, S);
  g.S = S;
  g.W = 64;
  g.nseg = (g.L + S - 1) / S;
  return g;
}

static constexpr int kBadCap = 8192;

size_t setvset_scratch_bytes(Dims d, int np) {
  const ChainGeom g = chain_geom(d, np);
  size_t b = sizeof(ClassConst) * (size_t)(np + 1);
  b += 2 * sizeof(double) * (size_t)g.nseg + sizeof(int) * (size_t)g.nseg;
  b += sizeof(int) * (kBadCap + 8) + 1024;
  b += sizeof(int) * 256 + sizeof(unsigned long long) + 512;  // per-SM claims, segment counter
  b += sizeof(double) * (size_t)d.cells() + 256;      // viscosity per cell
  b += 2 * sizeof(double) * (size_t)d.cells() + 256;  // Ganser cell factors
  return b;
}

void launch_setvset(Dims d, int nc, int np, int modv, const double* diam, const double* rhop,
                    const double* psi, const double* sphe, const double* tempe,
                    const double* rho, int aggregate, double vset_factor, double* vset,
                    int* iters, double* cd_state, void* scratch, int* status, cudaStream_t s,
                    int beside_step) {
  const ChainGeom g = chain_geom(d, np);
  unsigned char* p = reinterpret_cast<unsigned char*>(scratch);
  auto take = [&](size_t bytes) {
    unsigned char* r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  ClassConst* cc = reinterpret_cast<ClassConst*>(take(sizeof(ClassConst) * (size_t)(np + 1)));
  double* entry = reinterpret_cast<double*>(take(sizeof(double) * (size_t)g.nseg));
  double* exitv = reinterpret_cast<double*>(take(sizeof(double) * (size_t)g.nseg));
  int* nonconv = reinterpret_cast<int*>(take(sizeof(int) * (size_t)g.nseg));
  int* nbad = reinterpret_cast<int*>(take(sizeof(int) * 8));
  int* bad = reinterpret_cast<int*>(take(sizeof(int) * kBadCap));
  double* visc = reinterpret_cast<double*>(take(sizeof(double) * (size_t)d.cells()));
  double2* cf = reinterpret_cast<double2*>(take(2 * sizeof(double) * (size_t)d.cells()));
  int* claim = reinterpret_cast<int*>(take(sizeof(int) * 256));
  unsigned long long* next = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
  cudaMemsetAsync(nbad, 0, sizeof(int), s);
  cudaMemsetAsync(status, 0, sizeof(int), s);
  if (np > 0 && g.L > 0) {
    k_class_consts<<<(np + 31) / 32, 32, 0, s>>>(np, modv, diam, rhop, psi, sphe, cc);
    k_visc<<<(int)std::min<long long>((d.cells() + 255) / 256, 152LL * 16), 256, 0, s>>>(d.cells(), tempe,
                                                                                         rho, visc, cf);
    const int bs = 64;
    const long long nb = (g.nseg + bs - 1) / bs;
    if (beside_step) {
      static int nsm = 0;
      if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        // an SM holding this block must still take a step-kernel block
        cudaFuncSetAttribute(k_chain_beside, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
      }
      cudaMemsetAsync(claim, 0, sizeof(int) * 256, s);
      cudaMemsetAsync(next, 0, sizeof(unsigned long long), s);
      k_chain_beside<<<(unsigned)(4 * std::max(1, nsm)), 128, 0, s>>>(g, modv, cc, visc, cf, rho, vset, iters,
                                                                      cd_state, entry, exitv, nonconv, claim,
                                                                      next);
    } else {
      k_chain_segments<<<(unsigned)nb, bs, 0, s>>>(g, modv, cc, visc, cf, rho, vset, iters, cd_state, entry,
                                                   exitv, nonconv);
    }
    k_chain_check<<<(unsigned)((g.nseg + 255) / 256), 256, 0, s>>>(g, entry, exitv, bad, nbad, kBadCap);
    k_chain_fix<<<1, 32, 0, s>>>(g, modv, cc, visc, cf, rho, vset, iters, entry, exitv, nonconv, bad,
                                 nbad, kBadCap, cd_state);
    k_chain_status<<<(unsigned)((g.nseg + 255) / 256), 256, 0, s>>>(g, nonconv, status);
    count_launch(6);
  }
  const long long n = d.cells() * nc;
  k_vset_finish<<<(int)std::min<long long>((n + 255) / 256, 152LL * 16), 256, 0, s>>>(
      d.cells(), nc, np, aggregate, vset_factor, vset);
  count_launch();
}

}  // namespace f3d

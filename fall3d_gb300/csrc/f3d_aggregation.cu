// f3d_aggregation.cu -- aggregation in transport (Costa et al. 2010;
// AGGREGATION_IN_TRANSPORT = yes, Sources/readat.f90:350-440):
//
//  * agrpar (Sources/agrsrc.f90:95-319), run once after every source or
//    meteo update (Fall3d.f90:101-110): per cell the Brownian, shear and
//    differential-settling coefficients Abagr, Asagr, Adagr and the mean
//    sticking efficiency Alagr (0.09 in ice, the Stokes-number average over
//    the aggregating class pairs in liquid water, 0 in vapour), the water
//    phase from the plume temperature or, in the cloud, from QV, P and the
//    first gas (water_phase, :393-440); then vset of class iaggr times
//    vset_factor (:295-301);
//  * agrsrc (:1-91) every ndtagr steps inside setsrc (setsrc.f90:37-76): the
//    number of aggregating particles lost per unit time from the fractal
//    kernels, split over the classes iaggr..np-1 by Ni, a sink for them and a
//    source for the aggregate class np, added to c with ndtagr*dt, and the
//    accumulated aggregate mass Maggr.
//
// Both run one thread per cell in binary64 (--fmad=false) with CUDA's
// transcendentals; the per-class constants (Ni, d3 and the class sums) are
// evaluated on the host in the reference's order.
#include <cmath>
#include <vector>

#include "f3d_ctx_impl.h"

namespace f3d {
namespace {

constexpr double kPi = 3.14159265358979323846;  // Numeric.f90 pi

struct AgrPar {
  int iaggr, np, ng;
  double sumff, rhopmean, psi3, psi4, vset_factor, dX1, dX2;
};

__device__ int water_phase_dev(double qv, double P, double T, double wcloud) {
  double w = qv / (1.0 - qv);
  w = w + wcloud;
  const double e = P * w / (w + 0.622);
  double ew = 6.112 * exp(17.67 * (T - 273.16) / (T - 273.16 + 243.5));
  ew = 100.0 * ew;
  double ei = -(9.09718 * (273.16 / T - 1.0)) - 3.56654 * log10(273.16 / T) + 0.876793 * (1.0 - T / 273.16) +
              log10(6.1071);
  ei = 100.0 * pow(10.0, ei);
  if (e > ew) return T > (double)255.f ? 1 : 2;  // 1 water, 2 ice
  return e > ei ? 2 : 0;                         // 0 vapour
}

// get_gamas (agrsrc.f90:446-531): sqrt(1.3*2*SijSij) of the scaled winds
__device__ double gamas_dev(Dims d, int i, int j, int k, double dX1, double dX2, const double* dz,
                            const double* Hm1, const double* vx, const double* vy, const double* vz) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const double dXX = Hm1[d.P(i, j)] * dX1;
  double g[3][3];  // g[f][a]: d(field f)/d(axis a), f = u, v, w
  const double* f3[3] = {vx, vy, vz};
  for (int f = 0; f < 3; ++f) {
    const double* v = f3[f];
    if (i == 1)
      g[f][0] = (v[d.M(2, j, k)] - v[d.M(1, j, k)]) / dXX;
    else if (i == nx)
      g[f][0] = (v[d.M(nx, j, k)] - v[d.M(nx - 1, j, k)]) / dXX;
    else
      g[f][0] = (v[d.M(i + 1, j, k)] - v[d.M(i - 1, j, k)]) / (2.0 * dXX);
    if (j == 1)
      g[f][1] = (v[d.M(i, 2, k)] - v[d.M(i, 1, k)]) / dX2;
    else if (j == ny)
      g[f][1] = (v[d.M(i, ny, k)] - v[d.M(i, ny - 1, k)]) / dX2;
    else
      g[f][1] = (v[d.M(i, j + 1, k)] - v[d.M(i, j - 1, k)]) / (2.0 * dX2);
    if (k == 1)
      g[f][2] = (v[d.M(i, j, 2)] - v[d.M(i, j, 1)]) / dz[1];
    else if (k == nz)
      g[f][2] = (v[d.M(i, j, nz)] - v[d.M(i, j, nz - 1)]) / dz[nz - 1];
    else
      g[f][2] = (v[d.M(i, j, k + 1)] - v[d.M(i, j, k - 1)]) / (dz[k - 1] + dz[k]);
  }
  const double half = (double)0.5f;
  const double S11 = g[0][0], S12 = half * (g[1][0] + g[0][1]), S13 = half * (g[2][0] + g[0][2]);
  const double S21 = S12, S22 = g[1][1], S23 = half * (g[2][1] + g[1][2]);
  const double S31 = S13, S32 = S23, S33 = g[2][2];
  const double eps = S11 * S11 + S12 * S12 + S13 * S13 + S21 * S21 + S22 * S22 + S23 * S23 + S31 * S31 +
                     S32 * S32 + S33 * S33;
  return sqrt((double)(1.3f * 2.0f) * eps);
}

// agrpar (agrsrc.f90:160-301) for one cell, and vset(iaggr) *= vset_factor
template <class T>
__global__ void k_agrpar(Dims d, AgrPar a, const double* tplume, const double* tempe, const double* rho,
                         const double* qv, const double* pres, const T* c, const double* Hm1,
                         const double* vx, const double* vy, const double* vz, const double* dz,
                         const double* diam, const double* fc, double* vset, double* Alagr, double* Abagr,
                         double* Asagr, double* Adagr) {
  const long long s3 = d.cells();
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < s3;
       m += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(m % d.nx) + 1, j = (int)((m / d.nx) % d.ny) + 1, k = (int)(m / d.plane()) + 1;
    const double g = 9.81, kb = 1.38e-23, visc0 = 1.827e-5, Tair0 = (double)291.15f;
    const double Stcr = 1.3, qq = 0.8;
    const double tp = tplume[m];
    const double Tc = tp > 0.0 ? tp : tempe[m];
    const double rhoa = rho[m];
    const double visc = visc0 * ((Tair0 + 120.0) / (Tc + 120.0)) * pow(Tc / Tair0, 1.5);
    const double viscl = 2.414e-5 * pow(10.0, 247.7 / (Tc - 140.0));
    int phase;
    if (tp > 0.0) {
      phase = Tc < 255 ? 2 : (Tc < 373 ? 1 : 0);  // the plume's 'vapour' matches no case
    } else {
      double wcloud = a.ng > 0 ? (double)c[(long long)a.np * d.halo() + d.C(i, j, k)] / Hm1[d.P(i, j)]
                               : (double)0.f;
      wcloud = wcloud / rhoa;
      phase = water_phase_dev(qv[m], pres[m], Tc, wcloud);
    }
    const double ab = -(4.0 * kb * Tc / (3.0 * visc));
    const double gamas = gamas_dev(d, i, j, k, a.dX1, a.dX2, dz, Hm1, vx, vy, vz);
    const double as = -(2.0 * gamas * a.psi3 / 3.0);
    Abagr[m] = ab;
    Asagr[m] = as;
    Adagr[m] = -(kPi * (a.rhopmean - rhoa) * g * a.psi4 / (48.0 * visc));
    double al = 0.0;
    if (phase == 2) {
      al = 0.09;
    } else if (phase == 1) {
      for (int ic = a.iaggr; ic <= a.np - 1; ++ic)
        for (int jc = a.iaggr; jc <= a.np - 1; ++jc) {
          const double di = diam[ic - 1], dj = diam[jc - 1];
          const double vij = fabs(vset[(long long)(ic - 1) * s3 + m] - vset[(long long)(jc - 1) * s3 + m]) -
                             ab / (2.0 * kPi * di * dj) - as * di * dj / (4.0 * kPi);
          const double w = fc[ic - 1] * fc[jc - 1] / a.sumff;
          const double Stij = 8.0 * a.rhopmean * vij * di * dj / (9.0 * viscl * (di + dj));
          double alfa = 1.0 + pow(Stij / Stcr, qq);
          alfa = 1.0 / alfa;
          al = al + w * alfa;
        }
    }
    Alagr[m] = al;
    double& vs = vset[(long long)(a.iaggr - 1) * s3 + m];
    vs = a.vset_factor * vs;  // read above by this cell only
  }
}

struct AgrSrc {
  int iaggr, np;
  double Df, exps, expd, sumNi, dt, fac, dX1, dX2;
};

// agrsrc (agrsrc.f90:38-84) and the update of setsrc.f90:50-74 for one cell;
// cls[2*ic] = Ni(ic), cls[2*ic+1] = d3(ic) for ic = iaggr..np-1
template <class T>
__global__ void k_agrsrc(T* c, Dims d, AgrSrc a, const double* cls, const double* rhop, const double* Hm1,
                         const double* dz, const double* Alagr, const double* Abagr, const double* Asagr,
                         const double* Adagr, double* Maggr) {
  const long long s3 = d.cells(), hb = d.halo();
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < s3;
       m += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(m % d.nx) + 1, j = (int)((m / d.nx) % d.ny) + 1, k = (int)(m / d.plane()) + 1;
    const long long q = d.C(i, j, k);
    const double h = Hm1[d.P(i, j)];
    double ntot = 0.0, fi = 0.0;
    for (int ic = a.iaggr; ic <= a.np - 1; ++ic) {
      const double cv = (double)c[(long long)(ic - 1) * hb + q];
      fi = fi + cv / rhop[ic - 1];
      ntot = ntot + 6.0 * cv / cls[2 * ic + 1];
    }
    ntot = ntot / h;
    fi = fi / h;
    double dntot = Abagr[m] * pow(ntot, 2.0) + Asagr[m] * pow(ntot, a.exps) * pow(fi, 3.0 / a.Df) +
                   Adagr[m] * pow(ntot, a.expd) * pow(fi, 4.0 / a.Df);
    dntot = Alagr[m] * dntot;
    double tnp = 0.0;
    for (int ic = a.iaggr; ic <= a.np - 1; ++ic) {
      T& cr = c[(long long)(ic - 1) * hb + q];
      const double cv = (double)cr;
      const double dnj = dntot * cls[2 * ic] / a.sumNi;
      double t = dnj * cls[2 * ic + 1] / 6.0;
      if (cv + a.dt * t < 0.0) t = -cv / a.dt;
      tnp = tnp - t;
      cr = (T)(cv + a.fac * t);
    }
    T& ca = c[(long long)(a.np - 1) * hb + q];
    ca = (T)((double)ca + a.fac * tnp);
    const double dzeta = 0.5 * (dz[k - 1] + dz[k]);
    Maggr[m] = Maggr[m] + a.fac * tnp * h * a.dX1 * a.dX2 * dzeta;
  }
}

// settemplume: the plume temperature at the listed cells, 0 elsewhere
__global__ void k_plume_scatter(Dims d, int n, const int* ijk, const double* t, double* tplume) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) tplume[d.M(ijk[3 * q], ijk[3 * q + 1], ijk[3 * q + 2])] = t[q];
}

// vset(:,:,:,iaggr) = vset_factor*vset(:,:,:,iaggr) (agrsrc.f90:295-301)
__global__ void k_vset_scale(double* v, long long n, double f, int times) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double x = v[m];
    for (int q = 0; q < times; ++q) x = f * x;
    v[m] = x;
  }
}

unsigned grid_of(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16); }

}  // namespace

// agrpar after the updates of this step (Fall3d.f90:101-110)
int agg_agrpar(f3d_ctx* x) {
  const f3d_grid& g = x->g;
  const Dims d = x->d;
  const int np = g.np, iaggr = x->agr_iaggr;
  const double* fc = x->agr_fc.data();
  double sumfc = 0.0;
  for (int ic = iaggr; ic <= np - 1; ++ic) sumfc = sumfc + fc[ic - 1];
  double sumff = 0.0;
  for (int ic = iaggr; ic <= np - 1; ++ic)
    for (int jc = iaggr; jc <= np - 1; ++jc) sumff = sumff + fc[ic - 1] * fc[jc - 1];
  double rhopmean = 0.0;
  for (int ic = iaggr; ic <= np - 1; ++ic) rhopmean = rhopmean + fc[ic - 1] * x->h_rhop[ic - 1];
  rhopmean = rhopmean / sumfc;
  AgrPar a;
  a.iaggr = iaggr;
  a.np = np;
  a.ng = g.nc - np;
  a.sumff = sumff;
  a.rhopmean = rhopmean;
  a.psi3 = 6.0 / kPi;
  a.psi4 = a.psi3 * std::pow(6.0 / kPi, 1.0 / 3.0);
  a.vset_factor = g.vset_factor;
  a.dX1 = g.dX1;
  a.dX2 = g.dX2;
  cudaStream_t s = x->stream;
  if (x->prec == F3D_PREC_FP32)
    k_agrpar<float><<<grid_of(d.cells()), 256, 0, s>>>(d, a, x->agr_tplume, x->tempe, x->rho, x->agr_qv,
                                                       x->agr_p, x->c32, x->Hm1, x->vx, x->vy, x->vz, x->dz,
                                                       x->diam, x->agr_fc_dev, x->vset, x->agr_al, x->agr_ab,
                                                       x->agr_as, x->agr_ad);
  else
    k_agrpar<double><<<grid_of(d.cells()), 256, 0, s>>>(d, a, x->agr_tplume, x->tempe, x->rho, x->agr_qv,
                                                        x->agr_p, x->c64, x->Hm1, x->vx, x->vy, x->vz, x->dz,
                                                        x->diam, x->agr_fc_dev, x->vset, x->agr_al, x->agr_ab,
                                                        x->agr_as, x->agr_ad);
  count_launch();
  x->agr_npar = x->agr_npar + 1;
  if (x->prec == F3D_PREC_FP32) refresh_fp32_class(x, iaggr - 1);
  return cudaGetLastError() == cudaSuccess ? F3D_OK : ctx_error(F3D_ERR_CUDA, "agrpar launch failed");
}

// A restored run: the coefficients of its last agrpar come from the
// checkpoint (they depend on the state at that time); the replayed meteo
// update only needs class iaggr's settling velocity scaled once per agrpar
// the saved run made since its meteo update.
int agg_restore_vset(f3d_ctx* x, int times) {
  const long long s3 = x->d.cells();
  k_vset_scale<<<grid_of(s3), 256, 0, x->stream>>>(x->vset + (long long)(x->agr_iaggr - 1) * s3, s3,
                                                   x->g.vset_factor, times);
  count_launch();
  x->agr_npar = times;
  if (x->prec == F3D_PREC_FP32) refresh_fp32_class(x, x->agr_iaggr - 1);
  return cudaGetLastError() == cudaSuccess ? F3D_OK : ctx_error(F3D_ERR_CUDA, "vset scaling launch failed");
}

// setsrc.f90:37-76 after the point sources of this step
int agg_setsrc(f3d_ctx* x) {
  x->agr_ipass = x->agr_ipass + 1;
  if (x->agr_ipass % x->agr_ndtagr != 0) return F3D_OK;
  const f3d_grid& g = x->g;
  const Dims d = x->d;
  const int np = g.np, iaggr = x->agr_iaggr;
  cudaStream_t s = x->stream;
  AgrSrc a;
  a.iaggr = iaggr;
  a.np = np;
  a.Df = x->agr_Df;
  a.exps = 2.0 - (3.0 / x->agr_Df);
  a.expd = 2.0 - (4.0 / x->agr_Df);
  a.sumNi = x->agr_sumNi;
  a.dt = x->dt;
  a.fac = (double)x->agr_ndtagr * x->dt;
  a.dX1 = g.dX1;
  a.dX2 = g.dX2;
  if (x->prec == F3D_PREC_FP32)
    k_agrsrc<float><<<grid_of(d.cells()), 256, 0, s>>>(x->c32, d, a, x->agr_cls, x->rhop, x->Hm1, x->dz,
                                                       x->agr_al, x->agr_ab, x->agr_as, x->agr_ad, x->agr_maggr);
  else
    k_agrsrc<double><<<grid_of(d.cells()), 256, 0, s>>>(x->c64, d, a, x->agr_cls, x->rhop, x->Hm1, x->dz,
                                                        x->agr_al, x->agr_ab, x->agr_as, x->agr_ad,
                                                        x->agr_maggr);
  count_launch();
  return cudaGetLastError() == cudaSuccess ? F3D_OK : ctx_error(F3D_ERR_CUDA, "agrsrc launch failed");
}

}  // namespace f3d

using namespace f3d;

extern "C" {

int f3d_set_aggregation(f3d_ctx* x, const f3d_aggregation* ag) {
  if (!x) return ctx_error(F3D_ERR_ARG, "NULL context");
  ctx_prefetch_drop(x);  // a look-ahead meteo update does not run the aggregation model
  if (!ag) {
    x->agr_on = 0;
    return F3D_OK;
  }
  const f3d_grid& g = x->g;
  const int np = g.np;
  if (!g.aggregate) return ctx_error(F3D_ERR_ARG, "Aggregated class does not exist in the grn file");
  if (np < 2 || ag->ndtagr < 1 || !ag->fc) return ctx_error(F3D_ERR_ARG, "aggregation needs np >= 2, ndtagr >= 1, fc");
  // readat.f90:400-409
  int iaggr = 0;
  for (int ic = np - 1; ic >= 1; --ic)
    if (x->h_diam[np - 1] > x->h_diam[ic - 1]) iaggr = ic;
  if (iaggr == 0) iaggr = np - 1;
  const size_t s3 = (size_t)x->d.cells();
  if (!x->agr_al) {
    double** arrs[] = {&x->agr_al, &x->agr_ab, &x->agr_as, &x->agr_ad, &x->agr_maggr, &x->agr_tplume,
                       &x->agr_qv, &x->agr_p};
    for (double** a : arrs)
      if (int rc = ctx_alloc(x, reinterpret_cast<void**>(a), sizeof(double) * s3)) return rc;
    if (int rc = ctx_alloc(x, reinterpret_cast<void**>(&x->agr_fc_dev), sizeof(double) * (size_t)np)) return rc;
    if (int rc = ctx_alloc(x, reinterpret_cast<void**>(&x->agr_cls), sizeof(double) * 2 * (size_t)(np + 1)))
      return rc;
  }
  x->agr_fc.assign(ag->fc, ag->fc + np);
  // Ni and d3 of the aggregating classes (agrsrc.f90:27-32), constant
  std::vector<double> cls(2 * (size_t)(np + 1), 0.0);
  double sumNi = 0.0;
  for (int ic = iaggr; ic <= np - 1; ++ic) {
    const double di = x->h_diam[ic - 1];
    cls[2 * ic + 1] = kPi * x->h_rhop[ic - 1] * di * di * di;
    cls[2 * ic] = 1.0 * std::pow(x->h_diam[np - 1] / di, ag->Df);
    sumNi = sumNi + cls[2 * ic];
  }
  x->agr_sumNi = sumNi;
  if (cudaMemcpyAsync(x->agr_fc_dev, x->agr_fc.data(), sizeof(double) * np, cudaMemcpyHostToDevice, x->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(x->agr_cls, cls.data(), sizeof(double) * cls.size(), cudaMemcpyHostToDevice, x->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(x->stream) != cudaSuccess)
    return ctx_error(F3D_ERR_CUDA, "aggregation upload failed");
  x->agr_iaggr = iaggr;
  x->agr_Df = ag->Df;
  x->agr_ndtagr = ag->ndtagr;
  x->agr_ipass = 0;
  x->agr_on = 1;
  return F3D_OK;
}

int f3d_aggregation_met(f3d_ctx* x, const double* qv, const double* p) {
  if (!x || !qv || !p) return ctx_error(F3D_ERR_ARG, "NULL argument");
  if (!x->agr_on) return ctx_error(F3D_ERR_STATE, "aggregation is off");
  const size_t n = sizeof(double) * (size_t)x->d.cells();
  if (cudaMemcpyAsync(x->agr_qv, qv, n, cudaMemcpyDefault, x->stream) != cudaSuccess ||
      cudaMemcpyAsync(x->agr_p, p, n, cudaMemcpyDefault, x->stream) != cudaSuccess ||
      cudaStreamSynchronize(x->stream) != cudaSuccess)
    return ctx_error(F3D_ERR_CUDA, "QV/P upload failed");
  return F3D_OK;
}

int f3d_aggregation_plume(f3d_ctx* x, int n, const int* ix, const int* iy, const int* iz, const double* temp,
                          const double* water) {
  if (!x) return ctx_error(F3D_ERR_ARG, "NULL context");
  if (!x->agr_on) return ctx_error(F3D_ERR_STATE, "aggregation is off");
  if (n < 0 || (n > 0 && (!ix || !iy || !iz || !temp))) return ctx_error(F3D_ERR_ARG, "invalid plume list");
  (void)water;  // wplume is read by no computation of the reference
  const Dims d = x->d;
  std::vector<int> ijk(3 * (size_t)n);
  std::vector<double> t(temp, temp + n);
  for (int q = 0; q < n; ++q) {
    if (ix[q] < 1 || ix[q] > d.nx || iy[q] < 1 || iy[q] > d.ny || iz[q] < 1 || iz[q] > d.nz)
      return ctx_error(F3D_ERR_RANGE, "plume cell outside the grid");
    ijk[3 * q] = ix[q];
    ijk[3 * q + 1] = iy[q];
    ijk[3 * q + 2] = iz[q];
  }
  cudaStream_t s = x->stream;
  void* buf = nullptr;
  bool ok = cudaMemsetAsync(x->agr_tplume, 0, sizeof(double) * (size_t)d.cells(), s) == cudaSuccess;
  if (ok && n > 0) {
    ok = cudaMallocAsync(&buf, (sizeof(int) * 3 + sizeof(double)) * (size_t)n + 8, s) == cudaSuccess;
    int* dijk = reinterpret_cast<int*>(buf);
    double* dt = reinterpret_cast<double*>(dijk + 3 * (size_t)n + ((3 * n) & 1));
    ok = ok && cudaMemcpyAsync(dijk, ijk.data(), sizeof(int) * ijk.size(), cudaMemcpyHostToDevice, s) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(dt, t.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s) == cudaSuccess;
    if (ok) {
      k_plume_scatter<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(d, n, dijk, dt, x->agr_tplume);
      count_launch();
    }
    if (buf) cudaFreeAsync(buf, s);
  }
  // the host lists go out of scope
  if (!ok || cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return ctx_error(F3D_ERR_CUDA, "plume upload failed");
  return F3D_OK;
}

int f3d_download_maggr(f3d_ctx* x, double* maggr) {
  if (!x || !maggr) return ctx_error(F3D_ERR_ARG, "NULL argument");
  if (!x->agr_on) return ctx_error(F3D_ERR_STATE, "aggregation is off");
  if (cudaMemcpyAsync(maggr, x->agr_maggr, sizeof(double) * (size_t)x->d.cells(), cudaMemcpyDefault, x->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(x->stream) != cudaSuccess)
    return ctx_error(F3D_ERR_CUDA, "Maggr download failed");
  return F3D_OK;
}

}  // extern "C"

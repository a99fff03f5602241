/*
 * f3d_oracle.cpp -- CPU oracle of the FALL3D 7.0 transport step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file checks the results of the CUDA
 * library in fall3d_gb300/: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU baseline may load it, and the library never does.
 *
 * It restates, routine by routine and in the reference's own operation
 * order, the binary64 Fortran of lmingari/Fall3D (FALL3D 7.0, 2013):
 * every function cites the reference file:line it follows.  It is built
 * with -O2 -ffp-contract=off and no fast-math so that each Fortran
 * expression is evaluated as written (left-to-right, no FMA contraction).
 *
 * Semantics fixed where the Fortran is processor dependent:
 *  - MAX(a,b) / MIN(a,b) follow gfortran 4.8 (the reference's compiler,
 *    config.log:164): mvar=a; if (b .op. mvar .or. isnan(mvar)) mvar=b.
 *    They return the non-NaN operand and keep the first operand on ties.
 *  - SIGN(1,b) is copysign(1,b) (gfortran -fsign-zero), and a NaN b counts
 *    as positive: the default NaN of aarch64 and of CUDA is positive, while
 *    x86 produces a negative one, so the policy is written out explicitly.
 *  - libm: pow/exp/log/log10/acos/tan/atan/sin of the host C library.
 *
 * Parity status: pinned against outputs of the reference itself.  The
 * reference ships no tests, golden vectors or fixtures, and there is no
 * Fortran compiler here; oracle/ref_translate.py translates the reference's
 * own hot-path Fortran mechanically into C and builds it (oracle/_ref/),
 * tests/golden/make_golden.py runs that build on six scenarios (every
 * turbulence and settling model, UTM and lon-lat, wet deposition, two
 * meteo updates, 60 steps of cfg0) and stores the fields, budgets and
 * iteration counts, and tests/test_golden_cpu.py checks this oracle against
 * them bit for bit.  Known-answer tests (tests/test_oracle_cpu.py) add
 * analytic checks.
 */
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/fall3d_gpu.h"

namespace {

/* gfortran 4.8 MAX/MIN on two reals. */
inline double fmax2(double a, double b) { return (b > a || std::isnan(a)) ? b : a; }
inline double fmin2(double a, double b) { return (b < a || std::isnan(a)) ? b : a; }
/* SIGN(1.0,b) with a NaN b taken as positive. */
inline double sign1(double b) {
  if (std::isnan(b)) return 1.0;
  return std::signbit(b) ? -1.0 : 1.0;
}

struct Dims {
  int nx, ny, nz;
  size_t C(int i, int j, int k) const {  // c(0:nx+1,0:ny+1,0:nz+1)
    return (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k);
  }
  size_t M(int i, int j, int k) const {  // a(nx,ny,nz), 1-based
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
  }
  size_t P(int i, int j) const { return (size_t)(i - 1) + (size_t)nx * (size_t)(j - 1); }
  size_t halo() const { return (size_t)(nx + 2) * (ny + 2) * (nz + 2); }
  size_t cells() const { return (size_t)nx * ny * nz; }
  size_t plane() const { return (size_t)nx * ny; }
};

}  // namespace

extern "C" {

/* ---------------------------------------------------------------- setbcc */
/* Sources/setbcc.f90:19-109 */
void orc_setbcc(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
                const double* vx, const double* vy, const double* vz,
                const double* vset, const double* vdep, const double* rkver,
                const double* dz) {
  Dims d{nx, ny, nz};
  // Bottom (setbcc.f90:19-33)
  if (iz_loc == 1) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        if ((vz[d.M(i, j, 1)] + vset[d.M(i, j, 1)]) >= 0.0)
          c[d.C(i, j, 0)] = 0.0;
        else
          c[d.C(i, j, 0)] = c[d.C(i, j, 1)] * (1.0 + dz[0] * vdep[d.P(i, j)] / rkver[d.M(i, j, 1)]);
      }
  } else {
    for (int j = 0; j <= ny + 1; ++j)
      for (int i = 0; i <= nx + 1; ++i) c[d.C(i, j, 0)] = 0.0;
  }
  // Top (setbcc.f90:37-49)
  if ((iz_loc + nz_loc - 1) == nz) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        if ((vz[d.M(i, j, nz)] + vset[d.M(i, j, nz)]) <= 0.0)
          c[d.C(i, j, nz + 1)] = 0.0;
        else
          c[d.C(i, j, nz + 1)] = c[d.C(i, j, nz)];
      }
  } else {
    for (int j = 0; j <= ny + 1; ++j)
      for (int i = 0; i <= nx + 1; ++i) c[d.C(i, j, nz + 1)] = 0.0;
  }
  // Left/Right (setbcc.f90:53-66)
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k)
    for (int j = 1; j <= ny; ++j) {
      c[d.C(0, j, k)] = (vx[d.M(1, j, k)] >= 0.0) ? 0.0 : c[d.C(1, j, k)];
      c[d.C(nx + 1, j, k)] = (vx[d.M(nx, j, k)] <= 0.0) ? 0.0 : c[d.C(nx, j, k)];
    }
  // Up/Down (setbcc.f90:70-83)
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k)
    for (int i = 1; i <= nx; ++i) {
      c[d.C(i, 0, k)] = (vy[d.M(i, 1, k)] >= 0.0) ? 0.0 : c[d.C(i, 1, k)];
      c[d.C(i, ny + 1, k)] = (vy[d.M(i, ny, k)] <= 0.0) ? 0.0 : c[d.C(i, ny, k)];
    }
  // Corners (setbcc.f90:87-109)
  if (iz_loc == 1) {
    c[d.C(0, 0, 0)] = c[d.C(1, 1, 1)];
    c[d.C(nx + 1, 0, 0)] = c[d.C(nx, 1, 1)];
    c[d.C(0, ny + 1, 0)] = c[d.C(1, ny, 1)];
    c[d.C(nx + 1, ny + 1, 0)] = c[d.C(nx, ny, 1)];
  } else {
    c[d.C(0, 0, 0)] = 0.0;
    c[d.C(nx + 1, 0, 0)] = 0.0;
    c[d.C(0, ny + 1, 0)] = 0.0;
    c[d.C(nx + 1, ny + 1, 0)] = 0.0;
  }
  if ((iz_loc + nz_loc - 1) == nz) {
    c[d.C(0, 0, nz + 1)] = c[d.C(1, 1, nz)];
    c[d.C(nx + 1, 0, nz + 1)] = c[d.C(nx, 1, nz)];
    c[d.C(0, ny + 1, nz + 1)] = c[d.C(1, ny, nz)];
    c[d.C(nx + 1, ny + 1, nz + 1)] = c[d.C(nx, ny, nz)];
  } else {
    c[d.C(0, 0, nz + 1)] = 0.0;
    c[d.C(nx + 1, 0, nz + 1)] = 0.0;
    c[d.C(0, ny + 1, nz + 1)] = 0.0;
    c[d.C(nx + 1, ny + 1, nz + 1)] = 0.0;
  }
}

/* --------------------------------------------------------------- advctzc */
/* Sources/advctzc.f90:28-81 */
void orc_advctzc(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
                 const double* vz, const double* vset, const double* dz,
                 double dt) {
  Dims d{nx, ny, nz};
  // work(nx,ny,nz+1,2) (advctzc.f90:28)
  std::vector<double> w1((size_t)nx * ny * (nz + 1), 0.0), w2((size_t)nx * ny * (nz + 1), 0.0);
  auto W = [&](int i, int j, int k) { return d.M(i, j, k); };
  const int k0 = std::max(1, iz_loc - 1), k1 = std::min(nz, iz_loc + nz_loc);
  for (int k = k0; k <= k1; ++k) {
    const double dzz = 2.0 / (dz[k] + dz[k - 1]);
    const double dzk = 1.0 / dz[k];
    const double dzk_1 = 1.0 / dz[k - 1];
    const int kmax = std::max(1, k - 1);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const double vk = vz[d.M(i, j, k)] + vset[d.M(i, j, k)];
        const double vk_1 = vz[d.M(i, j, kmax)] + vset[d.M(i, j, kmax)];
        const double vk_12 = 0.5 * (vk + vk_1);
        w1[W(i, j, k)] = dt * (vk * c[d.C(i, j, k)] - vk_1 * c[d.C(i, j, k - 1)]) * dzz;
        const double deltar = (c[d.C(i, j, k + 1)] - c[d.C(i, j, k)]) * dzk;
        const double deltal = (c[d.C(i, j, k)] - c[d.C(i, j, k - 1)]) * dzk_1;
        const double sigma = 0.5 * (sign1(deltar) + sign1(deltal)) *
                             fmin2(std::fabs(deltar), std::fabs(deltal));
        const double Crk = std::fabs(vk_12) * dt * dzk_1;
        w2[W(i, j, k)] = dt * 0.5 * dz[k - 1] * (1.0 - Crk) * sigma * std::fabs(vk_12) * dzz;
      }
  }
  const double dznz = 1.0 / dz[nz];
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const double vk = vz[d.M(i, j, nz)] + vset[d.M(i, j, nz)];
      w1[W(i, j, nz + 1)] = dt * vk * (c[d.C(i, j, nz + 1)] - c[d.C(i, j, nz)]) * dznz;
    }
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k) {
    const int kmax = std::max(1, k - 1);
    const int kmin = std::min(nz, k + 1);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const double vk = vz[d.M(i, j, k)] + vset[d.M(i, j, k)];
        double& ck = c[d.C(i, j, k)];
        if (vk > 0.0)
          ck = ck - w1[W(i, j, k)] - (w2[W(i, j, k)] - w2[W(i, j, kmax)]);
        else
          ck = ck - w1[W(i, j, k + 1)] - (w2[W(i, j, kmin)] - w2[W(i, j, k)]);
      }
  }
}

/* ---------------------------------------------------------------- advctx */
/* Sources/advctx.f90:24-56.  The line kernel is shared with advcty: `at`
 * maps the line coordinate (0..n+1) to the concentration index and `vel`
 * maps 1..n to the velocity index. */
}  // extern "C"
template <class CIdx, class VIdx>
static void adv_line(double* c, int n, const double* v, double dx, double dt,
                     double* work1, double* work2, CIdx at, VIdx vel) {
  const double auxv = dt / dx;
  double vi = 0.0;
  for (int i = 1; i <= n; ++i) {
    vi = v[vel(i)];
    const double vi_1 = v[vel(std::max(1, i - 1))];
    const double vi_12 = 0.5 * (vi + vi_1);
    work1[i] = auxv * (vi * c[at(i)] - vi_1 * c[at(i - 1)]);
    const double deltar = (c[at(i + 1)] - c[at(i)]) / dx;
    const double deltal = (c[at(i)] - c[at(i - 1)]) / dx;
    const double sigma = 0.5 * (sign1(deltar) + sign1(deltal)) *
                         fmin2(std::fabs(deltar), std::fabs(deltal));
    const double Cri = auxv * std::fabs(vi_12);
    work2[i] = dt * 0.5 * (1.0 - Cri) * sigma * std::fabs(vi_12);
  }
  // advctx.f90:46: vi is the loop-leftover velocity at i = n.
  work1[n + 1] = auxv * vi * (c[at(n + 1)] - c[at(n)]);
  for (int i = 1; i <= n; ++i) {
    double& ci = c[at(i)];
    if (v[vel(i)] > 0.0)
      ci = ci - work1[i] - (work2[i] - work2[std::max(1, i - 1)]);
    else
      ci = ci - work1[i + 1] - (work2[std::min(n, i + 1)] - work2[i]);
  }
}

extern "C" {
void orc_advctx(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
                const double* vx, double dx, double dt) {
  Dims d{nx, ny, nz};
  std::vector<double> w1(nx + 2), w2(nx + 2);
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k)
    for (int j = 1; j <= ny; ++j)
      adv_line(c, nx, vx, dx, dt, w1.data(), w2.data(),
               [&](int i) { return d.C(i, j, k); }, [&](int i) { return d.M(i, j, k); });
}

/* Sources/advcty.f90:24-55 */
void orc_advcty(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
                const double* vy, double dy, double dt) {
  Dims d{nx, ny, nz};
  std::vector<double> w1(ny + 2), w2(ny + 2);
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k)
    for (int i = 1; i <= nx; ++i)
      adv_line(c, ny, vy, dy, dt, w1.data(), w2.data(),
               [&](int j) { return d.C(i, j, k); }, [&](int j) { return d.M(i, j, k); });
}

/* ----------------------------------------------------------------- diffz */
/* Sources/diffz.f90:22-62 */
void orc_diffz(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
               const double* dz, double dt, const double* rkver, const double* rho) {
  Dims d{nx, ny, nz};
  std::vector<double> l_dz(nz + 1), l_dzdz(nz + 1), work(nz + 1);
  for (int k = 0; k <= nz; ++k) l_dz[k] = 1.0 / dz[k];
  for (int k = 1; k <= nz; ++k) l_dzdz[k] = 2.0 / (dz[k] + dz[k - 1]);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      auto C = [&](int k) { return c[d.C(i, j, k)]; };
      auto R = [&](int k) { return rho[d.M(i, j, k)]; };
      auto K = [&](int k) { return rkver[d.M(i, j, k)]; };
      if (iz_loc == 1) {
        const double rkst = K(2) * R(2);
        const double rksb = K(1) * R(1);
        const double gradt = rkst * ((C(2) / R(2)) - (C(1) / R(1))) * l_dz[1];
        double gradb = rksb * ((C(1) / R(1)) - (C(0) / R(1))) * l_dz[0];
        gradb = fmax2(0.0, gradb);
        work[1] = dt * (gradt - gradb) * l_dzdz[1];
      }
      for (int k = std::max(2, iz_loc); k <= std::min(iz_loc + nz_loc - 1, nz - 1); ++k) {
        const double rkst = 0.5 * (R(k + 1) * K(k + 1) + R(k) * K(k));
        const double rksb = 0.5 * (R(k) * K(k) + R(k - 1) * K(k - 1));
        const double gradt = rkst * ((C(k + 1) / R(k + 1)) - (C(k) / R(k))) * l_dz[k];
        const double gradb = rksb * ((C(k) / R(k)) - (C(k - 1) / R(k - 1))) * l_dz[k - 1];
        work[k] = dt * (gradt - gradb) * l_dzdz[k];
      }
      if (iz_loc + nz_loc - 1 == nz) {
        const double rkst = K(nz) * R(nz);
        const double rksb = K(nz - 1) * R(nz - 1);
        double gradt = rkst * ((C(nz + 1) / R(nz)) - (C(nz) / R(nz))) * l_dz[nz];
        const double gradb = rksb * ((C(nz) / R(nz)) - (C(nz - 1) / R(nz - 1))) * l_dz[nz - 1];
        gradt = fmin2(0.0, gradt);
        work[nz] = dt * (gradt - gradb) * l_dz[nz];
      }
      for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k) c[d.C(i, j, k)] = C(k) + work[k];
    }
}

/* ----------------------------------------------------------- diffx/diffy */
/* Sources/diffx.f90:20-55 and Sources/diffy.f90:20-55 (same line form). */
}  // extern "C"
template <class CIdx, class VIdx>
static void diff_line(double* c, int n, const double* rkh, const double* rho,
                      double dtdx2, double* l_rho, double* work, CIdx at, VIdx m) {
  for (int i = 1; i <= n; ++i) l_rho[i] = 1.0 / rho[m(i)];
  {
    const double rksr = rkh[m(2)] * rho[m(2)];
    const double rksl = rkh[m(1)] * rho[m(1)];
    const double gradr = rksr * (c[at(2)] * l_rho[2] - c[at(1)] * l_rho[1]);
    double gradl = rksl * (c[at(1)] * l_rho[1] - c[at(0)] * l_rho[1]);
    gradl = fmax2(0.0, gradl);
    work[1] = dtdx2 * (gradr - gradl);
  }
  for (int i = 2; i <= n - 1; ++i) {
    const double rksr = 0.5 * (rho[m(i + 1)] * rkh[m(i + 1)] + rho[m(i)] * rkh[m(i)]);
    const double rksl = 0.5 * (rho[m(i)] * rkh[m(i)] + rho[m(i - 1)] * rkh[m(i - 1)]);
    const double gradr = rksr * (c[at(i + 1)] * l_rho[i + 1] - c[at(i)] * l_rho[i]);
    const double gradl = rksl * (c[at(i)] * l_rho[i] - c[at(i - 1)] * l_rho[i - 1]);
    work[i] = dtdx2 * (gradr - gradl);
  }
  {
    const double rksr = rkh[m(n)] * rho[m(n)];
    const double rksl = rkh[m(n - 1)] * rho[m(n - 1)];
    double gradr = rksr * (c[at(n + 1)] * l_rho[n] - c[at(n)] * l_rho[n]);
    const double gradl = rksl * (c[at(n)] * l_rho[n] - c[at(n - 1)] * l_rho[n - 1]);
    gradr = fmin2(0.0, gradr);
    work[n] = dtdx2 * (gradr - gradl);
  }
  for (int i = 1; i <= n; ++i) c[at(i)] = c[at(i)] + work[i];
}

extern "C" {
void orc_diffx(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
               double dx, double dt, const double* rkhor, const double* rho) {
  Dims d{nx, ny, nz};
  const double dtdx2 = dt / (dx * dx);
  std::vector<double> l_rho(nx + 2), work(nx + 2);
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k)
    for (int j = 1; j <= ny; ++j)
      diff_line(c, nx, rkhor, rho, dtdx2, l_rho.data(), work.data(),
                [&](int i) { return d.C(i, j, k); }, [&](int i) { return d.M(i, j, k); });
}

void orc_diffy(double* c, int nx, int ny, int nz, int nz_loc, int iz_loc,
               double dy, double dt, const double* rkhor, const double* rho) {
  Dims d{nx, ny, nz};
  const double dtdy2 = dt / (dy * dy);
  std::vector<double> l_rho(ny + 2), work(ny + 2);
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k)
    for (int i = 1; i <= nx; ++i)
      diff_line(c, ny, rkhor, rho, dtdy2, l_rho.data(), work.data(),
                [&](int j) { return d.C(i, j, k); }, [&](int j) { return d.M(i, j, k); });
}

/* ---------------------------------------------------------------- wetdep */
/* Sources/wetdep.f90:28-50.  cwet points at cwet(1,1,0); ic is 1-based. */
void orc_wetdep(double* c, double* cwet, int ic, int nx, int ny, int nz,
                int nz_loc, int iz_loc, double dt, const double* diam,
                const double* zlayer, const double* dz, const double* zi,
                const double* prate) {
  Dims d{nx, ny, nz};
  double diam_max = 100.0;
  diam_max = diam_max * 1e-6;
  if (diam[ic - 1] > diam_max) return;
  const double a = 8.4e-5, b = 0.79;
  double* cw = cwet + (size_t)ic * d.plane();
  for (int ix = 1; ix <= nx; ++ix)
    for (int iy = 1; iy <= ny; ++iy) {
      const double lambda = fmin2(dt * a * std::pow(prate[d.P(ix, iy)], b), 1.0);
      for (int iz = iz_loc; iz <= iz_loc + nz_loc - 1; ++iz) {
        if (zlayer[iz - 1] <= zi[d.P(ix, iy)]) {
          cw[d.P(ix, iy)] = cw[d.P(ix, iy)] + dz[iz] * lambda * c[d.C(ix, iy, iz)];
          c[d.C(ix, iy, iz)] = c[d.C(ix, iy, iz)] * (1.0 - lambda);
        }
      }
    }
}

/* ----------------------------------------------------------------- accum */
/* Sources/accum.f90:17-25.  cdry points at cdry(1,1,0). */
void orc_accum(double* c, double* cdry, int ic, int nx, int ny, int nz,
               int nz_loc, int iz_loc, double dt, const double* vset,
               const double* vdep) {
  (void)nz_loc;
  Dims d{nx, ny, nz};
  if (iz_loc != 1) return;
  double* cd = cdry + (size_t)ic * d.plane();
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      cd[d.P(i, j)] = cd[d.P(i, j)] - dt * c[d.C(i, j, 1)] *
                                          fmin2(0.0, vset[d.M(i, j, 1)] + vdep[d.P(i, j)]);
}

/* ------------------------------------------------------------------ clip */
/* Sources/sizloop.f90:77-78 */
void orc_clip(double* c, int nx, int ny, int nz, int ic_loc, int nc_loc) {
  Dims d{nx, ny, nz};
  const size_t h = d.halo();
  for (size_t q = (size_t)(ic_loc - 1) * h; q < (size_t)(ic_loc - 1 + nc_loc) * h; ++q)
    c[q] = fmax2(0.0, c[q]);
}

/* --------------------------------------------------------------- cmass2d */
/* Sources/cmass2d.f90:36-105, serial build (nproc = 1, mymass(0)). */
void orc_cmass2d(const double* c, const double* vx, const double* vy,
                 const double* vz, const double* vset, int nx, int ny, int nz,
                 int nc, int ic_loc, int nc_loc, int iz_loc, int nz_loc,
                 double dx, double dy, const double* dz, double dt,
                 double* outmass) {
  (void)nc;
  Dims d{nx, ny, nz};
  const size_t h = d.halo(), s3 = d.cells();
  double mymass = 0.0;
  for (int ic = ic_loc; ic <= ic_loc + nc_loc - 1; ++ic) {
    const double* cc = c + (size_t)(ic - 1) * h;
    for (int j = 1; j <= ny; ++j) {
      double faty = 1.0;
      if (j == 1 || j == ny) faty = 0.5;
      for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k) {
        const double area = faty * dy * 0.5 * (dz[k] + dz[k - 1]);
        double velo = vx[d.M(1, j, k)];
        double conc = cc[d.C(0, j, k)];
        mymass = mymass - dt * area * velo * conc;
        velo = vx[d.M(nx, j, k)];
        conc = cc[d.C(nx + 1, j, k)];
        mymass = mymass + dt * area * velo * conc;
      }
    }
  }
  for (int ic = ic_loc; ic <= ic_loc + nc_loc - 1; ++ic) {
    const double* cc = c + (size_t)(ic - 1) * h;
    for (int i = 1; i <= nx; ++i) {
      double fatx = 1.0;
      if (i == 1 || i == nx) fatx = 0.5;
      for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k) {
        const double area = fatx * dx * 0.5 * (dz[k] + dz[k - 1]);
        double velo = vy[d.M(i, 1, k)];
        double conc = cc[d.C(i, 0, k)];
        mymass = mymass - dt * area * velo * conc;
        velo = vy[d.M(i, ny, k)];
        conc = cc[d.C(i, ny + 1, k)];
        mymass = mymass + dt * area * velo * conc;
      }
    }
  }
  for (int ic = ic_loc; ic <= ic_loc + nc_loc - 1; ++ic) {
    const double* cc = c + (size_t)(ic - 1) * h;
    const double* vs = vset + (size_t)(ic - 1) * s3;
    if ((iz_loc + nz_loc - 1) == nz) {
      for (int j = 1; j <= ny; ++j) {
        double faty = 1.0;
        if (j == 1 || j == ny) faty = 0.5;
        for (int i = 1; i <= nx; ++i) {
          double fatx = 1.0;
          if (i == 1 || i == nx) fatx = 0.5;
          const double area = fatx * faty * dx * dy;
          const double velo = vz[d.M(i, j, nz)] + vs[d.M(i, j, nz)];
          const double conc = cc[d.C(i, j, nz + 1)];
          mymass = mymass + dt * area * velo * conc;
        }
      }
    }
  }
  // parallel_sum is a no-op in the serial build; sum(mymass) = 0 + mymass(0).
  double s = 0.0;
  s = s + mymass;
  *outmass = *outmass + s;
}

/* --------------------------------------------------------------- cmass3d */
/* Sources/cmass3d.f90:29-58 */
void orc_cmass3d(const double* c, const double* cload, const double* cdry,
                 const double* cwet, int nx, int ny, int nz, int nc, double dx,
                 double dy, const double* dz, double* out4) {
  Dims d{nx, ny, nz};
  const size_t h = d.halo();
  double massvol = 0.0, massdep = 0.0, massdry = 0.0, masswet = 0.0;
  for (int i = 1; i <= nx; ++i) {
    double fatx = 1.0;
    if (i == 1 || i == nx) fatx = 0.5;
    for (int j = 1; j <= ny; ++j) {
      double faty = 1.0;
      if (j == 1 || j == ny) faty = 0.5;
      for (int ic = 1; ic <= nc; ++ic) {
        const double* cc = c + (size_t)(ic - 1) * h;
        double zmass = 0.0;
        for (int k = 1; k <= nz - 1; ++k)
          zmass = zmass + 0.5 * dz[k] * (cc[d.C(i, j, k)] + cc[d.C(i, j, k + 1)]);
        massvol = massvol + fatx * faty * zmass;
      }
      massdep = massdep + fatx * faty * cload[d.P(i, j)];
      massdry = massdry + fatx * faty * cdry[d.P(i, j)];
      masswet = masswet + fatx * faty * cwet[d.P(i, j)];
    }
  }
  out4[0] = massvol * dx * dy;
  out4[1] = massdep * dx * dy;
  out4[2] = massdry * dx * dy;
  out4[3] = masswet * dx * dy;
}

/* ----------------------------------------------------------------- getc0 */
/* Sources/endstep.f90:94-104, then cload = cdry + cwet (endstep.f90:35,60) */
void orc_getc0(double* cdry, double* cwet, double* cload, int nx, int ny,
               int nc, int np) {
  Dims d{nx, ny, 1};
  const size_t pl = d.plane();
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      const size_t p = d.P(i, j);
      cdry[p] = 0.0;
      cwet[p] = 0.0;
      for (int ic = 1; ic <= np; ++ic) {
        cdry[p] = cdry[p] + cdry[(size_t)ic * pl + p];
        cwet[p] = cwet[p] + cwet[(size_t)ic * pl + p];
      }
    }
  for (size_t q = 0; q < (size_t)(nc + 1) * pl; ++q) cload[q] = cdry[q] + cwet[q];
}

/* ---------------------------------------------------------------- setsrc */
/* Sources/setsrc.f90:20-35 (serial build: every k in 1..nz is local).
 * Returns 0, or 6 when a source lies outside the horizontal grid (the
 * reference would write outside the interior). */
int orc_setsrc(double* c, int nx, int ny, int nz, int nc, int nsou,
               const int* isrc, const int* jsrc, const int* ksrc,
               const double* tmrat, const double* dz, const double* zlayer,
               const double* Hm1, double dX1, double dX2, double dt) {
  Dims d{nx, ny, nz};
  const size_t h = d.halo();
  for (int is = 0; is < nsou; ++is)
    if (isrc[is] < 1 || isrc[is] > nx || jsrc[is] < 1 || jsrc[is] > ny || ksrc[is] > nz) return 6;
  for (int is = 0; is < nsou; ++is) {
    const int i = isrc[is], j = jsrc[is], k = ksrc[is];
    if (k >= 1 && k <= nz) {
      double dzeta;
      if (k == 1)
        dzeta = 0.5 * dz[k] + zlayer[k - 1];
      else
        dzeta = 0.5 * (dz[k - 1] + dz[k]);
      const double vol0 = Hm1[d.P(i, j)] * dX1 * dX2 * dzeta;
      for (int ic = 1; ic <= nc; ++ic) {
        double& cc = c[(size_t)(ic - 1) * h + d.C(i, j, k)];
        cc = cc + dt * tmrat[(size_t)is + (size_t)nsou * (ic - 1)] / vol0;
      }
    }
  }
  return 0;
}

/* ---------------------------------------------------------------- finddt */
/* Sources/finddt.f90:26-61 */
void orc_finddt(int nx, int ny, int nz, int nc, double dX1, double dX2,
                const double* dz, const double* vx, const double* vy,
                const double* vz, const double* vset, const double* rkh1,
                const double* rkhor, const double* rkver, double safety,
                double* dt, double* dtc) {
  Dims d{nx, ny, nz};
  const size_t s3 = d.cells();
  const double R8MIN = 1e-13;
  double dtcn = 0.0;
  for (int ic = 1; ic <= nc; ++ic) {
    const double* vs = vset + (size_t)(ic - 1) * s3;
    for (int k = 1; k <= nz; ++k) {
      const double ddz = fmin2(dz[k - 1], dz[k]);
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double dvsetdz;
          if (k == 1)
            dvsetdz = (vs[d.M(i, j, 2)] - vs[d.M(i, j, 1)]) / (dz[1]);
          else if (k == nz)
            dvsetdz = (vs[d.M(i, j, nz)] - vs[d.M(i, j, nz - 1)]) / (dz[nz - 1]);
          else
            dvsetdz = (vs[d.M(i, j, k + 1)] - vs[d.M(i, j, k - 1)]) / (dz[k] + dz[k - 1]);
          const size_t m = d.M(i, j, k);
          // x**2.0_rp is exact as x*x (IEEE pow(x,2) is correctly rounded).
          const double dtcni = (2.0 * rkh1[m] / (dX1 * dX1)) + (std::fabs(vx[m]) / dX1) +
                               (2.0 * rkhor[m] / (dX2 * dX2)) + (std::fabs(vy[m]) / dX2) +
                               (2.0 * rkver[m] / (ddz * ddz)) +
                               (std::fabs((vz[m] + vs[m])) / ddz) + (std::fabs(dvsetdz));
          dtcn = fmax2(dtcn, dtcni);
        }
    }
  }
  dtcn = fmax2(dtcn, R8MIN);
  *dtc = 1.0 / dtcn;
  *dt = safety * (*dtc);
}

/* ---------------------------------------------------------------- kappa3 */
/* Sources/kappa3.f90:50-236 */
void orc_kappa3(int nx, int ny, int nz, int modkv, int modkh, int coord_sys,
                double rkv0, double rkh0, double Csh, double dX1, double dX2,
                double dx, double dy, const double* dz, const double* zlayer,
                const double* Hm1, const double* vx, const double* vy,
                const double* vptemp, const double* ustar, const double* zi,
                const double* rl, double* rkver, double* rkhor) {
  Dims d{nx, ny, nz};
  const double vkarm = 0.4, beta1 = 9.2, beta2 = 13.0, gi = 9.81, alfa = 0.28;
  const double rlamb = 30.0, rkhmin = 1e2, rkvmin = 1.0, hinf = 5.0, hsup = 5e3;
  const double Khf = 8000.0;
  if (modkv == 0) {
    for (size_t q = 0; q < d.cells(); ++q) rkver[q] = rkv0;
  } else if (modkv == 1) {
    double rich = 0.0, dvdz2 = 0.0;  // carried across points (kappa3.f90:64-71)
    for (int k = 2; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          if (k < nz) {
            const double dzs = dz[k] + dz[k - 1];
            const double gx = (vx[d.M(i, j, k + 1)] - vx[d.M(i, j, k - 1)]) / dzs;
            const double gy = (vy[d.M(i, j, k + 1)] - vy[d.M(i, j, k - 1)]) / dzs;
            dvdz2 = gx * gx + gy * gy;
            dvdz2 = fmax2(dvdz2, 1e-10);
            rich = gi * ((vptemp[d.M(i, j, k + 1)] - vptemp[d.M(i, j, k - 1)]) / (dz[k] + dz[k - 1])) /
                   (vptemp[d.M(i, j, k)] * dvdz2);
          }
          const double h = fmin2(fmax2(zi[d.P(i, j)], hinf), hsup);
          const double zeta = zlayer[k - 1] / h;
          const double zl = zlayer[k - 1];
          double& kv = rkver[d.M(i, j, k)];
          if (zeta < 1.0) {
            if (rl[d.P(i, j)] >= 0.0)
              kv = vkarm * ustar[d.P(i, j)] * zl * (1.0 - zeta) / (1.0 + beta1 * zl * rl[d.P(i, j)]);
            else
              kv = vkarm * ustar[d.P(i, j)] * zl * (1.0 - zeta) * std::sqrt(1.0 - beta2 * zl * rl[d.P(i, j)]);
          } else {
            const double lc = 1.0 / ((1.0 / (vkarm * zl)) + (1.0 / rlamb));
            if (rich >= 0.0) {
              kv = lc * lc * std::sqrt(dvdz2) / (1.0 + 10.0 * rich * (1.0 + 8.0 * rich));
              kv = fmax2(kv, rkvmin);
            } else {
              kv = lc * lc * std::sqrt(dvdz2) * std::sqrt(1.0 - 18.0 * rich);
              kv = fmax2(kv, rkvmin);
            }
          }
        }
  } else if (modkv == 2) {
    const double gh = 11.6, betah = 7.8, prt = 0.95;
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double zl = zlayer[k - 1];
          const double us = ustar[d.P(i, j)];
          double zeta = zl * rl[d.P(i, j)];
          double& kv = rkver[d.M(i, j, k)];
          if (zeta < 0.0)
            kv = vkarm * us * zl * std::sqrt(1.0 - gh * zeta) / prt;
          else if (zeta > 0.0)
            kv = vkarm * us * zl / (prt + betah * zeta);
          else
            kv = vkarm * us * zl / prt;
          const double h = fmin2(fmax2(zi[d.P(i, j)], hinf), hsup);
          zeta = zl / h;
          if (zeta > 1.0) zeta = 1.0;
          kv = kv * (1.0 - zeta);
        }
  }
  if (modkh == 0) {
    for (size_t q = 0; q < d.cells(); ++q) rkhor[q] = rkh0;
  } else if (modkh == 1 || modkh == 2) {
    const double Khn0 = (coord_sys == F3D_COORD_LONLAT) ? 3.6e-2 : 4000.0;
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double dXX = Hm1[d.P(i, j)] * dX1;
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
          double& kh = rkhor[d.M(i, j, k)];
          if (modkh == 1) {
            const double Kmh = 0.075 * std::pow(dXX * dX2, 2.0 / 3.0);
            const double s1 = dvxdy + dvydx;
            kh = Csh * Csh * dXX * dX2 * std::sqrt(s1 * s1 + 2.0 * (dvxdx * dvxdx + dvydy * dvydy));
            kh = 1.0 * fmax2(kh, Kmh);
            kh = fmax2(kh, rkhmin);
          } else {
            const double s1 = dvxdx - dvydy, s2 = dvydx + dvxdy;
            const double Kht = alfa * alfa * dXX * dX2 * std::sqrt(s1 * s1 + s2 * s2);
            const double Khn = Khf * (Khn0 / Hm1[d.P(i, j)] / dx) * (Khn0 / dy);
            kh = (1.0 / Kht) + (1.0 / Khn);
            kh = fmax2(1.0 / kh, rkhmin);
          }
        }
  }
}

/* -------------------------------------------------- get_gama and vsettl */
/* Sources/setpsi.f90:65-127.  Returns the iteration count, or -1 when the
 * bisection does not converge (the reference calls runend). */
int orc_get_gama(double diam, double sphe, double* gama_out) {
  const double d = diam * 1e3;
  const int niter = 1000;
  const double toler = 1e-8;
  double gmin = 1e-3, gmax = 1.0;
  const double pi = 4.0 * std::atan(1.0);
  const double h = 0.5 * d;
  const double Vp = 4.0 * pi * (h * h * h) / 3.0;
  const double Ap = std::pow(pi, 1.0 / 3.0) * std::pow(6.0 * Vp, 2.0 / 3.0) / sphe;
  double gama = 0.0;
  for (int it = 1; it <= niter; ++it) {
    gama = 0.5 * (gmin + gmax);
    const double e = std::acos(gama);
    const double Ao = 0.5 * pi * d * d * std::pow(gama, -4.0 / 3.0) * (gama * gama + (e / std::tan(e)));
    if (Ao < Ap)
      gmax = gama;
    else
      gmin = gama;
    if ((it > 1) && (std::fabs(Ao - Ap) < toler)) {
      *gama_out = gama;
      return it;
    }
  }
  *gama_out = gama;
  return -1;
}

/* Sources/setvset.f90:65-181.  cd is the SAVEd drag coefficient (in/out).
 * gama is get_gama(diam,sphe) (pure per class, passed in).  Returns the
 * iteration count at convergence (0 for the closed-form Dellino model) or
 * -1 when the fixed point does not converge within maxit. */
int orc_vsettl(double diam, double rhop, double rhoa, double visc, double* vset,
               int model, double psi, double gama, double* cd) {
  const double gi = 9.81, eps = 1e-3;
  const int maxit = 100;
  double vold = 1e5;
  double v = 0.0;
  if (model == 1) {
    for (int it = 1; it <= maxit; ++it) {
      v = std::sqrt(4.0 * gi * diam * rhop / (3.0 * (*cd) * rhoa));
      const double rey = rhoa * v * diam / visc;
      if (rey <= 988.947)
        *cd = 24.0 / rey * (1.0 + 0.15 * std::pow(rey, 0.687));
      else
        *cd = 0.44;
      if (it > 1 && std::fabs(v - vold) <= eps) {
        *vset = std::sqrt(4.0 * gi * diam * rhop / (3.0 * (*cd) * rhoa));
        return it;
      }
      vold = v;
    }
  } else if (model == 2) {
    // gama**(-2.0/3.0): the exponent is a default-real (binary32) constant.
    const double dnd = 0.5 * (1.0 + gama) * std::pow(gama, (double)(-2.0f / 3.0f));
    for (int it = 1; it <= maxit; ++it) {
      v = std::sqrt(4.0 * gi * diam * rhop / (3.0 * (*cd) * rhoa));
      const double rey = rhoa * v * diam / visc;
      const double rk1 = 1.0 / (dnd / 3.0 + 2.0 / (3.0 * std::sqrt(psi)));
      const double rk2 = std::pow(10.0, 1.8148 * std::pow(-std::log10(psi), 0.5743));
      *cd = 24.0 / (rey * rk1) * (1.0 + 0.1118 * std::pow(rey * rk1 * rk2, 0.6567)) +
            0.4305 * rk2 / (1.0 + 3305.0 / (rey * rk1 * rk2));
      if (it > 1 && std::fabs(v - vold) <= eps) {
        *vset = std::sqrt(4.0 * gi * diam * rhop / (3.0 * (*cd) * rhoa));
        return it;
      }
      vold = v;
    }
  } else if (model == 3) {
    for (int it = 1; it <= maxit; ++it) {
      v = std::sqrt(4.0 * gi * diam * rhop / (3.0 * (*cd) * rhoa));
      const double rey = rhoa * v * diam / visc;
      if (rey <= 100.0) {
        *cd = 24.0 / rey * std::pow(psi, -0.828) + 2.0 * std::sqrt(1.0 - psi);
      } else if (rey > 100.0 && rey < 1000.0) {
        const double cd100 = 0.24 * std::pow(psi, -0.828) + 2.0 * std::sqrt(1.0 - psi);
        const double a = (1.0 - cd100) / 900.0;
        const double b = 1.0 - 1000.0 * a;
        *cd = a * rey + b;
      } else {
        *cd = 1.0;
      }
      if (it > 1 && std::fabs(v - vold) <= eps) {
        *vset = std::sqrt(4.0 * gi * diam * rhop / (3.0 * (*cd) * rhoa));
        return it;
      }
      vold = v;
    }
  } else if (model == 4) {
    v = std::pow((diam * diam * diam * gi * (rhop - rhoa) * rhoa * std::pow(psi, 1.6)) / (visc * visc), 0.5206);
    v = (1.2065 * visc * v) / (diam * rhoa);
    *vset = v;
    return 0;
  }
  *vset = v;
  return -1;
}

/* Sources/setvset.f90:25-60.  The cd chain runs ic -> i -> j -> k.  iters
 * (optional, nx*ny*nz*np) receives each call's iteration count.  Returns 0,
 * or 3 on non-convergence (runend in the reference). */
int orc_setvset(int nx, int ny, int nz, int nc, int np, int modv,
                const double* diam, const double* rhop, const double* psi,
                const double* sphe, const double* tempe, const double* rho,
                int aggregate, double vset_factor, double* vset, double* cd,
                int* iters) {
  Dims d{nx, ny, nz};
  const size_t s3 = d.cells();
  const double visc0 = 1.827e-5;
  const double Tair0 = (double)291.15f;  // default-real literal (setvset.f90:23)
  for (int ic = 1; ic <= np; ++ic) {
    double gama = 0.0;
    if (modv == 2) {
      // get_gama is a pure function of (diam, sphe): one evaluation per class
      // gives the value every call of setvset.f90:119 computes.
      if (orc_get_gama(diam[ic - 1], sphe[ic - 1], &gama) < 0) return 3;
    }
    for (int i = 1; i <= nx; ++i)
      for (int j = 1; j <= ny; ++j)
        for (int k = 1; k <= nz; ++k) {
          const double T = tempe[d.M(i, j, k)];
          const double visc = visc0 * ((Tair0 + 120.0) / (T + 120.0)) * std::pow(T / Tair0, 1.5);
          double v = 0.0;
          const int it = orc_vsettl(diam[ic - 1], rhop[ic - 1], rho[d.M(i, j, k)], visc, &v, modv,
                                    psi[ic - 1], gama, cd);
          if (it < 0) return 3;
          vset[(size_t)(ic - 1) * s3 + d.M(i, j, k)] = v;
          if (iters) iters[(size_t)(ic - 1) * s3 + d.M(i, j, k)] = it;
        }
  }
  // setvset.f90:48-56 indexes class np+1 (the loop variable after the loop):
  // a gas class (vset = 0) when nc > np, outside the array otherwise.
  if (aggregate && nc > np) {
    double* vs = vset + (size_t)np * s3;
    for (size_t q = 0; q < s3; ++q) vs[q] = vset_factor * vs[q];
  }
  for (size_t q = 0; q < s3 * nc; ++q) vset[q] = -vset[q];
  return 0;
}

/* ------------------------------------------------------------ setvdrydep */
/* Sources/setvdrydep.f90:74-264 */
void orc_setvdrydep(int nx, int ny, int nc, const double* diam,
                    const double* zlayer, const double* ldu, const double* rl,
                    const double* znt, const double* ustar, const double* tempe,
                    const double* rho, double* vdep) {
  Dims d{nx, ny, 1};
  const double vkarm = 0.4, visc0 = 1.827e-5, Tair0 = 291.15;
  static const double A[6][4] = {{0.0048, 0.0315, 1.2891, 1.0338}, {0.0037, 0.0120, 1.3977, 1.0707},
                                 {0.0042, 0.2928, 1.3970, 0.9155}, {0.0032, 0.1201, 1.1838, 1.0096},
                                 {0.0043, 0.1337, 1.2834, 1.1595}, {0.0045, 0.0925, 1.2654, 1.0891}};
  static const double B[6][4] = {{1.0, 2.7925, 2.6878, 1.2644}, {1.0, 2.2413, 2.5838, 1.3247},
                                 {1.0, 3.8581, 2.5580, 1.0364}, {1.0, 3.4407, 2.8033, 1.2069},
                                 {1.0, 3.5456, 2.7157, 1.4863}, {1.0, 3.2920, 2.7227, 1.4240}};
  std::vector<int> imode(nc);
  bool have_to_work = false;
  for (int ic = 0; ic < nc; ++ic) {
    if (diam[ic] > 100e-6) imode[ic] = 0;
    else if (diam[ic] > 10e-6) { imode[ic] = 4; have_to_work = true; }
    else if (diam[ic] > 2.5e-6) { imode[ic] = 3; have_to_work = true; }
    else if (diam[ic] > 0.1e-6) { imode[ic] = 2; have_to_work = true; }
    else { imode[ic] = 1; have_to_work = true; }
  }
  if (!have_to_work) return;
  static const int usgs_to_feng[25] = {6, 1, 6, 6, 6, 6, 6, 6, 6, 6, 3, 6, 6, 6,
                                       6, 6, 5, 6, 6, 3, 2, 2, 2, 2, 4};
  for (int iy = 1; iy <= ny; ++iy)
    for (int ix = 1; ix <= nx; ++ix) {
      const size_t p = d.P(ix, iy);
      const double lv = ldu[p];
      int iland = 6;
      // INT() truncates toward zero; codes outside 1..24 map to 6.
      if (lv > -1.0 && lv < 25.0) {
        const int code = (int)lv;
        if (code >= 1 && code <= 24) iland = usgs_to_feng[code];
      }
      const double zeta = rl[p] * zlayer[0];
      const double zeta0 = rl[p] * znt[p];
      double ra;
      if (ustar[p] > 0.0) {
        ra = std::log(zlayer[0] / znt[p]);
        if (zeta > 0) {
          ra = ra + 4.7 * (zeta - zeta0);
        } else if (zeta < 0) {
          const double eta = std::pow(1.0 - 15.0 * zeta, 0.25);
          const double eta0 = std::pow(1.0 - 15.0 * zeta0, 0.25);
          ra = ra + std::log((eta0 * eta0 + 1) * ((eta0 + 1) * (eta0 + 1)) /
                             ((eta * eta + 1) * ((eta + 1) * (eta + 1))));
          ra = ra + 2 * (std::atan(eta) - std::atan(eta0));
        }
        ra = ra / (ustar[p] * vkarm);
      } else {
        ra = 1e20;
      }
      const double T = tempe[p];  // tempe(ix,iy,1)
      const double visc = visc0 * ((Tair0 + 120.0) / (T + 120.0)) * std::pow(T / Tair0, 1.5);
      double Re = ustar[p] * znt[p] * rho[p] / visc;
      if (Re > 40300.0) Re = 40300.0;
      double Vd1 = -0.5 * ((Re - 40300.0) / 15330.0) * ((Re - 40300.0) / 15330.0);
      Vd1 = 0.0226 * ustar[p] * std::exp(Vd1);
      for (int ic = 0; ic < nc; ++ic) {
        if (imode[ic] > 0) {
          double Vd = Vd1 + A[iland - 1][imode[ic] - 1] * std::pow(ustar[p], B[iland - 1][imode[ic] - 1]);
          Vd = ra + 1.0 / Vd;
          vdep[(size_t)ic * d.plane() + p] = -1.0 / Vd;
        }
      }
    }
}

/* ----------------------------------------------- scaling, corvver, divu */
/* Sources/meteo.f90:108-123, Sources/corvver.f90:21-34, setdivu.f90:16-30 */
/* Sources/setdivu.f90 */
static void orc_setdivu(int nx, int ny, int nz, double dX1, double dX2, const double* dz,
                        const double* Hm1, const double* vx, const double* vy, const double* vz,
                        double* divu) {
  Dims d{nx, ny, nz};
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      for (int k = 1; k <= nz; ++k) {
        const double vi = vx[d.M(i, j, k)], vi_1 = vx[d.M(std::max(1, i - 1), j, k)];
        const double vj = vy[d.M(i, j, k)], vj_1 = vy[d.M(i, std::max(1, j - 1), k)];
        const double vk = vz[d.M(i, j, k)], vk_1 = vz[d.M(i, j, std::max(1, k - 1))];
        divu[d.M(i, j, k)] = (vi - vi_1) / (Hm1[d.P(i, j)] * dX1) + (vj - vj_1) / dX2 + (vk - vk_1) / dz[k];
      }
}

void orc_meteo_scale(int nx, int ny, int nz, int coord_sys, double dX1,
                     double dX2, const double* dz, const double* Hm1,
                     const double* topg, double* vx, double* vy, double* vz,
                     double* rho, const double* rkhor, double* rkh1, double* divu) {
  Dims d{nx, ny, nz};
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t m = d.M(i, j, k);
        const double h = Hm1[d.P(i, j)];
        vx[m] = vx[m] / h;
        rho[m] = rho[m] * h;
        rkh1[m] = rkhor[m] / (h * h);
      }
  if (coord_sys == F3D_COORD_LONLAT) {
    const double dyinv = 1.0 / dX2;
    for (int iy = 1; iy <= ny; ++iy)
      for (int ix = 1; ix <= nx; ++ix) {
        const double dxinv = 1.0 / (Hm1[d.P(ix, iy)] * dX1);
        const double zx = dxinv * (topg[d.P(std::min(ix + 1, nx), iy)] - topg[d.P(ix, iy)]);
        const double zy = dyinv * (topg[d.P(ix, std::min(iy + 1, ny))] - topg[d.P(ix, iy)]);
        for (int iz = 1; iz <= nz; ++iz) {
          const size_t m = d.M(ix, iy, iz);
          const double vs = zx * vx[m] + zy * vy[m];
          vz[m] = vz[m] - vs;
        }
      }
  }
  if (divu) orc_setdivu(nx, ny, nz, dX1, dX2, dz, Hm1, vx, vy, vz, divu);
}

/* --------------------------------------------------------- output fields */
/* Sources/printres_nc.f90.  Class sums run from 0 in class order over the
 * selected classes and are divided by Hm1 afterwards ("work3d = work3d +
 * c(...,ic)" then "work3d = work3d/Hm1"), the column trapezoid runs from
 * the first layer upwards, and the unit factor multiplies the finished sum. */
static double orc_class_sum(const double* c, const Dims& d, int i, int j, int k, const int* cls,
                            int ncls) {
  double s = 0.0;
  for (int n = 0; n < ncls; ++n) s = s + c[(size_t)cls[n] * d.halo() + d.C(i, j, k)];
  return s;
}

/* z-cumulative concentration, g/m2: :216-247 (particles), :249-279 (one
 * gas), :281-387 (PM05/PM10/PM20); cls are 0-based class indices. */
void orc_out_column(const double* c, int nx, int ny, int nz, const int* cls, int ncls,
                    const double* dz, const double* Hm1, double* out) {
  Dims d{nx, ny, nz};
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const size_t p = d.P(i, j);
      double work2d = 0.0;
      for (int iz = 1; iz <= nz - 1; ++iz) {
        const double w0 = orc_class_sum(c, d, i, j, iz, cls, ncls) / Hm1[p];
        const double w1 = orc_class_sum(c, d, i, j, iz + 1, cls, ncls) / Hm1[p];
        work2d = work2d + dz[iz] * 0.5 * (w0 + w1);
      }
      out[p] = 1e3 * work2d;
    }
}

/* first-layer concentration, g/m3: :389-411 (particles), :413-493 (PM) */
void orc_out_ground(const double* c, int nx, int ny, int nz, const int* cls, int ncls,
                    const double* Hm1, double* out) {
  Dims d{nx, ny, nz};
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const size_t p = d.P(i, j);
      const double work2d = orc_class_sum(c, d, i, j, 1, cls, ncls);
      out[p] = 1e3 * work2d / Hm1[p];
    }
}

/* PM selections of :284-370 and :416-479: particle classes (1..np) with
 * diam <= 5e-6, 1e-5 or 2e-5 m; returns their count, 0-based in cls. */
int orc_pm_classes(int np, const double* diam, int microns, int* cls) {
  const double thr = microns == 5 ? 5e-6 : microns == 10 ? 1e-5 : 2e-5;
  int n = 0;
  for (int ic = 1; ic <= np; ++ic)
    if (diam[ic - 1] <= thr) cls[n++] = ic - 1;
  return n;
}

/* get_AOT_prop, :2066-2123: effective radii (um -> m) and efficiencies */
static void orc_aot_prop(double* reff, double* qeff) {
  static const double r[20] = {0.014, 0.020, 0.028, 0.040, 0.056, 0.079, 0.112, 0.158, 0.224, 0.316,
                               0.447, 0.631, 0.891, 1.259, 1.778, 2.512, 3.548, 5.012, 7.079, 10.000};
  static const double q[20] = {0.00213, 0.00386, 0.00864, 0.02324, 0.06674, 0.18285, 0.44613,
                               0.93225, 1.63000, 2.35760, 2.83130, 2.90880, 2.72340, 2.50530,
                               2.35970, 2.27100, 2.21020, 2.16410, 2.12830, 2.10050};
  for (int b = 0; b < 20; ++b) {
    reff[b] = r[b] * 1e-6;
    qeff[b] = q[b];
  }
}

/* aerosol optical thickness, :495-540 */
void orc_out_aot(const double* c, int nx, int ny, int nz, int np, const double* diam,
                 const double* rhop, const double* dz, const double* Hm1, double* out) {
  Dims d{nx, ny, nz};
  double reff[20], qeff[20];
  orc_aot_prop(reff, qeff);
  const size_t pl = d.plane();
  std::vector<double> work2d(pl, 0.0), work3d(d.cells());
  for (int ic = 1; ic <= np; ++ic) {
    if (!(0.5 * diam[ic - 1] >= reff[0] && 0.5 * diam[ic - 1] <= reff[19])) continue;
    int ieff = 0;  /* 1-based as in the reference */
    for (int i = 1; i <= 19; ++i)
      if (0.5 * diam[ic - 1] >= reff[i - 1] && 0.5 * diam[ic - 1] <= reff[i]) ieff = i + 1;
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          work3d[d.M(i, j, k)] = c[(size_t)(ic - 1) * d.halo() + d.C(i, j, k)] / Hm1[d.P(i, j)];
    for (int iz = 1; iz <= nz - 1; ++iz)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t p = d.P(i, j);
          work2d[p] = work2d[p] + dz[iz] * 0.5 * (work3d[d.M(i, j, iz)] + work3d[d.M(i, j, iz + 1)]) *
                                      0.75 * qeff[ieff - 1] / (rhop[ic - 1] * reff[ieff - 1]);
        }
  }
  for (size_t p = 0; p < pl; ++p) out[p] = work2d[p];
}

/* deposit thickness, cm, :191-214 (cload is (nx,ny,0:nc)) */
void orc_out_thick(const double* cload, int nx, int ny, int np, const double* rhop,
                   const double* Hm1, double* out) {
  const size_t pl = (size_t)nx * ny;
  for (size_t p = 0; p < pl; ++p) {
    double work2d = 0.0;
    for (int ic = 1; ic <= np; ++ic) work2d = work2d + cload[(size_t)ic * pl + p] / rhop[ic - 1];
    out[p] = 1e2 * work2d / Hm1[p];
  }
}

/* Sources/setcut.f90:60-107 (standard_atm): ICAO pressure at height z */
double orc_standard_pressure(double z) {
  const double goo = 9.80665, Roo = 8.31432, Moo = 0.0289644;
  const double zoo = 0.0, Too = 288.15, poo = 101325.0, Loo = -0.0065;
  const double zo1 = 11000.0, To1 = 216.65, po1 = 22632.0;
  const double zo2 = 20000.0, To2 = 216.65, po2 = 5474.0, Lo2 = 0.001;
  double T, P;
  if (z < zo1) {
    T = Too + Loo * (z - zoo);
    P = poo * std::pow(Too / T, goo * Moo / (Roo * Loo));
  } else if (z < zo2) {
    T = To1;
    P = po1 * std::exp(-(goo * Moo * (z - zo1) / (Roo * To1)));
  } else {
    T = To2 + Lo2 * (z - zo2);
    P = po2 * std::pow(To2 / T, goo * Moo / (Roo * Lo2));
  }
  (void)T;
  return P;
}

/* Sources/setcut.f90:1-54 (setcut_FL) on a precomputed var3d (nx,ny,nz) */
void orc_setcut_fl(int nx, int ny, int nz, double* var2d, const double* var3d, const double* p,
                   double fl) {
  const double pnom = orc_standard_pressure(fl);
  const size_t pl = (size_t)nx * ny;
  for (size_t q = 0; q < pl; ++q) {
    if (pnom > p[q]) {
      var2d[q] = 0.0;
      continue;
    }
    bool go_on = true;
    int iz = 0;
    while (go_on) {
      iz = iz + 1;
      const double p0 = p[(size_t)(iz - 1) * pl + q], p1 = p[(size_t)iz * pl + q];
      if (pnom <= p0 && pnom > p1) {
        go_on = false;
        const double s = (pnom - p0) / (p1 - p0);
        var2d[q] = var3d[(size_t)(iz - 1) * pl + q] * (1.0 - s) + var3d[(size_t)iz * pl + q] * s;
      }
      if (iz + 1 == nz && go_on) {
        var2d[q] = 0.0;
        go_on = false;
      }
    }
  }
}

/* Sources/ter2asl.f90:1-55 in place on conc (nx,ny,nz) */
void orc_ter2asl(double* conc, const double* topg, const double* zlayer, int nx, int ny, int nz) {
  const size_t pl = (size_t)nx * ny;
  std::vector<double> c(conc, conc + pl * nz);
  for (size_t q = 0; q < pl; ++q) {
    const double zo = fmax2(0.0, topg[q]);
    for (int iz = 1; iz <= nz; ++iz) {
      const double zasl = zlayer[iz - 1];
      double& o = conc[(size_t)(iz - 1) * pl + q];
      if (zasl < zo + zlayer[0]) {
        o = 0.0;
        continue;
      }
      bool found = false;
      int izz = 0;
      while (!found) {
        izz = izz + 1;
        if (zasl >= zo + zlayer[izz - 1] && zasl <= zo + zlayer[izz]) {
          found = true;
          const double s = (zo + zlayer[izz] - zasl) / (zlayer[izz] - zlayer[izz - 1]);
          o = s * c[(size_t)(izz - 1) * pl + q] + (1.0 - s) * c[(size_t)izz * pl + q];
        }
        if (izz + 1 == nz && !found) {
          o = 0.0;
          found = true;
        }
      }
    }
  }
}

/* particle concentration w = (sum_{ic<=np} c)/Hm1 on the model levels
 * (the work3d of :545-556, :577-584) */
static void orc_particle_conc(const double* c, const Dims& d, int np, const double* Hm1,
                              std::vector<double>& w) {
  w.assign(d.cells(), 0.0);
  for (int ic = 1; ic <= np; ++ic)
    for (int k = 1; k <= d.nz; ++k)
      for (int j = 1; j <= d.ny; ++j)
        for (int i = 1; i <= d.nx; ++i)
          w[d.M(i, j, k)] = w[d.M(i, j, k)] + c[(size_t)(ic - 1) * d.halo() + d.C(i, j, k)];
  for (int k = 1; k <= d.nz; ++k)
    for (int j = 1; j <= d.ny; ++j)
      for (int i = 1; i <= d.nx; ++i) w[d.M(i, j, k)] = w[d.M(i, j, k)] / Hm1[d.P(i, j)];
}

/* flight-level cut, g/m3, :542-573 (fl in hundreds of feet) */
void orc_out_fl(const double* c, int nx, int ny, int nz, int np, const double* p, double fl,
                const double* Hm1, double* out) {
  Dims d{nx, ny, nz};
  std::vector<double> w;
  orc_particle_conc(c, d, np, Hm1, w);
  const double flm = fl * 30.48;
  orc_setcut_fl(nx, ny, nz, out, w.data(), p, flm);
  for (size_t q = 0; q < d.plane(); ++q) out[q] = 1e3 * out[q];
}

/* 3-D concentration, g/m3: ic 0 = all particles (:575-601), else class ic
 * (:646-671); asl: ter2asl as when terrain_following is false */
void orc_out_con(const double* c, int nx, int ny, int nz, int np, int ic, const double* Hm1,
                 const double* zlayer, const double* topg, int asl, double* out) {
  Dims d{nx, ny, nz};
  std::vector<double> w;
  if (ic == 0) {
    orc_particle_conc(c, d, np, Hm1, w);
  } else {
    w.assign(d.cells(), 0.0);
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          w[d.M(i, j, k)] = c[(size_t)(ic - 1) * d.halo() + d.C(i, j, k)] / Hm1[d.P(i, j)];
  }
  for (size_t q = 0; q < d.cells(); ++q) out[q] = 1e3 * w[q];
  if (asl) orc_ter2asl(out, topg, zlayer, nx, ny, nz);
}

/* Tracking points: Sources/reaout.f90:180-224 (get_pts_st), writps.f90:
 * 64-148, writps_air.f90:64-109, writps.f90:205-222 (writps_end); cload
 * is (nx,ny,0:nc) after getc0.  out per point: 7 + 3*nz + 1 + np values. */
int orc_track_points(const double* c, const double* cload, int nx, int ny, int nz, int np,
                     const double* diam, const double* rhop, const double* dz, const double* Hm1,
                     double dxo, double dyo, double xo, double yo, int npts, const double* xpts,
                     const double* ypts, double* out) {
  Dims d{nx, ny, nz};
  const size_t pl = d.plane();
  double reff[20], qeff[20];
  orc_aot_prop(reff, qeff);
  const double pi = 3.14159265358979323846;
  const int stride = 7 + 3 * nz + 1 + np;
  for (int n = 0; n < npts; ++n) {
    int ip = 0, jp = 0;
    double sp = 0.0, tp = 0.0;
    bool found = false;
    for (int ix = 1; ix <= nx - 1; ++ix) {
      const double x = xo + (ix - 1) * dxo;
      if (xpts[n] >= x && xpts[n] <= x + dxo) {
        ip = ix;
        sp = (xpts[n] - x) / dxo;
        sp = 2.0 * sp - 1.0;
        found = true;
      }
    }
    if (!found) return 6;
    found = false;
    for (int iy = 1; iy <= ny - 1; ++iy) {
      const double y = yo + (iy - 1) * dyo;
      if (ypts[n] >= y && ypts[n] <= y + dyo) {
        jp = iy;
        tp = (ypts[n] - y) / dyo;
        tp = 2.0 * tp - 1.0;
        found = true;
      }
    }
    if (!found) return 6;
    const double s = sp, t = tp, st = s * t;
    const double v1 = (1.0 - t - s + st) * 0.25, v2 = (1.0 - t + s - st) * 0.25;
    const double v3 = (1.0 + t + s + st) * 0.25, v4 = (1.0 + t - s - st) * 0.25;
    const size_t p1 = d.P(ip, jp), p2 = d.P(ip + 1, jp), p3 = d.P(ip + 1, jp + 1), p4 = d.P(ip, jp + 1);
    const double h1 = Hm1[p1], h2 = Hm1[p2], h3 = Hm1[p3], h4 = Hm1[p4];
    auto C = [&](int ic, int i, int j, int k) { return c[(size_t)(ic - 1) * d.halo() + d.C(i, j, k)]; };
    double* o = out + (size_t)n * stride;
    o[0] = v1 * (cload[p1] / h1) + v2 * (cload[p2] / h2) + v3 * (cload[p3] / h3) + v4 * (cload[p4] / h4);
    double thick = 0.0;
    for (int ic = 1; ic <= np; ++ic) {
      const double* f = cload + (size_t)ic * pl;
      thick = thick + v1 * (f[p1] / h1 / rhop[ic - 1]) + v2 * (f[p2] / h2 / rhop[ic - 1]) +
              v3 * (f[p3] / h3 / rhop[ic - 1]) + v4 * (f[p4] / h4 / rhop[ic - 1]);
    }
    o[1] = 1e2 * thick;
    auto acc = [&](double a, int ic, int k) {
      return a + v1 * (C(ic, ip, jp, k) / h1) + v2 * (C(ic, ip + 1, jp, k) / h2) +
             v3 * (C(ic, ip + 1, jp + 1, k) / h3) + v4 * (C(ic, ip, jp + 1, k) / h4);
    };
    double cg = 0.0, pm5 = 0.0, pm10 = 0.0, pm20 = 0.0;
    for (int ic = 1; ic <= np; ++ic) cg = acc(cg, ic, 1);
    for (int ic = 1; ic <= np; ++ic)
      if (diam[ic - 1] <= 5e-6) pm5 = acc(pm5, ic, 1);
    for (int ic = 1; ic <= np; ++ic)
      if (diam[ic - 1] <= 1e-5) pm10 = acc(pm10, ic, 1);
    for (int ic = 1; ic <= np; ++ic)
      if (diam[ic - 1] <= 2e-5) pm20 = acc(pm20, ic, 1);
    o[2] = cg * 1e3;
    o[3] = pm5 * 1e3;
    o[4] = pm10 * 1e3;
    o[5] = pm20 * 1e3;
    double cummc = 0.0;
    for (int ic = 1; ic <= np; ++ic)
      for (int iz = 1; iz <= nz - 1; ++iz) {
        const double cp1 = acc(0.0, ic, iz), cp2 = acc(0.0, ic, iz + 1);
        cummc = cummc + dz[iz] * 0.5 * (cp1 + cp2);
      }
    o[6] = 1e3 * cummc;
    double aod = 0.0;
    for (int iz = 1; iz <= nz; ++iz) {
      double cz = 0.0, ext = 0.0, nco = 0.0;
      for (int ic = 1; ic <= np; ++ic) {
        const double cc = v1 * (C(ic, ip, jp, iz) / h1) + v2 * (C(ic, ip + 1, jp, iz) / h2) +
                          v3 * (C(ic, ip + 1, jp + 1, iz) / h3) + v4 * (C(ic, ip, jp + 1, iz) / h4);
        cz = cz + cc;
        const double rad = (double)0.5f * diam[ic - 1];
        if (rad >= reff[0] && rad <= reff[19]) {
          int ieff = 0;
          for (int jeff = 1; jeff <= 19; ++jeff)
            if (rad >= reff[jeff - 1] && rad <= reff[jeff]) ieff = jeff + 1;
          ext = ext + (cc * 0.75 * qeff[ieff - 1]) / (rhop[ic - 1] * reff[ieff - 1]);
          aod = aod + (dz[iz] * cc * 0.75 * qeff[ieff - 1]) / (rhop[ic - 1] * reff[ieff - 1]);
        }
        if (rad <= 32e-6)
          nco = nco + (6.0 * cc) / (rhop[ic - 1] * pi * diam[ic - 1] * diam[ic - 1] * diam[ic - 1]);
      }
      o[7 + iz - 1] = cz * 1e3;
      o[7 + nz + iz - 1] = ext * 1e6;
      o[7 + 2 * nz + iz - 1] = nco * 1e-6;
    }
    o[7 + 3 * nz] = aod;
    for (int ic = 1; ic <= np; ++ic) {
      const double* f = cload + (size_t)ic * pl;
      o[8 + 3 * nz + ic - 1] = v1 * (f[p1] / h1) + v2 * (f[p2] / h2) + v3 * (f[p3] / h3) + v4 * (f[p4] / h4);
    }
  }
  return 0;
}

/* LOAD, COL_MASS and C_GRND of the context's state (:105-123, :216-247,
 * :389-411) */
void orc_outputs(const double* c, const double* cload, int nx, int ny, int nz,
                 int np, const double* dz, const double* Hm1, double* load,
                 double* col_mass, double* c_grnd) {
  std::vector<int> cls(np);
  for (int ic = 0; ic < np; ++ic) cls[ic] = ic;
  const size_t pl = (size_t)nx * ny;
  if (load)
    for (size_t p = 0; p < pl; ++p) load[p] = cload[p] / Hm1[p];
  if (col_mass) orc_out_column(c, nx, ny, nz, cls.data(), np, dz, Hm1, col_mass);
  if (c_grnd) orc_out_ground(c, nx, ny, nz, cls.data(), np, Hm1, c_grnd);
}

/* ===================================================================== */
/* Context mirroring the coarse API, driven by the same time loop.       */
/* ===================================================================== */
struct orc_ctx {
  int nx, ny, nz, nc, np, coord, modkv, modkh, modv, wetdep, aggregate;
  double dX1, dX2, dx, dy, rkh0, rkv0, Csh, safety, vset_factor;
  std::vector<double> dz, zlayer, Hm1, topg, diam, rhop, psi, sphe;
  std::vector<double> c, cdry, cwet, cload;
  std::vector<double> vx, vy, vz, tempe, vptemp, rho, rkhor, rkh1, rkver, vset, vdep, divu;
  std::vector<double> ustar, zi, rl, znt, prate, ldu;
  std::vector<int> vset_iters;
  double cd = 1.0;
  int nsou = 0;
  std::vector<int> isrc, jsrc, ksrc;
  std::vector<double> tmrat;
  double flowrate = 0.0, time = 0.0, dt = 1.0, dtc = 0.0, erumass = 0.0, outmass = 0.0;
  int iiter = 0;
  int have_met = 0;
  int nthreads = 1;
  // f3d_run loop state (Fall3d.f90:73-78)
  int run_started = 0, meteotime = 1, sourcetime = 1;
  double meteo_time = 0.0, source_time = 0.0;
  // gravity current (readat.f90:150-213)
  int gc_on = 0;
  f3d_gravity_current gc{};
  // aggregation in transport (readat.f90:350-440, agrsrc.f90)
  int agg_on = 0, iaggr = 0, ndtagr = 1, agr_ipass = 0, agr_due = 0;
  double Df = 3.0;
  std::vector<double> fc, qv, pres, tplume, wplume, Alagr, Abagr, Asagr, Adagr, Maggr;
};

orc_ctx* orc_ctx_create(const f3d_grid* g, int nthreads) {
  orc_ctx* x = new orc_ctx();
  x->nx = g->nx; x->ny = g->ny; x->nz = g->nz; x->nc = g->nc; x->np = g->np;
  x->coord = g->coord_sys; x->modkv = g->modkv; x->modkh = g->modkh; x->modv = g->modv;
  x->wetdep = g->wetdep; x->aggregate = g->aggregate;
  x->dX1 = g->dX1; x->dX2 = g->dX2; x->dx = g->dx; x->dy = g->dy;
  x->rkh0 = g->rkh0; x->rkv0 = g->rkv0; x->Csh = g->Csh; x->safety = g->safety_factor;
  x->vset_factor = g->vset_factor;
  const int nx = g->nx, ny = g->ny, nz = g->nz, nc = g->nc;
  const size_t s3 = (size_t)nx * ny * nz, pl = (size_t)nx * ny;
  x->dz.assign(g->dz, g->dz + nz + 1);
  x->zlayer.assign(g->zlayer, g->zlayer + nz);
  x->Hm1.assign(g->Hm1, g->Hm1 + pl);
  x->topg.assign(g->topg, g->topg + pl);
  x->diam.assign(g->diam, g->diam + nc);
  x->rhop.assign(g->rhop, g->rhop + nc);
  x->psi.assign(g->psi, g->psi + nc);
  x->sphe.assign(g->sphe, g->sphe + nc);
  x->c.assign((size_t)(nx + 2) * (ny + 2) * (nz + 2) * nc, 0.0);
  x->cdry.assign(pl * (nc + 1), 0.0);
  x->cwet.assign(pl * (nc + 1), 0.0);
  x->cload.assign(pl * (nc + 1), 0.0);
  for (auto* v : {&x->vx, &x->vy, &x->vz, &x->tempe, &x->vptemp, &x->rho, &x->rkhor, &x->rkh1,
                  &x->rkver, &x->divu})
    v->assign(s3, 0.0);
  x->vset.assign(s3 * nc, 0.0);
  x->vset_iters.assign(s3 * nc, 0);
  x->vdep.assign(pl * nc, 0.0);
  for (auto* v : {&x->ustar, &x->zi, &x->rl, &x->znt, &x->prate}) v->assign(pl, 0.0);
  x->ldu.assign(pl, -99.0);
  x->nthreads = nthreads > 0 ? nthreads : 1;
  return x;
}

void orc_ctx_destroy(orc_ctx* x) { delete x; }

/* Threads of the class loop of later steps (1 = the serial build). */
void orc_ctx_set_threads(orc_ctx* x, int nthreads) { x->nthreads = nthreads > 0 ? nthreads : 1; }

/* gfortran MAX/MIN of two reals (see the header) */
static double orc_fmin2(double a, double b) { return (b < a || std::isnan(a)) ? b : a; }

/* Sources/addradialwind.f90:46-166 on the scaled winds of the context */
static void orc_addradialwind(orc_ctx* x) {
  const f3d_gravity_current& gc = x->gc;
  const int nx = x->nx, ny = x->ny, nz = x->nz;
  Dims d{nx, ny, nz};
  const double pi = 3.14159265358979323846;
  const double min_radius =
      (double)1.5f * std::sqrt(x->Hm1[0] * x->dX1 * x->Hm1[0] * x->dX1 + x->dX2 * x->dX2);
  const double wind_center_x = gc.center_x, wind_center_y = gc.center_y;
  const double time_eruption = x->time - gc.beg_time;
  double mass_flow_rate = 0.0;  /* sum(tmrat(1:nsou,1:nc)) in element order */
  for (int ic = 0; ic < x->nc; ++ic)
    for (int is = 0; is < x->nsou; ++is) mass_flow_rate = mass_flow_rate + x->tmrat[(size_t)is + (size_t)x->nsou * ic];
  if (mass_flow_rate <= (double)0.1f) return;
  const double vol_flow_rate = gc.c_flow_rate * std::sqrt(gc.k_entrain) * std::pow(mass_flow_rate, 0.75) /
                               std::pow(gc.brunt_vaisala, 0.625);
  const double c_gravr = 3.0 * gc.lambda_grav * gc.brunt_vaisala * vol_flow_rate / (2.0 * pi);
  double radius_grav = std::pow(c_gravr * (time_eruption * time_eruption), 0.33333);
  radius_grav = fmax2(radius_grav, min_radius);
  const double c_gravu = std::sqrt(2.0 * gc.lambda_grav * gc.brunt_vaisala * vol_flow_rate / (3.0 * pi));
  const double c_grav_factor = 0.75 * c_gravu * std::sqrt(radius_grav);
  const double th_grav = c_gravu / (std::sqrt(radius_grav) * gc.lambda_grav * gc.brunt_vaisala);
  const double h_tot = gc.h_tot;
  const double h_umbr = h_tot / 1.32;
  const double hmin = fmax2(h_umbr - 0.5 * th_grav, 0.5 * h_tot);
  const double hmax = orc_fmin2(h_umbr + 0.5 * th_grav, h_tot);
  int i_wind = (int)((wind_center_x - gc.xorigr) / x->dx);
  int j_wind = (int)((wind_center_y - gc.yorigr) / x->dy);
  i_wind = std::max(1, i_wind);
  j_wind = std::max(1, j_wind);
  int k_wind = 1;
  double store = x->zlayer[nz - 1];
  for (int k = 1; k <= nz; ++k) {
    const double dist = std::fabs(x->zlayer[k - 1] - h_umbr);
    if (dist <= store) { k_wind = k; store = dist; }
  }
  const double wx = x->vx[d.M(i_wind, j_wind, k_wind)], wy = x->vy[d.M(i_wind, j_wind, k_wind)];
  const double v_wind = std::sqrt(wx * wx + wy * wy);
  const double max_radius = 1.7777 * c_gravr / fmax2(v_wind * v_wind, 0.1);
  int kmin = 1;
  store = x->zlayer[nz - 1];
  for (int k = 1; k <= nz; ++k) {
    const double dist = std::fabs(x->zlayer[k - 1] - hmin);
    if (dist <= store) { kmin = k; store = dist; }
  }
  int kmax = nz;
  store = x->zlayer[nz - 1];
  for (int k = 1; k <= nz; ++k) {
    const double dist = std::fabs(x->zlayer[k - 1] - hmax);
    if (dist <= store) { kmax = k; store = dist; }
  }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const double h = x->Hm1[d.P(i, j)];
      const double deltax = x->dX1 * h * ((gc.xorigr + i * x->dx) - wind_center_x) / x->dx;
      const double deltay = x->dX2 * ((gc.yorigr + j * x->dy) - wind_center_y) / x->dy;
      const double radius = std::sqrt(deltax * deltax + deltay * deltay);
      if (std::fabs(radius) <= min_radius) continue;
      if (std::fabs(radius) > max_radius) continue;
      const double rvel = c_grav_factor / radius * (1.0 + radius * radius / (3.0 * (radius_grav * radius_grav)));
      for (int k = kmin; k <= kmax; ++k) {
        x->vx[d.M(i, j, k)] = x->vx[d.M(i, j, k)] + rvel * deltax / radius / h;
        x->vy[d.M(i, j, k)] = x->vy[d.M(i, j, k)] + rvel * deltay / radius;
      }
    }
}

/* Sources/divcorr.f90:21-38 with the budget of the log step */
static void orc_divcorr(orc_ctx* x, double massvol, double massdep) {
  const double compmass = massvol + massdep + x->outmass;
  const double eps = 0.005, eps1 = 10.0 * eps;
  const double corrdiv = fmax2(orc_fmin2((x->erumass - compmass) / (x->erumass), eps1), -eps1);
  Dims d{x->nx, x->ny, x->nz};
  for (int k = 1; k <= x->nz; ++k)
    for (int j = 1; j <= x->ny; ++j)
      for (int i = 1; i <= x->nx; ++i) {
        const double dive = x->divu[d.M(i, j, k)];
        if (std::fabs(dive * x->dt) >= eps)
          for (int ic = 1; ic <= x->nc; ++ic) {
            double& c = x->c[(size_t)(ic - 1) * d.halo() + d.C(i, j, k)];
            c = c * (1.0 + corrdiv);
          }
      }
}

/* --------------------------------------------------------- aggregation */
/* agrsrc.f90:393-440 (water_phase): 0 vapour, 1 water, 2 ice */
static int orc_water_phase(double qv, double P, double T, double wcloud) {
  double w = qv / (1.0 - qv);
  w = w + wcloud;
  const double e = P * w / (w + 0.622);
  double ew = 6.112 * std::exp(17.67 * (T - 273.16) / (T - 273.16 + 243.5));
  ew = 100.0 * ew;
  double ei = -(9.09718 * (273.16 / T - 1.0)) - 3.56654 * std::log10(273.16 / T) +
              0.876793 * (1.0 - T / 273.16) + std::log10(6.1071);
  ei = 100.0 * std::pow(10.0, ei);
  if (e > ew) return T > (double)255.f ? 1 : 2;
  return e > ei ? 2 : 0;
}

/* agrsrc.f90:446-531 (get_gamas) on the scaled winds */
static double orc_get_gamas(const orc_ctx* x, int i, int j, int k) {
  Dims d{x->nx, x->ny, x->nz};
  const int nx = x->nx, ny = x->ny, nz = x->nz;
  const double* vx = x->vx.data();
  const double* vy = x->vy.data();
  const double* vz = x->vz.data();
  const double dXX = x->Hm1[d.P(i, j)] * x->dX1;
  double dudx, dvdx, dwdx, dudy, dvdy, dwdy, dudz, dvdz, dwdz;
  auto V = [&](const double* f, int a, int b, int c) { return f[d.M(a, b, c)]; };
  if (i == 1) {
    dudx = (V(vx, 2, j, k) - V(vx, 1, j, k)) / dXX;
    dvdx = (V(vy, 2, j, k) - V(vy, 1, j, k)) / dXX;
    dwdx = (V(vz, 2, j, k) - V(vz, 1, j, k)) / dXX;
  } else if (i == nx) {
    dudx = (V(vx, nx, j, k) - V(vx, nx - 1, j, k)) / dXX;
    dvdx = (V(vy, nx, j, k) - V(vy, nx - 1, j, k)) / dXX;
    dwdx = (V(vz, nx, j, k) - V(vz, nx - 1, j, k)) / dXX;
  } else {
    dudx = (V(vx, i + 1, j, k) - V(vx, i - 1, j, k)) / (2.0 * dXX);
    dvdx = (V(vy, i + 1, j, k) - V(vy, i - 1, j, k)) / (2.0 * dXX);
    dwdx = (V(vz, i + 1, j, k) - V(vz, i - 1, j, k)) / (2.0 * dXX);
  }
  if (j == 1) {
    dudy = (V(vx, i, 2, k) - V(vx, i, 1, k)) / x->dX2;
    dvdy = (V(vy, i, 2, k) - V(vy, i, 1, k)) / x->dX2;
    dwdy = (V(vz, i, 2, k) - V(vz, i, 1, k)) / x->dX2;
  } else if (j == ny) {
    dudy = (V(vx, i, ny, k) - V(vx, i, ny - 1, k)) / x->dX2;
    dvdy = (V(vy, i, ny, k) - V(vy, i, ny - 1, k)) / x->dX2;
    dwdy = (V(vz, i, ny, k) - V(vz, i, ny - 1, k)) / x->dX2;
  } else {
    dudy = (V(vx, i, j + 1, k) - V(vx, i, j - 1, k)) / (2.0 * x->dX2);
    dvdy = (V(vy, i, j + 1, k) - V(vy, i, j - 1, k)) / (2.0 * x->dX2);
    dwdy = (V(vz, i, j + 1, k) - V(vz, i, j - 1, k)) / (2.0 * x->dX2);
  }
  const double* dz = x->dz.data();
  if (k == 1) {
    dudz = (V(vx, i, j, 2) - V(vx, i, j, 1)) / dz[1];
    dvdz = (V(vy, i, j, 2) - V(vy, i, j, 1)) / dz[1];
    dwdz = (V(vz, i, j, 2) - V(vz, i, j, 1)) / dz[1];
  } else if (k == nz) {
    dudz = (V(vx, i, j, nz) - V(vx, i, j, nz - 1)) / dz[nz - 1];
    dvdz = (V(vy, i, j, nz) - V(vy, i, j, nz - 1)) / dz[nz - 1];
    dwdz = (V(vz, i, j, nz) - V(vz, i, j, nz - 1)) / dz[nz - 1];
  } else {
    dudz = (V(vx, i, j, k + 1) - V(vx, i, j, k - 1)) / (dz[k - 1] + dz[k]);
    dvdz = (V(vy, i, j, k + 1) - V(vy, i, j, k - 1)) / (dz[k - 1] + dz[k]);
    dwdz = (V(vz, i, j, k + 1) - V(vz, i, j, k - 1)) / (dz[k - 1] + dz[k]);
  }
  const double half = (double)0.5f;
  const double S11 = dudx, S12 = half * (dvdx + dudy), S13 = half * (dwdx + dudz);
  const double S21 = S12, S22 = dvdy, S23 = half * (dwdy + dvdz);
  const double S31 = S13, S32 = S23, S33 = dwdz;
  const double epsilon = S11 * S11 + S12 * S12 + S13 * S13 + S21 * S21 + S22 * S22 + S23 * S23 +
                         S31 * S31 + S32 * S32 + S33 * S33;
  return std::sqrt((double)(1.3f * 2.0f) * epsilon);
}

/* agrsrc.f90:95-319 (agrpar), called after a source or meteo update */
static void orc_agrpar(orc_ctx* x) {
  const int nx = x->nx, ny = x->ny, nz = x->nz, np = x->np, ng = x->nc - x->np;
  Dims d{nx, ny, nz};
  const size_t s3 = d.cells();
  const double pi = 3.14159265358979323846;
  const double g = 9.81, kb = 1.38e-23, visc0 = 1.827e-5, Tair0 = (double)291.15f;
  const double Stcr = 1.3, qq = 0.8;
  const double psi3 = 6.0 / pi;
  const double psi4 = psi3 * std::pow(6.0 / pi, 1.0 / 3.0);
  const double* fc = x->fc.data();  /* fc(1:np) at fc[0..np-1] */
  double sumfc = 0.0;
  for (int ic = x->iaggr; ic <= np - 1; ++ic) sumfc = sumfc + fc[ic - 1];
  double sumff = 0.0;
  for (int ic = x->iaggr; ic <= np - 1; ++ic)
    for (int jc = x->iaggr; jc <= np - 1; ++jc) sumff = sumff + fc[ic - 1] * fc[jc - 1];
  double rhopmean = 0.0;
  for (int ic = x->iaggr; ic <= np - 1; ++ic) rhopmean = rhopmean + fc[ic - 1] * x->rhop[ic - 1];
  rhopmean = rhopmean / sumfc;
  for (int iz = 1; iz <= nz; ++iz)
    for (int iy = 1; iy <= ny; ++iy)
      for (int ix = 1; ix <= nx; ++ix) {
        const size_t m = d.M(ix, iy, iz);
        const double tp = x->tplume[m];
        const double T = tp > 0.0 ? tp : x->tempe[m];
        const double rhoa = x->rho[m];
        const double visc = visc0 * ((Tair0 + 120.0) / (T + 120.0)) * std::pow(T / Tair0, 1.5);
        const double viscl = 2.414e-5 * std::pow(10.0, 247.7 / (T - 140.0));
        int phase;  /* 0 vapour (or the plume's truncated 'vapou'), 1 water, 2 ice */
        if (tp > 0.0) {
          phase = T < 255 ? 2 : (T < 373 ? 1 : 0);
        } else {
          double wcloud = ng > 0 ? x->c[(size_t)np * d.halo() + d.C(ix, iy, iz)] / x->Hm1[d.P(ix, iy)]
                                 : (double)0.f;
          wcloud = wcloud / rhoa;
          phase = orc_water_phase(x->qv[m], x->pres[m], T, wcloud);
        }
        x->Abagr[m] = -(4.0 * kb * T / (3.0 * visc));
        const double gamas = orc_get_gamas(x, ix, iy, iz);
        x->Asagr[m] = -(2.0 * gamas * psi3 / 3.0);
        x->Adagr[m] = -(pi * (rhopmean - rhoa) * g * psi4 / (48.0 * visc));
        double al = 0.0;
        if (phase == 2) {
          al = 0.09;
        } else if (phase == 1) {
          for (int ic = x->iaggr; ic <= np - 1; ++ic)
            for (int jc = x->iaggr; jc <= np - 1; ++jc) {
              const double di = x->diam[ic - 1], dj = x->diam[jc - 1];
              const double vij = std::fabs(x->vset[(size_t)(ic - 1) * s3 + m] - x->vset[(size_t)(jc - 1) * s3 + m]) -
                                 x->Abagr[m] / (2.0 * pi * di * dj) - x->Asagr[m] * di * dj / (4.0 * pi);
              const double w = fc[ic - 1] * fc[jc - 1] / sumff;
              const double Stij = 8.0 * rhopmean * vij * di * dj / (9.0 * viscl * (di + dj));
              double alfa = 1.0 + std::pow(Stij / Stcr, qq);
              alfa = 1.0 / alfa;
              al = al + w * alfa;
            }
        }
        x->Alagr[m] = al;
      }
  /* agrsrc.f90:295-301: the settling velocity of class iaggr */
  for (size_t m = 0; m < s3; ++m)
    x->vset[(size_t)(x->iaggr - 1) * s3 + m] = x->vset_factor * x->vset[(size_t)(x->iaggr - 1) * s3 + m];
}

/* agrsrc.f90:1-91 (agrsrc) and setsrc.f90:37-76: the aggregation source of
 * one aggregation step added to c, and Maggr */
static void orc_agrsrc(orc_ctx* x) {
  const int nx = x->nx, ny = x->ny, nz = x->nz, np = x->np, iaggr = x->iaggr;
  Dims d{nx, ny, nz};
  const double pi = 3.14159265358979323846;
  const double ka = 1.0, expb = 2.0, exps = 2.0 - (3.0 / x->Df), expd = 2.0 - (4.0 / x->Df);
  std::vector<double> Ni(np + 1, 0.0), d3(np + 1, 0.0), tarat(np + 1, 0.0);
  double sumNi = 0.0;
  for (int ic = iaggr; ic <= np - 1; ++ic) {
    const double di = x->diam[ic - 1];
    d3[ic] = pi * x->rhop[ic - 1] * di * di * di;
    Ni[ic] = ka * std::pow(x->diam[np - 1] / di, x->Df);
    sumNi = sumNi + Ni[ic];
  }
  const double fac = (double)x->ndtagr * x->dt;
  for (int iz = 1; iz <= nz; ++iz) {
    const double dzeta = 0.5 * (x->dz[iz - 1] + x->dz[iz]);
    for (int iy = 1; iy <= ny; ++iy)
      for (int ix = 1; ix <= nx; ++ix) {
        const size_t q = d.C(ix, iy, iz), m = d.M(ix, iy, iz);
        const double h = x->Hm1[d.P(ix, iy)];
        double ntot = 0.0, fi = 0.0;
        for (int ic = iaggr; ic <= np - 1; ++ic) {
          const double c = x->c[(size_t)(ic - 1) * d.halo() + q];
          fi = fi + c / x->rhop[ic - 1];
          ntot = ntot + 6.0 * c / d3[ic];
        }
        ntot = ntot / h;
        fi = fi / h;
        double dntot = x->Abagr[m] * std::pow(ntot, expb) +
                       x->Asagr[m] * std::pow(ntot, exps) * std::pow(fi, 3.0 / x->Df) +
                       x->Adagr[m] * std::pow(ntot, expd) * std::pow(fi, 4.0 / x->Df);
        dntot = x->Alagr[m] * dntot;
        tarat[np] = 0.0;
        for (int ic = iaggr; ic <= np - 1; ++ic) {
          const double c = x->c[(size_t)(ic - 1) * d.halo() + q];
          const double dnj = dntot * Ni[ic] / sumNi;
          tarat[ic] = dnj * d3[ic] / 6.0;
          if (c + x->dt * tarat[ic] < 0.0) tarat[ic] = -c / x->dt;
          tarat[np] = tarat[np] - tarat[ic];
        }
        for (int ic = iaggr; ic <= np; ++ic) {
          double& c = x->c[(size_t)(ic - 1) * d.halo() + q];
          c = c + fac * tarat[ic];
        }
        x->Maggr[m] = x->Maggr[m] + fac * tarat[np] * h * x->dX1 * x->dX2 * dzeta;
      }
  }
}

/* the aggregation model switched on: Df, ndtagr and the .grn fractions
 * fc(1:np); iaggr as readat.f90:400-409 */
int orc_set_aggregation(orc_ctx* x, double Df, int ndtagr, const double* fc) {
  if (!fc) {
    x->agg_on = 0;
    return 0;
  }
  const int np = x->np;
  if (np < 2 || ndtagr < 1) return 1;
  int iaggr = 0;
  for (int ic = np - 1; ic >= 1; --ic)
    if (x->diam[np - 1] > x->diam[ic - 1]) iaggr = ic;
  if (iaggr == 0) iaggr = np - 1;
  x->iaggr = iaggr;
  x->Df = Df;
  x->ndtagr = ndtagr;
  x->fc.assign(fc, fc + np);
  const size_t s3 = (size_t)x->nx * x->ny * x->nz;
  for (auto* v : {&x->qv, &x->pres, &x->tplume, &x->wplume, &x->Alagr, &x->Abagr, &x->Asagr, &x->Adagr,
                  &x->Maggr})
    v->assign(s3, 0.0);
  x->agg_on = 1;
  x->agr_ipass = 0;
  return 0;
}

/* QV and P (nx,ny,nz) of the DBS snapshot of the next meteo update */
void orc_aggregation_met(orc_ctx* x, const double* qv, const double* p) {
  const size_t s3 = (size_t)x->nx * x->ny * x->nz;
  std::copy(qv, qv + s3, x->qv.begin());
  std::copy(p, p + s3, x->pres.begin());
}

/* settemplume (source.f90:89-149): plume temperature and water rate of
 * the current source interval at n cells (1-based indices) */
void orc_aggregation_plume(orc_ctx* x, int n, const int* ix, const int* iy, const int* iz,
                           const double* t, const double* w) {
  Dims d{x->nx, x->ny, x->nz};
  std::fill(x->tplume.begin(), x->tplume.end(), 0.0);
  std::fill(x->wplume.begin(), x->wplume.end(), 0.0);
  for (int q = 0; q < n; ++q) {
    x->tplume[d.M(ix[q], iy[q], iz[q])] = t[q];
    x->wplume[d.M(ix[q], iy[q], iz[q])] = w[q];
  }
}

void orc_download_maggr(orc_ctx* x, double* maggr) {
  if (x->agg_on) std::copy(x->Maggr.begin(), x->Maggr.end(), maggr);
}

void orc_set_gravity_current(orc_ctx* x, const f3d_gravity_current* gc) {
  if (gc) {
    x->gc = *gc;
    x->gc_on = 1;
  } else {
    x->gc_on = 0;
  }
}

/* Sources/meteo.f90:19-149 for one snapshot (reamet.f90:146,153 included). */
int orc_meteo(orc_ctx* x, const double* u, const double* v, const double* w,
              const double* t, const double* tp, const double* rho,
              const double* ust, const double* pblh, const double* rmol,
              const double* znt, const double* prate, const double* ldu) {
  const int nx = x->nx, ny = x->ny, nz = x->nz;
  const size_t s3 = (size_t)nx * ny * nz, pl = (size_t)nx * ny;
  std::copy(u, u + s3, x->vx.begin());
  std::copy(v, v + s3, x->vy.begin());
  std::copy(w, w + s3, x->vz.begin());
  std::copy(t, t + s3, x->tempe.begin());
  std::copy(tp, tp + s3, x->vptemp.begin());
  std::copy(rho, rho + s3, x->rho.begin());
  std::copy(ust, ust + pl, x->ustar.begin());
  std::copy(pblh, pblh + pl, x->zi.begin());
  std::copy(rmol, rmol + pl, x->rl.begin());
  std::copy(znt, znt + pl, x->znt.begin());
  if (ldu) std::copy(ldu, ldu + pl, x->ldu.begin());
  if (x->wetdep) {
    for (size_t p = 0; p < pl; ++p) x->prate[p] = prate[p] * 3600.0;
  }
  for (size_t p = 0; p < pl; ++p) x->vz[p] = 0.0;  // vz(:,:,1) = 0
  orc_kappa3(nx, ny, nz, x->modkv, x->modkh, x->coord, x->rkv0, x->rkh0, x->Csh, x->dX1, x->dX2,
             x->dx, x->dy, x->dz.data(), x->zlayer.data(), x->Hm1.data(), x->vx.data(), x->vy.data(),
             x->vptemp.data(), x->ustar.data(), x->zi.data(), x->rl.data(), x->rkver.data(),
             x->rkhor.data());
  if (orc_setvset(nx, ny, nz, x->nc, x->np, x->modv, x->diam.data(), x->rhop.data(), x->psi.data(),
                  x->sphe.data(), x->tempe.data(), x->rho.data(), x->aggregate, x->vset_factor,
                  x->vset.data(), &x->cd, x->vset_iters.data()) != 0)
    return 3;
  orc_setvdrydep(nx, ny, x->nc, x->diam.data(), x->zlayer.data(), x->ldu.data(), x->rl.data(),
                 x->znt.data(), x->ustar.data(), x->tempe.data(), x->rho.data(), x->vdep.data());
  orc_meteo_scale(nx, ny, nz, x->coord, x->dX1, x->dX2, x->dz.data(), x->Hm1.data(), x->topg.data(),
                  x->vx.data(), x->vy.data(), x->vz.data(), x->rho.data(), x->rkhor.data(),
                  x->rkh1.data(), nullptr);
  if (x->gc_on) orc_addradialwind(x);  // meteo.f90:140
  orc_setdivu(nx, ny, nz, x->dX1, x->dX2, x->dz.data(), x->Hm1.data(), x->vx.data(), x->vy.data(),
              x->vz.data(), x->divu.data());
  orc_finddt(nx, ny, nz, x->nc, x->dX1, x->dX2, x->dz.data(), x->vx.data(), x->vy.data(),
             x->vz.data(), x->vset.data(), x->rkh1.data(), x->rkhor.data(), x->rkver.data(),
             x->safety, &x->dt, &x->dtc);
  x->have_met = 1;
  if (x->agg_on) x->agr_due = 1;  /* Fall3d.f90:94-96 */
  return 0;
}

/* Sources/source.f90:132-185 after reasrc.f90:26-80. */
int orc_source(orc_ctx* x, int nsou, const int* isrc, const int* jsrc,
               const int* ksrc, const double* tmrat) {
  const int nc = x->nc, np = x->np;
  for (int is = 0; is < nsou; ++is)
    if (isrc[is] > x->nx || jsrc[is] > x->ny || ksrc[is] > x->nz || isrc[is] < 1 || jsrc[is] < 1)
      return 6;
  x->nsou = nsou;
  x->isrc.assign(isrc, isrc + nsou);
  x->jsrc.assign(jsrc, jsrc + nsou);
  x->ksrc.assign(ksrc, ksrc + nsou);
  x->tmrat.assign(tmrat, tmrat + (size_t)nsou * nc);
  double fr = 0.0;  // SUM over the (nsou,nc) array in element order
  for (int ic = 0; ic < nc; ++ic)
    for (int is = 0; is < nsou; ++is) fr = fr + x->tmrat[(size_t)is + (size_t)nsou * ic];
  x->flowrate = fr;
  (void)np;
  for (int is = 0; is < nsou; ++is) {
    const double h = x->Hm1[(size_t)(isrc[is] - 1) + (size_t)x->nx * (jsrc[is] - 1)];
    for (int ic = 0; ic < nc; ++ic) x->tmrat[(size_t)is + (size_t)nsou * ic] *= h;
  }
  if (x->agg_on) x->agr_due = 1;  /* Fall3d.f90:84-86 */
  return 0;
}

/* Sources/sizloop.f90:31-83 (serial: ic_loc=1, nc_loc=nc, iz_loc=1, nz_loc=nz).
 * Classes are independent, so they may run on several threads. */
static void orc_sizloop(orc_ctx* x) {
  const int nx = x->nx, ny = x->ny, nz = x->nz, nc = x->nc;
  const size_t h = (size_t)(nx + 2) * (ny + 2) * (nz + 2), s3 = (size_t)nx * ny * nz, pl = (size_t)nx * ny;
  const double dt = x->dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(x->nthreads)
#endif
  for (int ic = 1; ic <= nc; ++ic) {
    double* cc = x->c.data() + (size_t)(ic - 1) * h;
    const double* vs = x->vset.data() + (size_t)(ic - 1) * s3;
    const double* vd = x->vdep.data() + (size_t)(ic - 1) * pl;
    orc_setbcc(cc, nx, ny, nz, nz, 1, x->vx.data(), x->vy.data(), x->vz.data(), vs, vd,
               x->rkver.data(), x->dz.data());
    orc_advctzc(cc, nx, ny, nz, nz, 1, x->vz.data(), vs, x->dz.data(), dt);
    if (x->iiter % 2 == 0) {
      orc_advctx(cc, nx, ny, nz, nz, 1, x->vx.data(), x->dX1, dt);
      orc_advcty(cc, nx, ny, nz, nz, 1, x->vy.data(), x->dX2, dt);
    } else {
      orc_advcty(cc, nx, ny, nz, nz, 1, x->vy.data(), x->dX2, dt);
      orc_advctx(cc, nx, ny, nz, nz, 1, x->vx.data(), x->dX1, dt);
    }
    orc_diffz(cc, nx, ny, nz, nz, 1, x->dz.data(), dt, x->rkver.data(), x->rho.data());
    if (x->iiter % 2 == 0) {
      orc_diffx(cc, nx, ny, nz, nz, 1, x->dX1, dt, x->rkh1.data(), x->rho.data());
      orc_diffy(cc, nx, ny, nz, nz, 1, x->dX2, dt, x->rkhor.data(), x->rho.data());
    } else {
      orc_diffy(cc, nx, ny, nz, nz, 1, x->dX2, dt, x->rkhor.data(), x->rho.data());
      orc_diffx(cc, nx, ny, nz, nz, 1, x->dX1, dt, x->rkh1.data(), x->rho.data());
    }
    if (x->wetdep && ic <= x->np)
      orc_wetdep(cc, x->cwet.data(), ic, nx, ny, nz, nz, 1,
                 dt, x->diam.data(), x->zlayer.data(), x->dz.data(), x->zi.data(), x->prate.data());
    orc_accum(cc, x->cdry.data(), ic, nx, ny, nz, nz, 1, dt, vs, vd);
  }
  orc_clip(x->c.data(), nx, ny, nz, 1, nc);
  orc_cmass2d(x->c.data(), x->vx.data(), x->vy.data(), x->vz.data(), x->vset.data(), nx, ny, nz, nc, 1,
              nc, 1, nz, x->dX1, x->dX2, x->dz.data(), dt, &x->outmass);
}

/* Sources/Fall3d.f90:112-117 */
int orc_step(orc_ctx* x) {
  if (!x->have_met) return 4;
  if (x->agg_on && x->agr_due) {  /* Fall3d.f90:101-110, after the updates */
    orc_agrpar(x);
    x->agr_due = 0;
  }
  x->time = x->time + x->dt;
  x->iiter = x->iiter + 1;
  x->erumass = x->erumass + x->flowrate * x->dt;
  int rc = orc_setsrc(x->c.data(), x->nx, x->ny, x->nz, x->nc, x->nsou, x->isrc.data(), x->jsrc.data(),
                      x->ksrc.data(), x->tmrat.data(), x->dz.data(), x->zlayer.data(), x->Hm1.data(),
                      x->dX1, x->dX2, x->dt);
  if (rc) return rc;
  if (x->agg_on) {  /* setsrc.f90:37-76 */
    x->agr_ipass = x->agr_ipass + 1;
    if (x->agr_ipass % x->ndtagr == 0) orc_agrsrc(x);
  }
  orc_sizloop(x);
  return 0;
}

/* endstep.f90:59-60 then writim.f90:18 */
void orc_budget(orc_ctx* x, double* out4) {
  orc_getc0(x->cdry.data(), x->cwet.data(), x->cload.data(), x->nx, x->ny, x->nc, x->np);
  orc_cmass3d(x->c.data(), x->cload.data(), x->cdry.data(), x->cwet.data(), x->nx, x->ny, x->nz, x->nc,
              x->dX1, x->dX2, x->dz.data(), out4);
}

void orc_get_state(const orc_ctx* x, int* iiter, double* s7) {
  *iiter = x->iiter;
  s7[0] = x->time; s7[1] = x->dt; s7[2] = x->dtc; s7[3] = x->erumass;
  s7[4] = x->outmass; s7[5] = x->flowrate; s7[6] = x->cd;
}

void orc_set_time(orc_ctx* x, double time, int iiter) { x->time = time; x->iiter = iiter; }

void orc_download(const orc_ctx* x, double* c, double* cdry, double* cwet,
                  double* vset, double* vdep) {
  if (c) std::copy(x->c.begin(), x->c.end(), c);
  if (cdry) std::copy(x->cdry.begin(), x->cdry.end(), cdry);
  if (cwet) std::copy(x->cwet.begin(), x->cwet.end(), cwet);
  if (vset) std::copy(x->vset.begin(), x->vset.end(), vset);
  if (vdep) std::copy(x->vdep.begin(), x->vdep.end(), vdep);
}

void orc_upload_state(orc_ctx* x, const double* c, const double* cdry,
                      const double* cwet, double erumass, double outmass, double cd) {
  if (c) std::copy(c, c + x->c.size(), x->c.begin());
  if (cdry) std::copy(cdry, cdry + x->cdry.size(), x->cdry.begin());
  if (cwet) std::copy(cwet, cwet + x->cwet.size(), x->cwet.begin());
  x->erumass = erumass; x->outmass = outmass; x->cd = cd;
}

void orc_download_coeffs(const orc_ctx* x, double* vx, double* vy, double* vz,
                         double* rho, double* rkhor, double* rkh1, double* rkver) {
  if (vx) std::copy(x->vx.begin(), x->vx.end(), vx);
  if (vy) std::copy(x->vy.begin(), x->vy.end(), vy);
  if (vz) std::copy(x->vz.begin(), x->vz.end(), vz);
  if (rho) std::copy(x->rho.begin(), x->rho.end(), rho);
  if (rkhor) std::copy(x->rkhor.begin(), x->rkhor.end(), rkhor);
  if (rkh1) std::copy(x->rkh1.begin(), x->rkh1.end(), rkh1);
  if (rkver) std::copy(x->rkver.begin(), x->rkver.end(), rkver);
}

void orc_download_iters(const orc_ctx* x, int* iters) {
  std::copy(x->vset_iters.begin(), x->vset_iters.end(), iters);
}

void orc_outputs_ctx(orc_ctx* x, double* load, double* col_mass, double* c_grnd) {
  orc_getc0(x->cdry.data(), x->cwet.data(), x->cload.data(), x->nx, x->ny, x->nc, x->np);
  orc_outputs(x->c.data(), x->cload.data(), x->nx, x->ny, x->nz, x->np, x->dz.data(), x->Hm1.data(),
              load, col_mass, c_grnd);
}

void orc_run_reset(orc_ctx* x) { x->run_started = 0; }

/* Sources/Fall3d.f90:73-121 with libMaster interval selection
 * (get_dbs_value_plane.f90:100-114, get_source_nsrc.f90:41-59). */
int orc_run(orc_ctx* x, const f3d_met_series* met, const f3d_src_series* src,
            double beg_time, double end_time, int max_steps,
            f3d_log_record* log, int log_cap, int* nlog) {
  const int nx = x->nx, ny = x->ny, nz = x->nz, nc = x->nc;
  const size_t s3 = (size_t)nx * ny * nz, pl = (size_t)nx * ny;
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
    go_on = x->time < end_time;  // resuming a run that already reached end_time
    // a later end time than the last call's: the updates it switched off are due again
    if (x->meteo_time < end_time) x->meteotime = 1;
    if (x->source_time < end_time) x->sourcetime = 1;
  }
  int steps = 0;
  while (go_on) {
    if (x->source_time <= x->time) {
      if (x->sourcetime) {
        const int ts = (int)x->time;
        int found = -1;
        size_t off = 0, off_found = 0;
        for (int it = 0; it < src->nint; ++it) {
          if (found < 0 && ts >= src->t1[it] && ts < src->t2[it]) { found = it; off_found = off; }
          off += (size_t)src->nsou[it];
        }
        if (found < 0) return 6;
        size_t roff = 0;
        for (int it = 0; it < found; ++it) roff += (size_t)src->nsou[it] * nc;
        const int rc = orc_source(x, src->nsou[found], src->isrc + off_found, src->jsrc + off_found,
                                  src->ksrc + off_found, src->tmrat + roff);
        if (rc) return rc;
        if (x->agg_on && src->nplume) {  /* settemplume at the end of source (source.f90:82) */
          size_t po = 0;
          for (int it = 0; it < found; ++it) po += (size_t)src->nplume[it];
          orc_aggregation_plume(x, src->nplume[found], src->pix + po, src->piy + po, src->piz + po,
                                src->ptemp + po, src->pwater + po);
        }
        x->source_time = (double)src->t2[found];
      }
      if (x->source_time >= end_time) x->sourcetime = 0;
    }
    if (x->meteo_time <= x->time) {
      if (x->meteotime) {
        const int ts = (int)(met->time_lag + x->time);
        const int nt = met->nt;
        if (ts < met->times[0] || ts > met->times[nt - 1]) return 6;
        int itime = nt - 1;
        int endsec = met->times[nt - 1];
        for (int it = 0; it < nt - 1; ++it)
          if (ts >= met->times[it] && ts < met->times[it + 1]) { itime = it; endsec = met->times[it + 1]; }
        const size_t o3 = (size_t)itime * s3, o2 = (size_t)itime * pl;
        if (x->agg_on && met->qv && met->p) orc_aggregation_met(x, met->qv + o3, met->p + o3);
        const int rc = orc_meteo(x, met->u + o3, met->v + o3, met->w + o3, met->t + o3, met->tp + o3,
                                 met->rho + o3, met->ust + o2, met->pblh + o2, met->rmol + o2,
                                 met->znt + o2, met->prate ? met->prate + o2 : nullptr, met->ldu);
        if (rc) return rc;
        x->meteo_time = (double)endsec - met->time_lag;
      }
      if (x->meteo_time >= end_time) x->meteotime = 0;
    }
    const int rc = orc_step(x);
    if (rc) return rc;
    ++steps;
    // endstep.f90:51: log every 10 minutes of simulated time
    if (x->iiter == 1 || std::fmod(x->time, 600.0) <= x->dt) {
      const bool rec = log && nlog && *nlog < log_cap;
      if (rec || x->gc_on) {
        double b[4];
        orc_budget(x, b);
        if (rec) {
          f3d_log_record& r = log[(*nlog)++];
          r.iiter = x->iiter; r.time = x->time; r.dt = x->dt; r.dtc = x->dtc;
          r.massvol = b[0]; r.massdep = b[1]; r.massdry = b[2]; r.masswet = b[3];
          r.outmass = x->outmass; r.erumass = x->erumass;
        }
        if (x->gc_on) orc_divcorr(x, b[0], b[1]);  /* endstep.f90:71 */
      }
    }
    if (x->time >= end_time) go_on = false;
    if (max_steps > 0 && steps >= max_steps) go_on = false;
  }
  return 0;
}

}  // extern "C"

// f3d_transport.cu -- one kernel per reference transport routine.
//
// Each kernel restates one subroutine of Sources/ in the reference's own
// operation order (compiled with --fmad=false, so the binary64 instances
// round every operation as the Fortran does) and is batched over classes:
// classes are independent within a step (Sources/sizloop.f90:31-72), so
// running a sweep for all classes before the next sweep is the same
// computation as the reference's class-by-class loop.
//
// Thread layout (x fastest everywhere, so every warp touches consecutive
// addresses of the (nx+2)(ny+2)(nz+2) class block):
//  * column kernels (advctzc, diffz, wetdep): one thread per (i,j) column,
//    marching k with a register window;
//  * x-line kernels (advctx, diffx): one block per x line, taking it through
//    every class, the line staged in shared memory;
//  * y-line kernels (advcty, diffy): one block per tile of TI adjacent y
//    lines at one k, through every class, the tile staged in shared memory,
//    rows of TI consecutive x addresses per load.
// A block owns whole lines, so the in-place update cannot race with a
// neighbour block's reads.
//
// GB300 issues binary64 arithmetic at 1/64 of the binary32 rate, and a
// binary64 division costs many times a multiply-add, so the sweeps keep
// the reference's results bit for bit while issuing fewer binary64
// operations: the class-independent factors of a line are formed once for
// all classes, values shared by neighbouring cells are formed once, the
// limiter's sign and minimum logic runs on the bit patterns, and divisions
// by a per-launch or per-meteo-update divisor use its reciprocal with
// Markstein's correction (div_rn_recip, f3d_common.cuh).
#include <algorithm>
#include <cstdio>

#include "f3d_internal.h"

namespace f3d {

// ------------------------------------------------------------- setbcc
// Sources/setbcc.f90:19-109.  One thread per ghost cell written; reads
// only interior cells, so all writes are independent.
template <class T>
__global__ void k_setbcc(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vx,
                         const T* vy, const T* vz, const T* vset, long long vstride,
                         const T* vdep, long long dstride, const T* rkver, const T* dz) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  T* cc = c + (long long)blockIdx.y * cstride;
  const T* vs = vset + (long long)blockIdx.y * vstride;
  const T* vd = vdep + (long long)blockIdx.y * dstride;
  const bool bot = (iz_loc == 1), top = (iz_loc + nz_loc - 1 == nz);
  const long long nb = bot ? (long long)nx * ny : (long long)(nx + 2) * (ny + 2);
  const long long nt = top ? (long long)nx * ny : (long long)(nx + 2) * (ny + 2);
  const long long nxf = 2LL * ny * nz_loc, nyf = 2LL * nx * nz_loc;
  const long long total = nb + nt + nxf + nyf + 8;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long u = t;
    if (u < nb) {  // bottom plane (setbcc.f90:19-33)
      if (bot) {
        const int i = (int)(u % nx) + 1, j = (int)(u / nx) + 1;
        if ((vz[d.M(i, j, 1)] + vs[d.M(i, j, 1)]) >= T(0))
          cc[d.C(i, j, 0)] = T(0);
        else
          cc[d.C(i, j, 0)] = cc[d.C(i, j, 1)] * (T(1) + dz[0] * vd[d.P(i, j)] / rkver[d.M(i, j, 1)]);
      } else {
        const int i = (int)(u % (nx + 2)), j = (int)(u / (nx + 2));
        cc[d.C(i, j, 0)] = T(0);
      }
      continue;
    }
    u -= nb;
    if (u < nt) {  // top plane (setbcc.f90:37-49)
      if (top) {
        const int i = (int)(u % nx) + 1, j = (int)(u / nx) + 1;
        if ((vz[d.M(i, j, nz)] + vs[d.M(i, j, nz)]) <= T(0))
          cc[d.C(i, j, nz + 1)] = T(0);
        else
          cc[d.C(i, j, nz + 1)] = cc[d.C(i, j, nz)];
      } else {
        const int i = (int)(u % (nx + 2)), j = (int)(u / (nx + 2));
        cc[d.C(i, j, nz + 1)] = T(0);
      }
      continue;
    }
    u -= nt;
    if (u < nxf) {  // x faces (setbcc.f90:53-66)
      const int side = (int)(u % 2);
      const long long r = u / 2;
      const int j = (int)(r % ny) + 1, k = (int)(r / ny) + iz_loc;
      if (side == 0)
        cc[d.C(0, j, k)] = (vx[d.M(1, j, k)] >= T(0)) ? T(0) : cc[d.C(1, j, k)];
      else
        cc[d.C(nx + 1, j, k)] = (vx[d.M(nx, j, k)] <= T(0)) ? T(0) : cc[d.C(nx, j, k)];
      continue;
    }
    u -= nxf;
    if (u < nyf) {  // y faces (setbcc.f90:70-83)
      const int side = (int)(u % 2);
      const long long r = u / 2;
      const int i = (int)(r % nx) + 1, k = (int)(r / nx) + iz_loc;
      if (side == 0)
        cc[d.C(i, 0, k)] = (vy[d.M(i, 1, k)] >= T(0)) ? T(0) : cc[d.C(i, 1, k)];
      else
        cc[d.C(i, ny + 1, k)] = (vy[d.M(i, ny, k)] <= T(0)) ? T(0) : cc[d.C(i, ny, k)];
      continue;
    }
    u -= nyf;
    // corners (setbcc.f90:87-109)
    const int q = (int)u;
    const int ci = (q & 1) ? nx + 1 : 0, cj = (q & 2) ? ny + 1 : 0;
    const int si = (q & 1) ? nx : 1, sj = (q & 2) ? ny : 1;
    if (q < 4) {
      cc[d.C(ci, cj, 0)] = bot ? cc[d.C(si, sj, 1)] : T(0);
    } else {
      cc[d.C(ci, cj, nz + 1)] = top ? cc[d.C(si, sj, nz)] : T(0);
    }
  }
}

template <class T>
void launch_setbcc(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vx,
                   const T* vy, const T* vz, const T* vset, long long vstride, const T* vdep,
                   long long dstride, const T* rkver, const T* dz, int ncls, cudaStream_t s) {
  const long long total = 2LL * (d.nx + 2) * (d.ny + 2) + 2LL * (d.nx + d.ny) * nz_loc + 8;
  const int bs = 256;
  const int nb = (int)std::min<long long>((total + bs - 1) / bs, 4096);
  k_setbcc<T><<<dim3(nb, ncls), bs, 0, s>>>(c, cstride, d, nz_loc, iz_loc, vx, vy, vz, vset,
                                              vstride, vdep, dstride, rkver, dz);
  count_launch();
}

// ------------------------------------------------------------ advctzc
// Sources/advctzc.f90:28-81.  work(k,1), work(k,2) of the reference are
// evaluated from the ORIGINAL column, so a register window of originals
// (c(k-1), c(k), c(k+1), c(k+2)) carries them as k advances.
template <class T>
struct ZTab {  // per-level constants of advctzc.f90:34-36 (IEEE, as on the host)
  T dzz, dzk, dzk_1, hdzm1;  // hdzm1 = (dt*0.5)*dz(k-1), the first factors of work(k,2)
};

// work(k,1), work(k,2) (advctzc.f90:37-46) at a level with c0 = c(k),
// cp = c(k+1), vk = vk(k), vk_1 = vk(k-1), given the previous level's
// product pm = vk(k-1)*c(k-1) and difference dm = c(k)-c(k-1); returns this
// level's p0 = vk(k)*c(k) and d0 = c(k+1)-c(k) for the next one (the
// reference forms both twice, with the same operations).
template <class T>
__device__ __forceinline__ void adv_z_work(T c0, T cp, T vk, T vk_1, T pm, T dm, const ZTab<T>& z, T dt,
                                           T& w1, T& w2, T& p0, T& d0) {
  const T vk_12 = T(0.5) * (vk + vk_1);
  p0 = vk * c0;
  w1 = dt * (p0 - pm) * z.dzz;
  d0 = cp - c0;
  const T sigma = minmod_ref(d0 * z.dzk, dm * z.dzk_1);
  const T Crk = absd(vk_12) * dt * z.dzk_1;
  w2 = z.hdzm1 * (T(1) - Crk) * sigma * absd(vk_12) * z.dzz;
}

template <class T>
__global__ void k_advctzc(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vz,
                          const T* vset, long long vstride, const T* dz, T dt) {
  extern __shared__ unsigned char smem_raw[];
  ZTab<T>* tab = reinterpret_cast<ZTab<T>*>(smem_raw);
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  for (int k = threadIdx.x + 1; k <= nz; k += blockDim.x) {
    tab[k].dzz = T(2) / (dz[k] + dz[k - 1]);
    tab[k].dzk = T(1) / dz[k];
    tab[k].dzk_1 = T(1) / dz[k - 1];
    tab[k].hdzm1 = dt * T(0.5) * dz[k - 1];
  }
  __syncthreads();
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= (long long)nx * ny) return;
  const int i = (int)(col % nx) + 1, j = (int)(col / nx) + 1;
  T* cc = c + (long long)blockIdx.y * cstride;
  const T* vs = vset + (long long)blockIdx.y * vstride;
  const long long cb = d.C(i, j, 0), cs = (long long)(nx + 2) * (ny + 2);
  const long long mb = d.M(i, j, 1), ms = (long long)nx * ny;
  auto VK = [&](int k) { return vz[mb + (k - 1) * ms] + vs[mb + (k - 1) * ms]; };
  auto CO = [&](int k) { return cc[cb + k * cs]; };
  const T dznz = T(1) / dz[nz];
  const int kb = iz_loc, ke = iz_loc + nz_loc - 1;
  T c_m1 = CO(kb - 1), c_0 = CO(kb), c_p1 = CO(kb + 1);
  T vk_0 = VK(kb), vk_m1 = VK(kb > 1 ? kb - 1 : 1);
  T w1_k, w2_k, w2_km, pk, dk;
  adv_z_work(c_0, c_p1, vk_0, vk_m1, vk_m1 * c_m1, c_0 - c_m1, tab[kb], dt, w1_k, w2_k, pk, dk);
  if (kb == 1) {
    w2_km = w2_k;
  } else {
    T w1_dummy, p_dummy, d_dummy;
    const T c_m2 = CO(kb - 2), vk_m2 = VK(kb - 1 > 1 ? kb - 2 : 1);
    adv_z_work(c_m1, c_0, vk_m1, vk_m2, vk_m2 * c_m2, c_m1 - c_m2, tab[kb - 1], dt, w1_dummy, w2_km,
               p_dummy, d_dummy);
  }
  for (int k = kb; k <= ke; ++k) {
    T w1_n, w2_n, c_p2 = T(0), vk_p1 = T(0);
    if (k + 1 <= nz) {
      c_p2 = CO(k + 2);
      vk_p1 = VK(k + 1);
      adv_z_work(c_p1, c_p2, vk_p1, vk_0, pk, dk, tab[k + 1], dt, w1_n, w2_n, pk, dk);
    } else {
      w1_n = dt * vk_0 * (c_p1 - c_0) * dznz;  // work(nz+1,1), advctzc.f90:58-64
      w2_n = w2_k;                             // kmin = nz
    }
    T cn;
    if (gt0(vk_0))
      cn = c_0 - w1_k - (w2_k - w2_km);
    else
      cn = c_0 - w1_n - (w2_n - w2_k);
    cc[cb + k * cs] = cn;
    w2_km = w2_k;
    w2_k = w2_n;
    w1_k = w1_n;
    c_m1 = c_0;
    c_0 = c_p1;
    c_p1 = c_p2;
    vk_m1 = vk_0;
    vk_0 = vk_p1;
  }
  (void)c_m1;
  (void)vk_m1;
}

template <class T>
void launch_advctzc(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vz,
                    const T* vset, long long vstride, const T* dz, T dt, int ncls,
                    cudaStream_t s) {
  const int bs = 128;
  const long long cols = (long long)d.nx * d.ny;
  const size_t sm = sizeof(ZTab<T>) * (d.nz + 1);
  k_advctzc<T><<<dim3((unsigned)((cols + bs - 1) / bs), ncls), bs, sm, s>>>(
      c, cstride, d, nz_loc, iz_loc, vz, vset, vstride, dz, dt);
  count_launch();
}

// ------------------------------------------------------ advctx / advcty
// Sources/advctx.f90:24-56 and Sources/advcty.f90:24-55 on staged lines.
// A block takes one line (advctx) or a tile of lines (advcty) through every
// class: the class-independent factors of the line are formed once,
//   a(q) = |0.5*(v(q)+v(q-1))|,  b(q) = (dt*0.5)*(1 - auxv*a(q)),
// so that work(q,2) = dt*0.5*(1-Cri)*sigma*|v_12| is (b(q)*sigma)*a(q),
// the reference's product left to right; then per class the line's
// concentrations are staged with the products v(q)*c(q) and differences
// c(q+1)-c(q) that neighbouring positions share (each formed once, as the
// reference forms it), work(q,1), work(q,2) formed and the line updated.
template <class T>
struct AdvLine {  // a line's staged arrays at stride st
  T *v, *a, *b, *cl, *w1, *w2;
  T *p, *dc;  // p(q) = v(q)*c(q) (1..n), dc(q) = c(q+1)-c(q) (0..n): shared by neighbours
};

// Stages position q (0..n+1) of a class's line: c, and the products and
// differences that work(q,1) and the limiter of neighbouring positions share.
// c0 = c(q), c1 = c(q+1) (read only for q <= n).  SH: stage p and dc (the
// x sweep); the y sweep's tiles of lines keep to six arrays, whose shared
// memory lets more blocks share an SM, and form them per position.
template <bool SH, class T>
__device__ __forceinline__ void adv_line_stage(const AdvLine<T>& L, int q, int n, int st, T c0, T c1) {
  L.cl[q * st] = c0;
  if constexpr (SH) {
    if (q >= 1 && q <= n) L.p[q * st] = L.v[q * st] * c0;
    if (q <= n) L.dc[q * st] = c1 - c0;
  }
}

template <class T>
__device__ __forceinline__ void adv_line_coef(T vq, T vq_1, T auxv, T dth, T& a, T& b) {
  a = absd(T(0.5) * (vq + vq_1));
  b = dth * (T(1) - auxv * a);
}

// work(q,1), work(q,2) of position q (1..n), or work(n+1,1) (advctx.f90:46)
template <bool SH, class T>
__device__ __forceinline__ void adv_line_work(const AdvLine<T>& L, int q, int n, int st, T dx, T rdx, T auxv) {
  auto C = [&](int i) { return L.cl[i * st]; };
  if (q > n) {
    L.w1[(n + 1) * st] = auxv * L.v[n * st] * (SH ? L.dc[n * st] : C(n + 1) - C(n));
    return;
  }
  const T vq = L.v[q * st], vq_1 = L.v[(q > 1 ? q - 1 : 1) * st];
  if constexpr (SH) {
    // vq_1*c(q-1) is the left neighbour's product, or v(1)*c(0) at q = 1
    const T pl = q > 1 ? L.p[(q - 1) * st] : vq_1 * C(0);
    L.w1[q * st] = auxv * (L.p[q * st] - pl);
  } else {
    L.w1[q * st] = auxv * (vq * C(q) - vq_1 * C(q - 1));
  }
  const T sigma = SH ? minmod_div(L.dc[q * st], L.dc[(q - 1) * st], dx, rdx)
                     : minmod_div(C(q + 1) - C(q), C(q) - C(q - 1), dx, rdx);
  L.w2[q * st] = L.b[q * st] * sigma * L.a[q * st];
}

template <class T>
__device__ __forceinline__ T adv_line_update(const AdvLine<T>& L, int q, int n, int st) {
  const T cq = L.cl[q * st], vq = L.v[q * st];
  if (gt0(vq)) return cq - L.w1[q * st] - (L.w2[q * st] - L.w2[(q > 1 ? q - 1 : 1) * st]);
  return cq - L.w1[(q + 1) * st] - (L.w2[(q < n ? q + 1 : n) * st] - L.w2[q * st]);
}

// One block per x line (j,k) through classes 0..ncls-1; threads stride over i.
template <class T>
__global__ void k_advctx(T* c, long long cstride, int ncls, Dims d, int iz_loc, const T* vx, T dx, T dt) {
  extern __shared__ unsigned char smem_raw[];
  const int nx = d.nx, ny = d.ny, n2 = nx + 2;
  T* base = reinterpret_cast<T*>(smem_raw);
  const AdvLine<T> L{base,          base + n2,     base + 2 * n2, base + 3 * n2,
                     base + 4 * n2, base + 5 * n2, base + 6 * n2, base + 7 * n2};
  const int j = blockIdx.x % ny + 1, k = blockIdx.x / ny + iz_loc;
  const T* vl = vx + d.M(1, j, k) - 1;  // vl[i] = vx(i,j,k)
  const T auxv = dt / dx, dth = dt * T(0.5), rdx = T(1) / dx;
  for (int q = threadIdx.x + 1; q <= nx; q += blockDim.x) {
    const T vq = vl[q];
    L.v[q] = vq;
    adv_line_coef(vq, vl[q > 1 ? q - 1 : 1], auxv, dth, L.a[q], L.b[q]);
  }
  for (int ic = 0; ic < ncls; ++ic) {
    T* cc = c + (long long)ic * cstride + d.C(0, j, k);
    __syncthreads();  // the coefficients are staged; the previous class is done with cl, w1, w2
    for (int q = threadIdx.x; q <= nx + 1; q += blockDim.x)
      adv_line_stage<true>(L, q, nx, 1, cc[q], q <= nx ? cc[q + 1] : T(0));
    __syncthreads();
    for (int q = threadIdx.x + 1; q <= nx + 1; q += blockDim.x) adv_line_work<true>(L, q, nx, 1, dx, rdx, auxv);
    __syncthreads();
    for (int q = threadIdx.x + 1; q <= nx; q += blockDim.x) cc[q] = adv_line_update(L, q, nx, 1);
  }
}

// One block per tile of TI adjacent y lines (i0..i0+TI-1) at one k, through
// classes 0..ncls-1.
template <class T>
__global__ void k_advcty(T* c, long long cstride, int ncls, Dims d, int iz_loc, const T* vy, T dy, T dt) {
  extern __shared__ unsigned char smem_raw[];
  const int nx = d.nx, ny = d.ny, TI = blockDim.x;
  const int ntile = (nx + TI - 1) / TI;
  const int i0 = (blockIdx.x % ntile) * TI + 1, k = blockIdx.x / ntile + iz_loc;
  const int tx = threadIdx.x, ty = threadIdx.y, TJ = blockDim.y;
  const int i = i0 + tx;
  const bool act = i <= nx;
  const size_t n2 = (size_t)(ny + 2) * TI;
  T* base = reinterpret_cast<T*>(smem_raw) + tx;  // [q][TI], this thread's line
  const AdvLine<T> L{base, base + n2, base + 2 * n2, base + 3 * n2, base + 4 * n2, base + 5 * n2, nullptr, nullptr};
  const long long rowstride = nx + 2;
  const long long cbase = d.C(act ? i : nx, 0, k);
  const long long vb = d.M(act ? i : nx, 1, k) - nx;  // vb + q*nx = vy(i,q,k)
  const T auxv = dt / dy, dth = dt * T(0.5), rdy = T(1) / dy;
  if (act)
    for (int q = ty + 1; q <= ny; q += TJ) {
      const T vq = vy[vb + (long long)q * nx];
      L.v[q * TI] = vq;
      adv_line_coef(vq, vy[vb + (long long)(q > 1 ? q - 1 : 1) * nx], auxv, dth, L.a[q * TI], L.b[q * TI]);
    }
  for (int ic = 0; ic < ncls; ++ic) {
    T* cc = c + (long long)ic * cstride;
    __syncthreads();
    if (act)
      for (int q = ty; q <= ny + 1; q += TJ)
        adv_line_stage<false>(L, q, ny, TI, cc[cbase + q * rowstride], T(0));
    __syncthreads();
    if (act)
      for (int q = ty + 1; q <= ny + 1; q += TJ) adv_line_work<false>(L, q, ny, TI, dy, rdy, auxv);
    __syncthreads();
    if (act)
      for (int q = ty + 1; q <= ny; q += TJ) cc[cbase + q * rowstride] = adv_line_update(L, q, ny, TI);
  }
}

static int pick_ti(int nline, size_t elem, int arrays) {
  // Widest tile whose staging fits in 96 KB (at least 4 lines when they
  // fit in the 227 KB a block may have).
  for (int ti = 32; ti >= 4; ti >>= 1)
    if ((size_t)arrays * (nline + 2) * ti * elem <= 96 * 1024) return ti;
  for (int ti = 4; ti > 1; ti >>= 1)
    if ((size_t)arrays * (nline + 2) * ti * elem <= 227 * 1024) return ti;
  return 1;
}

static void set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <class T>
void launch_advctx(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vx, T dx,
                   T dt, int ncls, cudaStream_t s) {
  const size_t sm = 8 * (size_t)(d.nx + 2) * sizeof(T);
  set_smem((const void*)k_advctx<T>, sm);
  const int bs = d.nx >= 256 ? 256 : 128;
  k_advctx<T><<<dim3(d.ny * nz_loc), bs, sm, s>>>(c, cstride, ncls, d, iz_loc, vx, dx, dt);
  count_launch();
}

template <class T>
void launch_advcty(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* vy, T dy,
                   T dt, int ncls, cudaStream_t s) {
  const int TI = pick_ti(d.ny, sizeof(T), 6);
  const int TJ = 256 / TI;
  const size_t sm = 6 * (size_t)(d.ny + 2) * TI * sizeof(T);
  set_smem((const void*)k_advcty<T>, sm);
  const int ntile = (d.nx + TI - 1) / TI;
  k_advcty<T><<<dim3(ntile * nz_loc), dim3(TI, TJ), sm, s>>>(c, cstride, ncls, d, iz_loc, vy, dy, dt);
  count_launch();
}

// -------------------------------------------------------------- diffz
// Sources/diffz.f90:22-62, one thread per column.  The four kinds of face
// flux (bottom/top non-averaged, interior averaged) are evaluated exactly as
// written; an interior face shared by cells k and k+1 is the same
// expression in both, so it is computed once and carried.
// c/rho of diffz.f90: with lr = RN(1/rho) precomputed, the binary64 form
// forms RN(c/rho) by div_rn_recip (same bits, no division).
template <class T>
__device__ __forceinline__ T c_over_rho(T c, T r, const T* lr, long long m) {
  (void)lr;
  (void)m;
  return c / r;
}
__device__ __forceinline__ double c_over_rho(double c, double r, const double* lr, long long m) {
  return lr ? div_rn_recip(c, r, lr[m]) : div_ieee(c, r);
}

template <class T>
__global__ void k_diffz(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* dz, T dt,
                        const T* rkver, const T* rho, const T* rksz, const T* lrz) {
  extern __shared__ unsigned char smem_raw[];
  T* l_dz = reinterpret_cast<T*>(smem_raw);  // 0..nz
  T* l_dzdz = l_dz + (d.nz + 1);             // 1..nz
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  for (int k = threadIdx.x; k <= nz; k += blockDim.x) {
    l_dz[k] = T(1) / dz[k];
    if (k >= 1) l_dzdz[k] = T(2) / (dz[k] + dz[k - 1]);
  }
  __syncthreads();
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= (long long)nx * ny) return;
  const int i = (int)(col % nx) + 1, j = (int)(col / nx) + 1;
  T* cc = c + (long long)blockIdx.y * cstride;
  const long long cb = d.C(i, j, 0), cs = (long long)(nx + 2) * (ny + 2);
  const long long mb = d.M(i, j, 1), ms = (long long)nx * ny;
  auto C = [&](int k) { return cc[cb + k * cs]; };
  auto R = [&](int k) { return rho[mb + (k - 1) * ms]; };
  auto K = [&](int k) { return rkver[mb + (k - 1) * ms]; };
  const int kb = iz_loc, ke = iz_loc + nz_loc - 1;
  // Interior face flux between k and k+1 (diffz.f90:42-45):
  //   0.5*(rho(k+1)K(k+1) + rho(k)K(k)) * (c(k+1)/rho(k+1) - c(k)/rho(k)) * l_dz(k)
  // rksz, when given, holds that face's 0.5*(...) for the meteo update
  auto face = [&](int k, T qk, T qk1, T rk, T rk1, T Kk, T Kk1) {
    const T rks = rksz ? rksz[mb + (k - 1) * ms] : T(0.5) * (rk1 * Kk1 + rk * Kk);
    return rks * (qk1 - qk) * l_dz[k];
  };
  // Window of originals: c(k-1), c(k), c(k+1); rho, K at k-1, k, k+1.
  T cm = C(kb - 1), c0 = C(kb), cp = C(kb + 1);
  T rm = (kb > 1) ? R(kb - 1) : T(0), r0 = R(kb), rp = (kb < nz) ? R(kb + 1) : T(0);
  T Km = (kb > 1) ? K(kb - 1) : T(0), K0 = K(kb), Kp = (kb < nz) ? K(kb + 1) : T(0);
  auto Q = [&](T cv, T rv, int kk) { return c_over_rho(cv, rv, lrz, mb + (long long)(kk - 1) * ms); };
  T qm = (kb > 1) ? Q(cm, rm, kb - 1) : T(0), q0 = Q(c0, r0, kb), qp = (kb < nz) ? Q(cp, rp, kb + 1) : T(0);
  // gradb of the first interior cell needs the face (kb-1, kb).
  T fprev = (kb >= 3) ? face(kb - 1, qm, q0, rm, r0, Km, K0) : T(0);
  for (int k = kb; k <= ke; ++k) {
    T work;
    if (k == 1) {  // bottom (diffz.f90:32-39); kb == 1 here
      const T rkst = K(2) * R(2);
      const T rksb = K(1) * R(1);
      const T gradt = rkst * ((cp / rp) - (c0 / r0)) * l_dz[1];
      T gradb = rksb * ((c0 / r0) - (cm / r0)) * l_dz[0];
      gradb = fmax2(T(0), gradb);
      work = dt * (gradt - gradb) * l_dzdz[1];
      fprev = face(1, q0, qp, r0, rp, K0, Kp);  // interior face (1,2) for k = 2
    } else if (k == nz) {  // top (diffz.f90:51-58)
      const T rkst = K0 * r0;
      const T rksb = Km * rm;
      T gradt = rkst * ((cp / r0) - (c0 / r0)) * l_dz[nz];
      const T gradb = rksb * ((c0 / r0) - (cm / rm)) * l_dz[nz - 1];
      gradt = fmin2(T(0), gradt);
      work = dt * (gradt - gradb) * l_dz[nz];
    } else {  // interior (diffz.f90:41-47)
      if (k == 2 && kb == 2) fprev = face(1, qm, q0, rm, r0, Km, K0);
      const T gradt = face(k, q0, qp, r0, rp, K0, Kp);
      const T gradb = fprev;
      work = dt * (gradt - gradb) * l_dzdz[k];
      fprev = gradt;
    }
    cc[cb + k * cs] = c0 + work;
    // advance the window (originals)
    if (k < ke) {
      cm = c0; c0 = cp; cp = C(k + 2);
      rm = r0; r0 = rp; rp = (k + 2 <= nz) ? R(k + 2) : T(0);
      Km = K0; K0 = Kp; Kp = (k + 2 <= nz) ? K(k + 2) : T(0);
      qm = q0; q0 = qp; qp = (k + 2 <= nz) ? Q(cp, rp, k + 2) : T(0);
    }
  }
}

template <class T>
void launch_diffz(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, const T* dz, T dt,
                  const T* rkver, const T* rho, const T* rksz, const T* lrz, int ncls, cudaStream_t s) {
  const int bs = 128;
  const long long cols = (long long)d.nx * d.ny;
  const size_t sm = 2 * sizeof(T) * (d.nz + 1);
  k_diffz<T><<<dim3((unsigned)((cols + bs - 1) / bs), ncls), bs, sm, s>>>(c, cstride, d, nz_loc,
                                                                         iz_loc, dz, dt, rkver, rho,
                                                                         rksz, lrz);
  count_launch();
}

// ------------------------------------------------------- diffx / diffy
// Sources/diffx.f90:20-55, Sources/diffy.f90:20-55.  A line is staged with
// what its cells share: c (0..n+1), cl = c*(1/rho) (1..n), the averaged face
// coefficient fk(q) = 0.5*(pk(q+1)+pk(q)) (1..n-1), pk = rkh*rho, and the
// interior face flux ff(q) = fk(q)*(cl(q+1)-cl(q)) (1..n-1), each formed once
// with the reference's operations, so every cell reads the bits it would
// have computed itself.  The end cells (non-averaged faces, ghost products)
// fetch their own factors.

// 1/rho and rkh*rho of one position: precomputed (lrp, pkp) or formed here.
template <class T>
__device__ __forceinline__ void diff_factors(const T* lrp, const T* pkp, const T* rho, const T* rkh,
                                             long long m, T& l, T& p) {
  if (lrp) {
    l = lrp[m];
    p = pkp[m];
  } else {
    const T r = rho[m];
    l = T(1) / r;
    p = rkh[m] * r;
  }
}

template <class T>
struct DiffSrc {  // the line's factors in global memory: position q at m1 + (q-1)*ms
  const T *lrp, *pkp, *rho, *rkh;
  long long m1, ms;
  __device__ void at(int q, T& l, T& p) const { diff_factors(lrp, pkp, rho, rkh, m1 + (q - 1) * ms, l, p); }
};

// ff(q) = fk(q)*(cl(q+1) - cl(q)): the interior face flux, gradr of cell q
// and gradl of cell q+1 (diffx.f90:34-40), formed once per face.
template <class T>
__device__ __forceinline__ T diff_line_cell(int q, int n, const T* cv, const T* cl, const T* ff,
                                            const DiffSrc<T>& src, int st, T dtdx2) {
  // st: stride between consecutive line positions in the staged arrays
  auto Cq = [&](int a) { return cv[a * st]; };
  auto Q = [&](int a) { return cl[a * st]; };
  T gradr, gradl;
  if (q == 1) {
    T l1, p1, l2, p2;
    src.at(1, l1, p1);
    src.at(2, l2, p2);
    gradr = p2 * (Q(2) - Q(1));
    gradl = p1 * (Q(1) - Cq(0) * l1);
    gradl = fmax2(T(0), gradl);
  } else if (q == n) {
    T ln, pn, lm, pm;
    src.at(n, ln, pn);
    src.at(n - 1, lm, pm);
    gradr = pn * (Cq(n + 1) * ln - Q(n));
    gradl = pm * (Q(n) - Q(n - 1));
    gradr = fmin2(T(0), gradr);
  } else {
    gradr = ff[q * st];
    gradl = ff[(q - 1) * st];
  }
  return Cq(q) + dtdx2 * (gradr - gradl);
}

// Stages the class-independent factors of position q (1..n) of a line:
// 1/rho(q) and, below n, fk(q).
template <class T>
__device__ __forceinline__ void diff_stage(int q, int n, const DiffSrc<T>& src, T* lq, T* fkq) {
  T l, p;
  src.at(q, l, p);
  *lq = l;
  if (q < n) {
    T l1, p1;
    src.at(q + 1, l1, p1);
    *fkq = T(0.5) * (p1 + p);
  }
}

// One block per x line (j,k) through classes 0..ncls-1.
template <class T>
__global__ void k_diffx(T* c, long long cstride, int ncls, Dims d, int iz_loc, T dx, T dt, const T* rkh,
                        const T* rho, const T* lrp, const T* pkp) {
  extern __shared__ unsigned char smem_raw[];
  const int nx = d.nx, ny = d.ny;
  T* lr = reinterpret_cast<T*>(smem_raw);
  T* fk = lr + (nx + 2);
  T* cv = fk + (nx + 2);
  T* cl = cv + (nx + 2);
  T* ff = cl + (nx + 2);
  const int j = blockIdx.x % ny + 1, k = blockIdx.x / ny + iz_loc;
  const DiffSrc<T> src{lrp, pkp, rho, rkh, d.M(1, j, k), 1};
  for (int q = threadIdx.x + 1; q <= nx; q += blockDim.x) diff_stage(q, nx, src, lr + q, fk + q);
  const T dtdx2 = dt / (dx * dx);
  for (int ic = 0; ic < ncls; ++ic) {
    T* cc = c + (long long)ic * cstride + d.C(0, j, k);
    __syncthreads();  // factors staged; the previous class is done with cv, cl
    for (int q = threadIdx.x; q <= nx + 1; q += blockDim.x) {
      const T v = cc[q];
      cv[q] = v;
      if (q >= 1 && q <= nx) cl[q] = v * lr[q];
    }
    __syncthreads();
    for (int q = threadIdx.x + 1; q < nx; q += blockDim.x) ff[q] = fk[q] * (cl[q + 1] - cl[q]);
    __syncthreads();
    for (int q = threadIdx.x + 1; q <= nx; q += blockDim.x)
      cc[q] = diff_line_cell(q, nx, cv, cl, ff, src, 1, dtdx2);
  }
}

// One block per tile of TI adjacent y lines at one k, through classes 0..ncls-1.
template <class T>
__global__ void k_diffy(T* c, long long cstride, int ncls, Dims d, int iz_loc, T dy, T dt, const T* rkh,
                        const T* rho, const T* lrp, const T* pkp) {
  extern __shared__ unsigned char smem_raw[];
  const int nx = d.nx, ny = d.ny, TI = blockDim.x;
  const int ntile = (nx + TI - 1) / TI;
  const int i0 = (blockIdx.x % ntile) * TI + 1, k = blockIdx.x / ntile + iz_loc;
  const int tx = threadIdx.x, ty = threadIdx.y, TJ = blockDim.y;
  const int i = i0 + tx;
  const bool act = i <= nx;
  const size_t n2 = (size_t)(ny + 2) * TI;
  T* lr = reinterpret_cast<T*>(smem_raw) + tx;  // [q][TI], this thread's line
  T* fk = lr + n2;
  T* cv = fk + n2;
  T* cl = cv + n2;
  T* ff = cl + n2;
  const long long rowstride = nx + 2;
  const long long base = d.C(act ? i : nx, 0, k);
  const DiffSrc<T> src{lrp, pkp, rho, rkh, d.M(act ? i : nx, 1, k), nx};
  if (act)
    for (int q = ty + 1; q <= ny; q += TJ) diff_stage(q, ny, src, lr + q * TI, fk + q * TI);
  const T dtdy2 = dt / (dy * dy);
  for (int ic = 0; ic < ncls; ++ic) {
    T* cc = c + (long long)ic * cstride;
    __syncthreads();
    if (act)
      for (int q = ty; q <= ny + 1; q += TJ) {
        const T v = cc[base + q * rowstride];
        cv[q * TI] = v;
        if (q >= 1 && q <= ny) cl[q * TI] = v * lr[q * TI];
      }
    __syncthreads();
    if (act)
      for (int q = ty + 1; q < ny; q += TJ) ff[q * TI] = fk[q * TI] * (cl[(q + 1) * TI] - cl[q * TI]);
    __syncthreads();
    if (act)
      for (int q = ty + 1; q <= ny; q += TJ)
        cc[base + q * rowstride] = diff_line_cell(q, ny, cv, cl, ff, src, TI, dtdy2);
  }
}

template <class T>
void launch_diffx(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, T dx, T dt,
                  const T* rkh, const T* rho, const T* lr, const T* pk, int ncls, cudaStream_t s) {
  const size_t sm = 5 * (size_t)(d.nx + 2) * sizeof(T);
  set_smem((const void*)k_diffx<T>, sm);
  const int bs = d.nx >= 256 ? 256 : 128;
  k_diffx<T><<<dim3(d.ny * nz_loc), bs, sm, s>>>(c, cstride, ncls, d, iz_loc, dx, dt, rkh, rho, lr, pk);
  count_launch();
}

template <class T>
void launch_diffy(T* c, long long cstride, Dims d, int nz_loc, int iz_loc, T dy, T dt,
                  const T* rkh, const T* rho, const T* lr, const T* pk, int ncls, cudaStream_t s) {
  // at most ~48 KB per block, so that several blocks share an SM
  int TI = pick_ti(d.ny, sizeof(T), 5);
  while (TI > 4 && 5 * (size_t)(d.ny + 2) * TI * sizeof(T) > 48 * 1024) TI >>= 1;
  const int TJ = 256 / TI;
  const size_t sm = 5 * (size_t)(d.ny + 2) * TI * sizeof(T);
  set_smem((const void*)k_diffy<T>, sm);
  const int ntile = (d.nx + TI - 1) / TI;
  k_diffy<T><<<dim3(ntile * nz_loc), dim3(TI, TJ), sm, s>>>(c, cstride, ncls, d, iz_loc, dy, dt,
                                                             rkh, rho, lr, pk);
  count_launch();
}

// The class-independent factors of diffx/diffy for one meteo update, with
// the sweeps' own operations (so the sweeps read the same bits).
// rksz(i,j,k) = 0.5*(rho(k+1)*rkver(k+1) + rho(k)*rkver(k)), the face
// (k, k+1) coefficient of diffz.f90:43 for k < nz.
__global__ void k_diff_coeffs(Dims d, const double* rho, const double* rkh1, const double* rkhor,
                              const double* rkver, double* lr, double* pkx, double* pky,
                              double* rksz) {
  const long long n = d.cells(), pl = d.plane(), top = n - pl;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    const double r = rho[m];
    lr[m] = 1.0 / r;
    pkx[m] = rkh1[m] * r;
    pky[m] = rkhor[m] * r;
    rksz[m] = m < top ? 0.5 * (rho[m + pl] * rkver[m + pl] + r * rkver[m]) : 0.0;
  }
}

void launch_diff_coeffs(Dims d, const double* rho, const double* rkh1, const double* rkhor,
                        const double* rkver, double* lr, double* pkx, double* pky, double* rksz,
                        cudaStream_t s) {
  const int nb = (int)std::min<long long>((d.cells() + 255) / 256, 152LL * 16);
  k_diff_coeffs<<<nb, 256, 0, s>>>(d, rho, rkh1, rkhor, rkver, lr, pkx, pky, rksz);
  count_launch();
}

// ------------------------------------------------------------- wetdep
// Sources/wetdep.f90:28-50.  lambda and the deposit are binary64 in every
// form (the wet deposit is a ground-deposit accumulation).
template <class T>
__global__ void k_wetdep(T* c, long long cstride, double* cwet, int ic0, Dims d, int nz_loc,
                         int iz_loc, double dt, const double* diam, const double* zlayer,
                         const double* dz, const double* zi, const double* prate,
                         const double* lam2d) {
  const int ic = ic0 + blockIdx.y;  // 0-based class
  double diam_max = 100.0;
  diam_max = diam_max * 1e-6;
  if (diam[ic] > diam_max) return;
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= (long long)d.nx * d.ny) return;
  const int i = (int)(col % d.nx) + 1, j = (int)(col / d.nx) + 1;
  const double a = 8.4e-5, b = 0.79;
  const long long p = d.P(i, j);
  // lam2d: the same lambda formed once per meteo update for all classes
  const double lambda = lam2d ? lam2d[p] : fmin2(dt * a * pow(prate[p], b), 1.0);
  T* cc = c + (long long)blockIdx.y * cstride;
  double* cw = cwet + (long long)(ic + 1) * d.plane();
  const double z = zi[p];
  double acc = cw[p];
  for (int k = iz_loc; k <= iz_loc + nz_loc - 1; ++k) {
    if (zlayer[k - 1] <= z) {
      const long long q = d.C(i, j, k);
      const double ck = (double)cc[q];
      acc = acc + dz[k] * lambda * ck;
      cc[q] = (T)(ck * (1.0 - lambda));
    }
  }
  cw[p] = acc;
}

template <class T>
void launch_wetdep(T* c, long long cstride, double* cwet, int ic0, Dims d, int nz_loc, int iz_loc,
                   double dt, const double* diam, const double* zlayer, const double* dz,
                   const double* zi, const double* prate, const double* lam2d, int ncls, cudaStream_t s) {
  if (ncls <= 0) return;
  const int bs = 128;
  const long long cols = (long long)d.nx * d.ny;
  k_wetdep<T><<<dim3((unsigned)((cols + bs - 1) / bs), ncls), bs, 0, s>>>(
      c, cstride, cwet, ic0, d, nz_loc, iz_loc, dt, diam, zlayer, dz, zi, prate, lam2d);
  count_launch();
}

// -------------------------------------------------------------- accum
// Sources/accum.f90:17-25 (binary64).
template <class T>
__global__ void k_accum(const T* c, long long cstride, double* cdry, int ic0, Dims d, double dt,
                        const double* vset, long long vstride, const double* vdep,
                        long long dstride) {
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= (long long)d.nx * d.ny) return;
  const int i = (int)(col % d.nx) + 1, j = (int)(col / d.nx) + 1;
  const int ic = ic0 + blockIdx.y;
  const T* cc = c + (long long)blockIdx.y * cstride;
  const double* vs = vset + (long long)blockIdx.y * vstride;
  const double* vd = vdep + (long long)blockIdx.y * dstride;
  double* cd = cdry + (long long)(ic + 1) * d.plane();
  const long long p = d.P(i, j);
  cd[p] = cd[p] - dt * (double)cc[d.C(i, j, 1)] * fmin2(0.0, vs[d.M(i, j, 1)] + vd[p]);
}

template <class T>
void launch_accum(const T* c, long long cstride, double* cdry, int ic0, Dims d, int iz_loc,
                  double dt, const double* vset, long long vstride, const double* vdep,
                  long long dstride, int ncls, cudaStream_t s) {
  if (iz_loc != 1 || ncls <= 0) return;
  const int bs = 128;
  const long long cols = (long long)d.nx * d.ny;
  k_accum<T><<<dim3((unsigned)((cols + bs - 1) / bs), ncls), bs, 0, s>>>(
      c, cstride, cdry, ic0, d, dt, vset, vstride, vdep, dstride);
  count_launch();
}

// --------------------------------------------------------------- clip
// Sources/sizloop.f90:77-78: c = MAX(0,c) over the whole halo array.
template <class T>
__global__ void k_clip(T* c, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    c[q] = fmax2(T(0), c[q]);
}

template <class T>
void launch_clip(T* c, long long n, cudaStream_t s) {
  const int bs = 256;
  const int nb = (int)std::min<long long>((n + bs - 1) / bs, 152LL * 16);
  k_clip<T><<<nb, bs, 0, s>>>(c, n);
  count_launch();
}

// ------------------------------------------------------------- setsrc
// Sources/setsrc.f90:20-35.  One thread per (first source of a cell, class)
// walks the sources of that cell in file order (source_links), so several
// sources in one cell add in the reference's order.
constexpr int SRC_B = 128;

template <class T>
__device__ __forceinline__ void setsrc_chain(T* cc, int s0, int ic, Dims d, int nsou, const int* isrc,
                                             const int* jsrc, const int* ksrc, const int* link,
                                             const double* tmrat, const double* dz,
                                             const double* zlayer, const double* Hm1, double dX1,
                                             double dX2, double dt) {
  const int i = isrc[s0], j = jsrc[s0], k = ksrc[s0];
  double dzeta;
  if (k == 1)
    dzeta = 0.5 * dz[k] + zlayer[k - 1];
  else
    dzeta = 0.5 * (dz[k - 1] + dz[k]);
  const double vol0 = Hm1[d.P(i, j)] * dX1 * dX2 * dzeta;
  const long long q = d.C(i, j, k);
  double v = (double)cc[q];
  for (int is = s0; is >= 0; is = link[is])
    v = (double)(T)(v + dt * tmrat[is + (long long)nsou * ic] / vol0);
  cc[q] = (T)v;
}

template <class T>
__global__ void k_setsrc(T* c, long long cstride, Dims d, int nsou, const int* isrc, const int* jsrc,
                         const int* ksrc, const int* link, const double* tmrat, const double* dz,
                         const double* zlayer, const double* Hm1, double dX1, double dX2,
                         double dt) {
  const int s0 = blockIdx.x * SRC_B + threadIdx.x, ic = blockIdx.y;
  if (s0 >= nsou || !link[nsou + s0]) return;
  setsrc_chain<T>(c + (long long)ic * cstride, s0, ic, d, nsou, isrc, jsrc, ksrc, link, tmrat, dz,
                  zlayer, Hm1, dX1, dX2, dt);
}

template <class T>
void launch_setsrc(T* c, long long cstride, Dims d, int nc, int nsou, const int* isrc,
                   const int* jsrc, const int* ksrc, const int* link, const double* tmrat,
                   const double* dz, const double* zlayer, const double* Hm1, double dX1, double dX2,
                   double dt, cudaStream_t s) {
  if (nsou <= 0 || nc <= 0) return;
  k_setsrc<T><<<dim3((nsou + SRC_B - 1) / SRC_B, nc), SRC_B, 0, s>>>(
      c, cstride, d, nsou, isrc, jsrc, ksrc, link, tmrat, dz, zlayer, Hm1, dX1, dX2, dt);
  count_launch();
}

// Batched form: scenario blockIdx.y, class blockIdx.z; the state before
// the step is in c_a after an even number of batch steps, else in c_b.
__global__ void k_setsrc_batch(const BatchAux* tab, const int* bstep) {
  const BatchAux& b = tab[blockIdx.y];
  const int s0 = blockIdx.x * SRC_B + threadIdx.x, ic = blockIdx.z;
  if (ic >= b.nc || s0 >= b.nsou || !b.link[b.nsou + s0]) return;
  float* cc = ((bstep[blockIdx.y] & 1) ? b.c_b : b.c_a) + (long long)ic * b.cstride;
  setsrc_chain<float>(cc, s0, ic, b.d, b.nsou, b.isrc, b.jsrc, b.ksrc, b.link, b.tmrat, b.dz, b.zlayer,
                      b.Hm1, b.dX1, b.dX2, b.dt);
}

void launch_setsrc_batch(const BatchAux* tab, const int* bstep, int nscen, int max_nc, int max_nsou,
                         cudaStream_t s) {
  if (nscen <= 0 || max_nsou <= 0 || max_nc <= 0) return;
  k_setsrc_batch<<<dim3((max_nsou + SRC_B - 1) / SRC_B, nscen, max_nc), SRC_B, 0, s>>>(tab, bstep);
  count_launch();
}

__global__ void k_batch_advance(int* bstep, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) bstep[q] = bstep[q] + 1;
}

void launch_batch_advance(int* bstep, int nscen, cudaStream_t s) {
  if (nscen <= 0) return;
  k_batch_advance<<<(nscen + 127) / 128, 128, 0, s>>>(bstep, nscen);
  count_launch();
}

// ------------------------------------------------------- conversions
__global__ void k_d2f(float* dst, const double* src, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    dst[q] = (float)src[q];
}
__global__ void k_f2d(double* dst, const float* src, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    dst[q] = (double)src[q];
}
void launch_d2f(float* dst, const double* src, long long n, cudaStream_t s) {
  if (n <= 0) return;
  const int nb = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  k_d2f<<<nb, 256, 0, s>>>(dst, src, n);
  count_launch();
}
void launch_f2d(double* dst, const float* src, long long n, cudaStream_t s) {
  if (n <= 0) return;
  const int nb = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  k_f2d<<<nb, 256, 0, s>>>(dst, src, n);
  count_launch();
}

// ---------------------------------------------------- instantiations
#define F3D_INST(T)                                                                              \
  template void launch_setbcc<T>(T*, long long, Dims, int, int, const T*, const T*, const T*,    \
                                 const T*, long long, const T*, long long, const T*, const T*,   \
                                 int, cudaStream_t);                                             \
  template void launch_advctzc<T>(T*, long long, Dims, int, int, const T*, const T*, long long,  \
                                  const T*, T, int, cudaStream_t);                               \
  template void launch_advctx<T>(T*, long long, Dims, int, int, const T*, T, T, int,             \
                                 cudaStream_t);                                                  \
  template void launch_advcty<T>(T*, long long, Dims, int, int, const T*, T, T, int,             \
                                 cudaStream_t);                                                  \
  template void launch_diffz<T>(T*, long long, Dims, int, int, const T*, T, const T*, const T*,  \
                                const T*, const T*,                                              \
                                int, cudaStream_t);                                              \
  template void launch_diffx<T>(T*, long long, Dims, int, int, T, T, const T*, const T*,        \
                                const T*, const T*, int, cudaStream_t);                          \
  template void launch_diffy<T>(T*, long long, Dims, int, int, T, T, const T*, const T*,        \
                                const T*, const T*, int, cudaStream_t);                          \
  template void launch_wetdep<T>(T*, long long, double*, int, Dims, int, int, double,            \
                                 const double*, const double*, const double*, const double*,     \
                                 const double*, const double*, int, cudaStream_t);               \
  template void launch_accum<T>(const T*, long long, double*, int, Dims, int, double,            \
                                const double*, long long, const double*, long long, int,         \
                                cudaStream_t);                                                   \
  template void launch_clip<T>(T*, long long, cudaStream_t);                                     \
  template void launch_setsrc<T>(T*, long long, Dims, int, int, const int*, const int*,          \
                                 const int*, const int*, const double*, const double*,           \
                                 const double*, const double*, double, double, double,           \
                                 cudaStream_t);

F3D_INST(double)
F3D_INST(float)

}  // namespace f3d

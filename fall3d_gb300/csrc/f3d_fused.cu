// f3d_fused.cu -- the precision form's whole transport step in one kernel.
//
// One CTA owns an output tile of TX x TY columns of one class and marches
// up the column, so each concentration is read from and written to HBM
// once per step.  The sweeps of Sources/sizloop.f90:35-71 are pipelined per
// horizontal plane k:
//
//   A  setbcc + advctzc     per column in registers (window of the
//                           original column c(k-1..k+2), work(k), work(k+1))
//   B  advctx / advcty      on shared-memory planes, order by parity of iiter
//   D  diffz (plane k-1)    per column in registers (needs plane k of B)
//   E  diffx / diffy        on shared-memory planes, order by parity of iiter
//   F  wetdep, accum, clip  per output cell; store
//
// The x/y sweeps need +-2 cells (advection) then +-1 (diffusion), so the
// tile carries a halo of 3 on each side: region H = (TX+6) x (TY+6).  The
// ghost cells of setbcc are formed from the original column and written
// into the planes by the adjacent interior cells (setbcc.f90:53-83), and
// they stay unchanged through the sweeps (the "stale ghosts" of the
// reference).  Input and output are distinct buffers (halos are read by
// neighbouring CTAs while this one writes).
//
// Arithmetic is binary32 with the reference's formulas; divisions by dx,
// dy and rho become multiplications by precomputed reciprocals.  The wet
// deposit and the dry-deposition accumulation stay binary64.
#include <algorithm>

#include "f3d_fused.h"

namespace f3d {

namespace {

struct ZT32 {
  float dzz, dzk, dzk_1, dzm1, l_dz, l_dzdz;
};

__device__ __forceinline__ void zwork(float cm, float c0, float cp, float vk, float vk_1,
                                      const ZT32& z, float dt, float& w1, float& w2) {
  const float vk_12 = 0.5f * (vk + vk_1);
  w1 = dt * (vk * c0 - vk_1 * cm) * z.dzz;
  const float deltar = (cp - c0) * z.dzk;
  const float deltal = (c0 - cm) * z.dzk_1;
  const float sigma = 0.5f * (sign1(deltar) + sign1(deltal)) * fmin2(fabsf(deltar), fabsf(deltal));
  const float Crk = fabsf(vk_12) * dt * z.dzk_1;
  w2 = dt * 0.5f * z.dzm1 * (1.0f - Crk) * sigma * fabsf(vk_12) * z.dzz;
}

// diffx/diffy cell of Sources/diffx.f90:20-55 with l = 1/rho and
// P = rkh*rho; m, 0, p = positions q-1, q, q+1 on the line.
__device__ __forceinline__ float diff_cell(int q, int n, float cm, float c0, float cp, float lm,
                                           float l0, float lp, float Pm, float P0, float Pp,
                                           float dtdx2) {
  float gradr, gradl;
  if (q == 1) {
    gradr = Pp * (cp * lp - c0 * l0);
    gradl = fmax2(0.0f, P0 * (c0 * l0 - cm * l0));
  } else if (q == n) {
    gradr = fmin2(0.0f, P0 * (cp * l0 - c0 * l0));
    gradl = Pm * (c0 * l0 - cm * lm);
  } else {
    const float rksr = 0.5f * (Pp + P0);
    const float rksl = 0.5f * (P0 + Pm);
    gradr = rksr * (cp * lp - c0 * l0);
    gradl = rksl * (c0 * l0 - cm * lm);
  }
  return c0 + dtdx2 * (gradr - gradl);
}

// One flux-limited advection sweep (advctx.f90:24-56) over lines of the
// H plane.  AX = 0: lines are rows (x sweep), AX = 1: columns (y sweep).
// Lines: interior lines [la, lb]; outputs at line positions [qa, qb];
// `in` -> `out` (positions not updated are copied).
template <int HX, int HY, int NT, int AX>
__device__ __forceinline__ void adv_sweep(const float* in, float* out, float* w1, float* w2,
                                          const float* __restrict__ v, long long vplane,
                                          int gx0, int gy0, int nx, int ny, int la, int lb, int qa,
                                          int qb, float auxv, float invd, float dt) {
  constexpr int NP = HX * HY;
  const int n = AX == 0 ? nx : ny;
  const int wa = max(1, qa - 1), wb = min(n + 1, qb + 1);
  // phase 1: work arrays at line positions [wa, wb]
  for (int p = threadIdx.x; p < NP; p += NT) {
    const int hx = p % HX, hy = p / HX;
    const int gi = gx0 + hx, gj = gy0 + hy;
    const int line = AX == 0 ? gj : gi;
    const int q = AX == 0 ? gi : gj;
    if (line < la || line > lb || q < wa || q > wb) continue;
    const int st = AX == 0 ? 1 : HX;  // plane stride along the line
    // velocity at line position r (1..n) of this line
    auto V = [&](int r) {
      const int ii = AX == 0 ? r : gi, jj = AX == 0 ? gj : r;
      return __ldg(v + vplane + (long long)(ii - 1) + (long long)nx * (jj - 1));
    };
    if (q <= n) {
      const float vq = V(q), vq_1 = V(q > 1 ? q - 1 : 1);
      const float cq = in[p], cm = in[p - st], cp = in[p + st];
      w1[p] = auxv * (vq * cq - vq_1 * cm);
      const float deltar = (cp - cq) * invd;
      const float deltal = (cq - cm) * invd;
      const float sigma = 0.5f * (sign1(deltar) + sign1(deltal)) * fmin2(fabsf(deltar), fabsf(deltal));
      const float vq_12 = 0.5f * (vq + vq_1);
      const float Cri = auxv * fabsf(vq_12);
      w2[p] = dt * 0.5f * (1.0f - Cri) * sigma * fabsf(vq_12);
    } else {  // q == n+1: work(n+1,1) with the velocity at n (advctx.f90:46)
      w1[p] = auxv * V(n) * (in[p] - in[p - st]);
    }
  }
  __syncthreads();
  // phase 2: update positions [qa, qb] of the lines, copy the rest
  for (int p = threadIdx.x; p < NP; p += NT) {
    const int hx = p % HX, hy = p / HX;
    const int gi = gx0 + hx, gj = gy0 + hy;
    const int line = AX == 0 ? gj : gi;
    const int q = AX == 0 ? gi : gj;
    if (line < la || line > lb || q < qa || q > qb) {
      out[p] = in[p];
      continue;
    }
    const int st = AX == 0 ? 1 : HX;
    const int ii = AX == 0 ? q : gi, jj = AX == 0 ? gj : q;
    const float vq = __ldg(v + vplane + (long long)(ii - 1) + (long long)nx * (jj - 1));
    const float cq = in[p];
    float cn;
    if (vq > 0.0f) {
      const float w2m = q > 1 ? w2[p - st] : w2[p];
      cn = cq - w1[p] - (w2[p] - w2m);
    } else {
      const float w2p = q < n ? w2[p + st] : w2[p];
      cn = cq - w1[p + st] - (w2p - w2[p]);
    }
    out[p] = cn;
  }
}

// One diffusion sweep (diffx.f90 / diffy.f90) over lines of the plane.
template <int HX, int HY, int NT, int AX>
__device__ __forceinline__ void diff_sweep(const float* in, float* out,
                                           const float* __restrict__ lrho,
                                           const float* __restrict__ pk, long long vplane, int gx0,
                                           int gy0, int nx, int ny, int la, int lb, int qa, int qb,
                                           float dtdx2) {
  constexpr int NP = HX * HY;
  const int n = AX == 0 ? nx : ny;
  for (int p = threadIdx.x; p < NP; p += NT) {
    const int hx = p % HX, hy = p / HX;
    const int gi = gx0 + hx, gj = gy0 + hy;
    const int line = AX == 0 ? gj : gi;
    const int q = AX == 0 ? gi : gj;
    if (line < la || line > lb || q < qa || q > qb) {
      out[p] = in[p];
      continue;
    }
    const int st = AX == 0 ? 1 : HX;
    const long long m0 = vplane + (long long)(gi - 1) + (long long)nx * (gj - 1);
    const long long ms = AX == 0 ? 1 : nx;
    const float l0 = __ldg(lrho + m0), P0 = __ldg(pk + m0);
    const float lm = q > 1 ? __ldg(lrho + m0 - ms) : 0.0f;
    const float Pm = q > 1 ? __ldg(pk + m0 - ms) : 0.0f;
    const float lp = q < n ? __ldg(lrho + m0 + ms) : 0.0f;
    const float Pp = q < n ? __ldg(pk + m0 + ms) : 0.0f;
    out[p] = diff_cell(q, n, in[p - st], in[p], in[p + st], lm, l0, lp, Pm, P0, Pp, dtdx2);
  }
}

template <int HX, int HY, int NT>
__global__ void __launch_bounds__(NT, (NT >= 512 ? 1 : 2)) k_step_fused(const FusedArgs a) {
  constexpr int TX = HX - 6, TY = HY - 6, NP = HX * HY, NCOL = NP / NT;
  constexpr int NOUT = (TX * TY + NT - 1) / NT;
  static_assert(NP % NT == 0, "tile must divide among threads");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* s1 = reinterpret_cast<float*>(smem_raw);
  float* sa = s1 + NP;
  float* w1 = sa + NP;
  float* w2 = w1 + NP;
  float* s2b = w2 + NP;  // two planes: S2(k) alternates
  float* s3 = s2b + 2 * NP;
  float* s3a = s3 + NP;
  double* wacc = reinterpret_cast<double*>(s3a + NP);  // per output cell: wet deposit,
  double* wlam = wacc + TX * TY;                        //   lambda, PBL height
  double* wzi = wlam + TX * TY;
  ZT32* tab = reinterpret_cast<ZT32*>(wzi + TX * TY);

  const Dims d = a.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int cls = blockIdx.x % a.ncls;
  const int tile = blockIdx.x / a.ncls;
  const int tiles_x = (nx + TX - 1) / TX;
  const int i0 = 1 + (tile % tiles_x) * TX, j0 = 1 + (tile / tiles_x) * TY;
  const int gx0 = i0 - 3, gy0 = j0 - 3;
  const int oi1 = min(nx, i0 + TX - 1), oj1 = min(ny, j0 + TY - 1);  // output tile end

  for (int p = threadIdx.x; p < 8 * NP; p += NT) s1[p] = 0.0f;
  for (int k = threadIdx.x; k <= nz; k += NT) {
    ZT32 z;
    const float dzk = a.dz[k];
    const float dzkm = k > 0 ? a.dz[k - 1] : dzk;
    z.dzz = 2.0f / (dzk + dzkm);
    z.dzk = 1.0f / dzk;
    z.dzk_1 = 1.0f / dzkm;
    z.dzm1 = dzkm;
    z.l_dz = 1.0f / dzk;
    z.l_dzdz = 2.0f / (dzk + dzkm);
    tab[k] = z;
  }
  __syncthreads();

  const long long hb = d.halo(), s3n = d.cells(), pl = d.plane();
  const long long cs = (long long)(nx + 2) * (ny + 2);  // plane stride in c
  const float* __restrict__ cin = a.c_in + (long long)cls * a.cstride;
  float* __restrict__ cout = a.c_out + (long long)cls * a.cstride;
  const float* __restrict__ vs = a.vset + (long long)cls * a.vstride;
  const float dt = a.dt;
  const float dznz = 1.0f / a.dz[nz];
  (void)hb;

  // ---------------- per-column state (columns of H owned by this thread)
  float o_0[NCOL], o_p1[NCOL], vk0[NCOL], w1k[NCOL], w2km[NCOL], w2k[NCOL], gtop[NCOL];
  float ra[NCOL], rb[NCOL], rc[NCOL], la_[NCOL], lb_[NCOL], lc_[NCOL], pa_[NCOL], pb_[NCOL],
      pc_[NCOL], fprev[NCOL];
  unsigned inter_mask = 0, out_mask = 0;
  // c(gi,gj,0) and met(gi,gj,1) offsets of owned column m
  auto CB = [&](int m) {
    const int p = threadIdx.x + NT * m;
    return (long long)(gx0 + p % HX) + (long long)(nx + 2) * (gy0 + p / HX);
  };
  auto MB = [&](int m) {
    const int p = threadIdx.x + NT * m;
    return (long long)(gx0 + p % HX - 1) + (long long)nx * (gy0 + p / HX - 1);
  };
#pragma unroll
  for (int m = 0; m < NCOL; ++m) {
    const int p = threadIdx.x + NT * m;
    const int gi = gx0 + p % HX, gj = gy0 + p / HX;
    const bool in = gi >= 1 && gi <= nx && gj >= 1 && gj <= ny;
    o_0[m] = o_p1[m] = vk0[m] = w1k[m] = w2km[m] = w2k[m] = gtop[m] = 0.0f;
    ra[m] = rb[m] = rc[m] = la_[m] = lb_[m] = lc_[m] = pa_[m] = pb_[m] = pc_[m] = fprev[m] = 0.0f;
    if (!in) continue;
    inter_mask |= 1u << m;
    const bool mine = gi >= i0 && gi <= oi1 && gj >= j0 && gj <= oj1;
    if (mine) out_mask |= 1u << m;
    const long long cbm = CB(m), mbm = MB(m);
    const float c1 = cin[cbm + cs], c2 = cin[cbm + 2 * cs];
    const float vk1 = __ldg(a.vz + mbm) + __ldg(vs + mbm);
    // setbcc bottom (setbcc.f90:19-33)
    float gb;
    if (vk1 >= 0.0f)
      gb = 0.0f;
    else
      gb = c1 * (1.0f + a.dz[0] * __ldg(a.vdep + (long long)cls * a.dstride + mbm) / __ldg(a.rkver1 + mbm));
    o_0[m] = c1;
    o_p1[m] = c2;
    vk0[m] = vk1;
    zwork(gb, c1, c2, vk1, vk1, tab[1], dt, w1k[m], w2k[m]);
    w2km[m] = w2k[m];
    rc[m] = gb;  // diffz window: c(0) is the bottom ghost
    if (mine) {
      cout[cbm] = fmax2(0.0f, gb);  // clipped ghost (sizloop.f90:77)
      // bottom corners (setbcc.f90:87-91)
      if (gi == 1 && gj == 1) cout[d.C(0, 0, 0)] = fmax2(0.0f, c1);
      if (gi == nx && gj == 1) cout[d.C(nx + 1, 0, 0)] = fmax2(0.0f, c1);
      if (gi == 1 && gj == ny) cout[d.C(0, ny + 1, 0)] = fmax2(0.0f, c1);
      if (gi == nx && gj == ny) cout[d.C(nx + 1, ny + 1, 0)] = fmax2(0.0f, c1);
    }
  }

  // ---------------- per-output-cell state (wet deposit accumulators)
  const bool wet = a.wet_class && a.wet_class[cls];
  for (int o = threadIdx.x; o < TX * TY; o += NT) {
    const int gi = i0 + o % TX, gj = j0 + o / TX;
    wacc[o] = 0.0;
    wlam[o] = 0.0;
    wzi[o] = -1e300;
    if (!wet || gi > oi1 || gj > oj1) continue;
    const long long p2 = (long long)(gi - 1) + (long long)nx * (gj - 1);
    wlam[o] = a.lambda2d[p2];
    wzi[o] = a.zi[p2];
    wacc[o] = a.cwet[(long long)(cls + 1) * pl + p2];
  }
  __syncthreads();

  const float auxvx = a.auxvx, auxvy = a.auxvy;
  for (int t = 1; t <= nz + 1; ++t) {
    float* s2cur = s2b + (t & 1) * NP;
    float* s2prev = s2b + ((t - 1) & 1) * NP;
    if (t <= nz) {
      const long long vpl = (long long)(t - 1) * pl;  // met plane t
      // ---------------- A: advctzc for plane t (advctzc.f90:32-79)
#pragma unroll
      for (int m = 0; m < NCOL; ++m) {
        if (!(inter_mask >> m & 1u)) continue;
        const int p = threadIdx.x + NT * m;
        const int hx = p % HX, hy = p / HX;
        const int gi = gx0 + hx, gj = gy0 + hy;
        const long long cbm = CB(m), mbm = MB(m);
        float w1n, w2n, o_p2 = 0.0f, vkp = 0.0f;
        if (t + 1 <= nz) {
          vkp = __ldg(a.vz + mbm + (long long)t * pl) + __ldg(vs + mbm + (long long)t * pl);
          if (t + 2 <= nz) {
            o_p2 = cin[cbm + (long long)(t + 2) * cs];
          } else {  // t+2 == nz+1: the top ghost (setbcc.f90:37-49), vkp = vk(nz)
            o_p2 = (vkp <= 0.0f) ? 0.0f : o_p1[m];
            gtop[m] = o_p2;
            if (out_mask >> m & 1u) {
              cout[cbm + (long long)(nz + 1) * cs] = fmax2(0.0f, o_p2);
              if (gi == 1 && gj == 1) cout[d.C(0, 0, nz + 1)] = fmax2(0.0f, o_p1[m]);
              if (gi == nx && gj == 1) cout[d.C(nx + 1, 0, nz + 1)] = fmax2(0.0f, o_p1[m]);
              if (gi == 1 && gj == ny) cout[d.C(0, ny + 1, nz + 1)] = fmax2(0.0f, o_p1[m]);
              if (gi == nx && gj == ny) cout[d.C(nx + 1, ny + 1, nz + 1)] = fmax2(0.0f, o_p1[m]);
            }
          }
          zwork(o_0[m], o_p1[m], o_p2, vkp, vk0[m], tab[t + 1], dt, w1n, w2n);
        } else {  // t == nz: work(nz+1,1) (advctzc.f90:58-64)
          w1n = dt * vk0[m] * (gtop[m] - o_0[m]) * dznz;
          w2n = w2k[m];
        }
        float cn;
        if (vk0[m] > 0.0f)
          cn = o_0[m] - w1k[m] - (w2k[m] - w2km[m]);
        else
          cn = o_0[m] - w1n - (w2n - w2k[m]);
        s1[p] = cn;
        // ghost faces of plane t from the original column (setbcc.f90:53-83)
        const float c0 = o_0[m];
        if (gi == 1 && hx >= 1) s1[p - 1] = (__ldg(a.vx + vpl + mbm) >= 0.0f) ? 0.0f : c0;
        if (gi == nx && hx + 1 < HX) s1[p + 1] = (__ldg(a.vx + vpl + mbm) <= 0.0f) ? 0.0f : c0;
        if (gj == 1 && hy >= 1) s1[p - HX] = (__ldg(a.vy + vpl + mbm) >= 0.0f) ? 0.0f : c0;
        if (gj == ny && hy + 1 < HY) s1[p + HX] = (__ldg(a.vy + vpl + mbm) <= 0.0f) ? 0.0f : c0;
        w2km[m] = w2k[m];
        w2k[m] = w2n;
        w1k[m] = w1n;
        o_0[m] = o_p1[m];
        o_p1[m] = o_p2;
        vk0[m] = vkp;
      }
      __syncthreads();
      // ---------------- B: advctx / advcty (sizloop.f90:42-48)
      const int ca = max(1, i0 - 1), cb2 = min(nx, i0 + TX);
      const int ra2 = max(1, j0 - 1), rb2 = min(ny, j0 + TY);
      if (a.xfirst) {
        adv_sweep<HX, HY, NT, 0>(s1, sa, w1, w2, a.vx, vpl, gx0, gy0, nx, ny, max(1, gy0),
                                 min(ny, gy0 + HY - 1), ca, cb2, auxvx, a.inv_dx, dt);
        __syncthreads();
        adv_sweep<HX, HY, NT, 1>(sa, s2cur, w1, w2, a.vy, vpl, gx0, gy0, nx, ny, ca, cb2, ra2, rb2,
                                 auxvy, a.inv_dy, dt);
      } else {
        adv_sweep<HX, HY, NT, 1>(s1, sa, w1, w2, a.vy, vpl, gx0, gy0, nx, ny, max(1, gx0),
                                 min(nx, gx0 + HX - 1), ra2, rb2, auxvy, a.inv_dy, dt);
        __syncthreads();
        adv_sweep<HX, HY, NT, 0>(sa, s2cur, w1, w2, a.vx, vpl, gx0, gy0, nx, ny, ra2, rb2, ca, cb2,
                                 auxvx, a.inv_dx, dt);
      }
      __syncthreads();
      // diffz window: S2(t)
#pragma unroll
      for (int m = 0; m < NCOL; ++m) {
        if (!(inter_mask >> m & 1u)) continue;
        const int p = threadIdx.x + NT * m;
        ra[m] = rb[m];
        rb[m] = rc[m];
        rc[m] = s2cur[p];
        la_[m] = lb_[m];
        lb_[m] = lc_[m];
        lc_[m] = __ldg(a.lrho + vpl + MB(m));
        pa_[m] = pb_[m];
        pb_[m] = pc_[m];
        pc_[m] = __ldg(a.pkz + vpl + MB(m));
      }
    } else {
#pragma unroll
      for (int m = 0; m < NCOL; ++m) {
        ra[m] = rb[m];
        rb[m] = rc[m];
        rc[m] = gtop[m];  // c(nz+1): the top ghost (diffz.f90:54)
        la_[m] = lb_[m];
        lb_[m] = lc_[m];
        pa_[m] = pb_[m];
        pb_[m] = pc_[m];
      }
    }
    if (t < 2) continue;
    // ---------------- D: diffz for plane k = t-1 (diffz.f90:22-62)
    const int k = t - 1;
    const ZT32 zk = tab[k];
#pragma unroll
    for (int m = 0; m < NCOL; ++m) {
      const int p = threadIdx.x + NT * m;
      if (!(inter_mask >> m & 1u)) {
        s3[p] = s2prev[p];
        continue;
      }
      float work;
      if (k == 1) {
        const float qt = rc[m] * lc_[m] - rb[m] * lb_[m];
        const float gradt = pc_[m] * qt * tab[1].l_dz;
        const float gradb = fmax2(0.0f, pb_[m] * (rb[m] * lb_[m] - ra[m] * lb_[m]) * tab[0].l_dz);
        work = dt * (gradt - gradb) * tab[1].l_dzdz;
        fprev[m] = 0.5f * (pc_[m] + pb_[m]) * qt * tab[1].l_dz;
      } else if (k == nz) {
        const float gradt = fmin2(0.0f, pb_[m] * (rc[m] * lb_[m] - rb[m] * lb_[m]) * tab[nz].l_dz);
        const float gradb = pa_[m] * (rb[m] * lb_[m] - ra[m] * la_[m]) * tab[nz - 1].l_dz;
        work = dt * (gradt - gradb) * tab[nz].l_dz;
      } else {
        const float gradt = 0.5f * (pc_[m] + pb_[m]) * (rc[m] * lc_[m] - rb[m] * lb_[m]) * zk.l_dz;
        work = dt * (gradt - fprev[m]) * zk.l_dzdz;
        fprev[m] = gradt;
      }
      s3[p] = rb[m] + work;
    }
    __syncthreads();
    // ---------------- E/F: diffx / diffy (sizloop.f90:55-61), then per cell
    const long long kpl = (long long)(k - 1) * pl;
    const int ca = max(1, i0 - 1), cb2 = min(nx, i0 + TX);
    const int ra2 = max(1, j0 - 1), rb2 = min(ny, j0 + TY);
    if (a.xfirst) {
      diff_sweep<HX, HY, NT, 0>(s3, s3a, a.lrho, a.pkx, kpl, gx0, gy0, nx, ny, ra2, rb2, i0, oi1,
                                a.dtdx2);
    } else {
      diff_sweep<HX, HY, NT, 1>(s3, s3a, a.lrho, a.pky, kpl, gx0, gy0, nx, ny, ca, cb2, j0, oj1,
                                a.dtdy2);
    }
    __syncthreads();
    const double zl = a.zlayer[k - 1], dzk64 = a.dz64[k];
#pragma unroll
    for (int u = 0; u < NOUT; ++u) {
      const int o = threadIdx.x + NT * u;
      if (o >= TX * TY) continue;
      const int gi = i0 + o % TX, gj = j0 + o / TX;
      if (gi > oi1 || gj > oj1) continue;
      const int p = (gi - gx0) + HX * (gj - gy0);
      const long long m0 = kpl + (long long)(gi - 1) + (long long)nx * (gj - 1);
      float cnew;
      if (a.xfirst) {  // second sweep: y
        const int q = gj;
        const float l0 = __ldg(a.lrho + m0), P0 = __ldg(a.pky + m0);
        const float lm = q > 1 ? __ldg(a.lrho + m0 - nx) : 0.0f, Pm = q > 1 ? __ldg(a.pky + m0 - nx) : 0.0f;
        const float lp = q < ny ? __ldg(a.lrho + m0 + nx) : 0.0f, Pp = q < ny ? __ldg(a.pky + m0 + nx) : 0.0f;
        cnew = diff_cell(q, ny, s3a[p - HX], s3a[p], s3a[p + HX], lm, l0, lp, Pm, P0, Pp, a.dtdy2);
      } else {
        const int q = gi;
        const float l0 = __ldg(a.lrho + m0), P0 = __ldg(a.pkx + m0);
        const float lm = q > 1 ? __ldg(a.lrho + m0 - 1) : 0.0f, Pm = q > 1 ? __ldg(a.pkx + m0 - 1) : 0.0f;
        const float lp = q < nx ? __ldg(a.lrho + m0 + 1) : 0.0f, Pp = q < nx ? __ldg(a.pkx + m0 + 1) : 0.0f;
        cnew = diff_cell(q, nx, s3a[p - 1], s3a[p], s3a[p + 1], lm, l0, lp, Pm, P0, Pp, a.dtdx2);
      }
      // wetdep (wetdep.f90:37-49): binary64 deposit, binary32 concentration
      if (wet && zl <= wzi[o]) {
        wacc[o] = wacc[o] + dzk64 * wlam[o] * (double)cnew;
        cnew = (float)((double)cnew * (1.0 - wlam[o]));
      }
      const long long p2 = (long long)(gi - 1) + (long long)nx * (gj - 1);
      if (k == 1) {  // accum (accum.f90:17-25), binary64
        double* cd = a.cdry + (long long)(cls + 1) * pl + p2;
        const double vsd = a.vset64[(long long)cls * a.vstride + p2] + a.vdep64[(long long)cls * pl + p2];
        *cd = *cd - a.dt64 * (double)cnew * fmin2(0.0, vsd);
      }
      const long long cidx = (long long)gi + (long long)(nx + 2) * (gj + (long long)(ny + 2) * k);
      cout[cidx] = fmax2(0.0f, cnew);  // clip (sizloop.f90:77)
      // clipped ghost faces of plane k (written by the adjacent output cell)
      if (gi == 1) cout[cidx - 1] = fmax2(0.0f, s3[p - 1]);
      if (gi == nx) cout[cidx + 1] = fmax2(0.0f, s3[p + 1]);
      if (gj == 1) cout[cidx - (nx + 2)] = fmax2(0.0f, s3[p - HX]);
      if (gj == ny) cout[cidx + (nx + 2)] = fmax2(0.0f, s3[p + HX]);
    }
    (void)s3n;
  }
  if (wet) {
    for (int o = threadIdx.x; o < TX * TY; o += NT) {
      const int gi = i0 + o % TX, gj = j0 + o / TX;
      if (gi > oi1 || gj > oj1) continue;
      a.cwet[(long long)(cls + 1) * pl + (long long)(gi - 1) + (long long)nx * (gj - 1)] = wacc[o];
    }
  }
}

template <int HX, int HY, int NT>
size_t fused_smem(int nz) {
  return sizeof(float) * 8 * HX * HY + 3 * sizeof(double) * (HX - 6) * (HY - 6) +
         sizeof(ZT32) * (size_t)(nz + 1);
}

template <int HX, int HY, int NT>
void launch_fused_t(const FusedArgs& a, cudaStream_t s) {
  constexpr int TX = HX - 6, TY = HY - 6;
  const int tiles = ((a.d.nx + TX - 1) / TX) * ((a.d.ny + TY - 1) / TY);
  const size_t sm = fused_smem<HX, HY, NT>(a.d.nz);
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_step_fused<HX, HY, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_step_fused<HX, HY, NT><<<tiles * a.ncls, NT, sm, s>>>(a);
  count_launch();
}

}  // namespace

void launch_step_fused(const FusedArgs& a, int shape, cudaStream_t s) {
  switch (shape) {
    case 1:
      launch_fused_t<64, 32, 512>(a, s);
      break;
    case 2:
      launch_fused_t<32, 32, 512>(a, s);
      break;
    default:
      launch_fused_t<32, 32, 256>(a, s);
      break;
  }
}

// wet-deposition rate per column for the fused kernel: lambda =
// min(dt*a*prate^b, 1) (wetdep.f90:40), constant between meteo updates.
__global__ void k_wet_lambda(long long n, double dt, const double* prate, double* lam) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double aa = 8.4e-5, b = 0.79;
  lam[p] = fmin2(dt * aa * pow(prate[p], b), 1.0);
}

void launch_wet_lambda(long long n, double dt, const double* prate, double* lam, cudaStream_t s) {
  k_wet_lambda<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, dt, prate, lam);
  count_launch();
}

// FP32-form coefficient fields: 1/rho and the face products rkh*rho.
__global__ void k_fp32_coeffs(long long n, const double* rho, const double* rkh1,
                              const double* rkhor, const double* rkver, float* lrho, float* pkx,
                              float* pky, float* pkz) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const double r = rho[q];
    lrho[q] = (float)(1.0 / r);
    pkx[q] = (float)(rkh1[q] * r);
    pky[q] = (float)(rkhor[q] * r);
    pkz[q] = (float)(rkver[q] * r);
  }
}

void launch_fp32_coeffs(long long n, const double* rho, const double* rkh1, const double* rkhor,
                        const double* rkver, float* lrho, float* pkx, float* pky, float* pkz,
                        cudaStream_t s) {
  const int nb = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  k_fp32_coeffs<<<nb, 256, 0, s>>>(n, rho, rkh1, rkhor, rkver, lrho, pkx, pky, pkz);
  count_launch();
}

}  // namespace f3d

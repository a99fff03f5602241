// f3d_fused.cu -- the precision form's whole transport step in one kernel.
//
// One CTA owns an output tile of one class and marches up the column, so
// each concentration is read from and written to HBM once per step.  The
// sweeps of Sources/sizloop.f90:35-71 are pipelined per horizontal plane k:
//
//   A  setbcc + advctzc   per column in registers (window of the original
//                         column c(k-1..k+2) and work(k), work(k+1))
//   B  advctx / advcty    x: warp shuffles along a row; y: shared memory
//   C  diffz (plane k-1)  per column in registers (needs plane k of B)
//   D  diffx / diffy      x: warp shuffles; y: shared memory
//   E  wetdep, accum, clip, store (per cell)
//
// Thread layout: the tile region H is 32 columns (one warp lane each) by HY
// rows; warp w owns rows w, w+NW, w+2NW, ...  Every thread keeps the state of
// its RPW columns in registers for the whole march; x neighbours are lanes of
// the same warp, y neighbours go through one shared-memory plane.  The x/y
// sweeps need +-2 cells (advection) then +-1 (diffusion), so the output tile
// is (32-6) x (HY-6).  The ghost cells of setbcc are formed from the original
// column (setbcc.f90:53-83) by the thread that owns the ghost position and
// stay unchanged through the sweeps (the reference's stale ghosts).  Input
// and output are distinct buffers (halos are read by neighbouring CTAs).
//
// Arithmetic is binary32 with the reference's formulas; divisions by dx, dy
// and rho become multiplications by precomputed reciprocals.  The unit is
// compiled with --fmad=false: each cell's result is then independent of the
// tile shape.  The wet deposit and the dry-deposition accumulation stay
// binary64.
#include <algorithm>

#include "f3d_fused.h"

namespace f3d {

namespace {

constexpr unsigned FULL = 0xffffffffu;

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

// work(q,1), work(q,2) of advctx.f90:24-44 at line position q.
__device__ __forceinline__ void line_work(float cm, float c0, float cp, float vq, float vq_1,
                                          float auxv, float invd, float dt, float& w1, float& w2) {
  const float vq_12 = 0.5f * (vq + vq_1);
  w1 = auxv * (vq * c0 - vq_1 * cm);
  const float deltar = (cp - c0) * invd;
  const float deltal = (c0 - cm) * invd;
  const float sigma = 0.5f * (sign1(deltar) + sign1(deltal)) * fmin2(fabsf(deltar), fabsf(deltal));
  const float Cri = auxv * fabsf(vq_12);
  w2 = dt * 0.5f * (1.0f - Cri) * sigma * fabsf(vq_12);
}

// The update of advctx.f90:48-54.
__device__ __forceinline__ float line_update(float c0, float vq, float w1, float w1p, float w2,
                                             float w2m, float w2p) {
  if (vq > 0.0f) return c0 - w1 - (w2 - w2m);
  return c0 - w1p - (w2p - w2);
}

// diffx/diffy cell of Sources/diffx.f90:20-55 with l = 1/rho, P = rkh*rho.
__device__ __forceinline__ float diff_cell(bool first, bool last, float cm, float c0, float cp,
                                           float lm, float l0, float lp, float Pm, float P0,
                                           float Pp, float dtdx2) {
  float gradr, gradl;
  if (first) {
    gradr = Pp * (cp * lp - c0 * l0);
    gradl = fmax2(0.0f, P0 * (c0 * l0 - cm * l0));
  } else if (last) {
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

// Position kinds inside the tile region.
enum : int { K_OUT = 0, K_IN = 1, K_GX = 2, K_GY = 3 };

template <int HY, int NW>
__global__ void __launch_bounds__(32 * NW, (32 * NW >= 512 ? 1 : 2)) k_step_fused(const FusedArgs a) {
  constexpr int HX = 32, NT = 32 * NW, RPW = HY / NW, TX = HX - 6, TY = HY - 6;
  static_assert(HY % NW == 0, "rows must divide among warps");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* P0s = reinterpret_cast<float*>(smem_raw);  // y-sweep plane (advection)
  float* W1s = P0s + HX * HY;
  float* W2s = W1s + HX * HY;
  float* P1s = W2s + HX * HY;                      // y-sweep plane (diffusion)
  double* wacc = reinterpret_cast<double*>(P1s + HX * HY);  // wet state per output cell
  double* wlam = wacc + TX * TY;
  double* wzi = wlam + TX * TY;
  ZT32* tab = reinterpret_cast<ZT32*>(wzi + TX * TY);

  const Dims d = a.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int cls = blockIdx.x % a.ncls;
  const int tile = blockIdx.x / a.ncls;
  const int tiles_x = (nx + TX - 1) / TX;
  const int i0 = 1 + (tile % tiles_x) * TX, j0 = 1 + (tile / tiles_x) * TY;
  const int gx0 = i0 - 3, gy0 = j0 - 3;
  const int oi1 = min(nx, i0 + TX - 1), oj1 = min(ny, j0 + TY - 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gi = gx0 + lane;

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
  const bool wet = a.wet_class && a.wet_class[cls];
  const long long pl = d.plane();
  for (int o = threadIdx.x; o < TX * TY; o += NT) {
    const int oi = i0 + o % TX, oj = j0 + o / TX;
    wacc[o] = 0.0;
    wlam[o] = 0.0;
    wzi[o] = -1e300;
    if (!wet || oi > oi1 || oj > oj1) continue;
    const long long p2 = (long long)(oi - 1) + (long long)nx * (oj - 1);
    wlam[o] = a.lambda2d[p2];
    wzi[o] = a.zi[p2];
    wacc[o] = a.cwet[(long long)(cls + 1) * pl + p2];
  }
  __syncthreads();

  const long long cs = (long long)(nx + 2) * (ny + 2);
  const float* __restrict__ cin = a.c_in + (long long)cls * a.cstride;
  float* __restrict__ cout = a.c_out + (long long)cls * a.cstride;
  const float* __restrict__ vs = a.vset + (long long)cls * a.vstride;
  const float dt = a.dt;
  const float dznz = 1.0f / a.dz[nz];
  const bool xin = gi >= 1 && gi <= nx;  // interior x line position

  // ------------------------------------------------ per-position state
  int kind[RPW];
  float o_0[RPW], o_p1[RPW], vk0[RPW], w1k[RPW], w2km[RPW], w2k[RPW], gtop[RPW];
  float ra[RPW], rb[RPW], rc[RPW], fprev[RPW], gprev[RPW];
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    const int hy = warp + NW * r;
    const int gj = gy0 + hy;
    const bool yin = gj >= 1 && gj <= ny;
    int kd = K_OUT;
    if (xin && yin) kd = K_IN;
    else if ((gi == 0 || gi == nx + 1) && yin) kd = K_GX;
    else if ((gj == 0 || gj == ny + 1) && xin) kd = K_GY;
    kind[r] = kd;
    o_0[r] = o_p1[r] = vk0[r] = w1k[r] = w2km[r] = w2k[r] = gtop[r] = 0.0f;
    ra[r] = rb[r] = rc[r] = fprev[r] = gprev[r] = 0.0f;
    if (kd != K_IN) continue;
    const long long cb = (long long)gi + (long long)(nx + 2) * gj;
    const long long mb = (long long)(gi - 1) + (long long)nx * (gj - 1);
    const float c1 = cin[cb + cs], c2 = cin[cb + 2 * cs];
    const float vk1 = __ldg(a.vz + mb) + __ldg(vs + mb);
    float gb;  // setbcc bottom (setbcc.f90:19-33)
    if (vk1 >= 0.0f)
      gb = 0.0f;
    else
      gb = c1 * (1.0f + a.dz[0] * __ldg(a.vdep + (long long)cls * a.dstride + mb) / __ldg(a.rkver1 + mb));
    o_0[r] = c1;
    o_p1[r] = c2;
    vk0[r] = vk1;
    zwork(gb, c1, c2, vk1, vk1, tab[1], dt, w1k[r], w2k[r]);
    w2km[r] = w2k[r];
    rc[r] = gb;  // diffz window: c(0) is the bottom ghost
    if (gi >= i0 && gi <= oi1 && gj >= j0 && gj <= oj1) {
      cout[cb] = fmax2(0.0f, gb);  // clipped ghost (sizloop.f90:77)
      if (gi == 1 && gj == 1) cout[d.C(0, 0, 0)] = fmax2(0.0f, c1);  // setbcc.f90:87-91
      if (gi == nx && gj == 1) cout[d.C(nx + 1, 0, 0)] = fmax2(0.0f, c1);
      if (gi == 1 && gj == ny) cout[d.C(0, ny + 1, 0)] = fmax2(0.0f, c1);
      if (gi == nx && gj == ny) cout[d.C(nx + 1, ny + 1, 0)] = fmax2(0.0f, c1);
    }
  }

  const float auxvx = a.auxvx, auxvy = a.auxvy;
  for (int t = 1; t <= nz + 1; ++t) {
    const long long vpl = (long long)(t - 1) * pl;  // met plane t
    float s2[RPW];
    if (t <= nz) {
      float s1[RPW];
      // ---------------- A: setbcc ghosts + advctzc for plane t
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int gj = gy0 + warp + NW * r;
        s1[r] = 0.0f;
        if (kind[r] == K_GX) {  // x-face ghost from the original column (setbcc.f90:53-66)
          const int ia = gi == 0 ? 1 : nx;
          const float cadj = cin[(long long)ia + (long long)(nx + 2) * (gj + (long long)(ny + 2) * t)];
          const float v = __ldg(a.vx + vpl + (long long)(ia - 1) + (long long)nx * (gj - 1));
          s1[r] = (gi == 0) ? (v >= 0.0f ? 0.0f : cadj) : (v <= 0.0f ? 0.0f : cadj);
        } else if (kind[r] == K_GY) {  // y-face ghost (setbcc.f90:70-83)
          const int ja = gj == 0 ? 1 : ny;
          const float cadj = cin[(long long)gi + (long long)(nx + 2) * (ja + (long long)(ny + 2) * t)];
          const float v = __ldg(a.vy + vpl + (long long)(gi - 1) + (long long)nx * (ja - 1));
          s1[r] = (gj == 0) ? (v >= 0.0f ? 0.0f : cadj) : (v <= 0.0f ? 0.0f : cadj);
        } else if (kind[r] == K_IN) {
          const long long cb = (long long)gi + (long long)(nx + 2) * gj;
          const long long mb = (long long)(gi - 1) + (long long)nx * (gj - 1);
          float w1n, w2n, o_p2 = 0.0f, vkp = 0.0f;
          if (t + 1 <= nz) {
            vkp = __ldg(a.vz + mb + (long long)t * pl) + __ldg(vs + mb + (long long)t * pl);
            if (t + 2 <= nz) {
              o_p2 = cin[cb + (long long)(t + 2) * cs];
            } else {  // the top ghost (setbcc.f90:37-49), vkp = vk(nz)
              o_p2 = (vkp <= 0.0f) ? 0.0f : o_p1[r];
              gtop[r] = o_p2;
              if (gi >= i0 && gi <= oi1 && gj >= j0 && gj <= oj1) {
                cout[cb + (long long)(nz + 1) * cs] = fmax2(0.0f, o_p2);
                if (gi == 1 && gj == 1) cout[d.C(0, 0, nz + 1)] = fmax2(0.0f, o_p1[r]);
                if (gi == nx && gj == 1) cout[d.C(nx + 1, 0, nz + 1)] = fmax2(0.0f, o_p1[r]);
                if (gi == 1 && gj == ny) cout[d.C(0, ny + 1, nz + 1)] = fmax2(0.0f, o_p1[r]);
                if (gi == nx && gj == ny) cout[d.C(nx + 1, ny + 1, nz + 1)] = fmax2(0.0f, o_p1[r]);
              }
            }
            zwork(o_0[r], o_p1[r], o_p2, vkp, vk0[r], tab[t + 1], dt, w1n, w2n);
          } else {  // t == nz: work(nz+1,1) (advctzc.f90:58-64)
            w1n = dt * vk0[r] * (gtop[r] - o_0[r]) * dznz;
            w2n = w2k[r];
          }
          if (vk0[r] > 0.0f)
            s1[r] = o_0[r] - w1k[r] - (w2k[r] - w2km[r]);
          else
            s1[r] = o_0[r] - w1n - (w2n - w2k[r]);
          w2km[r] = w2k[r];
          w2k[r] = w2n;
          w1k[r] = w1n;
          o_0[r] = o_p1[r];
          o_p1[r] = o_p2;
          vk0[r] = vkp;
        }
      }
      // ---------------- B: advctx (shuffles) and advcty (shared memory)
      auto adv_x = [&](const float* in, float* out) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int gj = gy0 + warp + NW * r;
          const bool row = gj >= 1 && gj <= ny;
          const float c0 = in[r];
          const float v = (row && xin) ? __ldg(a.vx + vpl + (long long)(gi - 1) + (long long)nx * (gj - 1)) : 0.0f;
          const float cm = __shfl_up_sync(FULL, c0, 1), cp = __shfl_down_sync(FULL, c0, 1);
          const float vm_raw = __shfl_up_sync(FULL, v, 1);
          const float vm = gi > 1 ? vm_raw : v;  // v(max(1,q-1))
          float w1 = 0.0f, w2 = 0.0f;
          if (xin) line_work(cm, c0, cp, v, vm, auxvx, a.inv_dx, dt, w1, w2);
          else if (gi == nx + 1) w1 = auxvx * vm_raw * (c0 - cm);  // work(nx+1,1) (advctx.f90:46)
          const float w1p = __shfl_down_sync(FULL, w1, 1);
          const float w2m_raw = __shfl_up_sync(FULL, w2, 1), w2p_raw = __shfl_down_sync(FULL, w2, 1);
          const float w2m = gi > 1 ? w2m_raw : w2;
          const float w2p = gi < nx ? w2p_raw : w2;
          out[r] = (row && xin) ? line_update(c0, v, w1, w1p, w2, w2m, w2p) : c0;
        }
      };
      auto adv_y = [&](const float* in, float* out) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) P0s[(warp + NW * r) * HX + lane] = in[r];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int hy = warp + NW * r;
          const int gj = gy0 + hy;
          float w1 = 0.0f, w2 = 0.0f;
          if (xin && gj >= 1 && gj <= ny + 1) {
            const float c0 = P0s[hy * HX + lane];
            const float cm = P0s[max(hy - 1, 0) * HX + lane];
            const long long mcol = vpl + (long long)(gi - 1);
            if (gj <= ny) {
              const float cp = P0s[min(hy + 1, HY - 1) * HX + lane];
              const float v = __ldg(a.vy + mcol + (long long)nx * (gj - 1));
              const float vm = __ldg(a.vy + mcol + (long long)nx * (gj > 1 ? gj - 2 : 0));
              line_work(cm, c0, cp, v, vm, auxvy, a.inv_dy, dt, w1, w2);
            } else {  // work(ny+1,1) (advcty.f90:45)
              w1 = auxvy * __ldg(a.vy + mcol + (long long)nx * (ny - 1)) * (c0 - cm);
            }
          }
          W1s[hy * HX + lane] = w1;
          W2s[hy * HX + lane] = w2;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int hy = warp + NW * r;
          const int gj = gy0 + hy;
          out[r] = in[r];
          if (xin && gj >= 1 && gj <= ny) {
            const float v = __ldg(a.vy + vpl + (long long)(gi - 1) + (long long)nx * (gj - 1));
            const int hm = max(hy - 1, 0), hp = min(hy + 1, HY - 1);
            const float w2 = W2s[hy * HX + lane];
            const float w2m = gj > 1 ? W2s[hm * HX + lane] : w2;
            const float w2p = gj < ny ? W2s[hp * HX + lane] : w2;
            out[r] = line_update(in[r], v, W1s[hy * HX + lane], W1s[hp * HX + lane], w2, w2m, w2p);
          }
        }
      };
      float sa[RPW];
      if (a.xfirst) {  // sizloop.f90:42-48
        adv_x(s1, sa);
        adv_y(sa, s2);
      } else {
        adv_y(s1, sa);
        adv_x(sa, s2);
      }
    } else {
#pragma unroll
      for (int r = 0; r < RPW; ++r) s2[r] = 0.0f;
    }
    if (t < 2) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        if (kind[r] == K_IN) {
          ra[r] = rb[r];
          rb[r] = rc[r];
          rc[r] = s2[r];
        } else {
          gprev[r] = s2[r];  // ghost (or unused) value of plane t
        }
      }
      continue;
    }
    // ---------------- C: diffz for plane k = t-1 (diffz.f90:22-62)
    const int k = t - 1;
    const long long kpl = (long long)(k - 1) * pl;
    float s3[RPW];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      if (kind[r] != K_IN) {
        s3[r] = gprev[r];  // ghost value of plane k (unchanged by the sweeps)
        gprev[r] = s2[r];
        continue;
      }
      const int gj = gy0 + warp + NW * r;
      ra[r] = rb[r];
      rb[r] = rc[r];
      rc[r] = (t <= nz) ? s2[r] : gtop[r];  // c(nz+1): the top ghost (diffz.f90:54)
      const long long m = kpl + (long long)(gi - 1) + (long long)nx * (gj - 1);
      const float lb = __ldg(a.lrho + m), pb = __ldg(a.pkz + m);
      float work;
      if (k == 1) {
        const float lc = __ldg(a.lrho + m + pl), pc = __ldg(a.pkz + m + pl);
        const float qt = rc[r] * lc - rb[r] * lb;
        const float gradt = pc * qt * tab[1].l_dz;
        const float gradb = fmax2(0.0f, pb * (rb[r] * lb - ra[r] * lb) * tab[0].l_dz);
        work = dt * (gradt - gradb) * tab[1].l_dzdz;
        fprev[r] = 0.5f * (pc + pb) * qt * tab[1].l_dz;
      } else if (k == nz) {
        const float la = __ldg(a.lrho + m - pl), pa = __ldg(a.pkz + m - pl);
        const float gradt = fmin2(0.0f, pb * (rc[r] * lb - rb[r] * lb) * tab[nz].l_dz);
        const float gradb = pa * (rb[r] * lb - ra[r] * la) * tab[nz - 1].l_dz;
        work = dt * (gradt - gradb) * tab[nz].l_dz;
      } else {
        const float lc = __ldg(a.lrho + m + pl), pc = __ldg(a.pkz + m + pl);
        const ZT32 zk = tab[k];
        const float gradt = 0.5f * (pc + pb) * (rc[r] * lc - rb[r] * lb) * zk.l_dz;
        work = dt * (gradt - fprev[r]) * zk.l_dzdz;
        fprev[r] = gradt;
      }
      s3[r] = rb[r] + work;
    }
    // ---------------- D: diffx (shuffles) and diffy (shared memory)
    auto dif_x = [&](const float* in, float* out) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int gj = gy0 + warp + NW * r;
        const bool row = gj >= 1 && gj <= ny;
        const long long m = kpl + (long long)(gi - 1) + (long long)nx * (gj - 1);
        const float l0 = (row && xin) ? __ldg(a.lrho + m) : 0.0f;
        const float P0 = (row && xin) ? __ldg(a.pkx + m) : 0.0f;
        const float c0 = in[r];
        const float cm = __shfl_up_sync(FULL, c0, 1), cp = __shfl_down_sync(FULL, c0, 1);
        const float lm = __shfl_up_sync(FULL, l0, 1), lp = __shfl_down_sync(FULL, l0, 1);
        const float Pm = __shfl_up_sync(FULL, P0, 1), Pp = __shfl_down_sync(FULL, P0, 1);
        out[r] = (row && xin) ? diff_cell(gi == 1, gi == nx, cm, c0, cp, lm, l0, lp, Pm, P0, Pp, a.dtdx2)
                              : c0;
      }
    };
    auto dif_y = [&](const float* in, float* out) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) P1s[(warp + NW * r) * HX + lane] = in[r];
      __syncthreads();
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int hy = warp + NW * r;
        const int gj = gy0 + hy;
        out[r] = in[r];
        if (xin && gj >= 1 && gj <= ny) {
          const long long m = kpl + (long long)(gi - 1) + (long long)nx * (gj - 1);
          const float l0 = __ldg(a.lrho + m), P0 = __ldg(a.pky + m);
          const bool first = gj == 1, last = gj == ny;
          const float lm = first ? 0.0f : __ldg(a.lrho + m - nx), Pm = first ? 0.0f : __ldg(a.pky + m - nx);
          const float lp = last ? 0.0f : __ldg(a.lrho + m + nx), Pp = last ? 0.0f : __ldg(a.pky + m + nx);
          const float cm = P1s[max(hy - 1, 0) * HX + lane], cp = P1s[min(hy + 1, HY - 1) * HX + lane];
          out[r] = diff_cell(first, last, cm, in[r], cp, lm, l0, lp, Pm, P0, Pp, a.dtdy2);
        }
      }
    };
    float s3a[RPW], s4[RPW];
    if (a.xfirst) {  // sizloop.f90:55-61
      dif_x(s3, s3a);
      dif_y(s3a, s4);
    } else {
      dif_y(s3, s3a);
      dif_x(s3a, s4);
    }
    // ---------------- E: wetdep, accum, clip, store (plane k)
    const double zl = a.zlayer[k - 1], dzk64 = a.dz64[k];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int gj = gy0 + warp + NW * r;
      const bool rows_out = gj >= j0 && gj <= oj1;
      if (kind[r] == K_GX && rows_out && ((gi == 0 && i0 == 1) || (gi == nx + 1 && oi1 == nx))) {
        cout[(long long)gi + (long long)(nx + 2) * (gj + (long long)(ny + 2) * k)] = fmax2(0.0f, s3[r]);
        continue;
      }
      const bool cols_out = gi >= i0 && gi <= oi1;
      if (kind[r] == K_GY && cols_out && ((gj == 0 && j0 == 1) || (gj == ny + 1 && oj1 == ny))) {
        cout[(long long)gi + (long long)(nx + 2) * (gj + (long long)(ny + 2) * k)] = fmax2(0.0f, s3[r]);
        continue;
      }
      if (kind[r] != K_IN || !rows_out || !cols_out) continue;
      float cnew = s4[r];
      const int o = (gi - i0) + TX * (gj - j0);
      if (wet && zl <= wzi[o]) {  // wetdep (wetdep.f90:37-49)
        wacc[o] = wacc[o] + dzk64 * wlam[o] * (double)cnew;
        cnew = (float)((double)cnew * (1.0 - wlam[o]));
      }
      const long long p2 = (long long)(gi - 1) + (long long)nx * (gj - 1);
      if (k == 1) {  // accum (accum.f90:17-25), binary64
        double* cd = a.cdry + (long long)(cls + 1) * pl + p2;
        const double vsd = a.vset64[(long long)cls * a.vstride + p2] + a.vdep64[(long long)cls * pl + p2];
        *cd = *cd - a.dt64 * (double)cnew * fmin2(0.0, vsd);
      }
      cout[(long long)gi + (long long)(nx + 2) * (gj + (long long)(ny + 2) * k)] = fmax2(0.0f, cnew);
    }
  }
  if (wet) {
    __syncthreads();
    for (int o = threadIdx.x; o < TX * TY; o += NT) {
      const int oi = i0 + o % TX, oj = j0 + o / TX;
      if (oi > oi1 || oj > oj1) continue;
      a.cwet[(long long)(cls + 1) * pl + (long long)(oi - 1) + (long long)nx * (oj - 1)] = wacc[o];
    }
  }
}

template <int HY>
size_t fused_smem(int nz) {
  return sizeof(float) * 4 * 32 * HY + 3 * sizeof(double) * 26 * (HY - 6) + sizeof(ZT32) * (size_t)(nz + 1);
}

template <int HY, int NW>
void launch_fused_t(const FusedArgs& a, cudaStream_t s) {
  constexpr int TX = 26, TY = HY - 6;
  const int tiles = ((a.d.nx + TX - 1) / TX) * ((a.d.ny + TY - 1) / TY);
  const size_t sm = fused_smem<HY>(a.d.nz);
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_step_fused<HY, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_step_fused<HY, NW><<<tiles * a.ncls, 32 * NW, sm, s>>>(a);
  count_launch();
}

}  // namespace

void launch_step_fused(const FusedArgs& a, int shape, cudaStream_t s) {
  switch (shape) {
    case 1:
      launch_fused_t<64, 16>(a, s);
      break;
    case 2:
      launch_fused_t<32, 16>(a, s);
      break;
    default:
      launch_fused_t<32, 8>(a, s);
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

// f3d_fused.cu -- the precision form's whole transport step in one kernel.
//
// One CTA owns an output tile of one class and marches up the column, so
// each concentration is read from and written to HBM once per step.  The
// sweeps of Sources/sizloop.f90:35-71 are pipelined per horizontal plane:
// iteration t runs
//
//   A  setbcc + advctzc   plane t, per column in registers (window of the
//                         original column c(t-1..t+2) and work(t), work(t+1))
//   B  advctx / advcty    plane t; x: warp shuffles along a row; y: shared
//                         memory
//   C  diffz              plane k = t-1 (needs plane t of B)
//   D  diffx / diffy      plane k; x: warp shuffles; y: shared memory
//   E  wetdep, accum, clip, store (plane k)
//
// Thread layout: the tile region is 32 columns (one warp lane each) by HY
// rows; warp w owns rows w, w+NW, w+2NW, ...  Every thread keeps the state of
// its RPW columns in registers for the whole march.  The x/y sweeps need +-2
// cells (advection) then +-1 (diffusion), so the output tile is
// (32-6) x (HY-6).  The ghost cells of setbcc are formed from the original
// column (setbcc.f90:53-83) and stay unchanged through the sweeps (the
// reference's stale ghosts).  Input and output are distinct buffers (halos
// are read by neighbouring CTAs).
//
// Tiles whose region lies inside the domain (no ghost cell, no boundary
// face within reach of an output cell) run a body without any boundary
// logic; so do the planes 3..nz-2 (no top/bottom special case).  Halo cells
// of the region compute with the interior formulas; their values are wrong
// but never reach an output cell.
//
// Memory pipeline: the inputs of iteration t+1 are copied global -> shared
// with cp.async while iteration t computes, into a double-buffered staging
// area; each thread copies the positions it owns (coalesced rows of 32).
//
// Arithmetic is binary32 with the reference's formulas and operation order;
// divisions by dx, dy and rho are multiplications by precomputed
// reciprocals.  The unit is compiled with --fmad=false, so each cell's result
// is independent of the tile shape.  The wet deposit and the dry-deposition
// accumulation stay binary64.
#include <algorithm>
#include <type_traits>

#include "f3d_fused_math.cuh"

namespace f3d {

namespace {

using namespace fz;

// One tile of one class: the whole march.  c_in / c_out are the class
// blocks' base (all classes); commit = 0 skips the deposit writes (cdry, cwet)
// so that the autotuner can time the kernel on a live state.
template <int HY, int NW>
__device__ __forceinline__ void fused_tile(const FusedArgs& a, const float* c_in, float* c_out,
                                           const int xfirst, const int commit, const int cls,
                                           const int tile, unsigned char* smem_raw) {
  constexpr int HX = 32, NT = 32 * NW, RPW = HY / NW, TX = HX - 6, TY = HY - 6, NP = HX * HY;
  static_assert(HY % NW == 0, "rows must divide among warps");
  // a guard row on either side keeps the +-1 row reads of halo rows in bounds
  float* stage = reinterpret_cast<float*>(smem_raw) + HX;  // [2][NF][NP]
  float* P0s = stage + 2 * NF * NP;                          // y-sweep planes
  float* W1s = P0s + NP;
  float* W2s = W1s + NP;
  float* P1s = W2s + NP;
  double* wacc = reinterpret_cast<double*>(P1s + NP + HX);  // wet state per output cell
  double* wlam = wacc + TX * TY;
  int* wkz = reinterpret_cast<int*>(wlam + TX * TY);  // highest k with zlayer(k) <= zi
  ZT32* tab = reinterpret_cast<ZT32*>(wkz + TX * TY);

  const Dims d = a.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int tiles_x = (nx + TX - 1) / TX;
  const int i0 = 1 + (tile % tiles_x) * TX, j0 = 1 + (tile / tiles_x) * TY;
  const int gx0 = i0 - 3, gy0 = j0 - 3;
  const int oi1 = min(nx, i0 + TX - 1), oj1 = min(ny, j0 + TY - 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gi = gx0 + lane;
  const bool xin = gi >= 1 && gi <= nx;  // interior x line position
  const int pl = nx * ny;                 // met plane (32-bit offsets: checked on the host)
  const int cs = (nx + 2) * (ny + 2);     // c plane
  const bool edge = !(gx0 >= 1 && gx0 + HX - 1 <= nx && gy0 >= 1 && gy0 + HY - 1 <= ny);

  for (int k = threadIdx.x; k <= nz; k += NT) {
    const float dzk = a.dz[k];
    tab[k] = make_zt32(dzk, k > 0 ? a.dz[k - 1] : dzk, a.dt);
  }
  const bool wet = a.wet_class && a.wet_class[cls];
  for (int o = threadIdx.x; o < TX * TY; o += NT) {
    const int oi = i0 + o % TX, oj = j0 + o / TX;
    wacc[o] = 0.0;
    wlam[o] = 0.0;
    wkz[o] = 0;
    if (!wet || oi > oi1 || oj > oj1) continue;
    const int p2 = (oi - 1) + nx * (oj - 1);
    wlam[o] = a.lambda2d[p2];
    wacc[o] = a.cwet[(long long)(cls + 1) * pl + p2];
    // zlayer is non-decreasing (checked on the host), so the layers below
    // the mixing height are a prefix of the column (wetdep.f90:37)
    const double zi = a.zi[p2];
    int kz = 0;
    while (kz < nz && a.zlayer[kz] <= zi) ++kz;
    wkz[o] = kz;
  }

  const float* __restrict__ cin = c_in + (long long)cls * a.cstride;
  float* __restrict__ cout = c_out + (long long)cls * a.cstride;
  const float* __restrict__ vkc = a.vk + (long long)cls * a.vstride;
  const float dt = a.dt;
  const float dznz = 1.0f / a.dz[nz];
  const float auxvx = a.auxvx, auxvy = a.auxvy;
  const float dtdx2h = 0.5f * a.dtdx2, dtdy2h = 0.5f * a.dtdy2;
  const int cb0 = gi + (nx + 2) * (gy0 + warp);  // c(gi, gj, 0) of row r = 0
  const int mb0 = (gi - 1) + nx * (gy0 + warp - 1);

  // ------------------------------------------------ per-position state
  unsigned kin = 0, kgx = 0, kgy = 0;  // position kinds as bit masks over r
  float o_0[RPW], o_p1[RPW], vk0[RPW], w1k[RPW], w2km[RPW], w2k[RPW], gtop[RPW];
  float ra[RPW], rb[RPW], rc[RPW], fprev[RPW], gprev[RPW], pb[RPW];
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    const int gj = gy0 + warp + NW * r;
    const bool yin = gj >= 1 && gj <= ny;
    if (xin && yin) kin |= 1u << r;
    else if ((gi == 0 || gi == nx + 1) && yin) kgx |= 1u << r;
    else if ((gj == 0 || gj == ny + 1) && xin) kgy |= 1u << r;
    o_0[r] = o_p1[r] = vk0[r] = w1k[r] = w2km[r] = w2k[r] = gtop[r] = 0.0f;
    ra[r] = rb[r] = rc[r] = fprev[r] = gprev[r] = pb[r] = 0.0f;
  }

  // issue the staged inputs of iteration t into buffer t&1; positions outside
  // the domain copy nothing (zero fill) from a clamped, valid address
  auto prefetch = [&](auto edge_c, const int t) {
    constexpr bool EDGE = decltype(edge_c)::value;
    float* sb = stage + (t & 1) * (NF * NP);
    const bool okc = t + 2 <= nz, okk = t + 1 <= nz, okm = t <= nz, okl = t >= 2;
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int p = (warp + NW * r) * HX + lane;
      const bool in = !EDGE || (kin >> r & 1u);
      const int co = in ? cb0 + NW * r * (nx + 2) : 0;
      const int mo = in ? mb0 + NW * r * nx : 0;
      if (okc) cp_async4(sb + F_C * NP + p, cin + co + (t + 2) * cs, in);
      if (okk) cp_async4(sb + F_VK * NP + p, vkc + mo + t * pl, in);
      if (okm) {
        const int m = mo + (t - 1) * pl;
        cp_async4(sb + F_VX * NP + p, a.vx + m, in);
        cp_async4(sb + F_VY * NP + p, a.vy + m, in);
        cp_async4(sb + F_L * NP + p, a.lrho + m, in);
        cp_async4(sb + F_PZ * NP + p, a.pkz + m, in);
      }
      if (okl) {
        const int m = mo + (t - 2) * pl;
        cp_async4(sb + F_L1 * NP + p, a.lrho + m, in);
        cp_async4(sb + F_PX * NP + p, a.pkx + m, in);
        cp_async4(sb + F_PY * NP + p, a.pky + m, in);
      }
    }
    cp_async_commit();
  };
  if (edge)
    prefetch(True_{}, 1);
  else
    prefetch(False_{}, 1);

  __syncthreads();  // tables and wet state
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    if (!(kin >> r & 1u)) continue;
    const int gj = gy0 + warp + NW * r;
    const int cb = cb0 + NW * r * (nx + 2), mb = mb0 + NW * r * nx;
    const float c1 = cin[cb + cs], c2 = cin[cb + 2 * cs];
    const float vk1 = __ldg(vkc + mb);
    float gb;  // setbcc bottom (setbcc.f90:19-33)
    if (vk1 >= 0.0f)
      gb = 0.0f;
    else
      gb = c1 * (1.0f + a.dz[0] * __ldg(a.vdep + (long long)cls * a.dstride + mb) / __ldg(a.rkver1 + mb));
    o_0[r] = c1;
    o_p1[r] = c2;
    vk0[r] = vk1;
    zwork(gb, c1, c2, vk1, vk1, tab[1], w1k[r], w2k[r]);
    w2km[r] = w2k[r];
    rc[r] = gb;  // diffz window: c(0) is the bottom ghost
    if (gi >= i0 && gi <= oi1 && gj >= j0 && gj <= oj1) {
      cout[cb] = clip0(gb);  // clipped ghost (sizloop.f90:77)
      if (gi == 1 && gj == 1) cout[d.C(0, 0, 0)] = clip0(c1);  // setbcc.f90:87-91
      if (gi == nx && gj == 1) cout[d.C(nx + 1, 0, 0)] = clip0(c1);
      if (gi == 1 && gj == ny) cout[d.C(0, ny + 1, 0)] = clip0(c1);
      if (gi == nx && gj == ny) cout[d.C(nx + 1, ny + 1, 0)] = clip0(c1);
    }
  }

  // ------------------------------------------------ one iteration of the march
  auto plane_generic = [&](auto edge_c, auto steady_c, const int t) {
    constexpr bool EDGE = decltype(edge_c)::value;
    constexpr bool STEADY = decltype(steady_c)::value;  // 3 <= t <= nz-2
    cp_async_wait_all();  // own staged inputs of iteration t are in shared memory
    const float* sb = stage + (t & 1) * (NF * NP);
    float s2[RPW];
    if (STEADY || t <= nz) {
      float s1[RPW];
      const ZT32 zn = tab[(STEADY || t + 1 <= nz) ? t + 1 : nz];
      // ---------------- A: setbcc ghosts + advctzc for plane t
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int hy = warp + NW * r;
        const int p = hy * HX + lane;
        float ghost = 0.0f;
        if constexpr (EDGE) {
          const int gj = gy0 + hy;
          // x-face ghosts take c(1|nx, j, t) and vx from the neighbour lane
          // (setbcc.f90:53-66)
          const float cn_up = shup(o_0[r]), cn_dn = shdn(o_0[r]);
          const float vxo = sb[F_VX * NP + p];
          const float vx_up = shup(vxo), vx_dn = shdn(vxo);
          ghost = (gi == 0) ? (vx_dn >= 0.0f ? 0.0f : cn_dn) : (vx_up <= 0.0f ? 0.0f : cn_up);
          if (gj == 0 || gj == ny + 1) {  // y-face ghosts (setbcc.f90:70-83)
            ghost = 0.0f;
            if (xin) {
              const int ja = gj == 0 ? 1 : ny;
              const float cadj = cin[gi + (nx + 2) * ja + t * cs];
              const float v = __ldg(a.vy + (t - 1) * pl + (gi - 1) + nx * (ja - 1));
              ghost = (gj == 0) ? (v >= 0.0f ? 0.0f : cadj) : (v <= 0.0f ? 0.0f : cadj);
            }
          }
        }
        {  // the column update, on every position (zero inputs outside the domain)
          float w1n, w2n, o_p2 = 0.0f, vkp = 0.0f;
          if (STEADY || t + 1 <= nz) {
            vkp = sb[F_VK * NP + p];
            if (STEADY || t + 2 <= nz) {
              o_p2 = sb[F_C * NP + p];
            } else {  // the top ghost (setbcc.f90:37-49), vkp = vk(nz)
              o_p2 = (vkp <= 0.0f) ? 0.0f : o_p1[r];
              gtop[r] = o_p2;
              const int gj = gy0 + hy;
              if (gi >= i0 && gi <= oi1 && gj >= j0 && gj <= oj1) {  // an interior position
                cout[cb0 + NW * r * (nx + 2) + (nz + 1) * cs] = clip0(o_p2);
                if (gi == 1 && gj == 1) cout[d.C(0, 0, nz + 1)] = clip0(o_p1[r]);
                if (gi == nx && gj == 1) cout[d.C(nx + 1, 0, nz + 1)] = clip0(o_p1[r]);
                if (gi == 1 && gj == ny) cout[d.C(0, ny + 1, nz + 1)] = clip0(o_p1[r]);
                if (gi == nx && gj == ny) cout[d.C(nx + 1, ny + 1, nz + 1)] = clip0(o_p1[r]);
              }
            }
            zwork(o_0[r], o_p1[r], o_p2, vkp, vk0[r], zn, w1n, w2n);
          } else {  // t == nz: work(nz+1,1) (advctzc.f90:58-64)
            w1n = dt * vk0[r] * (gtop[r] - o_0[r]) * dznz;
            w2n = w2k[r];
          }
          s1[r] = (vk0[r] > 0.0f) ? o_0[r] - w1k[r] - (w2k[r] - w2km[r]) : o_0[r] - w1n - (w2n - w2k[r]);
          w2km[r] = w2k[r];
          w2k[r] = w2n;
          w1k[r] = w1n;
          o_0[r] = o_p1[r];
          o_p1[r] = o_p2;
          vk0[r] = vkp;
        }
        if constexpr (EDGE) {
          if ((kgx | kgy) >> r & 1u) s1[r] = ghost;
        }
      }
      // ---------------- B: advctx (shuffles) and advcty (shared memory)
      auto adv_x = [&](const float* in, float* out) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int p = (warp + NW * r) * HX + lane;
          const float c0 = in[r];
          const float v = sb[F_VX * NP + p];  // 0 outside the domain
          const float cm = shup(c0), cp = shdn(c0);
          const float vm_raw = shup(v);
          float w1, w2;
          if constexpr (EDGE) {
            const float vm = gi == 1 ? v : vm_raw;  // v(max(1,q-1))
            line_work(cm, c0, cp, v, vm, auxvx, a.inv_dx, dt, w1, w2);
            if (gi == nx + 1) w1 = auxvx * vm_raw * (c0 - cm);  // work(nx+1,1) (advctx.f90:46)
          } else {
            line_work(cm, c0, cp, v, vm_raw, auxvx, a.inv_dx, dt, w1, w2);
          }
          const float w1p = shdn(w1);
          const float w2m_raw = shup(w2), w2p_raw = shdn(w2);
          if constexpr (EDGE) {
            const float w2m = gi == 1 ? w2 : w2m_raw;
            const float w2p = gi == nx ? w2 : w2p_raw;
            const float u = line_update(c0, v, w1, w1p, w2, w2m, w2p);
            out[r] = (kin >> r & 1u) ? u : c0;
          } else {
            out[r] = line_update(c0, v, w1, w1p, w2, w2m_raw, w2p_raw);
          }
        }
      };
      auto adv_y = [&](const float* in, float* out) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) P0s[(warp + NW * r) * HX + lane] = in[r];
        __syncthreads();
        // every thread is past iteration t-1: its staging buffer may be refilled
        prefetch(edge_c, t + 1);
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int hy = warp + NW * r;
          const int p = hy * HX + lane;
          float w1, w2;
          const float c0 = P0s[p], cm = P0s[p - HX], cp = P0s[p + HX];
          const float v = sb[F_VY * NP + p], vm_raw = sb[F_VY * NP + p - HX];  // vy(i, j-1)
          if constexpr (EDGE) {  // row conditions are uniform across the warp
            const int gj = gy0 + hy;
            line_work(cm, c0, cp, v, gj == 1 ? v : vm_raw, auxvy, a.inv_dy, dt, w1, w2);
            if (gj == ny + 1) w1 = auxvy * vm_raw * (c0 - cm);  // work(ny+1,1) (advcty.f90:45)
          } else {
            line_work(cm, c0, cp, v, vm_raw, auxvy, a.inv_dy, dt, w1, w2);
          }
          W1s[p] = w1;
          W2s[p] = w2;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int hy = warp + NW * r;
          const int p = hy * HX + lane;
          const float v = sb[F_VY * NP + p];
          const float w2 = W2s[p], w2m_raw = W2s[p - HX], w2p_raw = W2s[p + HX];
          if constexpr (EDGE) {
            const int gj = gy0 + hy;
            const float w2m = gj == 1 ? w2 : w2m_raw;
            const float w2p = gj == ny ? w2 : w2p_raw;
            const float u = line_update(in[r], v, W1s[p], W1s[p + HX], w2, w2m, w2p);
            out[r] = (kin >> r & 1u) ? u : in[r];
          } else {
            out[r] = line_update(in[r], v, W1s[p], W1s[p + HX], w2, w2m_raw, w2p_raw);
          }
        }
      };
      float sa[RPW];
      if (xfirst) {  // sizloop.f90:42-48
        adv_x(s1, sa);
        adv_y(sa, s2);
      } else {
        adv_y(s1, sa);
        adv_x(sa, s2);
      }
    } else {
#pragma unroll
      for (int r = 0; r < RPW; ++r) s2[r] = 0.0f;
      __syncthreads();  // the y-sweep plane of the previous iteration is read by all warps
    }
    if (!STEADY && t < 2) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int p = (warp + NW * r) * HX + lane;
        if (EDGE) gprev[r] = s2[r];  // ghost value of plane t
        ra[r] = rb[r];
        rb[r] = rc[r];
        rc[r] = s2[r];
        pb[r] = sb[F_PZ * NP + p];  // rkver*rho at plane 1
      }
      return;
    }
    // ---------------- C: diffz for plane k = t-1 (diffz.f90:22-62)
    const int k = t - 1;
    float s3[RPW];
    const ZT32 zk = tab[k];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int p = (warp + NW * r) * HX + lane;
      // window c(k-1), c(k), c(k+1); past the last plane c(nz+1) is the top
      // ghost (diffz.f90:54)
      ra[r] = rb[r];
      rb[r] = rc[r];
      rc[r] = (STEADY || t <= nz) ? s2[r] : gtop[r];
      // 1/rho at k and k+1, K*rho at k (carried) and k+1
      const float lb = sb[F_L1 * NP + p];
      if (STEADY || (k > 1 && k < nz)) {
        const float lc = sb[F_L * NP + p], pc = sb[F_PZ * NP + p];
        s3[r] = diffz_mid(pc, pb[r], rc[r], lc, rb[r], lb, fprev[r], zk);
        pb[r] = pc;
      } else if (k == 1) {
        const float lc = sb[F_L * NP + p], pc = sb[F_PZ * NP + p];
        s3[r] = diffz_bottom(pc, pb[r], rc[r], lc, rb[r], lb, ra[r], fprev[r], tab[0], tab[1]);
        pb[r] = pc;
      } else {  // k == nz
        const int m = ((kin >> r & 1u) ? mb0 + NW * r * nx : 0) + (nz - 2) * pl;
        const float la = __ldg(a.lrho + m), pa = __ldg(a.pkz + m);
        s3[r] = diffz_top(pa, la, pb[r], rc[r], rb[r], lb, ra[r], tab[nz - 1], tab[nz]);
      }
      if constexpr (EDGE) {
        if (!(kin >> r & 1u)) s3[r] = gprev[r];  // ghost value of plane k (unchanged by the sweeps)
        gprev[r] = s2[r];
      }
    }
    // ---------------- D: diffx (shuffles) and diffy (shared memory)
    auto dif_x = [&](const float* in, float* out) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int p = (warp + NW * r) * HX + lane;
        const float l0 = sb[F_L1 * NP + p], P0 = sb[F_PX * NP + p];
        const float c0 = in[r];
        const float cm = shup(c0), cp = shdn(c0);
        const float lm = shup(l0), lp = shdn(l0);
        const float Pm = shup(P0), Pp = shdn(P0);
        if constexpr (EDGE) {
          float u = diff_mid(cm, c0, cp, lm, l0, lp, Pm, P0, Pp, dtdx2h);
          if (gi == 1 || gi == nx) u = diff_cell(gi == 1, gi == nx, cm, c0, cp, lm, l0, lp, Pm, P0, Pp, dtdx2h);
          out[r] = (kin >> r & 1u) ? u : c0;
        } else {
          out[r] = diff_mid(cm, c0, cp, lm, l0, lp, Pm, P0, Pp, dtdx2h);
        }
      }
    };
    auto dif_y = [&](const float* in, float* out) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) P1s[(warp + NW * r) * HX + lane] = in[r];
      __syncthreads();
      const float* L = sb + F_L1 * NP;
      const float* PY = sb + F_PY * NP;
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int hy = warp + NW * r;
        const int p = hy * HX + lane;
        const int hm = p - HX, hp = p + HX;
        if constexpr (EDGE) {
          const int gj = gy0 + hy;
          const float u = diff_cell(gj == 1, gj == ny, P1s[hm], in[r], P1s[hp], L[hm], L[p], L[hp], PY[hm],
                                    PY[p], PY[hp], dtdy2h);
          out[r] = (kin >> r & 1u) ? u : in[r];
        } else {
          out[r] = diff_mid(P1s[hm], in[r], P1s[hp], L[hm], L[p], L[hp], PY[hm], PY[p], PY[hp], dtdy2h);
        }
      }
    };
    float s3a[RPW], s4[RPW];
    if (xfirst) {  // sizloop.f90:55-61
      dif_x(s3, s3a);
      dif_y(s3a, s4);
    } else {
      dif_y(s3, s3a);
      dif_x(s3a, s4);
    }
    // ---------------- E: wetdep, accum, clip, store (plane k)
    const double dzk64 = a.dz64[k];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int hy = warp + NW * r;
      const int gj = gy0 + hy;
      const int cidx = cb0 + NW * r * (nx + 2) + k * cs;
      bool out_cell;
      if constexpr (EDGE) {
        const bool rows_out = gj >= j0 && gj <= oj1;
        const bool cols_out = gi >= i0 && gi <= oi1;
        if ((kgx >> r & 1u) && rows_out && ((gi == 0 && i0 == 1) || (gi == nx + 1 && oi1 == nx))) {
          cout[cidx] = clip0(s3[r]);
          continue;
        }
        if ((kgy >> r & 1u) && cols_out && ((gj == 0 && j0 == 1) || (gj == ny + 1 && oj1 == ny))) {
          cout[cidx] = clip0(s3[r]);
          continue;
        }
        out_cell = (kin >> r & 1u) && rows_out && cols_out;
      } else {
        out_cell = lane >= 3 && lane < 3 + TX && hy >= 3 && hy < 3 + TY;
      }
      if (!out_cell) continue;
      float cnew = s4[r];
      if (wet) {
        const int o = (gi - i0) + TX * (gj - j0);
        if (k <= wkz[o]) {  // wetdep (wetdep.f90:37-49)
          wacc[o] = wacc[o] + dzk64 * wlam[o] * (double)cnew;
          cnew = (float)((double)cnew * (1.0 - wlam[o]));
        }
      }
      if (!STEADY && k == 1 && commit) {  // accum (accum.f90:17-25), binary64
        const int mb = mb0 + NW * r * nx;
        double* cd = a.cdry + (long long)(cls + 1) * pl + mb;
        const double vsd = a.vset64[(long long)cls * a.vstride + mb] + a.vdep64[(long long)cls * pl + mb];
        *cd = *cd - a.dt64 * (double)cnew * fmin2(0.0, vsd);
      }
      cout[cidx] = clip0(cnew);
    }
  };

  // The steady planes of interior tiles: the same formulas on pairs of rows
  // (r = 2q, 2q+1) carried as float2 values.
  auto plane_packed = [&](const int t) {
    constexpr int RP = RPW / 2;
    static_assert(RPW % 2 == 0, "rows per warp must pair up");
    cp_async_wait_all();
    const float* sb = stage + (t & 1) * (NF * NP);
    auto rowpos = [&](int q) { return (warp + NW * 2 * q) * HX + lane; };  // row 2q; row 2q+1 is +NW*HX
    auto ld2 = [&](const float* base, int p0) { return make_float2(base[p0], base[p0 + NW * HX]); };
    auto pk = [](const float* v, int q) { return make_float2(v[2 * q], v[2 * q + 1]); };
    auto up = [](float* v, int q, float2 x) {
      v[2 * q] = x.x;
      v[2 * q + 1] = x.y;
    };
    float2 s2v[RP];
    {
      const ZT32 zn = tab[t + 1];
      float2 s1v[RP];
#pragma unroll
      for (int q = 0; q < RP; ++q) {  // A: advctzc
        const int p0 = rowpos(q);
        const float2 vkp = ld2(sb + F_VK * NP, p0), o2 = ld2(sb + F_C * NP, p0);
        const float2 O0 = pk(o_0, q), O1 = pk(o_p1, q), VK0 = pk(vk0, q);
        const float2 W1K = pk(w1k, q), W2KM = pk(w2km, q), W2K = pk(w2k, q);
        float2 w1n, w2n;
        zwork2(O0, O1, o2, vkp, VK0, zn, w1n, w2n);
        s1v[q] = line_update2(O0, VK0, W1K, w1n, W2K, W2KM, w2n);
        up(w2km, q, W2K);
        up(w2k, q, w2n);
        up(w1k, q, w1n);
        up(o_0, q, O1);
        up(o_p1, q, o2);
        up(vk0, q, vkp);
      }
      auto adv_x2 = [&](const float2* in, float2* out) {
#pragma unroll
        for (int q = 0; q < RP; ++q) {
          const int p0 = rowpos(q);
          const float2 c0 = in[q], v = ld2(sb + F_VX * NP, p0);
          float2 w1, w2;
          line_work2(shup2(c0), c0, shdn2(c0), v, shup2(v), auxvx, a.inv_dx, dt, w1, w2);
          out[q] = line_update2(c0, v, w1, shdn2(w1), w2, shup2(w2), shdn2(w2));
        }
      };
      auto adv_y2 = [&](const float2* in, float2* out) {
#pragma unroll
        for (int q = 0; q < RP; ++q) {
          const int p0 = rowpos(q);
          P0s[p0] = in[q].x;
          P0s[p0 + NW * HX] = in[q].y;
        }
        __syncthreads();
        prefetch(False_{}, t + 1);
#pragma unroll
        for (int q = 0; q < RP; ++q) {
          const int p0 = rowpos(q);
          float2 w1, w2;
          line_work2(ld2(P0s - HX, p0), in[q], ld2(P0s + HX, p0), ld2(sb + F_VY * NP, p0),
                     ld2(sb + F_VY * NP - HX, p0), auxvy, a.inv_dy, dt, w1, w2);
          W1s[p0] = w1.x;
          W1s[p0 + NW * HX] = w1.y;
          W2s[p0] = w2.x;
          W2s[p0 + NW * HX] = w2.y;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < RP; ++q) {
          const int p0 = rowpos(q);
          out[q] = line_update2(in[q], ld2(sb + F_VY * NP, p0), ld2(W1s, p0), ld2(W1s + HX, p0), ld2(W2s, p0),
                                ld2(W2s - HX, p0), ld2(W2s + HX, p0));
        }
      };
      float2 sav[RP];
      if (xfirst) {  // sizloop.f90:42-48
        adv_x2(s1v, sav);
        adv_y2(sav, s2v);
      } else {
        adv_y2(s1v, sav);
        adv_x2(sav, s2v);
      }
    }
    // C: diffz for plane k = t-1 (an interior plane)
    const int k = t - 1;
    const ZT32 zk = tab[k];
    float2 s3v[RP];
#pragma unroll
    for (int q = 0; q < RP; ++q) {
      const int p0 = rowpos(q);
      const float2 RB = pk(rc, q), RC = s2v[q];
      up(rb, q, RB);
      up(rc, q, RC);
      const float2 lb = ld2(sb + F_L1 * NP, p0), lc = ld2(sb + F_L * NP, p0), pc = ld2(sb + F_PZ * NP, p0);
      float2 fp = pk(fprev, q);
      s3v[q] = diffz_mid2(pc, pk(pb, q), RC, lc, RB, lb, fp, zk);
      up(fprev, q, fp);
      up(pb, q, pc);
    }
    // D: diffx and diffy
    auto dif_x2 = [&](const float2* in, float2* out) {
#pragma unroll
      for (int q = 0; q < RP; ++q) {
        const int p0 = rowpos(q);
        const float2 l0 = ld2(sb + F_L1 * NP, p0), P0 = ld2(sb + F_PX * NP, p0), c0 = in[q];
        out[q] = diff_mid2(shup2(c0), c0, shdn2(c0), shup2(l0), l0, shdn2(l0), shup2(P0), P0, shdn2(P0), dtdx2h);
      }
    };
    auto dif_y2 = [&](const float2* in, float2* out) {
#pragma unroll
      for (int q = 0; q < RP; ++q) {
        const int p0 = rowpos(q);
        P1s[p0] = in[q].x;
        P1s[p0 + NW * HX] = in[q].y;
      }
      __syncthreads();
      const float* L = sb + F_L1 * NP;
      const float* PY = sb + F_PY * NP;
#pragma unroll
      for (int q = 0; q < RP; ++q) {
        const int p0 = rowpos(q);
        out[q] = diff_mid2(ld2(P1s - HX, p0), in[q], ld2(P1s + HX, p0), ld2(L - HX, p0), ld2(L, p0), ld2(L + HX, p0),
                           ld2(PY - HX, p0), ld2(PY, p0), ld2(PY + HX, p0), dtdy2h);
      }
    };
    float2 s3a[RP], s4v[RP];
    if (xfirst) {  // sizloop.f90:55-61
      dif_x2(s3v, s3a);
      dif_y2(s3a, s4v);
    } else {
      dif_y2(s3v, s3a);
      dif_x2(s3a, s4v);
    }
    // E: wetdep, clip, store (plane k; no accum above k = 1)
    const double dzk64 = a.dz64[k];
    const bool lane_out = lane >= 3 && lane < 3 + TX;
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int hy = warp + NW * r;
      if (!(lane_out && hy >= 3 && hy < 3 + TY)) continue;
      float cnew = (r & 1) ? s4v[r >> 1].y : s4v[r >> 1].x;
      if (wet) {
        const int o = (lane - 3) + TX * (hy - 3);
        if (k <= wkz[o]) {  // wetdep (wetdep.f90:37-49)
          wacc[o] = wacc[o] + dzk64 * wlam[o] * (double)cnew;
          cnew = (float)((double)cnew * (1.0 - wlam[o]));
        }
      }
      cout[cb0 + NW * r * (nx + 2) + k * cs] = clip0(cnew);
    }
  };

  auto plane = [&](auto edge_c, auto steady_c, const int t) {
    if constexpr (!decltype(edge_c)::value && decltype(steady_c)::value)
      plane_packed(t);
    else
      plane_generic(edge_c, steady_c, t);
  };

  auto march = [&](auto edge_c) {
    for (int t = 1; t <= 2; ++t) plane(edge_c, False_{}, t);
    for (int t = 3; t <= nz - 2; ++t) plane(edge_c, True_{}, t);
    for (int t = max(3, nz - 1); t <= nz + 1; ++t) plane(edge_c, False_{}, t);
  };
  if (edge)
    march(True_{});
  else
    march(False_{});

  if (wet && commit) {
    __syncthreads();
    for (int o = threadIdx.x; o < TX * TY; o += NT) {
      const int oi = i0 + o % TX, oj = j0 + o / TX;
      if (oi > oi1 || oj > oj1) continue;
      a.cwet[(long long)(cls + 1) * pl + (oi - 1) + nx * (oj - 1)] = wacc[o];
    }
  }
}

template <int HY, int NW>
__global__ void __launch_bounds__(32 * NW, (32 * NW >= 512 ? 1 : 2)) k_step_fused(const FusedArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fused_tile<HY, NW>(a, a.c_in, a.c_out, a.xfirst, 1, (int)(blockIdx.x % a.ncls), (int)(blockIdx.x / a.ncls),
                     smem_raw);
}

// ------------------------------------------------------------ batched form
// The step of every scenario of a batch in one persistent launch: the work
// items are (scenario, tile, class), numbered scenario by scenario
// (item_off[s] .. item_off[s+1]-1, class fastest); each CTA takes the next
// item from a counter until none is left.  A scenario's arguments live in
// constant memory; its buffers alternate with the number of batch steps it
// has taken (bstep[s] even: c_in -> c_out, odd: c_out -> c_in), and the x/y
// order follows iiter = iiter0[s] + bstep[s] + 1 (sizloop.f90:42-48).
__constant__ FusedArgs c_batch[F3D_BATCH_MAX];
static_assert(sizeof(FusedArgs) * F3D_BATCH_MAX <= 48 * 1024, "batch argument table exceeds constant memory");

template <int HY, int NW>
__global__ void __launch_bounds__(32 * NW, (32 * NW >= 512 ? 1 : 2))
    k_step_fused_batch(const int* __restrict__ item_off, int nscen, int* counter,
                       const int* __restrict__ bstep, const int* __restrict__ iiter0, int commit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const int total = item_off[nscen];
  for (;;) {
    __syncthreads();  // the previous item is done with shared memory
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    int lo = 0, hi = nscen;  // item_off[lo] <= item < item_off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (item_off[mid] <= item) lo = mid;
      else hi = mid;
    }
    const FusedArgs& a = c_batch[lo];
    const int local = item - item_off[lo];
    const int bs = bstep[lo];
    const float* cin = (bs & 1) ? a.c_out : a.c_in;
    float* cout = (bs & 1) ? const_cast<float*>(a.c_in) : a.c_out;
    const int iiter = iiter0[lo] + bs + 1;
    fused_tile<HY, NW>(a, cin, cout, (iiter % 2 == 0) ? 1 : 0, commit, local % a.ncls, local / a.ncls, smem_raw);
  }
}

template <int HY>
size_t fused_smem(int nz) {
  return sizeof(float) * ((2 * NF + 4) * 32 * HY + 2 * 32) +
         (2 * sizeof(double) + sizeof(int)) * 26 * (HY - 6) + sizeof(ZT32) * (size_t)(nz + 1);
}

// persistent grid: as many CTAs as fit on the device at once
template <int HY, int NW>
int fused_batch_grid_t(int max_nz) {
  const size_t sm = fused_smem<HY>(max_nz);
  if (cudaFuncSetAttribute(k_step_fused_batch<HY, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
      cudaSuccess)
    return -1;
  int per_sm = 0, nsm = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_fused_batch<HY, NW>, 32 * NW, sm) !=
          cudaSuccess)
    return -1;
  return per_sm < 1 ? -1 : per_sm * nsm;
}

template <int HY, int NW>
void launch_fused_batch_t(int grid, const int* item_off, int nscen, int* counter, const int* bstep,
                          const int* iiter0, int commit, int max_nz, cudaStream_t s) {
  k_step_fused_batch<HY, NW><<<grid, 32 * NW, fused_smem<HY>(max_nz), s>>>(item_off, nscen, counter, bstep,
                                                                            iiter0, commit);
  count_launch();
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

int fused_tiles(int nx, int ny, int shape) {
  if (shape == 3) return ((nx + 57) / 58) * ((ny + 25) / 26);
  const int TY = (shape == 1 ? 64 : 32) - 6;
  return ((nx + 25) / 26) * ((ny + TY - 1) / TY);
}

int upload_batch_args(const FusedArgs* h, int n, cudaStream_t s) {
  if (n > F3D_BATCH_MAX) return 1;
  if (cudaMemcpyToSymbolAsync(c_batch, h, sizeof(FusedArgs) * (size_t)n, 0, cudaMemcpyHostToDevice, s) !=
      cudaSuccess)
    return 1;
  return upload_batch_args2(h, n, s);
}

int fused_batch_grid(int shape, int max_nz) {
  switch (shape) {
    case 3:
      return fused2_batch_grid(max_nz);
    case 1:
      return fused_batch_grid_t<64, 16>(max_nz);
    case 2:
      return fused_batch_grid_t<32, 16>(max_nz);
    default:
      return fused_batch_grid_t<32, 8>(max_nz);
  }
}

void launch_step_fused_batch(int shape, int grid, const int* item_off, int nscen, int split, int total,
                             int* counter, const int* bstep, const int* iiter0, int commit, int max_nz,
                             const F2Maps* maps, cudaStream_t s, const BatchFork* fork) {
  switch (shape) {
    case 3:
      launch_step_fused2_batch(grid, item_off, nscen, split, total, counter, bstep, iiter0, commit, max_nz, maps, s,
                               fork);
      break;
    case 1:
      launch_fused_batch_t<64, 16>(grid, item_off, nscen, counter, bstep, iiter0, commit, max_nz, s);
      break;
    case 2:
      launch_fused_batch_t<32, 16>(grid, item_off, nscen, counter, bstep, iiter0, commit, max_nz, s);
      break;
    default:
      launch_fused_batch_t<32, 8>(grid, item_off, nscen, counter, bstep, iiter0, commit, max_nz, s);
      break;
  }
}

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

// vz + vset per class in binary32 (the vertical velocity of advctzc.f90:23).
__global__ void k_vk32(long long n, int nc, const float* vz, const float* vset, float* vk) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = vz[q];
    for (int c = 0; c < nc; ++c) vk[c * n + q] = v + vset[c * n + q];
  }
}

void launch_vk32(long long n, int nc, const float* vz, const float* vset, float* vk, cudaStream_t s) {
  const int nb = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  k_vk32<<<nb, 256, 0, s>>>(n, nc, vz, vset, vk);
  count_launch();
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

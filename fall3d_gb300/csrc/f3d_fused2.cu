// f3d_fused2.cu -- the precision form's whole transport step in one kernel,
// two columns per lane.
//
// Same march as f3d_fused.cu (one CTA per tile and class, up the column;
// iteration t: setbcc + advctzc and advctx/advcty on plane t, then diffz,
// diffx/diffy, wetdep, accum, clip and store on plane t-1), laid out for
// fewer instructions per cell:
//
//  * a lane owns two neighbouring columns, so every field of a position pair
//    is one 64-bit value: f32x2 arithmetic, 64-bit shared-memory accesses
//    and 8-byte asynchronous copies; an x neighbour costs one shuffle per
//    pair instead of one per cell;
//  * the tile region is 64 x 32 (58 x 26 output cells, 16 warps, two rows
//    per warp), so fewer halo cells are recomputed per output cell;
//  * the met fields come in the halo layout of c, so one offset addresses
//    all nine staged fields of a position and interior tiles need no bounds
//    logic at all.
//
// Every cell gets the bits of the scalar formulas (f3d_fused_math.cuh).
#include <algorithm>
#include <type_traits>

#include "f3d_fused_math.cuh"

namespace f3d {

namespace {

using namespace fz;

constexpr int HX = 64, HY = 32, NW = 16, NT = 32 * NW, RPW = HY / NW, TX = HX - 6, TY = HY - 6,
              NP = HX * HY;
// The staged fields are boxes of RS x HY values: a tensor copy's first column
// must lie on a 16-byte boundary, so a box starts at the region's first
// column rounded down to a multiple of 4 (gx0 is even: the region then
// starts 0 or 2 values into the box) and is 4 values wider than the region.
constexpr int RS = HX + 4, FS = RS * HY;
constexpr int GUARD = 512;  // bytes before the staging area (reads one row above a field)

// value of the column to the left / right of each of the lane's two columns
__device__ __forceinline__ float2 left2(float2 v) { return make_float2(shup(v.y), v.x); }
__device__ __forceinline__ float2 right2(float2 v) { return make_float2(v.y, shdn(v.x)); }
__device__ __forceinline__ float2 sel2(bool cx, bool cy, float2 a, float2 b) {
  return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}
__device__ __forceinline__ float cmp(const float2& v, int c) { return c ? v.y : v.x; }
__device__ __forceinline__ float& cmp(float2& v, int c) { return c ? v.y : v.x; }

__device__ __forceinline__ void cp_async8(unsigned dst, const float* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 8 : 0));
}
__device__ __forceinline__ void cp_async4s(unsigned dst, const float* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 4 : 0));
}

__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

size_t fused2_smem(int nz) {
  return 128 + GUARD + sizeof(float) * ((size_t)2 * NF * FS + 4 * (size_t)NP + HX) +
         (2 * sizeof(double) + sizeof(int)) * TX * TY + sizeof(ZT32) * (size_t)(nz + 1) + 32;
}

// ------------------------------------------------ tensor copies (TMA)
// Elected thread 0 stages the eight met fields of a plane with
// cp.async.bulk.tensor into the buffer of that plane; completion is counted
// in bytes on the buffer's mbarrier, which every thread waits on.
__device__ __forceinline__ void mbar_init(unsigned bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// waits for the phase of the given parity, at most ~2^20 polls; false on a timeout
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (int i = 0; i < (1 << 20); ++i) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load3(unsigned dst, const CUtensorMap* map, int x, int y, int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// One tile of one class (see fused_tile in f3d_fused.cu for the arguments).
// P8: nx is even, so every column pair starts on an 8-byte boundary and lies
// wholly inside or wholly outside the halo array; otherwise the pairs are
// copied and stored one value at a time.
// The met fields come by tensor copies (maps: this scenario's tensor maps),
// c by every thread's own cp.async copies.
template <bool P8>
__device__ __forceinline__ void fused2_tile(const FusedArgs& a, const F2Maps* maps, const float* c_in, float* c_out,
                                            const int xfirst, const int commit, const int cls, const int tile,
                                            unsigned char* smem_raw) {
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<size_t>(smem_raw) + 127) & ~(size_t)127);
  float* stage = reinterpret_cast<float*>(base + GUARD);  // [2][NF][FS], 128-byte aligned fields
  float* P0s = stage + 2 * NF * FS;
  float* W1s = P0s + NP;
  float* W2s = W1s + NP;
  float* P1s = W2s + NP;
  double* wacc = reinterpret_cast<double*>(P1s + NP + HX);
  double* wlam = wacc + TX * TY;
  int* wkz = reinterpret_cast<int*>(wlam + TX * TY);
  ZT32* tab = reinterpret_cast<ZT32*>(wkz + TX * TY);
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(
      (reinterpret_cast<size_t>(tab + (a.d.nz + 1)) + 7) & ~(size_t)7);  // one per staging buffer

  const Dims d = a.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int tiles_x = (nx + TX - 1) / TX;
  const int i0 = 1 + (tile % tiles_x) * TX, j0 = 1 + (tile / tiles_x) * TY;
  const int gx0 = i0 - 3, gy0 = j0 - 3;
  const int oi1 = min(nx, i0 + TX - 1), oj1 = min(ny, j0 + TY - 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gi = gx0 + 2 * lane;  // the lane's first column; the second is gi + 1
  const int px = nx + 2;          // halo row pitch of c
  const int cs = px * (ny + 2);   // halo plane of c
  const int hp = a.hpitch;        // row pitch of the met fields (padded to a multiple of 4)
  const int hs = hp * (ny + 2);   // their plane
  const int xs = gx0 & ~3;        // first column of the staged boxes
  const int sft = gx0 - xs;       // the region's offset in a box row (0 or 2)
  const int pl = nx * ny;
  const bool edge = !(gx0 >= 1 && gx0 + HX - 1 <= nx && gy0 >= 1 && gy0 + HY - 1 <= ny);
  const bool xedge = gx0 <= 1 || gx0 + HX - 1 >= nx;  // the region holds column 1 or nx

  const unsigned mbar0 = (unsigned)__cvta_generic_to_shared(mbar);
  if (threadIdx.x == 0) {
    mbar_init(mbar0);
    mbar_init(mbar0 + 8);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int k = threadIdx.x; k <= nz; k += NT) {
    const float dzk = a.dz[k];
    tab[k] = make_zt32(dzk, k > 0 ? a.dz[k - 1] : dzk, a.dt);
  }
  const bool wet = a.wet_class && a.wet_class[cls];
  __shared__ int s_kzmax;  // the highest wet layer of the tile: above it the wet code is skipped
  if (threadIdx.x == 0) s_kzmax = 0;
  __syncthreads();
  for (int o = threadIdx.x; o < TX * TY; o += NT) {
    const int oi = i0 + o % TX, oj = j0 + o / TX;
    wacc[o] = 0.0;
    wlam[o] = 0.0;
    wkz[o] = 0;
    if (!wet || oi > oi1 || oj > oj1) continue;
    const int p2 = (oi - 1) + nx * (oj - 1);
    wlam[o] = a.lambda2d[p2];
    wacc[o] = a.cwet[(long long)(cls + 1) * pl + p2];
    // zlayer is non-decreasing (checked on the host): the layers below the
    // mixing height are a prefix of the column (wetdep.f90:37)
    const double zi = a.zi[p2];
    int kz = 0;
    while (kz < nz && a.zlayer[kz] <= zi) ++kz;
    wkz[o] = kz;
    if (kz > 0) atomicMax(&s_kzmax, kz);
  }

  const float* __restrict__ cin = c_in + (long long)cls * a.cstride;
  float* __restrict__ cout = c_out + (long long)cls * a.cstride;
  const float* __restrict__ vkc = a.vkh + (long long)cls * a.hstride;
  const float dt = a.dt;
  const float dznz = 1.0f / a.dz[nz];
  const float auxvx = a.auxvx, auxvy = a.auxvy;
  const float dtdx2h = 0.5f * a.dtdx2, dtdy2h = 0.5f * a.dtdy2;

  // ------------------------------------------------ per-position state
  // bit 2r+c: row r (gj = gy0 + 2*warp + r), column c (gi + c); a warp owns
  // two adjacent rows, so each row's y-neighbour on the other side is the
  // same lane's other row
  unsigned kin = 0, kgx = 0, kgy = 0, inr = 0;  // inr: the pair of row r lies in the halo array
  int h0[RPW];                                  // halo offset of (gi, gj, plane 0), clamped
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    const int gj = gy0 + 2 * warp + r;
    const bool yin = gj >= 1 && gj <= ny;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int g = gi + c;
      const bool xin = g >= 1 && g <= nx;
      const unsigned bit = 1u << (2 * r + c);
      if (xin && yin) kin |= bit;
      else if ((g == 0 || g == nx + 1) && yin) kgx |= bit;
      else if ((gj == 0 || gj == ny + 1) && xin) kgy |= bit;
      if (g >= 0 && g <= nx + 1 && gj >= 0 && gj <= ny + 1) inr |= bit;
    }
    h0[r] = (inr >> (2 * r) & 1u) ? gi + px * gj : cs;  // clamped for pairs outside (plane 1 stays in range)
  }
  float2 o_0[RPW], o_p1[RPW], vk0[RPW], w1k[RPW], w2km[RPW], w2k[RPW], gtop[RPW];
  float2 ra[RPW], rb[RPW], rc[RPW], fprev[RPW], gprev[RPW], pb[RPW];
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    o_0[r] = o_p1[r] = vk0[r] = w1k[r] = w2km[r] = w2k[r] = gtop[r] = make_float2(0.0f, 0.0f);
    ra[r] = rb[r] = rc[r] = fprev[r] = gprev[r] = pb[r] = make_float2(0.0f, 0.0f);
  }
  const unsigned stage0 = (unsigned)__cvta_generic_to_shared(stage);
  const unsigned sbase = stage0 + 4u * (unsigned)(2 * warp * RS + sft + 2 * lane);
  bool timed_out = false;

  // the staged inputs of iteration t into buffer t&1 (fields as in
  // f3d_fused.cu): c by each thread for its own positions (positions outside
  // the halo array copy nothing: zero fill), the met boxes by thread 0's
  // tensor copies (outside the arrays: zero fill).  Group 0: the fields the
  // advection phases read (c, vz+vset, vx, vy); group 1: those the diffusion
  // phases read (1/rho, K*rho); 2: both.  Group 0 of iteration t+1 is issued
  // as iteration t starts where every warp has passed the last barrier of
  // iteration t-1 (after which nobody reads those fields of that buffer),
  // group 1 after the first barrier of iteration t.
  auto prefetch = [&](auto edge_c, const int t, const int group) {
    constexpr bool EDGE = decltype(edge_c)::value;
    const unsigned sb = sbase + 4u * (unsigned)((t & 1) * NF * FS);
    const bool g0 = group != 1, g1 = group != 0;
    const bool okc = g0 && t + 2 <= nz, okk = g0 && t + 1 <= nz, okv = g0 && t <= nz, okm = g1 && t <= nz,
               okl = g1 && t >= 2 && t <= nz + 1;
    {
      if (threadIdx.x == 0) {
        const unsigned bar = mbar0 + 8u * (unsigned)(t & 1);
        const unsigned db = stage0 + 4u * (unsigned)((t & 1) * NF * FS);
        // the warps' reads of this buffer (ordered before this point by a
        // block barrier) come before the tensor copies overwrite it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (g0) {  // the buffer's next phase: every met box of plane t, both groups
          const unsigned n = (unsigned)((t + 1 <= nz) + 4 * (t <= nz) + 3 * (t >= 2 && t <= nz + 1));
          if (n) mbar_expect(bar, n * (unsigned)(FS * sizeof(float)));
        }
        auto ld = [&](int field, int map, int z) { tma_load3(db + 4u * (unsigned)(field * FS), &maps->m[map], xs, gy0, z, bar); };
        if (okk) ld(F_VK, F2Maps::VK, cls * (nz + 2) + t + 1);
        if (okv) {
          ld(F_VX, F2Maps::VX, t);
          ld(F_VY, F2Maps::VY, t);
        }
        if (okm) {
          ld(F_L, F2Maps::L, t);
          ld(F_PZ, F2Maps::PZ, t);
        }
        if (okl) {
          ld(F_L1, F2Maps::L, t - 1);
          ld(F_PX, F2Maps::PX, t - 1);
          ld(F_PY, F2Maps::PY, t - 1);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const unsigned dst = sb + 4u * (unsigned)(r * RS);
      const int ht = h0[r] + t * cs;  // this row's offset at plane t (c)
      const bool v0 = !EDGE || (inr >> (2 * r) & 1u), v1 = !EDGE || (inr >> (2 * r + 1) & 1u);
      auto cp = [&](int field, const float* src, int off) {
        const unsigned dd = dst + 4u * (unsigned)(field * FS);
        if constexpr (P8) {
          (void)v1;
          cp_async8(dd, src + off, v0);
        } else {  // an odd nx: a pair may straddle the last ghost column
          cp_async4s(dd, src + off, v0);
          cp_async4s(dd + 4u, v1 ? src + off + 1 : src + off, v1);
        }
      };
      if (okc) cp(F_C, cin, ht + 2 * cs);
    }
    cp_async_commit();
  };
  // all staged inputs of iteration t are in buffer t&1
  auto staged = [&](const int t) {
    cp_async_wait_all();
    if (!mbar_wait(mbar0 + 8u * (unsigned)(t & 1), (unsigned)(((t - 1) >> 1) & 1))) timed_out = true;
  };
  if (edge)
    prefetch(True_{}, 1, 2);
  else
    prefetch(False_{}, 1, 2);

  __syncthreads();  // tables and wet state
  // bottom ghost, first window (setbcc.f90:19-33, advctzc work(1))
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    const int gj = gy0 + 2 * warp + r;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      if (!(kin >> (2 * r + c) & 1u)) continue;
      const int g = gi + c;
      const int hb = g + px * gj, mb = (g - 1) + nx * (gj - 1);
      const float c1 = cin[hb + cs], c2 = cin[hb + 2 * cs];
      const float vk1 = __ldg(vkc + g + hp * gj + hs);
      float gb;
      if (vk1 >= 0.0f)
        gb = 0.0f;
      else
        gb = c1 * (1.0f + a.dz[0] * __ldg(a.vdep + (long long)cls * a.dstride + mb) / __ldg(a.rkver1 + mb));
      cmp(o_0[r], c) = c1;
      cmp(o_p1[r], c) = c2;
      cmp(vk0[r], c) = vk1;
      float w1, w2;
      zwork(gb, c1, c2, vk1, vk1, tab[1], w1, w2);
      cmp(w1k[r], c) = w1;
      cmp(w2k[r], c) = w2;
      cmp(w2km[r], c) = w2;
      cmp(rc[r], c) = gb;
      if (g >= i0 && g <= oi1 && gj >= j0 && gj <= oj1) {
        cout[hb] = clip0(gb);  // clipped ghost (sizloop.f90:77)
        if (g == 1 && gj == 1) cout[d.C(0, 0, 0)] = clip0(c1);  // setbcc.f90:87-91
        if (g == nx && gj == 1) cout[d.C(nx + 1, 0, 0)] = clip0(c1);
        if (g == 1 && gj == ny) cout[d.C(0, ny + 1, 0)] = clip0(c1);
        if (g == nx && gj == ny) cout[d.C(nx + 1, ny + 1, 0)] = clip0(c1);
      }
    }
  }

  // ------------------------------------------------ one iteration of the march
  auto plane = [&](auto edge_c, auto steady_c, const int t) {
    constexpr bool EDGE = decltype(edge_c)::value;
    constexpr bool STEADY = decltype(steady_c)::value;  // 3 <= t <= nz-2
    staged(t);
    // from iteration 3 on, the previous iteration ended with the diffy
    // barrier, after which no warp reads its advection fields
    const bool early = STEADY || (t >= 3 && t <= nz);
    if (early) prefetch(edge_c, t + 1, 0);
    const float* sb = stage + (t & 1) * (NF * FS) + 2 * warp * RS + sft + 2 * lane;  // this lane's row-0 position
    auto at = [&](int field, int r) { return sb + field * FS + r * RS; };
    auto km = [&](int r, int c) { return (kin >> (2 * r + c) & 1u) != 0; };
    float2 s2[RPW];
    if (STEADY || t <= nz) {
      float2 s1[RPW];
      const ZT32 zn = tab[(STEADY || t + 1 <= nz) ? t + 1 : nz];
      // ---------------- A: setbcc ghosts + advctzc for plane t
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int gj = gy0 + 2 * warp + r;
        float2 ghost = make_float2(0.0f, 0.0f);
        if constexpr (EDGE) {
          // x-face ghosts from the neighbouring column's original c and vx (setbcc.f90:53-66)
          const float2 cL = left2(o_0[r]), cR = right2(o_0[r]);
          const float2 vxo = lds2(at(F_VX, r));
          const float2 vL = left2(vxo), vR = right2(vxo);
#pragma unroll
          for (int c = 0; c < 2; ++c)
            cmp(ghost, c) = (gi + c == 0) ? (cmp(vR, c) >= 0.0f ? 0.0f : cmp(cR, c))
                                          : (cmp(vL, c) <= 0.0f ? 0.0f : cmp(cL, c));
          if (gj == 0 || gj == ny + 1) {  // y-face ghosts (setbcc.f90:70-83)
            const int ja = gj == 0 ? 1 : ny;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
              const int g = gi + c;
              float gv = 0.0f;
              if (g >= 1 && g <= nx) {
                const float cadj = cin[g + px * ja + t * cs];
                const float v = __ldg(a.vyh + g + hp * ja + t * hs);
                gv = (gj == 0) ? (v >= 0.0f ? 0.0f : cadj) : (v <= 0.0f ? 0.0f : cadj);
              }
              cmp(ghost, c) = gv;
            }
          }
        }
        {  // the column update, on every position
          float2 w1n, w2n, o_p2 = make_float2(0.0f, 0.0f), vkp = make_float2(0.0f, 0.0f);
          if (STEADY || t + 1 <= nz) {
            vkp = lds2(at(F_VK, r));
            if (STEADY || t + 2 <= nz) {
              o_p2 = lds2(at(F_C, r));
            } else {  // the top ghost (setbcc.f90:37-49), vkp = vk(nz)
#pragma unroll
              for (int c = 0; c < 2; ++c) {
                cmp(o_p2, c) = (cmp(vkp, c) <= 0.0f) ? 0.0f : cmp(o_p1[r], c);
                const int g = gi + c;
                if (g >= i0 && g <= oi1 && gj >= j0 && gj <= oj1) {  // an interior position
                  const int hb = g + px * gj;
                  const float top = cmp(o_p1[r], c);
                  cout[hb + (nz + 1) * cs] = clip0(cmp(o_p2, c));
                  if (g == 1 && gj == 1) cout[d.C(0, 0, nz + 1)] = clip0(top);
                  if (g == nx && gj == 1) cout[d.C(nx + 1, 0, nz + 1)] = clip0(top);
                  if (g == 1 && gj == ny) cout[d.C(0, ny + 1, nz + 1)] = clip0(top);
                  if (g == nx && gj == ny) cout[d.C(nx + 1, ny + 1, nz + 1)] = clip0(top);
                }
              }
              gtop[r] = o_p2;
            }
            zwork2(o_0[r], o_p1[r], o_p2, vkp, vk0[r], zn, w1n, w2n);
          } else {  // t == nz: work(nz+1,1) (advctzc.f90:58-64)
            w1n = mul2(mul2(mul2(splat(dt), vk0[r]), sub2(gtop[r], o_0[r])), splat(dznz));
            w2n = w2k[r];
          }
          s1[r] = line_update2(o_0[r], vk0[r], w1k[r], w1n, w2k[r], w2km[r], w2n);
          w2km[r] = w2k[r];
          w2k[r] = w2n;
          w1k[r] = w1n;
          o_0[r] = o_p1[r];
          o_p1[r] = o_p2;
          vk0[r] = vkp;
        }
        if constexpr (EDGE) {
          const unsigned gm = (kgx | kgy) >> (2 * r);
          s1[r] = sel2(gm & 1u, gm & 2u, ghost, s1[r]);
        }
      }
      // ---------------- B: advctx (shuffles) and advcty (shared memory)
      auto adv_x = [&](const float2* in, float2* out) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const float2 c0 = in[r];
          const float2 v = lds2(at(F_VX, r));
          const float2 cm = left2(c0), cp = right2(c0), vmr = left2(v);
          float2 w1, w2;
          if constexpr (EDGE) {
            const float2 vm = sel2(gi == 1, gi + 1 == 1, v, vmr);  // v(max(1,q-1))
            line_work2(cm, c0, cp, v, vm, auxvx, a.inv_dx, dt, w1, w2);
#pragma unroll
            for (int c = 0; c < 2; ++c)  // work(nx+1,1) (advctx.f90:46)
              if (gi + c == nx + 1) cmp(w1, c) = auxvx * cmp(vmr, c) * (cmp(c0, c) - cmp(cm, c));
          } else {
            line_work2(cm, c0, cp, v, vmr, auxvx, a.inv_dx, dt, w1, w2);
          }
          const float2 w1p = right2(w1);
          float2 w2m = left2(w2), w2p = right2(w2);
          if constexpr (EDGE) {
            w2m = sel2(gi == 1, gi + 1 == 1, w2, w2m);
            w2p = sel2(gi == nx, gi + 1 == nx, w2, w2p);
            const float2 u = line_update2(c0, v, w1, w1p, w2, w2m, w2p);
            out[r] = sel2(km(r, 0), km(r, 1), u, c0);
          } else {
            out[r] = line_update2(c0, v, w1, w1p, w2, w2m, w2p);
          }
        }
      };
      auto adv_y = [&](const float2* in, float2* out) {
        float* P0 = P0s + 2 * warp * HX + 2 * lane;
        float* W1 = W1s + 2 * warp * HX + 2 * lane;
        float* W2 = W2s + 2 * warp * HX + 2 * lane;
#pragma unroll
        for (int r = 0; r < RPW; ++r) sts2(P0 + r * HX, in[r]);
        __syncthreads();
        // every thread is past iteration t-1: its staging buffer may be refilled
        prefetch(edge_c, t + 1, early ? 1 : 2);
        static_assert(RPW == 2, "a warp owns a pair of adjacent rows");
        float2 w1s[RPW], w2s[RPW], vs[RPW];
        // y-neighbours: the rows below and above this lane's pair come from
        // the neighbouring warps, the rest from its own registers
        vs[0] = lds2(at(F_VY, 0));
        vs[1] = lds2(at(F_VY, 1));
        const float2 cmv[RPW] = {lds2(P0 - HX), in[0]};
        const float2 cpv[RPW] = {in[1], lds2(P0 + 2 * HX)};
        const float2 vmv[RPW] = {lds2(at(F_VY, 0) - RS), vs[0]};  // vy(i, j-1)
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int gj = gy0 + 2 * warp + r;
          const float2 c0 = in[r];
          const float2 cm = cmv[r], cp = cpv[r];
          const float2 v = vs[r], vmr = vmv[r];
          if constexpr (EDGE) {  // row conditions are uniform across the warp
            line_work2(cm, c0, cp, v, gj == 1 ? v : vmr, auxvy, a.inv_dy, dt, w1s[r], w2s[r]);
            if (gj == ny + 1) w1s[r] = mul2(mul2(splat(auxvy), vmr), sub2(c0, cm));  // advcty.f90:45
          } else {
            line_work2(cm, c0, cp, v, vmr, auxvy, a.inv_dy, dt, w1s[r], w2s[r]);
          }
        }
        sts2(W1, w1s[0]);  // the row above the pair below reads it
        sts2(W2, w2s[0]);
        sts2(W2 + HX, w2s[1]);
        __syncthreads();
        const float2 w1pv[RPW] = {w1s[1], lds2(W1 + 2 * HX)};
        const float2 w2mv[RPW] = {lds2(W2 - HX), w2s[0]};
        const float2 w2pv[RPW] = {w2s[1], lds2(W2 + 2 * HX)};
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const float2 w1p = w1pv[r];
          float2 w2m = w2mv[r], w2p = w2pv[r];
          if constexpr (EDGE) {
            const int gj = gy0 + 2 * warp + r;
            if (gj == 1) w2m = w2s[r];
            if (gj == ny) w2p = w2s[r];
            const float2 u = line_update2(in[r], vs[r], w1s[r], w1p, w2s[r], w2m, w2p);
            out[r] = sel2(km(r, 0), km(r, 1), u, in[r]);
          } else {
            out[r] = line_update2(in[r], vs[r], w1s[r], w1p, w2s[r], w2m, w2p);
          }
        }
      };
      float2 sa[RPW];
      if (xfirst) {  // sizloop.f90:42-48
        adv_x(s1, sa);
        adv_y(sa, s2);
      } else {
        adv_y(s1, sa);
        adv_x(sa, s2);
      }
    } else {
#pragma unroll
      for (int r = 0; r < RPW; ++r) s2[r] = make_float2(0.0f, 0.0f);
      __syncthreads();  // the y-sweep plane of the previous iteration is read by all warps
    }
    if (!STEADY && t < 2) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        if (EDGE) gprev[r] = s2[r];  // ghost value of plane t
        ra[r] = rb[r];
        rb[r] = rc[r];
        rc[r] = s2[r];
        pb[r] = lds2(at(F_PZ, r));  // rkver*rho at plane 1
      }
      return;
    }
    // ---------------- C: diffz for plane k = t-1 (diffz.f90:22-62)
    const int k = t - 1;
    float2 s3[RPW], lbv[RPW];
    const ZT32 zk = tab[k];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      ra[r] = rb[r];
      rb[r] = rc[r];
      rc[r] = (STEADY || t <= nz) ? s2[r] : gtop[r];  // c(nz+1) is the top ghost (diffz.f90:54)
      const float2 lb = lds2(at(F_L1, r));
      lbv[r] = lb;
      if (STEADY || (k > 1 && k < nz)) {
        const float2 lc = lds2(at(F_L, r)), pc = lds2(at(F_PZ, r));
        s3[r] = diffz_mid2(pc, pb[r], rc[r], lc, rb[r], lb, fprev[r], zk);
        pb[r] = pc;
      } else if (k == 1) {
        const float2 lc = lds2(at(F_L, r)), pc = lds2(at(F_PZ, r));
        s3[r] = diffz_bottom2(pc, pb[r], rc[r], lc, rb[r], lb, ra[r], fprev[r], tab[0], tab[1]);
        pb[r] = pc;
      } else {  // k == nz
        float2 la, pa;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const bool ok = (inr >> (2 * r + c) & 1u) != 0;
          const int hh = ok ? gi + c + hp * (gy0 + 2 * warp + r) + (nz - 1) * hs : 0;
          cmp(la, c) = __ldg(a.lrhoh + hh);
          cmp(pa, c) = __ldg(a.pkzh + hh);
        }
        s3[r] = diffz_top2(pa, la, pb[r], rc[r], rb[r], lb, ra[r], tab[nz - 1], tab[nz]);
      }
      if constexpr (EDGE) {
        s3[r] = sel2(km(r, 0), km(r, 1), s3[r], gprev[r]);  // ghosts keep their value
        gprev[r] = s2[r];
      }
    }
    // ---------------- D: diffx (shuffles) and diffy (shared memory)
    auto dif_x = [&](const float2* in, float2* out) {
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const float2 l0 = lbv[r], P0 = lds2(at(F_PX, r)), c0 = in[r];
        // the face flux (P(q)+P(q+1))*(c(q+1)/rho(q+1) - c(q)/rho(q)) is gradr at q and
        // gradl at q+1 (diffx.f90:34-40): computed once per face, the left one by shuffle
        const float2 q0 = mul2(c0, l0), qp = right2(q0), Pp = right2(P0);
        const float2 fr = diff_face2(Pp, P0, qp, q0);
        float2 u = diff_apply2(dtdx2h, fr, left2(fr), c0);
        if constexpr (EDGE) {
          if (xedge) {  // the line's first and last cells (diffx.f90:22-33, 44-55)
            const float2 cm = left2(c0), cp = right2(c0), qm = left2(q0), Pm = left2(P0);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
              const int g = gi + c;
              if (g == 1)
                cmp(u, c) = diff_first_q(cmp(qp, c), cmp(q0, c), cmp(cm, c), cmp(l0, c), cmp(P0, c), cmp(Pp, c),
                                         cmp(c0, c), dtdx2h);
              else if (g == nx)
                cmp(u, c) = diff_last_q(cmp(q0, c), cmp(qm, c), cmp(cp, c), cmp(l0, c), cmp(P0, c), cmp(Pm, c),
                                        cmp(c0, c), dtdx2h);
            }
          }
          u = sel2(km(r, 0), km(r, 1), u, c0);  // ghosts and outside positions keep their value
        }
        out[r] = u;
      }
    };
    auto dif_y = [&](const float2* in, float2* out) {
      float* P1 = P1s + 2 * warp * HX + 2 * lane;
      const float2 P0v[RPW] = {lds2(at(F_PY, 0)), lds2(at(F_PY, 1))};
      const float2 Pmv[RPW] = {lds2(at(F_PY, 0) - RS), P0v[0]};
      const float2 Ppv[RPW] = {P0v[1], lds2(at(F_PY, 1) + RS)};
      // neighbours read c/rho: the products c*(1/rho) of diffy.f90:34-40,
      // each computed once by its owner; a ghost row (edge tiles) holds c
      // itself, which is what the line's first and last cells read of it
      const int gj0 = gy0 + 2 * warp;  // the pair's first row
      float2 q[RPW];
      bool ghost[RPW];
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        q[r] = mul2(in[r], lbv[r]);
        ghost[r] = EDGE && (gj0 + r == 0 || gj0 + r == ny + 1);  // uniform across the warp
        sts2(P1 + r * HX, ghost[r] ? in[r] : q[r]);
      }
      __syncthreads();
      if constexpr (!EDGE) {
        const float2 qm[RPW] = {lds2(P1 - HX), q[0]};
        const float2 qp[RPW] = {q[1], lds2(P1 + 2 * HX)};
        // three faces: below the pair, between its rows (gradr of row 0 and
        // gradl of row 1, the same operations on the same values), above it
        const float2 fb = diff_face2(P0v[0], Pmv[0], q[0], qm[0]);
        const float2 fm = diff_face2(Ppv[0], P0v[0], qp[0], q[0]);
        const float2 ft = diff_face2(Ppv[1], P0v[1], qp[1], q[1]);
        out[0] = diff_apply2(dtdy2h, fm, fb, in[0]);
        out[1] = diff_apply2(dtdy2h, ft, fm, in[1]);
      } else {
        // the stored values of the rows below and above each row
        const float2 vmv[RPW] = {lds2(P1 - HX), ghost[0] ? in[0] : q[0]};
        const float2 vpv[RPW] = {ghost[1] ? in[1] : q[1], lds2(P1 + 2 * HX)};
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const int gj = gj0 + r;
          float2 u;
          if (gj == 1) {  // the first row (diffy.f90:22-33): the row below is the ghost, stored as c
#pragma unroll
            for (int c = 0; c < 2; ++c)
              cmp(u, c) = diff_first_q(cmp(vpv[r], c), cmp(q[r], c), cmp(vmv[r], c), cmp(lbv[r], c),
                                       cmp(P0v[r], c), cmp(Ppv[r], c), cmp(in[r], c), dtdy2h);
          } else if (gj == ny) {  // the last row (diffy.f90:44-55): the row above is the ghost
#pragma unroll
            for (int c = 0; c < 2; ++c)
              cmp(u, c) = diff_last_q(cmp(q[r], c), cmp(vmv[r], c), cmp(vpv[r], c), cmp(lbv[r], c),
                                      cmp(P0v[r], c), cmp(Pmv[r], c), cmp(in[r], c), dtdy2h);
          } else {  // an inner row: its two faces
            u = diff_apply2(dtdy2h, diff_face2(Ppv[r], P0v[r], vpv[r], q[r]), diff_face2(P0v[r], Pmv[r], q[r], vmv[r]),
                            in[r]);
          }
          out[r] = sel2(km(r, 0), km(r, 1), u, in[r]);
        }
      }
    };
    float2 s3a[RPW], s4[RPW];
    if (xfirst) {  // sizloop.f90:55-61
      dif_x(s3, s3a);
      dif_y(s3a, s4);
    } else {
      dif_y(s3, s3a);
      dif_x(s3a, s4);
    }
    // ---------------- E: wetdep, accum, clip, store (plane k)
    const double dzk64 = a.dz64[k];
    if constexpr (!EDGE && STEADY) {  // interior tile, no accum: predicated stores, no divergence
      // the pair's columns inside the output tile (columns 3 .. 3+TX-1 of the region)
      const bool o0 = 2 * lane >= 3 && 2 * lane < 3 + TX, o1 = 2 * lane + 1 >= 3 && 2 * lane + 1 < 3 + TX;
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const int hy = 2 * warp + r;
        if (hy < 3 || hy >= 3 + TY) continue;  // uniform across the warp
        float2 res = s4[r];
        if (wet && k <= s_kzmax) {  // uniform across the block
          const int o = (2 * lane - 3) + TX * (hy - 3);
          if (o0 && k <= wkz[o]) {  // wetdep (wetdep.f90:37-49)
            wacc[o] = wacc[o] + dzk64 * wlam[o] * (double)res.x;
            res.x = (float)((double)res.x * (1.0 - wlam[o]));
          }
          if (o1 && k <= wkz[o + 1]) {
            wacc[o + 1] = wacc[o + 1] + dzk64 * wlam[o + 1] * (double)res.y;
            res.y = (float)((double)res.y * (1.0 - wlam[o + 1]));
          }
        }
        res = make_float2(clip0(res.x), clip0(res.y));
        float* q = cout + gi + px * (gy0 + hy) + k * cs;
        if (P8 && o0 && o1) {
          *reinterpret_cast<float2*>(q) = res;
        } else {
          if (o0) q[0] = res.x;
          if (o1) q[1] = res.y;
        }
      }
      return;
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int hy = 2 * warp + r;
      const int gj = gy0 + hy;
      const int hrow = gi + px * gj + k * cs;  // halo index of the first column
      float2 res = s4[r];
      bool st[2];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int g = gi + c;
        bool out_cell;
        st[c] = false;
        if constexpr (EDGE) {
          const bool rows_out = gj >= j0 && gj <= oj1;
          const bool cols_out = g >= i0 && g <= oi1;
          const unsigned bit = 1u << (2 * r + c);
          if (((kgx & bit) && rows_out && ((g == 0 && i0 == 1) || (g == nx + 1 && oi1 == nx))) ||
              ((kgy & bit) && cols_out && ((gj == 0 && j0 == 1) || (gj == ny + 1 && oj1 == ny)))) {
            cmp(res, c) = clip0(cmp(s3[r], c));  // an outer ghost keeps its setbcc value
            st[c] = true;
            continue;
          }
          out_cell = (kin & bit) && rows_out && cols_out;
        } else {
          const int col = 2 * lane + c;
          out_cell = col >= 3 && col < 3 + TX && hy >= 3 && hy < 3 + TY;
        }
        if (!out_cell) continue;
        float cnew = cmp(res, c);
        if (wet && k <= s_kzmax) {
          const int o = (g - i0) + TX * (gj - j0);
          if (k <= wkz[o]) {  // wetdep (wetdep.f90:37-49)
            wacc[o] = wacc[o] + dzk64 * wlam[o] * (double)cnew;
            cnew = (float)((double)cnew * (1.0 - wlam[o]));
          }
        }
        if (!STEADY && k == 1 && commit) {  // accum (accum.f90:17-25), binary64
          const int mb = (g - 1) + nx * (gj - 1);
          double* cd = a.cdry + (long long)(cls + 1) * pl + mb;
          const double vsd = a.vset64[(long long)cls * a.vstride + mb] + a.vdep64[(long long)cls * pl + mb];
          *cd = *cd - a.dt64 * (double)cnew * fmin2(0.0, vsd);
        }
        cmp(res, c) = clip0(cnew);
        st[c] = true;
      }
      if (P8 && st[0] && st[1])
        *reinterpret_cast<float2*>(cout + hrow) = res;
      else {
        if (st[0]) cout[hrow] = res.x;
        if (st[1]) cout[hrow + 1] = res.y;
      }
    }
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
  {
    if (timed_out) {  // a tensor copy did not arrive in time: report, and let copies in flight land
      atomicOr(a.status, F3D_STEP_STAGING_TIMEOUT);
      mbar_wait(mbar0 + 8u * (unsigned)(nz & 1), (unsigned)(((nz - 1) >> 1) & 1));
      mbar_wait(mbar0 + 8u * (unsigned)((nz + 1) & 1), (unsigned)((nz >> 1) & 1));
    }
    __syncthreads();  // nobody waits on the barriers any more: they may be reused (next batch item)
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(mbar0) : "memory");
      asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(mbar0 + 8) : "memory");
    }
  }
}

template <bool P8>
__global__ void __launch_bounds__(NT, 1) k_step_fused2(const FusedArgs a, const __grid_constant__ F2Maps maps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fused2_tile<P8>(a, &maps, a.c_in, a.c_out, a.xfirst, 1, (int)(blockIdx.x % a.ncls),
                        (int)(blockIdx.x / a.ncls), smem_raw);
}

// The same step with at most 112 registers, launched while a look-ahead
// meteo update runs on the context's second stream: four warps of it take
// 14336 of an SM sub-partition's 16384 registers, which leaves one
// 64-register warp of the settling-velocity chain room beside it on each
// sub-partition.  Same operations, same results.
template <bool P8>
__global__ void __maxnreg__(112) k_step_fused2_beside(const FusedArgs a, const __grid_constant__ F2Maps maps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fused2_tile<P8>(a, &maps, a.c_in, a.c_out, a.xfirst, 1, (int)(blockIdx.x % a.ncls),
                        (int)(blockIdx.x / a.ncls), smem_raw);
}

// Batched form (see k_step_fused_batch in f3d_fused.cu).  The scenarios with
// an even nx come first in the batch; their items [0, split) run in the P8
// kernel, the rest in the other one (counter[0] and counter[1]).
__constant__ FusedArgs c_batch2[F3D_BATCH_MAX];
static_assert(sizeof(FusedArgs) * F3D_BATCH_MAX <= 48 * 1024, "batch argument table exceeds constant memory");

template <bool P8>
__global__ void __launch_bounds__(NT, 1)
    k_step_fused2_batch(const int* __restrict__ item_off, int nscen, int begin, int end, int* counter,
                        const int* __restrict__ bstep, const int* __restrict__ iiter0, int commit,
                        const F2Maps* __restrict__ maps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();  // the previous item is done with shared memory
    if (threadIdx.x == 0) s_item = begin + atomicAdd(counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= end) break;
    int lo = 0, hi = nscen;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (item_off[mid] <= item) lo = mid;
      else hi = mid;
    }
    const FusedArgs& a = c_batch2[lo];
    const int local = item - item_off[lo];
    const int bs = bstep[lo];
    const float* cin = (bs & 1) ? a.c_out : a.c_in;
    float* cout = (bs & 1) ? const_cast<float*>(a.c_in) : a.c_out;
    const int iiter = iiter0[lo] + bs + 1;
    fused2_tile<P8>(a, maps + lo, cin, cout, (iiter % 2 == 0) ? 1 : 0, commit, local % a.ncls,
                          local / a.ncls, smem_raw);
  }
}

// met field (nx,ny,nz) -> halo layout with row pitch hp
__global__ void k_to_halo(Dims d, int hp, const float* src, float* dst) {
  const long long s3 = d.cells();
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < s3;
       m += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(m % d.nx) + 1;
    const long long r = m / d.nx;
    const int j = (int)(r % d.ny) + 1, k = (int)(r / d.ny) + 1;
    dst[i + (long long)hp * (j + (long long)(d.ny + 2) * k)] = src[m];
  }
}

}  // namespace

void launch_step_fused2(const FusedArgs& a, const F2Maps& maps, cudaStream_t s, int beside) {
  const int tiles = ((a.d.nx + TX - 1) / TX) * ((a.d.ny + TY - 1) / TY);
  const size_t sm = fused2_smem(a.d.nz);
  auto go = [&](auto kernel) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kernel<<<tiles * a.ncls, NT, sm, s>>>(a, maps);
  };
  if (a.pair_aligned)
    beside ? go(k_step_fused2_beside<true>) : go(k_step_fused2<true>);
  else
    beside ? go(k_step_fused2_beside<false>) : go(k_step_fused2<false>);
  count_launch();
}

int fused2_max_nz() {
  const size_t cap = (size_t)227 * 1024, base = fused2_smem(0);
  return cap > base ? (int)((cap - base) / sizeof(ZT32)) - 1 : 0;
}

// cuTensorMapEncodeTiled, reached through the runtime's driver entry point
// (no link against the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int make_fused2_maps(const FusedArgs& a, F2Maps* out) {
  static EncodeTiledFn enc = nullptr;
  if (!enc) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return 1;
    enc = reinterpret_cast<EncodeTiledFn>(fn);
  }
  const Dims d = a.d;
  if (a.hpitch % 4 != 0 || a.hpitch < d.nx + 2) return 2;
  // x (the padded row), y (rows 0..ny+1), z (planes 0..nz+1, times the classes for vz+vset)
  auto one = [&](CUtensorMap* m, const float* p, long long planes) {
    const cuuint64_t dim[3] = {(cuuint64_t)a.hpitch, (cuuint64_t)(d.ny + 2), (cuuint64_t)planes};
    const cuuint64_t stride[2] = {(cuuint64_t)a.hpitch * sizeof(float),
                                  (cuuint64_t)a.hpitch * (d.ny + 2) * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)RS, (cuuint32_t)HY, 1u};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(p), dim, stride, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
               ? 0
               : 3;
  };
  const long long np = d.nz + 2;
  int rc = one(&out->m[F2Maps::VK], a.vkh, np * a.ncls);
  if (!rc) rc = one(&out->m[F2Maps::VX], a.vxh, np);
  if (!rc) rc = one(&out->m[F2Maps::VY], a.vyh, np);
  if (!rc) rc = one(&out->m[F2Maps::L], a.lrhoh, np);
  if (!rc) rc = one(&out->m[F2Maps::PZ], a.pkzh, np);
  if (!rc) rc = one(&out->m[F2Maps::PX], a.pkxh, np);
  if (!rc) rc = one(&out->m[F2Maps::PY], a.pkyh, np);
  return rc;
}

int upload_batch_args2(const FusedArgs* h, int n, cudaStream_t s) {
  if (n > F3D_BATCH_MAX) return 1;
  return cudaMemcpyToSymbolAsync(c_batch2, h, sizeof(FusedArgs) * (size_t)n, 0, cudaMemcpyHostToDevice, s) ==
                 cudaSuccess
             ? 0
             : 1;
}

int fused2_batch_grid(int max_nz) {
  const size_t sm = fused2_smem(max_nz);
  if (cudaFuncSetAttribute(k_step_fused2_batch<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_step_fused2_batch<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
          cudaSuccess)
    return -1;
  int per_sm = 0, nsm = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_fused2_batch<true>, NT, sm) != cudaSuccess)
    return -1;
  return per_sm < 1 ? -1 : per_sm * nsm;
}

void launch_step_fused2_batch(int grid, const int* item_off, int nscen, int split, int total, int* counter,
                              const int* bstep, const int* iiter0, int commit, int max_nz, const F2Maps* maps,
                              cudaStream_t s, const BatchFork* fork) {
  const size_t sm = fused2_smem(max_nz);
  const bool both = split > 0 && total > split && fork && fork->s2;
  cudaStream_t s_odd = s;
  if (both) {  // the two parts are independent (their own scenarios and counters)
    cudaEventRecord(fork->a, s);
    cudaStreamWaitEvent(fork->s2, fork->a, 0);
    s_odd = fork->s2;
  }
  if (split > 0) {
    k_step_fused2_batch<true><<<grid, NT, sm, s>>>(item_off, nscen, 0, split, counter, bstep, iiter0, commit, maps);
    count_launch();
  }
  if (total > split) {
    k_step_fused2_batch<false><<<grid, NT, sm, s_odd>>>(item_off, nscen, split, total, counter + 1, bstep, iiter0,
                                                         commit, maps);
    count_launch();
  }
  if (both) {
    cudaEventRecord(fork->b, fork->s2);
    cudaStreamWaitEvent(s, fork->b, 0);
  }
}

void launch_to_halo(Dims d, int hp, int nfield, const float* const* src, float* const* dst, cudaStream_t s) {
  const int nb = (int)std::min<long long>((d.cells() + 255) / 256, 152LL * 16);
  for (int f = 0; f < nfield; ++f) {
    k_to_halo<<<nb, 256, 0, s>>>(d, hp, src[f], dst[f]);
    count_launch();
  }
}

}  // namespace f3d

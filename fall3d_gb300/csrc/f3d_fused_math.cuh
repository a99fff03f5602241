// f3d_fused_math.cuh -- device arithmetic shared by the fused step kernels
// (f3d_fused.cu: one column per lane; f3d_fused2.cu: two columns per lane).
//
// Every formula keeps the reference's binary64 operation order in binary32
// (sizloop's routines, cited at each function); the float2 versions apply
// the same operations to both values of a pair, so all kernel variants give
// the same bits for the same cell.
#pragma once

#include <type_traits>

#include "f3d_fused.h"

namespace f3d {
namespace fz {

constexpr unsigned FULL = 0xffffffffu;

struct ZT32 {
  float dzz, dzk, dzk_1, dzm1, l_dz, l_dzdz;
};

// 0.5*(SIGN(1,dr)+SIGN(1,dl))*MIN(|dr|,|dl|) (advctx.f90:40): +-min when
// the signs agree, +0 when they differ.  Exact for every non-NaN dr, dl
// (the reference's formula gives a NaN only for infinite slopes of opposite
// sign).
__device__ __forceinline__ float minmod(float dr, float dl) {
  const float m = fminf(fabsf(dr), fabsf(dl));
  const unsigned sr = __float_as_uint(dr) & 0x80000000u;
  const unsigned diff = (__float_as_uint(dr) ^ __float_as_uint(dl)) & 0x80000000u;
  return diff ? 0.0f : __uint_as_float(__float_as_uint(m) | sr);
}

__device__ __forceinline__ void zwork(float cm, float c0, float cp, float vk, float vk_1,
                                      const ZT32& z, float dt, float& w1, float& w2) {
  const float vk_12 = 0.5f * (vk + vk_1);
  w1 = dt * (vk * c0 - vk_1 * cm) * z.dzz;
  const float sigma = minmod((cp - c0) * z.dzk, (c0 - cm) * z.dzk_1);
  const float Crk = fabsf(vk_12) * dt * z.dzk_1;
  w2 = dt * 0.5f * z.dzm1 * (1.0f - Crk) * sigma * fabsf(vk_12) * z.dzz;
}

// work(q,1), work(q,2) of advctx.f90:24-44 at line position q.
__device__ __forceinline__ void line_work(float cm, float c0, float cp, float vq, float vq_1,
                                          float auxv, float invd, float dt, float& w1, float& w2) {
  const float vq_12 = 0.5f * (vq + vq_1);
  w1 = auxv * (vq * c0 - vq_1 * cm);
  const float sigma = minmod((cp - c0) * invd, (c0 - cm) * invd);
  const float Cri = auxv * fabsf(vq_12);
  w2 = dt * 0.5f * (1.0f - Cri) * sigma * fabsf(vq_12);
}

// The update of advctx.f90:48-54 (and advctzc.f90:66-72).
__device__ __forceinline__ float line_update(float c0, float vq, float w1, float w1p, float w2,
                                             float w2m, float w2p) {
  const bool up = vq > 0.0f;
  const float a = up ? w1 : w1p;
  const float b = up ? (w2 - w2m) : (w2p - w2);
  return c0 - a - b;
}

// diffx/diffy cell of Sources/diffx.f90:20-55 with l = 1/rho, P = rkh*rho.
// MAX(0,g) / MIN(0,g) of the reference keep 0 for a NaN g.
__device__ __forceinline__ float diff_mid(float cm, float c0, float cp, float lm, float l0, float lp,
                                          float Pm, float P0, float Pp, float dtdx2) {
  const float gradr = 0.5f * (Pp + P0) * (cp * lp - c0 * l0);
  const float gradl = 0.5f * (P0 + Pm) * (c0 * l0 - cm * lm);
  return c0 + dtdx2 * (gradr - gradl);
}
__device__ __forceinline__ float diff_cell(bool first, bool last, float cm, float c0, float cp,
                                           float lm, float l0, float lp, float Pm, float P0,
                                           float Pp, float dtdx2) {
  float gradr, gradl;
  if (first) {
    gradr = Pp * (cp * lp - c0 * l0);
    const float g = P0 * (c0 * l0 - cm * l0);
    gradl = g > 0.0f ? g : 0.0f;
  } else if (last) {
    const float g = P0 * (cp * l0 - c0 * l0);
    gradr = g < 0.0f ? g : 0.0f;
    gradl = Pm * (c0 * l0 - cm * lm);
  } else {
    return diff_mid(cm, c0, cp, lm, l0, lp, Pm, P0, Pp, dtdx2);
  }
  return c0 + dtdx2 * (gradr - gradl);
}

__device__ __forceinline__ float clip0(float x) { return x > 0.0f ? x : 0.0f; }  // MAX(0,x)

__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 4 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(FULL, v, 1); }
__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(FULL, v, 1); }

// Pairs of binary32 values (two rows or two columns of one lane): the
// formulas below apply the scalar ones to both lanes of a float2.
// Arithmetic on the two columns (or rows) of a pair, one IEEE binary32
// operation per lane.  (The f32x2 instructions were measured to differ from
// the scalar ones by one ulp in rare cells, which would make a cell's result
// depend on the kernel variant; the scalar forms keep every variant bitwise
// identical at the cost of ~2% in time.)
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 abs2(float2 v) { return make_float2(fabsf(v.x), fabsf(v.y)); }
__device__ __forceinline__ float2 shup2(float2 v) { return make_float2(shup(v.x), shup(v.y)); }
__device__ __forceinline__ float2 shdn2(float2 v) { return make_float2(shdn(v.x), shdn(v.y)); }

__device__ __forceinline__ void zwork2(float2 cm, float2 c0, float2 cp, float2 vk, float2 vk_1,
                                       const ZT32& z, float dt, float2& w1, float2& w2) {
  const float2 vk_12 = mul2(splat(0.5f), add2(vk, vk_1));
  w1 = mul2(mul2(splat(dt), sub2(mul2(vk, c0), mul2(vk_1, cm))), splat(z.dzz));
  const float2 dr = mul2(sub2(cp, c0), splat(z.dzk)), dl = mul2(sub2(c0, cm), splat(z.dzk_1));
  const float2 sigma = make_float2(minmod(dr.x, dl.x), minmod(dr.y, dl.y));
  const float2 avk = abs2(vk_12);
  const float2 Crk = mul2(mul2(avk, splat(dt)), splat(z.dzk_1));
  w2 = mul2(mul2(mul2(mul2(splat(dt * 0.5f * z.dzm1), sub2(splat(1.0f), Crk)), sigma), avk), splat(z.dzz));
}

__device__ __forceinline__ void line_work2(float2 cm, float2 c0, float2 cp, float2 vq, float2 vq_1,
                                           float auxv, float invd, float dt, float2& w1, float2& w2) {
  const float2 vq_12 = mul2(splat(0.5f), add2(vq, vq_1));
  w1 = mul2(splat(auxv), sub2(mul2(vq, c0), mul2(vq_1, cm)));
  const float2 dr = mul2(sub2(cp, c0), splat(invd)), dl = mul2(sub2(c0, cm), splat(invd));
  const float2 sigma = make_float2(minmod(dr.x, dl.x), minmod(dr.y, dl.y));
  const float2 avq = abs2(vq_12);
  const float2 Cri = mul2(splat(auxv), avq);
  w2 = mul2(mul2(mul2(splat(dt * 0.5f), sub2(splat(1.0f), Cri)), sigma), avq);
}

__device__ __forceinline__ float2 line_update2(float2 c0, float2 vq, float2 w1, float2 w1p, float2 w2,
                                               float2 w2m, float2 w2p) {
  const float2 dm = sub2(w2, w2m), dp = sub2(w2p, w2);
  const float2 a = make_float2(vq.x > 0.0f ? w1.x : w1p.x, vq.y > 0.0f ? w1.y : w1p.y);
  const float2 b = make_float2(vq.x > 0.0f ? dm.x : dp.x, vq.y > 0.0f ? dm.y : dp.y);
  return sub2(sub2(c0, a), b);
}

__device__ __forceinline__ float2 diff_mid2(float2 cm, float2 c0, float2 cp, float2 lm, float2 l0, float2 lp,
                                            float2 Pm, float2 P0, float2 Pp, float dtdx2) {
  const float2 c0l0 = mul2(c0, l0);
  const float2 gradr = mul2(mul2(splat(0.5f), add2(Pp, P0)), sub2(mul2(cp, lp), c0l0));
  const float2 gradl = mul2(mul2(splat(0.5f), add2(P0, Pm)), sub2(c0l0, mul2(cm, lm)));
  return add2(c0, mul2(splat(dtdx2), sub2(gradr, gradl)));
}

// Staged fields of iteration t (plane index in parentheses).
enum : int { F_C = 0, F_VK, F_VX, F_VY, F_L, F_PZ, F_L1, F_PX, F_PY, NF };
//            c(t+2) vz+vset(t+1) vx(t) vy(t) 1/rho(t) K*rho_z(t) 1/rho(t-1) K*rho_x(t-1) K*rho_y(t-1)

using False_ = std::integral_constant<bool, false>;
using True_ = std::integral_constant<bool, true>;


}  // namespace fz
}  // namespace f3d

// f3d_fused_math.cuh -- device arithmetic shared by the fused step kernels
// (f3d_fused.cu: one column per lane; f3d_fused2.cu: two columns per lane).
//
// Every formula is the reference's (sizloop's routines, cited at each
// function) in binary32, with products that share a factor contracted into
// one fused multiply-add (__fmaf_rn, explicit, so that no compiler choice
// enters) and the plane's and the step's constant factors multiplied once;
// the float2 versions apply the scalar ones to both values of a pair, and
// every kernel variant calls these functions, so all of them give the same
// bits for the same cell.
#pragma once

#include <type_traits>

#include "f3d_fused.h"

namespace f3d {
namespace fz {

constexpr unsigned FULL = 0xffffffffu;

struct ZT32 {
  float dzz, dzk, dzk_1, dzm1, l_dz, l_dzdz;
  // the factors with dt of this plane (the same in every kernel)
  float dt_dzz, dt_dzk_1, w2f, hl_dz, dt_l_dzdz, dt_l_dz;
};

// Per-plane factors of advctzc.f90:19-40 (dz(k), dz(k-1)) and diffz.f90:22-62.
__device__ __forceinline__ ZT32 make_zt32(float dzk, float dzkm, float dt) {
  ZT32 z;
  z.dzz = 2.0f / (dzk + dzkm);
  z.dzk = 1.0f / dzk;
  z.dzk_1 = 1.0f / dzkm;
  z.dzm1 = dzkm;
  z.l_dz = 1.0f / dzk;
  z.l_dzdz = 2.0f / (dzk + dzkm);
  z.dt_dzz = dt * z.dzz;
  z.dt_dzk_1 = dt * z.dzk_1;
  z.w2f = ((dt * 0.5f) * z.dzm1) * z.dzz;
  z.hl_dz = 0.5f * z.l_dz;
  z.dt_l_dzdz = dt * z.l_dzdz;
  z.dt_l_dz = dt * z.l_dz;
  return z;
}

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

// work(k,1), work(k,2) of advctzc.f90:36-44: dt*(vk*c0 - vk_1*cm)*dzz and
// dt*0.5*dz(k-1)*(1 - |vk_12|*dt/dz(k-1))*sigma*|vk_12|*dzz.
__device__ __forceinline__ void zwork(float cm, float c0, float cp, float vk, float vk_1, const ZT32& z,
                                      float& w1, float& w2) {
  const float avk = fabsf(0.5f * (vk + vk_1));
  w1 = z.dt_dzz * __fmaf_rn(vk, c0, -(vk_1 * cm));
  const float sigma = minmod((cp - c0) * z.dzk, (c0 - cm) * z.dzk_1);
  w2 = ((z.w2f * __fmaf_rn(-avk, z.dt_dzk_1, 1.0f)) * sigma) * avk;
}

// work(q,1), work(q,2) of advctx.f90:24-44 at line position q:
// auxv*(vq*c0 - vq_1*cm) and dt*0.5*(1 - auxv*|vq_12|)*sigma*|vq_12|.
__device__ __forceinline__ void line_work(float cm, float c0, float cp, float vq, float vq_1,
                                          float auxv, float invd, float dt, float& w1, float& w2) {
  const float avq = fabsf(0.5f * (vq + vq_1));
  w1 = auxv * __fmaf_rn(vq, c0, -(vq_1 * cm));
  const float sigma = minmod((cp - c0) * invd, (c0 - cm) * invd);
  w2 = (((dt * 0.5f) * __fmaf_rn(-auxv, avq, 1.0f)) * sigma) * avq;
}

// The update of advctx.f90:48-54 (and advctzc.f90:66-72).
__device__ __forceinline__ float line_update(float c0, float vq, float w1, float w1p, float w2,
                                             float w2m, float w2p) {
  const bool up = vq > 0.0f;
  const float a = up ? w1 : w1p;
  const float b = up ? (w2 - w2m) : (w2p - w2);
  return c0 - a - b;
}

// diffx/diffy cell of Sources/diffx.f90:20-55 with l = 1/rho, P = rkh*rho
// and dtdx2h = 0.5*dt/dx^2 (the 0.5 of the face average folded in): a face
// flux is (P(q)+P(q+1))*(c(q+1)*l(q+1) - c(q)*l(q)), the same value for the
// two cells that share it.  MAX(0,g) / MIN(0,g) of the reference keep 0 for
// a NaN g.
__device__ __forceinline__ float diff_face(float Pa, float Pb, float qa, float qb) { return (Pa + Pb) * (qa - qb); }
__device__ __forceinline__ float diff_mid(float cm, float c0, float cp, float lm, float l0, float lp,
                                          float Pm, float P0, float Pp, float dtdx2h) {
  const float c0l0 = c0 * l0;
  const float gradr = diff_face(Pp, P0, cp * lp, c0l0);
  const float gradl = diff_face(P0, Pm, c0l0, cm * lm);
  return __fmaf_rn(dtdx2h, gradr - gradl, c0);
}
// the first and last cell of a line (diffx.f90:22-33, 44-55): faces
// without the average, so the full dt/dx^2 = 2*dtdx2h
__device__ __forceinline__ float diff_cell(bool first, bool last, float cm, float c0, float cp,
                                           float lm, float l0, float lp, float Pm, float P0,
                                           float Pp, float dtdx2h) {
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
    return diff_mid(cm, c0, cp, lm, l0, lp, Pm, P0, Pp, dtdx2h);
  }
  return __fmaf_rn(2.0f * dtdx2h, gradr - gradl, c0);
}

// diff_cell from the products q = c*l of the cell's neighbours inside the
// line and the ghost's c: the first cell (qp = c(2)*l(2), q0 = c(1)*l(1),
// cm = c(0)) and the last (q0, qm = c(n-1)*l(n-1), cp = c(n+1)); the same
// operations on the same values as diff_cell.
__device__ __forceinline__ float diff_first_q(float qp, float q0, float cm, float l0, float P0, float Pp, float c0,
                                              float dtdx2h) {
  const float gradr = Pp * (qp - q0);
  const float g = P0 * (q0 - cm * l0);
  const float gradl = g > 0.0f ? g : 0.0f;
  return __fmaf_rn(2.0f * dtdx2h, gradr - gradl, c0);
}
__device__ __forceinline__ float diff_last_q(float q0, float qm, float cp, float l0, float P0, float Pm, float c0,
                                             float dtdx2h) {
  const float g = P0 * (cp * l0 - q0);
  const float gradr = g < 0.0f ? g : 0.0f;
  const float gradl = Pm * (q0 - qm);
  return __fmaf_rn(2.0f * dtdx2h, gradr - gradl, c0);
}

// diffz.f90:22-62 at plane k with c(k-1) = ra, c(k) = rb, c(k+1) = rc,
// l = 1/rho at k (lb), k+1 (lc) and k-1 (la), P = rkver*rho at k (pb),
// k+1 (pc) and k-1 (pa).  An interior plane: the face flux above k (kept in
// fprev for the next plane) minus the one below.
__device__ __forceinline__ float diffz_mid(float pc, float pb, float rc, float lc, float rb, float lb,
                                           float& fprev, const ZT32& zk) {
  const float gradt = ((pc + pb) * __fmaf_rn(rc, lc, -(rb * lb))) * zk.hl_dz;
  const float r = __fmaf_rn(zk.dt_l_dzdz, gradt - fprev, rb);
  fprev = gradt;
  return r;
}
// the first plane (diffz.f90:24-33): the ground face MAX(0, ...)
__device__ __forceinline__ float diffz_bottom(float pc, float pb, float rc, float lc, float rb, float lb, float ra,
                                              float& fprev, const ZT32& z0, const ZT32& z1) {
  const float qt = __fmaf_rn(rc, lc, -(rb * lb));
  const float gradt = (pc * qt) * z1.l_dz;
  const float g = (pb * __fmaf_rn(rb, lb, -(ra * lb))) * z0.l_dz;
  const float gradb = g > 0.0f ? g : 0.0f;
  fprev = ((pc + pb) * qt) * z1.hl_dz;
  return __fmaf_rn(z1.dt_l_dzdz, gradt - gradb, rb);
}
// the last plane (diffz.f90:50-61): the top face MIN(0, ...)
__device__ __forceinline__ float diffz_top(float pa, float la, float pb, float rc, float rb, float lb, float ra,
                                           const ZT32& znm1, const ZT32& znz) {
  const float g = (pb * __fmaf_rn(rc, lb, -(rb * lb))) * znz.l_dz;
  const float gradt = g < 0.0f ? g : 0.0f;
  const float gradb = (pa * __fmaf_rn(rb, lb, -(ra * la))) * znm1.l_dz;
  return __fmaf_rn(znz.dt_l_dz, gradt - gradb, rb);
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

__device__ __forceinline__ void zwork2(float2 cm, float2 c0, float2 cp, float2 vk, float2 vk_1, const ZT32& z,
                                       float2& w1, float2& w2) {
  zwork(cm.x, c0.x, cp.x, vk.x, vk_1.x, z, w1.x, w2.x);
  zwork(cm.y, c0.y, cp.y, vk.y, vk_1.y, z, w1.y, w2.y);
}

__device__ __forceinline__ void line_work2(float2 cm, float2 c0, float2 cp, float2 vq, float2 vq_1,
                                           float auxv, float invd, float dt, float2& w1, float2& w2) {
  line_work(cm.x, c0.x, cp.x, vq.x, vq_1.x, auxv, invd, dt, w1.x, w2.x);
  line_work(cm.y, c0.y, cp.y, vq.y, vq_1.y, auxv, invd, dt, w1.y, w2.y);
}

__device__ __forceinline__ float2 line_update2(float2 c0, float2 vq, float2 w1, float2 w1p, float2 w2,
                                               float2 w2m, float2 w2p) {
  return make_float2(line_update(c0.x, vq.x, w1.x, w1p.x, w2.x, w2m.x, w2p.x),
                     line_update(c0.y, vq.y, w1.y, w1p.y, w2.y, w2m.y, w2p.y));
}

__device__ __forceinline__ float2 diff_face2(float2 Pa, float2 Pb, float2 qa, float2 qb) {
  return make_float2(diff_face(Pa.x, Pb.x, qa.x, qb.x), diff_face(Pa.y, Pb.y, qa.y, qb.y));
}

__device__ __forceinline__ float2 diff_mid2(float2 cm, float2 c0, float2 cp, float2 lm, float2 l0, float2 lp,
                                            float2 Pm, float2 P0, float2 Pp, float dtdx2h) {
  return make_float2(diff_mid(cm.x, c0.x, cp.x, lm.x, l0.x, lp.x, Pm.x, P0.x, Pp.x, dtdx2h),
                     diff_mid(cm.y, c0.y, cp.y, lm.y, l0.y, lp.y, Pm.y, P0.y, Pp.y, dtdx2h));
}

// c0 + dtdx2h*(fr - fl) for a pair, the update of diff_mid from its faces
__device__ __forceinline__ float2 diff_apply2(float dtdx2h, float2 fr, float2 fl, float2 c0) {
  return make_float2(__fmaf_rn(dtdx2h, fr.x - fl.x, c0.x), __fmaf_rn(dtdx2h, fr.y - fl.y, c0.y));
}

__device__ __forceinline__ float2 diffz_mid2(float2 pc, float2 pb, float2 rc, float2 lc, float2 rb, float2 lb,
                                             float2& fprev, const ZT32& zk) {
  return make_float2(diffz_mid(pc.x, pb.x, rc.x, lc.x, rb.x, lb.x, fprev.x, zk),
                     diffz_mid(pc.y, pb.y, rc.y, lc.y, rb.y, lb.y, fprev.y, zk));
}
__device__ __forceinline__ float2 diffz_bottom2(float2 pc, float2 pb, float2 rc, float2 lc, float2 rb, float2 lb,
                                                float2 ra, float2& fprev, const ZT32& z0, const ZT32& z1) {
  return make_float2(diffz_bottom(pc.x, pb.x, rc.x, lc.x, rb.x, lb.x, ra.x, fprev.x, z0, z1),
                     diffz_bottom(pc.y, pb.y, rc.y, lc.y, rb.y, lb.y, ra.y, fprev.y, z0, z1));
}
__device__ __forceinline__ float2 diffz_top2(float2 pa, float2 la, float2 pb, float2 rc, float2 rb, float2 lb,
                                             float2 ra, const ZT32& znm1, const ZT32& znz) {
  return make_float2(diffz_top(pa.x, la.x, pb.x, rc.x, rb.x, lb.x, ra.x, znm1, znz),
                     diffz_top(pa.y, la.y, pb.y, rc.y, rb.y, lb.y, ra.y, znm1, znz));
}

// Staged fields of iteration t (plane index in parentheses).
enum : int { F_C = 0, F_VK, F_VX, F_VY, F_L, F_PZ, F_L1, F_PX, F_PY, NF };
//            c(t+2) vz+vset(t+1) vx(t) vy(t) 1/rho(t) K*rho_z(t) 1/rho(t-1) K*rho_x(t-1) K*rho_y(t-1)

using False_ = std::integral_constant<bool, false>;
using True_ = std::integral_constant<bool, true>;


}  // namespace fz
}  // namespace f3d

// Double-float (FP32 pair) Jacobi rotations: warp reductions of double-float sums, rotation
// parameters formed on the FP32 pipes, and the rotation of a column pair in its cheapest exact
// form.  Shared by the polish sweeps of the mixed SVD (svd.cu) and the batched engine's gate
// step (batch.cu).
#pragma once
#include "df.cuh"

namespace qr {

__device__ __forceinline__ dfl df_shfl_xor(dfl v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}
__device__ __forceinline__ dfl df_shfl(dfl v, int src) {
  return {__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
}
__device__ __forceinline__ dfl df_sel(bool t, dfl a, dfl b) { return t ? a : b; }

// warp_sum4_t in double-float arithmetic
__device__ __forceinline__ dfl df_warp_sum4_t(dfl a, dfl b, dfl c, dfl d) {
  const int l = threadIdx.x & 31;
  const bool h16 = (l & 16) != 0, h8 = (l & 8) != 0;
  dfl k0 = df_sel(h16, c, a), k1 = df_sel(h16, d, b);
  const dfl s0 = df_sel(h16, a, c), s1 = df_sel(h16, b, d);
  k0 = df_add(k0, df_shfl_xor(s0, 16));
  k1 = df_add(k1, df_shfl_xor(s1, 16));
  dfl k = df_sel(h8, k1, k0);
  k = df_add(k, df_shfl_xor(df_sel(h8, k0, k1), 8));
  k = df_add(k, df_shfl_xor(k, 4));
  k = df_add(k, df_shfl_xor(k, 2));
  k = df_add(k, df_shfl_xor(k, 1));
  return k;
}

// x' = c x - conj(s) y ; y' = s x + c y  on (hi, lo) complex pairs
__device__ __forceinline__ void df_rot(float2& xh, float2& xl, float2& yh, float2& yl, dfl c, dfl sr, dfl si) {
  const dfl xr{xh.x, xl.x}, xi{xh.y, xl.y}, yr{yh.x, yl.x}, yi{yh.y, yl.y};
  const dfl nxr = df_add(df_mul(c, xr), df_neg(df_add(df_mul(sr, yr), df_mul(si, yi))));
  const dfl nxi = df_add(df_mul(c, xi), df_neg(df_add(df_mul(sr, yi), df_neg(df_mul(si, yr)))));
  const dfl nyr = df_add(df_add(df_mul(sr, xr), df_neg(df_mul(si, xi))), df_mul(c, yr));
  const dfl nyi = df_add(df_add(df_mul(sr, xi), df_mul(si, xr)), df_mul(c, yi));
  xh = make_float2(nxr.h, nxi.h);
  xl = make_float2(nxr.l, nxi.l);
  yh = make_float2(nyr.h, nyi.h);
  yl = make_float2(nyr.l, nyi.l);
}

__device__ __forceinline__ void df_dot_acc(const float2& xh, const float2& xl, const float2& yh, const float2& yl,
                                           DotAcc& a, DotAcc& b, DotAcc& gr, DotAcc& gi) {
  dot2_step(a, xh.x, xl.x, xh.x, xl.x);
  dot2_step(a, xh.y, xl.y, xh.y, xl.y);
  dot2_step(b, yh.x, yl.x, yh.x, yl.x);
  dot2_step(b, yh.y, yl.y, yh.y, yl.y);
  dot2_step(gr, xh.x, xl.x, yh.x, yl.x);
  dot2_step(gr, xh.y, xl.y, yh.y, yl.y);
  dot2_step(gi, xh.x, xl.x, yh.y, yl.y);
  dot2_step(gi, -xh.y, -xl.y, yh.x, yl.x);
}
// Small-angle rotation (|t| < 2^-24): c = 1 - t^2/2 equals 1 to double-float precision and
// s y needs only the high part of y (|s| |y_lo| < 2^-48 |y|), so x' = x - conj(s) y_hi and
// y' = y + s x_hi with FP32 products and one double-float addition per component.
__device__ __forceinline__ void df_rot_small(float2& xh, float2& xl, float2& yh, float2& yl, float sr, float si) {
  const float dxr = -(sr * yh.x + si * yh.y), dxi = -(sr * yh.y - si * yh.x);
  const float dyr = sr * xh.x - si * xh.y, dyi = sr * xh.y + si * xh.x;
  const dfl nxr = df_add_f({xh.x, xl.x}, dxr), nxi = df_add_f({xh.y, xl.y}, dxi);
  const dfl nyr = df_add_f({yh.x, yl.x}, dyr), nyi = df_add_f({yh.y, yl.y}, dyi);
  xh = make_float2(nxr.h, nxi.h);
  xl = make_float2(nxr.l, nxi.l);
  yh = make_float2(nyr.h, nyi.h);
  yl = make_float2(nyr.l, nyi.l);
}

// a.h b.h + c.h d.h exactly (FMA products, TwoSum) plus the hi x lo cross terms, as (sum, lo)
__device__ __forceinline__ dfl df_prod2(dfl a, dfl b, dfl c, dfl d) {
  const float p1 = __fmul_rn(a.h, b.h), e1 = fmaf(a.h, b.h, -p1);
  const float p2 = __fmul_rn(c.h, d.h), e2 = fmaf(c.h, d.h, -p2);
  const dfl s = df_two_sum(p1, p2);
  float lo = __fadd_rn(__fadd_rn(s.l, e1), e2);
  lo = fmaf(a.h, b.l, lo);
  lo = fmaf(a.l, b.h, lo);
  lo = fmaf(c.h, d.l, lo);
  lo = fmaf(c.l, d.h, lo);
  return {s.h, lo};
}
// x + v - delta x_hi for double-float x, unnormalised v and FP32 delta
__device__ __forceinline__ dfl df_add_shift(dfl x, dfl v, float delta) {
  const dfl s = df_two_sum(x.h, v.h);
  float lo = __fadd_rn(__fadd_rn(s.l, x.l), v.l);
  lo = fmaf(-delta, x.h, lo);
  return df_fast_two_sum(s.h, lo);
}
// Medium-angle rotation (|t| <= 2^-12), the same map as df_rot in ~2/3 of its instructions:
// c = 1 - delta with delta = (1 - c_hi) - c_lo <= 3e-8 (1 - c_hi is exact), x' = x - conj(s) y -
// delta x and y' = y + s x - delta y.  The s y products are exact FP32 products of the high parts
// plus the hi x lo cross terms (the lo x lo terms are below 2^-48 |s| |y|), and delta x takes the
// high part only: delta |x_lo| and the FP32 rounding of delta x_hi are below 2^-48 |x|.
__device__ __forceinline__ void df_rot_medium(float2& xh, float2& xl, float2& yh, float2& yl, dfl c, dfl sr, dfl si) {
  const float delta = __fsub_rn(__fsub_rn(1.f, c.h), c.l);
  const dfl xr{xh.x, xl.x}, xi{xh.y, xl.y}, yr{yh.x, yl.x}, yi{yh.y, yl.y};
  const dfl nsi = df_neg(si);
  const dfl px = df_prod2(sr, yr, si, yi);   // Re(conj(s) y)
  const dfl qx = df_prod2(sr, yi, nsi, yr);  // Im(conj(s) y)
  const dfl py = df_prod2(sr, xr, nsi, xi);  // Re(s x)
  const dfl qy = df_prod2(sr, xi, si, xr);   // Im(s x)
  const dfl nxr = df_add_shift(xr, df_neg(px), delta), nxi = df_add_shift(xi, df_neg(qx), delta);
  const dfl nyr = df_add_shift(yr, py, delta), nyi = df_add_shift(yi, qy, delta);
  xh = make_float2(nxr.h, nxi.h);
  xl = make_float2(nxr.l, nxi.l);
  yh = make_float2(nyr.h, nyi.h);
  yl = make_float2(nyr.l, nyi.l);
}
struct DfParams {
  dfl c, sr, si;
  float tabs;
  int go;
};

// The rotation of DfParams P in its cheapest exact form.
__device__ __forceinline__ void df_rot_any(float2& xh, float2& xl, float2& yh, float2& yl, const DfParams& P) {
  if (P.tabs < 0x1p-24f) df_rot_small(xh, xl, yh, yl, P.sr.h, P.si.h);
  else if (P.tabs <= 0x1p-12f) df_rot_medium(xh, xl, yh, yl, P.c, P.sr, P.si);
  else df_rot(xh, xl, yh, yl, P.c, P.sr, P.si);
}

// 1 / sqrt(u) in double-float for u in [1/4, 4]: FP32 seed and two Newton steps with the
// residual 1 - u c^2 formed in double-float.
__device__ __forceinline__ dfl df_rsqrt(dfl u) {
  float c0 = rsqrtf(u.h);
  dfl c{c0, 0.f};
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const dfl c2 = df_mul(c, c);
    const dfl r = df_add({1.f, 0.f}, df_neg(df_mul(u, c2)));  // ~2^-23, then ~2^-46
    c = df_add(c, {0.5f * c.h * r.h, 0.f});
  }
  return c;
}

// Rotation parameters of a pair from double-float sums, on the FP32 pipes (the FP64 pipe of this
// part is slow even for a single lane).  Same criterion as rotation_params: rotate when
// |g| > tol sigma_max sqrt(min(a, b)) + (4 eps sigma_max)^2.  The tangent t comes from FP32
// (zeta from the double-float difference b - a); c = 1 / sqrt(1 + t^2), s = t c and the phase
// g / |g| are formed in double-float, so the rotation is unitary to ~2^-46 whatever t's rounding.
// For |t| < 2^-24, c = 1 and s is kept in FP32 (the small-angle rotation uses only s.h).
__device__ __forceinline__ bool rotation_params_df(dfl a, dfl b, dfl gr, dfl gi, float tol, float smax, DfParams& P) {
  if (!(a.h > 0.f) || !(b.h > 0.f)) return false;
  const float fl = 4.f * 2.220446049250313e-16f * smax;
  const float mg = fmaxf(fabsf(gr.h), fabsf(gi.h));
  if (!(mg > 0.5f * fl * fl)) return false;  // |g| <= sqrt(2) mg is below the rounding floor
  // exact power-of-two scaling of g so |g'| is in [1, 2)
  int e = 0;
  frexpf(mg, &e);
  const float sc = ldexpf(1.f, 1 - e);
  const dfl grs{gr.h * sc, gr.l * sc}, gis{gi.h * sc, gi.l * sc};
  const dfl n2 = df_add(df_mul(grs, grs), df_mul(gis, gis));  // [1, 8)
  const float gabs = sqrtf(n2.h) / sc;                        // |g| in FP32
  const float mn = fminf(a.h, b.h);
  if (!(gabs > tol * smax * sqrtf(mn) + fl * fl)) return false;
  const dfl d = df_add(b, df_neg(a));
  const float zeta = (0.5f * d.h) / gabs;
  const float az = fabsf(zeta);
  float t = az > 1e18f ? 0.5f / az : 1.f / (az + sqrtf(1.f + az * az));
  t = zeta >= 0.f ? t : -t;
  if (!(t != 0.f)) return false;
  P.tabs = fabsf(t);
  if (fabsf(t) < 0x1p-24f) {  // the small-angle rotation uses s in FP32 only
    const float rgf = rsqrtf(n2.h);
    P.c = {1.f, 0.f};
    P.sr = {t * grs.h * rgf, 0.f};
    P.si = {t * gis.h * rgf, 0.f};
    return true;
  }
  // phase e^{i phi} = g / |g| in double-float
  const dfl rg = df_rsqrt(n2);
  const dfl er = df_mul(grs, rg), ei = df_mul(gis, rg);
  const float tt = __fmul_rn(t, t);
  const dfl u = df_add({1.f, 0.f}, {tt, fmaf(t, t, -tt)});  // 1 + t^2, t^2 exact as a pair
  const dfl c = df_rsqrt(u);
  const dfl sabs = df_mul(c, {t, 0.f});
  P.c = c;
  P.sr = df_mul(sabs, er);
  P.si = df_mul(sabs, ei);
  return true;
}


}  // namespace qr

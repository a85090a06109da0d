// One-sided (Hestenes) Jacobi building blocks shared by the SVD kernels (svd.cu) and the batched
// gate-step kernel (batch.cu): machine epsilons, a warp sum, the plane rotation of a column pair
// and its parameters.
#pragma once
#include "common.cuh"

namespace qr {
namespace {

template <typename T> struct Eps;
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; };
template <> struct Eps<float> { static constexpr float v = 1.1920929e-07f; };

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename C, typename T>
__device__ __forceinline__ void rot(C& x, C& y, T c, T sr, T si) {
  C xn, yn;
  xn.x = c * x.x - (sr * y.x + si * y.y);
  xn.y = c * x.y - (sr * y.y - si * y.x);
  yn.x = (sr * x.x - si * x.y) + c * y.x;
  yn.y = (sr * x.y + si * x.x) + c * y.y;
  x = xn;
  y = yn;
}

// Rotation of the pair (p, q) from its Gram entries a = |b_p|^2, b = |b_q|^2, gamma = b_p^H b_q,
// for columns pre-scaled so that sigma_max ~ 1.  The angle is computed in FP32 (b - a first in
// the working precision, so near-degenerate pairs do not cancel); c = 1/sqrt(1 + t^2) and the unit
// phase gamma/|gamma| are then formed in the working precision from FP32 seeds and two Newton
// steps, so the rotation is unitary to working precision while FP64 square roots and divisions --
// expensive on this part -- are avoided.  A slightly inexact angle only leaves a coupling a
// factor ~1e-7 smaller, which the next sweep removes.
// |g| without forming |g|^2: in FP32 the squared coupling of two tiny columns underflows
template <typename T>
__device__ __forceinline__ T cabs_safe(T gr, T gi) {
  const T x = fabs(gr), y = fabs(gi);
  const T mx = x > y ? x : y, mn = x > y ? y : x;
  if (!(mx > T(0))) return T(0);
  const T r = mn / mx;
  return mx * sqrt(T(1) + r * r);
}

// tol < 0 selects the relative test |g| > |tol| sqrt(a b) (every pair is driven to the same
// relative orthogonality whatever its norms; used on the R^H of a QR preconditioning, where FP32
// keeps the small columns to full relative precision); otherwise the absolute test below.
template <typename T>
__device__ __forceinline__ bool rotation_params(T a, T b, T gr, T gi, T tol, T smax, T& c, T& sr, T& si, float& tabs) {
  if (!(a > 0) || !(b > 0)) return false;
  T rg;
  if (tol < T(0)) {
    const T gabs = cabs_safe(gr, gi);
    if (!(gabs > -tol * sqrt(a) * sqrt(b))) return false;
    rg = T(1) / gabs;
  } else {
    const T g2 = gr * gr + gi * gi;
    const T fl = T(4) * Eps<T>::v * smax;
    const T mn = a < b ? a : b;
    // g > tol smax sqrt(min(a, b)) + fl^2, compared in squares
    if (!(g2 > tol * tol * smax * smax * mn + fl * fl * fl * fl)) return false;
    // 1/|gamma| in working precision: FP32 seed of the exponent-normalised g2 (exact scaling), then
    // two Newton steps; gamma may be far below FP32 range while still above the rotation floor
    int e2 = 0;
    const T g2n = frexp(g2, &e2);  // g2 = g2n * 2^e2, g2n in [0.5, 1)
    const int h = e2 / 2;
    const T g2s = ldexp(g2n, e2 - 2 * h);  // in [0.25, 2)
    rg = (T)rsqrtf((float)g2s);
    rg = rg * (T(1.5) - T(0.5) * g2s * rg * rg);
    rg = rg * (T(1.5) - T(0.5) * g2s * rg * rg);
    rg = ldexp(rg, -h);
  }
  const float zeta = (float)(T(0.5) * (b - a) * rg);
  const float tf = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
  if (!(tf != 0.f)) return false;  // angle below FP32 resolution of the tangent: nothing to do
  const T t = (T)tf;
  const T u = T(1) + t * t;
  T cc = (T)rsqrtf((float)u);
  cc = cc * (T(1.5) - T(0.5) * u * cc * cc);
  cc = cc * (T(1.5) - T(0.5) * u * cc * cc);
  const T sc = t * cc;
  c = cc;
  sr = sc * gr * rg;
  si = sc * gi * rg;
  tabs = fabsf(tf);
  return true;
}

}  // namespace
}  // namespace qr

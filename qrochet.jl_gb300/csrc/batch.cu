// Batched engine: many independent chains of uneven length and bond dimension evolved together,
// one fused launch per brick-wall layer, the whole circuit captured in one CUDA graph.
//
// The work unit is evolve_2site! + truncate! (Chain.jl:606-661, 390-422) on |0...0> chains
// (convert(Chain, zeros(Product, n)), Chain.jl:174-183), then expect of Pauli strings
// (Chain.jl:724-735).  Everything a layer needs stays on the device:
//   - every chain's sites live in fixed-capacity buffers: bond b of an n-qubit chain can never
//     exceed cap_b = min(chi_max, 2^min(b+1, n-b-1)), so site i is allocated as
//     cap_{i-1} x 2 x cap_i and holds its current (chi_l, 2, chi_r) array densely;
//   - bond dimensions, Lambda flags and Lambda vectors are device arrays that the kernels read
//     and rewrite: the truncation decision (the first min(k, maxdim) singular values above the
//     threshold) is taken on the device, so no layer waits for the host;
//   - one CTA runs one whole gate step: theta = A_l diag(Lambda) A_r, the gate, a one-sided
//     Jacobi SVD (theta of at most 128 x 128: chi_max <= 64; FP64, or with QR_MIXED FP32 sweeps
//     first and a double-float finish on the FP32 pipes), the sort, the truncation,
//     re-orthonormalisation of the kept vectors when their singular values fall below 1e-3
//     sigma_max (classical Gram-Schmidt twice), and the write-back of U, Vh and Lambda.  A
//     layer's gates sit on disjoint bonds, so the CTAs of one launch never touch the same site;
//   - the expectation values are one more launch: one CTA per Pauli string sweeps the chain's
//     environment (FP64).
// The layer kernel's CTA size comes from a small autotuner (timed on synthetic gate steps of the
// batch's largest bond class, cached per device and class, optionally in a file).
#include <vector>
#include <mutex>
#include <map>
#include <string>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <algorithm>
#include "kernels.cuh"
#include "jacobi_rot.cuh"
#include "jacobi_df.cuh"

namespace qr {
namespace {

constexpr int BT_MAXK = 128;         // largest theta side: chi_max <= 64
constexpr int BT_MAXCHI = BT_MAXK / 2;
constexpr int BT_MAX_SWEEPS = 60;
constexpr size_t BT_SLOT = 4 * (size_t)BT_MAXK * BT_MAXK;  // B, V, W, Tm (double2) per CTA slot
constexpr int BT_MIXED_MIN = 32;  // the mixed SVD precondition in FP32 above this many columns

struct BTask {
  double2* sl;          // left site buffer
  double2* sr;          // right site buffer
  double* lam;          // Lambda buffer of the bond
  int* bd;              // bond dimensions of the chain
  int* haslam;          // Lambda flags of the chain
  const double2* gate;  // 4 x 4 row-major, [(o1',o2'),(o1,o2)]
  int* status;          // the request's status word
  double threshold;
  int bond, nb, maxdim, pad;
};

struct BObs {
  double2* const* sites;  // n site pointers
  double* const* lams;    // n-1 Lambda pointers
  const int* bd;
  const int* haslam;
  const int* pauli;  // per site 0 I, 1 X, 2 Y, 3 Z
  double2* out;
  int n, pad;
};

// ---- the fused gate step ------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul(double2 a, double2 b) { return cmul(a, b); }

// Hestenes sweeps of one CTA on B (rows x k, ld rows) accumulating V (k x k, ld k) in precision
// T: round-robin pairs, one warp per pair, a CTA barrier between rounds.  Stops after a sweep that
// rotates nothing or whose largest rotation tangent is below tan_stop; returns that verdict.
template <typename T>
__device__ bool cta_sweeps(cplx_t<T>* __restrict__ B, cplx_t<T>* __restrict__ V, int rows, int k, T tol, T smax,
                           int max_sweeps, float tan_stop, unsigned* rot_count, unsigned* tmax_bits) {
  using Cx = cplx_t<T>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int np = k + (k & 1), npairs = np / 2;
  bool converged = false;
  for (int sweep = 0; sweep < max_sweeps && !converged; sweep++) {
    if (threadIdx.x == 0) { *rot_count = 0u; *tmax_bits = 0u; }
    __syncthreads();
    for (int round = 0; round < np - 1; round++) {
      for (int pair = warp; pair < npairs; pair += nw) {
        int p, q;
        if (pair == 0) { p = round; q = np - 1; }
        else { p = (round + pair) % (np - 1); q = (round - pair + np - 1) % (np - 1); }
        if (p > q) { const int x = p; p = q; q = x; }
        if (q >= k) continue;
        Cx* bp = B + (long)rows * p;
        Cx* bq = B + (long)rows * q;
        T a = 0, bb = 0, gr = 0, gi = 0;
        for (int r = lane; r < rows; r += 32) {
          const Cx x = bp[r], y = bq[r];
          a += x.x * x.x + x.y * x.y;
          bb += y.x * y.x + y.y * y.y;
          gr += x.x * y.x + x.y * y.y;
          gi += x.x * y.y - x.y * y.x;
        }
        a = warp_sum(a); bb = warp_sum(bb); gr = warp_sum(gr); gi = warp_sum(gi);
        T c, sr, si;
        float tabs;
        if (!rotation_params<T>(a, bb, gr, gi, tol, smax, c, sr, si, tabs)) continue;
        for (int r = lane; r < rows; r += 32) {
          Cx x = bp[r], y = bq[r];
          rot(x, y, c, sr, si);
          bp[r] = x;
          bq[r] = y;
        }
        Cx* vp = V + (long)k * p;
        Cx* vq = V + (long)k * q;
        for (int r = lane; r < k; r += 32) {
          Cx x = vp[r], y = vq[r];
          rot(x, y, c, sr, si);
          vp[r] = x;
          vq[r] = y;
        }
        if (lane == 0) {
          atomicAdd(rot_count, 1u);
          atomicMax(tmax_bits, __float_as_uint(tabs));
        }
      }
      __syncthreads();
    }
    converged = *rot_count == 0u || __uint_as_float(*tmax_bits) < tan_stop;
    __syncthreads();
  }
  return converged;
}

// ---- the mixed finish in double-float (FP32 pairs, on the FP32 pipes) ----------------------------
// One CTA's double-float Hestenes sweeps on B (Bh, Bl: rows x k, ld rows) accumulating V (Vh,
// Vl: k x k, ld k): round-robin pairs, one warp per pair.  Every lane forms the pair's
// compensated sums over its rows, the warp reduces them, and every lane derives the same rotation
// from the broadcast sums (rotation_params_df), so a pair needs no shared memory; a CTA barrier
// between rounds.  Stops after a sweep that rotates nothing or whose largest tangent is below
// tan_stop; returns that verdict.
__device__ bool cta_sweeps_df(float2* __restrict__ Bh, float2* __restrict__ Bl, float2* __restrict__ Vh,
                              float2* __restrict__ Vl, int rows, int k, float tol, float smax, int max_sweeps,
                              float tan_stop, unsigned* rot_count, unsigned* tmax_bits) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int np = k + (k & 1), npairs = np / 2;
  bool converged = false;
  for (int sweep = 0; sweep < max_sweeps && !converged; sweep++) {
    if (threadIdx.x == 0) { *rot_count = 0u; *tmax_bits = 0u; }
    __syncthreads();
    for (int round = 0; round < np - 1; round++) {
      for (int pair = warp; pair < npairs; pair += nw) {
        int p, q;
        if (pair == 0) { p = round; q = np - 1; }
        else { p = (round + pair) % (np - 1); q = (round - pair + np - 1) % (np - 1); }
        if (p > q) { const int x = p; p = q; q = x; }
        if (q >= k) continue;
        float2 *bph = Bh + (long)rows * p, *bpl = Bl + (long)rows * p;
        float2 *bqh = Bh + (long)rows * q, *bql = Bl + (long)rows * q;
        DotAcc a{0.f, 0.f}, b{0.f, 0.f}, gr{0.f, 0.f}, gi{0.f, 0.f};
        for (int r = lane; r < rows; r += 32) df_dot_acc(bph[r], bpl[r], bqh[r], bql[r], a, b, gr, gi);
        const dfl k4 = df_warp_sum4_t(dot_final(a), dot_final(b), dot_final(gr), dot_final(gi));
        DfParams P;
        if (!rotation_params_df(df_shfl(k4, 0), df_shfl(k4, 8), df_shfl(k4, 16), df_shfl(k4, 24), tol, smax, P))
          continue;
        for (int r = lane; r < rows; r += 32) {
          float2 xh = bph[r], xl = bpl[r], yh = bqh[r], yl = bql[r];
          df_rot_any(xh, xl, yh, yl, P);
          bph[r] = xh; bpl[r] = xl; bqh[r] = yh; bql[r] = yl;
        }
        float2 *vph = Vh + (long)k * p, *vpl = Vl + (long)k * p;
        float2 *vqh = Vh + (long)k * q, *vql = Vl + (long)k * q;
        for (int r = lane; r < k; r += 32) {
          float2 xh = vph[r], xl = vpl[r], yh = vqh[r], yl = vql[r];
          df_rot_any(xh, xl, yh, yl, P);
          vph[r] = xh; vpl[r] = xl; vqh[r] = yh; vql[r] = yl;
        }
        if (lane == 0) {
          atomicAdd(rot_count, 1u);
          atomicMax(tmax_bits, __float_as_uint(P.tabs));
        }
      }
      __syncthreads();
    }
    converged = *rot_count == 0u || __uint_as_float(*tmax_bits) < tan_stop;
    __syncthreads();
  }
  return converged;
}

// R = I - X^H X (FP32 values of compensated double-float sums), X = (Xh, Xl) k x k, ld k.
__device__ void cta_gram_df(const float2* __restrict__ Xh, const float2* __restrict__ Xl, int k, float2* __restrict__ R) {
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
    const int i = t % k, j = t / k;
    DotAcc re{0.f, 0.f}, im{0.f, 0.f};
    for (int x = 0; x < k; x++) {
      const float2 ah = Xh[x + (long)k * i], al = Xl[x + (long)k * i];
      const float2 bh = Xh[x + (long)k * j], bl = Xl[x + (long)k * j];
      dot2_step(re, ah.x, al.x, bh.x, bl.x);  // conj(a) b
      dot2_step(re, ah.y, al.y, bh.y, bl.y);
      dot2_step(im, ah.x, al.x, bh.y, bl.y);
      dot2_step(im, -ah.y, -al.y, bh.x, bl.x);
    }
    const dfl r = df_add({i == j ? 1.f : 0.f, 0.f}, df_neg(dot_final(re))), m = df_neg(dot_final(im));
    R[t] = make_float2(r.h + r.l, m.h + m.l);
  }
}

// Y = X + X_hi R / 2: FP32 products (|R| << 1), double-float sum; k x k, ld k.
__device__ void cta_ns_update(const float2* __restrict__ Xh, const float2* __restrict__ Xl, const float2* __restrict__ R,
                              int k, float2* __restrict__ Yh, float2* __restrict__ Yl) {
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
    const int i = t % k, j = t / k;
    float ar = 0.f, ai = 0.f;
    for (int x = 0; x < k; x++) {
      const float2 a = Xh[i + (long)k * x], r = R[x + (long)k * j];
      ar = fmaf(a.x, r.x, fmaf(-a.y, r.y, ar));
      ai = fmaf(a.x, r.y, fmaf(a.y, r.x, ai));
    }
    const dfl yr = df_add_f({Xh[t].x, Xl[t].x}, 0.5f * ar), yi = df_add_f({Xh[t].y, Xl[t].y}, 0.5f * ai);
    Yh[t] = make_float2(yr.h, yi.h);
    Yl[t] = make_float2(yr.l, yi.l);
  }
}

// C = A X in double-float: A (Ah, Al) rows x k (ld rows), X (Xh, Xl) k x k, C rows x k (ld rows).
__device__ void cta_gemm_df(const float2* __restrict__ Ah, const float2* __restrict__ Al, int rows,
                            const float2* __restrict__ Xh, const float2* __restrict__ Xl, int k, float2* __restrict__ Ch,
                            float2* __restrict__ Cl) {
  for (int t = threadIdx.x; t < rows * k; t += blockDim.x) {
    const int i = t % rows, j = t / rows;
    DotAcc re{0.f, 0.f}, im{0.f, 0.f};
    for (int x = 0; x < k; x++) {
      const float2 ah = Ah[i + (long)rows * x], al = Al[i + (long)rows * x];
      const float2 bh = Xh[x + (long)k * j], bl = Xl[x + (long)k * j];
      dot2_step(re, ah.x, al.x, bh.x, bl.x);
      dot2_step(re, -ah.y, -al.y, bh.y, bl.y);
      dot2_step(im, ah.x, al.x, bh.y, bl.y);
      dot2_step(im, ah.y, al.y, bh.x, bl.x);
    }
    const dfl r = dot_final(re), m = dot_final(im);
    Ch[t] = make_float2(r.h, m.h);
    Cl[t] = make_float2(r.l, m.l);
  }
}

// One CTA per task (strided over the layer's tasks).  ws: BT_SLOT double2 per CTA.  dry = 1 runs
// the arithmetic without writing the chain (the autotuner's timing runs).  MIXED: above
// BT_MIXED_MIN columns the SVD first runs FP32 sweeps on a copy of theta (64x the FP64 rate on
// this part), then finishes in double-float on the FP32 pipes: two Newton-Schulz steps
// X <- X + X (I - X^H X) / 2 make the rotations unitary to rounding, B = theta X is formed with
// compensated products, and double-float sweeps (cta_sweeps_df) finish from couplings of ~1e-6
// in two or three sweeps.  The FP64 finish this replaces kept the FP64 pipe 76 % busy.
template <bool MIXED>
__global__ void __launch_bounds__(512, 1)
    batch_gate_k(const BTask* __restrict__ tasks, int ntasks, double2* __restrict__ ws, int dry) {
  __shared__ BTask T;
  __shared__ double2 G[16];
  __shared__ double sig[BT_MAXK], srt[BT_MAXK];
  __shared__ int perm[BT_MAXK];
  __shared__ unsigned rot_count, tmax_bits;
  __shared__ double red[32];
  __shared__ double2 coef[BT_MAXK];
  __shared__ double scale_f, smax_s;
  __shared__ int keep_s, reorth_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  double2* B = ws + (size_t)blockIdx.x * BT_SLOT;
  double2* V = B + (size_t)BT_MAXK * BT_MAXK;
  double2* W = V + (size_t)BT_MAXK * BT_MAXK;
  double2* Tm = W + (size_t)BT_MAXK * BT_MAXK;

  for (int ti = blockIdx.x; ti < ntasks; ti += gridDim.x) {
    if (tid == 0) T = tasks[ti];
    __syncthreads();
    if (tid < 16) G[tid] = T.gate[tid];
    const int b = T.bond;
    const int cl = b > 0 ? T.bd[b - 1] : 1, cc = T.bd[b], cr = b + 1 < T.nb ? T.bd[b + 1] : 1;
    const int m = 2 * cl, nn = 2 * cr;
    const bool tall = m >= nn;
    const int rows = tall ? m : nn, k = tall ? nn : m;
    const bool lam_on = T.haslam[b] != 0;
    __syncthreads();

    // ---- theta' = G (A_l diag(Lambda) A_r), into B (tall) or B = theta'^H (wide)
    for (int t = tid; t < cl * cr; t += blockDim.x) {
      const int l = t % cl, r = t / cl;
      double2 acc[2][2];
      acc[0][0] = acc[0][1] = acc[1][0] = acc[1][1] = make_double2(0.0, 0.0);
      for (int x = 0; x < cc; x++) {
        const double w = lam_on ? T.lam[x] : 1.0;
        const double2 a0 = cscale(T.sl[l + (long)cl * (2 * x)], w), a1 = cscale(T.sl[l + (long)cl * (1 + 2 * x)], w);
        const double2 b0 = T.sr[x + (long)cc * (2 * r)], b1 = T.sr[x + (long)cc * (1 + 2 * r)];
        acc[0][0] = cadd(acc[0][0], zmul(a0, b0));
        acc[0][1] = cadd(acc[0][1], zmul(a0, b1));
        acc[1][0] = cadd(acc[1][0], zmul(a1, b0));
        acc[1][1] = cadd(acc[1][1], zmul(a1, b1));
      }
#pragma unroll
      for (int p1 = 0; p1 < 2; p1++)
#pragma unroll
        for (int p2 = 0; p2 < 2; p2++) {
          double2 v = make_double2(0.0, 0.0);
#pragma unroll
          for (int o1 = 0; o1 < 2; o1++)
#pragma unroll
            for (int o2 = 0; o2 < 2; o2++) v = cadd(v, zmul(G[(2 * p1 + p2) * 4 + 2 * o1 + o2], acc[o1][o2]));
          const int rt = l + cl * p1, ct = p2 + 2 * r;
          if (tall) B[rt + (long)rows * ct] = v;
          else B[ct + (long)rows * rt] = cconj(v);
        }
    }
    for (int t = tid; t < k * k; t += blockDim.x) V[t] = make_double2((t % k) == (t / k) ? 1.0 : 0.0, 0.0);
    __syncthreads();

    // ---- column norms, power-of-two prescale (sigma_max of the scaled columns in [1/2, 1))
    for (int j = warp; j < k; j += nw) {
      double s = 0.0;
      for (int r = lane; r < rows; r += 32) {
        const double2 v = B[r + (long)rows * j];
        s += v.x * v.x + v.y * v.y;
      }
      s = warp_sum(s);
      if (lane == 0) sig[j] = sqrt(s);
    }
    __syncthreads();
    if (tid == 0) {
      double mx = 0.0;
      for (int j = 0; j < k; j++) mx = fmax(mx, sig[j]);
      int e = 0;
      if (mx > 0.0) frexp(mx, &e);
      scale_f = ldexp(1.0, e);
      smax_s = mx > 0.0 ? ldexp(mx, -e) : 0.0;
    }
    __syncthreads();
    {
      const double inv = 1.0 / scale_f;
      for (int t = tid; t < rows * k; t += blockDim.x) B[t] = cscale(B[t], inv);
    }
    __syncthreads();

    // ---- Hestenes sweeps (optionally preconditioned in FP32)
    const double tol = sqrt((double)rows) * Eps<double>::v;
    const double smax = smax_s;
    if (MIXED && k > BT_MIXED_MIN) {
      float2* B32 = reinterpret_cast<float2*>(W);
      float2* V32 = B32 + (size_t)rows * k;
      for (int t = tid; t < rows * k; t += blockDim.x) B32[t] = make_float2((float)B[t].x, (float)B[t].y);
      for (int t = tid; t < k * k; t += blockDim.x) V32[t] = make_float2((t % k) == (t / k) ? 1.f : 0.f, 0.f);
      __syncthreads();
      const float tol32 = fmaxf(4e-6f, 2.f * sqrtf((float)rows) * Eps<float>::v);
      cta_sweeps<float>(B32, V32, rows, k, tol32, (float)smax, 20, 0.15f, &rot_count, &tmax_bits);
      // the finish in double-float on the FP32 pipes.  The CTA's four slot regions (B, V, W, Tm;
      // 2 BT_MAXK^2 float2 each) hold, phase by phase:
      //   W: B32 | V32 -> theta (hi | lo) -> X (hi | lo) before the conversion back
      //   Tm: X0 (hi | lo) -> R2 | X2 hi
      //   V: R1 | X1 hi -> B' (hi | lo) -> V (FP64)
      //   B: theta (FP64) -> X1 lo | X2 lo -> B (FP64)
      constexpr size_t H = (size_t)BT_MAXK * BT_MAXK;  // float2 per half region
      float2 *rW = reinterpret_cast<float2*>(W), *rT = reinterpret_cast<float2*>(Tm);
      float2 *rV = reinterpret_cast<float2*>(V), *rB = reinterpret_cast<float2*>(B);
      for (int t = tid; t < k * k; t += blockDim.x) { rT[t] = V32[t]; rT[H + t] = make_float2(0.f, 0.f); }
      __syncthreads();
      for (int t = tid; t < rows * k; t += blockDim.x) {
        const dfl re = df_from(B[t].x), im = df_from(B[t].y);
        rW[t] = make_float2(re.h, im.h);
        rW[H + t] = make_float2(re.l, im.l);
      }
      __syncthreads();
      // two Newton-Schulz steps X <- X + X (I - X^H X) / 2 (1e-6 -> 1e-12 -> rounding)
      cta_gram_df(rT, rT + H, k, rV);
      __syncthreads();
      cta_ns_update(rT, rT + H, rV, k, rV + H, rB);
      __syncthreads();
      cta_gram_df(rV + H, rB, k, rT);
      __syncthreads();
      cta_ns_update(rV + H, rB, rT, k, rT + H, rB + H);
      __syncthreads();
      float2 *Xh = rT + H, *Xl = rB + H;
      // B' = theta X into V's region, then the double-float sweeps on (B', X)
      cta_gemm_df(rW, rW + H, rows, Xh, Xl, k, rV, rV + H);
      __syncthreads();
      const float toldf = (float)(32.0 * sqrt((double)rows) * Eps<double>::v);
      const bool conv_df = cta_sweeps_df(rV, rV + H, Xh, Xl, rows, k, toldf, (float)smax, BT_MAX_SWEEPS, 1e-7f,
                                         &rot_count, &tmax_bits);
      if (!conv_df && tid == 0) atomicExch(T.status, (int)QR_ENOCONV);
      // back to FP64: X into W first (its lo part sits in B's region), then B, then V
      for (int t = tid; t < k * k; t += blockDim.x) { rW[t] = Xh[t]; rW[H + t] = Xl[t]; }
      __syncthreads();
      for (int t = tid; t < rows * k; t += blockDim.x) {
        const float2 h = rV[t], l = rV[H + t];
        B[t] = make_double2((double)h.x + l.x, (double)h.y + l.y);
      }
      __syncthreads();
      for (int t = tid; t < k * k; t += blockDim.x) {
        const float2 h = rW[t], l = rW[H + t];
        V[t] = make_double2((double)h.x + l.x, (double)h.y + l.y);
      }
      __syncthreads();
    }
    const bool converged = (MIXED && k > BT_MIXED_MIN) ||
                           cta_sweeps<double>(B, V, rows, k, tol, smax, BT_MAX_SWEEPS, 1e-8f, &rot_count, &tmax_bits);
    if (!converged && tid == 0) atomicExch(T.status, (int)QR_ENOCONV);

    // ---- sigma, descending order (ties by index), truncation on the device
    for (int j = warp; j < k; j += nw) {
      double s = 0.0;
      for (int r = lane; r < rows; r += 32) {
        const double2 v = B[r + (long)rows * j];
        s += v.x * v.x + v.y * v.y;
      }
      s = warp_sum(s);
      if (lane == 0) sig[j] = sqrt(s);
    }
    __syncthreads();
    for (int j = tid; j < k; j += blockDim.x) {
      int rank = 0;
      const double v = sig[j];
      for (int i = 0; i < k; i++) rank += (sig[i] > v) || (sig[i] == v && i < j);
      perm[rank] = j;
      srt[rank] = v;
    }
    __syncthreads();
    if (tid == 0) {
      const int upto = T.maxdim >= 0 && T.maxdim < k ? T.maxdim : k;
      const double thr = isnan(T.threshold) ? 1e-16 : T.threshold;
      int kp = 0;
      while (kp < upto && fabs(srt[kp] * scale_f) > thr) kp++;
      if (kp == 0) {  // the chain would be left with an empty bond: keep one vector, flag the request
        atomicExch(T.status, (int)QR_EINVAL);
        kp = 1;
      }
      keep_s = kp;
      reorth_s = !(srt[kp - 1] > 1e-3 * srt[0]);
    }
    __syncthreads();
    const int keep = keep_s;

    // ---- the kept left vectors of B (columns perm[j] / sigma) into W
    for (int t = tid; t < rows * keep; t += blockDim.x) {
      const int r = t % rows, j = t / rows;
      const double s = srt[j];
      W[r + (long)rows * j] = s > 0.0 ? cscale(B[r + (long)rows * perm[j]], 1.0 / s) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    if (reorth_s) {
      // classical Gram-Schmidt twice: keeps each column's direction and phase, orthonormal to ~eps
      for (int j = 1; j < keep; j++) {
        double2* wj = W + (long)rows * j;
        for (int pass = 0; pass < 2; pass++) {
          for (int i = warp; i < j; i += nw) {
            const double2* wi = W + (long)rows * i;
            double cr_ = 0.0, ci_ = 0.0;
            for (int r = lane; r < rows; r += 32) {
              const double2 x = wi[r], y = wj[r];
              cr_ += x.x * y.x + x.y * y.y;
              ci_ += x.x * y.y - x.y * y.x;
            }
            cr_ = warp_sum(cr_);
            ci_ = warp_sum(ci_);
            if (lane == 0) coef[i] = make_double2(cr_, ci_);
          }
          __syncthreads();
          for (int r = tid; r < rows; r += blockDim.x) {
            double2 v = wj[r];
            for (int i = 0; i < j; i++) v = csub(v, zmul(W[r + (long)rows * i], coef[i]));
            wj[r] = v;
          }
          __syncthreads();
        }
        double s = 0.0;
        for (int r = tid; r < rows; r += blockDim.x) s += wj[r].x * wj[r].x + wj[r].y * wj[r].y;
        s = warp_sum(s);
        if (lane == 0) red[warp] = s;
        __syncthreads();
        if (tid == 0) {
          double tot = 0.0;
          for (int w = 0; w < nw; w++) tot += red[w];
          red[0] = tot > 0.0 ? 1.0 / sqrt(tot) : 0.0;
        }
        __syncthreads();
        const double inv = red[0];
        for (int r = tid; r < rows; r += blockDim.x) wj[r] = cscale(wj[r], inv);
        __syncthreads();
      }
    }

    // ---- write-back: A_l (cl, 2, keep), A_r (keep, 2, cr), Lambda, bond dimension
    if (!dry) {
      if (tall) {  // theta = W S (V[:, perm])^H
        for (int t = tid; t < m * keep; t += blockDim.x) T.sl[t] = W[t % m + (long)rows * (t / m)];
        for (int t = tid; t < keep * nn; t += blockDim.x) {
          const int j = t % keep, col = t / keep;
          T.sr[t] = cconj(V[col + (long)k * perm[j]]);
        }
      } else {  // theta^H = W S V^H  =>  theta = V[:, perm] S W^H
        for (int t = tid; t < m * keep; t += blockDim.x) {
          const int row = t % m, j = t / m;
          T.sl[t] = V[row + (long)k * perm[j]];
        }
        for (int t = tid; t < keep * nn; t += blockDim.x) {
          const int j = t % keep, col = t / keep;
          T.sr[t] = cconj(W[col + (long)rows * j]);
        }
      }
      for (int j = tid; j < keep; j += blockDim.x) T.lam[j] = srt[j] * scale_f;
      if (tid == 0) {
        T.bd[b] = keep;
        T.haslam[b] = 1;
      }
    }
    __syncthreads();
  }
}

// ---- expectation values of Pauli strings: one CTA per string, FP64 environment sweep ----------
// E[a, a'] (ket a, bra a') from the left; per site X[a', o, r] = sum_a E[a, a'] A[a, o, r], then
// E'[r, r'] = sum_{a', o'} conj(A[a', o', r']) sum_o P[o', o] X[a', o, r], times Lambda_r Lambda_r'
// when the bond to the right holds a Lambda.  ws: 3 * 64 * 128 double2 per CTA.
__device__ __forceinline__ double2 pauli_apply(int code, int op, const double2& x0, const double2& x1) {
  // (P x)[op] for x = (x0, x1)
  switch (code) {
    case 1: return op == 0 ? x1 : x0;                                                    // X
    case 2: return op == 0 ? make_double2(x1.y, -x1.x) : make_double2(-x0.y, x0.x);      // Y
    case 3: return op == 0 ? x0 : make_double2(-x1.x, -x1.y);                            // Z
    default: return op == 0 ? x0 : x1;                                                   // I
  }
}

__global__ void batch_expect_k(const BObs* __restrict__ obs, int nobs, double2* __restrict__ ws) {
  const BObs O = obs[blockIdx.x];
  double2* E0 = ws + (size_t)blockIdx.x * 3 * BT_MAXCHI * BT_MAXK;
  double2* E1 = E0 + BT_MAXCHI * BT_MAXCHI;
  double2* X = E1 + BT_MAXCHI * BT_MAXCHI;
  if (threadIdx.x == 0) E0[0] = make_double2(1.0, 0.0);
  __syncthreads();
  int ce = 1;  // current environment side
  for (int i = 0; i < O.n; i++) {
    const double2* A = O.sites[i];
    const int cl = i > 0 ? O.bd[i - 1] : 1, cr = i + 1 < O.n ? O.bd[i] : 1;
    const int code = O.pauli[i];
    // X[a', o, r] (a' fastest), 2 cl cr entries
    for (int t = threadIdx.x; t < cl * 2 * cr; t += blockDim.x) {
      const int ap = t % cl, orr = t / cl;  // orr = o + 2 r
      double2 acc = make_double2(0.0, 0.0);
      for (int a = 0; a < ce; a++) acc = cadd(acc, zmul(E0[a + ce * ap], A[a + (long)cl * orr]));
      X[t] = acc;
    }
    __syncthreads();
    const bool lam_on = i + 1 < O.n && O.haslam[i];
    const double* lam = lam_on ? O.lams[i] : nullptr;
    for (int t = threadIdx.x; t < cr * cr; t += blockDim.x) {
      const int r = t % cr, rp = t / cr;
      double2 acc = make_double2(0.0, 0.0);
      for (int ap = 0; ap < cl; ap++) {
        const double2 x0 = X[ap + cl * (0 + 2 * r)], x1 = X[ap + cl * (1 + 2 * r)];
#pragma unroll
        for (int op = 0; op < 2; op++) {
          const double2 y = pauli_apply(code, op, x0, x1);
          acc = cadd(acc, cmulc(A[ap + (long)cl * (op + 2 * rp)], y));
        }
      }
      if (lam_on) acc = cscale(acc, lam[r] * lam[rp]);
      E1[t] = acc;
    }
    __syncthreads();
    double2* tmp = E0;
    E0 = E1;
    E1 = tmp;
    ce = cr;
  }
  if (threadIdx.x == 0) O.out[0] = E0[0];
}

// state init: every site of every chain becomes |0> = (1, 0) in a (1, 2, 1) array
__global__ void batch_init_k(double2* const* __restrict__ sites, int nsites) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nsites; t += gridDim.x * blockDim.x) {
    sites[t][0] = make_double2(1.0, 0.0);
    sites[t][1] = make_double2(0.0, 0.0);
  }
}

// synthetic sites for the autotuner: deterministic values of unit magnitude scale
__global__ void batch_fill_k(double2* p, long count, double scale) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < count; t += (long)gridDim.x * blockDim.x) {
    const unsigned h1 = (unsigned)(t * 2654435761u) ^ 0x9e3779b9u, h2 = (unsigned)(t * 40503u + 12345u) * 2246822519u;
    p[t] = make_double2(scale * ((double)(h1 & 0xffffff) / 16777216.0 - 0.5),
                        scale * ((double)(h2 & 0xffffff) / 16777216.0 - 0.5));
  }
}

int cap_of(int n, int b, int chi_max) {
  const int e = std::min(b + 1, n - b - 1);
  long c = e >= 30 ? (1L << 30) : (1L << e);
  return (int)std::min<long>(c, chi_max);
}

struct BReq {
  int n = 0, chi_max = 0;
  double threshold = 1e-10;
  std::vector<int> gsite;
  std::vector<double2> gmat;  // 16 per gate
  std::vector<int> ow, os, op;
  // results
  int status = QR_OK;
  std::vector<double2> values;
  std::vector<int> bd;
  std::vector<std::vector<double>> lam;
  std::vector<int> layer_of_gate;
};

// Autotuner cache: (device name, chi class) -> warps per CTA of the layer kernel
std::mutex g_tune_mu;
std::map<std::string, int> g_tune;

std::string tune_file() {
  const char* p = getenv("QROCHET_TUNE_FILE");
  return p ? std::string(p) : std::string();
}

void tune_load() {
  static bool loaded = false;
  if (loaded) return;
  loaded = true;
  const std::string f = tune_file();
  if (f.empty()) return;
  FILE* fp = fopen(f.c_str(), "r");
  if (!fp) return;
  char key[256];
  int v = 0;
  // keep only choices the autotuner can make itself (4, 8 or 16 warps): the layer kernel's
  // shape depends on it, so a damaged or hand-edited entry is re-tuned instead of launched
  while (fscanf(fp, "%255s %d", key, &v) == 2)
    if (v == 4 || v == 8 || v == 16) g_tune[key] = v;
  fclose(fp);
}

void tune_save() {
  const std::string f = tune_file();
  if (f.empty()) return;
  FILE* fp = fopen(f.c_str(), "w");
  if (!fp) return;
  for (auto& kv : g_tune) fprintf(fp, "%s %d\n", kv.first.c_str(), kv.second);
  fclose(fp);
}

}  // namespace
}  // namespace qr

using namespace qr;

struct qr_batch {
  int device = 0;
  int precision = QR_FP64;
  std::vector<BReq> reqs;
  bool ran = false;
  int warps = 0, layers = 0, launches = 0, tuned_from_cache = 0;
  size_t graph_nodes = 0;
  double run_ms = 0.0, tune_ms = 0.0;
  std::vector<double> tune_candidates_ms;
};

namespace {
// warps per CTA for the layer kernel at bond class `chi` (the batch's largest), measured on
// synthetic gate steps of that class in dry mode (no chain is written)
int autotune(qr_batch* bt, cudaStream_t s, int chi, int slots, double2* ws) {
  cudaDeviceProp prop;
  QR_CUDA(cudaGetDeviceProperties(&prop, bt->device));
  const bool mixed = (bt->precision & QR_MIXED) != 0;
  std::string key = std::string(prop.name).substr(0, 40) + "/chi" + std::to_string(chi) + (mixed ? "/mixed" : "/fp64");
  for (char& ch : key)
    if (ch == ' ') ch = '_';
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      bt->warps = it->second;
      bt->tuned_from_cache = 1;
      return QR_OK;
    }
  }
  // synthetic chain of 3 bonds at chi on both sides of the middle one
  const int ntask = std::max(1, std::min(slots, 2 * 152));
  const size_t site = (size_t)chi * 2 * chi;
  double2* sites = nullptr;
  double* lam = nullptr;
  int* ints = nullptr;
  BTask* dt = nullptr;
  QR_CUDA(cudaMallocAsync((void**)&sites, sizeof(double2) * (2 * site + 16), s));
  QR_CUDA(cudaMallocAsync((void**)&lam, sizeof(double) * chi, s));
  QR_CUDA(cudaMallocAsync((void**)&ints, sizeof(int) * 8, s));
  QR_CUDA(cudaMallocAsync((void**)&dt, sizeof(BTask) * ntask, s));
  batch_fill_k<<<256, 256, 0, s>>>(sites, (long)(2 * site + 16), 1.0 / chi);
  count_launch();
  int hi[8] = {chi, chi, chi, 0, 0, 0, 0, 0};
  QR_CUDA(cudaMemcpyAsync(ints, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  std::vector<BTask> ht(ntask);
  for (int i = 0; i < ntask; i++) {
    BTask& t = ht[i];
    t.sl = sites;
    t.sr = sites + site;
    t.lam = lam;
    t.bd = ints;
    t.haslam = ints + 3;
    t.gate = sites + 2 * site;
    t.status = reinterpret_cast<int*>(ints + 7);
    t.threshold = 1e-10;
    t.bond = 1;
    t.nb = 3;
    t.maxdim = chi;
  }
  QR_CUDA(cudaMemcpyAsync(dt, ht.data(), sizeof(BTask) * ntask, cudaMemcpyHostToDevice, s));
  cudaEvent_t e0, e1;
  QR_CUDA(cudaEventCreate(&e0));
  QR_CUDA(cudaEventCreate(&e1));
  const int cand[3] = {4, 8, 16};
  float best = 1e30f;
  int bw = 8;
  bt->tune_candidates_ms.clear();
  for (int w : cand) {
    auto kern = mixed ? batch_gate_k<true> : batch_gate_k<false>;
    kern<<<ntask, 32 * w, 0, s>>>(dt, ntask, ws, 1);  // warm-up
    count_launch();
    QR_CUDA(cudaEventRecord(e0, s));
    kern<<<ntask, 32 * w, 0, s>>>(dt, ntask, ws, 1);
    count_launch();
    QR_CUDA(cudaEventRecord(e1, s));
    QR_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    QR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    bt->tune_candidates_ms.push_back(ms);
    bt->tune_ms += ms;
    if (ms < best) { best = ms; bw = w; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(sites, s);
  cudaFreeAsync(lam, s);
  cudaFreeAsync(ints, s);
  cudaFreeAsync(dt, s);
  QR_CUDA(cudaGetLastError());
  bt->warps = bw;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = bw;
  tune_save();
  return QR_OK;
}
}  // namespace

extern "C" {

int qr_batch_create(int device, qr_batch** out) try {
  if (!out) return fail(QR_EINVAL, "null output");
  qr_batch* b = new qr_batch();
  b->device = device;
  *out = b;
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_set_precision(qr_batch* b, int mode) try {
  if (!b) return fail(QR_EINVAL, "null batch");
  if (b->ran) return fail(QR_EINVAL, "the batch has already run");
  if (mode < 0 || mode > 3) return fail(QR_EINVAL, "bad precision");
  b->precision = mode;
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_free(qr_batch* b) try {
  delete b;
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_add(qr_batch* bt, int n, int chi_max, double threshold, int ngates, const int* gate_site,
                 const double* gate_mats, int nobs, const int* obs_weight, const int* obs_sites, const int* obs_paulis,
                 int* id) try {
  if (!bt || !id) return fail(QR_EINVAL, "null argument");
  if (bt->ran) return fail(QR_EINVAL, "the batch has already run");
  if (n < 2 || chi_max < 1) return fail(QR_EINVAL, "a request needs n >= 2 sites and chi_max >= 1");
  if (chi_max > BT_MAXCHI)
    return fail(QR_EINVAL, "the batched engine takes chi_max <= 64 (theta up to 128 x 128); serve larger requests");
  if (ngates < 0 || (ngates > 0 && (!gate_site || !gate_mats))) return fail(QR_EINVAL, "bad gate list");
  if (nobs < 0 || (nobs > 0 && (!obs_weight || !obs_sites || !obs_paulis))) return fail(QR_EINVAL, "bad observable list");
  BReq r;
  r.n = n;
  r.chi_max = chi_max;
  r.threshold = threshold;
  // layers: a gate opens a new layer when it shares a site with a gate of the current one
  std::vector<int> last_layer(n, -1);
  int cur = 0;
  std::vector<char> used(n, 0);
  for (int g = 0; g < ngates; g++) {
    const int s0 = gate_site[g];
    if (s0 < 0 || s0 + 1 >= n) return fail(QR_EINVAL, "gate site out of range");
    if (used[s0] || used[s0 + 1]) {
      cur++;
      std::fill(used.begin(), used.end(), 0);
    }
    used[s0] = used[s0 + 1] = 1;
    r.gsite.push_back(s0);
    r.layer_of_gate.push_back(cur);
    for (int e = 0; e < 16; e++) r.gmat.push_back(make_double2(gate_mats[32 * g + 2 * e], gate_mats[32 * g + 2 * e + 1]));
  }
  int pos = 0;
  for (int o = 0; o < nobs; o++) {
    if (obs_weight[o] < 0) return fail(QR_EINVAL, "bad observable weight");
    for (int w = 0; w < obs_weight[o]; w++, pos++) {
      if (obs_sites[pos] < 0 || obs_sites[pos] >= n || obs_paulis[pos] < 0 || obs_paulis[pos] > 3)
        return fail(QR_EINVAL, "bad Pauli string entry");
    }
    r.ow.push_back(obs_weight[o]);
  }
  r.os.assign(obs_sites, obs_sites + pos);
  r.op.assign(obs_paulis, obs_paulis + pos);
  bt->reqs.push_back(std::move(r));
  *id = (int)bt->reqs.size() - 1;
  return QR_OK;
} QR_ABI_CATCH

// layer index of every gate of request `id` (host-side schedule; no device needed)
int qr_batch_plan(const qr_batch* bt, int id, int* layer_of_gate, int* nlayers) try {
  if (!bt || id < 0 || id >= (int)bt->reqs.size()) return fail(QR_EINVAL, "bad batch request id");
  const BReq& r = bt->reqs[id];
  int mx = -1;
  for (size_t g = 0; g < r.layer_of_gate.size(); g++) {
    if (layer_of_gate) layer_of_gate[g] = r.layer_of_gate[g];
    mx = std::max(mx, r.layer_of_gate[g]);
  }
  if (nlayers) *nlayers = mx + 1;
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_run(qr_batch* bt, double* ms) try {
  if (!bt) return fail(QR_EINVAL, "null batch");
  if (bt->ran) return fail(QR_EINVAL, "the batch has already run");
  if (bt->reqs.empty()) return fail(QR_EINVAL, "empty batch");
  QR_CUDA(cudaSetDevice(bt->device));
  cudaStream_t s;
  QR_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  const int R = (int)bt->reqs.size();

  // ---- device layout: one allocation holding every buffer
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
  struct ROff { size_t site0, lam0, bd, hl, sp, lp, gates, paulis, out, status; std::vector<size_t> site, lam; };
  std::vector<ROff> ro(R);
  int maxchi = 1, nlayers = 0, nobs_total = 0, nsites_total = 0;
  for (int q = 0; q < R; q++) {
    const BReq& r = bt->reqs[q];
    ROff& o = ro[q];
    o.site.resize(r.n);
    o.lam.resize(r.n - 1);
    for (int i = 0; i < r.n; i++) {
      const int cl = i > 0 ? cap_of(r.n, i - 1, r.chi_max) : 1, cr = i + 1 < r.n ? cap_of(r.n, i, r.chi_max) : 1;
      o.site[i] = take(sizeof(double2) * (size_t)cl * 2 * cr);
      maxchi = std::max(maxchi, std::max(cl, cr));
    }
    for (int b = 0; b < r.n - 1; b++) o.lam[b] = take(sizeof(double) * cap_of(r.n, b, r.chi_max));
    o.bd = take(sizeof(int) * (r.n - 1));
    o.hl = take(sizeof(int) * (r.n - 1));
    o.sp = take(sizeof(double2*) * r.n);
    o.lp = take(sizeof(double*) * (r.n - 1));
    o.gates = take(sizeof(double2) * std::max<size_t>(1, r.gmat.size()));
    o.paulis = take(sizeof(int) * (size_t)r.n * std::max<size_t>(1, r.ow.size()));
    o.out = take(sizeof(double2) * std::max<size_t>(1, r.ow.size()));
    o.status = take(sizeof(int));
    nsites_total += r.n;
    nobs_total += (int)r.ow.size();
    for (int L : r.layer_of_gate) nlayers = std::max(nlayers, L + 1);
  }
  // per-layer task tables, larger bond classes first inside a layer
  std::vector<std::vector<std::pair<int, int>>> layer_tasks(nlayers);  // (request, gate)
  for (int q = 0; q < R; q++)
    for (size_t g = 0; g < bt->reqs[q].gsite.size(); g++) layer_tasks[bt->reqs[q].layer_of_gate[g]].push_back({q, (int)g});
  size_t ntask_total = 0;
  for (auto& L : layer_tasks) {
    std::stable_sort(L.begin(), L.end(), [&](const std::pair<int, int>& x, const std::pair<int, int>& y) {
      const BReq& a = bt->reqs[x.first];
      const BReq& c = bt->reqs[y.first];
      return cap_of(a.n, a.gsite[x.second], a.chi_max) > cap_of(c.n, c.gsite[y.second], c.chi_max);
    });
    ntask_total += L.size();
  }
  const size_t o_tasks = take(sizeof(BTask) * std::max<size_t>(1, ntask_total));
  const size_t o_obs = take(sizeof(BObs) * std::max(1, nobs_total));
  const size_t o_sites_tab = take(sizeof(double2*) * nsites_total);
  int sms = 0, per_sm = 0;
  QR_TRY(device_sm_count(&sms));
  // workspace slots: enough CTAs to fill the GPU with the largest candidate CTA
  const int slots = sms * 4;
  const size_t o_ws = take(sizeof(double2) * BT_SLOT * slots);
  const size_t o_ews = take(sizeof(double2) * 3 * BT_MAXCHI * BT_MAXK * std::max(1, nobs_total));
  char* base = nullptr;
  {
    cudaError_t e = cudaMallocAsync((void**)&base, off, s);
    if (e != cudaSuccess) return fail(QR_ENOMEM, std::string("batch state: ") + cudaGetErrorString(e));
  }
  struct MemGuard {
    void* p;
    cudaStream_t s;
    ~MemGuard() { cudaFreeAsync(p, s); cudaStreamSynchronize(s); }
  } mg{base, s};

  // ---- host images of the tables
  std::vector<BTask> tasks;
  tasks.reserve(ntask_total);
  std::vector<size_t> layer_start(nlayers + 1, 0);
  for (int L = 0; L < nlayers; L++) {
    layer_start[L] = tasks.size();
    for (auto& qg : layer_tasks[L]) {
      const BReq& r = bt->reqs[qg.first];
      const ROff& o = ro[qg.first];
      const int s0 = r.gsite[qg.second];
      BTask t;
      t.sl = reinterpret_cast<double2*>(base + o.site[s0]);
      t.sr = reinterpret_cast<double2*>(base + o.site[s0 + 1]);
      t.lam = reinterpret_cast<double*>(base + o.lam[s0]);
      t.bd = reinterpret_cast<int*>(base + o.bd);
      t.haslam = reinterpret_cast<int*>(base + o.hl);
      t.gate = reinterpret_cast<const double2*>(base + o.gates) + 16 * qg.second;
      t.status = reinterpret_cast<int*>(base + o.status);
      t.threshold = r.threshold;
      t.bond = s0;
      t.nb = r.n - 1;
      t.maxdim = cap_of(r.n, s0, r.chi_max);
      t.pad = 0;
      tasks.push_back(t);
    }
  }
  layer_start[nlayers] = tasks.size();
  std::vector<BObs> obs;
  std::vector<double2*> sites_tab;
  for (int q = 0; q < R; q++) {
    const BReq& r = bt->reqs[q];
    const ROff& o = ro[q];
    std::vector<double2*> sp(r.n);
    std::vector<double*> lp(r.n - 1);
    for (int i = 0; i < r.n; i++) sp[i] = reinterpret_cast<double2*>(base + o.site[i]), sites_tab.push_back(sp[i]);
    for (int b = 0; b < r.n - 1; b++) lp[b] = reinterpret_cast<double*>(base + o.lam[b]);
    std::vector<int> zeros(r.n - 1, 0), ones(r.n - 1, 1);
    QR_CUDA(cudaMemcpyAsync(base + o.bd, ones.data(), sizeof(int) * (r.n - 1), cudaMemcpyHostToDevice, s));
    QR_CUDA(cudaMemcpyAsync(base + o.hl, zeros.data(), sizeof(int) * (r.n - 1), cudaMemcpyHostToDevice, s));
    QR_CUDA(cudaMemcpyAsync(base + o.sp, sp.data(), sizeof(double2*) * r.n, cudaMemcpyHostToDevice, s));
    QR_CUDA(cudaMemcpyAsync(base + o.lp, lp.data(), sizeof(double*) * (r.n - 1), cudaMemcpyHostToDevice, s));
    if (!r.gmat.empty())
      QR_CUDA(cudaMemcpyAsync(base + o.gates, r.gmat.data(), sizeof(double2) * r.gmat.size(), cudaMemcpyHostToDevice, s));
    std::vector<int> pc((size_t)r.n * std::max<size_t>(1, r.ow.size()), 0);
    int pos = 0;
    for (size_t j = 0; j < r.ow.size(); j++) {
      for (int w = 0; w < r.ow[j]; w++, pos++) {
        // a repeated site multiplies its Paulis; strings come with distinct sites, later wins
        pc[(size_t)r.n * j + r.os[pos]] = r.op[pos];
      }
      BObs b;
      b.sites = reinterpret_cast<double2* const*>(base + o.sp);
      b.lams = reinterpret_cast<double* const*>(base + o.lp);
      b.bd = reinterpret_cast<const int*>(base + o.bd);
      b.haslam = reinterpret_cast<const int*>(base + o.hl);
      b.pauli = reinterpret_cast<const int*>(base + o.paulis) + (size_t)r.n * j;
      b.out = reinterpret_cast<double2*>(base + o.out) + j;
      b.n = r.n;
      b.pad = 0;
      obs.push_back(b);
    }
    QR_CUDA(cudaMemcpyAsync(base + o.paulis, pc.data(), sizeof(int) * pc.size(), cudaMemcpyHostToDevice, s));
    const int ok = QR_OK;
    QR_CUDA(cudaMemcpyAsync(base + o.status, &ok, sizeof(int), cudaMemcpyHostToDevice, s));
  }
  if (!tasks.empty())
    QR_CUDA(cudaMemcpyAsync(base + o_tasks, tasks.data(), sizeof(BTask) * tasks.size(), cudaMemcpyHostToDevice, s));
  if (!obs.empty()) QR_CUDA(cudaMemcpyAsync(base + o_obs, obs.data(), sizeof(BObs) * obs.size(), cudaMemcpyHostToDevice, s));
  QR_CUDA(cudaMemcpyAsync(base + o_sites_tab, sites_tab.data(), sizeof(double2*) * sites_tab.size(),
                          cudaMemcpyHostToDevice, s));
  QR_CUDA(cudaStreamSynchronize(s));  // the pageable host images above must be consumed

  double2* ws = reinterpret_cast<double2*>(base + o_ws);
  QR_TRY(autotune(bt, s, std::min(maxchi, BT_MAXCHI), slots, ws));
  auto gate_kernel = (bt->precision & QR_MIXED) ? batch_gate_k<true> : batch_gate_k<false>;
  QR_TRY(blocks_per_sm((const void*)gate_kernel, 32 * bt->warps, 0, &per_sm));
  const int grid_cap = std::min(slots, std::max(1, per_sm) * sms);

  // ---- one CUDA graph: init, every layer, the expectation sweep
  const BTask* dtasks = reinterpret_cast<const BTask*>(base + o_tasks);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  QR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int launches = 0;
  batch_init_k<<<std::max(1, std::min(1024, (nsites_total + 255) / 256)), 256, 0, s>>>(
      reinterpret_cast<double2* const*>(base + o_sites_tab), nsites_total);
  launches++;
  for (int L = 0; L < nlayers; L++) {
    const int nt = (int)(layer_start[L + 1] - layer_start[L]);
    if (nt == 0) continue;
    gate_kernel<<<std::min(nt, grid_cap), 32 * bt->warps, 0, s>>>(dtasks + layer_start[L], nt, ws, 0);
    launches++;
  }
  if (!obs.empty()) {
    batch_expect_k<<<(unsigned)obs.size(), 256, 0, s>>>(reinterpret_cast<const BObs*>(base + o_obs), (int)obs.size(),
                                                         reinterpret_cast<double2*>(base + o_ews));
    launches++;
  }
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
  struct GraphGuard {
    cudaGraph_t g;
    cudaGraphExec_t* x;
    ~GraphGuard() {
      if (*x) cudaGraphExecDestroy(*x);
      if (g) cudaGraphDestroy(g);
    }
  } gg{graph, &exec};
  QR_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  size_t nodes = 0;
  QR_CUDA(cudaGraphGetNodes(graph, nullptr, &nodes));
  cudaEvent_t e0, e1;
  QR_CUDA(cudaEventCreate(&e0));
  QR_CUDA(cudaEventCreate(&e1));
  QR_CUDA(cudaEventRecord(e0, s));
  QR_CUDA(cudaGraphLaunch(exec, s));
  QR_CUDA(cudaEventRecord(e1, s));
  QR_CUDA(cudaEventSynchronize(e1));
  float gms = 0.f;
  QR_CUDA(cudaEventElapsedTime(&gms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QR_CUDA(cudaGetLastError());
  count_launch((uint64_t)launches);
  bt->launches = launches;
  bt->layers = nlayers;
  bt->graph_nodes = nodes;
  bt->run_ms = gms;
  if (ms) *ms = gms;

  // ---- results
  for (int q = 0; q < R; q++) {
    BReq& r = bt->reqs[q];
    const ROff& o = ro[q];
    QR_CUDA(cudaMemcpy(&r.status, base + o.status, sizeof(int), cudaMemcpyDeviceToHost));
    r.values.resize(r.ow.size());
    if (!r.ow.empty())
      QR_CUDA(cudaMemcpy(r.values.data(), base + o.out, sizeof(double2) * r.ow.size(), cudaMemcpyDeviceToHost));
    r.bd.resize(r.n - 1);
    QR_CUDA(cudaMemcpy(r.bd.data(), base + o.bd, sizeof(int) * (r.n - 1), cudaMemcpyDeviceToHost));
    std::vector<int> hl(r.n - 1);
    QR_CUDA(cudaMemcpy(hl.data(), base + o.hl, sizeof(int) * (r.n - 1), cudaMemcpyDeviceToHost));
    r.lam.assign(r.n - 1, {});
    for (int b = 0; b < r.n - 1; b++) {
      if (!hl[b]) continue;
      r.lam[b].resize(r.bd[b]);
      QR_CUDA(cudaMemcpy(r.lam[b].data(), base + o.lam[b], sizeof(double) * r.bd[b], cudaMemcpyDeviceToHost));
    }
  }
  bt->ran = true;
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_result(const qr_batch* bt, int id, int* status, double* values) try {
  if (!bt || id < 0 || id >= (int)bt->reqs.size()) return fail(QR_EINVAL, "bad batch request id");
  if (!bt->ran) return fail(QR_EINVAL, "the batch has not run");
  const BReq& r = bt->reqs[id];
  if (status) *status = r.status;
  if (values)
    for (size_t j = 0; j < r.values.size(); j++) {
      values[2 * j] = r.values[j].x;
      values[2 * j + 1] = r.values[j].y;
    }
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_bond_dims(const qr_batch* bt, int id, int* out) try {
  if (!bt || id < 0 || id >= (int)bt->reqs.size()) return fail(QR_EINVAL, "bad batch request id");
  if (!bt->ran) return fail(QR_EINVAL, "the batch has not run");
  const BReq& r = bt->reqs[id];
  for (int b = 0; b < r.n - 1; b++) out[b] = r.bd[b];
  return QR_OK;
} QR_ABI_CATCH

int qr_batch_lambda(const qr_batch* bt, int id, int bond, double* out, int* len) try {
  if (!bt || id < 0 || id >= (int)bt->reqs.size()) return fail(QR_EINVAL, "bad batch request id");
  if (!bt->ran) return fail(QR_EINVAL, "the batch has not run");
  const BReq& r = bt->reqs[id];
  if (bond < 0 || bond >= r.n - 1) return fail(QR_EINVAL, "Invalid bond");
  if (len) *len = (int)r.lam[bond].size();
  if (out)
    for (size_t j = 0; j < r.lam[bond].size(); j++) out[j] = r.lam[bond][j];
  return QR_OK;
} QR_ABI_CATCH

// layers, kernel launches in the graph, graph nodes, warps per CTA chosen, 1 if the choice came
// from the tuning cache, graph time (ms), autotuning time (ms)
int qr_batch_info(const qr_batch* bt, int* layers, int* launches, int* graph_nodes, int* warps, int* cached,
                  double* run_ms, double* tune_ms) try {
  if (!bt) return fail(QR_EINVAL, "null batch");
  if (layers) *layers = bt->layers;
  if (launches) *launches = bt->launches;
  if (graph_nodes) *graph_nodes = (int)bt->graph_nodes;
  if (warps) *warps = bt->warps;
  if (cached) *cached = bt->tuned_from_cache;
  if (run_ms) *run_ms = bt->run_ms;
  if (tune_ms) *tune_ms = bt->tune_ms;
  return QR_OK;
} QR_ABI_CATCH

}  // extern "C"

// Thin complex SVD for canonize_site!(...; method=:svd) and evolve_2site!'s bond compression.
//
// QR_FP64 (plain): one-sided (Hestenes) Jacobi in FP64.  Columns of B = A (or A^H when A is
// wide) are rotated pairwise until mutually orthogonal: B V = U Sigma.  Pairs follow the
// round-robin (circle) ordering, so each round is n/2 independent pair rotations, one warp per
// pair.  Converged when no pair has |b_p^H b_q| > tol sqrt(|b_p|^2 |b_q|^2), tol = sqrt(m) eps.
//
// QR_MIXED: the same Jacobi in FP32 (FFMA runs ~70x faster than DFMA on GB300) gives
// approximate right singular vectors X.  FP64 then takes over: two Newton-Schulz steps make X
// unitary to FP64 (DMMA GEMMs), B = A X is formed in FP64, and FP64 Hestenes sweeps polish
// (B, X); they start from couplings ~1e-5 and converge quadratically, so a few sweeps replace
// the ~15 of the plain path.  Sigma = column norms of B in FP64, so singular values and the
// truncation cutoff are FP64.  (A first-order Ogita-Aishima update was tried as the polish and
// rejected: FP32 couplings (~1e-5 lambda_max) are not small against the lambda gaps of dense
// random spectra (~5e-4 lambda_max at n = 2048), and the update lost orthogonality.)
//
// Left singular vectors are the normalised columns B/sigma.  When the spectrum spans many
// decades (or has exact zeros) those columns lose orthogonality in proportion to
// sigma_max/sigma_j; they are then re-orthonormalised with a Householder QR, keeping each
// column's phase, which moves the represented matrix by O(eps sigma_max) only.
#include <vector>
#include <algorithm>
#include <functional>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <cmath>
#include <mutex>
#include "kernels.cuh"
#include "df.cuh"
#include "jacobi_df.cuh"
#include "prof.cuh"
#include "jacobi_rot.cuh"
#include "grid_sync.cuh"

namespace qr {

struct DBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes, cudaStream_t s) {
    if (bytes <= cap) return QR_OK;
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMallocAsync(&p, want, s);
    if (e != cudaSuccess) return fail(QR_ENOMEM, std::string("SVD workspace: ") + cudaGetErrorString(e));
    cap = want;
    return QR_OK;
  }
  template <typename T> T* as() { return reinterpret_cast<T*>(p); }
};

// page-locked host memory that grows on demand (the masked sweeps' schedules)
struct HBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return QR_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const size_t want = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) return fail(QR_ENOMEM, std::string("SVD host workspace: ") + cudaGetErrorString(e));
    cap = want;
    return QR_OK;
  }
  template <typename T> T* as() { return reinterpret_cast<T*>(p); }
};

struct SvdWork {
  DBuf B, V, B32, V32, X, Rm, E, T1, nrm, perm, cnt, tau, qtmp, host_sig, Bl, Qp, ml, pt, tcw;
  HBuf hl;
  cudaStream_t last = nullptr;
};

std::atomic<uint64_t> g_svd_path[SP_COUNT];

SvdWork* svd_work_create() { return new SvdWork(); }
void svd_work_free(SvdWork* w) {
  if (!w) return;
  DBuf* all[] = {&w->B, &w->V, &w->B32, &w->V32, &w->X, &w->Rm, &w->E, &w->T1,
                 &w->nrm, &w->perm, &w->cnt, &w->tau, &w->qtmp, &w->host_sig, &w->Bl, &w->Qp, &w->ml, &w->pt, &w->tcw};
  for (DBuf* b : all)
    if (b->p) cudaFree(b->p);
  if (w->hl.p) cudaFreeHost(w->hl.p);
  delete w;
}

namespace {

constexpr int TPB = 256;

// QR_DEBUG=1 in the environment prints sweep counts and refinement residuals to stderr
bool debug_on() {
  static const bool v = getenv("QR_DEBUG") != nullptr;
  return v;
}


// One round of the round-robin (circle) ordering: CTA b handles pair b.  When the column length
// fits (m <= NT * RPT) both columns stay in registers between the inner products and the
// rotation, so each round reads and writes every column of B once; V's columns are rotated in a
// second loop once the rotation is known.
template <typename T, int NT>
__device__ __forceinline__ void block_sum4(T& a, T& b, T& c, T& d) {
  __shared__ T red[4][NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();  // previous readers of red are done
  if (l == 0) { red[0][w] = a; red[1][w] = b; red[2][w] = c; red[3][w] = d; }
  __syncthreads();
  a = b = c = d = T(0);
#pragma unroll
  for (int k = 0; k < NT / 32; k++) { a += red[0][k]; b += red[1][k]; c += red[2][k]; d += red[3][k]; }
}


template <typename T, int NT, int RPT>
__device__ __forceinline__ void jacobi_pair(cplx_t<T>* __restrict__ B, long ldb, int m, int n,
                                            cplx_t<T>* __restrict__ V, long ldv, int nv, int np,
                                            int round, int pair, T tol, T smax,
                                            unsigned* __restrict__ count) {
  using C = cplx_t<T>;
  const int np1 = np - 1;
  int p, q;
  if (pair == 0) { p = round; q = np1; }
  else { p = (round + pair) % np1; q = (round - pair + np1) % np1; }
  if (p >= n || q >= n) return;
  if (p > q) { int t = p; p = q; q = t; }
  C* bp = B + (long)p * ldb;
  C* bq = B + (long)q * ldb;
  const bool fits = m <= NT * RPT;
  C x[RPT], y[RPT];
  T a = 0, b = 0, gr = 0, gi = 0;
  if (fits) {
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      int r = threadIdx.x + j * NT;
      if (r < m) { x[j] = bp[r]; y[j] = bq[r]; }
      else { x[j].x = x[j].y = y[j].x = y[j].y = T(0); }
    }
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      a += x[j].x * x[j].x + x[j].y * x[j].y;
      b += y[j].x * y[j].x + y[j].y * y[j].y;
      gr += x[j].x * y[j].x + x[j].y * y[j].y;
      gi += x[j].x * y[j].y - x[j].y * y[j].x;
    }
  } else {
    for (int r = threadIdx.x; r < m; r += NT) {
      C u = bp[r], w = bq[r];
      a += u.x * u.x + u.y * u.y;
      b += w.x * w.x + w.y * w.y;
      gr += u.x * w.x + u.y * w.y;
      gi += u.x * w.y - u.y * w.x;
    }
  }
  block_sum4<T, NT>(a, b, gr, gi);
  T g = sqrt(gr * gr + gi * gi);
  // rotate when the coupling exceeds tol * sigma_max * sigma_min(pair) plus a floor at the
  // rounding level (4 eps sigma_max)^2: columns end orthogonal to the backward-stable
  // (LAPACK-level) accuracy eps * ||A||, without chasing relative accuracy among columns far below
  // sigma_max, and pairs of columns that are rounding noise (rank-deficient blocks) stop rotating
  const T fl = T(4) * Eps<T>::v * smax;
  if (!(a > 0) || !(b > 0) || !(g > tol * smax * sqrt(a < b ? a : b) + fl * fl)) return;
  T zeta = (b - a) / (2 * g);
  T t = (zeta >= 0 ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  T c = T(1) / sqrt(T(1) + t * t);
  T sr = t * c * gr / g, si = t * c * gi / g;  // s = t c e^{i phi}, gamma = |gamma| e^{i phi}
  // p' = c p - conj(s) q ;  q' = s p + c q
  if (fits) {
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      int r = threadIdx.x + j * NT;
      rot(x[j], y[j], c, sr, si);
      if (r < m) { bp[r] = x[j]; bq[r] = y[j]; }
    }
  } else {
    for (int r = threadIdx.x; r < m; r += NT) {
      C u = bp[r], w = bq[r];
      rot(u, w, c, sr, si);
      bp[r] = u; bq[r] = w;
    }
  }
  C* vp = V + (long)p * ldv;
  C* vq = V + (long)q * ldv;
  for (int r = threadIdx.x; r < nv; r += NT) {
    C u = vp[r], w = vq[r];
    rot(u, w, c, sr, si);
    vp[r] = u; vq[r] = w;
  }
  if (threadIdx.x == 0) {
    atomicAdd(count, 1u);
    atomicMax(count + 1, __float_as_uint((float)fabs(t)));  // largest rotation tangent of the sweep
  }
}

// One full sweep (np-1 rounds) in one cooperative launch: CTAs stride over the round's pairs.
template <typename T, int NT, int RPT>
__global__ void __launch_bounds__(NT) jacobi_sweep_k(cplx_t<T>* __restrict__ B, long ldb, int m, int n,
                                                     cplx_t<T>* __restrict__ V, long ldv, int np, T tol,
                                                     T smax, unsigned* __restrict__ count,
                                                     unsigned* __restrict__ bar) {
  const int npairs = np / 2;
  for (int round = 0; round < np - 1; round++) {
    for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x)
      jacobi_pair<T, NT, RPT>(B, ldb, m, n, V, ldv, n, np, round, pair, tol, smax, count);
    if (!grid_barrier(bar)) return;
  }
}



// Warp sum of four values by a transposed butterfly: the first two levels split the values
// between lane halves, so each lane adds 6 times instead of 20.  Afterwards lane l holds the warp
// total of value (l >> 3) & 3 (lanes 0, 8, 16 and 24 hold a, b, c and d).
template <typename T>
__device__ __forceinline__ T warp_sum4_t(T a, T b, T c, T d) {
  const int l = threadIdx.x & 31;
  const bool h16 = (l & 16) != 0, h8 = (l & 8) != 0;
  T k0 = h16 ? c : a, k1 = h16 ? d : b;
  const T s0 = h16 ? a : c, s1 = h16 ? b : d;
  k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
  k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
  T k = h8 ? k1 : k0;
  k += __shfl_xor_sync(0xffffffffu, h8 ? k0 : k1, 8);
  k += __shfl_xor_sync(0xffffffffu, k, 4);
  k += __shfl_xor_sync(0xffffffffu, k, 2);
  k += __shfl_xor_sync(0xffffffffu, k, 1);
  return k;
}

// L2-coherent loads that stay behind earlier stores (volatile asm with a memory clobber), used
// for the second column pair of a rotation so its registers are not live during the first.
__device__ __forceinline__ float2 ld_cg_ordered(const float2* p) {
  float2 v;
  asm volatile("ld.global.cg.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ double2 ld_cg_ordered(const double2* p) {
  double2 v;
  asm volatile("ld.global.cg.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p) : "memory");
  return v;
}

template <typename T>
struct RotParams {
  T c, sr, si;
  float tabs;
  float rel;  // |g|^2 / (a b): the pair's relative coupling, squared
  int go;
};

// Per-sweep counters: state[8 + SW_STRIDE s + 0..2] = rotations, largest rotation tangent and
// largest |g|^2 / (a b) of a rotated pair (float bits; the last is recorded by the FP32 kernels);
// + 3 = pairs a masked double-float polish sweep skipped.
constexpr int SW_STRIDE = 4;

// Rotates rows [0, len) of the column pair (xp, xq) in chunks of NT * RPT rows: each chunk's
// loads are all issued before its first store, so a chunk costs one L2 round trip.
template <typename T, int NT, int RPT>
__device__ __forceinline__ void rot_cols_staged(cplx_t<T>* xp, cplx_t<T>* xq, int len, T c, T sr, T si) {
  using C = cplx_t<T>;
  for (int base = 0; base < len; base += NT * RPT) {
    C* pp = xp + base + threadIdx.x;
    C* pq = xq + base + threadIdx.x;
    const int lim = len - base - (int)threadIdx.x;  // row j*NT is valid when j*NT < lim
    C u[RPT], w[RPT];
#pragma unroll
    for (int j = 0; j < RPT; j++)
      if (j * NT < lim) { u[j] = ld_cg_ordered(pp + j * NT); w[j] = ld_cg_ordered(pq + j * NT); }
#pragma unroll
    for (int j = 0; j < RPT; j++)
      if (j * NT < lim) {
        rot(u[j], w[j], c, sr, si);
        __stcg(pp + j * NT, u[j]);
        __stcg(pq + j * NT, w[j]);
      }
  }
}

// One Hestenes pair (p, q) of a round: inner products, one block reduction, rotation parameters
// computed once (lane 0 of warp 0) and broadcast through shared memory, then the rotation of the
// B and V columns.  When a column fits (m <= NT * RPT) it stays in registers between the inner
// products and the rotation.
template <typename T, int NT, int RPT>
__device__ __forceinline__ void jacobi_pair_fast(cplx_t<T>* __restrict__ B, long ldb, int m,
                                                 cplx_t<T>* __restrict__ V, long ldv, int nv, int p, int q,
                                                 T tol, T smax, unsigned* __restrict__ count) {
  using C = cplx_t<T>;
  __shared__ T red[4][NT / 32];
  __shared__ RotParams<T> P;
  C* bp = B + (long)p * ldb;
  C* bq = B + (long)q * ldb;
  const bool fits = m <= NT * RPT;
  C x[RPT], y[RPT];
  T a = 0, b = 0, gr = 0, gi = 0;
  const int lim0 = m - (int)threadIdx.x;
  if (fits) {
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      if (j * NT < lim0) { x[j] = __ldcg(bp + threadIdx.x + j * NT); y[j] = __ldcg(bq + threadIdx.x + j * NT); }
      else { x[j].x = x[j].y = y[j].x = y[j].y = T(0); }
    }
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      a += x[j].x * x[j].x + x[j].y * x[j].y;
      b += y[j].x * y[j].x + y[j].y * y[j].y;
      gr += x[j].x * y[j].x + x[j].y * y[j].y;
      gi += x[j].x * y[j].y - x[j].y * y[j].x;
    }
  } else {
    for (int base = 0; base < m; base += NT * RPT) {
#pragma unroll
      for (int j = 0; j < RPT; j++) {
        if (base + j * NT < lim0) { x[j] = __ldcg(bp + base + threadIdx.x + j * NT); y[j] = __ldcg(bq + base + threadIdx.x + j * NT); }
        else { x[j].x = x[j].y = y[j].x = y[j].y = T(0); }
      }
#pragma unroll
      for (int j = 0; j < RPT; j++) {
        a += x[j].x * x[j].x + x[j].y * x[j].y;
        b += y[j].x * y[j].x + y[j].y * y[j].y;
        gr += x[j].x * y[j].x + x[j].y * y[j].y;
        gi += x[j].x * y[j].y - x[j].y * y[j].x;
      }
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const T k = warp_sum4_t<T>(a, b, gr, gi);
  if ((l & 7) == 0) red[l >> 3][w] = k;
  __syncthreads();
  if (w == 0) {
    T v = 0;
    if (l < 4) {
#pragma unroll
      for (int i = 0; i < NT / 32; i++) v += red[l][i];
    }
    const T sa = __shfl_sync(0xffffffffu, v, 0), sb = __shfl_sync(0xffffffffu, v, 1);
    const T sgr = __shfl_sync(0xffffffffu, v, 2), sgi = __shfl_sync(0xffffffffu, v, 3);
    if (l == 0) {
      T c, sr, si;
      float tabs = 0.f;
      const bool go = rotation_params<T>(sa, sb, sgr, sgi, tol, smax, c, sr, si, tabs);
      P.c = c; P.sr = sr; P.si = si; P.tabs = tabs; P.go = go ? 1 : 0;
      P.rel = (float)((sgr * sgr + sgi * sgi) / (sa * sb));
    }
  }
  __syncthreads();
  if (!P.go) return;
  const T c = P.c, sr = P.sr, si = P.si;
  if (fits) {
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      rot(x[j], y[j], c, sr, si);
      if (j * NT < lim0) { __stcg(bp + threadIdx.x + j * NT, x[j]); __stcg(bq + threadIdx.x + j * NT, y[j]); }
    }
  } else {  // rows beyond NT * RPT (rare): reload and rotate row by row
    for (int r = threadIdx.x; r < m; r += NT) {
      C u = __ldcg(bp + r), w = __ldcg(bq + r);
      rot(u, w, c, sr, si);
      __stcg(bp + r, u);
      __stcg(bq + r, w);
    }
  }
  // keep the V loads behind the B stores: the B registers die first and occupancy stays high
  asm volatile("" ::: "memory");
  rot_cols_staged<T, NT, RPT / 2>(V + (long)p * ldv, V + (long)q * ldv, nv, c, sr, si);
  if (threadIdx.x == 0) {
    atomicAdd(count, 1u);
    atomicMax(count + 1, __float_as_uint(P.tabs));
    atomicMax(count + 2, __float_as_uint(P.rel));
  }
}

// B *= 2^-e with 2^(e-1) <= max column norm < 2^e (exact), so sigma_max ~ 1 inside the sweeps;
// scale_out[0] = 2^e for the caller to undo it.  One block per column chunk reads the same max.
template <typename C>
__global__ void pow2_scale_k(C* __restrict__ B, long ldb, int rows, int k, double* __restrict__ smax_io,
                             double* __restrict__ scale_out, int undo) {
  const double sm = *smax_io;
  int e = 0;
  if (sm > 0.0) frexp(sm, &e);
  const double f = undo ? ldexp(1.0, e) : ldexp(1.0, -e);
  long total = (long)rows * k;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % rows, j = t / rows;
    C v = B[i + j * ldb];
    v.x = (decltype(v.x))(v.x * f);
    v.y = (decltype(v.y))(v.y * f);
    B[i + j * ldb] = v;
  }
  if (!undo && blockIdx.x == 0 && threadIdx.x == 0) scale_out[0] = ldexp(1.0, e);
}

// ---- dataflow ordering of the round-robin sweep -------------------------------------------------
// Round r of a sweep pairs column (r + i) mod (np - 1) with (r - i) mod (np - 1), and pair 0 with
// column np - 1 (a padding column when k is odd).  Instead of a grid barrier between rounds, each
// column carries the number of rounds it has completed (flags[c], counted from the first sweep of
// the call): the pair of global round R waits until both columns reached R, rotates, and publishes
// R + 1.  CTAs take work items (round, pair) in increasing order, so the earliest unfinished item
// always has its inputs ready and the persistent (co-resident) grid cannot deadlock.  The flags
// pay off when a round has more pairs than the grid has CTAs (they absorb the imbalance); with at
// most one pair per CTA the kernels keep the bounded grid barrier between rounds.  A wait gives
// up after ~2^22 polls: it sets state[4] (reported as an error) and state[5], which makes every
// other wait return at once.
__device__ __forceinline__ void pair_cols(int np, int round, int pair, int& p, int& q) {
  const int np1 = np - 1;
  if (pair == 0) { p = round; q = np1; }
  else { p = (round + pair) % np1; q = (round - pair + np1) % np1; }
  if (p > q) { int t = p; p = q; q = t; }
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* a) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* a, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}
// returns false when the sweep is aborted (this or another CTA timed out)
__device__ __forceinline__ bool wait_cols(const unsigned* flags, int p, int q, int n, unsigned R,
                                          unsigned* state) {
  __shared__ int ok;
  if (threadIdx.x == 0) {
    int good = 1;
    unsigned polls = 0;
    for (;;) {
      // both flags in one round trip
      const unsigned fp = p < n ? ld_acquire_u32(flags + p) : 0xffffffffu;
      const unsigned fq = q < n ? ld_acquire_u32(flags + q) : 0xffffffffu;
      if (fp >= R && fq >= R) break;
      if (((volatile unsigned*)state)[5]) { good = 0; break; }
      if (++polls > (1u << 22)) {
        atomicExch(state + 4, 1u);
        atomicExch(state + 5, 1u);
        good = 0;
        break;
      }
      __nanosleep(64);
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}
// as wait_cols with a target per column (the list order of a masked sweep)
__device__ __forceinline__ bool wait_cols2(const unsigned* flags, int p, int q, unsigned Rp, unsigned Rq,
                                           unsigned* state) {
  __shared__ int ok2;
  if (threadIdx.x == 0) {
    int good = 1;
    unsigned polls = 0;
    for (;;) {
      const unsigned fp = ld_acquire_u32(flags + p), fq = ld_acquire_u32(flags + q);
      if (fp >= Rp && fq >= Rq) break;
      if (((volatile unsigned*)state)[5]) { good = 0; break; }
      if (++polls > (1u << 22)) {
        atomicExch(state + 4, 1u);
        atomicExch(state + 5, 1u);
        good = 0;
        break;
      }
      __nanosleep(64);
    }
    ok2 = good;
  }
  __syncthreads();
  return ok2 != 0;
}
__device__ __forceinline__ void post_cols2(unsigned* flags, int p, int q, unsigned Rp, unsigned Rq) {
  __syncthreads();  // every thread's column stores precede thread 0's release (cumulative fence)
  if (threadIdx.x == 0) {
    __threadfence();
    st_release_u32(flags + p, Rp);
    st_release_u32(flags + q, Rq);
  }
}
__device__ __forceinline__ void post_cols(unsigned* flags, int p, int q, int n, unsigned R1) {
  __syncthreads();  // every thread's column stores precede thread 0's release (cumulative fence)
  if (threadIdx.x == 0) {
    __threadfence();
    if (p < n) st_release_u32(flags + p, R1);
    if (q < n) st_release_u32(flags + q, R1);
  }
}
// The last CTA to finish the sweep records it and decides convergence: no rotation, or a largest
// rotation tangent below tan_stop (1e-8 in FP64 and double-float, where the next sweep could only
// rotate at the rounding level; larger for the FP32 preconditioner, whose near-degenerate pairs
// the double-float polish resolves anyway; 0 = off).
__device__ __forceinline__ void finish_sweep(unsigned* state, const unsigned* cnt, int sweep, float tan_stop) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(state + 6, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      const unsigned h = ((volatile const unsigned*)cnt)[0];
      const float tmax = __uint_as_float(((volatile const unsigned*)cnt)[1]);
      state[1] = sweep + 1;
      if (h == 0 || tmax < tan_stop) state[0] = 1;
      state[6] = 0;
    }
  }
}

// Sweep `sweep` of a Jacobi whose convergence is decided on the device, so the host enqueues
// all sweeps at once and synchronises only at the end.  state[0] = converged flag (set by the
// sweep that finds no rotation, or, in FP64, whose largest rotation tangent is < 1e-8; later
// sweeps then return at once), state[1] = sweeps run, state[2..3] = grid barrier, state[4] /
// [5] = wait (flag or barrier) timeout / abort,
// state[6] = CTAs done with the sweep, state[8 + SW_STRIDE s ...] = the sweep's counters;
// flags[c] = rounds completed by column c (dataflow ordering above).
template <typename T, int NT, int RPT>
__global__ void __launch_bounds__(NT, 512 / NT) jacobi_sweep_dev_k(cplx_t<T>* __restrict__ B, long ldb, int m, int n,
                                                         cplx_t<T>* __restrict__ V, long ldv, int np, T tol,
                                                         const double* __restrict__ smax_p,
                                                         unsigned* __restrict__ state, int sweep,
                                                         unsigned* __restrict__ flags, float tan_stop) {
  if (((volatile unsigned*)state)[0]) return;
  const T smax = (T)(smax_p[0] / smax_p[1]);  // sigma_max of the pre-scaled columns (~1)
  unsigned* cnt = state + 8 + SW_STRIDE * sweep;
  const int npairs = np / 2;
  const unsigned base = (unsigned)sweep * (unsigned)(np - 1);
  // dataflow: work items in (round, pair) order dealt round-robin to the CTAs, so the surplus
  // pairs rotate over the CTAs from round to round; barrier mode: CTA b owns pair b of every round
  const bool dataflow = npairs > (int)gridDim.x;
  const long nit = dataflow ? ((long)(np - 1) * npairs - blockIdx.x + gridDim.x - 1) / gridDim.x : (long)(np - 1);
  for (long t = 0; t < nit; t++) {
    const long it = dataflow ? blockIdx.x + t * (long)gridDim.x : t * npairs + blockIdx.x;
    const int round = (int)(it / npairs), pair = (int)(it % npairs);
    int p, q;
    pair_cols(np, round, pair, p, q);
    if (dataflow && !wait_cols(flags, p, q, n, base + round, state)) return;
    if (q < n) jacobi_pair_fast<T, NT, RPT>(B, ldb, m, V, ldv, n, p, q, tol, smax, cnt);
    if (dataflow) post_cols(flags, p, q, n, base + round + 1);
    else if (!grid_barrier(state + 2)) return;
  }
  finish_sweep(state, cnt, sweep, tan_stop);
}

// Rotation parameters in FP32 for the preconditioner (same rule as rotation_params).  In FP32 the
// rounding floor (4 eps sigma_max)^2 is ~2e-13 after the power-of-two prescale, so g^2 never
// underflows where a rotation is due and the textbook formulas need no rescaling or Newton steps.
__device__ __forceinline__ bool rotation_params_f32(float a, float b, float gr, float gi, float tol, float smax,
                                                    float& c, float& sr, float& si, float& tabs) {
  if (!(a > 0.f) || !(b > 0.f)) return false;
  float rg;  // 1 / |g|
  if (tol < 0.f) {  // relative test (see rotation_params)
    const float gabs = cabs_safe(gr, gi);
    if (!(gabs > -tol * sqrtf(a) * sqrtf(b))) return false;
    rg = 1.f / gabs;
  } else {
    const float g2 = gr * gr + gi * gi;
    const float fl = 4.f * Eps<float>::v * smax;
    const float mn = fminf(a, b);
    if (!(g2 > tol * tol * smax * smax * mn + fl * fl * fl * fl)) return false;
    rg = rsqrtf(g2);
  }
  const float zeta = 0.5f * (b - a) * rg;
  const float az = fabsf(zeta);
  float t = az > 1e18f ? 0.5f / az : 1.f / (az + sqrtf(1.f + az * az));
  t = zeta >= 0.f ? t : -t;
  if (!(t != 0.f)) return false;
  c = rsqrtf(1.f + t * t);
  const float sc = t * c * rg;
  sr = sc * gr;
  si = sc * gi;
  tabs = fabsf(t);
  return true;
}

// ---- block Jacobi sweep (FP32 preconditioner, rows <= 2048) ------------------------------------
// The k columns form blocks of JR_W = 4; a work item is a pair of blocks.  Each of the 512 threads
// holds 4 rows of the item's 8 columns in registers, so a local round moves no column data
// through memory: the four pairs' inner products come from registers, one transposed butterfly
// reduces the 16 sums per warp, lanes 0-3 of warp 0 form the four rotations in parallel, and
// every thread rotates its rows in place.  Round 0 of a sweep (where every block appears once)
// takes all 28 pairs of the 8 columns (7 local rounds); later rounds take the 16 cross pairs (4
// local rounds), so every pair is met once per sweep.  The 8 x 8 product J of the rotations is
// accumulated in shared memory and V's 8 columns are updated once as V[:, cols] <- V[:, cols] J.
// Per sweep each column moves through L2 (nb - 1) times instead of (k - 1) times and (nb - 1)
// rounds are synchronised instead of (k - 1), with the same two orderings as the scalar sweep
// (per-block flags or the grid barrier).  Pair indices are compile-time constants (unrolled local
// rounds), so the column arrays stay in registers.
constexpr int JR_NT = 512, JR_RPT = 4, JR_C = 8, JR_W = 4;
constexpr int JR_MAXROWS = JR_NT * JR_RPT;  // 2048

__host__ __device__ constexpr int jr_p(bool full, int ir, int g) {
  return full ? (g == 0 ? ir : ((ir + g) % 7 < (ir - g + 7) % 7 ? (ir + g) % 7 : (ir - g + 7) % 7)) : g;
}
__host__ __device__ constexpr int jr_q(bool full, int ir, int g) {
  return full ? (g == 0 ? 7 : ((ir + g) % 7 > (ir - g + 7) % 7 ? (ir + g) % 7 : (ir - g + 7) % 7))
              : JR_W + (g + ir) % JR_W;
}

template <int NT>
struct JrShared {
  float red[16][NT / 32];
  RotParams<float> P[4];
  float2 J[JR_C][JR_C];  // J[col][row]
  int col[JR_C];
  int rotated;
};

// Warp sum of 16 values by a transposed butterfly: afterwards lanes 2v and 2v + 1 hold the warp
// total of value v (v = 0..15).
__device__ __forceinline__ float jr_warp_sum16(float (&v)[16]) {
  const int l = threadIdx.x & 31;
  float a8[8], a4[4], a2[2];
  const bool h16 = l & 16, h8 = l & 8, h4 = l & 4, h2 = l & 2;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const float keep = h16 ? v[8 + i] : v[i], send = h16 ? v[i] : v[8 + i];
    a8[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float keep = h8 ? a8[4 + i] : a8[i], send = h8 ? a8[i] : a8[4 + i];
    a4[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const float keep = h4 ? a4[2 + i] : a4[i], send = h4 ? a4[i] : a4[2 + i];
    a2[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  float a1 = h2 ? a2[1] : a2[0];
  a1 += __shfl_xor_sync(0xffffffffu, h2 ? a2[0] : a2[1], 2);
  a1 += __shfl_xor_sync(0xffffffffu, a1, 1);
  return a1;  // value index ((l >> 4) & 1) * 8 + ((l >> 3) & 1) * 4 + ((l >> 2) & 1) * 2 + ((l >> 1) & 1)
}

template <int NT, int RPT, bool FULL, int IR>
__device__ __forceinline__ void jr_local_round(float2 (&x)[JR_C][RPT], JrShared<NT>& sh, float tol, float smax,
                                               unsigned* cnt) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float v[16];
#pragma unroll
  for (int g = 0; g < 4; g++) {
    constexpr int dummy = 0;
    (void)dummy;
    const int p = jr_p(FULL, IR, g), q = jr_q(FULL, IR, g);
    float a = 0.f, b = 0.f, gr = 0.f, gi = 0.f;
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const float2 xx = x[p][j], yy = x[q][j];
      a += xx.x * xx.x + xx.y * xx.y;
      b += yy.x * yy.x + yy.y * yy.y;
      gr += xx.x * yy.x + xx.y * yy.y;
      gi += xx.x * yy.y - xx.y * yy.x;
    }
    v[4 * g] = a; v[4 * g + 1] = b; v[4 * g + 2] = gr; v[4 * g + 3] = gi;
  }
  const float k = jr_warp_sum16(v);
  if ((lane & 1) == 0) {
    const int vi = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
    sh.red[vi][warp] = k;
  }
  __syncthreads();
  if (warp == 0) {
    float tot = 0.f;
    if (lane < 16) {
#pragma unroll
      for (int w = 0; w < NT / 32; w++) tot += sh.red[lane][w];
    }
    const int g = lane & 3;
    const float sa = __shfl_sync(0xffffffffu, tot, 4 * g), sb = __shfl_sync(0xffffffffu, tot, 4 * g + 1);
    const float sgr = __shfl_sync(0xffffffffu, tot, 4 * g + 2), sgi = __shfl_sync(0xffffffffu, tot, 4 * g + 3);
    if (lane < 4) {
      const int p = jr_p(FULL, IR, lane), q = jr_q(FULL, IR, lane);
      float c = 1.f, sr = 0.f, si = 0.f, tabs = 0.f;
      const bool live = sh.col[p] >= 0 && sh.col[q] >= 0;
      const bool go = live && rotation_params_f32(sa, sb, sgr, sgi, tol, smax, c, sr, si, tabs);
      sh.P[lane].c = c; sh.P[lane].sr = sr; sh.P[lane].si = si; sh.P[lane].tabs = tabs; sh.P[lane].go = go ? 1 : 0;
      if (go) {
        atomicAdd(cnt, 1u);
        atomicMax(cnt + 1, __float_as_uint(tabs));
        atomicMax(cnt + 2, __float_as_uint((sgr * sgr + sgi * sgi) / (sa * sb)));
        sh.rotated = 1;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int g = 0; g < 4; g++) {
    const int p = jr_p(FULL, IR, g), q = jr_q(FULL, IR, g);
    if (sh.P[g].go) {
      const float c = sh.P[g].c, sr = sh.P[g].sr, si = sh.P[g].si;
#pragma unroll
      for (int j = 0; j < RPT; j++) rot(x[p][j], x[q][j], c, sr, si);
      if (tid < JR_C) {  // columns p, q of J, row tid (J is read only after a later barrier)
        float2 u = sh.J[p][tid], w = sh.J[q][tid];
        rot(u, w, c, sr, si);
        sh.J[p][tid] = u;
        sh.J[q][tid] = w;
      }
    }
  }
}

// One work item: block pair (bp, bq) of round `round`.  VPRE (n <= NT): V's rows of the 8
// columns are loaded with B's, before the local rounds, so their L2 round trip overlaps them.
template <int NT, int RPT, bool VPRE>
__device__ __forceinline__ void jr_block_pair(float2* __restrict__ B, long ldb, int m, int n, float2* __restrict__ V,
                                              long ldv, int nb, int bp, int bq, int round, float tol, float smax,
                                              unsigned* cnt, JrShared<NT>& sh) {
  const int tid = threadIdx.x;
  if (tid < JR_C) {
    const int blk = tid < JR_W ? bp : bq, c = blk * JR_W + (tid % JR_W);
    sh.col[tid] = (blk < nb && c < n) ? c : -1;
  }
  if (tid < JR_C * JR_C) sh.J[tid / JR_C][tid % JR_C] = make_float2((tid / JR_C) == (tid % JR_C) ? 1.f : 0.f, 0.f);
  if (tid == 0) sh.rotated = 0;
  __syncthreads();
  float2 x[JR_C][RPT];
#pragma unroll
  for (int l = 0; l < JR_C; l++) {
    const int c = sh.col[l];
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const int r = tid + NT * j;
      x[l][j] = (c >= 0 && r < m) ? __ldcg(B + (long)c * ldb + r) : make_float2(0.f, 0.f);
    }
  }
  float2 vpre[VPRE ? JR_C : 1];
  if constexpr (VPRE) {
#pragma unroll
    for (int l = 0; l < JR_C; l++) {
      const int c = sh.col[l];
      vpre[l] = (c >= 0 && tid < n) ? __ldcg(V + (long)c * ldv + tid) : make_float2(0.f, 0.f);
    }
  }
  if (round == 0) {
    jr_local_round<NT, RPT, true, 0>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, true, 1>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, true, 2>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, true, 3>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, true, 4>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, true, 5>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, true, 6>(x, sh, tol, smax, cnt);
  } else {
    jr_local_round<NT, RPT, false, 0>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, false, 1>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, false, 2>(x, sh, tol, smax, cnt);
    jr_local_round<NT, RPT, false, 3>(x, sh, tol, smax, cnt);
  }
  __syncthreads();  // J and the rotated flag are final
  if (!sh.rotated) return;
#pragma unroll
  for (int l = 0; l < JR_C; l++) {
    const int c = sh.col[l];
    if (c < 0) continue;
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const int r = tid + NT * j;
      if (r < m) __stcg(B + (long)c * ldb + r, x[l][j]);
    }
  }
  if constexpr (VPRE) {
    if (tid < n) {
#pragma unroll
      for (int l2 = 0; l2 < JR_C; l2++) {
        const int c = sh.col[l2];
        if (c < 0) continue;
        float2 o = make_float2(0.f, 0.f);
#pragma unroll
        for (int l = 0; l < JR_C; l++) {
          const float2 jv = sh.J[l2][l];
          o.x += vpre[l].x * jv.x - vpre[l].y * jv.y;
          o.y += vpre[l].x * jv.y + vpre[l].y * jv.x;
        }
        __stcg(V + (long)c * ldv + tid, o);
      }
    }
  } else {
    for (int r0 = tid; r0 < n; r0 += 2 * NT) {
      float2 vin[2][JR_C];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = r0 + h * NT;
#pragma unroll
        for (int l = 0; l < JR_C; l++) {
          const int c = sh.col[l];
          vin[h][l] = (c >= 0 && r < n) ? __ldcg(V + (long)c * ldv + r) : make_float2(0.f, 0.f);
        }
      }
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = r0 + h * NT;
        if (r >= n) continue;
#pragma unroll
        for (int l2 = 0; l2 < JR_C; l2++) {
          const int c = sh.col[l2];
          if (c < 0) continue;
          float2 o = make_float2(0.f, 0.f);
#pragma unroll
          for (int l = 0; l < JR_C; l++) {
            const float2 jv = sh.J[l2][l];
            o.x += vin[h][l].x * jv.x - vin[h][l].y * jv.y;
            o.y += vin[h][l].x * jv.y + vin[h][l].y * jv.x;
          }
          __stcg(V + (long)c * ldv + r, o);
        }
      }
    }
  }
}

// Marked pairs of a masked sweep and their schedule.  Layout (nv = even vertex count: columns, or
// 4-column blocks; mw = ceil(nv / 32); cap = nv (nv - 1) / 2):
//   mask   nv rows of mw words: bit (q & 31) of word p * mw + q / 32 marks the pair p < q
//   flag   nv words: 1 when a pair inside vertex v is marked (4-column blocks)
//   count  4 words: marked (element) pairs, a first-order tangent bound (float bits), listed pairs
//   items  cap words: the listed pairs, colour class by colour class: p | q << 15 | full << 30
//   ord    2 cap words: listed pairs before item i on p (ord[2 i]) and on q (ord[2 i + 1])
// The schedule (items, ord) is built on the host from the mask (schedule_pairs).
struct MaskedList {
  unsigned *mask, *flag, *count, *items, *ord;
  int mw;
};
__host__ __device__ inline size_t masked_list_words(int nv) {
  const size_t mw = ((size_t)nv + 31) / 32, cap = (size_t)nv * (nv - 1) / 2;
  return (size_t)nv * mw + nv + 4 + 3 * cap;
}
__host__ __device__ inline MaskedList masked_list(const unsigned* base, int nv) {
  const size_t mw = ((size_t)nv + 31) / 32, cap = (size_t)nv * (nv - 1) / 2;
  unsigned* b = const_cast<unsigned*>(base);
  MaskedList L;
  L.mw = (int)mw;
  L.mask = b;
  L.flag = L.mask + (size_t)nv * mw;
  L.count = L.flag + nv;
  L.items = L.count + 4;
  L.ord = L.items + cap;
  return L;
}
__device__ __forceinline__ bool marked(const MaskedList& L, int lo, int hi, int n, int k0) {
  return hi < n && lo < k0 && ((L.mask[(long)lo * L.mw + (hi >> 5)] >> (hi & 31)) & 1u);
}
__device__ __forceinline__ void list_item(const MaskedList& L, unsigned i, int& p, int& q, bool& full) {
  const unsigned v = L.items[i];
  p = (int)(v & 0x7fffu);
  q = (int)((v >> 15) & 0x7fffu);
  full = (v >> 30) & 1u;
}

__global__ void __launch_bounds__(JR_NT, 1)
    jacobi_block_reg_k(float2* __restrict__ B, long ldb, int m, int n, float2* __restrict__ V, long ldv, int nbp,
                       float tol, const double* __restrict__ smax_p, unsigned* __restrict__ state, int sweep,
                       unsigned* __restrict__ flags, float tan_stop, const unsigned* __restrict__ ml,
                       unsigned* __restrict__ done) {
  __shared__ JrShared<JR_NT> sh;
  if (((volatile unsigned*)state)[0]) return;
  const float smax = (float)(smax_p[0] / smax_p[1]);
  unsigned* cnt = state + 8 + SW_STRIDE * sweep;
  const int nb = (n + JR_W - 1) / JR_W;
  const int npairs = nbp / 2;
  if (ml) {
    // masked sweep: the listed block pairs (MaskedList over the nbp blocks) dealt round-robin to
    // the CTAs; a block pair waits until the listed block pairs before it on each of its blocks
    // are done, and `full` pairs also meet the pairs inside their blocks (as in round 0)
    const MaskedList L = masked_list(ml, nbp);
    const unsigned total = L.count[2];
    for (unsigned i = blockIdx.x; i < total; i += gridDim.x) {
      int bp, bq;
      bool full;
      list_item(L, i, bp, bq, full);
      const unsigned op = L.ord[2 * (long)i], oq = L.ord[2 * (long)i + 1];
      if (!wait_cols2(done, bp, bq, op, oq, state)) return;
      jr_block_pair<JR_NT, JR_RPT, false>(B, ldb, m, n, V, ldv, nb, bp, bq, full ? 0 : 1, tol, smax, cnt, sh);
      post_cols2(done, bp, bq, op + 1, oq + 1);
    }
    finish_sweep(state, cnt, sweep, tan_stop);
    return;
  }
  const unsigned base = (unsigned)sweep * (unsigned)(nbp - 1);
  const bool dataflow = npairs > (int)gridDim.x;
  const long nit = dataflow ? ((long)(nbp - 1) * npairs - blockIdx.x + gridDim.x - 1) / gridDim.x : (long)(nbp - 1);
  for (long t = 0; t < nit; t++) {
    const long it = dataflow ? blockIdx.x + t * (long)gridDim.x : t * npairs + blockIdx.x;
    const int round = (int)(it / npairs), pair = (int)(it % npairs);
    int bp, bq;
    pair_cols(nbp, round, pair, bp, bq);
    if (dataflow && !wait_cols(flags, bp, bq, nb, base + round, state)) return;
    if (bp < nb) jr_block_pair<JR_NT, JR_RPT, false>(B, ldb, m, n, V, ldv, nb, bp, bq, round, tol, smax, cnt, sh);
    if (dataflow) post_cols(flags, bp, bq, nb, base + round + 1);
    else {
      __syncthreads();
      if (!grid_barrier(state + 2)) return;
    }
  }
  finish_sweep(state, cnt, sweep, tan_stop);
}


// Barrier over all threads of a thread-block cluster; release/acquire orders the global-memory
// writes of a round before the reads of the next one.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// FP32 block Jacobi for k <= 128 columns of at most 128 rows: the whole iteration in one
// thread-block cluster with one 128-thread CTA per block pair of a round (one row per thread,
// V's rows prefetched with B's), the hardware cluster barrier between block rounds and all sweeps
// in one launch.  A sweep has nb - 1 block rounds (nb = k / 4 blocks) instead of the scalar
// kernel's k - 1 rounds; the local rounds inside a block pair need only CTA barriers.  state as in
// jacobi_cluster_k.
constexpr int JC_NT = 128;
__global__ void __launch_bounds__(JC_NT) jacobi_block_cluster_k(float2* __restrict__ B, long ldb, int m, int n,
                                                                float2* __restrict__ V, long ldv, float tol,
                                                                const double* __restrict__ smax_p, int max_sweeps,
                                                                unsigned* __restrict__ state, float tan_stop) {
  __shared__ JrShared<JC_NT> sh;
  const float smax = (float)(smax_p[0] / smax_p[1]);
  const int nb = (n + JR_W - 1) / JR_W, nbp = nb + (nb & 1), npairs = nbp / 2;
  int sweep = 0;
  bool conv = false;
  for (; sweep < max_sweeps && !conv; sweep++) {
    unsigned* cnt = state + 8 + SW_STRIDE * sweep;
    for (int round = 0; round < nbp - 1; round++) {
      for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
        int bp, bq;
        pair_cols(nbp, round, pair, bp, bq);
        if (bp < nb) jr_block_pair<JC_NT, 1, true>(B, ldb, m, n, V, ldv, nb, bp, bq, round, tol, smax, cnt, sh);
        __syncthreads();  // shared state is reused by the next item
      }
      cluster_sync_all();
    }
    const unsigned h = __ldcg(cnt);
    const float tmax = __uint_as_float(__ldcg(cnt + 1));
    conv = h == 0 || tmax < tan_stop;
    cluster_sync_all();  // everyone has read this sweep's counters
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    state[0] = conv ? 1u : 0u;
    state[1] = sweep;
  }
}

// Small problems (k <= 128 columns): the whole Jacobi iteration in one thread-block cluster of up
// to 16 CTAs.  Each warp owns a pair of the round (1-4 warps per CTA, so a round's work spreads
// over as many SMs as the cluster allows), the hardware
// cluster barrier separates rounds, and sweeps repeat inside the kernel until one rotates nothing
// or rotates by less than tan_stop.  Cluster CTAs are co-scheduled by the hardware, so the barrier
// needs no co-residency argument; column reads go to L2 (ld.global.cg) so a CTA always sees the
// rotations other CTAs made in the previous round.  Up to 128 rows, a pair's rows of B and of V
// are loaded into registers together at the start of the pair (4 rows per lane) and stay there
// through the rotation, so a round costs one L2 round trip instead of three.  state[0] =
// converged, state[1] = sweeps, state[8 + s] = rotations of sweep s (global counters, shared by
// the cluster).

constexpr int CCR = 4;  // rows per lane held in registers by the cluster kernels (m <= 128)

template <typename T>
__global__ void __launch_bounds__(128) jacobi_cluster_k(cplx_t<T>* __restrict__ B, long ldb, int m, int n,
                                                        cplx_t<T>* __restrict__ V, long ldv, T tol,
                                                        const double* __restrict__ smax_p, int max_sweeps,
                                                        unsigned* __restrict__ state, float tan_stop) {
  using C = cplx_t<T>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpc = blockDim.x >> 5;
  const int gw = blockIdx.x * wpc + warp, nw = gridDim.x * wpc;
  const int np = n + (n & 1), np1 = np - 1, npairs = np / 2;
  const T smax = (T)(smax_p[0] / smax_p[1]);
  int sweep = 0;
  bool conv = false;
  for (; sweep < max_sweeps && !conv; sweep++) {
    unsigned* cnt = state + 8 + SW_STRIDE * sweep;
    for (int round = 0; round < np1; round++) {
      for (int pair = gw; pair < npairs; pair += nw) {
        int p, q;
        if (pair == 0) { p = round; q = np1; }
        else { p = (round + pair) % np1; q = (round - pair + np1) % np1; }
        if (p >= n || q >= n) continue;
        if (p > q) { int t = p; p = q; q = t; }
        C* bp = B + (long)p * ldb;
        C* bq = B + (long)q * ldb;
        C* vp = V + (long)p * ldv;
        C* vq = V + (long)q * ldv;
        if (m <= 32 * CCR) {
          // rows in registers: one L2 round trip per round for B and V together
          C x[CCR], y[CCR], u[CCR], w[CCR];
#pragma unroll
          for (int j = 0; j < CCR; j++) {
            const int r = lane + 32 * j;
            x[j].x = x[j].y = y[j].x = y[j].y = u[j].x = u[j].y = w[j].x = w[j].y = T(0);
            if (r < m) { x[j] = __ldcg(bp + r); y[j] = __ldcg(bq + r); }
            if (r < n) { u[j] = __ldcg(vp + r); w[j] = __ldcg(vq + r); }
          }
          T a = 0, b = 0, gr = 0, gi = 0;
#pragma unroll
          for (int j = 0; j < CCR; j++) {
            if (32 * j >= m) break;  // warp-uniform: no arithmetic on padding rows
            a += x[j].x * x[j].x + x[j].y * x[j].y;
            b += y[j].x * y[j].x + y[j].y * y[j].y;
            gr += x[j].x * y[j].x + x[j].y * y[j].y;
            gi += x[j].x * y[j].y - x[j].y * y[j].x;
          }
          const T k4 = warp_sum4_t<T>(a, b, gr, gi);
          a = __shfl_sync(0xffffffffu, k4, 0);
          b = __shfl_sync(0xffffffffu, k4, 8);
          gr = __shfl_sync(0xffffffffu, k4, 16);
          gi = __shfl_sync(0xffffffffu, k4, 24);
          T c, sr, si;
          float tabs;
          if (!rotation_params<T>(a, b, gr, gi, tol, smax, c, sr, si, tabs)) continue;
#pragma unroll
          for (int j = 0; j < CCR; j++) {
            const int r = lane + 32 * j;
            if (32 * j < m) {
              rot(x[j], y[j], c, sr, si);
              if (r < m) { __stcg(bp + r, x[j]); __stcg(bq + r, y[j]); }
            }
            if (32 * j < n) {
              rot(u[j], w[j], c, sr, si);
              if (r < n) { __stcg(vp + r, u[j]); __stcg(vq + r, w[j]); }
            }
          }
          if (lane == 0) {
            atomicAdd(cnt, 1u);
            atomicMax(cnt + 1, __float_as_uint(tabs));
            atomicMax(cnt + 2, __float_as_uint((float)((gr * gr + gi * gi) / (a * b))));
          }
          continue;
        }
        T a = 0, b = 0, gr = 0, gi = 0;
        for (int r = lane; r < m; r += 32) {
          C x = __ldcg(bp + r), y = __ldcg(bq + r);
          a += x.x * x.x + x.y * x.y;
          b += y.x * y.x + y.y * y.y;
          gr += x.x * y.x + x.y * y.y;
          gi += x.x * y.y - x.y * y.x;
        }
        a = warp_sum(a); b = warp_sum(b); gr = warp_sum(gr); gi = warp_sum(gi);
        T c, sr, si;
        float tabs;
        if (!rotation_params<T>(a, b, gr, gi, tol, smax, c, sr, si, tabs)) continue;
        for (int r = lane; r < m; r += 32) {
          C x = __ldcg(bp + r), y = __ldcg(bq + r);
          rot(x, y, c, sr, si);
          __stcg(bp + r, x);
          __stcg(bq + r, y);
        }
        for (int r = lane; r < n; r += 32) {
          C x = __ldcg(vp + r), y = __ldcg(vq + r);
          rot(x, y, c, sr, si);
          __stcg(vp + r, x);
          __stcg(vq + r, y);
        }
        if (lane == 0) {
          atomicAdd(cnt, 1u);
          atomicMax(cnt + 1, __float_as_uint(tabs));
          atomicMax(cnt + 2, __float_as_uint((float)((gr * gr + gi * gi) / (a * b))));
        }
      }
      cluster_sync_all();
    }
    const unsigned h = __ldcg(cnt);
    const float tmax = __uint_as_float(__ldcg(cnt + 1));
    conv = h == 0 || tmax < tan_stop;
    cluster_sync_all();  // everyone has read this sweep's counters
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    state[0] = conv ? 1u : 0u;
    state[1] = sweep;
  }
}

// ---- double-float (FP32 pair) Jacobi polish ----------------------------------------------------
// Staged double-float rotation of rows [0, len) of a column pair (as rot_cols_staged).
template <int NT, int RPT>
__device__ __forceinline__ void df_rot_cols_staged(float2* ph, float2* pl, float2* qh, float2* ql, int len,
                                                   const DfParams& P) {
  for (int base = 0; base < len; base += NT * RPT) {
    float2 xh[RPT], xl[RPT], yh[RPT], yl[RPT];
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const int r = base + threadIdx.x + j * NT;
      if (r < len) {
        xh[j] = ld_cg_ordered(ph + r); xl[j] = ld_cg_ordered(pl + r);
        yh[j] = ld_cg_ordered(qh + r); yl[j] = ld_cg_ordered(ql + r);
      }
    }
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const int r = base + threadIdx.x + j * NT;
      if (r < len) {
        df_rot_any(xh[j], xl[j], yh[j], yl[j], P);
        __stcg(ph + r, xh[j]); __stcg(pl + r, xl[j]); __stcg(qh + r, yh[j]); __stcg(ql + r, yl[j]);
      }
    }
  }
}

// V's two columns (hi and lo, n rows each) are staged into shared memory (SV[4][n]) by cp.async
// right after the column flags are acquired, so their L2 round trip overlaps the inner products,
// the reduction and the rotation parameters (SV = nullptr: register-staged loads after them).
__device__ __forceinline__ void cp_async16_l2(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

template <int NT, int RPT>
__device__ __forceinline__ void jacobi_pair_df(float2* __restrict__ Bh, float2* __restrict__ Bl, long ldb, int m,
                                               int n, float2* __restrict__ Vh, float2* __restrict__ Vl, long ldv,
                                               int p, int q, double tol, double smax, unsigned* __restrict__ count,
                                               float2* SV) {
  __shared__ float red[8][NT / 32];
  __shared__ DfParams P;
  float2* const vcol[4] = {Vh + (long)p * ldv, Vl + (long)p * ldv, Vh + (long)q * ldv, Vl + (long)q * ldv};
  if (SV) {
    const int chunks = n / 2;  // 16-byte chunks per column (n even)
#pragma unroll
    for (int c = 0; c < 4; c++)
      for (int h = threadIdx.x; h < chunks; h += NT) cp_async16_l2(SV + (long)c * n + 2 * h, vcol[c] + 2 * h);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  float2 *bph = Bh + (long)p * ldb, *bpl = Bl + (long)p * ldb;
  float2 *bqh = Bh + (long)q * ldb, *bql = Bl + (long)q * ldb;
  const bool fits = m <= NT * RPT;
  float2 xh[RPT], xl[RPT], yh[RPT], yl[RPT];
  DotAcc a{0.f, 0.f}, b{0.f, 0.f}, gr{0.f, 0.f}, gi{0.f, 0.f};
  for (int base = 0; base < m; base += NT * RPT) {
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const int r = base + threadIdx.x + j * NT;
      if (r < m) { xh[j] = __ldcg(bph + r); xl[j] = __ldcg(bpl + r); yh[j] = __ldcg(bqh + r); yl[j] = __ldcg(bql + r); }
      else { xh[j] = xl[j] = yh[j] = yl[j] = make_float2(0.f, 0.f); }
    }
#pragma unroll
    for (int j = 0; j < RPT; j++) df_dot_acc(xh[j], xl[j], yh[j], yl[j], a, b, gr, gi);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const dfl k = df_warp_sum4_t(dot_final(a), dot_final(b), dot_final(gr), dot_final(gi));
  if ((l & 7) == 0) { red[2 * (l >> 3)][w] = k.h; red[2 * (l >> 3) + 1][w] = k.l; }
  __syncthreads();
  if (w == 0) {
    dfl v{0.f, 0.f};
    if (l < 4) {
#pragma unroll
      for (int i = 0; i < NT / 32; i++) v = df_add(v, {red[2 * l][i], red[2 * l + 1][i]});
    }
    const dfl sa = df_shfl(v, 0), sb = df_shfl(v, 1), sgr = df_shfl(v, 2), sgi = df_shfl(v, 3);
    if (l == 0) P.go = rotation_params_df(sa, sb, sgr, sgi, (float)tol, (float)smax, P) ? 1 : 0;
  }
  __syncthreads();
  if (!P.go) {
    if (SV) asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // SV is refilled by the next pair
    return;
  }
  const DfParams Pl = P;
  if (fits) {
#pragma unroll
    for (int j = 0; j < RPT; j++) {
      const int r = threadIdx.x + j * NT;
      df_rot_any(xh[j], xl[j], yh[j], yl[j], Pl);
      if (r < m) { __stcg(bph + r, xh[j]); __stcg(bpl + r, xl[j]); __stcg(bqh + r, yh[j]); __stcg(bql + r, yl[j]); }
    }
  } else {  // rows beyond NT * RPT (rare): reload and rotate row by row
    for (int r = threadIdx.x; r < m; r += NT) {
      float2 uh = __ldcg(bph + r), ul = __ldcg(bpl + r), wh = __ldcg(bqh + r), wl = __ldcg(bql + r);
      df_rot_any(uh, ul, wh, wl, Pl);
      __stcg(bph + r, uh); __stcg(bpl + r, ul); __stcg(bqh + r, wh); __stcg(bql + r, wl);
    }
  }
  asm volatile("" ::: "memory");
  if (SV) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();  // rows were copied by other threads
    for (int r = threadIdx.x; r < n; r += NT) {
      float2 uh = SV[r], ul = SV[n + r], wh = SV[2 * n + r], wl = SV[3 * n + r];
      df_rot_any(uh, ul, wh, wl, Pl);
      __stcg(vcol[0] + r, uh); __stcg(vcol[1] + r, ul); __stcg(vcol[2] + r, wh); __stcg(vcol[3] + r, wl);
    }
  } else {
    df_rot_cols_staged<NT, RPT / 2>(vcol[0], vcol[1], vcol[2], vcol[3], n, Pl);
  }
  if (threadIdx.x == 0) {
    atomicAdd(count, 1u);
    atomicMax(count + 1, __float_as_uint(P.tabs));
  }
}

// One polish sweep in double-float, convergence decided on the device (state layout as in
// jacobi_sweep_dev_k; sigma_max of the pre-scaled columns is smax_p[0] / smax_p[1]).
// Double-float polish for k <= 128 columns of at most 128 rows: the whole iteration in one
// thread-block cluster, laid out as jacobi_cluster_k (one warp per pair of a round, the hardware
// cluster barrier between rounds, all sweeps in one launch).  A pair's rows of B and V (hi and lo,
// 4 rows per lane) are loaded together and stay in registers through the rotation; every lane
// forms the same rotation parameters from the broadcast double-float sums, so a pair needs no
// shared memory and no CTA barrier.  Pairs with both columns at or beyond k0 are skipped, and the
// iteration stops after a sweep that rotates nothing or whose largest tangent is below tan_stop.
// state as in jacobi_cluster_k.
__global__ void __launch_bounds__(128) jacobi_cluster_df_k(float2* __restrict__ Bh, float2* __restrict__ Bl,
                                                           long ldb, int m, int n, float2* __restrict__ Vh,
                                                           float2* __restrict__ Vl, long ldv, float tol,
                                                           const double* __restrict__ smax_p, int max_sweeps,
                                                           unsigned* __restrict__ state, int k0, float tan_stop) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpc = blockDim.x >> 5;
  const int gw = blockIdx.x * wpc + warp, nw = gridDim.x * wpc;
  const int np = n + (n & 1), npairs = np / 2;
  const float smax = (float)(smax_p[0] / smax_p[1]);
  int sweep = 0;
  bool conv = false;
  for (; sweep < max_sweeps && !conv; sweep++) {
    unsigned* cnt = state + 8 + SW_STRIDE * sweep;
    for (int round = 0; round < np - 1; round++) {
      for (int pair = gw; pair < npairs; pair += nw) {
        int p, q;
        pair_cols(np, round, pair, p, q);
        if (q >= n || p >= k0) continue;
        float2 *bph = Bh + (long)p * ldb, *bpl = Bl + (long)p * ldb;
        float2 *bqh = Bh + (long)q * ldb, *bql = Bl + (long)q * ldb;
        float2 *vph = Vh + (long)p * ldv, *vpl = Vl + (long)p * ldv;
        float2 *vqh = Vh + (long)q * ldv, *vql = Vl + (long)q * ldv;
        float2 xh[CCR], xl[CCR], yh[CCR], yl[CCR], uh[CCR], ul[CCR], wh[CCR], wl[CCR];
#pragma unroll
        for (int j = 0; j < CCR; j++) {
          const int r = lane + 32 * j;
          const float2 z = make_float2(0.f, 0.f);
          xh[j] = xl[j] = yh[j] = yl[j] = uh[j] = ul[j] = wh[j] = wl[j] = z;
          if (r < m) { xh[j] = __ldcg(bph + r); xl[j] = __ldcg(bpl + r); yh[j] = __ldcg(bqh + r); yl[j] = __ldcg(bql + r); }
          if (r < n) { uh[j] = __ldcg(vph + r); ul[j] = __ldcg(vpl + r); wh[j] = __ldcg(vqh + r); wl[j] = __ldcg(vql + r); }
        }
        DotAcc a{0.f, 0.f}, b{0.f, 0.f}, gr{0.f, 0.f}, gi{0.f, 0.f};
#pragma unroll
        for (int j = 0; j < CCR; j++)
          if (32 * j < m) df_dot_acc(xh[j], xl[j], yh[j], yl[j], a, b, gr, gi);  // warp-uniform test
        const dfl k4 = df_warp_sum4_t(dot_final(a), dot_final(b), dot_final(gr), dot_final(gi));
        DfParams P;
        if (!rotation_params_df(df_shfl(k4, 0), df_shfl(k4, 8), df_shfl(k4, 16), df_shfl(k4, 24), tol, smax, P))
          continue;
        const bool small = P.tabs < 0x1p-24f;
#pragma unroll
        for (int j = 0; j < CCR; j++) {
          const int r = lane + 32 * j;
          if (32 * j < m) {
            if (small) df_rot_small(xh[j], xl[j], yh[j], yl[j], P.sr.h, P.si.h);
            else df_rot(xh[j], xl[j], yh[j], yl[j], P.c, P.sr, P.si);
            if (r < m) { __stcg(bph + r, xh[j]); __stcg(bpl + r, xl[j]); __stcg(bqh + r, yh[j]); __stcg(bql + r, yl[j]); }
          }
          if (32 * j < n) {
            if (small) df_rot_small(uh[j], ul[j], wh[j], wl[j], P.sr.h, P.si.h);
            else df_rot(uh[j], ul[j], wh[j], wl[j], P.c, P.sr, P.si);
            if (r < n) { __stcg(vph + r, uh[j]); __stcg(vpl + r, ul[j]); __stcg(vqh + r, wh[j]); __stcg(vql + r, wl[j]); }
          }
        }
        if (lane == 0) {
          atomicAdd(cnt, 1u);
          atomicMax(cnt + 1, __float_as_uint(P.tabs));
        }
      }
      cluster_sync_all();
    }
    const unsigned h = __ldcg(cnt);
    const float tmax = __uint_as_float(__ldcg(cnt + 1));
    conv = h == 0 || tmax < tan_stop;
    cluster_sync_all();  // everyone has read this sweep's counters
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    state[0] = conv ? 1u : 0u;
    state[1] = sweep;
  }
}

// ---- double-float block polish: pairs of 2-column blocks -------------------------------------
// A work item is a pair of 2-column blocks, 4 columns that one 512-thread CTA holds in registers
// (4 rows x 4 columns of double-float complex per thread, up to 2048 rows).  Its pairs are met in
// local rounds of 2 disjoint pairs: all 6 in 3 rounds in round 0 of a sweep (the pairs inside the
// blocks too), the 4 cross pairs in 2 rounds later, so each pair is met once per sweep.  A local
// round forms both pairs' double-float sums with one transposed warp reduction each and a
// shared-memory reduction across warps, two lanes form the two rotations in parallel, and every
// thread rotates its registers.  V's 4 columns (hi and lo) are staged in shared memory by
// cp.async while B is loaded and the local rounds run; the item's rotations are replayed on them
// in order afterwards.  Against the scalar sweep (one pair per item): half the dependent rounds
// per sweep (k / 2 - 1 instead of k - 1), half of B's and V's column loads and stores per pair,
// one flag wait and post per 4 pairs, and the two pairs' parameters formed side by side.
constexpr int DB_NT = 512, DB_RPT = 4, DB_C = 4;
constexpr int DB_MAXROWS = DB_NT * DB_RPT;  // 2048

struct DbShared {
  float red[2][8][DB_NT / 32];  // [pair][value (a, b, gr, gi) x (hi, lo)][warp]
  DfParams P[6];                // the item's rotations: slot 2 lr + g of local round lr, pair g
  int col[DB_C];
  int rotated;
};

// pair g (0, 1) of local round lr: round 0 of a sweep (FULL) meets (0,1)(2,3), (0,2)(1,3),
// (0,3)(1,2); later rounds meet the cross pairs (0,2)(1,3), (0,3)(1,2)
__device__ __forceinline__ void db_pair(bool full, int lr, int g, int& p, int& q) {
  if (full && lr == 0) {
    p = 2 * g;
    q = 2 * g + 1;
  } else {
    const int r = full ? lr - 1 : lr;
    p = g;
    q = r == 0 ? 2 + g : 3 - g;
  }
}

template <bool FULL, int LR>
__device__ __forceinline__ void db_local_round(float2 (&xh)[DB_C][DB_RPT], float2 (&xl)[DB_C][DB_RPT], DbShared& sh,
                                               int m, float tol, float smax, int k0, unsigned* cnt) {
  const int tid = threadIdx.x, l = tid & 31, w = tid >> 5;
  int p0, q0, p1, q1;
  db_pair(FULL, LR, 0, p0, q0);
  db_pair(FULL, LR, 1, p1, q1);
  DotAcc a0{0.f, 0.f}, b0{0.f, 0.f}, r0{0.f, 0.f}, i0{0.f, 0.f};
  DotAcc a1{0.f, 0.f}, b1{0.f, 0.f}, r1{0.f, 0.f}, i1{0.f, 0.f};
#pragma unroll
  for (int j = 0; j < DB_RPT; j++) {
    df_dot_acc(xh[p0][j], xl[p0][j], xh[q0][j], xl[q0][j], a0, b0, r0, i0);
    df_dot_acc(xh[p1][j], xl[p1][j], xh[q1][j], xl[q1][j], a1, b1, r1, i1);
  }
  const dfl k0s = df_warp_sum4_t(dot_final(a0), dot_final(b0), dot_final(r0), dot_final(i0));
  const dfl k1s = df_warp_sum4_t(dot_final(a1), dot_final(b1), dot_final(r1), dot_final(i1));
  if ((l & 7) == 0) {
    const int v = l >> 3;  // value index: a, b, gr, gi
    sh.red[0][2 * v][w] = k0s.h;
    sh.red[0][2 * v + 1][w] = k0s.l;
    sh.red[1][2 * v][w] = k1s.h;
    sh.red[1][2 * v + 1][w] = k1s.l;
  }
  __syncthreads();
  if (w == 0) {
    dfl v{0.f, 0.f};
    if (l < 8) {  // lanes 0-3: pair 0's values, 4-7: pair 1's
      const int g = l >> 2, vi = l & 3;
#pragma unroll
      for (int i = 0; i < DB_NT / 32; i++) v = df_add(v, {sh.red[g][2 * vi][i], sh.red[g][2 * vi + 1][i]});
    }
    const int base = (l >> 2) << 2;
    const dfl sa = df_shfl(v, base & 7), sb = df_shfl(v, (base + 1) & 7);
    const dfl sgr = df_shfl(v, (base + 2) & 7), sgi = df_shfl(v, (base + 3) & 7);
    if (l == 0 || l == 4) {
      const int g = l >> 2;
      const int p = g ? p1 : p0, q = g ? q1 : q0;
      const int cp = sh.col[p], cq = sh.col[q];
      DfParams P;
      const bool live = cp >= 0 && cq >= 0 && (cp < cq ? cp : cq) < k0;
      const bool go = live && rotation_params_df(sa, sb, sgr, sgi, tol, smax, P);
      P.go = go ? 1 : 0;
      sh.P[2 * LR + g] = P;
      if (go) {
        atomicAdd(cnt, 1u);
        atomicMax(cnt + 1, __float_as_uint(P.tabs));
        sh.rotated = 1;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int g = 0; g < 2; g++) {
    const DfParams& P = sh.P[2 * LR + g];
    if (!P.go) continue;
    const int p = g ? p1 : p0, q = g ? q1 : q0;
#pragma unroll
    for (int j = 0; j < DB_RPT; j++) df_rot_any(xh[p][j], xl[p][j], xh[q][j], xl[q][j], P);
  }
  (void)m;
}

// The item's rotations (sh.P, slot 2 lr + g) replayed in order on the staged rows of V's 4 columns,
// then V's columns stored; each thread takes rows tid, tid + DB_NT, ...
template <bool FULL>
__device__ __forceinline__ void db_replay_v(float2* __restrict__ Vh, float2* __restrict__ Vl, long ldv, int n,
                                            const DbShared& sh, const float2* SV) {
  constexpr int NLR = FULL ? 3 : 2;
  for (int r = threadIdx.x; r < n; r += DB_NT) {
    float2 vh[DB_C], vl[DB_C];
#pragma unroll
    for (int c = 0; c < DB_C; c++) {
      vh[c] = SV[(long)(2 * c) * n + r];
      vl[c] = SV[(long)(2 * c + 1) * n + r];
    }
#pragma unroll
    for (int lr = 0; lr < NLR; lr++)
#pragma unroll
      for (int g = 0; g < 2; g++) {
        const DfParams& P = sh.P[2 * lr + g];
        if (!P.go) continue;
        int p, q;
        db_pair(FULL, lr, g, p, q);  // compile-time after unrolling
        df_rot_any(vh[p], vl[p], vh[q], vl[q], P);
      }
#pragma unroll
    for (int c = 0; c < DB_C; c++) {
      const int col = sh.col[c];
      if (col < 0) continue;
      __stcg(Vh + (long)col * ldv + r, vh[c]);
      __stcg(Vl + (long)col * ldv + r, vl[c]);
    }
  }
}

// One work item: block pair (bp, bq) of round `round`.  SV: 4 columns x (hi, lo) x n staging.
__device__ __forceinline__ void db_block_pair(float2* __restrict__ Bh, float2* __restrict__ Bl, long ldb, int m, int n,
                                              float2* __restrict__ Vh, float2* __restrict__ Vl, long ldv, int nb,
                                              int bp, int bq, int round, float tol, float smax, int k0,
                                              unsigned* cnt, DbShared& sh, float2* SV) {
  const int tid = threadIdx.x;
  if (tid < DB_C) {
    const int blk = tid < 2 ? bp : bq, c = 2 * blk + (tid & 1);
    sh.col[tid] = (blk < nb && c < n) ? c : -1;
  }
  if (tid < 6) sh.P[tid].go = 0;
  if (tid == 0) sh.rotated = 0;
  __syncthreads();
  if (2 * bp >= k0) return;  // all four columns at or beyond k0: none of its pairs rotates
  // V's live columns into shared memory while B is loaded and the local rounds run
  const int chunks = n / 2;  // 16-byte chunks per column (n even)
#pragma unroll
  for (int c = 0; c < DB_C; c++) {
    const int col = sh.col[c];
    if (col < 0) continue;
    for (int h = tid; h < chunks; h += DB_NT) {
      cp_async16_l2(SV + ((long)(2 * c) * n) + 2 * h, Vh + (long)col * ldv + 2 * h);
      cp_async16_l2(SV + ((long)(2 * c + 1) * n) + 2 * h, Vl + (long)col * ldv + 2 * h);
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  float2 xh[DB_C][DB_RPT], xl[DB_C][DB_RPT];
#pragma unroll
  for (int c = 0; c < DB_C; c++) {
    const int col = sh.col[c];
#pragma unroll
    for (int j = 0; j < DB_RPT; j++) {
      const int r = tid + DB_NT * j;
      const bool ok = col >= 0 && r < m;
      xh[c][j] = ok ? __ldcg(Bh + (long)col * ldb + r) : make_float2(0.f, 0.f);
      xl[c][j] = ok ? __ldcg(Bl + (long)col * ldb + r) : make_float2(0.f, 0.f);
    }
  }
  if (round == 0) {
    db_local_round<true, 0>(xh, xl, sh, m, tol, smax, k0, cnt);
    db_local_round<true, 1>(xh, xl, sh, m, tol, smax, k0, cnt);
    db_local_round<true, 2>(xh, xl, sh, m, tol, smax, k0, cnt);
  } else {
    db_local_round<false, 0>(xh, xl, sh, m, tol, smax, k0, cnt);
    db_local_round<false, 1>(xh, xl, sh, m, tol, smax, k0, cnt);
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();  // the rotated flag is final; every thread's staged V rows have landed
  if (!sh.rotated) return;
#pragma unroll
  for (int c = 0; c < DB_C; c++) {
    const int col = sh.col[c];
    if (col < 0) continue;
#pragma unroll
    for (int j = 0; j < DB_RPT; j++) {
      const int r = tid + DB_NT * j;
      if (r < m) {
        __stcg(Bh + (long)col * ldb + r, xh[c][j]);
        __stcg(Bl + (long)col * ldb + r, xl[c][j]);
      }
    }
  }
  // the item's rotations on V's rows, in the order they were made (each thread its own rows)
  if (round == 0) db_replay_v<true>(Vh, Vl, ldv, n, sh, SV);
  else db_replay_v<false>(Vh, Vl, ldv, n, sh, SV);
}

// One block polish sweep (state, flags over the nbp blocks and convergence as jacobi_sweep_df_k).
__global__ void __launch_bounds__(DB_NT, 1)
    jacobi_block_df_k(float2* __restrict__ Bh, float2* __restrict__ Bl, long ldb, int m, int n, float2* __restrict__ Vh,
                      float2* __restrict__ Vl, long ldv, int nbp, double tol, const double* __restrict__ smax_p,
                      unsigned* __restrict__ state, int sweep, unsigned* __restrict__ flags, int k0) {
  __shared__ DbShared sh;
  extern __shared__ __align__(16) float2 db_sv[];
  if (((volatile unsigned*)state)[0]) return;
  const float smax = (float)(smax_p[0] / smax_p[1]);
  unsigned* cnt = state + 8 + SW_STRIDE * sweep;
  const int nb = (n + 1) / 2;
  const int npairs = nbp / 2;
  const unsigned base = (unsigned)sweep * (unsigned)(nbp - 1);
  const bool dataflow = npairs > (int)gridDim.x;
  const long nit = dataflow ? ((long)(nbp - 1) * npairs - blockIdx.x + gridDim.x - 1) / gridDim.x : (long)(nbp - 1);
  for (long t = 0; t < nit; t++) {
    const long it = dataflow ? blockIdx.x + t * (long)gridDim.x : t * npairs + blockIdx.x;
    const int round = (int)(it / npairs), pair = (int)(it % npairs);
    int bp, bq;
    pair_cols(nbp, round, pair, bp, bq);
    if (dataflow && !wait_cols(flags, bp, bq, nb, base + round, state)) return;
    if (bp < nb) db_block_pair(Bh, Bl, ldb, m, n, Vh, Vl, ldv, nb, bp, bq, round, (float)tol, smax, k0, cnt, sh, db_sv);
    if (dataflow) post_cols(flags, bp, bq, nb, base + round + 1);
    else {
      __syncthreads();
      if (!grid_barrier(state + 2)) return;
    }
  }
  finish_sweep(state, cnt, sweep, 1e-7f);
}

template <int NT, int RPT>
__global__ void __launch_bounds__(NT, 2) jacobi_sweep_df_k(float2* __restrict__ Bh, float2* __restrict__ Bl, long ldb,
                                                        int m, int n, float2* __restrict__ Vh, float2* __restrict__ Vl,
                                                        long ldv, int np, double tol, const double* __restrict__ smax_p,
                                                        unsigned* __restrict__ state, int sweep,
                                                        unsigned* __restrict__ flags, int k0,
                                                        const unsigned* __restrict__ ml, unsigned* __restrict__ done) {
  if (((volatile unsigned*)state)[0]) return;
  extern __shared__ __align__(16) float2 df_sv[];
  // the host allocates the staging buffer under exactly this condition (16-byte cp.async needs
  // even columns; k <= 4096 keeps two CTAs per SM)
  float2* SV = (n % 2 == 0 && ldv % 2 == 0 && n <= 4096) ? df_sv : nullptr;
  const double smax = smax_p[0] / smax_p[1];
  unsigned* cnt = state + 8 + SW_STRIDE * sweep;
  const int npairs = np / 2;
  const unsigned base = (unsigned)sweep * (unsigned)(np - 1);
  if (ml) {
    // masked sweep: the listed pairs (MaskedList) dealt round-robin to the CTAs; a pair waits
    // until the listed pairs before it on each of its columns are done
    const MaskedList L = masked_list(ml, np);
    const unsigned total = L.count[2];
    for (unsigned i = blockIdx.x; i < total; i += gridDim.x) {
      int p, q;
      bool full;
      list_item(L, i, p, q, full);
      const unsigned op = L.ord[2 * (long)i], oq = L.ord[2 * (long)i + 1];
      if (!wait_cols2(done, p, q, op, oq, state)) return;
      jacobi_pair_df<NT, RPT>(Bh, Bl, ldb, m, n, Vh, Vl, ldv, p, q, tol, smax, cnt, SV);
      post_cols2(done, p, q, op + 1, oq + 1);
    }
    finish_sweep(state, cnt, sweep, 1e-7f);
    return;
  }
  // dataflow: work items in (round, pair) order dealt round-robin to the CTAs, so the surplus
  // pairs rotate over the CTAs from round to round; barrier mode: CTA b owns pair b of every round
  const bool dataflow = npairs > (int)gridDim.x;
  const long nit = dataflow ? ((long)(np - 1) * npairs - blockIdx.x + gridDim.x - 1) / gridDim.x : (long)(np - 1);
  for (long t = 0; t < nit; t++) {
    const long it = dataflow ? blockIdx.x + t * (long)gridDim.x : t * npairs + blockIdx.x;
    const int round = (int)(it / npairs), pair = (int)(it % npairs);
    int p, q;
    pair_cols(np, round, pair, p, q);
    if (dataflow && !wait_cols(flags, p, q, n, base + round, state)) return;
    if (q < n && p < k0) jacobi_pair_df<NT, RPT>(Bh, Bl, ldb, m, n, Vh, Vl, ldv, p, q, tol, smax, cnt, SV);
    if (dataflow) post_cols(flags, p, q, n, base + round + 1);
    else if (!grid_barrier(state + 2)) return;
  }
  // a sweep whose largest tangent is below 1e-7 leaves couplings ~1e-15 (measured quadratic
  // constant 0.05-0.3): the next sweep would only confirm convergence
  finish_sweep(state, cnt, sweep, 1e-7f);
}

// Xh[:, j] = src[:, perm[j]], Xl = 0 (an FP32 matrix as a double-float one, columns permuted)
__global__ void gather_cols_f2_k(const float2* __restrict__ src, long lds, int rows, int cols,
                                 const int* __restrict__ perm, float2* __restrict__ hi, float2* __restrict__ lo,
                                 long ldd) {
  const long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long i = t % rows, j = t / rows;
    hi[i + j * ldd] = src[i + (long)perm[j] * lds];
    lo[i + j * ldd] = make_float2(0.f, 0.f);
  }
}


// out[0] = max_j nrm[j] (one block)
__global__ void max_reduce_k(const double* __restrict__ nrm, int k, double* __restrict__ out) {
  __shared__ double red[32];
  double v = 0.0;
  for (int j = threadIdx.x; j < k; j += blockDim.x) v = fmax(v, nrm[j]);
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) out[0] = v;
  }
}

// out = max over the rows x k entries of max(|re|, |im|), as the bits of a non-negative double
// (their unsigned order is the numeric order); NaN entries propagate as NaN
__global__ void max_abs_k(const double2* __restrict__ B, long ldb, int rows, int k, unsigned long long* out) {
  double m = 0.0;
  const long total = (long)rows * k;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const double2 v = B[t % rows + (t / rows) * ldb];
    double a = fabs(v.x);
    const double b = fabs(v.y);
    a = (b > a || b != b) ? b : a;  // fmax would drop a NaN
    m = (a > m || a != a) ? a : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double x = __shfl_xor_sync(0xffffffffu, m, o);
    m = (x > m || x != x) ? x : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// nrm[j] = |col_j| in FP64 (one warp per column)
template <typename C>
__global__ void col_norms_k(const C* __restrict__ B, long ldb, int m, int n, double* __restrict__ nrm) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  const C* col = B + (long)j * ldb;
  double acc = 0.0;
  for (int r = lane; r < m; r += 32) {
    double x = col[r].x, y = col[r].y;
    acc += x * x + y * y;
  }
  acc = warp_sum(acc);
  if (lane == 0) nrm[j] = sqrt(acc);
}

// perm[rank] = j, descending by key (ties by index), one thread per element
__global__ void rank_sort_k(const double* __restrict__ key, int n, int* __restrict__ perm, double* __restrict__ sorted) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double ki = key[i];
  int rank = 0;
  for (int j = 0; j < n; j++) {
    double kj = key[j];
    rank += (kj > ki) || (kj == ki && j < i);
  }
  perm[rank] = i;
  if (sorted) sorted[rank] = ki;
}

// dst[:, j] = src[:, perm[j]] * (scale ? 1/scale[j] : 1), with 1/0 -> 0
template <typename CS>
__global__ void gather_cols_k(const CS* __restrict__ src, long lds, int rows, int cols,
                              const int* __restrict__ perm, const double* __restrict__ sorted_scale,
                              double2* __restrict__ dst, long ldd) {
  long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % rows, j = t / rows;
    CS v = src[i + (long)perm[j] * lds];
    double f = 1.0;
    if (sorted_scale) { double sv = sorted_scale[j]; f = sv > 0.0 ? 1.0 / sv : 0.0; }
    dst[i + j * ldd] = make_double2((double)v.x * f, (double)v.y * f);
  }
}


// Q[:, j] *= phase(R_jj) (R_jj == 0 -> 1): keeps Q as close to the input columns as possible
__global__ void phase_fix_k(double2* Q, long ldq, int m, int k, const double2* R, long ldr) {
  long total = (long)m * k;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % m, j = t / m;
    double2 d = R[j + j * ldr];
    double a = sqrt(d.x * d.x + d.y * d.y);
    double2 ph = a > 0.0 ? make_double2(d.x / a, d.y / a) : make_double2(1.0, 0.0);
    Q[i + j * ldq] = cmul(Q[i + j * ldq], ph);
  }
}

inline unsigned gs(long n) {
  long g = (n + TPB - 1) / TPB;
  if (g > 152L * 32) g = 152L * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

// Hestenes sweeps on B (rows x k) accumulating V (k x k).  Small problems (k <= 32) run the
// whole iteration in one CTA; larger ones enqueue up to max_sweeps cooperative sweep launches
// whose convergence is decided on the device.  One host synchronisation per call.
template <typename T>
int jacobi(cudaStream_t s, SvdWork* w, cplx_t<T>* B, long ldb, int rows, int k, cplx_t<T>* V,
           long ldv, int max_sweeps, T tol, bool must_converge = true, float tan_stop = -1.f,
           int* converged = nullptr, double* last_frac = nullptr) {
  if (tan_stop < 0.f) tan_stop = sizeof(T) == 8 ? 1e-8f : 0.f;
  const int np = k + (k & 1);
  constexpr int NT = sizeof(T) == 8 ? 256 : 128;
  constexpr int RPT = sizeof(T) == 8 ? 8 : 16;
  const int kind = sizeof(T) == 8 ? PK_JACOBI64 : PK_JACOBI32;
  const double pairs = 0.5 * (double)k * (k - 1);
  const int nstate = 8 + SW_STRIDE * max_sweeps;
  // [state (nstate) | column flags (np) | pad | smax, scale (2 doubles)]
  const int soff = nstate + np + ((nstate + np) & 1);
  QR_TRY(w->cnt.ensure(sizeof(unsigned) * soff + 2 * sizeof(double) + 128, s));
  unsigned* state = w->cnt.as<unsigned>();
  unsigned* flags = state + nstate;
  double* nrm = w->nrm.as<double>();
  double* smax_d = reinterpret_cast<double*>(state + soff);
  QR_CUDA(cudaMemsetAsync(state, 0, sizeof(unsigned) * (nstate + np), s));
  // sigma_max scale from the largest column norm, on the device
  col_norms_k<cplx_t<T>><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, ldb, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  max_reduce_k<<<1, 256, 0, s>>>(nrm, k, smax_d);
  QR_CHECK_LAUNCH("max_reduce_k");
  {
    long tot = (long)rows * k;
    unsigned g = (unsigned)((tot + TPB - 1) / TPB);
    pow2_scale_k<cplx_t<T>><<<g > 4864 ? 4864 : g, TPB, 0, s>>>(B, ldb, rows, k, smax_d, smax_d + 1, 0);
    QR_CHECK_LAUNCH("pow2_scale_k");
  }
  int pr = prof_begin(s, kind, 0.0, 0.0);
  const bool small = k <= 128;  // (at 256 columns the FP32 block kernel is 2x faster than the cluster)
  if (small) {
    // one cluster of up to 16 CTAs with one warp per pair of a round: as many CTAs as pairs (up
    // to 16), then 2-4 warps per CTA
    // FP32 with at most 128 rows: the block form (one CTA per block pair of 4-column blocks)
    const bool blk = sizeof(T) == 4 && rows <= JC_NT && k > 2 * JR_W;
    const int nbk = (k + JR_W - 1) / JR_W;
    const int npairs = blk ? (nbk + (nbk & 1)) / 2 : (np / 2 > 0 ? np / 2 : 1);
    const int cl = npairs < 16 ? npairs : 16;
    const int wpc = blk ? JC_NT / 32 : std::min(4, (npairs + cl - 1) / cl);  // warps loop over pairs
    if (cl > 8) {
      const void* f = blk ? (const void*)jacobi_block_cluster_k : (const void*)jacobi_cluster_k<T>;
      QR_TRY(set_func_attr_once(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cl);
    cfg.blockDim = dim3(32 * wpc);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    svd_path(blk ? SP_BLOCK_CLUSTER : SP_CLUSTER);
    if (blk) {
      QR_CUDA(cudaLaunchKernelEx(&cfg, jacobi_block_cluster_k, (float2*)B, ldb, rows, k, (float2*)V, ldv, (float)tol,
                                 (const double*)smax_d, max_sweeps, state, tan_stop));
    } else {
      QR_CUDA(cudaLaunchKernelEx(&cfg, jacobi_cluster_k<T>, B, ldb, rows, k, V, ldv, tol, (const double*)smax_d,
                                 max_sweeps, state, tan_stop));
    }
    count_launch();
  } else if (sizeof(T) == 4 && rows <= JR_MAXROWS) {
    // FP32 with the rows in registers: block Jacobi (4-column blocks, pairs of blocks)
    const int nb = (k + JR_W - 1) / JR_W, nbp = nb + (nb & 1);
    int per_sm = 0, sms = 0;
    QR_TRY(device_sm_count(&sms));
    QR_TRY(blocks_per_sm((const void*)jacobi_block_reg_k, JR_NT, 0, &per_sm));
    if (per_sm < 1) return fail(QR_ECUDA, "block Jacobi sweep kernel cannot be resident");
    int grid = std::min(per_sm * sms, nbp / 2);
    if (grid < 1) grid = 1;
    svd_path(nbp / 2 > grid ? SP_BLOCK_DATAFLOW : SP_BLOCK_BARRIER);
    for (int sweep = 0; sweep < max_sweeps; sweep++) {
      float2* Bp = reinterpret_cast<float2*>(B);
      float2* Vp = reinterpret_cast<float2*>(V);
      long ldbb = ldb, ldvv = ldv;
      int mm = rows, kk2 = k, nbb = nbp, sw = sweep;
      float tl = (float)tol, ts = tan_stop;
      const double* sm = smax_d;
      unsigned* st = state;
      unsigned* fl = flags;
      const unsigned* mlp = nullptr;
      unsigned* dn = nullptr;
      void* args[] = {&Bp, &ldbb, &mm, &kk2, &Vp, &ldvv, &nbb, &tl, &sm, &st, &sw, &fl, &ts, &mlp, &dn};
      QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_block_reg_k, dim3(grid), dim3(JR_NT), args, 0, s));
      count_launch();
    }
  } else {
    int per_sm = 0, sms = 0;
    QR_TRY(device_sm_count(&sms));
    QR_TRY(blocks_per_sm((const void*)jacobi_sweep_dev_k<T, NT, RPT>, NT, 0, &per_sm));
    if (per_sm < 1) return fail(QR_ECUDA, "Jacobi sweep kernel cannot be resident");
    int grid = per_sm * sms;
    if (grid > np / 2) grid = np / 2;
    if (grid < 1) grid = 1;
    if (sizeof(T) == 8) svd_path(np / 2 > grid ? SP_F64_DATAFLOW : SP_F64_BARRIER);
    else svd_path(np / 2 > grid ? SP_F32_DATAFLOW : SP_F32_BARRIER);
    for (int sweep = 0; sweep < max_sweeps; sweep++) {
      cplx_t<T>* Bp = B;
      cplx_t<T>* Vp = V;
      int mm = rows, kk2 = k, npp = np, sw = sweep;
      long ldbb = ldb, ldvv = ldv;
      T tl = tol;
      const double* sm = smax_d;
      unsigned* st = state;
      unsigned* fl = flags;
      float ts = tan_stop;
      void* args[] = {&Bp, &ldbb, &mm, &kk2, &Vp, &ldvv, &npp, &tl, &sm, &st, &sw, &fl, &ts};
      QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_sweep_dev_k<T, NT, RPT>, dim3(grid), dim3(NT), args, 0, s));
      count_launch();
    }
  }
  prof_end(s, pr);
  {
    long tot = (long)rows * k;
    unsigned g = (unsigned)((tot + TPB - 1) / TPB);
    pow2_scale_k<cplx_t<T>><<<g > 4864 ? 4864 : g, TPB, 0, s>>>(B, ldb, rows, k, smax_d, smax_d + 1, 1);
    QR_CHECK_LAUNCH("pow2_scale_k");
  }
  unsigned* hs = static_cast<unsigned*>(host_scratch(sizeof(unsigned) * nstate));
  if (!hs) return fail(QR_ENOMEM, "page-locked host scratch");
  QR_CUDA(cudaMemcpyAsync(hs, state, sizeof(unsigned) * nstate, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  if (hs[4]) return fail(QR_ECUDA, "Jacobi sweep: a column wait timed out");
  const int ran = (int)hs[1];
  double rotated = 0;
  for (int sw = 0; sw < ran; sw++) {
    rotated += hs[8 + SW_STRIDE * sw];
    if (debug_on()) {
      float tmax, rmax;
      memcpy(&tmax, &hs[9 + SW_STRIDE * sw], sizeof(float));
      memcpy(&rmax, &hs[10 + SW_STRIDE * sw], sizeof(float));
      fprintf(stderr, "[qr] jacobi<%s> %dx%d sweep %d rotations %u max tan %.2e max coupling %.2e\n",
              sizeof(T) == 8 ? "f64" : "f32", rows, k, sw, hs[8 + SW_STRIDE * sw], tmax, sqrtf(rmax));
    }
  }
  if (debug_on() && small) fprintf(stderr, "[qr] jacobi_cluster<%s> %dx%d sweeps %d\n", sizeof(T) == 8 ? "f64" : "f32", rows, k, ran);
  // algorithmic work: three inner products per pair and sweep (16 real flops per row) and two
  // column rotations of B and V per rotated pair (20 flops per row and column)
  prof_account(pr, 16.0 * rows * pairs * ran + 40.0 * rotated * (rows + k),
               sizeof(cplx_t<T>) * ((double)rows + k) * 2.0 * (pairs * ran + rotated), ran);
  if (converged) *converged = hs[0] ? 1 : 0;
  if (last_frac) *last_frac = ran > 0 && pairs > 0 ? hs[8 + SW_STRIDE * (ran - 1)] / pairs : 0.0;
  if (!hs[0] && must_converge) return fail(QR_ENOCONV, "Jacobi SVD did not converge");
  return QR_OK;
}

// Schedule of a masked sweep, built on the host from the mask of the MaskedList at hb (a host
// copy of its mask, flag and count): a greedy edge colouring of the marked pairs.  Each colour
// class is a set of disjoint pairs, the classes are listed one after another, and ord gives each
// listed pair its place on its two vertices, so the sweep's dependency depth is the number of
// classes (at most 2 d - 1 for the largest vertex degree d) instead of the nv - 1 rounds of the
// full sweep's order.  A sweep may meet its pairs in any order; this one differs from the full
// sweep's restricted to the marked pairs.  With use_flag, the first listed pair of a flagged
// vertex carries the `full` bit (it also meets the pairs inside its two vertices), and a flagged
// vertex without marked pairs is listed with its neighbour v ^ 1.  Returns the listed pairs.
static long schedule_pairs(unsigned* hb, int nv, bool use_flag, int* classes) {
  const MaskedList H = masked_list(hb, nv);
  std::vector<std::pair<int, int>> e;
  std::vector<int> deg(nv, 0);
  for (int p = 0; p < nv; p++)
    for (int wd = 0; wd < H.mw; wd++) {
      unsigned bits = H.mask[(size_t)p * H.mw + wd];
      while (bits) {
        const int q = 32 * wd + __builtin_ctz(bits);
        bits &= bits - 1;
        e.emplace_back(p, q);
        deg[p]++;
        deg[q]++;
      }
    }
  if (use_flag)
    for (int v = 0; v < nv; v++)
      if (H.flag[v] && deg[v] == 0) {
        const int u = v ^ 1;
        e.emplace_back(std::min(u, v), std::max(u, v));
        deg[u]++;
        deg[v]++;
      }
  const int maxdeg = nv > 0 ? *std::max_element(deg.begin(), deg.end()) : 0;
  const int W = (2 * maxdeg + 63) / 64 + 1;  // colour bitset words per vertex
  std::vector<uint64_t> used((size_t)nv * W, 0);
  std::vector<int> col(e.size());
  int ncol = 0;
  for (size_t i = 0; i < e.size(); i++) {
    const int u = e[i].first, v = e[i].second;
    int c = -1;
    for (int wd = 0; wd < W && c < 0; wd++) {
      const uint64_t fr = ~(used[(size_t)u * W + wd] | used[(size_t)v * W + wd]);
      if (fr) c = 64 * wd + __builtin_ctzll(fr);
    }
    used[(size_t)u * W + c / 64] |= 1ull << (c % 64);
    used[(size_t)v * W + c / 64] |= 1ull << (c % 64);
    col[i] = c;
    ncol = std::max(ncol, c + 1);
  }
  std::vector<long> off(ncol + 1, 0);
  for (int c : col) off[c + 1]++;
  for (int c = 0; c < ncol; c++) off[c + 1] += off[c];
  std::vector<long> pos(e.size());
  for (size_t i = 0; i < e.size(); i++) pos[off[col[i]]++] = (long)i;
  std::vector<unsigned> seen(nv, 0);
  std::vector<char> full_done(nv, 0);
  for (size_t i = 0; i < e.size(); i++) {
    const int u = e[pos[i]].first, v = e[pos[i]].second;
    const bool full = use_flag && ((H.flag[u] && !full_done[u]) || (H.flag[v] && !full_done[v]));
    if (full) full_done[u] = full_done[v] = 1;
    H.items[i] = (unsigned)u | ((unsigned)v << 15) | (full ? 1u << 30 : 0u);
    H.ord[2 * i] = seen[u]++;
    H.ord[2 * i + 1] = seen[v]++;
  }
  *classes = ncol;
  return (long)e.size();
}

}  // namespace

// The host schedule of a masked sweep on caller arrays (for tests): mask and flag as in
// MaskedList (nv rows of ceil(nv / 32) words; flag: nv words or null), items and ord of
// nv (nv - 1) / 2 and 2 nv (nv - 1) / 2 words.  Returns the listed pairs; *classes = colour classes.
long schedule_pairs_host(const unsigned* mask, const unsigned* flag, int nv, int use_flag, unsigned* items,
                         unsigned* ord, int* classes) {
  std::vector<unsigned> hb(masked_list_words(nv), 0u);
  const MaskedList H = masked_list(hb.data(), nv);
  std::copy(mask, mask + (size_t)nv * H.mw, H.mask);
  if (flag) std::copy(flag, flag + nv, H.flag);
  const long n = schedule_pairs(hb.data(), nv, use_flag != 0, classes);
  std::copy(H.items, H.items + n, items);
  std::copy(H.ord, H.ord + 2 * n, ord);
  return n;
}

namespace {

// Brings the mask, flags and counts of the device MaskedList (w->ml, nv vertices) to the host,
// schedules the marked pairs and uploads the schedule and its length (count[2]).  Synchronises s.
static int upload_schedule(cudaStream_t s, SvdWork* w, int nv, bool use_flag, long* listed, int* classes) {
  QR_TRY(w->hl.ensure(sizeof(unsigned) * masked_list_words(nv)));
  unsigned* hb = w->hl.as<unsigned>();
  const MaskedList D = masked_list(w->ml.as<unsigned>(), nv), H = masked_list(hb, nv);
  const size_t pre = (size_t)(D.items - D.mask);  // mask, flag and count words
  QR_CUDA(cudaMemcpyAsync(hb, D.mask, sizeof(unsigned) * pre, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  const long n = schedule_pairs(hb, nv, use_flag, classes);
  H.count[2] = (unsigned)n;
  QR_CUDA(cudaMemcpyAsync(D.count + 2, H.count + 2, sizeof(unsigned), cudaMemcpyHostToDevice, s));
  if (n > 0) {
    QR_CUDA(cudaMemcpyAsync(D.items, H.items, sizeof(unsigned) * n, cudaMemcpyHostToDevice, s));
    QR_CUDA(cudaMemcpyAsync(D.ord, H.ord, sizeof(unsigned) * 2 * n, cudaMemcpyHostToDevice, s));
  }
  *listed = n;
  return QR_OK;
}

// A polish sweep that follows one whose largest tangent was below this value rotates few pairs:
// in a 2048-column polish the sweep after a 3e-4 sweep rotated 3.7 thousand of 2.1 million, with
// tangents below 3e-9.  Such a sweep is masked: the Gram matrix B^H B (one double-float GEMM,
// ~6 ms at 2048 columns against ~70 ms for a sweep that forms every pair's inner products in
// round order) picks the pairs that fail the rotation test, and only those are rotated.
constexpr float kPolishMaskTan = 1e-2f;
// When every marked pair's tangent is at most this, the masked sweep's rotations are applied at
// once to first order: B <- B (I + E), V <- V (I + E) with E_pq = g_pq / (|b_q|^2 - |b_p|^2)
// (g_pq = b_p^H b_q) on the marked pairs, E anti-Hermitian.  Rotating in sweep order instead
// differs by products of two tangents (< 1e-16), I + E is unitary to |E|^2 (< 1e-16 per pair), and
// the FP32 products of B_hi E add ~2^-24 |E| relative error.  Larger tangents take the ordered
// sweep over the marked pairs.
constexpr float kPolishLinTan = 1e-8f;

// |b_c|^2 of the double-float columns (FP64 sums of the double values).
__global__ void col_norms2_df_k(const float2* __restrict__ Bh, const float2* __restrict__ Bl, long ldb, int m, int n,
                                double* __restrict__ nrm2) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  double acc = 0.0;
  for (int r = lane; r < m; r += 32) {
    const float2 h = Bh[(long)j * ldb + r], l = Bl[(long)j * ldb + r];
    const double x = (double)h.x + l.x, y = (double)h.y + l.y;
    acc += x * x + y * y;
  }
  acc = warp_sum(acc);
  if (lane == 0) nrm2[j] = acc;
}

// Pairs a masked polish sweep rotates.  G = I - B^H B (FP32 values of double-float sums, so an
// off-diagonal entry is -b_p^H b_q to FP32 relative accuracy), nrm2[c] = |b_c|^2.  Bit (q & 31) of
// mask[p * words + q / 32] is set for p < q, p < k0, when |g_pq| exceeds the threshold of
// rotation_params_df (tol sigma_max min(|b_p|, |b_q|) + (4 eps sigma_max)^2).  The GEMM's and the
// sweep's summations differ at the rounding level that the threshold sits on (2x above it), so
// the two tests disagree only on pairs whose rotation is rounding noise.  count[0] += marked pairs;
// count[1] = max over marked pairs of |g| / | |b_q|^2 - |b_p|^2 | (float bits; the first-order
// tangent, infinite for equal norms).
__global__ void polish_mask_k(const float2* __restrict__ G, long ldg, const double* __restrict__ nrm2, int n, int k0,
                              double tol, const double* __restrict__ smax_p, unsigned* __restrict__ mask, int words,
                              unsigned* __restrict__ count) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int p = (int)(t % n), wd = (int)(t / n);
  unsigned bits = 0;
  float tmax = 0.f;
  if (wd < words) {
    const double smax = smax_p[0] / smax_p[1];
    const double fl = 4.0 * Eps<double>::v * smax;
    const double ap = nrm2[p], np_ = sqrt(ap);
    for (int b = 0; b < 32; b++) {
      const int q = 32 * wd + b;
      if (q >= n) break;
      if (q <= p || p >= k0) continue;
      const double aq = nrm2[q], nq = sqrt(aq);
      if (!(np_ > 0.0) || !(nq > 0.0)) continue;
      const float2 g = G[p + (long)q * ldg];
      const double gabs = sqrt((double)g.x * g.x + (double)g.y * g.y);
      if (gabs > tol * smax * fmin(np_, nq) + fl * fl) {
        bits |= 1u << b;
        const double d = fabs(aq - ap);
        tmax = fmaxf(tmax, d > 0.0 ? (float)(gabs / d) : __int_as_float(0x7f800000));
      }
    }
    mask[(long)p * words + wd] = bits;
  }
  unsigned c = __popc(bits);
  c = __reduce_add_sync(0xffffffffu, c);
  const unsigned tm = __reduce_max_sync(0xffffffffu, __float_as_uint(tmax));
  if ((threadIdx.x & 31) == 0) {
    if (c) atomicAdd(count, c);
    if (tm) atomicMax(count + 1, tm);
  }
}

// E (k x k, ld k, FP32) in place over G = I - B^H B: E_pq = g_pq / (|b_q|^2 - |b_p|^2) for the
// marked pairs (either order), g_pq = -G_pq; zero elsewhere (diagonal included).
__global__ void polish_lin_k(float2* __restrict__ G, const double* __restrict__ nrm2, int k, const unsigned* ml,
                             int np, int k0) {
  const MaskedList L = masked_list(ml, np);
  const long tot = (long)k * k;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot; e += (long)gridDim.x * blockDim.x) {
    const int p = (int)(e % k), q = (int)(e / k);
    float2 out = make_float2(0.f, 0.f);
    if (p != q && marked(L, p < q ? p : q, p < q ? q : p, k, k0)) {
      const float2 g = G[e];
      const double d = nrm2[q] - nrm2[p];
      out = make_float2((float)(-(double)g.x / d), (float)(-(double)g.y / d));
    }
    G[e] = out;
  }
}

// FP64-accurate polish of (B, V) in double-float on the FP32 pipes.  B (rows x k) and V (k x k)
// arrive as split (hi, lo) arrays with B's columns pre-scaled by a power of two; smax_d[0] /
// smax_d[1] is sigma_max of the scaled columns.  Up to 128 columns of at most 128 rows the whole
// iteration is one cluster launch; otherwise each sweep is one cooperative launch whose state
// (rotations, largest tangent, convergence) is read back before the next, and sweeps after a
// small-tangent sweep are masked (kPolishMaskTan).
// Pairs with both columns at index >= k0 are skipped (k0 = k: none): when the caller keeps only
// the leading singular triplets and the columns arrive sorted by an approximate sigma, the tail
// block needs no internal orthogonality (see zsvd_thin).
int jacobi_df(cudaStream_t s, SvdWork* w, float2* Bh, float2* Bl, long ldb, int rows, int k, float2* Vh,
              float2* Vl, long ldv, int max_sweeps, double tol, const double* smax_d, int k0) {
  constexpr int NT = 256, RPT = 8;
  const int np = k + (k & 1);
  const double pairs = 0.5 * (double)k * (k - 1);
  const int nstate = 8 + SW_STRIDE * max_sweeps;
  // state, the column flags, the masked sweeps' column counters and k column norms (doubles,
  // 8-byte aligned)
  const size_t nwords = (size_t)nstate + 2 * (size_t)np;
  QR_TRY(w->cnt.ensure(sizeof(unsigned) * nwords + sizeof(double) * (k + 1) + 128, s));
  unsigned* state = w->cnt.as<unsigned>();
  unsigned* flags = state + nstate;
  unsigned* done = flags + np;
  double* cnorm = reinterpret_cast<double*>(w->cnt.as<char>() + ((sizeof(unsigned) * nwords + 7) & ~(size_t)7));
  QR_CUDA(cudaMemsetAsync(state, 0, sizeof(unsigned) * (nstate + np), s));
  // V staging buffer: 4 columns (hi, lo of p and q) of k rows; k <= 4096 keeps two CTAs per SM
  const size_t vsm = (k % 2 == 0 && ldv % 2 == 0 && k <= 4096) ? sizeof(float2) * 4 * (size_t)k : 0;
  int per_sm = 0, sms = 0;
  QR_TRY(device_sm_count(&sms));
  QR_TRY(set_func_attr_once((const void*)jacobi_sweep_df_k<NT, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)sizeof(float2) * 4 * 4096));
  QR_TRY(blocks_per_sm((const void*)jacobi_sweep_df_k<NT, RPT>, NT, vsm, &per_sm));
  if (per_sm < 1) return fail(QR_ECUDA, "double-float sweep kernel cannot be resident");
  int grid = std::min(per_sm * sms, np / 2);
  if (grid < 1) grid = 1;
  const bool cluster = k <= 128 && rows <= 32 * CCR;
  // full sweeps as block sweeps (pairs of 2-column blocks) when the rows fit the registers and
  // V's columns can be staged by 16-byte copies
  const bool blockdf = !cluster && rows <= DB_MAXROWS && k % 2 == 0 && ldv % 2 == 0;
  const int nbp = (k + 1) / 2 + (((k + 1) / 2) & 1);
  const size_t dbsm = sizeof(float2) * 8 * (size_t)k;
  int dbgrid = 1;
  if (blockdf) {
    int dper = 0;
    QR_TRY(set_func_attr_once((const void*)jacobi_block_df_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(float2) * 8 * DB_MAXROWS)));
    QR_TRY(blocks_per_sm((const void*)jacobi_block_df_k, DB_NT, dbsm, &dper));
    if (dper < 1) return fail(QR_ECUDA, "double-float block sweep kernel cannot be resident");
    dbgrid = std::max(1, std::min(dper * sms, nbp / 2));
  }
  svd_path(cluster ? SP_DF_CLUSTER
                   : blockdf ? SP_DF_BLOCK : (np / 2 > grid ? SP_DF_DATAFLOW : SP_DF_BARRIER));
  // hs[nstate], hs[nstate + 1] receive a masked sweep's marked-pair count and largest tangent
  unsigned* hs = static_cast<unsigned*>(host_scratch(sizeof(unsigned) * (nstate + 2)));
  if (!hs) return fail(QR_ENOMEM, "page-locked host scratch");
  // FP32 operations: ~96 per row per inner-product pass (compensated sums) and ~100-340 per row
  // and column rotated (small-angle / general rotation); the count takes the general form
  auto account = [&](int pr, double examined, double rotated, long sweeps) {
    prof_account(pr, 96.0 * rows * examined + 344.0 * rotated * (rows + k),
                 sizeof(float2) * 2.0 * ((double)rows + k) * 2.0 * (examined + rotated), sweeps);
  };
  if (cluster) {
    int pr = prof_begin(s, PK_JACOBI_DF, 0.0, 0.0);
    // one cluster of up to 16 CTAs, one warp per pair of a round (as in jacobi<T>)
    const int npairs = np / 2 > 0 ? np / 2 : 1;
    const int cl = npairs < 16 ? npairs : 16;
    const int wpc = std::min(4, (npairs + cl - 1) / cl);
    if (cl > 8) QR_TRY(set_func_attr_once((const void*)jacobi_cluster_df_k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cl);
    cfg.blockDim = dim3(32 * wpc);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    QR_CUDA(cudaLaunchKernelEx(&cfg, jacobi_cluster_df_k, Bh, Bl, ldb, rows, k, Vh, Vl, ldv, (float)tol, smax_d,
                               max_sweeps, state, k0, 1e-7f));
    count_launch();
    prof_end(s, pr);
    QR_CUDA(cudaMemcpyAsync(hs, state, sizeof(unsigned) * nstate, cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaStreamSynchronize(s));
    const int ran = (int)hs[1];
    double rotated = 0;
    for (int sw = 0; sw < ran; sw++) rotated += hs[8 + SW_STRIDE * sw];
    account(pr, pairs * ran, rotated, ran);
    if (!hs[0]) return fail(QR_ENOCONV, "double-float Jacobi polish did not converge");
    return QR_OK;
  }
  // One launch per sweep, the state read back after each (~3 sweeps of tens of ms at the sizes
  // that take this path, so the host round trips cost nothing measurable).  From the first sweep
  // whose largest tangent is below kPolishMaskTan on, every sweep is masked: the Gram test marks
  // the pairs, they are listed in round order and the sweep runs over the list.
  bool masked = false;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    const unsigned* mk = nullptr;
    unsigned marked = 0;
    if (masked) {
      QR_TRY(w->E.ensure(sizeof(float2) * (size_t)k * k, s));
      QR_TRY(w->ml.ensure(sizeof(unsigned) * masked_list_words(np), s));
      float2* G = w->E.as<float2>();
      const MaskedList L = masked_list(w->ml.as<unsigned>(), np);
      QR_TRY(zgemm_df(s, DF_GRAM, OP_C, k, k, rows, Bh, Bl, ldb, Bh, Bl, ldb, G, nullptr, k));
      col_norms2_df_k<<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(Bh, Bl, ldb, rows, k, cnorm);
      QR_CHECK_LAUNCH("col_norms2_df_k");
      QR_CUDA(cudaMemsetAsync(L.mask, 0, sizeof(unsigned) * (size_t)(L.items - L.mask), s));  // mask, flag, count
      QR_CUDA(cudaMemsetAsync(done, 0, sizeof(unsigned) * np, s));
      polish_mask_k<<<ceil_div((long)np * L.mw, TPB), TPB, 0, s>>>(G, k, cnorm, k, k0, tol, smax_d, L.mask, L.mw,
                                                                    L.count);
      QR_CHECK_LAUNCH("polish_mask_k");
      QR_CUDA(cudaMemcpyAsync(hs + nstate, L.count, sizeof(unsigned) * 2, cudaMemcpyDeviceToHost, s));
      QR_CUDA(cudaStreamSynchronize(s));
      marked = hs[nstate];
      float tlin;
      memcpy(&tlin, &hs[nstate + 1], sizeof(float));
      if (marked == 0 || tlin <= kPolishLinTan) {
        if (marked > 0) {
          // first-order simultaneous rotation of the marked pairs (kPolishLinTan)
          svd_path(SP_DF_LINEAR);
          QR_TRY(w->pt.ensure(sizeof(float2) * 2 * ((size_t)rows * k + (size_t)k * k), s));
          float2 *Th = w->pt.as<float2>(), *Tl = Th + (size_t)rows * k;
          float2 *Uh = Tl + (size_t)rows * k, *Ul = Uh + (size_t)k * k;
          polish_lin_k<<<gs((long)k * k), TPB, 0, s>>>(G, cnorm, k, w->ml.as<unsigned>(), np, k0);
          QR_CHECK_LAUNCH("polish_lin_k");
          QR_TRY(zgemm_df(s, DF_F32_AXPY, OP_N, rows, k, k, Bh, nullptr, ldb, G, nullptr, k, Th, Tl, rows, Bh, Bl, ldb,
                          1.f));
          QR_TRY(zgemm_df(s, DF_F32_AXPY, OP_N, k, k, k, Vh, nullptr, ldv, G, nullptr, k, Uh, Ul, k, Vh, Vl, ldv, 1.f));
          const size_t cb = sizeof(float2);
          QR_CUDA(cudaMemcpy2DAsync(Bh, cb * ldb, Th, cb * rows, cb * rows, k, cudaMemcpyDeviceToDevice, s));
          QR_CUDA(cudaMemcpy2DAsync(Bl, cb * ldb, Tl, cb * rows, cb * rows, k, cudaMemcpyDeviceToDevice, s));
          QR_CUDA(cudaMemcpy2DAsync(Vh, cb * ldv, Uh, cb * k, cb * k, k, cudaMemcpyDeviceToDevice, s));
          QR_CUDA(cudaMemcpy2DAsync(Vl, cb * ldv, Ul, cb * k, cb * k, k, cudaMemcpyDeviceToDevice, s));
        }
        if (debug_on())
          fprintf(stderr, "[qr] jacobi<df> %dx%d sweep %d: %u pairs marked, largest first-order tangent %.2e: %s\n",
                  rows, k, sweep, marked, tlin, marked ? "rotated at once" : "converged");
        return QR_OK;
      }
      svd_path(SP_DF_MASKED);
      long listed = 0;
      int classes = 0;
      QR_TRY(upload_schedule(s, w, np, false, &listed, &classes));
      if (debug_on())
        fprintf(stderr, "[qr] jacobi<df> %dx%d sweep %d: %ld pairs listed in %d colour classes\n", rows, k, sweep, listed,
                classes);
      mk = w->ml.as<unsigned>();
    }
    int pr = prof_begin(s, PK_JACOBI_DF, 0.0, 0.0);
    float2 *a1 = Bh, *a2 = Bl, *a3 = Vh, *a4 = Vl;
    long l1 = ldb, l2 = ldv;
    int mm = rows, kk = k, npp = np, sw = sweep;
    double tl = tol;
    const double* sm = smax_d;
    unsigned* st = state;
    unsigned* fl = flags;
    int kz = k0;
    unsigned* dn = done;
    void* args[] = {&a1, &a2, &l1, &mm, &kk, &a3, &a4, &l2, &npp, &tl, &sm, &st, &sw, &fl, &kz, &mk, &dn};
    if (blockdf && !mk) {
      int nbb = nbp;
      void* bargs[] = {&a1, &a2, &l1, &mm, &kk, &a3, &a4, &l2, &nbb, &tl, &sm, &st, &sw, &fl, &kz};
      QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_block_df_k, dim3(dbgrid), dim3(DB_NT), bargs, dbsm, s));
    } else {
      QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_sweep_df_k<NT, RPT>, dim3(grid), dim3(NT), args, vsm, s));
    }
    count_launch();
    prof_end(s, pr);
    QR_CUDA(cudaMemcpyAsync(hs, state, sizeof(unsigned) * nstate, cudaMemcpyDeviceToHost, s));
    if (masked) {
      const MaskedList L = masked_list(w->ml.as<unsigned>(), np);
      QR_CUDA(cudaMemcpyAsync(hs + nstate, L.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    }
    QR_CUDA(cudaStreamSynchronize(s));
    if (hs[4]) return fail(QR_ECUDA, "double-float Jacobi sweep: a column wait timed out");
    marked = masked ? hs[nstate] : 0;
    const unsigned rot = hs[8 + SW_STRIDE * sweep], skipped = hs[11 + SW_STRIDE * sweep];
    float tmax;
    memcpy(&tmax, &hs[9 + SW_STRIDE * sweep], sizeof(float));
    if (debug_on())
      fprintf(stderr, "[qr] jacobi<df> %dx%d sweep %d%s rotations %u max tan %.2e (pairs marked %u, skipped %u)\n",
              rows, k, sweep, masked ? " masked" : "", rot, tmax, marked, skipped);
    account(pr, std::max(0.0, pairs - (double)skipped), rot, 1);
    if (hs[0]) return QR_OK;
    masked = masked || (tmax < kPolishMaskTan && np < 32768);  // list items hold 15-bit columns
  }
  return fail(QR_ENOCONV, "double-float Jacobi polish did not converge");
}

}  // namespace

// ---- masked FP32 block sweeps
// The masked FP32 sweeps turn only pairs whose first-order tangent is at least this: the FP32
// stage is a preconditioner, and its late sweeps exist for the strongly coupled near-degenerate
// clusters (tangents 0.1-1).  The many pairs at the rounding floor (a small column against each
// large one, tangents ~1e-6) would make one column meet hundreds of others in sequence, and the
// double-float polish turns them anyway in its first sweep, which already rotates every pair.
constexpr float kF32TailTan = 1e-3f;
// Block pairs a masked FP32 block sweep processes, from G = B^H B (k x k, ld k, the tcgen05 split
// product: FP32-level accuracy, like the sweep's own inner products).  An element pair p < q
// whose coupling fails rotation_params_f32's test and whose first-order tangent |g| / |a - b| is
// at least min_tan marks the pair of its
// two 4-column blocks or, inside one block, that block (its pairs are met by a `full` block pair
// pairs are met): flag[block] = 1.  count[0] += marked element pairs.
__global__ void f32_block_mask_k(const double2* __restrict__ G, int k, int nbp, float tol, double min_tan,
                                 const double* __restrict__ smax_p, unsigned* ml, unsigned* __restrict__ count) {
  const MaskedList L = masked_list(ml, nbp);
  const double smax = smax_p[0] / smax_p[1];
  const double fl = 4.0 * Eps<float>::v * smax, fl4 = fl * fl * fl * fl;
  const double t2 = (double)tol * tol * smax * smax;
  unsigned c = 0;
  const long tot = (long)k * k;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot; e += (long)gridDim.x * blockDim.x) {
    const int p = (int)(e % k), q = (int)(e / k);
    if (q <= p) continue;
    const double a = G[p + (long)p * k].x, b = G[q + (long)q * k].x;
    if (!(a > 0.0) || !(b > 0.0)) continue;
    const double2 g = G[e];
    const double g2 = g.x * g.x + g.y * g.y;
    const bool hit = tol < 0.f ? sqrt(g2) > (-(double)tol) * sqrt(a) * sqrt(b) : g2 > t2 * fmin(a, b) + fl4;
    if (!hit || sqrt(g2) < min_tan * fabs(b - a)) continue;
    c++;
    const int bp = p / JR_W, bq = q / JR_W;
    if (bp == bq) L.flag[bp] = 1u;
    else atomicOr(L.mask + (long)bp * L.mw + (bq >> 5), 1u << (bq & 31));
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// FP32 block Jacobi sweeps (B rows x k, rows <= JR_MAXROWS, k > 128; V k x k) that examine only
// the block pairs a Gram test marks.  Late in the FP32 stage a sweep rotates a few thousand of
// the 2 million pairs (near-degenerate clusters), yet a full block sweep costs its 511 dependent
// block rounds (~13 ms at 2048 columns) whatever it rotates.  Each masked sweep forms B^H B with
// the tcgen05 split GEMM (~0.5 ms), marks the block pairs with a coupling above half the rotation
// threshold, lists them in round order and runs jacobi_block_reg_k over the list.  Couplings that
// the sweep's own rotations raise above the threshold are marked by the next sweep's Gram test.
// Stops after a sweep whose largest tangent is below tan_stop, or when nothing is marked.
static int jacobi_f32_masked(cudaStream_t s, SvdWork* w, float2* B, int rows, int k, float2* V, int max_sweeps,
                             float tol, float tan_stop) {
  const int nb = (k + JR_W - 1) / JR_W, nbp = nb + (nb & 1);
  const int nstate = 8 + SW_STRIDE * max_sweeps;
  // [state (nstate) | block counters (nbp) | pad | smax, scale (2 doubles)]
  const int soff = nstate + nbp + ((nstate + nbp) & 1);
  QR_TRY(w->cnt.ensure(sizeof(unsigned) * soff + 2 * sizeof(double) + 128, s));
  unsigned* state = w->cnt.as<unsigned>();
  unsigned* done = state + nstate;
  double* smax_d = reinterpret_cast<double*>(state + soff);
  double* nrm = w->nrm.as<double>();
  QR_CUDA(cudaMemsetAsync(state, 0, sizeof(unsigned) * nstate, s));
  col_norms_k<float2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, rows, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  max_reduce_k<<<1, 256, 0, s>>>(nrm, k, smax_d);
  QR_CHECK_LAUNCH("max_reduce_k");
  pow2_scale_k<float2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, smax_d, smax_d + 1, 0);
  QR_CHECK_LAUNCH("pow2_scale_k");
  const size_t wsb = zgemm_tc_workspace(k, k, rows, 1, true);
  QR_TRY(w->tcw.ensure(256 + wsb, s));
  unsigned* err = w->tcw.as<unsigned>();
  void* ws = w->tcw.as<char>() + 256;
  QR_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), s));
  QR_TRY(w->pt.ensure(sizeof(double2) * (size_t)k * k, s));
  double2* G = w->pt.as<double2>();
  QR_TRY(w->ml.ensure(sizeof(unsigned) * masked_list_words(nbp), s));
  unsigned* ml = w->ml.as<unsigned>();
  const MaskedList L = masked_list(ml, nbp);
  int per_sm = 0, sms = 0;
  QR_TRY(device_sm_count(&sms));
  QR_TRY(blocks_per_sm((const void*)jacobi_block_reg_k, JR_NT, 0, &per_sm));
  if (per_sm < 1) return fail(QR_ECUDA, "block Jacobi sweep kernel cannot be resident");
  const int grid = std::max(1, std::min(per_sm * sms, nbp / 2));
  svd_path(SP_BLOCK_MASKED);
  // host: the state, then [-, -, tcgen05 error flag]
  unsigned* hs = static_cast<unsigned*>(host_scratch(sizeof(unsigned) * (nstate + 3)));
  if (!hs) return fail(QR_ENOMEM, "page-locked host scratch");
  int rc = QR_OK;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    QR_TRY(zgemm_tc(s, OP_C, OP_N, k, k, rows, B, rows, 0, B, rows, 0, G, k, 0, 1, ws, err));
    QR_CUDA(cudaMemsetAsync(ml, 0, sizeof(unsigned) * (size_t)(L.items - L.mask), s));  // mask, flag, count
    QR_CUDA(cudaMemsetAsync(done, 0, sizeof(unsigned) * nbp, s));
    f32_block_mask_k<<<gs((long)k * k), TPB, 0, s>>>(G, k, nbp, tol, (double)kF32TailTan, smax_d, ml, L.count);
    QR_CHECK_LAUNCH("f32_block_mask_k");
    long listed = 0;
    int classes = 0;
    QR_TRY(upload_schedule(s, w, nbp, true, &listed, &classes));
    const unsigned markedp = w->hl.as<unsigned>()[L.count - L.mask];
    if (listed == 0) break;
    int pr = prof_begin(s, PK_JACOBI32, 0.0, 0.0);
    {
      float2 *Bp = B, *Vp = V;
      long ldbb = rows, ldvv = k;
      int mm = rows, kk2 = k, nbb = nbp, sw = sweep;
      float tl = tol, ts = tan_stop;
      const double* sm = smax_d;
      unsigned* st = state;
      unsigned* fl = done;  // unused in list mode
      const unsigned* mlp = ml;
      unsigned* dn = done;
      void* args[] = {&Bp, &ldbb, &mm, &kk2, &Vp, &ldvv, &nbb, &tl, &sm, &st, &sw, &fl, &ts, &mlp, &dn};
      QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_block_reg_k, dim3(grid), dim3(JR_NT), args, 0, s));
      count_launch();
    }
    prof_end(s, pr);
    QR_CUDA(cudaMemcpyAsync(hs, state, sizeof(unsigned) * nstate, cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaMemcpyAsync(hs + nstate + 2, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaStreamSynchronize(s));
    if (hs[nstate + 2]) { rc = fail(QR_ECUDA, "tcgen05 Gram matrix: a bounded wait gave up"); break; }
    if (hs[4]) { rc = fail(QR_ECUDA, "masked block Jacobi sweep: a wait timed out"); break; }
    const unsigned rot = hs[8 + SW_STRIDE * sweep];
    float tmax;
    memcpy(&tmax, &hs[9 + SW_STRIDE * sweep], sizeof(float));
    // examined: the listed block pairs' cross pairs (16 each; 28 in round 0)
    prof_account(pr, 16.0 * rows * 16.0 * listed + 40.0 * rot * (rows + k),
                 sizeof(float2) * ((double)rows + k) * 2.0 * (8.0 * listed + rot), 1);
    if (debug_on())
      fprintf(stderr, "[qr] jacobi<f32 masked> %dx%d sweep %d: %u pairs marked, %ld block pairs listed in %d colour "
              "classes, rotations %u, max tan %.2e\n", rows, k, sweep, markedp, listed, classes, rot, tmax);
    if (listed == 0 || rot == 0 || tmax < tan_stop) break;
  }
  pow2_scale_k<float2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, smax_d, smax_d + 1, 1);
  QR_CHECK_LAUNCH("pow2_scale_k");
  return rc;
}

// Re-orthonormalise the m x k column block L in place (Householder QR, phase-preserving).
static int reorthonormalize(cudaStream_t s, SvdWork* w, double2* L, long ldl, int m, int k) {
  svd_path(SP_REORTH);
  QR_TRY(w->qtmp.ensure(sizeof(double2) * ((size_t)m * k + (size_t)k * k), s));
  QR_TRY(w->tau.ensure(sizeof(double2) * (size_t)k, s));
  double2* Rr = w->qtmp.as<double2>() + (size_t)m * k;
  // factor a copy; Q overwrites L
  double2* Acopy = w->qtmp.as<double2>();
  QR_CUDA(cudaMemcpy2DAsync(Acopy, sizeof(double2) * m, L, sizeof(double2) * ldl, sizeof(double2) * m, k,
                            cudaMemcpyDeviceToDevice, s));
  QR_TRY(zqr_thin(s, Acopy, m, k, m, L, ldl, Rr, k, w->tau.as<double2>()));
  phase_fix_k<<<gs((long)m * k), TPB, 0, s>>>(L, ldl, m, k, Rr, k);
  QR_CHECK_LAUNCH("phase_fix_k");
  return QR_OK;
}

// The FP32 preconditioner stops once a sweep's largest rotation is below this tangent: its last
// sweeps only turn near-degenerate pairs that FP32 cannot separate and the double-float polish
// turns again in its first sweep.
constexpr float kPrecondTanStop = 0.15f;
// Smallest block (columns) that takes the mixed path; below it the FP64 cluster Jacobi is as fast.
constexpr int kMixedMinCols = 16;
// QR preconditioning (Drmac and Veselic): B = Q R, then the one-sided Jacobi runs on W = R^H.
// When B's singular values are spread over many decades and its right singular vectors are not
// aligned with its columns (theta of a state with a decaying Schmidt spectrum), Hestenes sweeps on
// B need 30-40+ sweeps; on R^H they need ~10 (measured on a CPU model of these sweeps: 10
// decades at n = 320, 37 -> 10 sweeps; Gaussian, 13 -> 11).  The FP64 path always
// preconditions above kPrecondMinCols columns (the QR costs less than one FP64 sweep).
// The mixed path's cost on such matrices is the double-float polish, not the FP32 stage: the FP32
// test is absolute (tol * sigma_max), so FP32 never rotates pairs of columns far below sigma_max
// and the polish has to diagonalise that block from scratch (22 double-float sweeps at 2048
// columns over 10 decades).  So when the FP32 stage has not converged after kMixedProbeSweeps
// sweeps and more than kSmallColFrac of the columns the polish will touch are below
// kSmallCol * sigma_max, the FP32 stage restarts on R^H with a relative test, which FP32 resolves
// there (the polish then takes 2-3 sweeps).
constexpr int kPrecondMinCols = 32;
constexpr int kMixedProbeSweeps = 11;
constexpr double kSmallCol = 1e-4;
constexpr double kSmallColFrac = 0.1;

// B (rows x k, rows >= k) = Q R with Q in w->Qp (rows x k); B is replaced by W = R^H (k x k, ld k)
static int qr_precondition(cudaStream_t s, SvdWork* w, double2* B, int rows, int k) {
  QR_TRY(w->Qp.ensure(sizeof(double2) * (size_t)rows * k, s));
  QR_TRY(w->qtmp.ensure(sizeof(double2) * (size_t)k * k, s));
  QR_TRY(w->tau.ensure(sizeof(double2) * (size_t)k, s));
  double2* Rr = w->qtmp.as<double2>();
  QR_TRY(zqr_thin(s, B, rows, k, rows, w->Qp.as<double2>(), rows, Rr, k, w->tau.as<double2>()));
  return ztranspose(s, Rr, k, k, k, B, k, 1);
}

int zsvd_thin(cudaStream_t s, SvdWork* w, int mode, const double2* A, int m, int n, long lda,
              double2* U, long ldu, double* S, double2* Vh, long ldvh, int keep) {
  if (m <= 0 || n <= 0) return QR_OK;
  const bool tall = m >= n;
  const int rows0 = tall ? m : n;  // B = A (tall) or A^H (wide): rows0 x k
  const int k = tall ? n : m;
  int rows = rows0;  // rows of the matrix the Jacobi runs on: rows0, or k after QR preconditioning
  bool pre = false;
  QR_TRY(w->B.ensure(sizeof(double2) * (size_t)rows0 * k, s));
  QR_TRY(w->V.ensure(sizeof(double2) * (size_t)k * k, s));
  QR_TRY(w->nrm.ensure(sizeof(double) * (size_t)k * 2, s));
  QR_TRY(w->perm.ensure(sizeof(int) * (size_t)k, s));
  QR_TRY(w->cnt.ensure(sizeof(unsigned) * 8, s));
  double2* B = w->B.as<double2>();
  double2* V = w->V.as<double2>();
  double* nrm = w->nrm.as<double>();
  double* sorted = nrm + k;
  int* perm = w->perm.as<int>();

  // B = A or A^H (FP64 copy; A is preserved)
  if (tall) {
    QR_CUDA(cudaMemcpy2DAsync(B, sizeof(double2) * rows, A, sizeof(double2) * lda, sizeof(double2) * m, n,
                              cudaMemcpyDeviceToDevice, s));
  } else {
    QR_TRY(ztranspose(s, A, lda, m, n, B, rows, 1));
  }

  // The FP32-preconditioned path pays off above a few dozen columns; tiny blocks take the FP64
  // Jacobi directly (same accuracy).
  if (mode == QR_FP64 || k <= kMixedMinCols) {
    if (k > kPrecondMinCols) {
      svd_path(SP_QR_PRECOND_FP64);
      QR_TRY(qr_precondition(s, w, B, rows0, k));
      rows = k;
      pre = true;
    }
    QR_TRY(zset_identity(s, V, k, k, k));
    double tol = sqrt((double)rows) * Eps<double>::v;
    QR_TRY(jacobi<double>(s, w, B, rows, rows, k, V, k, 60, tol));
  } else {
    // ---- FP32 Jacobi preconditioner
    QR_TRY(w->B32.ensure(sizeof(float2) * (size_t)rows * k, s));
    QR_TRY(w->V32.ensure(sizeof(float2) * (size_t)k * k, s));
    float2* B32 = w->B32.as<float2>();
    float2* V32 = w->V32.as<float2>();
    QR_TRY(z2c(s, B, rows, B32, rows, rows, k));
    QR_TRY(cset_identity(s, V32, k, k, k));
    // a preconditioner: 1e-5 relative orthogonality is plenty for the FP64 refinement, and sits
    // above the FP32 rounding floor (~sqrt(m) eps32) so sweeps stop once rotations are noise
    float tol32 = fmaxf(4e-6f, 2.0f * sqrtf((float)rows) * Eps<float>::v);
    int conv32 = 0;
    double frac32 = 0.0;
    QR_TRY(jacobi<float>(s, w, B32, rows, rows, k, V32, k, kMixedProbeSweeps, tol32, false, kPrecondTanStop,
                         &conv32, &frac32));
    // columns the polish rotates: all, or the leading keep + margin (see below)
    const int k0 = keep > 0 && keep < k ? std::min(k, keep + std::max(32, keep / 8)) : k;
    bool slow = false;
    if (!conv32) {
      col_norms_k<float2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B32, rows, rows, k, nrm);
      QR_CHECK_LAUNCH("col_norms_k");
      double* hn = static_cast<double*>(host_scratch(sizeof(double) * k));
      if (!hn) return fail(QR_ENOMEM, "page-locked host scratch");
      QR_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
      QR_CUDA(cudaStreamSynchronize(s));
      std::vector<double> sn(hn, hn + k);
      std::sort(sn.begin(), sn.end(), std::greater<double>());
      int small = 0;
      for (int j = 0; j < k0; j++) small += sn[j] < kSmallCol * sn[0];
      slow = small > kSmallColFrac * k0;
      if (debug_on())
        fprintf(stderr, "[qr] mixed %dx%d: FP32 probe: last sweep rotated %.4f of the pairs; %d of the %d polished "
                "columns below %.0e sigma_max -> %s\n", rows, k, frac32, small, k0, kSmallCol,
                slow ? "QR preconditioning" : "continue");
    }
    if (!conv32 && !slow) {
      if (rows <= JR_MAXROWS && k > 128) {
        QR_TRY(jacobi_f32_masked(s, w, B32, rows, k, V32, 20 - kMixedProbeSweeps, tol32, kPrecondTanStop));
      } else {
        QR_TRY(jacobi<float>(s, w, B32, rows, rows, k, V32, k, 20 - kMixedProbeSweeps, tol32, false,
                             kPrecondTanStop));
      }
    } else if (!conv32) {
      // slow convergence (widely spread spectrum): precondition in FP64 and start over on R^H
      svd_path(SP_QR_PRECOND_MIXED);
      QR_TRY(qr_precondition(s, w, B, rows0, k));
      rows = k;
      pre = true;
      tol32 = fmaxf(4e-6f, 2.0f * sqrtf((float)rows) * Eps<float>::v);
      QR_TRY(z2c(s, B, rows, B32, rows, rows, k));
      QR_TRY(cset_identity(s, V32, k, k, k));
      // relative test: on R^H the small columns are exact to FP32 precision, not rounding noise
      QR_TRY(jacobi<float>(s, w, B32, rows, rows, k, V32, k, 20, -tol32, false, kPrecondTanStop));
    }
    // X = V32 with columns sorted by the FP32 column norms (descending), as a double-float
    // matrix (low parts zero); the Newton-Schulz steps and B = A X run in double-float on the
    // FP32 pipes and B goes straight into the double-float polish
    col_norms_k<float2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B32, rows, rows, k, nrm);
    QR_CHECK_LAUNCH("col_norms_k");
    rank_sort_k<<<ceil_div(k, TPB), TPB, 0, s>>>(nrm, k, perm, nullptr);
    QR_CHECK_LAUNCH("rank_sort_k");
    const size_t kk2 = (size_t)k * k, rk = (size_t)rows * k;
    QR_TRY(w->X.ensure(sizeof(float2) * 2 * kk2, s));   // X (hi, lo)
    QR_TRY(w->Rm.ensure(sizeof(float2) * 2 * kk2, s));  // Newton-Schulz output (hi, lo)
    QR_TRY(w->E.ensure(sizeof(float2) * kk2, s));       // R = I - X^H X (FP32)
    QR_TRY(w->T1.ensure(sizeof(float2) * 2 * rk, s));   // A (hi, lo)
    QR_TRY(w->Bl.ensure(sizeof(float2) * rk, s));       // B low parts (high parts reuse B32)
    float2 *Xh = w->X.as<float2>(), *Xl = Xh + kk2;
    float2 *Yh = w->Rm.as<float2>(), *Yl = Yh + kk2;
    float2* R = w->E.as<float2>();
    float2 *Ah = w->T1.as<float2>(), *Al = Ah + rk;
    float2 *Bh = B32, *Bl = w->Bl.as<float2>();
    gather_cols_f2_k<<<gs((long)k * k), TPB, 0, s>>>(V32, k, k, k, perm, Xh, Xl, k);
    QR_CHECK_LAUNCH("gather_cols_f2_k");
    // X must be unitary to double-float accuracy before it carries the polish rotations: two
    // Newton-Schulz steps X <- X + X (I - X^H X) / 2 square the FP32-level error twice
    // (1e-6 -> 1e-12 -> rounding).  I - X^H X needs the compensated products; X R has |R| << 1,
    // so FP32 products are accurate enough for the correction term.
    for (int it = 0; it < 2; it++) {
      QR_TRY(zgemm_df(s, DF_GRAM, OP_C, k, k, k, Xh, Xl, k, Xh, Xl, k, R, nullptr, k));
      QR_TRY(zgemm_df(s, DF_F32_AXPY, OP_N, k, k, k, Xh, nullptr, k, R, nullptr, k, Yh, Yl, k, Xh, Xl, k, 0.5f));
      std::swap(Xh, Yh);
      std::swap(Xl, Yl);
    }
    // A (B holds A or A^H in FP64) scaled by a power of two so sigma_max ~ 1, then B = A X
    double* smax_d = sorted;  // two scratch doubles; `sorted` is rewritten below
    col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, rows, rows, k, nrm);
    QR_CHECK_LAUNCH("col_norms_k");
    max_reduce_k<<<1, 256, 0, s>>>(nrm, k, smax_d);
    QR_CHECK_LAUNCH("max_reduce_k");
    pow2_scale_k<double2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, smax_d, smax_d + 1, 0);
    QR_CHECK_LAUNCH("pow2_scale_k");
    QR_TRY(z2df(s, B, rows, rows, k, nullptr, Ah, Al, rows));
    QR_TRY(zgemm_df(s, DF_STORE, OP_N, rows, k, k, Ah, Al, rows, Xh, Xl, k, Bh, Bl, rows));
    // Hestenes sweeps on (B, X) in double-float finish the near-degenerate pairs the FP32 sweeps
    // leave and bring the couplings down to the double-float tolerance (inner products carry
    // ~sqrt(rows) 2^-48 relative noise; the tolerance sits 2x above that floor)
    // When only the leading `keep` triplets are used (truncation to maxdim), pairs inside the
    // trailing block need no rotation: the cross pairs still decouple that block from the leading
    // columns, and every tail column's norm stays below the tail's largest sigma, so the final
    // sort separates the two sets.  The margin covers FP32 misordering at the boundary.
    QR_TRY(jacobi_df(s, w, Bh, Bl, rows, rows, k, Xh, Xl, k, 40, 32.0 * sqrt((double)rows) * Eps<double>::v,
                     smax_d, k0));
    QR_TRY(df2z(s, Bh, Bl, rows, rows, k, smax_d + 1, B, rows));
    QR_TRY(df2z(s, Xh, Xl, k, k, k, nullptr, V, k));
  }

  // ---- sigma, ordering, factors
  col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, rows, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  rank_sort_k<<<ceil_div(k, TPB), TPB, 0, s>>>(nrm, k, perm, sorted);
  QR_CHECK_LAUNCH("rank_sort_k");
  QR_CUDA(cudaMemcpyAsync(S, sorted, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
  // decide on re-orthonormalisation from the spectrum
  double* hsg = static_cast<double*>(host_scratch(sizeof(double) * k));
  if (!hsg) return fail(QR_ENOMEM, "page-locked host scratch");
  QR_CUDA(cudaMemcpyAsync(hsg, sorted, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  // columns that truncation may retain must be orthonormal to ~1e-11: B/sigma columns are
  // orthogonal to tol * sigma_max / sigma_j, so re-orthonormalise when sigma_keep < 1e-3 sigma_max
  const int kk = (keep > 0 && keep < k) ? keep : k;
  const double smax = hsg[0], smin = hsg[kk - 1];
  if (!(smax >= 0.0) || !std::isfinite(smax)) return fail(QR_ENOCONV, "non-finite singular values");
  const bool reorth = !(smin > 1e-3 * smax);

  // left factor L (rows x k) = B[:, perm] / sigma ; right factor Rf (k x k) = V[:, perm]
  QR_TRY(w->E.ensure(sizeof(double2) * (size_t)k * k, s));
  double2* Rf = w->E.as<double2>();
  if (pre) {
    // W = R^H = L Sigma Rf^H  =>  B0 = Q R = (Q Rf) Sigma L^H: the left factor of B0 is Q Rf
    // (orthonormal: Householder Q times accumulated rotations) and its right factor is L
    QR_TRY(w->Rm.ensure(sizeof(double2) * (size_t)k * k, s));
    double2* L = w->Rm.as<double2>();
    gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(B, k, k, k, perm, sorted, L, k);
    QR_CHECK_LAUNCH("gather_cols_k");
    if (reorth) QR_TRY(reorthonormalize(s, w, L, k, k, kk));
    gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, Rf, k);
    QR_CHECK_LAUNCH("gather_cols_k");
    const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0);
    if (tall) {  // A = B0: U = Q Rf (m x k), Vh = L^H
      QR_TRY(zgemm(s, OP_N, OP_N, rows0, k, k, one, w->Qp.as<double2>(), rows0, 0, Rf, k, 0, zero, U, ldu, 0, 1,
                   nullptr));
      QR_TRY(ztranspose(s, L, k, k, k, Vh, ldvh, 1));
    } else {  // A = B0^H = L Sigma (Q Rf)^H: U = L (m x m), Vh = (Q Rf)^H (m x n); B is free
      QR_TRY(zgemm(s, OP_N, OP_N, rows0, k, k, one, w->Qp.as<double2>(), rows0, 0, Rf, k, 0, zero, B, rows0, 0, 1,
                   nullptr));
      QR_CUDA(cudaMemcpy2DAsync(U, sizeof(double2) * ldu, L, sizeof(double2) * k, sizeof(double2) * k, k,
                                cudaMemcpyDeviceToDevice, s));
      QR_TRY(ztranspose(s, B, rows0, rows0, k, Vh, ldvh, 1));
    }
    return QR_OK;
  }
  if (tall) {
    gather_cols_k<double2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, perm, sorted, U, ldu);
    QR_CHECK_LAUNCH("gather_cols_k");
    if (reorth) QR_TRY(reorthonormalize(s, w, U, ldu, m, kk));
    gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, Rf, k);
    QR_CHECK_LAUNCH("gather_cols_k");
    QR_TRY(ztranspose(s, Rf, k, k, k, Vh, ldvh, 1));  // Vh = Rf^H (k x n)
  } else {
    // A^H = L Sigma Rf^H  =>  A = Rf Sigma L^H : U = Rf (m x m), Vh = L^H (m x n)
    QR_TRY(w->Rm.ensure(sizeof(double2) * (size_t)rows * k, s));
    double2* L = w->Rm.as<double2>();
    gather_cols_k<double2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, perm, sorted, L, rows);
    QR_CHECK_LAUNCH("gather_cols_k");
    if (reorth) QR_TRY(reorthonormalize(s, w, L, rows, rows, kk));
    gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, U, ldu);
    QR_CHECK_LAUNCH("gather_cols_k");
    QR_TRY(ztranspose(s, L, rows, rows, k, Vh, ldvh, 1));
  }
  return QR_OK;
}


// =================================================================================================
// Allocation-free thin SVD.
//
// Some callers cannot let a library call cudaMalloc: a Julia process whose CUDA.jl pool owns the
// device memory (an allocation behind its back breaks its accounting and can fail under its
// memory pressure), or a serving loop that may only allocate at start-up.  For them,
// qr_svd_noalloc runs the plain FP64 Jacobi SVD on caller-owned device buffers with all scratch
// in the file-scope array below, sized for matrices up to QR_NOALLOC_MAX_ROWS x
// QR_NOALLOC_MAX_K (rows = max(m, n), k = min(m, n)); the array stays reserved on every device
// that loads the library until the process exits.
// =================================================================================================
namespace {
constexpr int NOALLOC_MAX_ROWS = 512;
constexpr int NOALLOC_MAX_K = 256;
constexpr size_t NA_B = (size_t)NOALLOC_MAX_ROWS * NOALLOC_MAX_K;  // B, later the QR copy
constexpr size_t NA_V = (size_t)NOALLOC_MAX_K * NOALLOC_MAX_K;     // V, later the R factor
constexpr size_t NA_L = (size_t)NOALLOC_MAX_ROWS * NOALLOC_MAX_K;  // gathered left/right factor
constexpr size_t NA_BYTES = sizeof(double2) * (NA_B + NA_V + NA_L + NOALLOC_MAX_K) +
                            sizeof(double) * 2 * NOALLOC_MAX_K + sizeof(int) * NOALLOC_MAX_K +
                            sizeof(unsigned) * 8;
constexpr int NA_MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_na_mu;
void* g_na_ptr[NA_MAX_DEVICES] = {nullptr};

// The symbol's device address, looked up once per device with that device current.  In host
// code `g_noalloc_scratch` names a host-side stand-in, not device memory, so kernels must be
// given this address instead.
int noalloc_scratch(void** out) {
  int dev = 0;
  QR_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES) return fail(QR_EINVAL, "qr_svd_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "qr_svd_noalloc: cudaGetSymbolAddress");
    g_na_ptr[dev] = ptr;
  }
  *out = g_na_ptr[dev];
  return QR_OK;
}
}  // namespace

}  // namespace qr

using namespace qr;

extern "C" int qr_svd_noalloc(int m, int n, const double* A, long lda, double* U, long ldu, double* S, double* Vh,
                              long ldvh, void* stream) try {
  if (m <= 0 || n <= 0) return fail(QR_EINVAL, "qr_svd_noalloc: empty matrix");
  if (!A || !U || !S || !Vh) return fail(QR_EINVAL, "qr_svd_noalloc: null buffer");
  const bool tall = m >= n;
  const int rows = tall ? m : n, k = tall ? n : m;
  if (rows > NOALLOC_MAX_ROWS || k > NOALLOC_MAX_K)
    return fail(QR_EINVAL, "qr_svd_noalloc: matrix exceeds the 512 x 256 scratch limit (max(m,n) <= 512, "
                           "min(m,n) <= 256); use the allocating SVD for larger blocks");
  if (lda < m || ldu < m || ldvh < k) return fail(QR_EINVAL, "qr_svd_noalloc: bad leading dimension");
  cudaStream_t s = (cudaStream_t)stream;
  void* base = nullptr;
  QR_TRY(noalloc_scratch(&base));
  double2* B = (double2*)base;
  double2* V = B + NA_B;
  double2* L = V + NA_V;
  double2* tau = L + NA_L;
  double* nrm = (double*)(tau + NOALLOC_MAX_K);
  double* sorted = nrm + NOALLOC_MAX_K;
  int* perm = (int*)(sorted + NOALLOC_MAX_K);
  unsigned* cnt = (unsigned*)(perm + NOALLOC_MAX_K);
  unsigned* bar = cnt + 4;
  const double2* Ad = (const double2*)A;

  // B = A (tall) or A^H (wide): every buffer read below is written first
  if (tall) {
    QR_CUDA(cudaMemcpy2DAsync(B, sizeof(double2) * rows, Ad, sizeof(double2) * lda, sizeof(double2) * m, n,
                              cudaMemcpyDeviceToDevice, s));
  } else {
    QR_TRY(ztranspose(s, Ad, lda, m, n, B, rows, 1));
  }

  // Column norms on the host (a stack array: no allocation).  B is first scaled by the power of
  // two 2^-e that brings its largest entry into [1/2, 1): the rotation test squares column norms
  // and inner products, which would underflow below ~1e-154 or overflow above ~1e154.
  double hn[NOALLOC_MAX_K];
  auto host_max_norm = [&](const double2* X, long ldx, int r, double* out) -> int {
    col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(X, ldx, r, k, nrm);
    QR_CHECK_LAUNCH("col_norms_k");
    QR_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaStreamSynchronize(s));
    double mx = 0.0;
    for (int j = 0; j < k; j++) mx = hn[j] > mx ? hn[j] : mx;
    *out = mx;
    return QR_OK;
  };
  // the exponent comes from the largest |re| or |im| (squares of entries near the ends of the
  // range would under- or overflow); after the scaling every column norm is finite and O(1)
  QR_CUDA(cudaMemsetAsync(nrm, 0, sizeof(double), s));
  max_abs_k<<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, reinterpret_cast<unsigned long long*>(nrm));
  QR_CHECK_LAUNCH("max_abs_k");
  QR_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(double), cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  const double amax = hn[0];
  if (!std::isfinite(amax)) return fail(QR_EINVAL, "qr_svd_noalloc: non-finite entries");
  int e2 = 0;
  if (amax > 0.0) frexp(amax, &e2);
  QR_TRY(zscale_matrix(s, rows, k, make_double2(ldexp(1.0, -e2), 0.0), B, rows, 0, 1));
  double smax = 0.0;
  QR_TRY(host_max_norm(B, rows, rows, &smax));

  // QR preconditioning above 32 columns, as in the allocating FP64 path: B = Q R and the sweeps
  // run on W = R^H (k x k), which converges in ~10 sweeps even when the singular values spread
  // over many decades.  Q goes to L, R to V, W to the head of B.
  const bool pre = k > 32;
  int jr = rows;  // rows of the matrix the sweeps rotate
  if (pre) {
    QR_TRY(zqr_thin_steps(s, B, rows, k, rows, L, rows, V, k, tau));
    QR_TRY(ztranspose(s, V, k, k, k, B, k, 1));
    jr = k;
    QR_TRY(host_max_norm(B, k, k, &smax));
  }
  QR_TRY(zset_identity(s, V, k, k, k));

  constexpr int NT = 256, RPT = 8;
  const int np = k + (k & 1);
  int dev = 0, sms = 0, per_sm = 0;
  QR_CUDA(cudaGetDevice(&dev));
  QR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  QR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_sweep_k<double, NT, RPT>, NT, 0));
  int grid = per_sm * sms;
  if (grid > np / 2) grid = np / 2;
  if (grid < 1) grid = 1;
  double tol = sqrt((double)jr) * Eps<double>::v;
  bool converged = false;
  for (int sweep = 0; sweep < 60 && !converged; sweep++) {
    // counters and the grid barrier start every sweep at zero
    QR_CUDA(cudaMemsetAsync(cnt, 0, 8 * sizeof(unsigned), s));
    double2* Bp = B;
    double2* Vp = V;
    int mm = jr, kk = k, npp = np;
    long ldbb = jr, ldvv = k;
    double tl = tol, sm = smax;
    void* args[] = {&Bp, &ldbb, &mm, &kk, &Vp, &ldvv, &npp, &tl, &sm, &cnt, &bar};
    QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_sweep_k<double, NT, RPT>, dim3(grid), dim3(NT), args, 0, s));
    count_launch();
    unsigned hh[3] = {0, 0, 0};
    QR_CUDA(cudaMemcpyAsync(hh, cnt, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaMemcpyAsync(hh + 2, bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaStreamSynchronize(s));
    if (hh[2]) return fail(QR_ECUDA, "qr_svd_noalloc: grid barrier timed out");
    float tmax;
    memcpy(&tmax, &hh[1], sizeof(float));
    converged = hh[0] == 0 || tmax < 1e-8f;
  }
  if (!converged) return fail(QR_ENOCONV, "qr_svd_noalloc: Jacobi SVD did not converge");

  // sigma of the scaled matrix, sorted; S = sigma 2^e
  col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, jr, jr, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  rank_sort_k<<<ceil_div(k, TPB), TPB, 0, s>>>(nrm, k, perm, sorted);
  QR_CHECK_LAUNCH("rank_sort_k");
  QR_CUDA(cudaMemcpyAsync(hn, sorted, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  if (!(hn[0] >= 0.0) || !std::isfinite(hn[0])) return fail(QR_ENOCONV, "qr_svd_noalloc: non-finite singular values");
  const bool reorth = !(hn[k - 1] > 1e-3 * hn[0]);
  for (int j = 0; j < k; j++) hn[j] = ldexp(hn[j], e2);
  QR_CUDA(cudaMemcpyAsync(S, hn, sizeof(double) * k, cudaMemcpyHostToDevice, s));

  // Re-orthonormalise the k columns of F (ld ldf, r rows) in place through the QR copy at X
  // (ld r), with R in V (free once the right factor has been gathered).
  auto reorthonormalize_noalloc = [&](double2* F, long ldf, int r, double2* X) -> int {
    QR_CUDA(cudaMemcpy2DAsync(X, sizeof(double2) * r, F, sizeof(double2) * ldf, sizeof(double2) * r, k,
                              cudaMemcpyDeviceToDevice, s));
    QR_TRY(zqr_thin_steps(s, X, r, k, r, F, ldf, V, k, tau));
    phase_fix_k<<<gs((long)r * k), TPB, 0, s>>>(F, ldf, r, k, V, k);
    QR_CHECK_LAUNCH("phase_fix_k");
    return QR_OK;
  };
  double2* Ud = (double2*)U;
  double2* Vhd = (double2*)Vh;
  const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0);
  if (pre) {
    // W = Lw Sigma Rf^H with Lw = W[:, perm] / sigma, Rf = V[:, perm]; B0 = Q R = (Q Rf) Sigma Lw^H
    double2* Bk = B + (size_t)k * k;  // second k x k slot of B
    if (tall) {  // A = B0: U = Q Rf, Vh = Lw^H; Rf waits in Vh (k x k) until the GEMM has read it
      gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(B, k, k, k, perm, sorted, Bk, k);
      QR_CHECK_LAUNCH("gather_cols_k");
      gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, Vhd, ldvh);
      QR_CHECK_LAUNCH("gather_cols_k");
      if (reorth) QR_TRY(reorthonormalize_noalloc(Bk, k, k, B));
      QR_TRY(zgemm(s, OP_N, OP_N, rows, k, k, one, L, rows, 0, Vhd, ldvh, 0, zero, Ud, ldu, 0, 1, nullptr));
      QR_TRY(ztranspose(s, Bk, k, k, k, Vhd, ldvh, 1));
    } else {  // A = B0^H = Lw Sigma (Q Rf)^H: U = Lw (m x m), Vh = Rf^H Q^H (m x n)
      gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(B, k, k, k, perm, sorted, Ud, ldu);
      QR_CHECK_LAUNCH("gather_cols_k");
      gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, Bk, k);
      QR_CHECK_LAUNCH("gather_cols_k");
      if (reorth) QR_TRY(reorthonormalize_noalloc(Ud, ldu, k, B));
      QR_TRY(zgemm(s, OP_C, OP_C, k, rows, k, one, Bk, k, 0, L, rows, 0, zero, Vhd, ldvh, 0, 1, nullptr));
    }
  } else {
    // left factor Lf (rows x k) = B[:, perm] / sigma ; right factor (k x k) = V[:, perm]
    double2* Lf = tall ? Ud : L;
    const long ldl = tall ? ldu : rows;
    double2* Rf = tall ? L : Ud;
    const long ldr = tall ? k : ldu;
    gather_cols_k<double2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, perm, sorted, Lf, ldl);
    QR_CHECK_LAUNCH("gather_cols_k");
    gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, Rf, ldr);
    QR_CHECK_LAUNCH("gather_cols_k");
    if (reorth) QR_TRY(reorthonormalize_noalloc(Lf, ldl, rows, B));
    if (tall) {
      QR_TRY(ztranspose(s, Rf, k, k, k, Vhd, ldvh, 1));  // Vh = Rf^H
    } else {
      QR_TRY(ztranspose(s, Lf, ldl, rows, k, Vhd, ldvh, 1));  // Vh = L^H
    }
  }
  QR_CUDA(cudaStreamSynchronize(s));
  return QR_OK;
} QR_ABI_CATCH

namespace qr {
}  // namespace qr

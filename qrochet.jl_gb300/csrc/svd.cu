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
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <cmath>
#include <mutex>
#include "kernels.cuh"
#include "prof.cuh"

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

struct SvdWork {
  DBuf B, V, B32, V32, X, Rm, Sm, E, T1, nrm, perm, cnt, tau, qtmp, host_sig;
  std::vector<double> hs;
  std::vector<unsigned> hc;
  cudaStream_t last = nullptr;
};

SvdWork* svd_work_create() { return new SvdWork(); }
void svd_work_free(SvdWork* w) {
  if (!w) return;
  DBuf* all[] = {&w->B, &w->V, &w->B32, &w->V32, &w->X, &w->Rm, &w->Sm, &w->E, &w->T1,
                 &w->nrm, &w->perm, &w->cnt, &w->tau, &w->qtmp, &w->host_sig};
  for (DBuf* b : all)
    if (b->p) cudaFree(b->p);
  delete w;
}

namespace {

constexpr int TPB = 256;

// QR_DEBUG=1 in the environment prints sweep counts and refinement residuals to stderr
bool debug_on() {
  static int v = -1;
  if (v < 0) v = getenv("QR_DEBUG") ? 1 : 0;
  return v == 1;
}

template <typename T> struct Eps;
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; };
template <> struct Eps<float> { static constexpr float v = 1.1920929e-07f; };

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
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
  // rotate when the coupling exceeds tol * sigma_max * sigma_min(pair): columns end orthogonal to
  // the backward-stable (LAPACK-level) accuracy eps * ||A||, without chasing relative accuracy
  // among columns far below sigma_max
  if (!(a > 0) || !(b > 0) || !(g > tol * smax * sqrt(a < b ? a : b))) return;
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

// Grid-wide barrier for a cooperative launch (all CTAs resident).  The wait is bounded: after
// ~2^22 polls (about a second) the CTA records a timeout in bar[2] and proceeds; every CTA checks
// bar[2] after the barrier and leaves the sweep, so the kernel always returns.
__device__ __forceinline__ bool grid_barrier(unsigned* bar) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vb = bar;
    const unsigned gen = vb[1];
    __threadfence();
    const unsigned arrived = atomicAdd(&bar[0], 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicAdd(&bar[1], 1u);
    } else {
      unsigned polls = 0;
      while (vb[1] == gen) {
        if (++polls > (1u << 22)) {
          atomicExch(&bar[2], 1u);
          break;
        }
        __nanosleep(200);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ((volatile unsigned*)bar)[2] == 0u;
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

__global__ void add_identity_k(double2* A, int n, long lda, double alpha) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[i + (long)i * lda].x += alpha;
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

// Hestenes sweeps on B (rows x k) accumulating V (k x k), until no rotation happens.
template <typename T>
int jacobi(cudaStream_t s, SvdWork* w, cplx_t<T>* B, long ldb, int rows, int k, cplx_t<T>* V,
           long ldv, int max_sweeps, T tol, bool must_converge = true) {
  const int np = k + (k & 1);
  unsigned* cnt = w->cnt.as<unsigned>();
  unsigned* bar = cnt + 4;
  constexpr int NT = sizeof(T) == 8 ? 256 : 128;
  constexpr int RPT = sizeof(T) == 8 ? 8 : 16;
  // persistent cooperative grid: as many CTAs as can be resident, at most one per pair
  int dev = 0, sms = 0, per_sm = 0;
  QR_CUDA(cudaGetDevice(&dev));
  QR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  QR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_sweep_k<T, NT, RPT>, NT, 0));
  if (per_sm < 1) return fail(QR_ECUDA, "Jacobi sweep kernel cannot be resident");
  int grid = per_sm * sms;
  if (grid > np / 2) grid = np / 2;
  if (grid < 1) grid = 1;
  const int kind = sizeof(T) == 8 ? PK_JACOBI64 : PK_JACOBI32;
  const double pairs = 0.5 * (double)k * (k - 1);
  // sigma_max from the largest column norm (the column norms' maximum never exceeds it and is
  // within a factor sqrt(k) of it; the criterion only needs its scale)
  double* nrm = w->nrm.as<double>();
  col_norms_k<cplx_t<T>><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, ldb, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  w->hs.resize(k);
  QR_CUDA(cudaMemcpyAsync(w->hs.data(), nrm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  double smax_h = 0.0;
  for (int j = 0; j < k; j++) smax_h = w->hs[j] > smax_h ? w->hs[j] : smax_h;
  const T smax = (T)smax_h;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    QR_CUDA(cudaMemsetAsync(cnt, 0, 8 * sizeof(unsigned), s));
    int pr = prof_begin(s, kind, 0.0, 0.0);
    {
      cplx_t<T>* Bp = B;
      cplx_t<T>* Vp = V;
      int mm = rows, kk2 = k, npp = np;
      long ldbb = ldb, ldvv = ldv;
      T tl = tol, sm = smax;
      void* args[] = {&Bp, &ldbb, &mm, &kk2, &Vp, &ldvv, &npp, &tl, &sm, &cnt, &bar};
      QR_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_sweep_k<T, NT, RPT>, dim3(grid), dim3(NT), args, 0, s));
      count_launch();
    }
    prof_end(s, pr);
    unsigned hh[3] = {0, 0, 0};
    QR_CUDA(cudaMemcpyAsync(hh, cnt, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaMemcpyAsync(hh + 2, bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaStreamSynchronize(s));
    if (hh[2]) return fail(QR_ECUDA, "Jacobi sweep: grid barrier timed out");
    const unsigned h = hh[0];
    float tmax;
    memcpy(&tmax, &hh[1], sizeof(float));
    // algorithmic work of the sweep: three inner products per pair (16 real flops per row) and
    // two column rotations of B and V for every rotated pair (20 flops per row and column)
    prof_account(pr, 16.0 * rows * pairs + 20.0 * (double)h * (rows + k) * 2.0,
                 sizeof(cplx_t<T>) * ((double)rows + k) * 2.0 * (pairs + h));
    if (debug_on())
      fprintf(stderr, "[qr] jacobi<%s> %dx%d sweep %d rotations %u max tan %.2e\n", sizeof(T) == 8 ? "f64" : "f32",
              rows, k, sweep, h, tmax);
    if (h == 0) return QR_OK;
    // a sweep whose rotations were all below tau leaves couplings O(tau^2): with tau < 1e-8 in
    // FP64 the next sweep would find nothing above the tolerance, so it is skipped
    if (sizeof(T) == 8 && tmax < 1e-8f) return QR_OK;
  }
  if (!must_converge) return QR_OK;
  return fail(QR_ENOCONV, "Jacobi SVD did not converge");
}

}  // namespace

// Re-orthonormalise the m x k column block L in place (Householder QR, phase-preserving).
static int reorthonormalize(cudaStream_t s, SvdWork* w, double2* L, long ldl, int m, int k) {
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

int zsvd_thin(cudaStream_t s, SvdWork* w, int mode, const double2* A, int m, int n, long lda,
              double2* U, long ldu, double* S, double2* Vh, long ldvh, int keep) {
  if (m <= 0 || n <= 0) return QR_OK;
  const bool tall = m >= n;
  const int rows = tall ? m : n;  // B = A (tall) or A^H (wide): rows x k
  const int k = tall ? n : m;
  QR_TRY(w->B.ensure(sizeof(double2) * (size_t)rows * k, s));
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

  if (mode == QR_FP64) {
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
    QR_TRY(jacobi<float>(s, w, B32, rows, rows, k, V32, k, 20, tol32, false));
    // X = V32 sorted by the FP32 column norms (descending), promoted to FP64
    col_norms_k<float2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B32, rows, rows, k, nrm);
    QR_CHECK_LAUNCH("col_norms_k");
    rank_sort_k<<<ceil_div(k, TPB), TPB, 0, s>>>(nrm, k, perm, nullptr);
    QR_CHECK_LAUNCH("rank_sort_k");
    QR_TRY(w->X.ensure(sizeof(double2) * (size_t)k * k, s));
    QR_TRY(w->Rm.ensure(sizeof(double2) * (size_t)k * k, s));
    QR_TRY(w->Sm.ensure(sizeof(double2) * (size_t)k * k, s));
    QR_TRY(w->E.ensure(sizeof(double2) * (size_t)k * k, s));
    double2* X = w->X.as<double2>();
    double2* Rm = w->Rm.as<double2>();
    double2* Sm = w->Sm.as<double2>();
    double2* E = w->E.as<double2>();
    gather_cols_k<float2><<<gs((long)k * k), TPB, 0, s>>>(V32, k, k, k, perm, nullptr, X, k);
    QR_CHECK_LAUNCH("gather_cols_k");
    unsigned long long* off = w->cnt.as<unsigned long long>();
    const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0), mone = make_double2(-1.0, 0.0);
    const double2* Bsrc = B;  // A (tall) or A^H (wide) in FP64, rows x k
    // B is reused below as the product A X, so keep the FP64 source in T1
    QR_TRY(w->T1.ensure(sizeof(double2) * (size_t)rows * k, s));
    double2* Asrc = w->T1.as<double2>();
    QR_CUDA(cudaMemcpyAsync(Asrc, Bsrc, sizeof(double2) * (size_t)rows * k, cudaMemcpyDeviceToDevice, s));
    // X must be unitary to FP64 before it can carry the polish rotations: two Newton-Schulz
    // steps X <- X + X (I - X^H X) / 2 square the FP32-level error twice (1e-5 -> 1e-10 -> 1e-20)
    const double2 half = make_double2(0.5, 0.0);
    for (int it = 0; it < 2; it++) {
      QR_TRY(zgemm(s, OP_C, OP_N, k, k, k, mone, X, k, 0, X, k, 0, zero, Rm, k, 0, 1, nullptr));
      add_identity_k<<<ceil_div(k, TPB), TPB, 0, s>>>(Rm, k, k, 1.0);
      QR_CHECK_LAUNCH("add_identity_k");
      QR_CUDA(cudaMemcpyAsync(V, X, sizeof(double2) * (size_t)k * k, cudaMemcpyDeviceToDevice, s));
      QR_TRY(zgemm(s, OP_N, OP_N, k, k, k, half, V, k, 0, Rm, k, 0, one, X, k, 0, 1, nullptr));
    }
    (void)E;
    (void)Sm;
    // B = A X, then FP64 Hestenes sweeps on (B, X): they finish the near-degenerate pairs the
    // first-order step leaves alone and certify orthogonality with the FP64 tolerance
    QR_TRY(zgemm(s, OP_N, OP_N, rows, k, k, one, Asrc, rows, 0, X, k, 0, zero, B, rows, 0, 1, nullptr));
    QR_CUDA(cudaMemcpyAsync(V, X, sizeof(double2) * (size_t)k * k, cudaMemcpyDeviceToDevice, s));
    QR_TRY(jacobi<double>(s, w, B, rows, rows, k, V, k, 60, sqrt((double)rows) * Eps<double>::v));
  }

  // ---- sigma, ordering, factors
  col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, rows, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  rank_sort_k<<<ceil_div(k, TPB), TPB, 0, s>>>(nrm, k, perm, sorted);
  QR_CHECK_LAUNCH("rank_sort_k");
  QR_CUDA(cudaMemcpyAsync(S, sorted, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
  // decide on re-orthonormalisation from the spectrum
  w->hs.resize(k);
  QR_CUDA(cudaMemcpyAsync(w->hs.data(), sorted, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  // columns that truncation may retain must be orthonormal to ~1e-11: B/sigma columns are
  // orthogonal to tol * sigma_max / sigma_j, so re-orthonormalise when sigma_keep < 1e-3 sigma_max
  const int kk = (keep > 0 && keep < k) ? keep : k;
  const double smax = w->hs[0], smin = w->hs[kk - 1];
  if (!(smax >= 0.0) || !std::isfinite(smax)) return fail(QR_ENOCONV, "non-finite singular values");
  const bool reorth = !(smin > 1e-3 * smax);

  // left factor L (rows x k) = B[:, perm] / sigma ; right factor Rf (k x k) = V[:, perm]
  QR_TRY(w->E.ensure(sizeof(double2) * (size_t)k * k, s));
  double2* Rf = w->E.as<double2>();
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
                              long ldvh, void* stream) {
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

  // B = A (tall) or A^H (wide); V = I: every buffer read below is written first
  if (tall) {
    QR_CUDA(cudaMemcpy2DAsync(B, sizeof(double2) * rows, Ad, sizeof(double2) * lda, sizeof(double2) * m, n,
                              cudaMemcpyDeviceToDevice, s));
  } else {
    QR_TRY(ztranspose(s, Ad, lda, m, n, B, rows, 1));
  }
  QR_TRY(zset_identity(s, V, k, k, k));

  // sigma_max scale for the rotation criterion (host copy into a stack array: no allocation)
  double hn[NOALLOC_MAX_K];
  col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, rows, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  QR_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  double smax = 0.0;
  for (int j = 0; j < k; j++) smax = hn[j] > smax ? hn[j] : smax;

  constexpr int NT = 256, RPT = 8;
  const int np = k + (k & 1);
  int dev = 0, sms = 0, per_sm = 0;
  QR_CUDA(cudaGetDevice(&dev));
  QR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  QR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_sweep_k<double, NT, RPT>, NT, 0));
  int grid = per_sm * sms;
  if (grid > np / 2) grid = np / 2;
  if (grid < 1) grid = 1;
  double tol = sqrt((double)rows) * Eps<double>::v;
  bool converged = false;
  for (int sweep = 0; sweep < 60 && !converged; sweep++) {
    // counters and the grid barrier start every sweep at zero
    QR_CUDA(cudaMemsetAsync(cnt, 0, 8 * sizeof(unsigned), s));
    double2* Bp = B;
    double2* Vp = V;
    int mm = rows, kk = k, npp = np;
    long ldbb = rows, ldvv = k;
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

  col_norms_k<double2><<<ceil_div((long)k * 32, TPB), TPB, 0, s>>>(B, rows, rows, k, nrm);
  QR_CHECK_LAUNCH("col_norms_k");
  rank_sort_k<<<ceil_div(k, TPB), TPB, 0, s>>>(nrm, k, perm, sorted);
  QR_CHECK_LAUNCH("rank_sort_k");
  QR_CUDA(cudaMemcpyAsync(S, sorted, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
  QR_CUDA(cudaMemcpyAsync(hn, sorted, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  if (!(hn[0] >= 0.0) || !std::isfinite(hn[0])) return fail(QR_ENOCONV, "qr_svd_noalloc: non-finite singular values");
  const bool reorth = !(hn[k - 1] > 1e-3 * hn[0]);

  // left factor Lf (rows x k) = B[:, perm] / sigma ; right factor (k x k) = V[:, perm]
  double2* Ud = (double2*)U;
  double2* Lf = tall ? Ud : L;
  const long ldl = tall ? ldu : rows;
  double2* Rf = tall ? L : Ud;
  const long ldr = tall ? k : ldu;
  gather_cols_k<double2><<<gs((long)rows * k), TPB, 0, s>>>(B, rows, rows, k, perm, sorted, Lf, ldl);
  QR_CHECK_LAUNCH("gather_cols_k");
  gather_cols_k<double2><<<gs((long)k * k), TPB, 0, s>>>(V, k, k, k, perm, nullptr, Rf, ldr);
  QR_CHECK_LAUNCH("gather_cols_k");
  if (reorth) {
    // B and V are free now: QR copy in B, R in V
    QR_CUDA(cudaMemcpy2DAsync(B, sizeof(double2) * rows, Lf, sizeof(double2) * ldl, sizeof(double2) * rows, k,
                              cudaMemcpyDeviceToDevice, s));
    QR_TRY(zqr_thin(s, B, rows, k, rows, Lf, ldl, V, k, tau));
    phase_fix_k<<<gs((long)rows * k), TPB, 0, s>>>(Lf, ldl, rows, k, V, k);
    QR_CHECK_LAUNCH("phase_fix_k");
  }
  if (tall) {
    QR_TRY(ztranspose(s, Rf, k, k, k, (double2*)Vh, ldvh, 1));  // Vh = Rf^H
  } else {
    QR_TRY(ztranspose(s, Lf, ldl, rows, k, (double2*)Vh, ldvh, 1));  // Vh = L^H
  }
  QR_CUDA(cudaStreamSynchronize(s));
  return QR_OK;
}

namespace qr {
}  // namespace qr

// Thin complex Householder QR (FP64) for canonize_site!(...; method=:qr) and for
// re-orthonormalising singular-vector blocks.
//
// Reflectors follow the published LAPACK zlarfg/zgeqr2/zung2r conventions (Householder vector
// with unit leading entry stored below the diagonal, beta real on the diagonal, H = I - tau v v^H,
// A <- H^H A during the factorisation, Q = H_0 H_1 ... H_{k-1} [I; 0]), so R has a real diagonal
// like the R that Julia's qr returns.
//
// Two schedules of the same arithmetic:
//  - zqr_thin: the whole factorisation in one cooperative launch.  CTA b owns the columns
//    c = b (mod grid).  At step j every CTA reads column j (final after step j - 1), forms the
//    reflector's scalars itself (the same reduction order in every CTA gives the same bits), and
//    applies H_j^H to its own columns c > j; the owner of column j writes beta and the scaled
//    reflector into it at the start of step j + 1, once no CTA reads it any more.  One bounded grid
//    barrier per step.  Q needs no barrier at all: applying H_{k-1} .. H_0 to a column of [I; 0]
//    touches that column only, so each CTA runs all steps for its own columns in one launch.
//  - zqr_thin_steps: one reflector launch and one trailing-update launch per column (and one
//    Q launch per column), no scratch beyond tau; the allocation-free SVD uses it.
#include "kernels.cuh"
#include "prof.cuh"
#include "grid_sync.cuh"

namespace qr {

namespace {

constexpr int TPB = 256;
constexpr int QR_COOP_NT = 512;  // threads per CTA of the persistent factorisation

__device__ double block_sum_d(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (blockDim.x >> 5)) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[0] = v;
  }
  __syncthreads();
  return red[0];
}

__device__ double2 block_sum_z(double2 v, double* red) {
  double re = block_sum_d(v.x, red);
  double im = block_sum_d(v.y, red);
  return make_double2(re, im);
}

// Householder reflector of x = A[j:m, j] (zlarfg).
__global__ void house_make_k(double2* A, int m, long lda, int j, double2* tau) {
  __shared__ double red[32];
  __shared__ double2 sh_scal;
  __shared__ int sh_skip;
  double2* x = A + j + (long)j * lda;
  const int len = m - j;
  double acc = 0.0;
  for (int t = 1 + threadIdx.x; t < len; t += blockDim.x) acc += x[t].x * x[t].x + x[t].y * x[t].y;
  double xnorm2 = block_sum_d(acc, red);
  if (threadIdx.x == 0) {
    double2 alpha = x[0];
    if (xnorm2 == 0.0 && alpha.y == 0.0) {
      tau[j] = make_double2(0.0, 0.0);
      sh_skip = 1;
    } else {
      double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
      tau[j] = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      double2 den = make_double2(alpha.x - beta, alpha.y);  // scal = 1 / (alpha - beta)
      double dd = den.x * den.x + den.y * den.y;
      sh_scal = make_double2(den.x / dd, -den.y / dd);
      x[0] = make_double2(beta, 0.0);
      sh_skip = 0;
    }
  }
  __syncthreads();
  if (sh_skip) return;
  double2 sc = sh_scal;
  for (int t = 1 + threadIdx.x; t < len; t += blockDim.x) x[t] = cmul(x[t], sc);
}

// A[j:m, c] <- (I - conj(tau_j) v v^H) A[j:m, c] for c in (j, n)   (H^H applied from the left)
__global__ void house_apply_left_k(double2* A, int m, int n, long lda, int j, const double2* tau) {
  __shared__ double red[32];
  const double2 t = tau[j];
  if (t.x == 0.0 && t.y == 0.0) return;
  const double2 tc = make_double2(t.x, -t.y);
  const double2* v = A + j + (long)j * lda;
  const int len = m - j;
  for (int c = j + 1 + blockIdx.x; c < n; c += gridDim.x) {
    double2* col = A + j + (long)c * lda;
    double2 acc = make_double2(0.0, 0.0);
    for (int r = threadIdx.x; r < len; r += blockDim.x) {
      double2 vr = (r == 0) ? make_double2(1.0, 0.0) : v[r];
      acc = cadd(acc, cmulc(vr, col[r]));
    }
    double2 w = cmul(tc, block_sum_z(acc, red));
    for (int r = threadIdx.x; r < len; r += blockDim.x) {
      double2 vr = (r == 0) ? make_double2(1.0, 0.0) : v[r];
      col[r] = csub(col[r], cmul(vr, w));
    }
    __syncthreads();
  }
}

// Q[j:m, c] <- (I - tau_j v v^H) Q[j:m, c] for c in [j, k)   (backward accumulation, zung2r)
__global__ void house_apply_q_k(double2* Q, int m, int k, long ldq, const double2* V, long ldv, int j,
                                const double2* tau) {
  __shared__ double red[32];
  const double2 t = tau[j];
  if (t.x == 0.0 && t.y == 0.0) return;
  const double2* v = V + j + (long)j * ldv;
  const int len = m - j;
  for (int c = j + blockIdx.x; c < k; c += gridDim.x) {
    double2* col = Q + j + (long)c * ldq;
    double2 acc = make_double2(0.0, 0.0);
    for (int r = threadIdx.x; r < len; r += blockDim.x) {
      double2 vr = (r == 0) ? make_double2(1.0, 0.0) : v[r];
      acc = cadd(acc, cmulc(vr, col[r]));
    }
    double2 w = cmul(t, block_sum_z(acc, red));
    for (int r = threadIdx.x; r < len; r += blockDim.x) {
      double2 vr = (r == 0) ? make_double2(1.0, 0.0) : v[r];
      col[r] = csub(col[r], cmul(vr, w));
    }
    __syncthreads();
  }
}

__global__ void extract_r_k(const double2* A, long lda, int k, int n, double2* R, long ldr) {
  long total = (long)k * n;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % k, c = t / k;
    R[i + c * ldr] = (i <= c) ? A[i + c * lda] : make_double2(0.0, 0.0);
  }
}

// zlarfg scalars of x = A[j:m, j] (len = m - j), computed by every CTA alike (the same reduction
// order everywhere gives the same bits): tau = 0 (skip), or beta, tau and
// scal = 1 / (alpha - beta), through shared memory.
struct Reflector {
  double2 tau, scal;
  double beta;
  int skip;
};
__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ void reflector_of(const double2* x, int len, Reflector* out, double* red) {
  double acc = 0.0;
#pragma unroll 4
  for (int t = 1 + threadIdx.x; t < len; t += blockDim.x) acc += x[t].x * x[t].x + x[t].y * x[t].y;
  const double xnorm2 = block_sum_d(acc, red);
  {
    if (threadIdx.x == 0) {
      const double2 alpha = x[0];
      Reflector r;
      if (xnorm2 == 0.0 && alpha.y == 0.0) {
        r.tau = make_double2(0.0, 0.0);
        r.scal = make_double2(0.0, 0.0);
        r.beta = alpha.x;
        r.skip = 1;
      } else {
        const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
        r.tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
        const double2 den = make_double2(alpha.x - beta, alpha.y);
        const double dd = den.x * den.x + den.y * den.y;
        r.scal = make_double2(den.x / dd, -den.y / dd);
        r.beta = beta;
        r.skip = 0;
      }
      *out = r;
    }
  }
  __syncthreads();
}

// the pivot column j after its step: beta on the diagonal, the reflector scaled below it
__device__ void store_reflector(double2* x, int len, const Reflector& r) {
  if (r.skip) return;
  for (int t = 1 + threadIdx.x; t < len; t += blockDim.x) x[t] = cmul(x[t], r.scal);
  if (threadIdx.x == 0) x[0] = make_double2(r.beta, 0.0);
}

// One warp per owned column: col[0:len) -= v (conj(tau) v^H col), v = (1, x[1:] scal)
__global__ void __launch_bounds__(QR_COOP_NT) house_qr_coop_k(double2* A, int m, int n, long lda, double2* tau,
                                                               unsigned* bar) {
  __shared__ Reflector cur;
  __shared__ double red[32];
  Reflector prev;
  prev.skip = 1;
  const int k = m < n ? m : n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int G = (int)gridDim.x, b = (int)blockIdx.x;
  for (int j = 0; j < k; j++) {
    if (j > 0 && (j - 1) % G == b) store_reflector(A + (j - 1) + (long)(j - 1) * lda, m - (j - 1), prev);
    const double2* x = A + j + (long)j * lda;
    const int len = m - j;
    reflector_of(x, len, &cur, red);
    const Reflector r = cur;
    if (j % G == b) {
      if (threadIdx.x == 0) tau[j] = r.tau;
      prev = r;
    }
    if (!r.skip) {
      const double2 tc = make_double2(r.tau.x, -r.tau.y);
      const int c0 = j + 1 + ((b - (j + 1)) % G + G) % G;  // smallest owned column above j
      for (int c = c0 + warp * G; c < n; c += nw * G) {
        double2* col = A + j + (long)c * lda;
        double wr = 0.0, wi = 0.0;
#pragma unroll 8
        for (int t = lane; t < len; t += 32) {
          const double2 v = t == 0 ? make_double2(1.0, 0.0) : cmul(x[t], r.scal);
          const double2 y = col[t];
          wr += v.x * y.x + v.y * y.y;
          wi += v.x * y.y - v.y * y.x;
        }
        const double2 w = cmul(tc, make_double2(warp_sum_d(wr), warp_sum_d(wi)));
#pragma unroll 8
        for (int t = lane; t < len; t += 32) {
          const double2 v = t == 0 ? make_double2(1.0, 0.0) : cmul(x[t], r.scal);
          col[t] = csub(col[t], cmul(v, w));
        }
      }
    }
    if (!grid_barrier(bar)) return;
  }
  if (k > 0 && (k - 1) % G == b) store_reflector(A + (k - 1) + (long)(k - 1) * lda, m - (k - 1), prev);
}

// Q (m x k) = H_0 .. H_{k-1} [I; 0]: one CTA per column c, formed from e_c through H_c, ..., H_0
// (H_j touches rows j.. of the columns c >= j only, so columns need no synchronisation).  The
// longest columns (most reflectors) are dealt first.
__global__ void house_q_cols_k(double2* Q, int m, int k, long ldq, const double2* V, long ldv, const double2* tau) {
  __shared__ double red[32];
  for (int cc = blockIdx.x; cc < k; cc += gridDim.x) {
    const int c = k - 1 - cc;
    double2* col = Q + (long)c * ldq;
    for (int t = threadIdx.x; t < m; t += blockDim.x) col[t] = make_double2(t == c ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int j = c; j >= 0; j--) {
      const double2 tj = tau[j];
      if (tj.x == 0.0 && tj.y == 0.0) continue;
      const double2* v = V + j + (long)j * ldv;
      const int len = m - j;
      double2 acc = make_double2(0.0, 0.0);
#pragma unroll 4
      for (int t = threadIdx.x; t < len; t += blockDim.x) {
        const double2 vr = t == 0 ? make_double2(1.0, 0.0) : v[t];
        acc = cadd(acc, cmulc(vr, col[j + t]));
      }
      const double2 w = cmul(tj, block_sum_z(acc, red));
#pragma unroll 4
      for (int t = threadIdx.x; t < len; t += blockDim.x) {
        const double2 vr = t == 0 ? make_double2(1.0, 0.0) : v[t];
        col[j + t] = csub(col[j + t], cmul(vr, w));
      }
      __syncthreads();
    }
  }
}

inline int cuda_ok_qr(cudaError_t e) { return e == cudaSuccess ? QR_OK : cuda_fail(e, "Householder QR"); }

inline unsigned cols_grid(int ncols) {
  int g = ncols < 1 ? 1 : ncols;
  return (unsigned)(g > 152 * 8 ? 152 * 8 : g);
}

}  // namespace

int zqr_thin_steps(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq, double2* R,
                   long ldr, double2* tau) {
  if (m <= 0 || n <= 0) return QR_OK;
  const int k = m < n ? m : n;
  for (int j = 0; j < k; j++) {
    house_make_k<<<1, TPB, 0, s>>>(A, m, lda, j, tau);
    QR_CHECK_LAUNCH("house_make_k");
    if (j + 1 < n) {
      house_apply_left_k<<<cols_grid(n - j - 1), TPB, 0, s>>>(A, m, n, lda, j, tau);
      QR_CHECK_LAUNCH("house_apply_left_k");
    }
  }
  if (R) {
    long total = (long)k * n;
    unsigned g = (unsigned)((total + TPB - 1) / TPB);
    extract_r_k<<<g > 4864 ? 4864 : g, TPB, 0, s>>>(A, lda, k, n, R, ldr);
    QR_CHECK_LAUNCH("extract_r_k");
  }
  if (Q) {
    QR_TRY(zset_identity(s, Q, m, k, ldq));
    for (int j = k - 1; j >= 0; j--) {
      house_apply_q_k<<<cols_grid(k - j), TPB, 0, s>>>(Q, m, k, ldq, A, lda, j, tau);
      QR_CHECK_LAUNCH("house_apply_q_k");
    }
  }
  return QR_OK;
}

static int zqr_thin_coop(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq, double2* R,
                         long ldr, double2* tau, int sms);

int zqr_thin(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq, double2* R,
             long ldr, double2* tau) {
  if (m <= 0 || n <= 0) return QR_OK;
  int sms = 0, per_sm = 0;
  QR_TRY(device_sm_count(&sms));
  QR_TRY(blocks_per_sm((const void*)house_qr_coop_k, QR_COOP_NT, 0, &per_sm));
  if (per_sm < 1) return zqr_thin_steps(s, A, m, n, lda, Q, ldq, R, ldr, tau);
  // complex flops: factorisation 8 (m n^2 - n^3 / 3), the same again to form Q
  const double fl = 8.0 * ((double)m * n * n - (double)n * n * n / 3.0) * (Q ? 2.0 : 1.0);
  const int pr = prof_begin(s, PK_QR, fl, 16.0 * (double)m * n * (Q ? 3.0 : 2.0));
  const int rc0 = zqr_thin_coop(s, A, m, n, lda, Q, ldq, R, ldr, tau, sms);
  prof_end(s, pr);
  return rc0;
}

// the cooperative factorisation, R and Q of zqr_thin
static int zqr_thin_coop(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq, double2* R,
                         long ldr, double2* tau, int sms) {
  const int k = m < n ? m : n;
  // one 512-thread CTA per SM, one warp per owned column: a step is the reflector (warp 0 of every
  // CTA), the column updates of the CTA's warps in parallel, and the grid barrier
  int grid = std::min(sms, std::max(1, n - 1));
  unsigned* bar = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&bar, 4 * sizeof(unsigned), s);
  if (e != cudaSuccess) return fail(QR_ENOMEM, std::string("QR barrier: ") + cudaGetErrorString(e));
  int rc = cuda_ok_qr(cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), s));
  if (!rc) {
    double2* Ap = A;
    int mm = m, nn = n;
    long ld = lda;
    double2* tp = tau;
    unsigned* bp = bar;
    void* args[] = {&Ap, &mm, &nn, &ld, &tp, &bp};
    rc = cuda_ok_qr(cudaLaunchCooperativeKernel((const void*)house_qr_coop_k, dim3(grid), dim3(QR_COOP_NT), args, 0, s));
    count_launch();
  }
  unsigned hb[3] = {0, 0, 0};
  if (!rc) rc = cuda_ok_qr(cudaMemcpyAsync(hb, bar, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  if (!rc) rc = cuda_ok_qr(cudaStreamSynchronize(s));
  cudaFreeAsync(bar, s);
  if (rc) return rc;
  if (hb[2]) return fail(QR_ECUDA, "Householder QR: a grid barrier timed out");
  if (R) {
    long total = (long)k * n;
    unsigned g = (unsigned)((total + TPB - 1) / TPB);
    extract_r_k<<<g > 4864 ? 4864 : g, TPB, 0, s>>>(A, lda, k, n, R, ldr);
    QR_CHECK_LAUNCH("extract_r_k");
  }
  if (Q) {
    house_q_cols_k<<<cols_grid(k), TPB, 0, s>>>(Q, m, k, ldq, A, lda, tau);
    QR_CHECK_LAUNCH("house_q_cols_k");
  }
  return QR_OK;
}

}  // namespace qr

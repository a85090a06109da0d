// Thin complex Householder QR (FP64) for canonize_site!(...; method=:qr) and for
// re-orthonormalising singular-vector blocks.
//
// Reflectors follow the published LAPACK zlarfg/zgeqr2/zung2r conventions (Householder vector
// with unit leading entry stored below the diagonal, beta real on the diagonal, H = I - tau v v^H,
// A <- H^H A during the factorisation, Q = H_0 H_1 ... H_{k-1} [I; 0]), so R has a real diagonal
// like the R that Julia's qr returns.
//
// Step j needs the updated column j, so the factorisation is one reflector launch plus one
// trailing-update launch per column; each trailing column is owned by one CTA.
#include "kernels.cuh"

namespace qr {

namespace {

constexpr int TPB = 256;

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

inline unsigned cols_grid(int ncols) {
  int g = ncols < 1 ? 1 : ncols;
  return (unsigned)(g > 152 * 8 ? 152 * 8 : g);
}

}  // namespace

int zqr_thin(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq, double2* R,
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

}  // namespace qr

// Complex FP64 GEMM on the FP64 tensor path (mma.sync m8n8k4 f64, "DMMA").
//
// GB300 runs DMMA at ~4.2 TFLOP/s against ~1.0 TFLOP/s for DFMA, so every FP64 contraction of
// the Chain path (bond merge theta = A_l diag(Lambda) A_r, R-merges after QR, SVD refinement
// products, environment steps) goes through this kernel.
//
//   C[b] = alpha * op(A[b]) * diag(dk) * op(B[b]) + beta * C[b]     (b = blockIdx.z)
//   op: N (as stored, column-major), T (transpose), C (conjugate transpose), R (conjugate).
//
// CTA tile 64x64 complex outputs, K-tile 16, 8 warps (2 x 4), warp tile 32x16 = 4x2 m8n8
// tiles, real and imaginary parts in separate accumulators (4 real MMAs per complex MMA).
#include "kernels.cuh"
#include "prof.cuh"

namespace qr {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, LDS = BK + 4;

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

template <int OPA, int OPB>
__global__ void __launch_bounds__(256) zgemm_dmma_kernel(
    int M, int N, int K, double2 alpha, const double2* __restrict__ A, long lda, long sA,
    const double2* __restrict__ B, long ldb, long sB, double2 beta, double2* __restrict__ C,
    long ldc, long sC, const double* __restrict__ dk) {
  __shared__ double As_re[BM * LDS], As_im[BM * LDS], Bs_re[BN * LDS], Bs_im[BN * LDS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  A += blockIdx.z * sA;
  B += blockIdx.z * sB;
  C += blockIdx.z * sC;

  double acc_re[4][2][2], acc_im[4][2][2];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      acc_re[i][j][0] = acc_re[i][j][1] = 0.0;
      acc_im[i][j][0] = acc_im[i][j][1] = 0.0;
    }

  for (int k0 = 0; k0 < K; k0 += BK) {
    // ---- A tile: op(A)[m0:m0+64, k0:k0+16] -> As[m][k]
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int i, k;
      if (OPA == OP_N || OPA == OP_R) { i = tid & 63; k = (tid >> 6) + 4 * j; }
      else { k = tid & 15; i = (tid >> 4) + 16 * j; }
      int gi = m0 + i, gk = k0 + k;
      double2 v = make_double2(0.0, 0.0);
      if (gi < M && gk < K) {
        v = (OPA == OP_N || OPA == OP_R) ? A[gi + (long)gk * lda] : A[gk + (long)gi * lda];
        if (OPA == OP_C || OPA == OP_R) v.y = -v.y;
        if (dk) { double s = dk[gk]; v.x *= s; v.y *= s; }
      }
      As_re[i * LDS + k] = v.x;
      As_im[i * LDS + k] = v.y;
    }
    // ---- B tile: op(B)[k0:k0+16, n0:n0+64] -> Bs[n][k]
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n, k;
      if (OPB == OP_N || OPB == OP_R) { k = tid & 15; n = (tid >> 4) + 16 * j; }
      else { n = tid & 63; k = (tid >> 6) + 4 * j; }
      int gn = n0 + n, gk = k0 + k;
      double2 v = make_double2(0.0, 0.0);
      if (gn < N && gk < K) {
        v = (OPB == OP_N || OPB == OP_R) ? B[gk + (long)gn * ldb] : B[gn + (long)gk * ldb];
        if (OPB == OP_C || OPB == OP_R) v.y = -v.y;
      }
      Bs_re[n * LDS + k] = v.x;
      Bs_im[n * LDS + k] = v.y;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double ar[4], ai[4], nai[4], br[2], bi[2];
#pragma unroll
      for (int mt = 0; mt < 4; mt++) {
        int r = wm * 32 + mt * 8 + (lane >> 2);
        ar[mt] = As_re[r * LDS + kk + (lane & 3)];
        ai[mt] = As_im[r * LDS + kk + (lane & 3)];
        nai[mt] = -ai[mt];
      }
#pragma unroll
      for (int nt = 0; nt < 2; nt++) {
        int c = wn * 16 + nt * 8 + (lane >> 2);
        br[nt] = Bs_re[c * LDS + kk + (lane & 3)];
        bi[nt] = Bs_im[c * LDS + kk + (lane & 3)];
      }
      // Operand order: consecutive MMAs share their A (or B) register so the operand-reuse
      // path feeds them; without reuse the FP64 tensor source path caps DMMA near DFMA rate.
#pragma unroll
      for (int mt = 0; mt < 4; mt++) {
        const int b0 = (mt & 1) ? 1 : 0, b1 = 1 - b0;  // snake over n-tiles
        dmma(acc_re[mt][b0], ar[mt], br[b0]);
        dmma(acc_im[mt][b0], ar[mt], bi[b0]);
        dmma(acc_im[mt][b1], ar[mt], bi[b1]);
        dmma(acc_re[mt][b1], ar[mt], br[b1]);
        dmma(acc_im[mt][b1], ai[mt], br[b1]);
        dmma(acc_im[mt][b0], ai[mt], br[b0]);
        dmma(acc_re[mt][b0], nai[mt], bi[b0]);
        dmma(acc_re[mt][b1], nai[mt], bi[b1]);
      }
    }
    __syncthreads();
  }
  // ---- epilogue: thread holds rows lane/4, cols 2*(lane%4)+{0,1} of each 8x8 tile
  const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
#pragma unroll
  for (int mt = 0; mt < 4; mt++)
#pragma unroll
    for (int nt = 0; nt < 2; nt++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int gi = m0 + wm * 32 + mt * 8 + (lane >> 2);
        int gj = n0 + wn * 16 + nt * 8 + 2 * (lane & 3) + h;
        if (gi < M && gj < N) {
          double2 a = make_double2(acc_re[mt][nt][h], acc_im[mt][nt][h]);
          double2 out = cmul(alpha, a);
          if (use_beta) out = cadd(out, cmul(beta, C[gi + (long)gj * ldc]));
          C[gi + (long)gj * ldc] = out;
        }
      }
}

template <int OPA>
int launch_b(int opB, dim3 grid, cudaStream_t s, int M, int N, int K, double2 alpha,
             const double2* A, long lda, long sA, const double2* B, long ldb, long sB,
             double2 beta, double2* C, long ldc, long sC, const double* dk) {
  switch (opB) {
    case OP_N: zgemm_dmma_kernel<OPA, OP_N><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    case OP_T: zgemm_dmma_kernel<OPA, OP_T><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    case OP_C: zgemm_dmma_kernel<OPA, OP_C><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    case OP_R: zgemm_dmma_kernel<OPA, OP_R><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    default: return fail(QR_EINVAL, "zgemm: bad opB");
  }
  QR_CHECK_LAUNCH("zgemm_dmma_kernel");
  return QR_OK;
}

}  // namespace

int zgemm(cudaStream_t s, int opA, int opB, int M, int N, int K, double2 alpha,
          const double2* A, long lda, long sA, const double2* B, long ldb, long sB,
          double2 beta, double2* C, long ldc, long sC, int batch, const double* dk) {
  if (M <= 0 || N <= 0 || batch <= 0) return QR_OK;
  if (K <= 0) {  // C = beta * C
    return zscale_matrix(s, M, N, beta, C, ldc, sC, batch);
  }
  dim3 grid(ceil_div(N, BN), ceil_div(M, BM), batch);
  const double fl = 8.0 * M * N * (double)K * batch;
  const double by = 16.0 * ((double)M * K + (double)K * N + 2.0 * M * N) * batch;
  int pr = prof_begin(s, PK_ZGEMM, fl, by);
  int rc;
  switch (opA) {
    case OP_N: rc = launch_b<OP_N>(opB, grid, s, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    case OP_T: rc = launch_b<OP_T>(opB, grid, s, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    case OP_C: rc = launch_b<OP_C>(opB, grid, s, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    case OP_R: rc = launch_b<OP_R>(opB, grid, s, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, dk); break;
    default: rc = fail(QR_EINVAL, "zgemm: bad opA");
  }
  prof_end(s, pr);
  return rc;
}

}  // namespace qr

// Split-precision complex GEMM on the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulate):
// the contraction kernel of the mixed-precision environment sweeps.
//
//   C[b] = op(A[b]) * op(B[b])        (assignment; FP64 complex in and out)
//
// Each FP64 operand is rounded to FP32 and split into three BF16 slices x = h + m + l (about 24
// significant bits; Ootomo & Yokota's split-precision tensor-core GEMM uses the same idea with
// TF32/FP16 pairs).  The complex product is real-ified,
//     [Cr; Ci] = [[Ar, -Ai], [Ai, Ar]] [Br; Bi],
// so one real GEMM with doubled M and K covers it, and six slice products
// (hh, hm, mh, hl, mm, lh) are accumulated in FP32.  The result carries ~FP32 accuracy
// (relative error ~sqrt(K) 2^-24), at (BF16 rate)/6 complex-flop throughput.
//
// CTA tile: 64 complex rows (128 real-ified rows) x 64 columns, complex K-tile 16 (real 32);
// 8 warps as 4 (M) x 2 (N), warp tile 32 x 32 = 2 x 4 m16n8 tiles.  Operands are split while
// they are staged into shared memory (row-major A [m][k], B as [n][k], BF16, rows padded to 40
// elements so fragment loads are conflict-free).
#include <cuda_bf16.h>
#include "kernels.cuh"
#include "prof.cuh"

namespace qr {

namespace {

constexpr int SBM = 64, SBN = 64, SBK = 16;  // complex tile sizes
constexpr int RM = 2 * SBM, RK = 2 * SBK;    // real-ified A tile: 128 x 32
constexpr int LDK = RK + 8;                  // padded row length (bf16 elements)

struct Split3 {
  __nv_bfloat16 h, m, l;
};

__device__ __forceinline__ Split3 split3(double x) {
  const float xf = (float)x;
  Split3 s;
  s.h = __float2bfloat16_rn(xf);
  const float r1 = xf - __bfloat162float(s.h);
  s.m = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(s.m);
  s.l = __float2bfloat16_rn(r2);
  return s;
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int OPA, int OPB>
__global__ void __launch_bounds__(256) zgemm_split_kernel(int M, int N, int K, const double2* __restrict__ A,
                                                          long lda, long sA, const double2* __restrict__ B,
                                                          long ldb, long sB, double2* __restrict__ C, long ldc,
                                                          long sC) {
  // slices: [0] = h, [1] = m, [2] = l
  __shared__ __align__(16) __nv_bfloat16 As[3][RM * LDK];
  __shared__ __align__(16) __nv_bfloat16 Bs[3][SBN * LDK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;  // 4 x 2 warps
  const int m0 = blockIdx.y * SBM, n0 = blockIdx.x * SBN;
  A += blockIdx.z * sA;
  B += blockIdx.z * sB;
  C += blockIdx.z * sC;

  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;

  for (int k0 = 0; k0 < K; k0 += SBK) {
    // ---- stage op(A)[m0:m0+64, k0:k0+16] as the real-ified 128 x 32 block, split in 3
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int i, k;
      if (OPA == OP_N || OPA == OP_R) { i = tid & 63; k = (tid >> 6) + 4 * j; }
      else { k = tid & 15; i = (tid >> 4) + 16 * j; }
      const int gi = m0 + i, gk = k0 + k;
      double2 v = make_double2(0.0, 0.0);
      if (gi < M && gk < K) {
        v = (OPA == OP_N || OPA == OP_R) ? A[gi + (long)gk * lda] : A[gk + (long)gi * lda];
        if (OPA == OP_C || OPA == OP_R) v.y = -v.y;
      }
      const Split3 re = split3(v.x), im = split3(v.y), nim = split3(-v.y);
      // rows i (real part of C) and 64 + i (imaginary part): [Ar, -Ai] and [Ai, Ar]
      As[0][i * LDK + k] = re.h; As[1][i * LDK + k] = re.m; As[2][i * LDK + k] = re.l;
      As[0][i * LDK + SBK + k] = nim.h; As[1][i * LDK + SBK + k] = nim.m; As[2][i * LDK + SBK + k] = nim.l;
      As[0][(SBM + i) * LDK + k] = im.h; As[1][(SBM + i) * LDK + k] = im.m; As[2][(SBM + i) * LDK + k] = im.l;
      As[0][(SBM + i) * LDK + SBK + k] = re.h;
      As[1][(SBM + i) * LDK + SBK + k] = re.m;
      As[2][(SBM + i) * LDK + SBK + k] = re.l;
    }
    // ---- stage op(B)[k0:k0+16, n0:n0+64] as [Br; Bi] (32 x 64), stored [n][k]
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n, k;
      if (OPB == OP_N || OPB == OP_R) { k = tid & 15; n = (tid >> 4) + 16 * j; }
      else { n = tid & 63; k = (tid >> 6) + 4 * j; }
      const int gn = n0 + n, gk = k0 + k;
      double2 v = make_double2(0.0, 0.0);
      if (gn < N && gk < K) {
        v = (OPB == OP_N || OPB == OP_R) ? B[gk + (long)gn * ldb] : B[gn + (long)gk * ldb];
        if (OPB == OP_C || OPB == OP_R) v.y = -v.y;
      }
      const Split3 re = split3(v.x), im = split3(v.y);
      Bs[0][n * LDK + k] = re.h; Bs[1][n * LDK + k] = re.m; Bs[2][n * LDK + k] = re.l;
      Bs[0][n * LDK + SBK + k] = im.h; Bs[1][n * LDK + SBK + k] = im.m; Bs[2][n * LDK + SBK + k] = im.l;
    }
    __syncthreads();
    // Tensor cores accumulate with truncation; chaining many MMAs into one running sum lets
    // that bias grow with K.  Each k-tile therefore accumulates into fresh fragments (the large
    // hh term and the five correction terms apart) that are then added to the running sum with
    // round-to-nearest FP32 adds.
    float tmain[2][4][4], tcorr[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) tmain[i][j][q] = tcorr[i][j][q] = 0.f;
#pragma unroll
    for (int kk = 0; kk < RK; kk += 16) {
      unsigned af[3][2][4], bfr[3][4][2];
#pragma unroll
      for (int s = 0; s < 3; s++) {
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
          const int r = wm * 32 + mt * 16 + (lane >> 2);
          const int c = kk + 2 * (lane & 3);
          af[s][mt][0] = *reinterpret_cast<const unsigned*>(&As[s][r * LDK + c]);
          af[s][mt][1] = *reinterpret_cast<const unsigned*>(&As[s][(r + 8) * LDK + c]);
          af[s][mt][2] = *reinterpret_cast<const unsigned*>(&As[s][r * LDK + c + 8]);
          af[s][mt][3] = *reinterpret_cast<const unsigned*>(&As[s][(r + 8) * LDK + c + 8]);
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
          const int n = wn * 32 + nt * 8 + (lane >> 2);
          const int c = kk + 2 * (lane & 3);
          bfr[s][nt][0] = *reinterpret_cast<const unsigned*>(&Bs[s][n * LDK + c]);
          bfr[s][nt][1] = *reinterpret_cast<const unsigned*>(&Bs[s][n * LDK + c + 8]);
        }
      }
#pragma unroll
      for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
          mma_bf16(tcorr[mt][nt], af[2][mt], bfr[0][nt]);
          mma_bf16(tcorr[mt][nt], af[1][mt], bfr[1][nt]);
          mma_bf16(tcorr[mt][nt], af[0][mt], bfr[2][nt]);
          mma_bf16(tcorr[mt][nt], af[1][mt], bfr[0][nt]);
          mma_bf16(tcorr[mt][nt], af[0][mt], bfr[1][nt]);
          mma_bf16(tmain[mt][nt], af[0][mt], bfr[0][nt]);
        }
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[i][j][q] += tmain[i][j][q] + tcorr[i][j][q];
    __syncthreads();
  }
  // ---- epilogue: real-ified rows r < 64 are Re(C), r >= 64 are Im(C); write each component
  double* Cd = reinterpret_cast<double*>(C);
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int r = wm * 32 + mt * 16 + (lane >> 2) + ((q & 2) ? 8 : 0);
        const int col = wn * 32 + nt * 8 + 2 * (lane & 3) + (q & 1);
        const int part = r >= SBM;
        const int gi = m0 + (r - part * SBM), gj = n0 + col;
        if (gi < M && gj < N) Cd[2 * (gi + (long)gj * ldc) + part] = (double)acc[mt][nt][q];
      }
}

template <int OPA>
int launch_split_b(int opB, dim3 grid, cudaStream_t s, int M, int N, int K, const double2* A, long lda, long sA,
                   const double2* B, long ldb, long sB, double2* C, long ldc, long sC) {
  switch (opB) {
    case OP_N: zgemm_split_kernel<OPA, OP_N><<<grid, 256, 0, s>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    case OP_T: zgemm_split_kernel<OPA, OP_T><<<grid, 256, 0, s>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    case OP_C: zgemm_split_kernel<OPA, OP_C><<<grid, 256, 0, s>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    case OP_R: zgemm_split_kernel<OPA, OP_R><<<grid, 256, 0, s>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    default: return fail(QR_EINVAL, "zgemm_split: bad opB");
  }
  QR_CHECK_LAUNCH("zgemm_split_kernel");
  return QR_OK;
}

}  // namespace

int zgemm_split(cudaStream_t s, int opA, int opB, int M, int N, int K, const double2* A, long lda, long sA,
                const double2* B, long ldb, long sB, double2* C, long ldc, long sC, int batch) {
  if (M <= 0 || N <= 0 || batch <= 0) return QR_OK;
  if (K <= 0) return zscale_matrix(s, M, N, make_double2(0.0, 0.0), C, ldc, sC, batch);
  dim3 grid(ceil_div(N, SBN), ceil_div(M, SBM), batch);
  const double fl = 8.0 * M * N * (double)K * batch;  // complex-equivalent flops
  const double by = 16.0 * ((double)M * K + (double)K * N + (double)M * N) * batch;
  int pr = prof_begin(s, PK_ZGEMM_SPLIT, fl, by);
  int rc;
  switch (opA) {
    case OP_N: rc = launch_split_b<OP_N>(opB, grid, s, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    case OP_T: rc = launch_split_b<OP_T>(opB, grid, s, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    case OP_C: rc = launch_split_b<OP_C>(opB, grid, s, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    case OP_R: rc = launch_split_b<OP_R>(opB, grid, s, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC); break;
    default: rc = fail(QR_EINVAL, "zgemm_split: bad opA");
  }
  prof_end(s, pr);
  return rc;
}

}  // namespace qr

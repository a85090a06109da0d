// Complex GEMM in double-float arithmetic on the FP32 pipes.
//
// On this part FP64 runs at ~1.1 TFLOP/s (DMMA and DFMA alike) against ~75 TFLOP/s for FFMA, so a
// product carried as hi + lo FP32 pairs with compensated (Dot2) accumulation reaches ~2^-48
// relative accuracy at several times the FP64 rate.  The mixed SVD uses it for the
// Newton-Schulz orthonormalisation of the FP32 Jacobi rotations and for B = A X, whose result
// feeds the double-float Jacobi polish without an FP64 round trip.
//
// Operands are column-major split arrays: the high parts (float2 complex) and the low parts
// (float2 complex) of each matrix, with the same leading dimension.  Modes:
//   DF_STORE   C = op(A) B                       (double-float result, Ch/Cl)
//   DF_I_MINUS C = I - op(A) B                   (FP32 complex result in Ch; used for I - X^H X)
//   F32_AXPY   C = D + alpha op(A_hi) B_hi       (FP32 products and accumulation, double-float
//                                                 addition to D; used for X + X R / 2, |R| << 1)
//   DF_GRAM    C = I - A^H A                     (as DF_I_MINUS for the Hermitian Gram matrix:
//                                                 only tiles on or above the diagonal are
//                                                 computed, each off-diagonal tile is stored twice)
// Tiling: a CTA of 256 threads owns a 64 x 64 block of C, each thread a 4 x 4 sub-block (rows
// tx + 16 i, columns ty + 16 j); K advances in steps of 16 through double-buffered shared
// memory filled by cp.async (8-byte copies, zero-filled outside the matrix).
// Split K: when C has too few tiles to occupy the GPU (the small blocks of a gate at chi <= 128),
// blockIdx.z takes a K-chunk, each CTA writes its unrounded double-float partial sums, and a second
// kernel adds the chunks in double-float and applies the mode's epilogue.
#include "kernels.cuh"
#include "df.cuh"
#include "prof.cuh"

namespace qr {
namespace {

constexpr int DBM = 64, DBN = 64, DBK = 16, DNT = 256, TPB = 256;
constexpr int DLD = DBM + 1;  // padded row: the transposing cp.async writes hit distinct banks

struct DfSmem {
  float2 ah[2][DBK][DLD], al[2][DBK][DLD];
  float2 bh[2][DBK][DLD], bl[2][DBK][DLD];
};

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 8 : 0;  // src-size 0: the 8 destination bytes are zero-filled
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issue the copies of K-tile k0 into stage st.  A is M x K after op (OP_N: A[r + c lda];
// OP_C / OP_T: A[c + r lda]); B is K x N, OP_N.  Low parts are skipped when LO is false.
template <int OPA, bool LO>
__device__ __forceinline__ void load_tile(DfSmem& sm, int st, int M, int N, int K, int m0, int n0, int k0,
                                          const float2* Ah, const float2* Al, long lda, const float2* Bh,
                                          const float2* Bl, long ldb) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    int r, c;
    if (OPA == OP_N) { r = tid & 63; c = (tid >> 6) + 4 * q; }
    else { c = tid & 15; r = (tid >> 4) + 16 * q; }
    const int gr = m0 + r, gc = k0 + c;
    const bool ok = gr < M && gc < K;
    const long off = ok ? (OPA == OP_N ? (long)gr + (long)gc * lda : (long)gc + (long)gr * lda) : 0;
    cp_async8(&sm.ah[st][c][r], Ah + off, ok);
    if (LO) cp_async8(&sm.al[st][c][r], Al + off, ok);
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int r = tid & 15, c = (tid >> 4) + 16 * q;  // r along K, c along N
    const int gk = k0 + r, gn = n0 + c;
    const bool ok = gk < K && gn < N;
    const long off = ok ? (long)gk + (long)gn * ldb : 0;
    cp_async8(&sm.bh[st][r][c], Bh + off, ok);
    if (LO) cp_async8(&sm.bl[st][r][c], Bl + off, ok);
  }
}

// The mode's output for element (row, col) from its double-float sums
template <int MODE>
__device__ __forceinline__ void df_epilogue(int row, int col, bool mirror, DotAcc re, DotAcc im, float2* Ch,
                                            float2* Cl, long ldc, const float2* Dh, const float2* Dl, long ldd,
                                            float alpha) {
  const long o = (long)row + (long)col * ldc;
  if (MODE == DF_STORE) {
    const dfl r = dot_final(re), m = dot_final(im);
    Ch[o] = make_float2(r.h, m.h);
    Cl[o] = make_float2(r.l, m.l);
  } else if (MODE == DF_I_MINUS || MODE == DF_GRAM) {
    const dfl r = df_add({row == col ? 1.f : 0.f, 0.f}, df_neg(dot_final(re)));
    const dfl m = df_neg(dot_final(im));
    Ch[o] = make_float2(r.h + r.l, m.h + m.l);
    if (MODE == DF_GRAM && mirror) Ch[(long)col + (long)row * ldc] = make_float2(r.h + r.l, -(m.h + m.l));
  } else {
    const long od = (long)row + (long)col * ldd;
    const float2 dh = Dh[od], dl = Dl[od];
    const dfl r = df_add_f({dh.x, dl.x}, alpha * re.s);
    const dfl m = df_add_f({dh.y, dl.y}, alpha * im.s);
    Ch[o] = make_float2(r.h, m.h);
    Cl[o] = make_float2(r.l, m.l);
  }
}

template <int OPA, int MODE>
__global__ void __launch_bounds__(DNT, 2)
    zgemm_df_k(int M, int N, int K, const float2* __restrict__ Ah, const float2* __restrict__ Al, long lda,
               const float2* __restrict__ Bh, const float2* __restrict__ Bl, long ldb, float2* __restrict__ Ch,
               float2* __restrict__ Cl, long ldc, const float2* __restrict__ Dh, const float2* __restrict__ Dl,
               long ldd, float alpha, int kc, float4* __restrict__ P) {
  constexpr bool LO = MODE != DF_F32_AXPY;
  constexpr float CJ = OPA == OP_C ? -1.f : 1.f;  // conjugation of A's imaginary part
  extern __shared__ __align__(16) unsigned char smraw[];
  DfSmem& sm = *reinterpret_cast<DfSmem*>(smraw);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  int bx = blockIdx.x, by = blockIdx.y;
  if (MODE == DF_GRAM) {  // linear index over the tiles with bx <= by
    const int t = blockIdx.x;
    by = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while (by * (by + 1) / 2 > t) by--;
    while ((by + 1) * (by + 2) / 2 <= t) by++;
    bx = t - by * (by + 1) / 2;
  }
  const int m0 = bx * DBM, n0 = by * DBN;
  DotAcc re[4][4], im[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) re[i][j] = im[i][j] = DotAcc{0.f, 0.f};

  // K-chunk of this CTA: [kb, ke) (the whole K without split)
  const int kb = P ? (int)blockIdx.z * kc : 0;
  const int ke = P ? min(K, kb + kc) : K;
  const int nk = (ke - kb + DBK - 1) / DBK;
  load_tile<OPA, LO>(sm, 0, M, N, ke, m0, n0, kb, Ah, Al, lda, Bh, Bl, ldb);
  cp_async_commit();
  for (int t = 0; t < nk; t++) {
    const int st = t & 1;
    if (t + 1 < nk) {
      load_tile<OPA, LO>(sm, st ^ 1, M, N, ke, m0, n0, kb + (t + 1) * DBK, Ah, Al, lda, Bh, Bl, ldb);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < DBK; kk++) {
      float2 ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        ah[i] = sm.ah[st][kk][tx + 16 * i];
        ah[i].y *= CJ;
        if (LO) { al[i] = sm.al[st][kk][tx + 16 * i]; al[i].y *= CJ; }
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        bh[j] = sm.bh[st][kk][ty + 16 * j];
        if (LO) bl[j] = sm.bl[st][kk][ty + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (LO) {
            dot2_step(re[i][j], ah[i].x, al[i].x, bh[j].x, bl[j].x);
            dot2_step(re[i][j], -ah[i].y, -al[i].y, bh[j].y, bl[j].y);
            dot2_step(im[i][j], ah[i].x, al[i].x, bh[j].y, bl[j].y);
            dot2_step(im[i][j], ah[i].y, al[i].y, bh[j].x, bl[j].x);
          } else {
            re[i][j].s = fmaf(ah[i].x, bh[j].x, re[i][j].s);
            re[i][j].s = fmaf(-ah[i].y, bh[j].y, re[i][j].s);
            im[i][j].s = fmaf(ah[i].x, bh[j].y, im[i][j].s);
            im[i][j].s = fmaf(ah[i].y, bh[j].x, im[i][j].s);
          }
        }
      if (LO) {
        // renormalise every K step: the correction term otherwise collects TwoSum errors of size
        // u |s| and its own rounding grows the error to ~n u^2 |s| instead of ~sqrt(n) u^2 |s|
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const dfl r = df_fast_two_sum(re[i][j].s, re[i][j].lo), m = df_fast_two_sum(im[i][j].s, im[i][j].lo);
            re[i][j] = DotAcc{r.h, r.l};
            im[i][j] = DotAcc{m.h, m.l};
          }
      }
    }
    __syncthreads();  // stage st is refilled by the next iteration's copies
  }

#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int row = m0 + tx + 16 * i;
    if (row >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int col = n0 + ty + 16 * j;
      if (col >= N) continue;
      if (P) {  // partial sums of this K-chunk, unrounded
        P[((long)blockIdx.z * N + col) * M + row] = make_float4(re[i][j].s, re[i][j].lo, im[i][j].s, im[i][j].lo);
      } else {
        df_epilogue<MODE>(row, col, bx != by, re[i][j], im[i][j], Ch, Cl, ldc, Dh, Dl, ldd, alpha);
      }
    }
  }
}

// Sum of the nz K-chunk partials of element (row, col) in double-float, then the mode's epilogue.
// DF_GRAM: only elements of tiles on or above the diagonal were computed; they are mirrored.
template <int MODE>
__global__ void zgemm_df_reduce_k(int M, int N, int nz, const float4* __restrict__ P, float2* __restrict__ Ch,
                                  float2* __restrict__ Cl, long ldc, const float2* __restrict__ Dh,
                                  const float2* __restrict__ Dl, long ldd, float alpha) {
  const long total = (long)M * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int row = (int)(t % M), col = (int)(t / M);
    const int tr = row / DBM, tc = col / DBN;
    if (MODE == DF_GRAM && tr > tc) continue;
    dfl r{0.f, 0.f}, m{0.f, 0.f};
    for (int z = 0; z < nz; z++) {
      const float4 v = P[((long)z * N + col) * M + row];
      r = df_add(r, df_fast_two_sum(v.x, v.y));
      m = df_add(m, df_fast_two_sum(v.z, v.w));
    }
    df_epilogue<MODE>(row, col, tr != tc, DotAcc{r.h, r.l}, DotAcc{m.h, m.l}, Ch, Cl, ldc, Dh, Dl, ldd, alpha);
  }
}

template <int OPA, int MODE>
int launch_df(cudaStream_t s, int M, int N, int K, const float2* Ah, const float2* Al, long lda, const float2* Bh,
              const float2* Bl, long ldb, float2* Ch, float2* Cl, long ldc, const float2* Dh, const float2* Dl,
              long ldd, float alpha) {
  const int bytes = (int)sizeof(DfSmem);
  QR_TRY(set_func_attr_once((const void*)zgemm_df_k<OPA, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  dim3 grid((M + DBM - 1) / DBM, (N + DBN - 1) / DBN);
  if (MODE == DF_GRAM) {
    const int tiles = (M + DBM - 1) / DBM;
    grid = dim3(tiles * (tiles + 1) / 2, 1);
  }
  // split K until the grid covers the SMs about once (chunks of at least one K step)
  int sms = 0;
  QR_TRY(device_sm_count(&sms));
  const int tiles = (int)(grid.x * grid.y), ksteps = (K + DBK - 1) / DBK;
  int nz = std::min(ksteps, std::max(1, sms / tiles));
  const int kc = ((ksteps + nz - 1) / nz) * DBK;
  nz = (K + kc - 1) / kc;
  if (nz < 2) {
    zgemm_df_k<OPA, MODE><<<grid, DNT, bytes, s>>>(M, N, K, Ah, Al, lda, Bh, Bl, ldb, Ch, Cl, ldc, Dh, Dl, ldd,
                                                   alpha, K, nullptr);
    QR_CHECK_LAUNCH("zgemm_df_k");
    return QR_OK;
  }
  float4* P = nullptr;
  QR_CUDA(cudaMallocAsync(&P, sizeof(float4) * (size_t)nz * M * N, s));
  grid.z = nz;
  zgemm_df_k<OPA, MODE><<<grid, DNT, bytes, s>>>(M, N, K, Ah, Al, lda, Bh, Bl, ldb, Ch, Cl, ldc, Dh, Dl, ldd,
                                                 alpha, kc, P);
  int rc = cudaGetLastError() == cudaSuccess ? QR_OK : fail(QR_ECUDA, "zgemm_df_k launch");
  count_launch();
  if (!rc) {
    const long total = (long)M * N;
    const unsigned g = (unsigned)std::min<long>((total + TPB - 1) / TPB, 4864);
    zgemm_df_reduce_k<MODE><<<g, TPB, 0, s>>>(M, N, nz, P, Ch, Cl, ldc, Dh, Dl, ldd, alpha);
    rc = cudaGetLastError() == cudaSuccess ? QR_OK : fail(QR_ECUDA, "zgemm_df_reduce_k launch");
    count_launch();
  }
  cudaFreeAsync(P, s);
  return rc;
}

__global__ void to_df_scaled_k(const double2* __restrict__ src, long lds, int rows, int cols,
                               const double* __restrict__ scale, float2* __restrict__ hi, float2* __restrict__ lo,
                               long ldd) {
  const double f = scale ? 1.0 / scale[0] : 1.0;
  const long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long i = t % rows, j = t / rows;
    const double2 v = src[i + j * lds];
    const dfl re = df_from(v.x * f), im = df_from(v.y * f);
    hi[i + j * ldd] = make_float2(re.h, im.h);
    lo[i + j * ldd] = make_float2(re.l, im.l);
  }
}

// hi/lo of src[:, j] * colscale[j] (the Lambda of a bond folded into a site's columns)
__global__ void to_df_cols_k(const double2* __restrict__ src, long lds, int rows, int cols,
                             const double* __restrict__ colscale, float2* __restrict__ hi, float2* __restrict__ lo,
                             long ldd) {
  const long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long i = t % rows, j = t / rows;
    const double f = colscale ? colscale[j] : 1.0;
    const double2 v = src[i + j * lds];
    const dfl re = df_from(v.x * f), im = df_from(v.y * f);
    hi[i + j * ldd] = make_float2(re.h, im.h);
    lo[i + j * ldd] = make_float2(re.l, im.l);
  }
}

__global__ void from_df_scaled_k(const float2* __restrict__ hi, const float2* __restrict__ lo, long lds, int rows,
                                 int cols, const double* __restrict__ scale, double2* __restrict__ dst, long ldd) {
  const double f = scale ? scale[0] : 1.0;
  const long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long i = t % rows, j = t / rows;
    const float2 h = hi[i + j * lds], l = lo[i + j * lds];
    dst[i + j * ldd] = make_double2(((double)h.x + (double)l.x) * f, ((double)h.y + (double)l.y) * f);
  }
}

unsigned grid_for(long total) {
  long g = (total + TPB - 1) / TPB;
  return (unsigned)(g > 4864 ? 4864 : (g < 1 ? 1 : g));
}

}  // namespace

int zgemm_df(cudaStream_t s, int mode, int opA, int M, int N, int K, const float2* Ah, const float2* Al, long lda,
             const float2* Bh, const float2* Bl, long ldb, float2* Ch, float2* Cl, long ldc, const float2* Dh,
             const float2* Dl, long ldd, float alpha) {
  if (M <= 0 || N <= 0) return QR_OK;
  if (K < 0) return fail(QR_EINVAL, "zgemm_df: negative K");
  if (opA != OP_N && opA != OP_C && opA != OP_T) return fail(QR_EINVAL, "zgemm_df: op(A) must be N, T or C");
  if (mode == DF_F32_AXPY && (!Dh || !Dl)) return fail(QR_EINVAL, "zgemm_df: AXPY mode needs D");
  if (mode != DF_F32_AXPY && !Al) return fail(QR_EINVAL, "zgemm_df: double-float mode needs low parts");
  if (mode == DF_GRAM && (opA != OP_C || M != N || Ah != Bh || Al != Bl))
    return fail(QR_EINVAL, "zgemm_df: the Gram mode computes I - A^H A (op C, B = A)");
  int pr = prof_begin(s, PK_ZGEMM_DF, (mode == DF_GRAM ? 4.0 : 8.0) * M * N * K,
                      (mode == DF_F32_AXPY ? 8.0 : 16.0) * ((double)M * K + (double)K * N) + 16.0 * M * N);
  int rc = QR_OK;
#define QR_DF_CASE(OPV, MV)                                                                                   \
  if (opA == OPV && mode == MV)                                                                               \
    rc = launch_df<OPV, MV>(s, M, N, K, Ah, Al, lda, Bh, Bl, ldb, Ch, Cl, ldc, Dh, Dl, ldd, alpha);
  QR_DF_CASE(OP_N, DF_STORE)
  QR_DF_CASE(OP_C, DF_STORE)
  QR_DF_CASE(OP_T, DF_STORE)
  QR_DF_CASE(OP_N, DF_I_MINUS)
  QR_DF_CASE(OP_C, DF_I_MINUS)
  QR_DF_CASE(OP_T, DF_I_MINUS)
  QR_DF_CASE(OP_N, DF_F32_AXPY)
  QR_DF_CASE(OP_C, DF_F32_AXPY)
  QR_DF_CASE(OP_T, DF_F32_AXPY)
  QR_DF_CASE(OP_C, DF_GRAM)
#undef QR_DF_CASE
  prof_end(s, pr);
  return rc;
}

int z2df(cudaStream_t s, const double2* src, long lds, int rows, int cols, const double* scale, float2* hi,
         float2* lo, long ldd) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  to_df_scaled_k<<<grid_for((long)rows * cols), TPB, 0, s>>>(src, lds, rows, cols, scale, hi, lo, ldd);
  QR_CHECK_LAUNCH("to_df_scaled_k");
  return QR_OK;
}

int z2df_cols(cudaStream_t s, const double2* src, long lds, int rows, int cols, const double* colscale, float2* hi,
              float2* lo, long ldd) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  to_df_cols_k<<<grid_for((long)rows * cols), TPB, 0, s>>>(src, lds, rows, cols, colscale, hi, lo, ldd);
  QR_CHECK_LAUNCH("to_df_cols_k");
  return QR_OK;
}

int df2z(cudaStream_t s, const float2* hi, const float2* lo, long lds, int rows, int cols, const double* scale,
         double2* dst, long ldd) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  from_df_scaled_k<<<grid_for((long)rows * cols), TPB, 0, s>>>(hi, lo, lds, rows, cols, scale, dst, ldd);
  QR_CHECK_LAUNCH("from_df_scaled_k");
  return QR_OK;
}

}  // namespace qr

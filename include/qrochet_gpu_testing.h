/*
 * qrochet_gpu_testing.h -- instrumentation and kernel-level test hooks of libqrochet_gpu.so.
 *
 * Not part of the reference-facing interface (qrochet_gpu.h): no Qrochet.jl method corresponds to
 * anything here.  Benchmarks read per-kernel-class timers and measure pipe peaks through these
 * calls; the GPU test suite drives single kernels on host matrices through the qr_test_* hooks.
 */
#ifndef QROCHET_GPU_TESTING_H
#define QROCHET_GPU_TESTING_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* per-kernel-class CUDA-event timing, for benchmarks: kinds 0 zgemm (FP64 DMMA), 1 Jacobi FP64,
   2 Jacobi FP32, 3 Householder QR, 4 environment mixing, 5 split-precision tensor-core zgemm,
   6 double-float Jacobi polish, 7 double-float zgemm.  `launches` counts kernel launches of the
   class (one per Jacobi sweep). */
int qr_prof_enable(int on);
int qr_prof_read(int kind, double* ms, uint64_t* launches, double* flops, double* bytes);
/* peak of one pipe measured now: 0 FP64 tensor (DMMA), 1 FP32 FFMA, 2 FP64 DFMA (TFLOP/s) */
int qr_probe_peak(int kind, double* tflops);

/* ---- kernel-level test hooks (no reference counterpart): host matrices in and out, complex
   interleaved, column-major; op codes 0 N, 1 T, 2 C (conjugate transpose), 3 R (conjugate) ----- */
int qr_test_zgemm(int opA, int opB, int M, int N, int K, const double* alpha, const double* A, long lda,
                  const double* B, long ldb, const double* beta, double* C, long ldc, const double* dk,
                  int iters, double* ms_per_iter);
/* C[b] = op(A[b]) op(B[b]) on the tcgen05 tensor cores (TMA-staged BF16x3 slices, TMEM
   accumulators); `batch` matrices at strides sA / sB (sB = 0: B shared), C[b] at b * ldc * N. */
int qr_test_zgemm_tc(int opA, int opB, int M, int N, int K, int batch, const double* A, long lda, long sA,
                     const double* B, long ldb, long sB, double* C, long ldc, int iters, double* ms_per_iter);
/* Double-float GEMM on the FP32 pipes.  mode 0: C = op(A) B; 1: C = I - op(A) B; 2: C = D + 0.5
   op(A) B with FP32 products (A, B rounded to FP32); 3: C = I - A^H A from the upper tiles (op C,
   B ignored).  op(A) in {0 N, 1 T, 2 C}; D used by mode 2. */
int qr_test_zgemm_df(int mode, int opA, int M, int N, int K, const double* A, long lda, const double* B, long ldb,
                     const double* D, double* C, long ldc, int iters, double* ms_per_iter);
int qr_test_svd(int mode, int m, int n, const double* A, double* U, double* S, double* Vh, double* ms);
/* how often each SVD code path ran in this process: 0 cluster Jacobi, 1 FP32 block cluster,
   2 / 3 FP32 block sweep with grid barrier / per-block flags, 4 / 5 FP64 sweep barrier / flags,
   6 / 7 FP32 scalar sweep barrier / flags, 8 double-float cluster polish, 9 / 10 double-float
   sweep barrier / flags, 11 FP64 QR preconditioning, 12 mixed restart on R^H, 13 Householder
   re-orthonormalisation, 14 masked FP32 block sweeps, 15 masked (listed) double-float sweep, 16
   first-order final polish rotation, 17 double-float block sweep.  Copies min(n, *total)
   counters; *total = number of paths. */
int qr_test_svd_paths(uint64_t* counts, int n, int* total);
/* The host-side greedy colour schedule of a masked Jacobi sweep (no GPU needed).  mask: nv rows
   of ceil(nv / 32) words, bit (q & 31) of word p * ceil(nv / 32) + q / 32 marks pair p < q; flag:
   nv words (or NULL), 1 = the pairs inside vertex v need a visit (with use_flag).  items
   (nv (nv - 1) / 2 words): listed pairs as p | q << 15 | full << 30, colour class by colour class;
   ord (2 per item): listed pairs before the item on p and on q.  nv even, 2 <= nv < 32768. */
int qr_test_schedule_pairs(const unsigned* mask, const unsigned* flag, int nv, int use_flag, unsigned* items,
                           unsigned* ord, long* listed, int* classes);
int qr_test_qr(int m, int n, const double* A, double* Q, double* R, double* ms);
/* Throws a C++ exception inside an exported function (kind 0: std::bad_alloc, 1: a standard
   std::runtime_error, 2: an object of no standard type) so that a test sees the ABI guard turn it
   into a status (QR_ENOMEM, QR_EHOST, QR_EHOST) and a message; any other kind returns QR_OK.
   Host only: no GPU needed. */
int qr_test_host_exception(int kind);

#ifdef __cplusplus
}
#endif
#endif /* QROCHET_GPU_TESTING_H */

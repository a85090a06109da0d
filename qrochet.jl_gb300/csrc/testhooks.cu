// Kernel-level entry points for unit tests and kernel benchmarks: host matrices in, host results
// and CUDA-event timings out.  They have no counterpart in the reference.
#include <vector>
#include <stdexcept>
#include "kernels.cuh"

using namespace qr;

namespace {
struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
};
int up(Dev& d, const double* h, size_t n_complex) {
  QR_CUDA(cudaMalloc(&d.p, sizeof(double2) * (n_complex ? n_complex : 1)));
  if (h) QR_CUDA(cudaMemcpy(d.p, h, sizeof(double2) * n_complex, cudaMemcpyHostToDevice));
  return QR_OK;
}
}  // namespace

extern "C" {

// C = alpha op(A) diag(dk) op(B) + beta C, column-major; `iters` timed repetitions (C is
// recomputed from the original each time).  ms_per_iter receives the average event time.
int qr_test_zgemm(int opA, int opB, int M, int N, int K, const double* alpha, const double* A, long lda,
                  const double* B, long ldb, const double* beta, double* C, long ldc, const double* dk,
                  int iters, double* ms_per_iter) try {
  if (M <= 0 || N <= 0 || K < 0 || iters < 1) return fail(QR_EINVAL, "bad gemm shape");
  long ra = (opA == OP_N || opA == OP_R) ? M : K, ca = (opA == OP_N || opA == OP_R) ? K : M;
  long rb = (opB == OP_N || opB == OP_R) ? K : N, cb = (opB == OP_N || opB == OP_R) ? N : K;
  if (lda < ra || ldb < rb || ldc < M) return fail(QR_EINVAL, "bad leading dimension");
  Dev dA, dB, dC, dC0, dD;
  QR_TRY(up(dA, A, (size_t)lda * ca));
  QR_TRY(up(dB, B, (size_t)ldb * cb));
  QR_TRY(up(dC0, C, (size_t)ldc * N));
  QR_TRY(up(dC, C, (size_t)ldc * N));
  if (dk) {
    QR_CUDA(cudaMalloc(&dD.p, sizeof(double) * (K ? K : 1)));
    QR_CUDA(cudaMemcpy(dD.p, dk, sizeof(double) * K, cudaMemcpyHostToDevice));
  }
  double2 al = make_double2(alpha[0], alpha[1]), be = make_double2(beta[0], beta[1]);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float total = 0;
  int rc = QR_OK;
  for (int it = 0; it < iters && rc == QR_OK; it++) {
    QR_CUDA(cudaMemcpy(dC.p, dC0.p, sizeof(double2) * ldc * N, cudaMemcpyDeviceToDevice));
    cudaEventRecord(e0);
    rc = zgemm(0, opA, opB, M, N, K, al, (double2*)dA.p, lda, 0, (double2*)dB.p, ldb, 0, be, (double2*)dC.p, ldc, 0,
               1, (double*)dD.p);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QR_TRY(rc);
  QR_CUDA(cudaMemcpy(C, dC.p, sizeof(double2) * ldc * N, cudaMemcpyDeviceToHost));
  if (ms_per_iter) *ms_per_iter = total / iters;
  return QR_OK;
} QR_ABI_CATCH

// C[b] = op(A[b]) op(B[b]) with the tcgen05 split-precision kernel (gemm_tc.cu); A and B hold
// `batch` matrices at strides sA and sB (sB = 0: one B shared by the batch), C at stride ldc * N.
int qr_test_zgemm_tc(int opA, int opB, int M, int N, int K, int batch, const double* A, long lda, long sA,
                     const double* B, long ldb, long sB, double* C, long ldc, int iters, double* ms_per_iter) try {
  if (M <= 0 || N <= 0 || K < 0 || iters < 1 || batch < 1) return fail(QR_EINVAL, "bad gemm shape");
  long ca = (opA == OP_N || opA == OP_R) ? K : M;
  long cb = (opB == OP_N || opB == OP_R) ? N : K;
  const long sC = ldc * N;
  if (sA < lda * ca && batch > 1) return fail(QR_EINVAL, "bad batch stride");
  Dev dA, dB, dC, dW;
  QR_TRY(up(dA, A, (size_t)(batch > 1 ? sA * (batch - 1) : 0) + (size_t)lda * ca));
  QR_TRY(up(dB, B, (size_t)(sB ? sB * (batch - 1) : 0) + (size_t)ldb * cb));
  QR_TRY(up(dC, nullptr, (size_t)sC * batch));
  const size_t wsb = zgemm_tc_workspace(M, N, K, batch, sB == 0);
  QR_CUDA(cudaMalloc(&dW.p, wsb + 256));
  unsigned* err = static_cast<unsigned*>(dW.p);
  void* ws = static_cast<char*>(dW.p) + 256;
  QR_CUDA(cudaMemset(err, 0, sizeof(unsigned)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float total = 0;
  int rc = QR_OK;
  for (int it = 0; it < iters && rc == QR_OK; it++) {
    cudaEventRecord(e0);
    rc = zgemm_tc(0, opA, opB, M, N, K, (double2*)dA.p, lda, sA, (double2*)dB.p, ldb, sB, (double2*)dC.p, ldc, sC,
                  batch, ws, err);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QR_TRY(rc);
  QR_CUDA(cudaDeviceSynchronize());
  unsigned herr = 0;
  QR_CUDA(cudaMemcpy(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (herr) return fail(QR_ECUDA, "tensor-core GEMM: a bounded wait gave up");
  QR_CUDA(cudaMemcpy(C, dC.p, sizeof(double2) * sC * batch, cudaMemcpyDeviceToHost));
  if (ms_per_iter) *ms_per_iter = total / iters;
  return QR_OK;
} QR_ABI_CATCH

// Double-float GEMM (gemm_df.cu) through FP64 host matrices: inputs are split into (hi, lo) FP32
// pairs on the device, the result converted back (mode 1 returns the FP32 value I - op(A) B).
int qr_test_zgemm_df(int mode, int opA, int M, int N, int K, const double* A, long lda, const double* B, long ldb,
                     const double* D, double* C, long ldc, int iters, double* ms_per_iter) try {
  if (M <= 0 || N <= 0 || K < 0 || iters < 1 || mode < 0 || mode > 3) return fail(QR_EINVAL, "bad gemm_df shape");
  if (opA != OP_N && opA != OP_T && opA != OP_C) return fail(QR_EINVAL, "op(A) must be N, T or C");
  const long ca = opA == OP_N ? K : M, rb = K;
  if (lda < (opA == OP_N ? M : K) || ldb < rb || ldc < M) return fail(QR_EINVAL, "bad leading dimension");
  if (mode == 2 && !D) return fail(QR_EINVAL, "mode 2 needs D");
  Dev dA, dB, dD, aS, bS, cS, dS;
  QR_TRY(up(dA, A, (size_t)lda * ca));
  QR_TRY(up(dB, B, (size_t)ldb * N));
  QR_TRY(up(aS, nullptr, (size_t)lda * ca));  // (hi, lo) float2 pairs: 16 bytes per element
  QR_TRY(up(bS, nullptr, (size_t)ldb * N));
  QR_TRY(up(cS, nullptr, (size_t)ldc * N));
  const size_t na = (size_t)lda * ca, nb = (size_t)ldb * N, nc = (size_t)ldc * N;
  float2 *Ah = (float2*)aS.p, *Al = Ah + na, *Bh = (float2*)bS.p, *Bl = Bh + nb, *Ch = (float2*)cS.p, *Cl = Ch + nc;
  float2 *Dh = nullptr, *Dl = nullptr;
  QR_TRY(z2df(0, (double2*)dA.p, lda, (int)lda, (int)ca, nullptr, Ah, Al, lda));
  QR_TRY(z2df(0, (double2*)dB.p, ldb, (int)ldb, N, nullptr, Bh, Bl, ldb));
  if (mode == 2) {
    QR_TRY(up(dD, D, nc));
    QR_TRY(up(dS, nullptr, nc));
    Dh = (float2*)dS.p;
    Dl = Dh + nc;
    QR_TRY(z2df(0, (double2*)dD.p, ldc, (int)ldc, N, nullptr, Dh, Dl, ldc));
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  int rc = QR_OK;
  for (int it = 0; it < iters && rc == QR_OK; it++)
    rc = mode == 3 ? zgemm_df(0, mode, opA, M, N, K, Ah, Al, lda, Ah, Al, lda, Ch, Cl, ldc)
                   : zgemm_df(0, mode, opA, M, N, K, Ah, mode == 2 ? nullptr : Al, lda, Bh, mode == 2 ? nullptr : Bl, ldb,
                              Ch, Cl, ldc, Dh, Dl, ldc, 0.5f);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QR_TRY(rc);
  if (ms_per_iter) *ms_per_iter = t / iters;
  if (mode == 1 || mode == 3) {
    std::vector<float2> h(nc);
    QR_CUDA(cudaMemcpy(h.data(), Ch, sizeof(float2) * nc, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nc; i++) { C[2 * i] = h[i].x; C[2 * i + 1] = h[i].y; }
    return QR_OK;
  }
  Dev dC;
  QR_TRY(up(dC, nullptr, nc));
  QR_TRY(df2z(0, Ch, Cl, ldc, (int)ldc, N, nullptr, (double2*)dC.p, ldc));
  QR_CUDA(cudaMemcpy(C, dC.p, sizeof(double2) * nc, cudaMemcpyDeviceToHost));
  return QR_OK;
} QR_ABI_CATCH

// Thin SVD of the m x n column-major A: U (m x k), S (k), Vh (k x n), k = min(m, n).
// counts[i] = how often SVD code path i ran in this process (i < min(n, SP_COUNT)); *total = SP_COUNT
int qr_test_schedule_pairs(const unsigned* mask, const unsigned* flag, int nv, int use_flag, unsigned* items,
                           unsigned* ord, long* listed, int* classes) try {
  if (nv < 2 || nv % 2 || nv >= 32768 || !mask || !items || !ord || !listed || !classes)
    return fail(QR_EINVAL, "schedule: nv must be even, in [2, 32768), and the arrays given");
  *listed = schedule_pairs_host(mask, flag, nv, use_flag, items, ord, classes);
  return QR_OK;
} QR_ABI_CATCH

int qr_test_svd_paths(uint64_t* counts, int n, int* total) try {
  for (int i = 0; i < n && i < SP_COUNT; i++) counts[i] = g_svd_path[i].load(std::memory_order_relaxed);
  if (total) *total = SP_COUNT;
  return QR_OK;
} QR_ABI_CATCH

int qr_test_svd(int mode, int m, int n, const double* A, double* U, double* S, double* Vh, double* ms) try {
  if (m <= 0 || n <= 0) return fail(QR_EINVAL, "bad svd shape");
  const int k = m < n ? m : n;
  Dev dA, dU, dV, dS;
  QR_TRY(up(dA, A, (size_t)m * n));
  QR_TRY(up(dU, nullptr, (size_t)m * k));
  QR_TRY(up(dV, nullptr, (size_t)k * n));
  QR_CUDA(cudaMalloc(&dS.p, sizeof(double) * k));
  cudaStream_t s;
  QR_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  SvdWork* w = svd_work_create();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  int rc = zsvd_thin(s, w, mode, (double2*)dA.p, m, n, m, (double2*)dU.p, m, (double*)dS.p, (double2*)dV.p, k);
  cudaEventRecord(e1, s);
  cudaStreamSynchronize(s);
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  svd_work_free(w);
  cudaStreamDestroy(s);
  QR_TRY(rc);
  if (U) QR_CUDA(cudaMemcpy(U, dU.p, sizeof(double2) * m * k, cudaMemcpyDeviceToHost));
  if (Vh) QR_CUDA(cudaMemcpy(Vh, dV.p, sizeof(double2) * k * n, cudaMemcpyDeviceToHost));
  if (S) QR_CUDA(cudaMemcpy(S, dS.p, sizeof(double) * k, cudaMemcpyDeviceToHost));
  return QR_OK;
} QR_ABI_CATCH

// Thin Householder QR of the m x n column-major A: Q (m x k), R (k x n).
int qr_test_qr(int m, int n, const double* A, double* Q, double* R, double* ms) try {
  if (m <= 0 || n <= 0) return fail(QR_EINVAL, "bad qr shape");
  const int k = m < n ? m : n;
  Dev dA, dQ, dR, dT;
  QR_TRY(up(dA, A, (size_t)m * n));
  QR_TRY(up(dQ, nullptr, (size_t)m * k));
  QR_TRY(up(dR, nullptr, (size_t)k * n));
  QR_TRY(up(dT, nullptr, (size_t)k));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  int rc = zqr_thin(0, (double2*)dA.p, m, n, m, (double2*)dQ.p, m, (double2*)dR.p, k, (double2*)dT.p);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QR_TRY(rc);
  QR_CUDA(cudaMemcpy(Q, dQ.p, sizeof(double2) * m * k, cudaMemcpyDeviceToHost));
  QR_CUDA(cudaMemcpy(R, dR.p, sizeof(double2) * k * n, cudaMemcpyDeviceToHost));
  return QR_OK;
} QR_ABI_CATCH

int qr_test_host_exception(int kind) try {
  struct NotStd {};
  if (kind == 0) throw std::bad_alloc();
  if (kind == 1) throw std::runtime_error("planted by qr_test_host_exception");
  if (kind == 2) throw NotStd();
  return QR_OK;
} QR_ABI_CATCH

}  // extern "C"

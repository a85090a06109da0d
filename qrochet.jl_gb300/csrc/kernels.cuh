// Internal launch wrappers of the qrochet GB300 library (all enqueue on the given stream).
#pragma once
#include "common.cuh"

namespace qr {

enum { OP_N = 0, OP_T = 1, OP_C = 2, OP_R = 3 };

// ---- gemm.cu -----------------------------------------------------------------------------------
int zgemm(cudaStream_t s, int opA, int opB, int M, int N, int K, double2 alpha,
          const double2* A, long lda, long sA, const double2* B, long ldb, long sB,
          double2 beta, double2* C, long ldc, long sC, int batch, const double* dk);

// ---- gemm_tc.cu: C = op(A) op(B) on the tcgen05 tensor cores: operands rounded to FP32 and split
// into three BF16 slices, six slice products, FP32 accumulation in TMEM, TMA-staged tiles.
// ws: device workspace of zgemm_tc_workspace(M, N, K, batch, sB == 0) bytes; err: device flag set to 1 if a CTA's bounded wait gave up (then C is not valid).
size_t zgemm_tc_workspace(int M, int N, int K, int batch, bool bshared);
int zgemm_tc(cudaStream_t s, int opA, int opB, int M, int N, int K, const double2* A, long lda, long sA,
             const double2* B, long ldb, long sB, double2* C, long ldc, long sC, int batch, void* ws,
             unsigned* err);
// the same product of complex FP32 operands (the FP32 Jacobi stage's Gram matrices)
int zgemm_tc(cudaStream_t s, int opA, int opB, int M, int N, int K, const float2* A, long lda, long sA,
             const float2* B, long ldb, long sB, double2* C, long ldc, long sC, int batch, void* ws,
             unsigned* err);

// ---- gemm_df.cu: complex GEMM in double-float (hi, lo FP32 pairs) on the FP32 pipes
enum { DF_STORE = 0, DF_I_MINUS = 1, DF_F32_AXPY = 2, DF_GRAM = 3 };
// DF_STORE: (Ch, Cl) = op(A) B; DF_I_MINUS: Ch = I - op(A) B (FP32); DF_F32_AXPY: (Ch, Cl) = D +
// alpha op(A_hi) B_hi with FP32 products; DF_GRAM: Ch = I - A^H A from the tiles on or above the
// diagonal (op C, B = A).  op(A) in {N, T, C}; B is not transformed.
int zgemm_df(cudaStream_t s, int mode, int opA, int M, int N, int K, const float2* Ah, const float2* Al, long lda,
             const float2* Bh, const float2* Bl, long ldb, float2* Ch, float2* Cl, long ldc,
             const float2* Dh = nullptr, const float2* Dl = nullptr, long ldd = 0, float alpha = 1.f);
// FP64 <-> double-float split arrays; the optional device scale divides on the way in and
// multiplies on the way out
int z2df(cudaStream_t s, const double2* src, long lds, int rows, int cols, const double* scale, float2* hi,
         float2* lo, long ldd);
int df2z(cudaStream_t s, const float2* hi, const float2* lo, long lds, int rows, int cols, const double* scale,
         double2* dst, long ldd);
// hi/lo of src with column j multiplied by colscale[j] (colscale may be null)
int z2df_cols(cudaStream_t s, const double2* src, long lds, int rows, int cols, const double* colscale, float2* hi,
              float2* lo, long ldd);

// ---- random.cu: E (rows x N, ld rows) = scale * the Gram-Schmidt orthonormalised rows of a
// uniform [0,1) random rows x N matrix (complex entries when cplx), from stream `stream` of `seed`
int rand_rows_isometry(cudaStream_t s, int rows, int N, uint64_t seed, uint32_t stream, int cplx, double scale,
                       double2* E);

// ---- misc.cu -----------------------------------------------------------------------------------
int zscale_matrix(cudaStream_t s, int M, int N, double2 alpha, double2* C, long ldc, long sC,
                  int batch);
// dst (column-major, dims dst_dims[0..nd)) gathers src through per-dst-dim source strides
struct Perm {
  int nd;
  long dims[4];
  long src_stride[4];
};
int zpermute(cudaStream_t s, const double2* src, double2* dst, const Perm& p);
// A[l,o,r] *= f(lam[l]) (side 0) or f(lam[r]) (side 2); f = x, or pinv with atol when inv
int zscale_bond(cudaStream_t s, double2* A, int cl, int d, int cr, const double* lam, int side,
                int inv, double atol);
// A[l,o',r] = sum_o G[o',o] A[l,o,r], G row-major d x d in device memory
int zgate1(cudaStream_t s, double2* A, int cl, int d, int cr, const double2* G);
// theta[(l,o1),(o2,r)] (ld cl*d) <- G[(o1',o2'),(o1,o2)] theta, G row-major d^2 x d^2 (device)
int zgate2(cudaStream_t s, double2* theta, int cl, int d, int cr, const double2* G);
// dst[j + i*ldd] = op(src[i + j*lds]) for i<rows, j<cols (transpose, optional conjugate)
int ztranspose(cudaStream_t s, const double2* src, long lds, int rows, int cols, double2* dst,
               long ldd, int conj);
int zset_identity(cudaStream_t s, double2* A, int rows, int cols, long lda);
int cset_identity(cudaStream_t s, float2* A, int rows, int cols, long lda);
int z2c(cudaStream_t s, const double2* src, long lds, float2* dst, long ldd, int rows, int cols);
// out[0] = || G - I ||_F for the n x n matrix G (ld n); out is device memory
int zdist_identity(cudaStream_t s, const double2* G, int n, double* out);
// lam[i] /= norm2(lam) in place (device)
int dnormalize(cudaStream_t s, double* lam, int len);

// ---- qr.cu -------------------------------------------------------------------------------------
// Thin Householder QR of the m x n matrix A (ld lda, overwritten).  Q: m x k (ld ldq) and
// R: k x n (ld ldr), k = min(m, n).  tau: device workspace of k entries.
int zqr_thin(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq,
             double2* R, long ldr, double2* tau);
// The same factorisation with one launch per column and no scratch beyond tau (for callers that
// must not allocate).
int zqr_thin_steps(cudaStream_t s, double2* A, int m, int n, long lda, double2* Q, long ldq,
                   double2* R, long ldr, double2* tau);

// ---- svd.cu ------------------------------------------------------------------------------------
struct SvdWork;  // opaque, grows on demand
SvdWork* svd_work_create();
void svd_work_free(SvdWork* w);
// Thin SVD of the m x n matrix A (ld lda; A is preserved).  U: m x k (ld ldu), S: k (device),
// Vh: k x n (ld ldvh), k = min(m,n), S descending.  mode: QR_FP64 or QR_MIXED.  The leading
// `keep` singular vectors (keep <= 0: all k) are orthonormal to ~1e-11; the rest may be less so
// when their singular values are many decades below sigma_max (callers then discard them).
int zsvd_thin(cudaStream_t s, SvdWork* w, int mode, const double2* A, int m, int n, long lda,
              double2* U, long ldu, double* S, double2* Vh, long ldvh, int keep = 0);
// The greedy colour schedule of a masked Jacobi sweep, on host arrays (tests; see svd.cu).
long schedule_pairs_host(const unsigned* mask, const unsigned* flag, int nv, int use_flag, unsigned* items,
                         unsigned* ord, int* classes);
// Process-wide counts of the SVD code paths taken (one per Jacobi stage of a call), so tests can
// check which ordering and which kernel a size reached.
enum SvdPath {
  SP_CLUSTER = 0,        // whole Jacobi in one thread-block cluster (k <= 128)
  SP_BLOCK_CLUSTER,      // FP32 block Jacobi in one cluster
  SP_BLOCK_BARRIER,      // FP32 block sweep, grid barrier between rounds
  SP_BLOCK_DATAFLOW,     // FP32 block sweep, per-block flags (more block pairs than CTAs)
  SP_F64_BARRIER,        // FP64 scalar sweep, grid barrier
  SP_F64_DATAFLOW,       // FP64 scalar sweep, per-column flags
  SP_F32_BARRIER,        // FP32 scalar sweep (rows > 2048), grid barrier
  SP_F32_DATAFLOW,       // FP32 scalar sweep, per-column flags
  SP_DF_CLUSTER,         // double-float polish in one cluster
  SP_DF_BARRIER,         // double-float polish sweep, grid barrier
  SP_DF_DATAFLOW,        // double-float polish sweep, per-column flags
  SP_QR_PRECOND_FP64,    // FP64 path on R^H of a Householder QR
  SP_QR_PRECOND_MIXED,   // mixed path restarted on R^H after its FP32 probe
  SP_REORTH,             // Householder re-orthonormalisation of the kept singular vectors
  SP_BLOCK_MASKED,       // FP32 block sweeps over the block pairs a Gram test marks
  SP_DF_MASKED,          // double-float polish sweep over the marked pairs in round order
  SP_DF_LINEAR,          // double-float polish: marked pairs rotated at once to first order
  SP_DF_BLOCK,           // double-float polish: full sweeps over pairs of 2-column blocks
  SP_COUNT
};
extern std::atomic<uint64_t> g_svd_path[SP_COUNT];
inline void svd_path(int p) { g_svd_path[p].fetch_add(1, std::memory_order_relaxed); }

}  // namespace qr

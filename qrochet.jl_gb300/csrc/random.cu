// Random isometries on the device for rand(Chain, Open, State / Operator)
// (src/Ansatz/Chain.jl:223-297).
//
// The reference draws A = rand(T, rows, N) (uniform [0, 1) entries; for a complex T the real and
// imaginary parts are independent uniforms) and orthonormalises its rows with Gram-Schmidt.  Row
// Gram-Schmidt equals the Q factor of A^H: A^H = Q R with R's diagonal positive gives
// A = R^H Q^H with R^H lower triangular, so the orthonormalised rows are Q^H.  Here A^H is formed
// directly from a counter-based generator, factored by the Householder QR (qr.cu), and the
// columns of Q are multiplied by the signs of R's (real) diagonal.
//
// Generator: Philox-4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC 2011), written from the published round function.  Element e of stream `stream`
// uses counter (e_lo, e_hi, stream, 0) and key (seed_lo, seed_hi), so every entry is a pure
// function of (seed, stream, e): the result does not depend on launch shapes.
#include "kernels.cuh"

namespace qr {
namespace {

constexpr int TPB = 256;

__device__ __forceinline__ void philox_round(uint32_t c[4], const uint32_t k[2]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t lo0 = M0 * c[0], hi0 = __umulhi(M0, c[0]);
  const uint32_t lo1 = M1 * c[2], hi1 = __umulhi(M1, c[2]);
  const uint32_t n0 = hi1 ^ c[1] ^ k[0], n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  uint32_t k[2] = {k0, k1};
#pragma unroll
  for (int r = 0; r < 10; r++) {
    philox_round(c, k);
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
}

// uniform double in [0, 1) with 53 random bits from two 32-bit words
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// W (N x rows, ld N) = A^H for A (rows x N) with A[l, c] ~ U[0,1) (+ i U[0,1) when cplx)
__global__ void rand_adjoint_k(double2* __restrict__ W, int rows, int N, uint64_t seed, uint32_t stream, int cplx) {
  const long total = (long)rows * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long c = t % N, l = t / N;  // W[c + N l] = conj(A[l, c])
    const uint64_t e = (uint64_t)l + (uint64_t)rows * (uint64_t)c;  // column-major index of A[l, c]
    uint32_t ctr[4] = {(uint32_t)e, (uint32_t)(e >> 32), stream, 0u};
    philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double re = u53(ctr[0], ctr[1]);
    const double im = cplx ? u53(ctr[2], ctr[3]) : 0.0;
    W[c + (long)N * l] = make_double2(re, -im);
  }
}

// E (rows x N, ld rows) = (Q diag(sign(beta)))^H, beta = the real diagonal of R left on Wf's
// diagonal by the Householder QR; `scale` multiplies the result
__global__ void rows_from_q_k(const double2* __restrict__ Q, const double2* __restrict__ Wf, int rows, int N,
                              double scale, double2* __restrict__ E) {
  const long total = (long)rows * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long l = t % rows, c = t / rows;
    const double sg = Wf[l + (long)N * l].x < 0.0 ? -scale : scale;
    const double2 q = Q[c + (long)N * l];
    E[l + (long)rows * c] = make_double2(sg * q.x, -sg * q.y);
  }
}

unsigned grid_for(long total) {
  long g = (total + TPB - 1) / TPB;
  return (unsigned)(g > 4864 ? 4864 : (g < 1 ? 1 : g));
}

}  // namespace

int rand_rows_isometry(cudaStream_t s, int rows, int N, uint64_t seed, uint32_t stream, int cplx, double scale,
                       double2* E) {
  if (rows <= 0 || N <= 0) return QR_OK;
  if (rows > N) return fail(QR_EINVAL, "an isometry with orthonormal rows needs rows <= columns");
  double2 *W = nullptr, *Q = nullptr, *tau = nullptr;
  QR_CUDA(cudaMallocAsync(&W, sizeof(double2) * (size_t)N * rows, s));
  cudaError_t e1 = cudaMallocAsync(&Q, sizeof(double2) * (size_t)N * rows, s);
  cudaError_t e2 = cudaMallocAsync(&tau, sizeof(double2) * (size_t)rows, s);
  int rc = QR_OK;
  if (e1 != cudaSuccess || e2 != cudaSuccess) rc = cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaMallocAsync");
  if (!rc) {
    rand_adjoint_k<<<grid_for((long)rows * N), TPB, 0, s>>>(W, rows, N, seed, stream, cplx);
    rc = cudaGetLastError() == cudaSuccess ? QR_OK : fail(QR_ECUDA, "rand_adjoint_k launch");
    count_launch();
  }
  if (!rc) rc = zqr_thin(s, W, N, rows, N, Q, N, nullptr, 0, tau);
  if (!rc) {
    rows_from_q_k<<<grid_for((long)rows * N), TPB, 0, s>>>(Q, W, rows, N, scale, E);
    rc = cudaGetLastError() == cudaSuccess ? QR_OK : fail(QR_ECUDA, "rows_from_q_k launch");
    count_launch();
  }
  if (W) cudaFreeAsync(W, s);
  if (Q) cudaFreeAsync(Q, s);
  if (tau) cudaFreeAsync(tau, s);
  return rc;
}

}  // namespace qr

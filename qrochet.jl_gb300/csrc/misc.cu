// Memory-bound kernels of the Chain path: layout permutes at the host boundary, bond scaling by
// Lambda (and its pseudo-inverse), physical-index gates, transposes, precision conversions.
// All are grid-stride loops over the output with coalesced writes.
#include "kernels.cuh"

namespace qr {

namespace {

constexpr int TPB = 256;

inline unsigned grid_for(long n) {
  long g = (n + TPB - 1) / TPB;
  if (g > 152L * 32) g = 152L * 32;  // grid-stride beyond 32 CTAs per SM
  return (unsigned)(g < 1 ? 1 : g);
}

__global__ void scale_matrix_k(int M, int N, double2 alpha, double2* C, long ldc, long sC) {
  C += blockIdx.y * sC;
  long total = (long)M * N;
  const bool zero = (alpha.x == 0.0 && alpha.y == 0.0);
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % M, j = t / M;
    double2* p = C + i + j * ldc;
    *p = zero ? make_double2(0.0, 0.0) : cmul(alpha, *p);
  }
}

__global__ void permute_k(const double2* __restrict__ src, double2* __restrict__ dst, Perm p, long total) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long rem = t, off = 0;
    for (int k = 0; k < p.nd; k++) {
      long c = rem % p.dims[k];
      rem /= p.dims[k];
      off += c * p.src_stride[k];
    }
    dst[t] = src[off];
  }
}

// Tiled permute for a layout change whose source-contiguous dimension `a` is not the
// destination's first dimension: per batch index (the other dimensions), a tile of TA elements
// along `a` by T0 = 1024 / TA along dimension 0 is read with consecutive threads on consecutive
// source addresses (dimension a), staged in shared memory, and written with consecutive threads
// on consecutive destination addresses (dimension 0).  For the site layouts (o,l,r) <-> (l,o,r)
// with d = 2 the tile is 1024 x 2 and both sides are fully contiguous.  Each thread issues its
// eight loads of a tile before the first shared-memory store, so a tile costs one DRAM round trip.
constexpr int PT_THREADS = 256, PT_PER = 8, PT_ELEMS = PT_THREADS * PT_PER;
__global__ void __launch_bounds__(PT_THREADS) permute_tiled_k(const double2* __restrict__ src,
                                                              double2* __restrict__ dst, Perm p, int a, int ta,
                                                              long nbatch) {
  // rows of ta + 1 elements: the store phase reads column-wise with a stride of ta + 1 elements,
  // which spreads a quarter-warp's 16-byte reads over all banks
  __shared__ double2 tile[PT_ELEMS + PT_ELEMS / 2];
  const int t0 = PT_ELEMS / ta, tp = ta + 1;
  const long d0 = p.dims[0], da = p.dims[a];
  long dstride[4];
  dstride[0] = 1;
  for (int k = 1; k < p.nd; k++) dstride[k] = dstride[k - 1] * p.dims[k - 1];
  const long ss0 = p.src_stride[0], dsa = dstride[a];
  const long tiles0 = (d0 + t0 - 1) / t0, tilesa = (da + ta - 1) / ta;
  const long ntiles = tiles0 * tilesa * nbatch;
  for (long tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
    const long i0t = tt % tiles0, iat = (tt / tiles0) % tilesa;
    long bidx = tt / (tiles0 * tilesa);
    long sbase = 0, dbase = 0;
    for (int k = 1; k < p.nd; k++) {
      if (k == a) continue;
      const long c = bidx % p.dims[k];
      bidx /= p.dims[k];
      sbase += c * p.src_stride[k];
      dbase += c * dstride[k];
    }
    const long o0 = i0t * t0, a0 = iat * ta;
    double2 v[PT_PER];
#pragma unroll
    for (int q = 0; q < PT_PER; q++) {  // consecutive threads: along a
      const int e = threadIdx.x + q * PT_THREADS, ia = e % ta, i0 = e / ta;
      if (o0 + i0 < d0 && a0 + ia < da) v[q] = src[sbase + (a0 + ia) + (o0 + i0) * ss0];
    }
#pragma unroll
    for (int q = 0; q < PT_PER; q++) {
      const int e = threadIdx.x + q * PT_THREADS, ia = e % ta, i0 = e / ta;
      if (o0 + i0 < d0 && a0 + ia < da) tile[i0 * tp + ia] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PT_PER; q++) {  // consecutive threads: along dim 0
      const int e = threadIdx.x + q * PT_THREADS, i0 = e % t0, ia = e / t0;
      if (o0 + i0 < d0 && a0 + ia < da) dst[dbase + (o0 + i0) + (a0 + ia) * dsa] = tile[i0 * tp + ia];
    }
    __syncthreads();  // the tile is refilled by the next iteration
  }
}

__global__ void scale_bond_k(double2* A, int cl, int d, int cr, const double* __restrict__ lam,
                             int side, int inv, double atol) {
  long total = (long)cl * d * cr;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long idx = (side == 0) ? (t % cl) : (t / ((long)cl * d));
    double x = lam[idx];
    double f = inv ? ((fabs(x) > atol) ? 1.0 / x : 0.0) : x;
    A[t] = cscale(A[t], f);
  }
}

__global__ void gate1_k(double2* A, int cl, int d, int cr, const double2* __restrict__ G) {
  long pairs = (long)cl * cr;
  double2 in[8];
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < pairs; t += (long)gridDim.x * blockDim.x) {
    long l = t % cl, r = t / cl;
    double2* base = A + l + (long)cl * d * r;
    for (int o = 0; o < d; o++) in[o] = base[(long)cl * o];
    for (int o2 = 0; o2 < d; o2++) {
      double2 acc = make_double2(0.0, 0.0);
      for (int o = 0; o < d; o++) acc = cadd(acc, cmul(G[o2 * d + o], in[o]));
      base[(long)cl * o2] = acc;
    }
  }
}

// theta rows (l + cl*o1), cols (o2 + d*r), ld = cl*d
__global__ void gate2_k(double2* th, int cl, int d, int cr, const double2* __restrict__ G) {
  long pairs = (long)cl * cr;
  const long ld = (long)cl * d;
  double2 in[16];
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < pairs; t += (long)gridDim.x * blockDim.x) {
    long l = t % cl, r = t / cl;
    for (int a = 0; a < d; a++)
      for (int b = 0; b < d; b++) in[a * d + b] = th[(l + (long)cl * a) + (b + (long)d * r) * ld];
    for (int a2 = 0; a2 < d; a2++)
      for (int b2 = 0; b2 < d; b2++) {
        double2 acc = make_double2(0.0, 0.0);
        const double2* g = G + (a2 * d + b2) * d * d;
        for (int q = 0; q < d * d; q++) acc = cadd(acc, cmul(g[q], in[q]));
        th[(l + (long)cl * a2) + (b2 + (long)d * r) * ld] = acc;
      }
  }
}

__global__ void transpose_k(const double2* __restrict__ src, long lds, int rows, int cols,
                            double2* __restrict__ dst, long ldd, int conj) {
  __shared__ double2 tile[32][33];
  int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int i = i0 + threadIdx.x, j = j0 + k;
    if (i < rows && j < cols) tile[k][threadIdx.x] = src[i + (long)j * lds];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int j = j0 + threadIdx.x, i = i0 + k;  // dst[j + i*ldd] = src[i + j*lds]
    if (i < rows && j < cols) {
      double2 v = tile[threadIdx.x][k];
      if (conj) v.y = -v.y;
      dst[j + (long)i * ldd] = v;
    }
  }
}

template <typename C>
__global__ void identity_k(C* A, int rows, int cols, long lda) {
  long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % rows, j = t / rows;
    C v; v.x = (i == j) ? 1 : 0; v.y = 0;
    A[i + j * lda] = v;
  }
}

__global__ void z2c_k(const double2* __restrict__ s, long lds, float2* __restrict__ d, long ldd, int rows, int cols) {
  long total = (long)rows * cols;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long i = t % rows, j = t / rows;
    double2 v = s[i + j * lds];
    d[i + j * ldd] = make_float2((float)v.x, (float)v.y);
  }
}

__device__ double block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;  // valid in thread 0
}

__global__ void dist_identity_k(const double2* G, int n, double* out) {
  double acc = 0.0;
  long total = (long)n * n;
  for (long t = threadIdx.x; t < total; t += blockDim.x) {
    long i = t % n, j = t / n;
    double2 v = G[t];
    double re = v.x - (i == j ? 1.0 : 0.0);
    acc += re * re + v.y * v.y;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) out[0] = sqrt(acc);
}

__global__ void dnormalize_k(double* lam, int len) {
  double acc = 0.0;
  for (int t = threadIdx.x; t < len; t += blockDim.x) acc += lam[t] * lam[t];
  acc = block_sum(acc);
  __shared__ double nrm;
  if (threadIdx.x == 0) nrm = sqrt(acc);
  __syncthreads();
  for (int t = threadIdx.x; t < len; t += blockDim.x) lam[t] = lam[t] / nrm;
}

}  // namespace

int zscale_matrix(cudaStream_t s, int M, int N, double2 alpha, double2* C, long ldc, long sC, int batch) {
  if (M <= 0 || N <= 0 || batch <= 0) return QR_OK;
  dim3 g(grid_for((long)M * N), batch);
  scale_matrix_k<<<g, TPB, 0, s>>>(M, N, alpha, C, ldc, sC);
  QR_CHECK_LAUNCH("scale_matrix_k");
  return QR_OK;
}

int zpermute(cudaStream_t s, const double2* src, double2* dst, const Perm& p) {
  long total = 1;
  for (int k = 0; k < p.nd; k++) total *= p.dims[k];
  if (total == 0) return QR_OK;
  // the destination dimension the source stores contiguously
  int a = -1;
  for (int k = 0; k < p.nd; k++)
    if (p.src_stride[k] == 1 && p.dims[k] > 1) a = k;
  if (a > 0 && p.dims[0] > 1) {
    const int ta = p.dims[a] >= 32 ? 32 : (p.dims[a] >= 16 ? 16 : (p.dims[a] >= 8 ? 8 : (p.dims[a] >= 4 ? 4 : 2)));
    const long t0 = PT_ELEMS / ta;
    const long tiles = ((p.dims[0] + t0 - 1) / t0) * ((p.dims[a] + ta - 1) / ta);
    const long nbatch = total / (p.dims[0] * p.dims[a]);
    const long g = std::min<long>(tiles * nbatch, 152L * 8);
    permute_tiled_k<<<(unsigned)g, PT_THREADS, 0, s>>>(src, dst, p, a, ta, nbatch);
    QR_CHECK_LAUNCH("permute_tiled_k");
    return QR_OK;
  }
  permute_k<<<grid_for(total), TPB, 0, s>>>(src, dst, p, total);
  QR_CHECK_LAUNCH("permute_k");
  return QR_OK;
}

int zscale_bond(cudaStream_t s, double2* A, int cl, int d, int cr, const double* lam, int side, int inv, double atol) {
  long total = (long)cl * d * cr;
  if (total == 0) return QR_OK;
  scale_bond_k<<<grid_for(total), TPB, 0, s>>>(A, cl, d, cr, lam, side, inv, atol);
  QR_CHECK_LAUNCH("scale_bond_k");
  return QR_OK;
}

int zgate1(cudaStream_t s, double2* A, int cl, int d, int cr, const double2* G) {
  if (d > 8) return fail(QR_EINVAL, "physical dimension above 8 is not supported");
  long pairs = (long)cl * cr;
  if (pairs == 0) return QR_OK;
  gate1_k<<<grid_for(pairs), TPB, 0, s>>>(A, cl, d, cr, G);
  QR_CHECK_LAUNCH("gate1_k");
  return QR_OK;
}

int zgate2(cudaStream_t s, double2* th, int cl, int d, int cr, const double2* G) {
  if (d > 4) return fail(QR_EINVAL, "two-site gates need physical dimension <= 4");
  long pairs = (long)cl * cr;
  if (pairs == 0) return QR_OK;
  gate2_k<<<grid_for(pairs), TPB, 0, s>>>(th, cl, d, cr, G);
  QR_CHECK_LAUNCH("gate2_k");
  return QR_OK;
}

int ztranspose(cudaStream_t s, const double2* src, long lds, int rows, int cols, double2* dst, long ldd, int conj) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  dim3 g(ceil_div(rows, 32), ceil_div(cols, 32)), b(32, 8);
  transpose_k<<<g, b, 0, s>>>(src, lds, rows, cols, dst, ldd, conj);
  QR_CHECK_LAUNCH("transpose_k");
  return QR_OK;
}

int zset_identity(cudaStream_t s, double2* A, int rows, int cols, long lda) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  identity_k<double2><<<grid_for((long)rows * cols), TPB, 0, s>>>(A, rows, cols, lda);
  QR_CHECK_LAUNCH("identity_k");
  return QR_OK;
}

int cset_identity(cudaStream_t s, float2* A, int rows, int cols, long lda) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  identity_k<float2><<<grid_for((long)rows * cols), TPB, 0, s>>>(A, rows, cols, lda);
  QR_CHECK_LAUNCH("identity_k");
  return QR_OK;
}

int z2c(cudaStream_t s, const double2* src, long lds, float2* dst, long ldd, int rows, int cols) {
  if (rows <= 0 || cols <= 0) return QR_OK;
  z2c_k<<<grid_for((long)rows * cols), TPB, 0, s>>>(src, lds, dst, ldd, rows, cols);
  QR_CHECK_LAUNCH("z2c_k");
  return QR_OK;
}

int zdist_identity(cudaStream_t s, const double2* G, int n, double* out) {
  dist_identity_k<<<1, 1024, 0, s>>>(G, n, out);
  QR_CHECK_LAUNCH("dist_identity_k");
  return QR_OK;
}

int dnormalize(cudaStream_t s, double* lam, int len) {
  if (len <= 0) return QR_OK;
  dnormalize_k<<<1, 1024, 0, s>>>(lam, len);
  QR_CHECK_LAUNCH("dnormalize_k");
  return QR_OK;
}

}  // namespace qr

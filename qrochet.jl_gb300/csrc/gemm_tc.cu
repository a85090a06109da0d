// Split-precision complex GEMM on the Blackwell tensor cores (tcgen05.mma, accumulators in TMEM,
// operand tiles moved by TMA): the contraction kernel of the mixed-precision environment sweeps.
//
//   C[b] = op(A[b]) * op(B[b])        (assignment; FP64 complex in and out)
//
// Two passes:
//  1. split (memory-bound): every FP64 operand element x is rounded to FP32 and split into three
//     BF16 slices x = h + m + l (the 24 bits of fl32(x)), and the complex product is real-ified,
//         [Cr; Ci] = [[Ar, -Ai], [Ai, Ar]] [Br; Bi],
//     so one real GEMM with doubled M and K covers it.  The slices are written once, K-major
//     (K contiguous), as bf16 planes [batch][slice][row][k'] with k' in [0, 2 Kh): the first Kh
//     columns carry the real parts of the complex K index, the next Kh the imaginary parts
//     (Kh = K rounded up to 32, zero padded).  A row tile of 128 real rows holds the real rows
//     of 64 complex rows followed by their imaginary rows, so the accumulator tile maps to one
//     64 x 128 complex output tile.
//  2. GEMM (tensor-bound): a persistent grid, one CTA per SM walking 128 x 128 real output tiles.
//     Warp 0 issues TMA loads of a k-block (64 k' columns: 128-byte rows, 128-byte swizzle) of all
//     three slices of A and B into one of two shared-memory stages; warp 1 issues, per k-block,
//     the six slice products (l h, h l, m m, m h, h m, h h) as tcgen05.mma kind::f16 (BF16 in,
//     FP32 accumulate, M = 128, N = 128, K = 16 per instruction): the five correction products into
//     one TMEM accumulator, the h h product into another; warps 2-9 drain both after every k-block
//     with tcgen05.ld and add them to FP32 registers with round-to-nearest adds.  The tensor
//     cores' own accumulation of the leading term thus spans 4 instructions (64 k'), which keeps
//     the bias of their FP32 accumulation at the level of one add per 64 products.  Two pairs of
//     TMEM accumulators alternate so the drain overlaps the next k-block's MMAs, and the next
//     tile's loads and MMAs run while the epilogue writes the previous tile.  Every wait on an
//     mbarrier is bounded; a timeout sets an error flag, the CTA drains its own copies and MMAs in
//     flight, frees its TMEM and returns.
//
// Result accuracy ~FP32 (relative error ~sqrt(K) 2^-24), at (BF16 rate) / 6 real-product
// throughput: 48 BF16 flops per complex multiply-add.
#include <cuda.h>
#include <cuda_bf16.h>
#include <mutex>
#include "kernels.cuh"
#include "prof.cuh"

namespace qr {

namespace {

constexpr int TC_BM = 128;  // real rows of an output tile (64 complex rows)
constexpr int TC_BN = 128;  // columns of an output tile
constexpr int TC_BK = 64;   // k' columns of a k-block (128-byte bf16 rows)
constexpr int TC_STAGES = 2;
constexpr int TC_TILE = TC_BM * TC_BK * 2;  // bytes of one slice tile (A and B alike: 16 KiB)
constexpr int TC_STAGE = 6 * TC_TILE;        // A h/m/l + B h/m/l
constexpr int TC_THREADS = 320;              // warp 0 TMA, warp 1 MMA + TMEM, warps 2-9 epilogue
constexpr int TC_EPI_WARPS = 8;              // two per TMEM lane quarter, 64 columns each
constexpr int TC_TMEM_COLS = 4 * TC_BN;      // two buffers x (corrections, leading term), FP32
constexpr int TC_SMEM = TC_STAGES * TC_STAGE + 1024 /* alignment */ + 256 /* barriers */;
constexpr unsigned TC_SPIN = 1u << 24;       // polls before a wait gives up (seconds)

// a flag nobody sets: waits that must run to completion (the CTA's own copies and MMAs in flight)
__device__ const uint32_t kNever = 0;

// slice pairs (A slice, B slice) of the six products, small terms first
__constant__ int kPairA[6] = {2, 0, 1, 1, 0, 0};
__constant__ int kPairB[6] = {0, 2, 1, 0, 1, 0};

// ---- PTX helpers ------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// true once the phase with the given parity has completed; false after TC_SPIN polls, or as soon
// as another role of the CTA has given up (abort flag, checked every 256 polls)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const volatile uint32_t* abort_flag) {
  const uint32_t a = smem_u32(bar);
  for (unsigned i = 0; i < TC_SPIN; i++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((i & 255u) == 255u && *abort_flag) return false;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major tile with 128-byte rows and the 128-byte swizzle:
// start address >> 4 (bits 0-13), leading byte offset (unused for this layout: 1), stride byte
// offset = 1024 B between 8-row groups (bits 32-45), descriptor version 1 (bit 46), layout type
// 2 = 128-byte swizzle (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                            ((uint32_t)(TC_BM >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%"
      "19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// ---- pass 1: BF16 slices of the real-ified operands --------------------------------------------
// x is rounded once to FP32 (the only FP64-pipe operation: this part's FP64 rate is 1/64 of FP32)
// and split exactly in FP32: h = bf16(x), m = bf16(x - h), l = bf16(x - h - m); h + m + l carries
// the 24 bits of fl32(x).  Two consecutive k of a row are handled together, so every store is a
// 4-byte bf16 pair.
struct Slices2 {
  __nv_bfloat162 h, m, l;
};
__device__ __forceinline__ Slices2 split3x2(double x0, double x1) {
  const float f0 = __double2float_rn(x0), f1 = __double2float_rn(x1);
  Slices2 r;
  r.h = __floats2bfloat162_rn(f0, f1);
  const float2 hf = __bfloat1622float2(r.h);
  const float a0 = __fsub_rn(f0, hf.x), a1 = __fsub_rn(f1, hf.y);
  r.m = __floats2bfloat162_rn(a0, a1);
  const float2 mf = __bfloat1622float2(r.m);
  r.l = __floats2bfloat162_rn(__fsub_rn(a0, mf.x), __fsub_rn(a1, mf.y));
  return r;
}
__device__ __forceinline__ Slices2 neg(Slices2 v) {
  v.h = __hneg2(v.h);
  v.m = __hneg2(v.m);
  v.l = __hneg2(v.l);
  return v;
}
// the three slices of a bf16 pair at element offset e of plane 0 (planes `plane` elements apart)
__device__ __forceinline__ void put3(__nv_bfloat16* o, long plane, long e, const Slices2& v) {
  *reinterpret_cast<__nv_bfloat162*>(o + e) = v.h;
  *reinterpret_cast<__nv_bfloat162*>(o + plane + e) = v.m;
  *reinterpret_cast<__nv_bfloat162*>(o + 2 * plane + e) = v.l;
}

// A side: elements (i, k), (i, k + 1) of op(A) (M x K) of batch b go to the four real-ified
// positions of their 128-row tile.  One thread per (k pair, i), k fastest.
template <int OPA, class CT>
__global__ void split_a_k(const CT* __restrict__ A, long lda, long sA, int M, int K, int Mp, int Kh,
                          __nv_bfloat16* __restrict__ out) {
  const int b = blockIdx.z;
  const long Kp = 2L * Kh, rows = 2L * Mp;
  const long plane = rows * Kp;
  __nv_bfloat16* o = out + (long)b * 3 * plane;
  A += (long)b * sA;
  const int Kh2 = Kh / 2;
  const long total = (long)Mp * Kh2;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int k = 2 * (int)(t % Kh2), i = (int)(t / Kh2);
    double ar[2] = {0.0, 0.0}, ai[2] = {0.0, 0.0};
#pragma unroll
    for (int u = 0; u < 2; u++) {
      if (i < M && k + u < K) {
        const CT v = (OPA == OP_N || OPA == OP_R) ? A[i + (long)(k + u) * lda] : A[k + u + (long)i * lda];
        ar[u] = v.x;
        ai[u] = (OPA == OP_C || OPA == OP_R) ? -v.y : v.y;
      }
    }
    const long rre = (long)(i / 64) * 128 + (i % 64), rim = rre + 64;
    const Slices2 re = split3x2(ar[0], ar[1]), im = split3x2(ai[0], ai[1]);
    put3(o, plane, rre * Kp + k, re);            // Re row, real block:  Ar
    put3(o, plane, rre * Kp + Kh + k, neg(im));  // Re row, imag block: -Ai
    put3(o, plane, rim * Kp + k, im);            // Im row, real block:  Ai
    put3(o, plane, rim * Kp + Kh + k, re);       // Im row, imag block:  Ar
  }
}

// B side: elements (k, n), (k + 1, n) of op(B) (K x N) go to row n, columns k (real parts) and
// Kh + k (imaginary parts).
template <int OPB, class CT>
__global__ void split_b_k(const CT* __restrict__ B, long ldb, long sB, int K, int N, int Np, int Kh,
                          __nv_bfloat16* __restrict__ out) {
  const int b = blockIdx.z;
  const long Kp = 2L * Kh;
  const long plane = (long)Np * Kp;
  __nv_bfloat16* o = out + (long)b * 3 * plane;
  B += (long)b * sB;
  const int Kh2 = Kh / 2;
  const long total = (long)Np * Kh2;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int k = 2 * (int)(t % Kh2), n = (int)(t / Kh2);
    double br[2] = {0.0, 0.0}, bi[2] = {0.0, 0.0};
#pragma unroll
    for (int u = 0; u < 2; u++) {
      if (n < N && k + u < K) {
        const CT v = (OPB == OP_N || OPB == OP_R) ? B[k + u + (long)n * ldb] : B[n + (long)(k + u) * ldb];
        br[u] = v.x;
        bi[u] = (OPB == OP_C || OPB == OP_R) ? -v.y : v.y;
      }
    }
    put3(o, plane, (long)n * Kp + k, split3x2(br[0], br[1]));
    put3(o, plane, (long)n * Kp + Kh + k, split3x2(bi[0], bi[1]));
  }
}

// ---- pass 2: the tcgen05 GEMM ------------------------------------------------------------------
// Grid (N tiles, M tiles, batch).  nk = k-blocks of 64 k' columns; bplanes = 1 when B is shared by
// the batch (its planes are 0..2), else B's planes of batch b are 3b..3b+2.
// Persistent: CTA b takes the output tiles t = b, b + grid, ... (tile t: column tile t % ntn, row
// tile (t / ntn) % ntm, batch t / (ntn ntm)); the three roles keep one running k-block count g over
// all its tiles, which selects the shared-memory stage (g % 2) and the TMEM accumulator pair
// (g & 1) with their mbarrier phases, so the loads and MMAs of the next tile start while the
// epilogue warps still write the previous tile's C.
__global__ void __launch_bounds__(TC_THREADS, 1)
    zgemm_tc_k(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, double2* __restrict__ C,
               long ldc, long sC, int M, int N, int nk, int bshared, int ntm, int ntn, int batch,
               unsigned* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + TC_STAGES * TC_STAGE);
  uint64_t* full = bars;        // [2] stage loaded
  uint64_t* empty = bars + 2;   // [2] stage consumed by the MMAs
  uint64_t* afull = bars + 4;   // [2] accumulator pair complete for a k-block
  uint64_t* aempty = bars + 6;  // [2] accumulator pair drained by the epilogue
  uint64_t* done = bars + 8;    // all MMAs of the CTA complete
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 9);
  volatile uint32_t* abort_flag = reinterpret_cast<volatile uint32_t*>(bars + 10);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = ntm * ntn * batch;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(afull + i, 1);
      mbar_init(aempty + i, TC_EPI_WARPS);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---- producer: TMA loads of the three slices of A and of B per k-block
      int issued[TC_STAGES] = {0, 0};
      unsigned g = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int tn = t % ntn, tm = (t / ntn) % ntm, b = t / (ntn * ntm);
        const int arow = tm * TC_BM, brow = tn * TC_BN;
        const int aplane = 3 * b, bplane = bshared ? 0 : 3 * b;
        for (int kb = 0; kb < nk; kb++, g++) {
          const int s = g % TC_STAGES;
          const uint32_t ph = (g / TC_STAGES) & 1u;
          if (*abort_flag || !mbar_wait(empty + s, ph ^ 1u, abort_flag)) {
            ok = false;
            break;
          }
          uint8_t* st = smem + s * TC_STAGE;
          mbar_expect_tx(full + s, TC_STAGE);
          for (int sl = 0; sl < 3; sl++) {
            tma_load_3d(st + sl * TC_TILE, &tmA, kb * TC_BK, arow, aplane + sl, full + s);
            tma_load_3d(st + (3 + sl) * TC_TILE, &tmB, kb * TC_BK, brow, bplane + sl, full + s);
          }
          issued[s]++;
        }
      }
      if (!ok) *abort_flag = 1;
      // every copy this thread started has landed before the CTA may exit
      for (int s = 0; s < TC_STAGES; s++)
        if (issued[s] > 0 && !mbar_wait(full + s, (uint32_t)(issued[s] - 1) & 1u, &kNever)) *abort_flag = 1;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer
      bool ok = true;
      unsigned g = 0;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int kb = 0; kb < nk; kb++, g++) {
          const int buf = g & 1u;
          const uint32_t aph = (g >> 1) & 1u;
          if (*abort_flag || !mbar_wait(aempty + buf, aph ^ 1u, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t dt = tmem + (uint32_t)(buf * 2 * TC_BN);  // corrections; + TC_BN: h h
          const int s = g % TC_STAGES;
          const uint32_t ph = (g / TC_STAGES) & 1u;
          if (*abort_flag || !mbar_wait(full + s, ph, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = smem_u32(smem + s * TC_STAGE);
#pragma unroll
          for (int p = 0; p < 6; p++) {
            const uint32_t a0 = st + kPairA[p] * TC_TILE, b0 = st + (3 + kPairB[p]) * TC_TILE;
            const bool lead = p == 5;  // h h
            const uint32_t d = lead ? dt + TC_BN : dt;
#pragma unroll
            for (int j = 0; j < TC_BK / 16; j++) {
              const uint32_t acc = ((!lead && p > 0) || j > 0) ? 1u : 0u;
              tc_mma(d, smem_desc(a0 + 32 * j), smem_desc(b0 + 32 * j), acc);
            }
          }
          tc_commit(empty + s);   // the stage is free once these MMAs have read it
          tc_commit(afull + buf);  // and the accumulator pair holds this k-block's products
        }
      }
      if (!ok) *abort_flag = 1;
      // all MMAs issued by this thread complete before the TMEM is released
      tc_commit(done);
      if (!mbar_wait(done, 0, &kNever)) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows of the output tile) and
    // the 64 columns of half (w - 2) / 4 of the accumulator
    const int q = warp & 3, half = (warp - 2) >> 2;
    constexpr int EC = TC_BN / 2;
    const int r = 32 * q + lane;
    bool ok = true;
    unsigned g = 0;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const int tn = t % ntn, tm = (t / ntn) % ntm, b = t / (ntn * ntm);
      float acc[EC];
#pragma unroll
      for (int j = 0; j < EC; j++) acc[j] = 0.f;
      for (int kb = 0; kb < nk; kb++, g++) {
        const int buf = g & 1u;
        const uint32_t aph = (g >> 1) & 1u;
        // lane 0 waits and the warp follows its verdict, so the warp-wide TMEM loads stay convergent
        int got = 0;
        if (lane == 0) got = (!*abort_flag && mbar_wait(afull + buf, aph, abort_flag)) ? 1 : 0;
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) { ok = false; break; }
        tc_fence_after();
        const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(buf * 2 * TC_BN + half * EC);
#pragma unroll
        for (int j = 0; j < EC / 32; j++) {
          float v[32], w[32];
          tmem_ld32(ta + 32 * j, v);          // corrections
          tmem_ld32(ta + TC_BN + 32 * j, w);  // leading term
#pragma unroll
          for (int i = 0; i < 32; i++) acc[32 * j + i] = __fadd_rn(acc[32 * j + i], __fadd_rn(w[i], v[i]));
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(aempty + buf);
      }
      if (!ok) break;
      // row r < 64: real part of complex row m0 + r; r >= 64: imaginary part of m0 + r - 64
      const int part = r >= 64;
      const int gi = tm * 64 + (r & 63);
      double* Cd = reinterpret_cast<double*>(C + (long)b * sC);
      if (gi < M) {
#pragma unroll
        for (int j = 0; j < EC; j++) {
          const int gj = tn * TC_BN + half * EC + j;
          if (gj < N) Cd[2 * (gi + (long)gj * ldc) + part] = (double)acc[j];
        }
      }
    }
    if (!ok) *abort_flag = 1;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, 1u);
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// ---- host side ----------------------------------------------------------------------------------
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_fn(EncodeTiled* out) {
  static std::mutex mu;
  static EncodeTiled fn = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
      return fail(QR_ECUDA, "cuTensorMapEncodeTiled is not available from the CUDA driver");
    fn = reinterpret_cast<EncodeTiled>(p);
  }
  *out = fn;
  return QR_OK;
}

// bf16 planes [planes][rows][Kp] with a 64 x 128 box and the 128-byte swizzle
int make_map(CUtensorMap* map, const void* base, long Kp, long rows, long planes) {
  EncodeTiled enc = nullptr;
  QR_TRY(encode_fn(&enc));
  cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)(Kp * 2), (cuuint64_t)(Kp * 2 * rows)};
  cuuint32_t box[3] = {TC_BK, 128, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(QR_ECUDA, "cuTensorMapEncodeTiled failed (code " + std::to_string((int)r) + ")");
  return QR_OK;
}

}  // namespace

// Bytes of the split workspace zgemm_tc needs for these shapes.
size_t zgemm_tc_workspace(int M, int N, int K, int batch, bool bshared) {
  const long Mp = (M + 63) / 64 * 64, Np = (N + TC_BN - 1) / TC_BN * TC_BN, Kh = (K + 31) / 32 * 32;
  const size_t a = (size_t)batch * 3 * (2 * Mp) * (2 * Kh) * 2;
  const size_t bb = (size_t)(bshared ? 1 : batch) * 3 * Np * (2 * Kh) * 2;
  return a + bb + 256;
}

// complex FP64 (double2) or FP32 (float2) operands; the split passes round to FP32 either way
template <class CT>
static int zgemm_tc_t(cudaStream_t s, int opA, int opB, int M, int N, int K, const CT* A, long lda, long sA,
                      const CT* B, long ldb, long sB, double2* C, long ldc, long sC, int batch, void* ws,
                      unsigned* err) {
  if (M <= 0 || N <= 0 || batch <= 0) return QR_OK;
  if (K <= 0) return zscale_matrix(s, M, N, make_double2(0.0, 0.0), C, ldc, sC, batch);
  const bool bshared = sB == 0;
  const int Mp = (M + 63) / 64 * 64, Np = (N + TC_BN - 1) / TC_BN * TC_BN, Kh = (K + 31) / 32 * 32;
  const long Kp = 2L * Kh;
  __nv_bfloat16* as = static_cast<__nv_bfloat16*>(ws);
  const size_t abytes = (size_t)batch * 3 * (2L * Mp) * Kp * 2;
  __nv_bfloat16* bs = reinterpret_cast<__nv_bfloat16*>(static_cast<uint8_t*>(ws) + (abytes + 255) / 256 * 256);
  const double fl = 8.0 * M * N * (double)K * batch;  // complex-equivalent flops
  const double by = 16.0 * ((double)M * K + (double)K * N + (double)M * N) * batch;
  int pr = prof_begin(s, PK_ZGEMM_SPLIT, fl, by);
  {
    const long ta = (long)Mp * (Kh / 2);
    dim3 g((unsigned)std::min<long>((ta + 255) / 256, 152 * 16), 1, batch);
    switch (opA) {
      case OP_N: split_a_k<OP_N, CT><<<g, 256, 0, s>>>(A, lda, sA, M, K, Mp, Kh, as); break;
      case OP_T: split_a_k<OP_T, CT><<<g, 256, 0, s>>>(A, lda, sA, M, K, Mp, Kh, as); break;
      case OP_C: split_a_k<OP_C, CT><<<g, 256, 0, s>>>(A, lda, sA, M, K, Mp, Kh, as); break;
      case OP_R: split_a_k<OP_R, CT><<<g, 256, 0, s>>>(A, lda, sA, M, K, Mp, Kh, as); break;
      default: return fail(QR_EINVAL, "zgemm_tc: bad opA");
    }
    QR_CHECK_LAUNCH("split_a_k");
    const long tb = (long)Np * (Kh / 2);
    dim3 gb((unsigned)std::min<long>((tb + 255) / 256, 152 * 16), 1, bshared ? 1 : batch);
    switch (opB) {
      case OP_N: split_b_k<OP_N, CT><<<gb, 256, 0, s>>>(B, ldb, sB, K, N, Np, Kh, bs); break;
      case OP_T: split_b_k<OP_T, CT><<<gb, 256, 0, s>>>(B, ldb, sB, K, N, Np, Kh, bs); break;
      case OP_C: split_b_k<OP_C, CT><<<gb, 256, 0, s>>>(B, ldb, sB, K, N, Np, Kh, bs); break;
      case OP_R: split_b_k<OP_R, CT><<<gb, 256, 0, s>>>(B, ldb, sB, K, N, Np, Kh, bs); break;
      default: return fail(QR_EINVAL, "zgemm_tc: bad opB");
    }
    QR_CHECK_LAUNCH("split_b_k");
  }
  CUtensorMap ma, mb;
  QR_TRY(make_map(&ma, as, Kp, 2L * Mp, 3L * batch));
  QR_TRY(make_map(&mb, bs, Kp, Np, 3L * (bshared ? 1 : batch)));
  QR_TRY(set_func_attr_once((const void*)zgemm_tc_k, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
  const int ntn = Np / TC_BN, ntm = Mp / 64;
  const long ntiles = (long)ntn * ntm * batch;
  int sms = 0;
  QR_TRY(device_sm_count(&sms));
  const int grid = (int)std::min<long>(ntiles, sms);  // one CTA per SM (its shared memory allows no more)
  const int nk = (int)(Kp / TC_BK);
  zgemm_tc_k<<<grid, TC_THREADS, TC_SMEM, s>>>(ma, mb, C, ldc, sC, M, N, nk, bshared ? 1 : 0, ntm, ntn, batch, err);
  QR_CHECK_LAUNCH("zgemm_tc_k");
  prof_end(s, pr);
  return QR_OK;
}

int zgemm_tc(cudaStream_t s, int opA, int opB, int M, int N, int K, const double2* A, long lda, long sA,
             const double2* B, long ldb, long sB, double2* C, long ldc, long sC, int batch, void* ws,
             unsigned* err) {
  return zgemm_tc_t<double2>(s, opA, opB, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, ws, err);
}
int zgemm_tc(cudaStream_t s, int opA, int opB, int M, int N, int K, const float2* A, long lda, long sA,
             const float2* B, long ldb, long sB, double2* C, long ldc, long sC, int batch, void* ws,
             unsigned* err) {
  return zgemm_tc_t<float2>(s, opA, opB, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, ws, err);
}

}  // namespace qr

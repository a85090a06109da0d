// Opt-in per-kernel-class timing with CUDA events on the launching stream, plus pinned host
// buffers.  Used by the benchmark to measure the dominant kernel's average launch duration and
// its algorithmic work over a run; disabled (zero cost beyond a flag test) otherwise.
#include <vector>
#include <mutex>
#include "prof.cuh"

namespace qr {

namespace {
struct Rec {
  int kind;
  double flops, bytes;
  cudaEvent_t e0, e1;
  uint64_t units;  // launches (or Jacobi sweeps) the record covers
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

bool prof_on() { return g_on; }

int prof_begin(cudaStream_t s, int kind, double flops, double bytes) {
  if (!g_on) return -1;
  std::lock_guard<std::mutex> lk(g_mu);
  Rec r{kind, flops, bytes, take_event(), take_event(), 1};
  cudaEventRecord(r.e0, s);
  g_recs.push_back(r);
  return (int)g_recs.size() - 1;
}

void prof_end(cudaStream_t s, int idx) {
  if (idx < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (idx < (int)g_recs.size()) cudaEventRecord(g_recs[idx].e1, s);
}

void prof_account(int idx, double flops, double bytes, long units) {
  if (idx < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (idx < (int)g_recs.size()) {
    g_recs[idx].flops = flops;
    g_recs[idx].bytes = bytes;
    if (units >= 0) g_recs[idx].units = (uint64_t)units;
  }
}

}  // namespace qr

using namespace qr;

namespace qr_probe {
constexpr int PROBE_ITERS = 2048;
__global__ void probe_dmma_k(double* out, double a) {
  double c0[2] = {0, 0}, c1[2] = {0, 0}, c2[2] = {0, 0}, c3[2] = {0, 0};
  double av = a * threadIdx.x, bv = a + threadIdx.x;
  for (int i = 0; i < PROBE_ITERS; i++) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(c0[0]), "+d"(c0[1]) : "d"(av), "d"(bv));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(c1[0]), "+d"(c1[1]) : "d"(av), "d"(bv));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(c2[0]), "+d"(c2[1]) : "d"(av), "d"(bv));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(c3[0]), "+d"(c3[1]) : "d"(av), "d"(bv));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0[0] + c0[1] + c1[0] + c1[1] + c2[0] + c2[1] + c3[0] + c3[1];
}
template <typename T>
__global__ void probe_fma_k(T* out, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < PROBE_ITERS; i++) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace qr_probe
using namespace qr_probe;

extern "C" {

// Peak rate of one arithmetic pipe, measured now on the current device: kind 0 = FP64 tensor
// (mma.sync m8n8k4 f64), 1 = FP32 FFMA, 2 = FP64 DFMA.  Best of three timed launches.
int qr_probe_peak(int kind, double* tflops) try {
  if (!tflops || kind < 0 || kind > 2) return fail(QR_EINVAL, "bad probe kind");
  int dev = 0, sms = 0;
  QR_CUDA(cudaGetDevice(&dev));
  QR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  const size_t nthr = (size_t)blocks * threads;
  void* out = nullptr;
  QR_CUDA(cudaMalloc(&out, nthr * sizeof(double)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0);
    if (kind == 0) probe_dmma_k<<<blocks, threads>>>((double*)out, 1e-3);
    else if (kind == 1) probe_fma_k<float><<<blocks, threads>>>((float*)out, 0.999f, 1e-3f);
    else probe_fma_k<double><<<blocks, threads>>>((double*)out, 0.999, 1e-3);
    count_launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double flops = (kind == 0) ? 2.0 * 256 * 4 * PROBE_ITERS * (double)(nthr / 32) : 2.0 * 8 * PROBE_ITERS * (double)nthr;
    double tf = flops / (ms * 1e-3) / 1e12;
    if (rep > 0 && tf > best) best = tf;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  QR_CUDA(cudaGetLastError());
  *tflops = best;
  return QR_OK;
} QR_ABI_CATCH

int qr_prof_enable(int on) try {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_recs) {
    g_pool.push_back(r.e0);
    g_pool.push_back(r.e1);
  }
  g_recs.clear();
  g_on = on != 0;
  return QR_OK;
} QR_ABI_CATCH

int qr_prof_read(int kind, double* ms, uint64_t* launches, double* flops, double* bytes) try {
  QR_CUDA(cudaDeviceSynchronize());
  std::lock_guard<std::mutex> lk(g_mu);
  double t = 0, f = 0, b = 0;
  uint64_t c = 0;
  for (auto& r : g_recs) {
    if (r.kind != kind) continue;
    float x = 0;
    if (cudaEventElapsedTime(&x, r.e0, r.e1) == cudaSuccess) t += x;
    f += r.flops;
    b += r.bytes;
    c += r.units;
  }
  if (ms) *ms = t;
  if (launches) *launches = c;
  if (flops) *flops = f;
  if (bytes) *bytes = b;
  return QR_OK;
} QR_ABI_CATCH

int qr_host_alloc(uint64_t bytes, void** ptr) try {
  if (!ptr) return fail(QR_EINVAL, "null output");
  QR_CUDA(cudaHostAlloc(ptr, bytes ? bytes : 16, cudaHostAllocDefault));
  return QR_OK;
} QR_ABI_CATCH

int qr_host_free(void* ptr) try {
  if (ptr) QR_CUDA(cudaFreeHost(ptr));
  return QR_OK;
} QR_ABI_CATCH

}  // extern "C"

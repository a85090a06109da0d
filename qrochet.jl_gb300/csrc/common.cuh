// Shared device/host helpers for the qrochet GB300 library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cmath>
#include <string>
#include <atomic>
#include <exception>
#include <new>

#include "../../include/qrochet_gpu.h"
#include "../../include/qrochet_gpu_testing.h"

namespace qr {

// ---- complex arithmetic on CUDA vector types (re = .x, im = .y) ------------------------------
template <typename T> struct cplx;
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<float> { using type = float2; };
template <typename T> using cplx_t = typename cplx<T>::type;

__host__ __device__ inline double2 mk(double r, double i) { return make_double2(r, i); }
__host__ __device__ inline float2 mk(float r, float i) { return make_float2(r, i); }
template <typename C> __host__ __device__ inline C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ inline C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __host__ __device__ inline C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// conj(a) * b
template <typename C> __host__ __device__ inline C cmulc(C a, C b) {
  C r; r.x = a.x * b.x + a.y * b.y; r.y = a.x * b.y - a.y * b.x; return r;
}
template <typename C> __host__ __device__ inline C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }
template <typename C, typename T> __host__ __device__ inline C cscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }

// ---- error plumbing ----------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Page-locked host scratch owned by the calling thread, for the small device-to-host reads on the
// hot path (sweep counters, singular values, a scalar result).  A read into pageable memory goes
// through the CUDA driver's staging buffer after the stream's earlier kernels; with many chains served
// by concurrent threads those reads serialise.  Valid until the thread's next call; nullptr if the
// allocation fails.
void* host_scratch(size_t bytes);

// Launch-configuration caches for the current device, safe to call from concurrent threads (the
// request server's workers): the SM count, a kernel's resident blocks per SM at a block size and
// dynamic shared-memory size, and function attributes set once per device (CUDA keeps them per
// device context).
int device_sm_count(int* out);
int blocks_per_sm(const void* func, int threads, size_t smem, int* out);
int set_func_attr_once(const void* func, cudaFuncAttribute attr, int value);

extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define QR_CUDA(call)                                        \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return ::qr::cuda_fail(_e, #call); \
  } while (0)

#define QR_CHECK_LAUNCH(what)                                   \
  do {                                                          \
    ::qr::count_launch();                                       \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return ::qr::cuda_fail(_e, what);    \
  } while (0)

// Every exported function is a function-try-block ending in QR_ABI_CATCH: a C++ exception (a
// failed host allocation, a thread or lock that cannot be created) becomes a status code and the
// thread's error message instead of unwinding into the caller's C, Julia or Python frames.
#define QR_ABI_CATCH                                                                              \
  catch (const std::bad_alloc&) {                                                                 \
    return ::qr::fail(QR_ENOMEM, "host memory allocation failed");                                \
  }                                                                                               \
  catch (const std::exception& _x) {                                                              \
    return ::qr::fail(QR_EHOST, std::string("host-side failure: ") + _x.what());                  \
  }                                                                                               \
  catch (...) {                                                                                   \
    return ::qr::fail(QR_EHOST, "host-side failure");                                             \
  }

#define QR_TRY(expr)              \
  do {                            \
    int _s = (expr);              \
    if (_s != QR_OK) return _s;   \
  } while (0)

inline unsigned ceil_div(long a, long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace qr

// C ABI of the GB300 Chain path: a device-resident open-boundary MPS (qr_chain) and MPO
// (qr_mpo), and the drivers of the reference's methods on them.
//
// Device layout: site i is a column-major (chi_l, d, chi_r) array with chi_l fastest, so both
// groupings the reference factorises are plain column-major matrices: [(l,o) x r] (ld chi_l*d)
// for direction=:right and [l x (o,r)] (ld chi_l) for direction=:left.  The two-site block
// theta[(l,o1) x (o2,r)] is then one GEMM of neighbouring sites, and its SVD factors U and Vh
// are directly the new site tensors.  The open ends carry bonds of size 1.  Lambda vectors live
// in their own device buffers, one per bond that holds one (the reference keeps them as
// separate hyperindex tensors on the bond, src/Ansatz/Chain.jl:338).
#include <vector>
#include <cstdio>
#include <string>
#include <complex>
#include <cstring>
#include <cmath>
#include <cstdlib>
#include <algorithm>
#include <mutex>
#include <map>
#include <tuple>
#include <thread>
#include <system_error>
#include "kernels.cuh"

namespace qr {

static thread_local std::string t_err;
std::atomic<uint64_t> g_launches{0};

void set_error(const std::string& msg) { t_err = msg; }

struct HostScratch {
  void* p = nullptr;
  size_t cap = 0;
  ~HostScratch() {
    if (p) cudaFreeHost(p);
  }
};
static thread_local HostScratch t_scratch;

static std::mutex g_cfg_mu;
static std::map<int, int> g_sms;
static std::map<std::tuple<int, const void*, int, size_t>, int> g_occ;
static std::map<std::tuple<int, const void*, int>, int> g_attr;

int device_sm_count(int* out) {
  int dev = 0;
  QR_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  auto it = g_sms.find(dev);
  if (it == g_sms.end()) {
    int v = 0;
    QR_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    it = g_sms.emplace(dev, v).first;
  }
  *out = it->second;
  return QR_OK;
}

int blocks_per_sm(const void* func, int threads, size_t smem, int* out) {
  int dev = 0;
  QR_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  const auto key = std::make_tuple(dev, func, threads, smem);
  auto it = g_occ.find(key);
  if (it == g_occ.end()) {
    int v = 0;
    QR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, func, threads, smem));
    it = g_occ.emplace(key, v).first;
  }
  *out = it->second;
  return QR_OK;
}

int set_func_attr_once(const void* func, cudaFuncAttribute attr, int value) {
  int dev = 0;
  QR_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  const auto key = std::make_tuple(dev, func, (int)attr);
  auto it = g_attr.find(key);
  if (it != g_attr.end() && it->second == value) return QR_OK;
  QR_CUDA(cudaFuncSetAttribute(func, attr, value));
  g_attr[key] = value;
  return QR_OK;
}

void* host_scratch(size_t bytes) {
  if (bytes > t_scratch.cap) {
    if (t_scratch.p) cudaFreeHost(t_scratch.p);
    t_scratch.p = nullptr;
    t_scratch.cap = 0;
    const size_t want = std::max<size_t>(bytes + bytes / 2, 4096);
    if (cudaMallocHost(&t_scratch.p, want) != cudaSuccess) {
      t_scratch.p = nullptr;
      return nullptr;
    }
    t_scratch.cap = want;
  }
  return t_scratch.p;
}
int fail(int code, const std::string& msg) {
  t_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  t_err = std::string(what) + ": " + cudaGetErrorString(e);
  return (e == cudaErrorMemoryAllocation) ? QR_ENOMEM
         : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? QR_ENODEV
                                                                        : QR_ECUDA;
}

static std::once_flag g_pool_once;
static void init_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    // Chains run concurrently on their own streams (the request server's workers).  Memory freed
    // on one stream is only reused by another once the free has completed, instead of through an
    // inserted cross-stream dependency that would chain the workers' streams together.
    int off = 0;
    cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &off);
    cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowOpportunistic, &off);
  }
}

}  // namespace qr

using namespace qr;

struct qr_chain {
  int n = 0, d = 0, precision = QR_FP64;
  bool periodic = false;          // Periodic boundary: bd[n-1] is the bond between site n and site 1
  cudaStream_t stream = nullptr;
  std::vector<int> bd;            // n-1 bond sizes
  std::vector<double2*> site;     // n site tensors
  std::vector<double*> lam;       // n-1 Lambda vectors or nullptr
  std::vector<int> lamlen;
  SvdWork* svd = nullptr;
  double2* gate = nullptr;        // d^4 complex scratch for gate matrices
  double2* gate_host = nullptr;   // pinned staging for gate uploads (async H2D)
  double2* ws = nullptr;          // theta / factorisation workspace
  size_t ws_cap = 0;
  double* scal = nullptr;         // small device scalars
  // execution lanes of qr_evolve_layer: chains that own only a stream and workspaces (the
  // fields above from `svd` on); their bookkeeping vectors are filled from this chain per layer
  std::vector<qr_chain*> lanes;
  bool is_lane = false;
  int cl(int i) const { return i == 0 ? (periodic ? bd[n - 1] : 1) : bd[i - 1]; }
  int cr(int i) const { return i == n - 1 ? (periodic ? bd[n - 1] : 1) : bd[i]; }
  size_t elems(int i) const { return (size_t)cl(i) * d * cr(i); }
};

struct qr_mpo {
  int n = 0, d = 0;
  std::vector<int> bd;
  std::vector<double2*> site;  // (wl, o, i, wr), wl fastest
  // host copies of the site tensors, read back once for the sparse mixing tables (see env_sweep)
  // and dropped by every upload
  mutable std::vector<std::vector<double2>> host_w;
  mutable bool host_ok = false;
  int wl(int i) const { return i == 0 ? 1 : bd[i - 1]; }
  int wr(int i) const { return i == n - 1 ? 1 : bd[i]; }
};

namespace {

int cuda_ok(cudaError_t e, const char* what) { return e == cudaSuccess ? QR_OK : cuda_fail(e, what); }

int dalloc(void** p, size_t bytes, cudaStream_t s) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) return fail(QR_ENOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
  return QR_OK;
}

int ensure_ws(qr_chain* h, size_t elems) {
  if (elems <= h->ws_cap) return QR_OK;
  if (h->ws) cudaFreeAsync(h->ws, h->stream);
  h->ws = nullptr;
  h->ws_cap = 0;
  size_t want = elems + elems / 4 + 64;
  QR_TRY(dalloc((void**)&h->ws, want * sizeof(double2), h->stream));
  h->ws_cap = want;
  return QR_OK;
}

// replace site i's buffer (frees the old one on the chain's stream)
void set_site(qr_chain* h, int i, double2* p) {
  if (h->site[i] && h->site[i] != p) cudaFreeAsync(h->site[i], h->stream);
  h->site[i] = p;
}

void drop_lambda(qr_chain* h, int b) {
  if (h->lam[b]) cudaFreeAsync(h->lam[b], h->stream);
  h->lam[b] = nullptr;
  h->lamlen[b] = 0;
}

// Bond b gets Lambda = the first len entries of src (device); src is copied.
int put_lambda(qr_chain* h, int b, const double* src, int len) {
  double* p = nullptr;
  QR_TRY(dalloc((void**)&p, sizeof(double) * len, h->stream));
  QR_CUDA(cudaMemcpyAsync(p, src, sizeof(double) * len, cudaMemcpyDeviceToDevice, h->stream));
  drop_lambda(h, b);
  h->lam[b] = p;
  h->lamlen[b] = len;
  return QR_OK;
}

// Gates are staged through a pinned buffer so the copy does not wait for the stream; every
// entry point synchronises before returning, so the buffer is free again on the next call.
int upload_gate(qr_chain* h, const double* g, int dim) {
  std::memcpy(h->gate_host, g, sizeof(double2) * dim * dim);
  QR_CUDA(cudaMemcpyAsync(h->gate, h->gate_host, sizeof(double2) * dim * dim, cudaMemcpyHostToDevice, h->stream));
  return QR_OK;
}

// filter the 3/4-letter order like the reference does for open ends
std::string filtered(const char* order, bool first, bool last) {
  std::string o(order ? order : "");
  std::string out;
  for (char c : o) {
    if (first && c == 'l') continue;
    if (last && c == 'r') continue;
    out.push_back(c);
  }
  return out;
}

bool is_perm(const std::string& o, const char* letters) {
  std::string a = o, b = letters;
  if (a.size() != b.size()) return false;
  for (char c : b)
    if (a.find(c) == std::string::npos) return false;
  return true;
}

// Perm that maps a host column-major array with dims named by `hord` into the internal layout
// `iord` (dims `idims` by letter).
Perm make_perm(const std::string& hord, const std::string& iord, const long* idims_by_iord) {
  // host strides by letter
  long stride[8] = {0};
  char letters[8];
  int nl = 0;
  long acc = 1;
  for (char c : hord) {
    long dim = 1;
    for (size_t k = 0; k < iord.size(); k++)
      if (iord[k] == c) dim = idims_by_iord[k];
    letters[nl] = c;
    stride[nl++] = acc;
    acc *= dim;
  }
  Perm p;
  p.nd = (int)iord.size();
  for (size_t k = 0; k < iord.size(); k++) {
    p.dims[k] = idims_by_iord[k];
    p.src_stride[k] = 0;
    for (int q = 0; q < nl; q++)
      if (letters[q] == iord[k]) p.src_stride[k] = stride[q];
  }
  return p;
}

inline int svd_mode(const qr_chain* h) { return (h->precision & QR_MIXED) ? QR_MIXED : QR_FP64; }

int check_site(const qr_chain* h, int i) {
  if (!h) return fail(QR_EINVAL, "null chain");
  if (i < 0 || i >= h->n) return fail(QR_EINVAL, "site out of range");
  return QR_OK;
}

// ---- canonize_site! (Chain.jl:339-376) ---------------------------------------------------------
// Canonical forms exist for Open chains only (src/Ansatz/Chain.jl:339,469,509 dispatch on ::Open).
// truncate! may slice a bond to an empty extent (Chain.jl:404-419): the chain then holds a size-0
// bond, i.e. the null state.  Contractions of such a chain are 0; factorisations and gates refuse.
bool has_empty_bond(const qr_chain* h) {
  for (int b : h->bd)
    if (b == 0) return true;
  return false;
}
int require_nonempty(const qr_chain* h) {
  if (h && has_empty_bond(h))
    return fail(QR_EINVAL, "the chain holds a bond of size 0 (truncate! kept no singular value): it is the null "
                           "state");
  return QR_OK;
}

int require_open(const qr_chain* h) {
  return h->periodic ? fail(QR_EINVAL, "canonical forms are defined for Open chains only") : QR_OK;
}

int canonize_site_impl(qr_chain* h, int i, int dir, int method) {
  QR_TRY(require_nonempty(h));
  QR_TRY(require_open(h));
  QR_TRY(check_site(h, i));
  if (dir == QR_DIR_LEFT) {
    if (i == 0) return fail(QR_EINVAL, "Cannot right-canonize left-most tensor");
  } else if (dir == QR_DIR_RIGHT) {
    if (i == h->n - 1) return fail(QR_EINVAL, "Cannot left-canonize right-most tensor");
  } else {
    return fail(QR_EINVAL, "Unknown direction");
  }
  if (method != QR_METHOD_QR && method != QR_METHOD_SVD) return fail(QR_EINVAL, "Unknown factorization method");
  cudaStream_t s = h->stream;
  const int d = h->d, cl = h->cl(i), cr = h->cr(i);
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  if (dir == QR_DIR_RIGHT) {
    const int m = cl * d, nn = cr, k = m < nn ? m : nn;
    const int cr2 = h->cr(i + 1);
    // ws: [M copy (m*nn)] [R or Vh (k*nn)] [S (k doubles)] [tau (k)]
    QR_TRY(ensure_ws(h, (size_t)m * nn + (size_t)k * nn + k + k));
    double2* W = h->ws;
    double2* Rr = W + (size_t)m * nn;
    double* S = (double*)(Rr + (size_t)k * nn);
    double2* tau = Rr + (size_t)k * nn + k;
    double2* Q = nullptr;
    QR_TRY(dalloc((void**)&Q, sizeof(double2) * (size_t)m * k, s));
    if (method == QR_METHOD_QR) {
      QR_CUDA(cudaMemcpyAsync(W, h->site[i], sizeof(double2) * (size_t)m * nn, cudaMemcpyDeviceToDevice, s));
      QR_TRY(zqr_thin(s, W, m, nn, m, Q, m, Rr, k, tau));
    } else {
      QR_TRY(zsvd_thin(s, h->svd, svd_mode(h), h->site[i], m, nn, m, Q, m, S, Rr, k));
    }
    // next site <- R diag(Lambda_i) A_{i+1}
    double2* nxt = nullptr;
    QR_TRY(dalloc((void**)&nxt, sizeof(double2) * (size_t)k * d * cr2, s));
    QR_TRY(zgemm(s, OP_N, OP_N, k, d * cr2, cr, one, Rr, k, 0, h->site[i + 1], cr, 0, zero, nxt, k, 0, 1,
                 h->lam[i]));
    set_site(h, i, Q);
    set_site(h, i + 1, nxt);
    h->bd[i] = k;
    drop_lambda(h, i);
    if (method == QR_METHOD_SVD) QR_TRY(put_lambda(h, i, S, k));
  } else {
    const int m = d * cr, nn = cl, k = m < nn ? m : nn;
    const int cl0 = h->cl(i - 1);
    // ws: [M = A^T (m*nn)] [Q (m*k)] [R or Vh (k*nn)] [S] [tau]
    QR_TRY(ensure_ws(h, (size_t)m * nn + (size_t)m * k + (size_t)k * nn + k + k));
    double2* W = h->ws;
    double2* Q = W + (size_t)m * nn;
    double2* Rr = Q + (size_t)m * k;
    double* S = (double*)(Rr + (size_t)k * nn);
    double2* tau = Rr + (size_t)k * nn + k;
    QR_TRY(ztranspose(s, h->site[i], cl, cl, d * cr, W, m, 0));  // M[(o,r), l] = A[l, (o,r)]
    if (method == QR_METHOD_QR) {
      QR_TRY(zqr_thin(s, W, m, nn, m, Q, m, Rr, k, tau));
    } else {
      QR_TRY(zsvd_thin(s, h->svd, svd_mode(h), W, m, nn, m, Q, m, S, Rr, k));
    }
    double2* cur = nullptr;
    QR_TRY(dalloc((void**)&cur, sizeof(double2) * (size_t)k * m, s));
    QR_TRY(ztranspose(s, Q, m, m, k, cur, k, 0));  // new site [k x (o,r)] = Q^T
    double2* prv = nullptr;
    QR_TRY(dalloc((void**)&prv, sizeof(double2) * (size_t)cl0 * d * k, s));
    // prev <- A_{i-1} diag(Lambda_{i-1}) R^T
    QR_TRY(zgemm(s, OP_N, OP_T, cl0 * d, k, cl, one, h->site[i - 1], cl0 * d, 0, Rr, k, 0, zero, prv, cl0 * d,
                 0, 1, h->lam[i - 1]));
    set_site(h, i, cur);
    set_site(h, i - 1, prv);
    h->bd[i - 1] = k;
    drop_lambda(h, i - 1);
    if (method == QR_METHOD_SVD) QR_TRY(put_lambda(h, i - 1, S, k));
  }
  return QR_OK;
}

int scale_site_by_lambda(qr_chain* h, int i, int side, const double* lam, int inv, double atol) {
  return zscale_bond(h->stream, h->site[i], h->cl(i), h->d, h->cr(i), lam, side, inv, atol);
}

// ---- truncate! (Chain.jl:390-422) -------------------------------------------------------------
int truncate_impl(qr_chain* h, int s1, int s2, double threshold, int maxdim) {
  if (!h) return fail(QR_EINVAL, "null chain");
  if (s2 != s1 + 1 || s1 < 0 || s2 >= h->n) return fail(QR_EINVAL, "Invalid bond");
  const int b = s1;
  if (!h->lam[b]) return fail(QR_ENO_SCHMIDT, "Can't access the spectrum on bond");
  const int dim = h->lamlen[b];
  double* hl = static_cast<double*>(host_scratch(sizeof(double) * dim));
  if (!hl) return fail(QR_ENOMEM, "page-locked host scratch");
  QR_CUDA(cudaMemcpyAsync(hl, h->lam[b], sizeof(double) * dim, cudaMemcpyDeviceToHost, h->stream));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  const std::vector<double> lam(hl, hl + dim);
  int upto = (maxdim >= 0) ? (maxdim < dim ? maxdim : dim) : dim;
  if (std::isnan(threshold)) threshold = 1e-16;
  std::vector<int> keep;
  for (int k = 0; k < upto; k++)
    if (std::fabs(lam[k]) > threshold) keep.push_back(k);
  const int nk = (int)keep.size();
  if (dim == 0) return QR_OK;  // already empty
  if (nk == 0) {
    // slice! to an empty extent: the bond keeps size 0, both sites hold no entries, Lambda is empty
    double2 *a = nullptr, *c = nullptr;
    double* nl = nullptr;
    QR_TRY(dalloc((void**)&a, 0, h->stream));
    QR_TRY(dalloc((void**)&c, 0, h->stream));
    QR_TRY(dalloc((void**)&nl, 0, h->stream));
    set_site(h, s1, a);
    set_site(h, s2, c);
    drop_lambda(h, b);
    h->lam[b] = nl;
    h->lamlen[b] = 0;
    h->bd[b] = 0;
    return QR_OK;
  }
  bool prefix = true;
  for (int k = 0; k < nk; k++) prefix = prefix && (keep[k] == k);
  if (nk == dim) return QR_OK;
  cudaStream_t s = h->stream;
  const int d = h->d, cl = h->cl(s1), cr2 = h->cr(s2);
  double2 *a = nullptr, *c = nullptr;
  QR_TRY(dalloc((void**)&a, sizeof(double2) * (size_t)cl * d * nk, s));
  QR_TRY(dalloc((void**)&c, sizeof(double2) * (size_t)nk * d * cr2, s));
  double* nl = nullptr;
  QR_TRY(dalloc((void**)&nl, sizeof(double) * nk, s));
  if (prefix) {
    QR_CUDA(cudaMemcpyAsync(a, h->site[s1], sizeof(double2) * (size_t)cl * d * nk, cudaMemcpyDeviceToDevice, s));
    QR_CUDA(cudaMemcpy2DAsync(c, sizeof(double2) * nk, h->site[s2], sizeof(double2) * dim, sizeof(double2) * nk,
                              (size_t)d * cr2, cudaMemcpyDeviceToDevice, s));
    QR_CUDA(cudaMemcpyAsync(nl, h->lam[b], sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
  } else {
    for (int k = 0; k < nk; k++) {
      int src = keep[k];
      QR_CUDA(cudaMemcpyAsync(a + (size_t)cl * d * k, h->site[s1] + (size_t)cl * d * src,
                              sizeof(double2) * (size_t)cl * d, cudaMemcpyDeviceToDevice, s));
      QR_CUDA(cudaMemcpy2DAsync(c + k, sizeof(double2) * nk, h->site[s2] + src, sizeof(double2) * dim,
                                sizeof(double2), (size_t)d * cr2, cudaMemcpyDeviceToDevice, s));
      QR_CUDA(cudaMemcpyAsync(nl + k, h->lam[b] + src, sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
  }
  set_site(h, s1, a);
  set_site(h, s2, c);
  drop_lambda(h, b);
  h->lam[b] = nl;
  h->lamlen[b] = nk;
  h->bd[b] = nk;
  return QR_OK;
}

int mixed_canonize_impl(qr_chain* h, int center) {
  QR_TRY(require_open(h));
  QR_TRY(check_site(h, center));
  for (int i = 0; i < center; i++) QR_TRY(canonize_site_impl(h, i, QR_DIR_RIGHT, QR_METHOD_QR));
  for (int i = h->n - 1; i > center; i--) QR_TRY(canonize_site_impl(h, i, QR_DIR_LEFT, QR_METHOD_QR));
  return canonize_site_impl(h, center, QR_DIR_LEFT, QR_METHOD_SVD);
}

int normalize_impl(qr_chain* h, int root) {
  QR_TRY(require_open(h));
  QR_TRY(mixed_canonize_impl(h, root));
  return dnormalize(h->stream, h->lam[root - 1], h->lamlen[root - 1]);
}

// ---- evolve_2site! (Chain.jl:606-661) + Vidal helpers (Chain.jl:669-722) ------------------------
// theta (m x nn, FP64 result) = A_l diag(Lambda) A_r through the double-float GEMM
int theta_df(qr_chain* h, int sl, int sr, int m, int nn, int cb, double2* th) {
  cudaStream_t s = h->stream;
  float2 *al = nullptr, *ar = nullptr, *tt = nullptr;
  const size_t nal = (size_t)m * cb, nar = (size_t)cb * nn, ntt = (size_t)m * nn;
  int rc = dalloc((void**)&al, sizeof(float2) * 2 * nal, s);
  if (!rc) rc = dalloc((void**)&ar, sizeof(float2) * 2 * nar, s);
  if (!rc) rc = dalloc((void**)&tt, sizeof(float2) * 2 * ntt, s);
  if (!rc) rc = z2df_cols(s, h->site[sl], m, m, cb, h->lam[sl], al, al + nal, m);
  if (!rc) rc = z2df_cols(s, h->site[sr], cb, cb, nn, nullptr, ar, ar + nar, cb);
  if (!rc) rc = zgemm_df(s, DF_STORE, OP_N, m, nn, cb, al, al + nal, m, ar, ar + nar, cb, tt, tt + ntt, m);
  if (!rc) rc = df2z(s, tt, tt + ntt, m, m, nn, nullptr, th, m);
  if (al) cudaFreeAsync(al, s);
  if (ar) cudaFreeAsync(ar, s);
  if (tt) cudaFreeAsync(tt, s);
  return rc;
}

int evolve2_impl(qr_chain* h, int sl, const double* g, double threshold, int maxdim, int iscanonical,
                 int renormalize) {
  if (!h) return fail(QR_EINVAL, "null chain");
  QR_TRY(require_nonempty(h));
  if (sl < 0 || sl + 1 >= h->n) return fail(QR_EINVAL, "The sites in the bond must be between 1 and n");
  const int sr = sl + 1, n = h->n, d = h->d;
  cudaStream_t s = h->stream;
  QR_TRY(upload_gate(h, g, d * d));
  const double* lam_prev = nullptr;
  const double* lam_next = nullptr;
  if (iscanonical) {
    lam_prev = (sl == 0) ? nullptr : h->lam[sl - 1];
    lam_next = (sl == n - 2) ? nullptr : h->lam[sr];
    if (lam_prev) QR_TRY(scale_site_by_lambda(h, sl, 0, lam_prev, 0, 0.0));
    if (lam_next) QR_TRY(scale_site_by_lambda(h, sr, 2, lam_next, 0, 0.0));
  }
  const int cl = h->cl(sl), cb = h->bd[sl], cr = h->cr(sr);
  const int m = cl * d, nn = d * cr, k = m < nn ? m : nn;
  QR_TRY(ensure_ws(h, (size_t)m * nn + k));
  double2* th = h->ws;
  double* S = (double*)(th + (size_t)m * nn);
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  // theta = A_l diag(Lambda) A_r  [(l,o1) x (o2,r)]
  if (svd_mode(h) == QR_MIXED && k > 16) {
    // The mixed SVD splits theta into double-float before B = A X, so theta is formed there
    // directly: the double-float GEMM on the FP32 pipes (~2^-48 relative) instead of the FP64 one
    QR_TRY(theta_df(h, sl, sr, m, nn, cb, th));
  } else {
    QR_TRY(zgemm(s, OP_N, OP_N, m, nn, cb, one, h->site[sl], m, 0, h->site[sr], cb, 0, zero, th, m, 0, 1, h->lam[sl]));
  }
  QR_TRY(zgate2(s, th, cl, d, cr, h->gate));
  double2 *U = nullptr, *Vh = nullptr;
  QR_TRY(dalloc((void**)&U, sizeof(double2) * (size_t)m * k, s));
  QR_TRY(dalloc((void**)&Vh, sizeof(double2) * (size_t)k * nn, s));
  QR_TRY(zsvd_thin(s, h->svd, svd_mode(h), th, m, nn, m, U, m, S, Vh, k, maxdim >= 0 ? maxdim : 0));
  set_site(h, sl, U);
  set_site(h, sr, Vh);
  h->bd[sl] = k;
  if (iscanonical) {
    if (lam_prev) QR_TRY(scale_site_by_lambda(h, sl, 0, lam_prev, 1, 1e-32));
    if (lam_next) QR_TRY(scale_site_by_lambda(h, sr, 2, lam_next, 1, 1e-32));
  }
  QR_TRY(put_lambda(h, sl, S, k));
  const bool trunc = !std::isnan(threshold) || maxdim >= 0;
  if (trunc) {
    QR_TRY(truncate_impl(h, sl, sr, threshold, maxdim));
    if (renormalize && iscanonical) {
      QR_TRY(dnormalize(s, h->lam[sl], h->lamlen[sl]));
    } else if (renormalize) {
      QR_TRY(normalize_impl(h, sl));  // at site 1 this raises after the QR sweeps, as the reference does
    }
  }
  return QR_OK;
}

// ---- environment sweeps: <b|W|a> with per-site operators W (or none) ----------------------------
__global__ void scale_env_k(double2* E, int ca, int w, int cb, const double* lk, const double* lb) {
  long total = (long)ca * w * cb;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long a = t % ca, b = t / ((long)ca * w);
    double f = (lk ? lk[a] : 1.0) * (lb ? lb[b] : 1.0);
    E[t] = cscale(E[t], f);
  }
}

// Y[b,o,w',a'] = sum_{w,i} W[w,o,i,w'] X[w,b,i,a']
__global__ void mix_k(const double2* __restrict__ X, double2* __restrict__ Y, const double2* __restrict__ W,
                      int wl, int wr, int d, int cb, int ca2) {
  extern __shared__ double2 Ws[];
  const int nw = wl * d * d * wr;
  for (int t = threadIdx.x; t < nw; t += blockDim.x) Ws[t] = W[t];
  __syncthreads();
  long pairs = (long)cb * ca2;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < pairs; t += (long)gridDim.x * blockDim.x) {
    long b = t % cb, a2 = t / cb;
    for (int o = 0; o < d; o++)
      for (int w2 = 0; w2 < wr; w2++) {
        double2 acc = make_double2(0, 0);
        for (int i = 0; i < d; i++)
          for (int w = 0; w < wl; w++) {
            double2 x = X[w + wl * (b + (long)cb * (i + (long)d * a2))];
            acc = cadd(acc, cmul(Ws[w + wl * (o + d * (i + d * w2))], x));
          }
        Y[b + (long)cb * (o + (long)d * (w2 + (long)wr * a2))] = acc;
      }
  }
}

// The nonzero entries of one site's W, grouped by output (o, w'): MPOs of local Hamiltonians and
// products of few-site observables are sparse (the XXZ MPO has 12 nonzeros among its 100 entries),
// so the mixing step does only their multiply-adds.  Passed to the kernel by value.
constexpr int MIX_MAX_TERMS = 96, MIX_MAX_OUT = 16;
struct MixTable {
  int nout;
  int start[MIX_MAX_OUT + 1];
  short w[MIX_MAX_TERMS], i[MIX_MAX_TERMS];
  double2 v[MIX_MAX_TERMS];
};

// false when W (host, (wl, o, i, wr) wl fastest) has too many outputs or nonzeros for a table
bool build_mix_table(const double2* W, int wl, int d, int wr, MixTable* t) {
  if (d * wr > MIX_MAX_OUT) return false;
  int nt = 0;
  t->nout = d * wr;
  for (int w2 = 0; w2 < wr; w2++)
    for (int o = 0; o < d; o++) {
      const int out = o + d * w2;
      t->start[out] = nt;
      for (int i = 0; i < d; i++)
        for (int w = 0; w < wl; w++) {
          const double2 v = W[w + wl * (o + d * (i + d * w2))];
          if (v.x == 0.0 && v.y == 0.0) continue;
          if (nt == MIX_MAX_TERMS) return false;
          t->w[nt] = (short)w;
          t->i[nt] = (short)i;
          t->v[nt] = v;
          nt++;
        }
    }
  t->start[d * wr] = nt;
  return true;
}

// mix_k over the nonzeros only: Y[b,o,w',a'] = sum over the table's (w, i) of W X[w,b,i,a']
__global__ void mix_sparse_k(const double2* __restrict__ X, double2* __restrict__ Y, const MixTable tab, int wl,
                             int d, int cb, int ca2) {
  const long pairs = (long)cb * ca2;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < pairs; t += (long)gridDim.x * blockDim.x) {
    const long b = t % cb, a2 = t / cb;
    for (int out = 0; out < tab.nout; out++) {
      double2 acc = make_double2(0, 0);
      for (int e = tab.start[out]; e < tab.start[out + 1]; e++)
        acc = cadd(acc, cmul(tab.v[e], X[tab.w[e] + wl * (b + (long)cb * (tab.i[e] + (long)d * a2))]));
      const int o = out % d, w2 = out / d;
      Y[b + (long)cb * (o + (long)d * (w2 + (long)(tab.nout / d) * a2))] = acc;
    }
  }
}

struct EnvOps {
  std::vector<const double2*> W;  // per site, device (wl,o,i,wr) or nullptr for identity
  std::vector<int> wl, wr;
  std::vector<MixTable> tab;      // per site, used where has_tab[i]
  std::vector<char> has_tab;
};

// With QR_SPLIT_CONTRACT the two contractions of every site step run on the tcgen05 tensor cores
// (zgemm_tc: BF16x3 slices, FP32 accumulation, ~FP32 accuracy); the operator mixing, Lambda
// scaling and the stored environments stay FP64.
// <b|a> of two periodic chains: the closing bond pair (a0, b0) rides along as a spectator index
// s = a0 + chi0a b0 in the environment E[a, s, b] (the slot an MPO index takes in env_sweep), the
// sweep starts from E = delta(a, a0) delta(b, b0) and ends with the trace over a_n = a0, b_n = b0.
// Per site: X[(s, b), (o, a')] = E^T A, the permute Y[(b, o), s, a'] = X, then the batched
// E'[a', s, b'] = sum_{(b,o)} Y conj(B).  Cost and memory grow with chi0a chi0b.
// Workspace of the tensor-core contractions of one sweep: a 256-byte header (the kernel's error
// flag, zeroed here) followed by the BF16 slices, freed on the stream when the sweep returns.
struct TcWork {
  void* base = nullptr;
  unsigned* err = nullptr;
  void* ws = nullptr;
  cudaStream_t s = nullptr;
  int init(size_t bytes, cudaStream_t st) {
    s = st;
    QR_TRY(dalloc(&base, bytes + 256, s));
    err = static_cast<unsigned*>(base);
    ws = static_cast<char*>(base) + 256;
    QR_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), s));
    return QR_OK;
  }
  ~TcWork() {
    if (base) cudaFreeAsync(base, s);
  }
};

__global__ void ring_init_k(double2* E, int ca, int cb) {
  const long total = (long)ca * ca * cb * cb;  // E[a, s, b], s = a0 + ca b0
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long a = t % ca, r = t / ca, sidx = r % ((long)ca * cb), b = r / ((long)ca * cb);
    const long a0 = sidx % ca, b0 = sidx / ca;
    E[t] = make_double2(a == a0 && b == b0 ? 1.0 : 0.0, 0.0);
  }
}
__global__ void ring_trace_k(const double2* E, int ca, int cb, double2* out) {
  // out[s] = E[a0, s, b0] for s = a0 + ca b0 (summed on the host in FP64)
  const long S = (long)ca * cb;
  for (long sidx = blockIdx.x * (long)blockDim.x + threadIdx.x; sidx < S; sidx += (long)gridDim.x * blockDim.x) {
    const long a0 = sidx % ca, b0 = sidx / ca;
    out[sidx] = E[a0 + ca * (sidx + S * b0)];
  }
}

int env_sweep_ring(const qr_chain* a, const qr_chain* b, cudaStream_t s, double out[2]) {
  const int n = a->n, d = a->d;
  const int c0a = a->cl(0), c0b = b->cl(0);
  const long S = (long)c0a * c0b;
  const bool split = (a->precision & QR_SPLIT_CONTRACT) != 0;
  size_t maxE = 1, maxX = 1;
  for (int i = 0; i < n; i++) {
    maxE = std::max(maxE, (size_t)std::max(a->cl(i), a->cr(i)) * S * std::max(b->cl(i), b->cr(i)));
    maxX = std::max(maxX, (size_t)S * b->cl(i) * d * a->cr(i));
  }
  double2 *E0 = nullptr, *E1 = nullptr, *X = nullptr, *Y = nullptr, *tr = nullptr;
  QR_TRY(dalloc((void**)&E0, sizeof(double2) * maxE, s));
  QR_TRY(dalloc((void**)&E1, sizeof(double2) * maxE, s));
  QR_TRY(dalloc((void**)&X, sizeof(double2) * maxX, s));
  QR_TRY(dalloc((void**)&Y, sizeof(double2) * maxX, s));
  QR_TRY(dalloc((void**)&tr, sizeof(double2) * S, s));
  TcWork tw;
  if (split) {
    size_t ws = 0;
    for (int i = 0; i < n; i++) {
      ws = std::max(ws, zgemm_tc_workspace((int)(S * b->cl(i)), d * a->cr(i), a->cl(i), 1, true));
      ws = std::max(ws, zgemm_tc_workspace(a->cr(i), b->cr(i), b->cl(i) * d, (int)S, true));
    }
    QR_TRY(tw.init(ws, s));
  }
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  {
    long tot = (long)c0a * S * c0b;
    unsigned g = (unsigned)std::min<long>((tot + 255) / 256, 4864);
    ring_init_k<<<g, 256, 0, s>>>(E0, c0a, c0b);
    count_launch();
  }
  int rc = QR_OK;
  for (int i = 0; i < n && rc == QR_OK; i++) {
    const int ca = a->cl(i), ca2 = a->cr(i), cb = b->cl(i), cb2 = b->cr(i);
    if (i > 0 && (a->lam[i - 1] || b->lam[i - 1])) {
      long tot = (long)ca * S * cb;
      unsigned g = (unsigned)std::min<long>((tot + 255) / 256, 4864);
      scale_env_k<<<g, 256, 0, s>>>(E0, ca, (int)S, cb, a->lam[i - 1], b->lam[i - 1]);
      count_launch();
    }
    // X[(s, b), (o, a')] = E^T A
    rc = split ? zgemm_tc(s, OP_T, OP_N, (int)(S * cb), d * ca2, ca, E0, ca, 0, a->site[i], ca, 0, X, S * cb, 0, 1,
                          tw.ws, tw.err)
               : zgemm(s, OP_T, OP_N, (int)(S * cb), d * ca2, ca, one, E0, ca, 0, a->site[i], ca, 0, zero, X, S * cb,
                       0, 1, nullptr);
    if (rc) break;
    // Y[(b, o), s, a'] = X[(s, b), (o, a')]
    Perm p;
    p.nd = 4;
    p.dims[0] = cb;
    p.dims[1] = d;
    p.dims[2] = S;
    p.dims[3] = ca2;
    p.src_stride[0] = S;
    p.src_stride[1] = S * cb;
    p.src_stride[2] = 1;
    p.src_stride[3] = S * cb * d;
    rc = zpermute(s, X, Y, p);
    if (rc) break;
    // E'[a', s, b'] = sum_{(b,o)} Y[(b,o), s, a'] conj(B[(b,o), b'])
    rc = split ? zgemm_tc(s, OP_T, OP_R, ca2, cb2, cb * d, Y, (long)cb * d * S, (long)cb * d, b->site[i],
                          (long)cb * d, 0, E1, (long)ca2 * S, ca2, (int)S, tw.ws, tw.err)
               : zgemm(s, OP_T, OP_R, ca2, cb2, cb * d, one, Y, (long)cb * d * S, (long)cb * d, b->site[i],
                       (long)cb * d, 0, zero, E1, (long)ca2 * S, ca2, (int)S, nullptr);
    std::swap(E0, E1);
  }
  if (rc == QR_OK) {
    unsigned g = (unsigned)std::min<long>((S + 255) / 256, 4864);
    ring_trace_k<<<g, 256, 0, s>>>(E0, c0a, c0b, tr);
    count_launch();
    double2* h = static_cast<double2*>(host_scratch(sizeof(double2) * (S + 1)));
    if (!h) rc = fail(QR_ENOMEM, "page-locked host scratch");
    if (!rc) rc = cuda_ok(cudaMemcpyAsync(h, tr, sizeof(double2) * S, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    if (!rc && split)
      rc = cuda_ok(cudaMemcpyAsync(h + S, tw.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    if (!rc) rc = cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (!rc && split && *reinterpret_cast<const unsigned*>(h + S))
      rc = fail(QR_ECUDA, "tensor-core contraction: a bounded wait gave up");
    double re = 0, im = 0;
    for (long i = 0; !rc && i < S; i++) { re += h[i].x; im += h[i].y; }
    out[0] = re;
    out[1] = im;
  }
  cudaFreeAsync(E0, s);
  cudaFreeAsync(E1, s);
  cudaFreeAsync(X, s);
  cudaFreeAsync(Y, s);
  cudaFreeAsync(tr, s);
  return rc;
}

int env_sweep(const qr_chain* a, const qr_chain* b, const EnvOps* ops, cudaStream_t s, double out[2]) {
  if (has_empty_bond(a) || has_empty_bond(b)) {  // a size-0 bond: the contraction is an empty sum
    out[0] = out[1] = 0.0;
    return QR_OK;
  }
  if (a->periodic || b->periodic) {
    if (!(a->periodic && b->periodic)) return fail(QR_EINVAL, "both chains must have the same boundary");
    if (ops) return fail(QR_EINVAL, "operator expectation values of periodic chains are not implemented");
    return env_sweep_ring(a, b, s, out);
  }
  const int n = a->n, d = a->d;
  const bool split = (a->precision & QR_SPLIT_CONTRACT) != 0;
  // largest buffers
  size_t maxE = 1, maxX = 1;
  for (int i = 0; i < n; i++) {
    int wl = ops ? ops->wl[i] : 1, wr = ops ? ops->wr[i] : 1;
    size_t e = (size_t)a->cr(i) * wr * b->cr(i);
    size_t x = (size_t)wl * b->cl(i) * d * a->cr(i);
    size_t y = (size_t)b->cl(i) * d * wr * a->cr(i);
    if (e > maxE) maxE = e;
    if (x > maxX) maxX = x;
    if (y > maxX) maxX = y;
  }
  double2 *E0 = nullptr, *E1 = nullptr, *X = nullptr, *Y = nullptr;
  QR_TRY(dalloc((void**)&E0, sizeof(double2) * maxE, s));
  QR_TRY(dalloc((void**)&E1, sizeof(double2) * maxE, s));
  QR_TRY(dalloc((void**)&X, sizeof(double2) * maxX, s));
  QR_TRY(dalloc((void**)&Y, sizeof(double2) * maxX, s));
  // split contractions: one BF16-slice workspace for the largest step, behind a 256-byte header
  // holding the tensor-core kernel's error flag
  TcWork tw;
  if (split) {
    size_t ws = 0;
    for (int i = 0; i < n; i++) {
      int wl = ops ? ops->wl[i] : 1, wr = ops ? ops->wr[i] : 1;
      ws = std::max(ws, zgemm_tc_workspace(wl * b->cl(i), d * a->cr(i), a->cl(i), 1, true));
      ws = std::max(ws, zgemm_tc_workspace(a->cr(i), b->cr(i), b->cl(i) * d, wr, true));
    }
    QR_TRY(tw.init(ws, s));
  }
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  double2 init = one;
  QR_CUDA(cudaMemcpyAsync(E0, &init, sizeof(double2), cudaMemcpyHostToDevice, s));
  int rc = QR_OK;
  for (int i = 0; i < n && rc == QR_OK; i++) {
    const int ca = a->cl(i), ca2 = a->cr(i), cb = b->cl(i), cb2 = b->cr(i);
    const int wl = ops ? ops->wl[i] : 1, wr = ops ? ops->wr[i] : 1;
    const double2* W = ops ? ops->W[i] : nullptr;
    if (i > 0 && (a->lam[i - 1] || b->lam[i - 1])) {
      long tot = (long)ca * wl * cb;
      unsigned g = (unsigned)((tot + 255) / 256);
      scale_env_k<<<g > 4864 ? 4864 : g, 256, 0, s>>>(E0, ca, wl, cb, a->lam[i - 1], b->lam[i - 1]);
      count_launch();
    }
    // X[(w,b) x (i,a')] = E^T A
    rc = split ? zgemm_tc(s, OP_T, OP_N, wl * cb, d * ca2, ca, E0, ca, 0, a->site[i], ca, 0, X, wl * cb, 0, 1, tw.ws,
                          tw.err)
               : zgemm(s, OP_T, OP_N, wl * cb, d * ca2, ca, one, E0, ca, 0, a->site[i], ca, 0, zero, X, wl * cb, 0, 1,
                       nullptr);
    if (rc) break;
    const double2* Yp = X;
    if (W) {
      long pairs = (long)cb * ca2;
      unsigned g = (unsigned)((pairs + 255) / 256);
      if (!ops->has_tab.empty() && ops->has_tab[i])
        mix_sparse_k<<<g > 4864 ? 4864 : g, 256, 0, s>>>(X, Y, ops->tab[i], wl, d, cb, ca2);
      else
        mix_k<<<g > 4864 ? 4864 : g, 256, sizeof(double2) * wl * d * d * wr, s>>>(X, Y, W, wl, wr, d, cb, ca2);
      count_launch();
      Yp = Y;
    }
    // E'_w' = Y_w'^T conj(B)
    rc = split ? zgemm_tc(s, OP_T, OP_R, ca2, cb2, cb * d, Yp, (long)cb * d * wr, (long)cb * d, b->site[i],
                          (long)cb * d, 0, E1, (long)ca2 * wr, ca2, wr, tw.ws, tw.err)
               : zgemm(s, OP_T, OP_R, ca2, cb2, cb * d, one, Yp, (long)cb * d * wr, (long)cb * d, b->site[i],
                       (long)cb * d, 0, zero, E1, (long)ca2 * wr, ca2, wr, nullptr);
    std::swap(E0, E1);
  }
  if (rc == QR_OK) {
    QR_CUDA(cudaGetLastError());
    double2* r = static_cast<double2*>(host_scratch(2 * sizeof(double2)));
    if (!r) return fail(QR_ENOMEM, "page-locked host scratch");
    QR_CUDA(cudaMemcpyAsync(r, E0, sizeof(double2), cudaMemcpyDeviceToHost, s));
    if (split) QR_CUDA(cudaMemcpyAsync(r + 1, tw.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QR_CUDA(cudaStreamSynchronize(s));
    if (split && *reinterpret_cast<const unsigned*>(r + 1))
      rc = fail(QR_ECUDA, "tensor-core contraction: a bounded wait gave up");
    out[0] = r->x;
    out[1] = r->y;
  }
  cudaFreeAsync(E0, s);
  cudaFreeAsync(E1, s);
  cudaFreeAsync(X, s);
  cudaFreeAsync(Y, s);
  return rc;
}

}  // namespace

// =================================================================================================
extern "C" {

const char* qr_last_error_string(void) { return t_err.c_str(); }

int qr_version(int* major, int* minor) try {
  if (major) *major = 0;
  if (minor) *minor = 1;
  return QR_OK;
} QR_ABI_CATCH

int qr_device_count(int* count) try {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (count) *count = (e == cudaSuccess) ? c : 0;
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  return QR_OK;
} QR_ABI_CATCH

int qr_set_device(int device) try {
  QR_CUDA(cudaSetDevice(device));
  return QR_OK;
} QR_ABI_CATCH

int qr_launch_count(uint64_t* count) try {
  if (count) *count = g_launches.load();
  return QR_OK;
} QR_ABI_CATCH

static int chain_create(int n, int d, const int* bond_dims, bool periodic, qr_chain** out);

int qr_chain_create(int n, int d, const int* bond_dims, qr_chain** out) try {
  return chain_create(n, d, bond_dims, false, out);
} QR_ABI_CATCH

int qr_chain_create_periodic(int n, int d, const int* bond_dims, qr_chain** out) try {
  return chain_create(n, d, bond_dims, true, out);
} QR_ABI_CATCH

int qr_chain_boundary(const qr_chain* h, int* periodic) try {
  if (!h || !periodic) return fail(QR_EINVAL, "null argument");
  *periodic = h->periodic ? 1 : 0;
  return QR_OK;
} QR_ABI_CATCH

static int chain_create(int n, int d, const int* bond_dims, bool periodic, qr_chain** out) {
  if (!out) return fail(QR_EINVAL, "null output");
  *out = nullptr;
  if (n < 2) return fail(QR_EINVAL, "a Chain needs at least 2 sites");
  if (d < 2 || d > 4) return fail(QR_EINVAL, "physical dimension must be 2..4");
  const int nb = periodic ? n : n - 1;
  for (int b = 0; b < nb; b++)
    if (!bond_dims || bond_dims[b] < 0) return fail(QR_EINVAL, "bond dimensions must be >= 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(QR_ENODEV, "no CUDA device");
  std::call_once(g_pool_once, init_pool);
  qr_chain* h = new qr_chain();
  h->n = n;
  h->d = d;
  h->periodic = periodic;
  h->bd.assign(bond_dims, bond_dims + nb);
  h->site.assign(n, nullptr);
  h->lam.assign(n - 1, nullptr);
  h->lamlen.assign(n - 1, 0);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaStreamCreate"); }
  h->svd = svd_work_create();
  int rc = dalloc((void**)&h->gate, sizeof(double2) * 256, h->stream);
  if (!rc) rc = cuda_ok(cudaHostAlloc((void**)&h->gate_host, sizeof(double2) * 256, cudaHostAllocDefault), "cudaHostAlloc");
  if (!rc) rc = dalloc((void**)&h->scal, sizeof(double) * 16, h->stream);
  for (int i = 0; i < n && !rc; i++) {
    rc = dalloc((void**)&h->site[i], sizeof(double2) * h->elems(i), h->stream);
    if (!rc) rc = cuda_ok(cudaMemsetAsync(h->site[i], 0, sizeof(double2) * h->elems(i), h->stream), "memset");
  }
  if (rc) { qr_chain_free(h); return rc; }
  *out = h;
  return QR_OK;
}

int qr_chain_free(qr_chain* h) try {
  if (!h) return QR_OK;
  cudaStreamSynchronize(h->stream);
  for (qr_chain* l : h->lanes) qr_chain_free(l);
  h->lanes.clear();
  if (!h->is_lane) {
    for (auto p : h->site) if (p) cudaFree(p);
    for (auto p : h->lam) if (p) cudaFree(p);
  }
  if (h->gate) cudaFree(h->gate);
  if (h->gate_host) cudaFreeHost(h->gate_host);
  if (h->scal) cudaFree(h->scal);
  if (h->ws) cudaFree(h->ws);
  svd_work_free(h->svd);
  cudaStreamDestroy(h->stream);
  delete h;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_copy(const qr_chain* src, qr_chain** out) try {
  if (!src || !out) return fail(QR_EINVAL, "null chain");
  *out = nullptr;
  QR_CUDA(cudaStreamSynchronize(src->stream));
  qr_chain* h = nullptr;
  QR_TRY(chain_create(src->n, src->d, src->bd.data(), src->periodic, &h));
  h->precision = src->precision;
  int rc = QR_OK;
  for (int i = 0; i < src->n && !rc; i++)
    rc = cuda_ok(cudaMemcpyAsync(h->site[i], src->site[i], sizeof(double2) * src->elems(i),
                                 cudaMemcpyDeviceToDevice, h->stream), "cudaMemcpyAsync");
  for (int b = 0; b < src->n - 1 && !rc; b++)
    if (src->lam[b]) rc = put_lambda(h, b, src->lam[b], src->lamlen[b]);
  if (rc) {  // no half-built copy is handed out
    qr_chain_free(h);
    return rc;
  }
  *out = h;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_upload_site(qr_chain* h, int site, const double* host, const char* order) try {
  QR_TRY(check_site(h, site));
  if (!host) return fail(QR_EINVAL, "null host array");
  if (!is_perm(order ? order : "", "olr")) return fail(QR_EINVAL, "order must be a permutation of (o, l, r)");
  std::string ho = filtered(order, site == 0 && !h->periodic, site == h->n - 1 && !h->periodic);
  long idims[3] = {h->cl(site), h->d, h->cr(site)};
  Perm p = make_perm(ho, "lor", idims);
  size_t ne = h->elems(site);
  QR_TRY(ensure_ws(h, ne));
  QR_CUDA(cudaMemcpyAsync(h->ws, host, sizeof(double2) * ne, cudaMemcpyHostToDevice, h->stream));
  QR_TRY(zpermute(h->stream, h->ws, h->site[site], p));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_download_site(const qr_chain* hc, int site, double* host, const char* order) try {
  qr_chain* h = const_cast<qr_chain*>(hc);
  QR_TRY(check_site(h, site));
  if (!host) return fail(QR_EINVAL, "null host array");
  if (!is_perm(order ? order : "", "olr")) return fail(QR_EINVAL, "order must be a permutation of (o, l, r)");
  std::string ho = filtered(order, site == 0 && !h->periodic, site == h->n - 1 && !h->periodic);
  // dst (host order) gathers from the internal (l,o,r) layout: build the inverse map
  long dims_by_letter[3] = {h->cl(site), h->d, h->cr(site)};  // l, o, r
  const std::string iord = "lor";
  long istride[3] = {1, dims_by_letter[0], dims_by_letter[0] * dims_by_letter[1]};
  Perm p;
  p.nd = (int)ho.size();
  for (int k = 0; k < p.nd; k++) {
    size_t q = iord.find(ho[k]);
    p.dims[k] = dims_by_letter[q];
    p.src_stride[k] = istride[q];
  }
  size_t ne = h->elems(site);
  QR_TRY(ensure_ws(h, ne));
  QR_TRY(zpermute(h->stream, h->site[site], h->ws, p));
  QR_CUDA(cudaMemcpyAsync(host, h->ws, sizeof(double2) * ne, cudaMemcpyDeviceToHost, h->stream));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

// ---- rand(Chain, Open, State / Operator) on the device ---------------------------------------
// Bond dimensions follow the reference's sampler (src/Ansatz/Chain.jl:223-297): site i (1-based)
// draws a (chi_l x chi_r p) random matrix with chi_l = min(chi, p^(m-1)), chi_r = min(chi, p^m),
// m = (n + 1 - |2i - n - 1|) / 2, the two swapped after the middle and equal at the middle site of
// an odd chain; the State's first site uses (chi_r, 1) (its rows become the right bond).  Rows are
// Gram-Schmidt orthonormalised (random.cu), the first site is divided by sqrt(p) for the State and
// by sqrt(min(chi, p^2)) for the Operator.
namespace {
long ipow_cap(long p, int e, long cap) {
  long v = 1;
  for (int k = 0; k < e && v < cap; k++) v *= p;
  return v < cap ? v : cap;
}
void sampler_dims(int n, long p, long chi, int i, long& l, long& r) {
  const bool after_mid = i > n / 2;
  const int m = (n + 1 - std::abs(2 * i - n - 1)) / 2;
  l = ipow_cap(p, m - 1, chi);
  r = ipow_cap(p, m, chi);
  if ((n % 2 == 1) && i == n / 2 + 1) r = l;
  else if (after_mid) std::swap(l, r);
}
}  // namespace

int qr_chain_random(int n, int d, int chi, uint64_t seed, int complex_entries, qr_chain** out) try {
  if (!out) return fail(QR_EINVAL, "null output");
  *out = nullptr;
  if (n < 2 || d < 2 || chi < d) return fail(QR_EINVAL, "rand(Chain, Open, State) needs n >= 2, p >= 2 and chi >= p");
  std::vector<long> L(n), Rr(n);
  for (int i = 1; i <= n; i++) sampler_dims(n, d, chi, i, L[i - 1], Rr[i - 1]);
  // site 1 samples (chi_r, 1) and its rows become the right bond; the last site has chi_r = 1
  std::vector<int> bd(n - 1);
  bd[0] = (int)Rr[0];
  for (int b = 1; b < n - 1; b++) bd[b] = (int)Rr[b];
  for (int b = 0; b < n - 1; b++)
    if (bd[b] != (int)L[b + 1]) return fail(QR_EDIM, "sampler bond dimensions do not chain");
  qr_chain* h = nullptr;
  QR_TRY(qr_chain_create(n, d, bd.data(), &h));
  int rc = QR_OK;
  double2* E = nullptr;
  for (int i = 0; i < n && !rc; i++) {
    // rows x N random isometry; device site (cl, d, cr), l fastest
    const long rows = i == 0 ? Rr[0] : L[i];
    const long rdim = (i == 0 || i == n - 1) ? 1 : Rr[i];
    const long N = rdim * d;
    const double scale = i == 0 ? 1.0 / std::sqrt((double)d) : 1.0;
    rc = cuda_ok(cudaMallocAsync(&E, sizeof(double2) * rows * N, h->stream), "cudaMallocAsync");
    if (!rc) rc = rand_rows_isometry(h->stream, (int)rows, (int)N, seed, (uint32_t)i, complex_entries, scale, E);
    if (!rc) {
      // E[row, r + rdim * o] -> site[l, o, r]; on site 1 the row index is the right bond
      Perm p;
      p.nd = 3;
      p.dims[0] = h->cl(i);
      p.dims[1] = d;
      p.dims[2] = h->cr(i);
      if (i == 0) {
        p.src_stride[0] = 0;
        p.src_stride[1] = rows;
        p.src_stride[2] = 1;
      } else {
        p.src_stride[0] = 1;
        p.src_stride[1] = rows * rdim;
        p.src_stride[2] = rows;
      }
      rc = zpermute(h->stream, E, h->site[i], p);
    }
    if (E) cudaFreeAsync(E, h->stream);
    E = nullptr;
  }
  if (!rc) rc = cuda_ok(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  if (rc) {
    qr_chain_free(h);
    return rc;
  }
  *out = h;
  return QR_OK;
} QR_ABI_CATCH

int qr_mpo_random(int n, int d, int chi, uint64_t seed, int complex_entries, qr_mpo** out) try {
  if (!out) return fail(QR_EINVAL, "null output");
  *out = nullptr;
  if (n < 2 || d < 2 || chi < 1) return fail(QR_EINVAL, "rand(Chain, Open, Operator) needs n >= 2, p >= 2 and chi >= 1");
  const long p2 = (long)d * d;
  std::vector<long> L(n), Rr(n);
  for (int i = 1; i <= n; i++) sampler_dims(n, p2, chi, i, L[i - 1], Rr[i - 1]);
  std::vector<int> bd(n - 1);
  for (int b = 0; b < n - 1; b++) bd[b] = (int)Rr[b];
  for (int b = 0; b < n - 1; b++)
    if (bd[b] != (int)L[b + 1]) return fail(QR_EDIM, "sampler bond dimensions do not chain");
  qr_mpo* w = nullptr;
  QR_TRY(qr_mpo_create(n, d, bd.data(), &w));
  int rc = QR_OK;
  double2* E = nullptr;
  for (int i = 0; i < n && !rc; i++) {
    // shapes (chi_r, ip, op) at site 1, (chi_l, chi_r, ip, op) inside, (chi_l, ip, op) at site n;
    // the rows are the first dimension, columns the rest (column-major)
    const long rows = i == 0 ? Rr[0] : L[i];
    const long rdim = (i == 0 || i == n - 1) ? 1 : Rr[i];
    const long N = rdim * p2;
    const double scale = i == 0 ? 1.0 / std::sqrt((double)std::min<long>(chi, p2)) : 1.0;
    rc = cuda_ok(cudaMalloc(&E, sizeof(double2) * rows * N), "cudaMalloc");
    if (!rc) rc = rand_rows_isometry(0, (int)rows, (int)N, seed, (uint32_t)(0x4000u + i), complex_entries, scale, E);
    if (!rc) {
      // E[row, r + rdim (o + d i)] -> W[wl, o, i, wr] (the permuted sampler array read as
      // (o, i, l, r)); on site 1 the row index is the right bond
      Perm p;
      p.nd = 4;
      p.dims[0] = w->wl(i);
      p.dims[1] = d;
      p.dims[2] = d;
      p.dims[3] = w->wr(i);
      if (i == 0) {
        p.src_stride[0] = 0;
        p.src_stride[1] = rows;
        p.src_stride[2] = rows * d;
        p.src_stride[3] = 1;
      } else {
        p.src_stride[0] = 1;
        p.src_stride[1] = rows * rdim;
        p.src_stride[2] = rows * rdim * d;
        p.src_stride[3] = rows;
      }
      rc = zpermute(0, E, w->site[i], p);
    }
    if (E) cudaFree(E);
    E = nullptr;
  }
  if (!rc) rc = cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  if (rc) {
    qr_mpo_free(w);
    return rc;
  }
  *out = w;
  return QR_OK;
} QR_ABI_CATCH

// ---- checkpoint / export ---------------------------------------------------------------------
// File layout (little-endian), written so a Julia reader can rebuild MPS(arrays) / pMPS(arrays):
//   "QRCHAIN1" | int32 n, d, precision, periodic | int32 bond_dims[n-1, or n when periodic: the
//   last is the bond between site n and site 1] | uint8 has_lambda[n-1]
//   | site 0 .. n-1: ComplexF64 data in the reference's (o, l, r) column-major order, the open ends
//     without l (site 1) and r (site n) | for every bond with has_lambda: Float64 Lambda[bond_dim]
namespace {
const char kChainMagic[8] = {'Q', 'R', 'C', 'H', 'A', 'I', 'N', '1'};
struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) fclose(f);
  }
};
}  // namespace

int qr_chain_save(const qr_chain* h, const char* path) try {
  if (!h || !path) return fail(QR_EINVAL, "null argument");
  FileCloser fc{fopen(path, "wb")};
  if (!fc.f) return fail(QR_EINVAL, std::string("cannot open for writing: ") + path);
  const int32_t hdr[4] = {h->n, h->d, h->precision, h->periodic ? 1 : 0};
  bool ok = fwrite(kChainMagic, 1, 8, fc.f) == 8 && fwrite(hdr, sizeof(int32_t), 4, fc.f) == 4;
  std::vector<int32_t> bd(h->bd.begin(), h->bd.end());  // n - 1 bonds, n for a periodic chain
  std::vector<uint8_t> fl(h->n - 1);
  for (int b = 0; b < h->n - 1; b++) fl[b] = h->lam[b] != nullptr;
  ok = ok && fwrite(bd.data(), sizeof(int32_t), bd.size(), fc.f) == bd.size();
  ok = ok && fwrite(fl.data(), 1, fl.size(), fc.f) == fl.size();
  std::vector<double> buf;
  for (int i = 0; i < h->n && ok; i++) {
    buf.resize(2 * h->elems(i));
    QR_TRY(qr_chain_download_site(h, i, buf.data(), "olr"));
    ok = fwrite(buf.data(), sizeof(double), buf.size(), fc.f) == buf.size();
  }
  for (int b = 0; b < h->n - 1 && ok; b++) {
    if (!fl[b]) continue;
    buf.resize(h->bd[b]);
    int len = 0;
    QR_TRY(qr_chain_get_lambda(h, b, buf.data(), &len));
    ok = fwrite(buf.data(), sizeof(double), (size_t)len, fc.f) == (size_t)len;
  }
  if (!ok) return fail(QR_EINVAL, std::string("write failed: ") + path);
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_load(const char* path, qr_chain** out) try {
  if (!path || !out) return fail(QR_EINVAL, "null argument");
  *out = nullptr;
  FileCloser fc{fopen(path, "rb")};
  if (!fc.f) return fail(QR_EINVAL, std::string("cannot open: ") + path);
  char magic[8];
  int32_t hdr[4];
  if (fread(magic, 1, 8, fc.f) != 8 || memcmp(magic, kChainMagic, 8) != 0 ||
      fread(hdr, sizeof(int32_t), 4, fc.f) != 4)
    return fail(QR_EINVAL, "not a chain checkpoint");
  const int n = hdr[0], d = hdr[1], prec = hdr[2], periodic = hdr[3];
  if (n < 2 || n > (1 << 20) || d < 1 || d > 64 || (periodic != 0 && periodic != 1))
    return fail(QR_EINVAL, "corrupt chain checkpoint header");
  std::vector<int32_t> bd(periodic ? n : n - 1);
  std::vector<uint8_t> fl(n - 1);
  if (fread(bd.data(), sizeof(int32_t), bd.size(), fc.f) != bd.size() || fread(fl.data(), 1, fl.size(), fc.f) != fl.size())
    return fail(QR_EINVAL, "truncated chain checkpoint");
  for (int32_t b : bd)
    if (b < 0) return fail(QR_EINVAL, "corrupt chain checkpoint bond dimensions");
  std::vector<int> bdi(bd.begin(), bd.end());
  qr_chain* h = nullptr;
  QR_TRY(chain_create(n, d, bdi.data(), periodic != 0, &h));
  int rc = qr_chain_set_precision(h, prec);
  std::vector<double> buf;
  for (int i = 0; i < n && !rc; i++) {
    buf.resize(2 * h->elems(i));
    if (fread(buf.data(), sizeof(double), buf.size(), fc.f) != buf.size()) rc = fail(QR_EINVAL, "truncated chain checkpoint");
    else rc = qr_chain_upload_site(h, i, buf.data(), "olr");
  }
  for (int b = 0; b < n - 1 && !rc; b++) {
    if (!fl[b]) continue;
    buf.resize(bd[b] > 0 ? bd[b] : 1);  // an empty bond keeps an empty Lambda: pass a non-null pointer
    if (fread(buf.data(), sizeof(double), (size_t)bd[b], fc.f) != (size_t)bd[b]) rc = fail(QR_EINVAL, "truncated chain checkpoint");
    else rc = qr_chain_set_lambda(h, b, buf.data(), bd[b]);
  }
  if (rc) {
    qr_chain_free(h);
    return rc;
  }
  *out = h;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_site_dims(const qr_chain* h, int site, int* chi_l, int* d, int* chi_r) try {
  QR_TRY(check_site(h, site));
  if (chi_l) *chi_l = h->cl(site);
  if (d) *d = h->d;
  if (chi_r) *chi_r = h->cr(site);
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_bond_dims(const qr_chain* h, int* out) try {
  if (!h || !out) return fail(QR_EINVAL, "null argument");
  for (int b = 0; b < (int)h->bd.size(); b++) out[b] = h->bd[b];
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_has_lambda(const qr_chain* h, int bond, int* flag) try {
  if (!h || !flag || bond < 0 || bond >= h->n - 1) return fail(QR_EINVAL, "Invalid bond");
  *flag = h->lam[bond] != nullptr;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_get_lambda(const qr_chain* h, int bond, double* out, int* len) try {
  if (!h || bond < 0 || bond >= h->n - 1) return fail(QR_EINVAL, "Invalid bond");
  if (!h->lam[bond]) {
    if (len) *len = 0;
    return fail(QR_ENO_SCHMIDT, "Can't access the spectrum on bond");
  }
  if (len) *len = h->lamlen[bond];
  if (out) {
    QR_CUDA(cudaMemcpyAsync(out, h->lam[bond], sizeof(double) * h->lamlen[bond], cudaMemcpyDeviceToHost, h->stream));
    QR_CUDA(cudaStreamSynchronize(h->stream));
  }
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_set_lambda(qr_chain* h, int bond, const double* lam, int len) try {
  if (!h || bond < 0 || bond >= h->n - 1) return fail(QR_EINVAL, "Invalid bond");
  if (!lam) { drop_lambda(h, bond); return QR_OK; }
  if (len != h->bd[bond]) return fail(QR_EDIM, "Lambda length must equal the bond dimension");
  double* p = nullptr;
  QR_TRY(dalloc((void**)&p, sizeof(double) * len, h->stream));
  QR_CUDA(cudaMemcpyAsync(p, lam, sizeof(double) * len, cudaMemcpyHostToDevice, h->stream));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  drop_lambda(h, bond);
  h->lam[bond] = p;
  h->lamlen[bond] = len;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_ntensors(const qr_chain* h, int* out) try {
  if (!h || !out) return fail(QR_EINVAL, "null argument");
  int c = h->n;
  for (auto p : h->lam) c += (p != nullptr);
  *out = c;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_nsites(const qr_chain* h, int* out) try {
  if (!h || !out) return fail(QR_EINVAL, "null argument");
  *out = h->n;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_set_precision(qr_chain* h, int mode) try {
  if (!h) return fail(QR_EINVAL, "null chain");
  if (mode < 0 || mode > (QR_MIXED | QR_SPLIT_CONTRACT))
    return fail(QR_EINVAL, "precision must be a combination of QR_MIXED and QR_SPLIT_CONTRACT");
  h->precision = mode;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_get_precision(const qr_chain* h, int* mode) try {
  if (!h || !mode) return fail(QR_EINVAL, "null argument");
  *mode = h->precision;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_stream(const qr_chain* h, void** stream) try {
  if (!h || !stream) return fail(QR_EINVAL, "null argument");
  *stream = (void*)h->stream;
  return QR_OK;
} QR_ABI_CATCH

int qr_chain_sync(const qr_chain* h) try {
  if (!h) return fail(QR_EINVAL, "null chain");
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

int qr_canonize_site(qr_chain* h, int site, int direction, int method) try {
  QR_TRY(canonize_site_impl(h, site, direction, method));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

// canonize! (Chain.jl:469-497)
int qr_canonize(qr_chain* h) try {
  if (!h) return fail(QR_EINVAL, "null chain");
  const int n = h->n;
  for (int i = n - 1; i >= 1; i--) QR_TRY(canonize_site_impl(h, i, QR_DIR_LEFT, QR_METHOD_QR));
  std::vector<double*> lams(n - 1, nullptr);
  std::vector<int> lens(n - 1, 0);
  for (int i = 0; i < n - 1; i++) {
    QR_TRY(canonize_site_impl(h, i, QR_DIR_RIGHT, QR_METHOD_SVD));
    // pop Lambda_i and absorb it into A_{i+1}
    lams[i] = h->lam[i];
    lens[i] = h->lamlen[i];
    h->lam[i] = nullptr;
    h->lamlen[i] = 0;
    QR_TRY(scale_site_by_lambda(h, i + 1, 0, lams[i], 0, 0.0));
  }
  for (int i = 1; i < n; i++) {
    QR_TRY(scale_site_by_lambda(h, i, 0, lams[i - 1], 1, 1e-64));
    h->lam[i - 1] = lams[i - 1];
    h->lamlen[i - 1] = lens[i - 1];
  }
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

int qr_mixed_canonize(qr_chain* h, int center) try {
  QR_TRY(mixed_canonize_impl(h, center));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

int qr_normalize(qr_chain* h, int root) try {
  QR_TRY(normalize_impl(h, root));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

// contract!(::Chain, Val(:between)) (Chain.jl:309-333)
int qr_contract_between(qr_chain* h, int site1, int site2, int direction, int delete_lambda) try {
  QR_TRY(check_site(h, site1));
  QR_TRY(check_site(h, site2));
  // tensors(tn; between) (Ansatz.jl:78-89): two different sites; none shared bond -> nothing to do
  if (site1 == site2) return fail(QR_EASSERT, "Sites must be different");
  if (std::abs(site2 - site1) != 1) return QR_OK;
  QR_TRY(require_nonempty(h));
  const int b = std::min(site1, site2);
  if (!h->lam[b]) return QR_OK;
  const bool fwd = site2 == site1 + 1;  // site1 is the bond's left site: the bond is its r index
  if (direction == QR_DIR_RIGHT) {
    QR_TRY(scale_site_by_lambda(h, site2, fwd ? 0 : 2, h->lam[b], 0, 0.0));
  } else if (direction == QR_DIR_LEFT) {
    QR_TRY(scale_site_by_lambda(h, site1, fwd ? 2 : 0, h->lam[b], 0, 0.0));
  } else {
    return fail(QR_EINVAL, "Unknown direction");
  }
  if (delete_lambda) drop_lambda(h, b);
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

int qr_canonicality_error(const qr_chain* hc, int site, int direction, double* err) try {
  qr_chain* h = const_cast<qr_chain*>(hc);
  QR_TRY(check_site(h, site));
  if (!err) return fail(QR_EINVAL, "null output");
  if (direction != QR_DIR_LEFT && direction != QR_DIR_RIGHT) return fail(QR_EINVAL, "Unknown direction");
  QR_TRY(require_nonempty(h));
  cudaStream_t s = h->stream;
  const int cl = h->cl(site), d = h->d, cr = h->cr(site);
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  int nn = (direction == QR_DIR_LEFT) ? cr : cl;
  QR_TRY(ensure_ws(h, (size_t)nn * nn));
  if (direction == QR_DIR_LEFT) {  // A^H A over [(l,o) x r]
    QR_TRY(zgemm(s, OP_C, OP_N, cr, cr, cl * d, one, h->site[site], cl * d, 0, h->site[site], cl * d, 0, zero, h->ws, cr, 0, 1, nullptr));
  } else {  // A A^H over [l x (o,r)]
    QR_TRY(zgemm(s, OP_N, OP_C, cl, cl, d * cr, one, h->site[site], cl, 0, h->site[site], cl, 0, zero, h->ws, cl, 0, 1, nullptr));
  }
  QR_TRY(zdist_identity(s, h->ws, nn, h->scal));
  QR_CUDA(cudaMemcpyAsync(err, h->scal, sizeof(double), cudaMemcpyDeviceToHost, s));
  QR_CUDA(cudaStreamSynchronize(s));
  return QR_OK;
} QR_ABI_CATCH

int qr_truncate(qr_chain* h, int site1, int site2, double threshold, int maxdim) try {
  QR_TRY(truncate_impl(h, site1, site2, threshold, maxdim));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

// evolve_1site! (Chain.jl:586-603)
int qr_evolve_1site(qr_chain* h, int site, const double* gate) try {
  QR_TRY(check_site(h, site));
  if (!gate) return fail(QR_EINVAL, "null gate");
  QR_TRY(require_nonempty(h));
  QR_TRY(upload_gate(h, gate, h->d));
  QR_TRY(zgate1(h->stream, h->site[site], h->cl(site), h->d, h->cr(site), h->gate));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

int qr_evolve_2site(qr_chain* h, int site_l, const double* gate, double threshold, int maxdim, int iscanonical,
                    int renormalize) try {
  if (!gate) return fail(QR_EINVAL, "null gate");
  QR_TRY(evolve2_impl(h, site_l, gate, threshold, maxdim, iscanonical, renormalize));
  QR_CUDA(cudaStreamSynchronize(h->stream));
  return QR_OK;
} QR_ABI_CATCH

// A brick-wall layer of two-site gates on disjoint site pairs, several gates at a time.
// A gate on sites (s, s + 1) writes sites s and s + 1, bond s and its Lambda, and reads only bonds
// s - 1 and s + 1 (their sizes, and their Lambdas for iscanonical), which no other gate of the
// layer writes: the gates are independent, as in the reference's evolve! loop over a layer.  Each
// lane is a chain that owns a stream and the workspaces (theta, gate staging, SVD) and works on a
// shallow copy of this chain's bookkeeping (bond sizes, site and Lambda pointers); a host thread
// per lane runs its gates through evolve2_impl, and the entries each gate wrote are copied back.
// renormalize=true sweeps the whole chain per gate (normalize!), so that case runs in order.
int qr_evolve_layer(qr_chain* h, int ngates, const int* sites, const double* gates, double threshold, int maxdim,
                    int iscanonical, int renormalize, int lanes) try {
  if (!h) return fail(QR_EINVAL, "null chain");
  if (ngates < 0 || (ngates > 0 && (!sites || !gates))) return fail(QR_EINVAL, "bad gate list");
  const int g4 = 2 * h->d * h->d * h->d * h->d;  // doubles per gate matrix
  for (int i = 0; i < ngates; i++) {
    if (sites[i] < 0 || sites[i] + 1 >= h->n) return fail(QR_EINVAL, "The sites in the bond must be between 1 and n");
    for (int j = 0; j < i; j++)
      if (std::abs(sites[i] - sites[j]) < 2) return fail(QR_EINVAL, "gates of a layer must act on disjoint sites");
  }
  const int L = std::max(1, std::min(ngates, lanes > 0 ? lanes : 4));
  if (L <= 1 || renormalize) {
    for (int i = 0; i < ngates; i++)
      QR_TRY(evolve2_impl(h, sites[i], gates + (size_t)g4 * i, threshold, maxdim, iscanonical, renormalize));
    QR_CUDA(cudaStreamSynchronize(h->stream));
    return QR_OK;
  }
  QR_CUDA(cudaStreamSynchronize(h->stream));
  int dev = 0;
  QR_CUDA(cudaGetDevice(&dev));
  while ((int)h->lanes.size() < L) {
    qr_chain* l = new qr_chain();
    l->n = h->n;
    l->d = h->d;
    l->periodic = h->periodic;
    l->is_lane = true;
    cudaError_t e = cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete l; return cuda_fail(e, "cudaStreamCreate"); }
    l->svd = svd_work_create();
    int rc = dalloc((void**)&l->gate, sizeof(double2) * 256, l->stream);
    if (!rc) rc = cuda_ok(cudaHostAlloc((void**)&l->gate_host, sizeof(double2) * 256, cudaHostAllocDefault), "cudaHostAlloc");
    if (!rc) rc = dalloc((void**)&l->scal, sizeof(double) * 16, l->stream);
    h->lanes.push_back(l);
    if (rc) return rc;
  }
  for (int j = 0; j < L; j++) {
    qr_chain* l = h->lanes[j];
    l->precision = h->precision;
    l->bd = h->bd;
    l->site = h->site;
    l->lam = h->lam;
    l->lamlen = h->lamlen;
  }
  std::vector<int> rcs(L, QR_OK);
  std::vector<std::string> msgs(L);
  auto run_lane = [&](int j) {
    qr_chain* l = h->lanes[j];
    int rc = cuda_ok(cudaSetDevice(dev), "cudaSetDevice");
    try {
      for (int i = j; i < ngates && !rc; i += L)
        rc = evolve2_impl(l, sites[i], gates + (size_t)g4 * i, threshold, maxdim, iscanonical, 0);
    } catch (const std::bad_alloc&) {
      rc = fail(QR_ENOMEM, "host memory allocation failed");
    } catch (const std::exception& x) {  // nothing may leave a lane's thread
      rc = fail(QR_EHOST, std::string("host-side failure: ") + x.what());
    }
    if (!rc) rc = cuda_ok(cudaStreamSynchronize(l->stream), "lane synchronisation");
    else cudaStreamSynchronize(l->stream);
    rcs[j] = rc;
    if (rc) msgs[j] = qr_last_error_string();
  };
  std::vector<std::thread> th;
  th.reserve(L);
  for (int j = 0; j < L; j++) {
    try {
      th.emplace_back(run_lane, j);
    } catch (const std::system_error&) {
      run_lane(j);  // no thread to spare: this lane's gates run on the calling thread
    }
  }
  for (auto& t : th) t.join();
  for (int i = 0; i < ngates; i++) {  // the entries each gate wrote, from its lane's view
    const qr_chain* l = h->lanes[i % L];
    const int s0 = sites[i];
    h->site[s0] = l->site[s0];
    h->site[s0 + 1] = l->site[s0 + 1];
    h->bd[s0] = l->bd[s0];
    h->lam[s0] = l->lam[s0];
    h->lamlen[s0] = l->lamlen[s0];
  }
  for (int j = 0; j < L; j++)
    if (rcs[j]) return fail(rcs[j], msgs[j]);
  return QR_OK;
} QR_ABI_CATCH

int qr_overlap(const qr_chain* a, const qr_chain* b, double* out) try {
  if (!a || !b || !out) return fail(QR_EINVAL, "null argument");
  if (a->n != b->n || a->d != b->d) return fail(QR_EASSERT, "Ansatzes must have the same sites");
  QR_CUDA(cudaStreamSynchronize(b->stream));
  return env_sweep(a, b, nullptr, a->stream, out);
} QR_ABI_CATCH

int qr_norm(const qr_chain* h, double* out) try {
  if (!h || !out) return fail(QR_EINVAL, "null argument");
  double z[2];
  QR_TRY(env_sweep(h, h, nullptr, h->stream, z));
  *out = std::abs(std::sqrt(std::complex<double>(z[0], z[1])));
  return QR_OK;
} QR_ABI_CATCH

// expect (Chain.jl:724-735): the product operator O_{k-1}...O_0 is built as a small MPO on the
// host (bond dimension d^2 per two-site observable) and contracted in one environment sweep.
int qr_expect(const qr_chain* h, int nobs, const int* first, const int* nlanes, const double* mats, double* out) try {
  if (!h || !out) return fail(QR_EINVAL, "null argument");
  if (nobs < 0 || (nobs > 0 && (!first || !nlanes || !mats))) return fail(QR_EINVAL, "bad observable list");
  const int n = h->n, d = h->d;
  if (has_empty_bond(h)) {
    out[0] = out[1] = 0.0;
    return QR_OK;
  }
  if (h->periodic) {
    // the reference's own algorithm (Chain.jl:724-735): evolve! a copy by every observable (no
    // truncation), then contract it with the adjoint of the original (the ring sweep)
    qr_chain* c = nullptr;
    QR_TRY(qr_chain_copy(h, &c));
    int rc = QR_OK;
    size_t off = 0;
    for (int j = 0; j < nobs && !rc; j++) {
      const int s0 = first[j], nl = nlanes[j];
      if (nl != 1 && nl != 2) rc = fail(QR_EINVAL, "Invalid number of lanes, maximum is 2");
      else if (s0 < 0 || s0 + nl > n) rc = fail(QR_EINVAL, "Gate inputs must be a subset of the TN sites");
      else if (nl == 1) rc = qr_evolve_1site(c, s0, mats + 2 * off);
      else rc = qr_evolve_2site(c, s0, mats + 2 * off, NAN, -1, 0, 0);
      off += nl == 1 ? (size_t)d * d : (size_t)d * d * d * d;
    }
    if (!rc) rc = qr_overlap(c, h, out);
    qr_chain_free(c);
    return rc;
  }
  typedef std::complex<double> cd;
  // per-site operator tensors (wl, o, i, wr), wl fastest
  std::vector<std::vector<cd>> W(n);
  std::vector<int> wl(n, 1), wr(n, 1);
  for (int i = 0; i < n; i++) {
    W[i].assign(d * d, cd(0));
    for (int o = 0; o < d; o++) W[i][o + d * o] = cd(1);
  }
  std::vector<bool> touched(n, false);
  size_t off = 0;
  for (int j = 0; j < nobs; j++) {
    const int s0 = first[j], nl = nlanes[j];
    if (nl != 1 && nl != 2) return fail(QR_EINVAL, "Invalid number of lanes, maximum is 2");
    if (s0 < 0 || s0 + nl > n) return fail(QR_EINVAL, "Gate inputs must be a subset of the TN sites");
    const int dim = nl == 1 ? d : d * d;
    const cd* G = reinterpret_cast<const cd*>(mats) + off;
    off += (size_t)dim * dim;
    if (nl == 1) {
      const int s = s0, a = wl[s], b = wr[s];
      std::vector<cd> nw(W[s].size(), cd(0));
      for (int w2 = 0; w2 < b; w2++)
        for (int i = 0; i < d; i++)
          for (int o = 0; o < d; o++)
            for (int w = 0; w < a; w++) {
              cd acc(0);
              for (int mm = 0; mm < d; mm++) acc += G[o * d + mm] * W[s][w + a * (mm + d * (i + d * w2))];
              nw[w + a * (o + d * (i + d * w2))] = acc;
            }
      W[s] = nw;
      touched[s] = true;
    } else {
      // G[(o1,o2),(m1,m2)] = sum_{t=(p,c)} |p><c| (x) R_t,  R_t[o2,m2] = G[(p,o2),(c,m2)]
      const int s = s0, s2 = s0 + 1;
      const int a1 = wl[s], b1 = wr[s], a2 = wl[s2], b2 = wr[s2];
      const int T = d * d;
      std::vector<cd> n1((size_t)a1 * d * d * b1 * T, cd(0));
      for (int t = 0; t < T; t++) {
        const int p = t % d, c = t / d;
        for (int w2 = 0; w2 < b1; w2++)
          for (int i = 0; i < d; i++)
            for (int w = 0; w < a1; w++)
              n1[w + a1 * (p + d * (i + d * (w2 + b1 * t)))] = W[s][w + a1 * (c + d * (i + d * w2))];
      }
      std::vector<cd> n2((size_t)a2 * T * d * d * b2, cd(0));
      for (int t = 0; t < T; t++) {
        const int p = t % d, c = t / d;
        for (int w2 = 0; w2 < b2; w2++)
          for (int i = 0; i < d; i++)
            for (int o2 = 0; o2 < d; o2++)
              for (int w = 0; w < a2; w++) {
                cd acc(0);
                for (int m2 = 0; m2 < d; m2++)
                  acc += G[(p * d + o2) * T + (c * d + m2)] * W[s2][w + a2 * (m2 + d * (i + d * w2))];
                n2[(w + a2 * t) + (a2 * T) * (o2 + d * (i + d * w2))] = acc;
              }
      }
      W[s] = n1;
      W[s2] = n2;
      wr[s] = b1 * T;
      wl[s2] = a2 * T;
      touched[s] = touched[s2] = true;
    }
  }
  EnvOps ops;
  ops.W.assign(n, nullptr);
  ops.wl = wl;
  ops.wr = wr;
  ops.tab.resize(n);
  ops.has_tab.assign(n, 0);
  for (int i = 0; i < n; i++) {
    if (!touched[i]) continue;
    std::vector<double2> wh(W[i].size());
    for (size_t e = 0; e < wh.size(); e++) wh[e] = make_double2(W[i][e].real(), W[i][e].imag());
    ops.has_tab[i] = build_mix_table(wh.data(), wl[i], d, wr[i], &ops.tab[i]) ? 1 : 0;
  }
  std::vector<double2*> dev(n, nullptr);
  int rc = QR_OK;
  for (int i = 0; i < n && !rc; i++) {
    if (!touched[i]) continue;
    rc = dalloc((void**)&dev[i], sizeof(double2) * W[i].size(), h->stream);
    if (!rc) rc = cuda_ok(cudaMemcpyAsync(dev[i], W[i].data(), sizeof(double2) * W[i].size(), cudaMemcpyHostToDevice, h->stream), "memcpy");
    ops.W[i] = dev[i];
  }
  if (!rc) rc = env_sweep(h, h, &ops, h->stream, out);
  cudaStreamSynchronize(h->stream);
  for (auto p : dev) if (p) cudaFreeAsync(p, h->stream);
  return rc;
} QR_ABI_CATCH

int qr_mpo_create(int n, int d, const int* bond_dims, qr_mpo** out) try {
  if (!out) return fail(QR_EINVAL, "null output");
  *out = nullptr;
  if (n < 2 || d < 2 || d > 4 || !bond_dims) return fail(QR_EINVAL, "bad MPO shape");
  qr_mpo* w = new qr_mpo();
  w->n = n;
  w->d = d;
  w->bd.assign(bond_dims, bond_dims + n - 1);
  w->site.assign(n, nullptr);
  for (int i = 0; i < n; i++) {
    size_t ne = (size_t)w->wl(i) * d * d * w->wr(i);
    if (cudaMalloc(&w->site[i], sizeof(double2) * ne) != cudaSuccess) { qr_mpo_free(w); return fail(QR_ENOMEM, "MPO allocation"); }
    cudaMemset(w->site[i], 0, sizeof(double2) * ne);
  }
  *out = w;
  return QR_OK;
} QR_ABI_CATCH

int qr_mpo_free(qr_mpo* w) try {
  if (!w) return QR_OK;
  for (auto p : w->site) if (p) cudaFree(p);
  delete w;
  return QR_OK;
} QR_ABI_CATCH

int qr_mpo_upload_site(qr_mpo* w, int site, const double* host, const char* order) try {
  if (!w || site < 0 || site >= w->n || !host) return fail(QR_EINVAL, "bad MPO site");
  w->host_ok = false;
  if (!is_perm(order ? order : "", "oilr")) return fail(QR_EINVAL, "order must be a permutation of (o, i, l, r)");
  std::string ho = filtered(order, site == 0, site == w->n - 1);
  long idims[4] = {w->wl(site), w->d, w->d, w->wr(site)};
  Perm p = make_perm(ho, "loir", idims);
  size_t ne = (size_t)idims[0] * idims[1] * idims[2] * idims[3];
  double2* tmp = nullptr;
  QR_CUDA(cudaMalloc(&tmp, sizeof(double2) * ne));
  cudaError_t e = cudaMemcpy(tmp, host, sizeof(double2) * ne, cudaMemcpyHostToDevice);
  int rc = (e == cudaSuccess) ? zpermute(0, tmp, w->site[site], p) : cuda_fail(e, "cudaMemcpy");
  cudaDeviceSynchronize();
  cudaFree(tmp);
  return rc;
} QR_ABI_CATCH

int qr_mpo_download_site(const qr_mpo* w, int site, double* host, const char* order) try {
  if (!w || site < 0 || site >= w->n || !host) return fail(QR_EINVAL, "bad MPO site");
  if (!is_perm(order ? order : "", "oilr")) return fail(QR_EINVAL, "order must be a permutation of (o, i, l, r)");
  std::string ho = filtered(order, site == 0, site == w->n - 1);
  // host order gathers from the internal (l, o, i, r) layout
  long dims_by_letter[4] = {w->wl(site), w->d, w->d, w->wr(site)};  // l, o, i, r
  const std::string iord = "loir";
  long istride[4] = {1, dims_by_letter[0], dims_by_letter[0] * w->d, dims_by_letter[0] * w->d * w->d};
  Perm p;
  p.nd = (int)ho.size();
  for (int k = 0; k < p.nd; k++) {
    size_t q = iord.find(ho[k]);
    p.dims[k] = dims_by_letter[q];
    p.src_stride[k] = istride[q];
  }
  const size_t ne = (size_t)dims_by_letter[0] * w->d * w->d * dims_by_letter[3];
  double2* tmp = nullptr;
  QR_CUDA(cudaMalloc(&tmp, sizeof(double2) * ne));
  int rc = zpermute(0, w->site[site], tmp, p);
  if (!rc) {
    cudaError_t e = cudaMemcpy(host, tmp, sizeof(double2) * ne, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy");
  }
  cudaFree(tmp);
  return rc;
} QR_ABI_CATCH

int qr_mpo_expect(const qr_chain* h, const qr_mpo* w, double* out) try {
  if (!h || !w || !out) return fail(QR_EINVAL, "null argument");
  if (w->n != h->n || w->d != h->d) return fail(QR_EASSERT, "Outputs of the state must match inputs of the operator");
  EnvOps ops;
  ops.W.assign(w->site.begin(), w->site.end());
  ops.wl.resize(h->n);
  ops.wr.resize(h->n);
  for (int i = 0; i < h->n; i++) { ops.wl[i] = w->wl(i); ops.wr[i] = w->wr(i); }
  if (!w->host_ok) {  // one read-back of the (small) site tensors, kept until the next upload
    w->host_w.resize(w->n);
    for (int i = 0; i < w->n; i++) {
      w->host_w[i].resize((size_t)w->wl(i) * w->d * w->d * w->wr(i));
      QR_CUDA(cudaMemcpy(w->host_w[i].data(), w->site[i], sizeof(double2) * w->host_w[i].size(),
                         cudaMemcpyDeviceToHost));
    }
    w->host_ok = true;
  }
  ops.tab.resize(h->n);
  ops.has_tab.assign(h->n, 0);
  for (int i = 0; i < h->n; i++)
    ops.has_tab[i] = build_mix_table(w->host_w[i].data(), ops.wl[i], h->d, ops.wr[i], &ops.tab[i]) ? 1 : 0;
  return env_sweep(h, h, &ops, h->stream, out);
} QR_ABI_CATCH

}  // extern "C"

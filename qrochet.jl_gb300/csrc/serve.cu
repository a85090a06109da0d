// Request server for simulate-and-measure jobs on one GPU: continuous batching over chains that
// stay resident in device memory while their gate layers run.
//
// A request is a brick-wall circuit on |0...0> (two-site gates, evolve! with threshold and
// maxdim = chi_max) followed by Pauli-string expectation values (expect with one single-site
// observable per non-identity Pauli).  Requests enter a FIFO queue; the head is admitted when its
// device-memory footprint fits the remaining budget, so work that arrives while other requests
// run starts as soon as a worker slot and memory free up.  Each worker thread owns its request's
// chain and CUDA stream, so admitted requests overlap on the GPU.  Requests whose footprint
// exceeds the whole budget are rejected at submission (QR_ENOMEM).
#include <vector>
#include <deque>
#include <thread>
#include <mutex>
#include <condition_variable>
#include <unordered_map>
#include <memory>
#include <chrono>
#include <cmath>
#include <cstring>
#include <algorithm>
#include "kernels.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  int n = 0, chi_max = 0;
  double threshold = NAN;
  std::vector<int> gate_site;
  std::vector<double> gate_mats;  // 32 doubles (4x4 complex) per gate
  std::vector<int> obs_weight, obs_sites, obs_paulis;
  uint64_t footprint = 0;
  Clock::time_point t_submit, t_start, t_end;
  int status = QR_OK;
  std::string error;
  std::vector<double> results;  // 2 per observable
  bool done = false;
};

uint64_t footprint_bytes(int n, int chi_max) {
  // sites at their largest (chi = min(chi_max, 2^i, 2^(n-i))) plus the SVD/theta workspaces of the
  // largest two-site block (about a dozen (2 chi) x (2 chi) complex buffers)
  uint64_t sites = 0;
  for (int i = 0; i < n; i++) {
    auto bond = [&](int b) -> uint64_t {  // bond b joins sites b and b+1
      if (b < 0 || b >= n - 1) return 1;
      double c = std::min((double)chi_max, std::min(std::ldexp(1.0, std::min(b + 1, 60)),
                                                     std::ldexp(1.0, std::min(n - b - 1, 60))));
      return (uint64_t)c;
    };
    sites += 16ull * 2 * bond(i - 1) * bond(i);
  }
  const uint64_t t = 2ull * chi_max;
  return sites + 12ull * t * t * 16ull + (64ull << 20);
}

}  // namespace

struct qr_server {
  int device = 0, precision = 0;
  uint64_t budget = 0, in_use = 0;
  uint64_t next_ticket = 1, submitted = 0, completed = 0;
  int in_flight = 0;
  bool stop = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> all;
  std::vector<std::thread> workers;
};

namespace {

const double kPauli[4][8] = {
    {1, 0, 0, 0, 0, 0, 1, 0},   // I
    {0, 0, 1, 0, 1, 0, 0, 0},   // X
    {0, 0, 0, -1, 0, 1, 0, 0},  // Y
    {1, 0, 0, 0, 0, 0, -1, 0},  // Z
};

int evolve_and_measure(qr_server* sv, Request* r, qr_chain*& h) {
  std::vector<int> bd(r->n - 1, 1);
  int rc = qr_set_device(sv->device);
  if (!rc) rc = qr_chain_create(r->n, 2, bd.data(), &h);
  if (!rc) rc = qr_chain_set_precision(h, sv->precision);
  const double zero_site[4] = {1.0, 0.0, 0.0, 0.0};  // |0>: (o=2) x 1 x 1
  for (int i = 0; i < r->n && !rc; i++) rc = qr_chain_upload_site(h, i, zero_site, "olr");
  for (size_t g = 0; g < r->gate_site.size() && !rc; g++)
    rc = qr_evolve_2site(h, r->gate_site[g], r->gate_mats.data() + 32 * g, r->threshold, r->chi_max, 0, 0);
  size_t off = 0;
  r->results.assign(2 * r->obs_weight.size(), 0.0);
  for (size_t j = 0; j < r->obs_weight.size() && !rc; j++) {
    const int w = r->obs_weight[j];
    std::vector<int> first, nl;
    std::vector<double> mats;
    for (int q = 0; q < w; q++) {
      const int p = r->obs_paulis[off + q];
      if (p == 0) continue;
      first.push_back(r->obs_sites[off + q]);
      nl.push_back(1);
      mats.insert(mats.end(), kPauli[p], kPauli[p] + 8);
    }
    off += w;
    if (first.empty()) {  // identity string: <psi|psi>
      double nrm = 0;
      rc = qr_norm(h, &nrm);
      r->results[2 * j] = nrm * nrm;
      continue;
    }
    rc = qr_expect(h, (int)first.size(), first.data(), nl.data(), mats.data(), &r->results[2 * j]);
  }
  return rc;
}

// One request on a worker thread: its status and message are the request's, and no exception
// leaves the worker (a failed host allocation fails this request only).
void run_request(qr_server* sv, Request* r) {
  qr_chain* h = nullptr;
  int rc;
  try {
    rc = evolve_and_measure(sv, r, h);
  } catch (const std::bad_alloc&) {
    rc = qr::fail(QR_ENOMEM, "host memory allocation failed");
  } catch (const std::exception& x) {
    rc = qr::fail(QR_EHOST, std::string("host-side failure: ") + x.what());
  }
  if (rc) r->error = qr_last_error_string();
  r->status = rc;
  if (h) qr_chain_free(h);
}

void worker_loop(qr_server* sv) {
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] {
        return sv->stop || (!sv->pending.empty() && sv->in_use + sv->pending.front()->footprint <= sv->budget);
      });
      if (sv->stop && sv->pending.empty()) return;
      if (sv->pending.empty() || sv->in_use + sv->pending.front()->footprint > sv->budget) {
        if (sv->stop) return;
        continue;
      }
      r = sv->pending.front();
      sv->pending.pop_front();
      sv->in_use += r->footprint;
      sv->in_flight++;
      r->t_start = Clock::now();
    }
    run_request(sv, r);
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      r->t_end = Clock::now();
      r->done = true;
      sv->in_use -= r->footprint;
      sv->in_flight--;
      sv->completed++;
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int qr_server_create(int device, int workers, uint64_t hbm_budget_bytes, int precision, qr_server** out) try {
  if (!out) return qr::fail(QR_EINVAL, "null output");
  *out = nullptr;
  if (workers < 1 || workers > 256) return qr::fail(QR_EINVAL, "workers must be 1..256");
  if (precision < 0 || precision > 3) return qr::fail(QR_EINVAL, "bad precision");
  if (hbm_budget_bytes == 0) return qr::fail(QR_EINVAL, "HBM budget must be positive");
  qr_server* sv = new qr_server();
  sv->device = device;
  sv->budget = hbm_budget_bytes;
  sv->precision = precision;
  try {
    for (int i = 0; i < workers; i++) sv->workers.emplace_back(worker_loop, sv);
  } catch (const std::exception& x) {  // a worker that cannot start: stop the ones that did
    qr_server_free(sv);
    return qr::fail(QR_EHOST, std::string("cannot start the server's workers: ") + x.what());
  }
  *out = sv;
  return QR_OK;
} QR_ABI_CATCH

int qr_server_free(qr_server* sv) try {
  if (!sv) return QR_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto& t : sv->workers) t.join();
  delete sv;
  return QR_OK;
} QR_ABI_CATCH

int qr_server_footprint(int n, int chi_max, uint64_t* bytes) try {
  if (!bytes || n < 2 || chi_max < 1) return qr::fail(QR_EINVAL, "bad request shape");
  *bytes = footprint_bytes(n, chi_max);
  return QR_OK;
} QR_ABI_CATCH

int qr_server_submit(qr_server* sv, int n, int chi_max, double threshold, int ngates, const int* gate_site,
                     const double* gate_mats, int nobs, const int* obs_weight, const int* obs_sites,
                     const int* obs_paulis, uint64_t* ticket) try {
  if (!sv || !ticket) return qr::fail(QR_EINVAL, "null argument");
  if (n < 2 || chi_max < 1) return qr::fail(QR_EINVAL, "a request needs n >= 2 sites and chi_max >= 1");
  if (ngates < 0 || (ngates > 0 && (!gate_site || !gate_mats))) return qr::fail(QR_EINVAL, "bad gate list");
  if (nobs < 0 || (nobs > 0 && (!obs_weight || !obs_sites || !obs_paulis))) return qr::fail(QR_EINVAL, "bad observable list");
  auto r = std::make_unique<Request>();
  r->n = n;
  r->chi_max = chi_max;
  r->threshold = threshold;
  r->gate_site.assign(gate_site, gate_site + ngates);
  for (int g = 0; g < ngates; g++)
    if (gate_site[g] < 0 || gate_site[g] + 1 >= n) return qr::fail(QR_EINVAL, "Gate lanes must be inside the chain");
  r->gate_mats.assign(gate_mats, gate_mats + 32 * (size_t)ngates);
  size_t tot = 0;
  for (int j = 0; j < nobs; j++) {
    if (obs_weight[j] < 0 || obs_weight[j] > n) return qr::fail(QR_EINVAL, "bad Pauli string weight");
    tot += obs_weight[j];
  }
  r->obs_weight.assign(obs_weight, obs_weight + nobs);
  r->obs_sites.assign(obs_sites, obs_sites + tot);
  r->obs_paulis.assign(obs_paulis, obs_paulis + tot);
  for (size_t q = 0; q < tot; q++) {
    if (obs_sites[q] < 0 || obs_sites[q] >= n) return qr::fail(QR_EINVAL, "Pauli string site outside the chain");
    if (obs_paulis[q] < 0 || obs_paulis[q] > 3) return qr::fail(QR_EINVAL, "Pauli code must be 0..3 (I, X, Y, Z)");
  }
  r->footprint = footprint_bytes(n, chi_max);
  if (r->footprint > sv->budget) return qr::fail(QR_ENOMEM, "request footprint exceeds the server's HBM budget");
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    r->ticket = sv->next_ticket++;
    r->t_submit = Clock::now();
    *ticket = r->ticket;
    sv->pending.push_back(r.get());
    sv->all.emplace(r->ticket, std::move(r));
    sv->submitted++;
  }
  sv->cv_work.notify_all();
  return QR_OK;
} QR_ABI_CATCH

// Waits up to timeout_s (< 0: forever).  Returns QR_OK with *done = 0 on timeout.  On completion
// copies the results and timings and forgets the ticket; *status is the request's own status.
int qr_server_wait(qr_server* sv, uint64_t ticket, double timeout_s, int* done, int* status, double* results,
                   double* latency_ms, double* queue_ms) try {
  if (!sv || !done) return qr::fail(QR_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->all.find(ticket);
  if (it == sv->all.end()) return qr::fail(QR_EINVAL, "unknown ticket");
  Request* r = it->second.get();
  auto pred = [&] { return r->done; };
  if (timeout_s < 0) sv->cv_done.wait(lk, pred);
  else sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  *done = r->done ? 1 : 0;
  if (!r->done) return QR_OK;
  if (status) *status = r->status;
  if (results) std::memcpy(results, r->results.data(), sizeof(double) * r->results.size());
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_end - r->t_submit).count();
  if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
  if (r->status) qr::set_error(r->error);
  sv->all.erase(it);
  return QR_OK;
} QR_ABI_CATCH

int qr_server_stats(qr_server* sv, uint64_t* submitted, uint64_t* completed, int* in_flight, uint64_t* hbm_in_use,
                    int* queued) try {
  if (!sv) return qr::fail(QR_EINVAL, "null server");
  std::lock_guard<std::mutex> lk(sv->mu);
  if (submitted) *submitted = sv->submitted;
  if (completed) *completed = sv->completed;
  if (in_flight) *in_flight = sv->in_flight;
  if (hbm_in_use) *hbm_in_use = sv->in_use;
  if (queued) *queued = (int)sv->pending.size();
  return QR_OK;
} QR_ABI_CATCH

}  // extern "C"

/*
 * qrochet_gpu.h -- C ABI of the GB300 (sm_103a) implementation of Qrochet.jl's Chain (MPS/MPO)
 * hot path.  Plain pointers and sizes only; every call returns a status code (QR_OK == 0) and
 * leaves a message for qr_last_error_string() on failure.
 *
 * Layout conventions at the boundary (what a Julia `ccall` passes from `Array{ComplexF64}`):
 *   - complex numbers are interleaved (re, im) doubles;
 *   - site arrays are column-major with dims named by a 3-letter `order` string over
 *     {'o','l','r'} (states) or a 4-letter string over {'o','i','l','r'} (operators); the open
 *     ends omit 'l' (site 1) and 'r' (site n) exactly like Chain(State(), Open(), arrays; order);
 *   - sites and bonds are 0-based here; bond b joins sites b and b+1;
 *   - gates are row-major matrices M[(o_1..o_k),(i_1..i_k)] with the left lane slowest.
 *
 * Reference interfaces replaced (paths inside Qrochet.jl v0.1.2):
 *   Chain(State(), Open(), arrays; order)   src/Ansatz/Chain.jl:64-100
 *   Chain(Operator(), Open(), arrays)       src/Ansatz/Chain.jl:133-172
 *   copy(::Chain)                           src/Ansatz/Chain.jl:11
 *   canonize_site!                          src/Ansatz/Chain.jl:339-376
 *   truncate!                               src/Ansatz/Chain.jl:390-422
 *   canonize!                               src/Ansatz/Chain.jl:469-497
 *   mixed_canonize!                         src/Ansatz/Chain.jl:509-524
 *   normalize!(::Chain, ::Site)             src/Ansatz/Chain.jl:532-536
 *   contract!(::Chain, Val(:between))       src/Ansatz/Chain.jl:309-333
 *   evolve! / evolve_1site! / evolve_2site! src/Ansatz/Chain.jl:543-661 (+669-722 Vidal path)
 *   expect                                  src/Ansatz/Chain.jl:724-735
 *   overlap(::State, ::Chain, ::State, ::Chain)  src/Ansatz/Chain.jl:740-748
 *   LinearAlgebra.norm(::Ansatz)            src/Ansatz.jl:101-109
 *   isleftcanonical / isrightcanonical      src/Ansatz/Chain.jl:424-458
 */
#ifndef QROCHET_GPU_H
#define QROCHET_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qr_chain qr_chain; /* one open-boundary MPS resident in device memory */
typedef struct qr_mpo qr_mpo;     /* one open-boundary MPO resident in device memory */

/* Status codes; the Julia shim maps them to the reference's exceptions. */
#define QR_OK 0
#define QR_EINVAL 1       /* ArgumentError */
#define QR_EASSERT 2      /* AssertionError (@assert) */
#define QR_ENO_SCHMIDT 3  /* MissingSchmidtCoefficientsException (src/Ansatz.jl:91-99) */
#define QR_EDIM 4         /* DimensionMismatch */
#define QR_ENOMEM 5       /* device or host allocation failed */
#define QR_ECUDA 6        /* CUDA runtime error */
#define QR_ENODEV 7       /* no CUDA device */
#define QR_ENOCONV 8      /* SVD sweeps did not converge */
#define QR_EHOST 9        /* other host-side failure (a worker thread that could not start) */

/* Precision of a chain's arithmetic (qr_chain_set_precision), a bit mask. */
#define QR_FP64 0           /* plain: all ComplexF64 */
#define QR_MIXED 1          /* two-site gates whose theta has more than 16 columns: theta formed by a
                               double-float GEMM (FP32 pairs, ~2^-48, on the FP32 pipes; the gate is
                               applied in FP64), then an SVD with an FP32 Jacobi preconditioner and
                               double-float Newton-Schulz, B = A X and Jacobi polish; singular values
                               and vectors and the truncation cutoff stay FP64.  Smaller SVDs run the
                               FP64 Jacobi. */
#define QR_SPLIT_CONTRACT 2 /* environment contractions (expect, overlap, norm, MPO expectation) on
                               the BF16 tensor cores with 3-way BF16 splits, FP32 accumulation */

#define QR_DIR_LEFT 0
#define QR_DIR_RIGHT 1
#define QR_METHOD_QR 0
#define QR_METHOD_SVD 1

/* ---- library ---------------------------------------------------------------------------- */
const char* qr_last_error_string(void);
int qr_version(int* major, int* minor);
int qr_device_count(int* count);
int qr_set_device(int device);
/* number of kernels this library has launched in this process (for launch accounting) */
int qr_launch_count(uint64_t* count);

/* page-locked host buffers for host<->device copies (cudaHostAlloc). */
int qr_host_alloc(uint64_t bytes, void** ptr);
int qr_host_free(void* ptr);

/* ---- chain lifecycle (Chain.jl:64-100, :11) --------------------------------------------- */
int qr_chain_create(int n, int d, const int* bond_dims /* n-1 */, qr_chain** out);
int qr_chain_free(qr_chain* h);
/* pMPS(arrays) / Chain(State(), Periodic(), arrays) (src/Ansatz/Chain.jl:19,36-62): n bonds, the
   last between site n and site 1; every site is (o, l, r) (no open ends).  Canonical forms stay
   Open-only as in the reference (QR_EINVAL); overlap, norm, expect, evolve! (1 site, and 2 sites
   on an inner bond), truncate! and the canonicality checks work on periodic chains. */
int qr_chain_create_periodic(int n, int d, const int* bond_dims /* n */, qr_chain** out);
int qr_chain_boundary(const qr_chain* h, int* periodic);
int qr_chain_copy(const qr_chain* src, qr_chain** out);
int qr_chain_upload_site(qr_chain* h, int site, const double* host, const char* order);
int qr_chain_download_site(const qr_chain* h, int site, double* host, const char* order);
int qr_chain_site_dims(const qr_chain* h, int site, int* chi_l, int* d, int* chi_r);
int qr_chain_bond_dims(const qr_chain* h, int* out /* n-1, or n for a periodic chain */);
int qr_chain_has_lambda(const qr_chain* h, int bond, int* flag);
int qr_chain_get_lambda(const qr_chain* h, int bond, double* out, int* len);
int qr_chain_set_lambda(qr_chain* h, int bond, const double* lam, int len);
int qr_chain_ntensors(const qr_chain* h, int* out);
int qr_chain_nsites(const qr_chain* h, int* out);
int qr_chain_set_precision(qr_chain* h, int mode);
/* Checkpoint / export for a round trip with Julia, little-endian:
   "QRCHAIN1" | int32 n, d, precision, periodic | int32 bond_dims[n-1, or n when periodic]
   | uint8 has_lambda[n-1] | per site its complex128 array in the reference's (o, l, r)
   column-major layout (open ends without l / r) | per bond with has_lambda: float64 Lambda.
   No reference counterpart beyond MPS(arrays) on the Julia side. */
int qr_chain_save(const qr_chain* h, const char* path);
int qr_chain_load(const char* path, qr_chain** out);
int qr_chain_get_precision(const qr_chain* h, int* mode);
/* the cudaStream_t this chain's work is ordered on (for caller-side CUDA events) */
int qr_chain_stream(const qr_chain* h, void** stream);
int qr_chain_sync(const qr_chain* h);

/* ---- canonical forms (Chain.jl:339-376, 469-536, 309-333) ------------------------------- */
int qr_canonize_site(qr_chain* h, int site, int direction, int method);
int qr_canonize(qr_chain* h);
int qr_mixed_canonize(qr_chain* h, int center);
int qr_normalize(qr_chain* h, int root);
/* contract!(tn, Val(:between), site1, site2; direction, delete_Λ): the Lambda of the bond the two
   sites share goes into site2 (QR_DIR_RIGHT) or site1 (QR_DIR_LEFT), in either site order; the
   same site twice is QR_EASSERT, sites that share no bond (or a bond without Lambda) are left
   as they are (tensors(tn; between) finds nothing, src/Ansatz.jl:78-89). */
int qr_contract_between(qr_chain* h, int site1, int site2, int direction, int delete_lambda);
/* ||A^dagger A - I||_F of a site viewed [(l,o) x r] (left) or A A^dagger over [l x (o,r)] */
int qr_canonicality_error(const qr_chain* h, int site, int direction, double* err);

/* ---- truncation (Chain.jl:390-422): threshold NaN -> 1e-16 default; maxdim < 0 -> none -- */
int qr_truncate(qr_chain* h, int site1, int site2, double threshold, int maxdim);

/* ---- gates (Chain.jl:543-661, 669-722) --------------------------------------------------- */
int qr_evolve_1site(qr_chain* h, int site, const double* gate /* d x d */);
/* threshold NaN and maxdim < 0 together mean: no truncate! call */
int qr_evolve_2site(qr_chain* h, int site_l, const double* gate /* d^2 x d^2 */,
                    double threshold, int maxdim, int iscanonical, int renormalize);
/* A layer of two-site gates on disjoint site pairs (the inner loop of a brick-wall evolve!),
   each as qr_evolve_2site on sites[i] (0-based left site) with the gate at gates + 2 d^4 i;
   `lanes` gates run at a time on their own streams (<= 0: 4).  Replaces a loop of evolve! calls
   over one layer (Chain.jl:543-661); renormalize = 1 runs the gates one after another. */
int qr_evolve_layer(qr_chain* h, int ngates, const int* sites, const double* gates, double threshold,
                    int maxdim, int iscanonical, int renormalize, int lanes);

/* ---- contractions (Chain.jl:724-748, Ansatz.jl:101-109) ---------------------------------- */
/* <b|a> (b conjugated), written as (re, im) */
int qr_overlap(const qr_chain* a, const qr_chain* b, double* out);
int qr_norm(const qr_chain* h, double* out);
/* unnormalised <psi| O_{k-1} ... O_0 |psi>; observable j acts on lanes first[j]..first[j]+nl[j]-1
   (nl in {1,2}) with the row-major matrix starting at mats + 2*offset_j (complex entries,
   offsets packed in order) */
int qr_expect(const qr_chain* h, int nobs, const int* first, const int* nlanes,
              const double* mats, double* out);

/* ---- MPO (Chain.jl:133-172) and <psi|H|psi> (merge, src/Quantum.jl:330-348) -------------- */
int qr_mpo_create(int n, int d, const int* bond_dims /* n-1 */, qr_mpo** out);
int qr_mpo_free(qr_mpo* w);
int qr_mpo_upload_site(qr_mpo* w, int site, const double* host, const char* order);
int qr_mpo_expect(const qr_chain* h, const qr_mpo* w, double* out);
int qr_mpo_download_site(const qr_mpo* w, int site, double* host, const char* order);
/* rand(Chain, Open, State; n, p = d, chi, eltype) and rand(Chain, Open, Operator; ...)
   (src/Ansatz/Chain.jl:223-297) generated on the device: the reference's bond-dimension pattern,
   uniform [0,1) entries (complex when complex_entries) with Gram-Schmidt orthonormalised rows,
   the first site normalised.  Entries come from a counter-based generator (Philox-4x32-10) keyed
   by seed, not from Julia's RNG. */
int qr_chain_random(int n, int d, int chi, uint64_t seed, int complex_entries, qr_chain** out);
int qr_mpo_random(int n, int d, int chi, uint64_t seed, int complex_entries, qr_mpo** out);

/* ---- request server: continuous batching of simulate-and-measure requests (no reference
   counterpart; the reference has no serving layer).  A request is a circuit of two-site gates on
   |0...0> (evolve! with `threshold` and maxdim = chi_max; gate g acts on sites gate_site[g] and
   gate_site[g]+1 with the 4x4 row-major complex matrix at gate_mats + 32 g) followed by Pauli
   strings (string j: obs_weight[j] entries of (site, code 0 I / 1 X / 2 Y / 3 Z), packed).  Requests
   are admitted FIFO when their device-memory footprint (qr_server_footprint) fits the budget;
   each of `workers` threads runs one admitted request on its own chain and stream, so admitted
   requests overlap on the GPU.  Results are the unnormalised <psi|P|psi> per string (re, im). */
typedef struct qr_server qr_server;
int qr_server_create(int device, int workers, uint64_t hbm_budget_bytes, int precision, qr_server** out);
int qr_server_free(qr_server* s); /* finishes queued work, then joins the workers */
int qr_server_footprint(int n, int chi_max, uint64_t* bytes);
int qr_server_submit(qr_server* s, int n, int chi_max, double threshold, int ngates, const int* gate_site,
                     const double* gate_mats, int nobs, const int* obs_weight, const int* obs_sites,
                     const int* obs_paulis, uint64_t* ticket);
/* timeout_s < 0 waits forever; *done = 0 on timeout.  *status is the request's own status. */
int qr_server_wait(qr_server* s, uint64_t ticket, double timeout_s, int* done, int* status, double* results,
                   double* latency_ms, double* queue_ms);
int qr_server_stats(qr_server* s, uint64_t* submitted, uint64_t* completed, int* in_flight, uint64_t* hbm_in_use,
                    int* queued);

/* ---- batched engine: many independent simulate-and-measure requests evolved together (the
   batched workload; no reference counterpart beyond the per-chain calls it fuses: evolve! +
   truncate!, Chain.jl:606-661 and 390-422, and expect, Chain.jl:724-735).  Requests have the
   qr_server_submit format (a gate circuit on |0...0>, then Pauli strings) with chi_max <= 64.
   qr_batch_run keeps every chain in fixed-capacity device buffers, takes each truncation decision
   on the device, runs each brick-wall layer of all requests as one fused launch (one CTA per
   gate: theta, gate, Jacobi SVD, truncation, write-back), captures the whole circuit and the
   expectation sweep in one CUDA graph and launches it once.  The layer kernel's CTA size is
   autotuned per device and bond class (cached in the process, and in the file named by
   QROCHET_TUNE_FILE when set).  A request whose truncation would empty a bond, or whose SVD did
   not converge, gets a nonzero status (QR_EINVAL / QR_ENOCONV) in qr_batch_result. */
typedef struct qr_batch qr_batch;
int qr_batch_create(int device, qr_batch** out);
int qr_batch_free(qr_batch* b);
/* QR_FP64 (default): every gate's SVD in FP64.  QR_MIXED: SVDs of more than 32 columns run FP32
   Jacobi sweeps first, one FP64 Newton-Schulz step on their rotations, then FP64 sweeps to the
   FP64 tolerance; singular values, vectors and truncation decisions stay FP64.  Before run. */
int qr_batch_set_precision(qr_batch* b, int mode);
int qr_batch_add(qr_batch* b, int n, int chi_max, double threshold, int ngates, const int* gate_site,
                 const double* gate_mats, int nobs, const int* obs_weight, const int* obs_sites,
                 const int* obs_paulis, int* id);
/* layer of every gate of request id (a gate starts a new layer when it shares a site with the
   current one); host-only */
int qr_batch_plan(const qr_batch* b, int id, int* layer_of_gate, int* nlayers);
int qr_batch_run(qr_batch* b, double* ms);
int qr_batch_result(const qr_batch* b, int id, int* status, double* values /* 2 per string */);
int qr_batch_bond_dims(const qr_batch* b, int id, int* out /* n-1 */);
int qr_batch_lambda(const qr_batch* b, int id, int bond, double* out, int* len);
int qr_batch_info(const qr_batch* b, int* layers, int* launches, int* graph_nodes, int* warps, int* cached,
                  double* run_ms, double* tune_ms);

/* ---- allocation-free thin SVD (no counterpart in the reference) ----------------------------
   For callers that must not have a library allocate device memory (a Julia process whose CUDA.jl
   pool owns the device, a serving loop that allocates only at start-up).  Plain FP64 Jacobi SVD
   A = U diag(S) Vh of the column-major m x n A, all in caller-owned device buffers (complex
   interleaved; U m x k, S k doubles, Vh k x n, k = min(m,n)), ordered on `stream` (a
   cudaStream_t, 0 = legacy default) and complete on return.  Limit: max(m,n) <= 512 and
   min(m,n) <= 256, larger sizes return QR_EINVAL.  Scratch is one ~5.3 MB static device array per
   device, reserved while the library is loaded and shared by all calls: calls that overlap on the
   GPU (other threads or streams) race on it.  The first call on a device looks up the array's
   device address; make that first call before any stream capture.  No cudaMalloc/cudaFree. */
int qr_svd_noalloc(int m, int n, const double* A, long lda, double* U, long ldu, double* S, double* Vh,
                   long ldvh, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QROCHET_GPU_H */

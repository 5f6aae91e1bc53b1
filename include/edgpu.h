/*
 * edgpu — C ABI of the GB300 exact-diagonalization engine (libedgpu.so).
 *
 * Every entry point takes plain device pointers and sizes, never allocates device memory
 * (scratch comes from a caller-provided workspace sized by the matching *_workspace query),
 * runs on the caller's CUDA stream and returns an edgpu_status.  Device-side conditions
 * (buffer overflow, Lanczos breakdown, NaN) are written to a caller-provided int32 device
 * status word, which the caller reads after synchronising the stream.
 *
 * Product states: n_words = ceil(n_spin_orbitals / 64) uint64 words per state, stored
 * contiguously (array of structures).  Orbital i is bit 63 - (i % 64) of word i / 64, so
 * lexicographic word order equals the order of the upstream big-endian ``bytes`` states.
 * n_words must be 1..8 (up to 512 spin-orbitals).
 *
 * Complex numbers are interleaved (re, im) doubles or floats.
 *
 * Each declaration names the upstream (impurityModel) interface it replaces.
 */
#ifndef EDGPU_H
#define EDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum edgpu_status {
  EDGPU_OK = 0,
  EDGPU_ERR_ARG = 1,        /* bad argument (upstream: ValueError / Exception on bad input) */
  EDGPU_ERR_OVERFLOW = 2,   /* a per-state scratch buffer or output capacity was exceeded */
  EDGPU_ERR_BREAKDOWN = 3,  /* Lanczos beta == 0 (upstream: ValueError, finite.py:1963,1988) */
  EDGPU_ERR_NAN = 4,        /* non-finite value produced */
  EDGPU_ERR_NOCONV = 5,     /* iteration cap reached before convergence */
  EDGPU_ERR_CUDA = 6,       /* a CUDA launch or runtime call failed */
  EDGPU_ERR_WORKSPACE = 7   /* workspace smaller than the matching *_workspace query */
} edgpu_status;

/* Filters of edgpu_apply_columns. */
enum { EDGPU_FILTER_NONE = 0, EDGPU_FILTER_IN_BASIS = 1, EDGPU_FILTER_NOT_IN_BASIS = 2 };

/*
 * Compiled operator (term table), device arrays of n_terms entries.
 *   ops[t]   : up to 4 elementary operators, 16 bits each, slot k = k-th operator of the
 *              upstream process tuple (left to right).  Slot bits: 15 present, 14 creation
 *              (0 = annihilation), 0..9 spin-orbital index.  Applied right to left.
 *   coeff[t] : complex128 amplitude (re, im).
 *   flags[t] : bit 0 set when the creation and annihilation index multisets are equal
 *              (the term maps a product state onto itself); bits 8..10 operator count.
 */
typedef struct edgpu_terms {
  const uint64_t* ops;
  const double* coeff;
  const uint32_t* flags;
  int32_t n_terms;
} edgpu_terms;

/*
 * Occupation restrictions ``{frozenset(indices): (lo, hi)}`` (upstream finite.applyOp
 * ``restrictions``): a state passes when lo <= popcount(state & mask[r]) <= hi for all r.
 * Host memory; copied into the kernel parameters.
 */
#define EDGPU_MAX_RESTRICTIONS 8
#define EDGPU_MAX_WORDS 8
typedef struct edgpu_restrictions {
  int32_t n;
  int32_t lo[EDGPU_MAX_RESTRICTIONS];
  int32_t hi[EDGPU_MAX_RESTRICTIONS];
  uint64_t mask[EDGPU_MAX_RESTRICTIONS][EDGPU_MAX_WORDS];
} edgpu_restrictions;

/* CSR matrix on the device: row_ptr[n+1], col[nnz], values complex (val_c) or real (val_r). */
typedef struct edgpu_csr {
  int64_t n;
  int64_t nnz;
  const int64_t* row_ptr;
  const int32_t* col;
  const double* val_c;  /* complex128 values, or NULL */
  const double* val_r;  /* real float64 values (used when val_c is NULL) */
  const float* val_cf;  /* complex64 copy for the mixed-precision form, or NULL */
  const float* val_rf;  /* float32 copy for the mixed-precision form, or NULL */
  const float* val_df;  /* real values as (hi, lo) float pairs, hi + lo = value to ~2^-48
                           relative, for the double-float Lanczos form; or NULL */
} edgpu_csr;

/* Bumped whenever a struct layout or a signature changes. */
#define EDGPU_ABI_VERSION 2
int edgpu_abi_version(void);
const char* edgpu_status_string(int status);

/*
 * H|b> for each single product state b of ``states`` (n_states x n_words).
 * Replaces upstream ``applyOp(n, hOp, {b: 1}, weight_min, restrictions)``
 * (impurityModel/ed/finite.py:1301-1511) as called per basis column by
 * ``get_hamiltonian_matrix`` (finite.py:1514-1610) and ``expand_basis`` (finite.py:1696-1803).
 * Per state: values of equal output states are summed in term order, entries with
 * |v|^2 < weight_min are dropped, outputs failing ``restr`` are dropped, and ``filter``
 * keeps only outputs present in / absent from the sorted ``basis``.  Entries are emitted
 * in upstream dict order (first occurrence in term order).
 *
 * Count pass: offsets == NULL; writes counts[n_states].
 * Fill pass : offsets[n_states] (exclusive scan of counts); writes any of out_states
 *             (n_words each), out_index (position in basis, FILTER_IN_BASIS) and out_vals
 *             (complex128; conjugated when conj_vals != 0).
 * scratch_entries: per-warp capacity for off-diagonal emissions (0 = default 256); on
 * overflow *status_dev receives EDGPU_ERR_OVERFLOW and the caller retries larger.
 * Work per state: with a power-of-two capacity and a term index that fits in shared memory,
 * only the terms whose created orbitals are empty in the state are tried (terms bucketed by
 * created orbital per block) and equal outputs are merged through a hash table; otherwise
 * every term is tried on every state.  Both give the same outputs bit for bit.
 */
int edgpu_apply_columns(int n_words, const uint64_t* states, int64_t n_states, const edgpu_terms* terms,
                        const edgpu_restrictions* restr, double weight_min, const uint64_t* basis,
                        int64_t n_basis, int filter, const int64_t* offsets, int64_t* counts,
                        uint64_t* out_states, int64_t* out_index, double* out_vals, int conj_vals,
                        int scratch_entries, int32_t* status_dev, void* stream);

/*
 * Raw emissions of an operator on a multi-configurational state psi = sum_k amps[k] |states[k]>.
 * Replaces the inner loops of upstream ``applyOp`` (finite.py:1355-1388): for every
 * (state k, term t) in that order the valid result amps[k] * h_t * sign is emitted; outputs
 * failing ``restr`` are skipped (upstream checks restrictions on first insertion, which is
 * the same filter).  Count pass (offsets == NULL) writes counts[n_states]; the fill pass
 * writes out_states (n_words each) and out_vals (complex128, product without fused
 * multiply-add, as CPython computes it) at offsets[k] + rank in term order.
 */
int edgpu_apply_vector(int n_words, const uint64_t* states, const double* amps, int64_t n_states,
                       const edgpu_terms* terms, const edgpu_restrictions* restr, const int64_t* offsets,
                       int64_t* counts, uint64_t* out_states, double* out_vals, void* stream);

/*
 * Stable LSD radix sort of n keys (n_words each) carrying a uint32 payload.  Replaces the
 * ``sorted(...)`` of upstream ``expand_basis`` (finite.py:1793) and the dict merging of
 * ``applyOp``.  keys/payload are sorted in place (results written back to the inputs).
 * vary_mask: OR over keys of (key XOR first key), n_words host words (NULL = all bits);
 * digits where it is zero are skipped.  Inputs with n <= 8192 and
 * next_pow2(n) * (8 n_words + 4) <= 160 KiB are sorted by one CTA in shared memory (bitonic
 * network over (key, position), the same stable order) and need no workspace.
 */
size_t edgpu_sort_states_workspace(int n_words, int64_t n);
int edgpu_sort_states(int n_words, uint64_t* keys, uint32_t* payload, int64_t n, const uint64_t* vary_mask,
                      void* workspace, size_t workspace_bytes, void* stream);

/* OR over rows of (row XOR row 0) into vary_out[n_words] (device). */
int edgpu_vary_mask(int n_words, const uint64_t* keys, int64_t n, uint64_t* vary_out, void* stream);

/*
 * Exclusive prefix sum of int64 ``in`` (n entries) into ``out`` (n + 1 entries; out[n] = total).
 */
size_t edgpu_scan_workspace(int64_t n);
int edgpu_scan_i64(const int64_t* in, int64_t* out, int64_t n, void* workspace, size_t workspace_bytes,
                   void* stream);

/*
 * Segment heads of sorted keys: head[i] = 1 if i == 0 or keys[i] != keys[i-1] (int64 0/1).
 */
int edgpu_segment_heads(int n_words, const uint64_t* keys, int64_t n, int64_t* head, void* stream);

/*
 * Compact sorted keys by segment: for every head i (head_scan[i+1] != head_scan[i]) write
 * keys[i] to out_keys[head_scan[i]], the first payload to out_first[head_scan[i]] and, when
 * vals != NULL, the sequential sum (in sorted order) of vals[payload[j]] over the segment
 * into out_vals.  Replaces upstream dict accumulation ``psiNew[s] += amp * h * sign``.
 */
int edgpu_segment_reduce(int n_words, const uint64_t* keys, const uint32_t* payload, int64_t n,
                         const int64_t* head_scan, const double* vals, uint64_t* out_keys, uint32_t* out_first,
                         double* out_vals, void* stream);

/*
 * Merge two sorted, disjoint state arrays a (na) and b (nb) into out (na + nb).
 * Replaces ``basis += sorted(basis_new)`` bookkeeping of upstream expand_basis, kept sorted.
 */
int edgpu_merge_states(int n_words, const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb, uint64_t* out,
                       void* stream);

/* Position of each query state in the sorted basis, or -1 (upstream ``basis_index`` dict). */
int edgpu_lookup_states(int n_words, const uint64_t* basis, int64_t n_basis, const uint64_t* query, int64_t nq,
                        int64_t* out_index, void* stream);

/*
 * y = H x for R vectors (row-major, complex128): x is [ncols][R] where ncols exceeds every
 * column index of H, y is [n][R].  Replaces ``h.dot(v)`` of upstream
 * get_tridiagonal_krylov_vectors (finite.py:1946-1989).
 */
int edgpu_spmv(const edgpu_csr* h, const double* x, double* y, int R, void* stream);

/* Same with complex64 vectors and float32 accumulation (mixed-precision form). */
int edgpu_spmv_c64(const edgpu_csr* h, const float* x, float* y, int R, void* stream);

/*
 * Row schedule for edgpu_spmv_planned (built once per matrix).  sched[n] (device, int32)
 * receives the rows in service order: first the *n_heavy (host) rows with at least
 * heavy_min entries, longest first, each served by a whole warp; then the other rows sorted
 * by length (longest first, stable) within windows of `window` consecutive rows (0: one
 * window).  Synchronises the stream (reads the heavy-row count).  n < 2^31.
 * The same y = H x as edgpu_spmv (h.dot of upstream get_tridiagonal_krylov_vectors,
 * finite.py:1946-1989); the schedule only changes which threads serve which rows.
 */
size_t edgpu_spmv_plan_workspace(int64_t n);
int edgpu_spmv_plan(const edgpu_csr* h, int64_t window, int heavy_min, int32_t* sched, int64_t* n_heavy,
                    void* workspace, size_t workspace_bytes, void* stream);
/*
 * y = H x with a row schedule from edgpu_spmv_plan: x [ncols][R], y [n][R] complex128 (or
 * complex64 with float32 accumulation for the _c64 form), 16-byte aligned; R a multiple of
 * the complex numbers per 16 bytes (1 for complex128, 2 for complex64) with R / that count
 * dividing 32.  unroll (gathers in flight per lane: 2, 4 or 8) and block (threads per block:
 * 64, 128, 256 or 512) are launch choices that leave the result unchanged up to the order
 * of the additions in heavy rows.  Replaces upstream's h.dot (finite.py:1946-1989).
 */
int edgpu_spmv_planned(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int unroll, int block,
                       const double* x, double* y, int R, void* stream);
int edgpu_spmv_planned_c64(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int unroll, int block,
                           const float* x, float* y, int R, void* stream);

/*
 * Paged copy of a scheduled matrix, for edgpu_spmv_paged[_c64].  In schedule order, each
 * heavy row (sched[0..n_heavy)) is a slice of its own whose entries are dealt in turn to the
 * 32 / lanes row groups of a warp (lanes = R / complex numbers per 16 bytes: the lanes serving
 * one row), and the light rows follow, 32 / lanes per slice; slices are packed whole into
 * pages of page_entries (256, 512 or 1024) entries: a header column, then per slice a header
 * column (its rows, heavy flag) and its entry columns.  Entries are 8 bytes (value_kind 0: real
 * float32 values from val_rf) or 16 bytes (1: real float64 from val_r; 2: complex64 from
 * val_cf).  Writes *n_pages; returns EDGPU_ERR_OVERFLOW without filling when it exceeds
 * cap_pages or pages is NULL (call again with room for *n_pages pages, 16-byte aligned), and
 * EDGPU_ERR_ARG when a slice does not fit a page.  Synchronises the stream.  No counterpart
 * upstream (a layout of upstream's sparse H for the product below).
 */
size_t edgpu_spmv_pages_workspace(int64_t n, int lanes);
int edgpu_spmv_pages_build(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int lanes, int page_entries,
                           int value_kind, void* pages, int64_t cap_pages, int64_t* n_pages, void* workspace,
                           size_t workspace_bytes, void* stream);
/*
 * y = H x from the pages of edgpu_spmv_pages_build, one launch: a warp copies one page into
 * shared memory with cp.async and gathers the x rows its columns name, unroll (4 or 8) per
 * lane in flight; heavy rows' partial sums are added across the warp's row groups with xor
 * shuffles.  flags bit 0: the next batch's gathers are issued before the current batch is
 * added up (two batches in flight); bit 1: L2 eviction hints (x rows evict-last, pages
 * evict-first).  Vectors as edgpu_spmv_planned; R / (complex numbers per 16 bytes) in {2, 4,
 * 8, 16} and equal to the lanes the pages were built for.  complex128 H values have no paged
 * form (EDGPU_ERR_ARG).  Replaces upstream's h.dot (finite.py:1946-1989).
 */
int edgpu_spmv_paged(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries, int unroll, int flags,
                     const double* x, double* y, int R, void* stream);
int edgpu_spmv_paged_c64(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries, int unroll,
                         int flags, const float* x, float* y, int R, void* stream);

/*
 * The same product from the same pages with the x rows brought into shared memory by the
 * tensor memory accelerator: each page column's x rows (one per row group) are fetched by
 * cp.async.bulk.tensor tile::gather4 copies (four rows each, from a 2-D tensor map of x) into a
 * ring of `slots` (2..32) column buffers per warp with one mbarrier each; lane 0 keeps `slots`
 * columns in flight and the lanes add the products from shared memory.  complex64 vectors, R in
 * {4, 8, 16, 32} (pages built for R / 2 lanes), page_entries in {256, 512, 1024}, x and y
 * 16-byte aligned, n < 2^31; y equals edgpu_spmv_paged_c64's bit for bit.  Waits are bounded: a
 * barrier that does not complete sets *status_dev = EDGPU_ERR_NOCONV (y then incomplete).
 * Replaces upstream's h.dot (finite.py:1946-1989).
 */
int edgpu_spmv_paged_tma_c64(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries, int slots,
                             const float* x, float* y, int R, int32_t* status_dev, void* stream);

/*
 * Batched Lanczos tridiagonalisation without reorthogonalisation, R independent runs on one
 * CSR matrix.  Replaces upstream ``get_tridiagonal_krylov_vectors`` (finite.py:1897-1995):
 * same recurrence (alpha_j = Re<H v_j, v_j>, w = H v_j - alpha_j v_j - beta_{j-1} v_{j-1},
 * beta_j = ||w||).  v0: [n][R] normalised start vectors (complex128, read only).
 * k_max[R]: per-run Krylov size (upstream min(krylovSize, dim of the run's basis)).
 * K = max over k_max.  Outputs alpha[R][K], beta[R][K] (beta[r][j] for j < k_max[r]-1).
 * precision: 0 = complex128 vectors and values; 1 = complex64 vectors, float32 SpMV
 * accumulation, float64 alpha/beta reductions; 3 = double-float vectors and values
 * (each number an unevaluated sum of two floats, ~48 significand bits, from h->val_df),
 * float64 alpha/beta reductions, for real H in the shared-memory path; precision 3
 * anywhere else runs as 0.  Breakdown (beta == 0 before k_max) sets
 * *status_dev = EDGPU_ERR_BREAKDOWN.  Sectors whose three Krylov vectors fit in shared
 * memory run as one persistent launch with one CTA per run; larger ones as three
 * grid-wide kernels per step.  In the double-float form the CTA keeps one vector in shared
 * memory and the previous one in the workspace, and, when the workspace size returned for
 * (n, R, K) also holds it, reads H through a sliced copy (rows sorted by length in 32-row
 * column-major slices) that one extra launch builds in the workspace; a matrix whose rows
 * repeat a column then sets *status_dev = EDGPU_ERR_WORKSPACE.
 */
size_t edgpu_lanczos_workspace(int64_t n, int R, int K, int precision);
int edgpu_lanczos(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, int precision,
                  double* alpha, double* beta, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                  void* stream);

/*
 * edgpu_lanczos with CUDA-event timing of its kernels on the launching stream:
 * kernel_ms (host, 3 doubles) receives the summed milliseconds of the SpMM + alpha,
 * axpy + beta and normalise launches.  Synchronises on the last event before returning.
 */
int edgpu_lanczos_timed(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, int precision,
                        double* alpha, double* beta, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                        void* stream, double* kernel_ms);

/* Number of kernels the library has launched in this process so far. */
long long edgpu_launch_count(void);

/*
 * edgpu_lanczos without any device allocation by the caller or the library, for callers
 * that cannot allocate device memory: for instance a host code whose memory manager owns
 * the whole GPU and forbids cudaMalloc, or a solver loop embedded in another program where
 * an allocation would synchronise the device between time steps.  The caller passes the
 * inputs and outputs of edgpu_lanczos (no workspace); this always runs the grid-wide
 * batched Lanczos (three kernels per step) and keeps its scratch (three [n][R] vectors
 * and partial sums, size edgpu_lanczos_workspace(n, R, K, precision)) in a static
 * device array of EDGPU_LANCZOS_NOALLOC_BYTES inside the library, which every GPU that
 * loads the library holds until the process exits.  Larger problems are rejected with
 * EDGPU_ERR_WORKSPACE before anything runs.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress,
 * with that device current); make that first call before any stream capture.
 * The looked-up address is cached per device index for the life of the process.  It is
 * not valid after cudaDeviceReset or after the device's primary context is destroyed and
 * created again: a caller that resets a device calls edgpu_lanczos_noalloc_forget() before
 * the next edgpu_lanczos_noalloc, which then looks the address up again.
 * All calls share the one array: calls that overlap on the GPU (different streams, or
 * threads without ordering) race on it and must be serialised by the caller.  No part of
 * the scratch needs to start at zero.  precision: 0, 1 or 3 as in edgpu_lanczos (3 runs
 * as 0 here); other values return EDGPU_ERR_ARG.
 * No counterpart in upstream impurityModel.
 */
#define EDGPU_LANCZOS_NOALLOC_BYTES (16u << 20)
int edgpu_lanczos_noalloc(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, int precision,
                          double* alpha, double* beta, int32_t* status_dev, void* stream);
/* Size in bytes of the static scratch array of edgpu_lanczos_noalloc
 * (EDGPU_LANCZOS_NOALLOC_BYTES of the library that was built).  No counterpart upstream. */
size_t edgpu_lanczos_noalloc_bytes(void);
/* Drops the cached device addresses of that array (all devices); the next
 * edgpu_lanczos_noalloc on a device looks its address up again.  Call it after a device
 * reset.  No counterpart in upstream impurityModel. */
void edgpu_lanczos_noalloc_forget(void);

/*
 * Lanczos with full (twice classical Gram-Schmidt) reorthogonalisation, one run, complex128,
 * storing the Krylov basis V[K_cap][n].  Runs steps j0 .. j1-1 (resumable: the caller keeps
 * V, alpha, beta and the work vector between calls).  Step j0 == 0 copies v0 into V[0].
 * Replaces upstream ``scipy.sparse.linalg.eigsh(which="SA")`` in ``eigensystem``
 * (finite.py:105) and the BiCGSTAB solves of ``getRIXSmap`` (spectra.py:962,1080) through
 * Ritz pairs and shifted tridiagonal solves on the host.
 * w: work vector [n] complex128 (carries H v_{j} - ... between calls).
 * Sectors with n <= 65536 run each call as one cooperative launch (one block per SM, the
 * phases of a step separated by grid barriers); larger ones, or devices without cooperative
 * launch, as seven grid-wide kernels per step.
 */
size_t edgpu_lanczos_reorth_workspace(int64_t n, int K_cap);
int edgpu_lanczos_reorth(const edgpu_csr* h, const double* v0, int j0, int j1, int K_cap, double* V, double* w,
                         double* alpha, double* beta, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                         void* stream);
/*
 * The same reorthogonalised Lanczos in double-float arithmetic (float hi/lo pairs, about 48
 * significand bits, on the FP32 pipe) for a real H with its val_df copy set and n <= 65536,
 * as one cooperative launch per call.  V and w hold double-float elements (re.hi, re.lo,
 * im.hi, im.lo as floats; 16 bytes like complex128); v0 is complex128; alpha and beta FP64.
 * V[j] is written by step j itself (v_{j+1} = w / beta_j is formed by the next call's first
 * step), so after steps j0 .. j1-1 V holds v_0 .. v_{j1-1} and w the unnormalised
 * remainder.  Same workspace as edgpu_lanczos_reorth.  EDGPU_ERR_ARG for a complex H, a
 * missing val_df, n > 65536 or a device without cooperative launch.  No counterpart in
 * upstream impurityModel (an arithmetic form of the call above).
 */
int edgpu_lanczos_reorth_df(const edgpu_csr* h, const double* v0, int j0, int j1, int K_cap, double* V, double* w,
                            double* alpha, double* beta, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                            void* stream);
/* Process-wide launch policy (default 0): CTA slots per SM that the double-float
 * one-CTA-per-run Lanczos of edgpu_lanczos (precision 3, small sectors) leaves free, so that
 * work on another stream can run beside it.  No counterpart in upstream impurityModel. */
void edgpu_set_small_reserve(int slots);
/* Process-wide launch choice (default -1): the CTA size of the double-float one-CTA-per-run
 * Lanczos of edgpu_lanczos (precision 3, small sectors) as an index into {512, 256, 192, 160,
 * 128} threads, or -1 for the built-in rule (fewest waves with a slot per SM kept back).  The
 * engine's autotuner times the choices per problem bucket and sets the fastest around each
 * call; the size changes the order of the block reductions, not the recurrence.  No
 * counterpart in upstream impurityModel. */
void edgpu_set_lanczos_cta(int index);
/* Process-wide switch (default 1): 0 sends every edgpu_lanczos_reorth call to the
 * per-step kernels (both paths compute the same recurrence; used to test one against the
 * other).  No counterpart in upstream impurityModel. */
void edgpu_set_reorth_fused(int enabled);

/*
 * Matrix-free H·v on a sorted sector basis (n states, n_words words each), for sectors whose
 * CSR is not kept.  Upstream builds the same matrix elements column by column with applyOp
 * (impurityModel/ed/finite.py:1514-1693) and multiplies with h.dot (finite.py:1946-1989).
 * The operator comes split in two term tables (edgpu_terms encoding):
 *   diagonal terms (those that map a product state onto itself): edgpu_hv_diag sums them per
 *     basis state into d[n] (FP64, term order) once per sector;
 *   off-diagonal terms, sorted by their key orbital (the first orbital a term creates without
 *     annihilating it, which must be empty in the state it acts on); bucket[k]..bucket[k+1]
 *     (host-built, device array of n_orb + 1 offsets) are the terms of key orbital k.
 * edgpu_hv_matfree: y = (H - shift I) x for R vectors ([n][R], complex128, or complex64 with
 * float32 accumulation for the _c64 form; 16-byte aligned; R / complex numbers per 16 bytes
 * dividing 32).  Row i applies only the terms keyed on the empty orbitals of b_i, keeps the
 * results inside ``restr`` and the basis (binary search), and adds conj(h) x_j; the diagonal
 * (d_i - shift) x_i.  complex_terms = 0 when every coefficient is real.
 */
int edgpu_hv_diag(int n_words, const uint64_t* basis, int64_t n, const edgpu_terms* diag_terms, double* d,
                  void* stream);
/* Open-addressing hash of the basis states for the lookups of edgpu_hv_matfree: table
 * (device int32, table_size a power of two >= 2 n) receives basis indices (-1 = empty);
 * replaces upstream's basis_index dict (finite.py:1613-1693). */
int edgpu_state_hash_build(int n_words, const uint64_t* basis, int64_t n, int32_t* table, int64_t table_size,
                           void* stream);
/* table: the hash of edgpu_state_hash_build (lookups by one or two probes), or NULL (binary
 * search in the sorted basis). */
int edgpu_hv_matfree(int n_words, const uint64_t* basis, int64_t n, const int32_t* table, int64_t table_size,
                     int n_orb, const int32_t* bucket, const edgpu_terms* offdiag_terms, int complex_terms,
                     const edgpu_restrictions* restr, const double* diag, double shift, const double* x, double* y,
                     int R, void* stream);
int edgpu_hv_matfree_c64(int n_words, const uint64_t* basis, int64_t n, const int32_t* table, int64_t table_size,
                         int n_orb, const int32_t* bucket, const edgpu_terms* offdiag_terms, int complex_terms,
                         const edgpu_restrictions* restr, const double* diag, double shift, const float* x, float* y,
                         int R, void* stream);

/*
 * Pieces of a batched Lanczos with full reorthogonalisation for large sectors (R runs; a
 * Krylov vector is [n][R] complex, the basis V[m][n][R] with `stride` complex numbers between
 * consecutive vectors; precision 1: complex64 vectors, 0: complex128).  Reductions are
 * accumulated in FP64 (each thread's partial over up to 8 rows in the vector type, then FP64,
 * blocks summed in a fixed order).  Used as: w = H v_j; h = V[0..j]^H w; w -= V h (alpha_j =
 * Re h_j); again; beta_j = |w|; v_{j+1} = w / beta_j.  Replaces upstream's recurrence
 * (finite.py:1897-1995) where a complex64 recurrence without reorthogonalisation would lose
 * orthogonality.
 *   edgpu_krylov_dot:       h[k][r] = sum_i conj(V[k][i][r]) w[i][r], k < m (complex128 out).
 *   edgpu_krylov_project:   w[i][r] -= sum_k h[k][r] V[k][i][r]; with_norm: leaves per-block
 *                           |w|^2 partials in the workspace for edgpu_krylov_normalize.
 *   edgpu_krylov_normalize: beta[r] = |w[.][r]| (FP64) and v = w / beta; beta == 0 sets
 *                           *status_dev = EDGPU_ERR_BREAKDOWN and v = 0 for that run.
 * R <= 256.  The workspace (edgpu_krylov_workspace for the largest m) is shared by the three.
 */
size_t edgpu_krylov_workspace(int64_t n, int R, int m_max);
int edgpu_krylov_dot(int precision, const void* V, int64_t stride, int m, int64_t n, int R, const void* w, double* h,
                     void* workspace, size_t workspace_bytes, void* stream);
int edgpu_krylov_project(int precision, const void* V, int64_t stride, int m, int64_t n, int R, const double* h,
                         void* w, int with_norm, void* workspace, size_t workspace_bytes, void* stream);
int edgpu_krylov_normalize(int precision, int64_t n, int R, const void* w, void* v, double* beta, int32_t* status_dev,
                           void* workspace, size_t workspace_bytes, void* stream);

/*
 * Shifted solves X[r][z] = (zs[r][z] - H)^{-1} Y[r] for n_rhs right-hand sides (Y: [n_rhs][n]
 * complex128) and nz <= 512 complex shifts each, from one Krylov space per right-hand side
 * (Lanczos, FP64, CTA per right-hand side), iterated until every shift's residual estimate
 * ||r|| / ||y|| <= tol or k_cap steps.  X: [n_rhs][nz][n] complex128; m_out[r]: Krylov size
 * used.  Replaces upstream's BiCGSTAB per incoming energy in getRIXSmap (spectra.py:962,1080).
 * Requires 3 * n * 16 bytes of shared memory <= 200 KiB.
 */
size_t edgpu_shifted_solve_workspace(int64_t n, int n_rhs, int nz, int k_cap);
int edgpu_shifted_solve(const edgpu_csr* h, const double* Y, int n_rhs, const double* zs, int nz, int k_cap,
                        double tol, double* X, int32_t* m_out, int32_t* status_dev, void* workspace,
                        size_t workspace_bytes, void* stream);
/*
 * The same solves with the Krylov recurrence in double-float arithmetic (float hi/lo pairs,
 * about 48 significand bits, on the FP32 pipe) for a real H with its val_df copy set; the
 * residual estimate that decides when to stop runs in FP32, the tridiagonal solves in FP64
 * and the assembly of X in double-float.  Same arguments, workspace and outputs.
 * EDGPU_ERR_ARG for a complex H or without val_df.  No counterpart in upstream
 * impurityModel (an arithmetic form of the solves above).
 */
int edgpu_shifted_solve_df(const edgpu_csr* h, const double* Y, int n_rhs, const double* zs, int nz, int k_cap,
                           double tol, double* X, int32_t* m_out, int32_t* status_dev, void* workspace,
                           size_t workspace_bytes, void* stream);

/* X[m][n] = sum_k C[k][m] V[k][n] (complex128): Ritz vectors / shifted-solve solutions. */
int edgpu_combine(const double* V, int K, int64_t n, const double* C, int M, double* X, void* stream);

/*
 * Ragged batches: the sectors of many models (different sizes and Hamiltonians) concatenated
 * into one CSR.  The edgpu_csr then holds the concatenated row_ptr (global offsets into col
 * and the values) and column indices LOCAL to each sector.  Sector s owns rows
 * [sec_row0[s], sec_row0[s+1]); run r works on sector run_sec[r] and its vectors live at
 * offset run_vec0[r] of packed complex128 arrays (run_vec0[r+1] - run_vec0[r] = the sector's
 * size).  max_rows (host) bounds every sector size used by the runs.
 * Replaces upstream's one-model-at-a-time calls (eigensystem, finite.py:58-118, and getGreen,
 * spectra.py:551-681) for an ensemble of models; no single upstream function takes a batch.
 */
typedef struct edgpu_ragged {
  int32_t n_sectors;
  int32_t n_runs;
  const int64_t* sec_row0; /* [n_sectors + 1], device */
  const int32_t* run_sec;  /* [n_runs], device */
  const int64_t* run_vec0; /* [n_runs + 1], device */
  int64_t max_rows;
} edgpu_ragged;

/* Upstream's Lanczos recurrence (as edgpu_lanczos, precision 0) for every run of a ragged
 * batch in one launch, one CTA per run with its three vectors in shared memory
 * (edgpu_lanczos_ragged_smem(max_rows) <= 200 KiB).  alpha/beta [n_runs][K]. */
size_t edgpu_lanczos_ragged_smem(int64_t max_rows);
int edgpu_lanczos_ragged(const edgpu_csr* h, const edgpu_ragged* rg, const double* v0, const int32_t* k_max, int K,
                         double* alpha, double* beta, int32_t* status_dev, void* stream);

/* Lanczos with full reorthogonalisation (classical Gram-Schmidt against the whole basis, a
 * second pass only when the first removed more than half of |w|^2) for every run of
 * a ragged batch in one launch, one CTA per run.  Run r keeps its Krylov basis at
 * V + 2 * run_V0[r] doubles ([k_max[r]][n] complex128, caller-allocated); beta[r][k_max-1] is
 * the last step's residual norm (Ritz residual estimates); breakdown before k_max sets
 * *status_dev = EDGPU_ERR_BREAKDOWN and ends that run. */
size_t edgpu_lanczos_reorth_ragged_smem(int64_t max_rows, int K);
int edgpu_lanczos_reorth_ragged(const edgpu_csr* h, const edgpu_ragged* rg, const double* v0, const int32_t* k_max,
                                int K, const int64_t* run_V0, double* V, double* alpha, double* beta,
                                int32_t* status_dev, void* stream);

/*
 * C[M][N] (float32) = A[M][K] * B[N][K]^T with A and B row-major BF16 (K-major), on the
 * tcgen05 tensor cores: K tiles of A and B brought into a shared-memory ring by bulk-tensor
 * copies (3-4 stages in flight), FP32 accumulator in tensor memory, 128-row tiles 256, 64 or
 * 16 columns wide (the widest that gives most SMs a tile).  M % 128 == 0, K % 64 == 0,
 * N % 16 == 0, N <= 1048560, A and B 16-byte aligned (C of any alignment).  A wait that runs
 * out of its iteration limit sets *status_dev = EDGPU_ERR_NOCONV.  No counterpart in upstream
 * impurityModel (the GEMM of the basis-pruning network).
 */
int edgpu_gemm_bf16(const void* A, const void* B, int M, int N, int K, float* C, int32_t* status_dev, void* stream);
/* Columns of the output tiles (256, 64 or 16) edgpu_gemm_bf16 and edgpu_gemm_bf16_epi use for
 * an M x N product on the current device; 0 when they reject the shape.  Host only. */
int edgpu_gemm_tile_width(int M, int N);

/*
 * Basis-pruning network (input bits -> 256 -> 256 -> 1, BF16 operands, FP32 accumulation);
 * no counterpart in upstream impurityModel.  The GEMM with a fused epilogue:
 *   epi 0: C = acc (float32 [M][N]);
 *   epi 1: Y = relu(acc + bias[col]) as BF16 [M][N], and Yt = Y^T [N][M] when not NULL;
 *   epi 2: Y = acc where mask[row][col] > 0 else 0 (BF16 mask [M][N]), Y and Yt as epi 1.
 * Shapes as edgpu_gemm_bf16.
 */
int edgpu_gemm_bf16_epi(int epi, const void* A, const void* B, int M, int N, int K, float* C, const float* bias,
                        const void* mask, void* Y, void* Yt, int32_t* status_dev, void* stream);
/* X[b][i] = occupation of spin-orbital i of states[b] (W words, bit 63 - i%64 of word i/64),
 * BF16 [B][n_in]; Xt = X^T [n_in][B] when not NULL. */
int edgpu_mlp_bits(const uint64_t* states, int W, int64_t B, int n_in, void* X, void* Xt, void* stream);
/* y[b] = sum_j H[b][j] w3[j] + b3[0] (H BF16 [B][n_h]). */
int edgpu_mlp_head(const void* H, const float* w3, const float* b3, int64_t B, int n_h, float* y, void* stream);
/* Mean-squared-error head backward: dy = 2 (y - target) / B, dH = dy w3 masked by H > 0
 * (BF16 [B][n_h] and its transpose dHt). */
int edgpu_mlp_head_backward(const void* H, const float* y, const float* target, const float* w3, int64_t B, int n_h,
                            float* dy, void* dH, void* dHt, void* stream);
/* out[r] = sum_c M[r][c] v[c] (v NULL: plain row sums) for BF16 M [rows][cols]. */
int edgpu_mlp_row_dot(const void* M, int rows, int64_t cols, const float* v, float* out, void* stream);
/* Adam step on a flat FP32 vector; lr_t is the bias-corrected step size. */
int edgpu_mlp_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr_t, float beta1, float beta2,
                   float eps, void* stream);
/* BF16 copy Wb of a row-major FP32 [rows][cols] matrix and/or of its transpose Wt. */
int edgpu_mlp_to_bf16(const float* Wf, int rows, int cols, void* Wb, void* Wt, void* stream);

/*
 * One-body density matrices of R states: out[r][p] = <psi_r| T_p |psi_r> (complex128) for P
 * packed two-operator terms T_p (edgpu_terms ops encoding, e.g. c_j^dagger c_i).  State r is
 * states[run_off[r] .. run_off[r+1]) (n_words words each, SORTED within the state) with
 * complex128 amplitudes.  Replaces the per-pair loops of upstream getDensityMatrix
 * (impurityModel/ed/finite.py:967-1012); the occupation observables of finite.py:843-1112 are
 * linear in its result.  R <= 65535.
 */
int edgpu_density_matrix(int n_words, const uint64_t* states, const double* amps, const int64_t* run_off, int R,
                         const uint64_t* pair_ops, int P, double* out, void* stream);

/*
 * Single-call sector and ground-state construction, for hosts that drive the engine without
 * the Python layer.  Each is synchronous on `stream` (sizes are read back between phases) and
 * takes all scratch from the workspace of its *_workspace query.
 *
 * edgpu_build_csr: the sector Hamiltonian on a SORTED basis (n states), replacing upstream
 * get_hamiltonian_matrix / get_hamiltonian_matrix_from_h_dict (finite.py:1514-1693): row j
 * holds H|b_j> conjugated (= row j of the Hermitian H), outputs outside the basis or the
 * restrictions dropped, duplicates summed in term order, |v|^2 < weight_min dropped.
 * row_ptr[n + 1] is always written; *nnz_out receives the entry count, and when it exceeds
 * nnz_cap (or col/val is NULL) the call returns EDGPU_ERR_OVERFLOW without writing entries:
 * call again with nnz_cap >= *nnz_out.  real_values != 0: val is float64 [nnz] (the real
 * parts); else complex128 [nnz][2].
 */
size_t edgpu_build_csr_workspace(int n_words, int64_t n, int64_t nnz_cap);
int edgpu_build_csr(int n_words, const edgpu_terms* terms, const edgpu_restrictions* restr, double weight_min,
                    const uint64_t* basis, int64_t n, int real_values, int64_t* row_ptr, int32_t* col, double* val,
                    int64_t nnz_cap, int64_t* nnz_out, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                    void* stream);
/*
 * edgpu_expand: closure of basis0 (n0 states) under the restricted operator, replacing
 * upstream expand_basis (finite.py:1696-1803): breadth-first layers, each layer the sorted
 * new states.  out_sorted[capacity] receives the closure sorted (lexicographic word order =
 * upstream bytes order); out_layered (optional, [capacity]) upstream's basis order (basis0
 * as given, then each layer sorted); *n_out its size.  Candidates are generated at most
 * emit_cap at a time (the frontier is split).  EDGPU_ERR_OVERFLOW with *n_out a lower bound
 * when the closure exceeds capacity.
 */
size_t edgpu_expand_workspace(int n_words, int64_t capacity, int64_t emit_cap);
int edgpu_expand(int n_words, const edgpu_terms* terms, const edgpu_restrictions* restr, double weight_min,
                 const uint64_t* basis0, int64_t n0, int64_t capacity, int64_t emit_cap, uint64_t* out_sorted,
                 uint64_t* out_layered, int64_t* n_out, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                 void* stream);
/*
 * edgpu_eig_lowest: the k lowest eigenpairs of a Hermitian CSR H by Lanczos with full
 * reorthogonalisation from a seeded random start vector (edgpu_lanczos_reorth, chunks of 32
 * steps), replacing upstream eigensystem's eigsh(k, which="SA") (finite.py:58-118).  Ritz
 * values of the Krylov tridiagonal come from bisection on Sturm counts and its eigenvectors
 * from inverse iteration; the run stops when every wanted residual beta |s_last| is below
 * tol_rel * max(1, |theta|), when the Krylov space is exhausted, or at k_cap steps
 * (EDGPU_ERR_NOCONV, best pairs still written).  evals (host, k) ascending, evecs (device,
 * [k][n] complex128), *k_found the pairs written.  One Krylov space holds one vector of each
 * eigenspace: the copies of an exactly degenerate eigenvalue beyond the first are found by
 * further deflated runs, which the Python layer adds (finite.eig_lowest).
 */
size_t edgpu_eig_lowest_workspace(int64_t n, int k_cap);
int edgpu_eig_lowest(const edgpu_csr* h, int k, double tol_rel, int k_cap, uint64_t seed, double* evals,
                     double* evecs, int* k_found, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                     void* stream);

/*
 * Connected components of a sector's (symmetric) sparsity pattern: label[i] = smallest state
 * index of i's component, for n <= 65536 in one launch (one CTA iterating minimum-label
 * propagation with pointer jumping on chip until a round changes nothing; *rounds receives
 * the number of rounds when not NULL).  Gives the dimension of each Green's-function run's
 * basis closure, upstream's Krylov-size cap (impurityModel/ed/spectra.py:646-676).
 */
int edgpu_components(const edgpu_csr* h, int64_t* label, int32_t* rounds, void* stream);

/* Ritz vectors of a ragged batch: X[r][q] = sum_{k < k_len[r]} S[r][k][q] V_r[k] for q < Q
 * (S real [n_runs][K][Q]); X packed complex128 at offset Q * run_vec0[r]. */
int edgpu_combine_ragged(const double* V, const edgpu_ragged* rg, const int64_t* run_V0, const int32_t* k_len,
                         const double* S, int K, int Q, double* X, void* stream);

/*
 * Continued fractions (upstream spectra.py:678-680) for R runs on n_omega points:
 * g[r][w] = scale[r] / (z - a0 - b0^2 / (z - a1 - ...)), z = omega[w] + i*delta + e[r],
 * depth k_len[r] (alpha[r][0..k_len), beta[r][0..k_len-1), row stride K).
 */
int edgpu_cfrac(const double* alpha, const double* beta, const int32_t* k_len, int K, int R, const double* omega,
                int n_omega, double delta, const double* e, const double* scale, double* g, void* stream);

/*
 * Continued fractions of edgpu_cfrac in float32 for the mixed-precision form: alpha - e_r and
 * beta^2 are formed in float64 first (so the common energy offset cancels exactly), then
 * the fraction is evaluated in float32; results are scaled and stored as complex128.
 */
size_t edgpu_cfrac_f32_workspace(int K, int R);
int edgpu_cfrac_f32(const double* alpha, const double* beta, const int32_t* k_len, int K, int R, const double* omega,
                    int n_omega, double delta, const double* e, const double* scale, double* g, void* workspace,
                    size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* EDGPU_H */

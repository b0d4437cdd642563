/*
 * qpeps.h — C ABI of the GB300 exact N-Queens PEPS row-boundary contraction.
 *
 * Plain C types only (fixed-width integers, pointers, sizes); no CUDA or
 * C++ types cross this boundary, so a Rust `extern "C"` block, Python ctypes
 * or a C program can bind it directly.
 *
 * Each entry point names the reference interface it replaces (Rust crate
 * `nqueens-peps-naive`, file:line within that project).
 *
 * Ownership: the caller owns every output buffer; the library owns device
 * memory behind an opaque `qpeps_ctx`. Threading: one context is used by one
 * thread at a time; separate contexts may run concurrently (each owns one CUDA
 * stream). Errors: every fallible call returns 0 on success or a QPEPS_ERR_*
 * code, and writes a NUL-terminated message into `err` (when non-NULL)
 * phrased like the reference's `Err(String)` values.
 */
#ifndef QPEPS_H
#define QPEPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QPEPS_ABI_VERSION 1

/* Return codes. */
#define QPEPS_OK 0
#define QPEPS_ERR_RANGE 1     /* N out of range, key too wide, bad prefix column */
#define QPEPS_ERR_OOM 2       /* device or host allocation failed */
#define QPEPS_ERR_CAPACITY 3  /* a device table or probe bound was exceeded */
#define QPEPS_ERR_CRT_BOUND 4 /* reconstructed count fails the N! certificate */
#define QPEPS_ERR_CUDA 5      /* CUDA runtime error */
#define QPEPS_ERR_INVALID 6   /* invalid argument, or C failed certification */
#define QPEPS_ERR_OVERFLOW 7  /* checked u128 arithmetic overflowed */
#define QPEPS_ERR_TIMEOUT 8   /* a bounded device wait gave up */

/* u128 as two little-endian u64 halves (Rust u128 / C unsigned __int128). */
typedef struct qpeps_u128 {
  uint64_t lo;
  uint64_t hi;
} qpeps_u128;

/* Per-row metrics; field-for-field the reference's LayerMetric
 * (src/lib.rs:388-401). `row` is 0-based like the reference (the CLI prints
 * row+1). `peak_rss_bytes` reports device bytes in use by the context. */
typedef struct qpeps_layer {
  uint32_t row;
  uint64_t input_states;
  qpeps_u128 tensor_entries_examined;
  qpeps_u128 tensor_entries_matched;
  qpeps_u128 row_operator_candidates;
  qpeps_u128 row_operator_matched;
  qpeps_u128 completed_row_terms;
  uint64_t output_states;
  qpeps_u128 output_weight;
  double elapsed_s;
  uint64_t peak_rss_bytes;
} qpeps_layer;

/* Whole-contraction result; the reference's ContractionResult
 * (src/lib.rs:403-415) plus device-side facts. */
typedef struct qpeps_result {
  uint32_t n;
  qpeps_u128 count;
  double elapsed_s;
  uint64_t peak_states;
  qpeps_u128 tensor_entries_examined;
  qpeps_u128 tensor_entries_matched;
  qpeps_u128 row_operator_candidates;
  qpeps_u128 row_operator_matched;
  uint64_t peak_rss_bytes;
  uint32_t n_layers;
  /* device-side facts (no reference counterpart) */
  uint32_t residues;          /* CRT primes used */
  uint32_t key_bits;          /* 64 or 128 */
  uint32_t slice_depth;       /* rows enumerated on the host into slices */
  uint32_t batches;           /* device batches run */
  uint32_t merge;             /* merge strategy actually used (QPEPS_MERGE_*) */
  uint64_t entries_in;        /* sum over row steps of boundary entries read */
  uint64_t entries_out;       /* sum over row steps of boundary entries written */
  uint64_t candidates;        /* sum over row steps of successor terms */
  uint64_t gpu_launches;      /* kernels launched by this call */
  uint64_t peak_device_bytes; /* high-water mark of the context's device pool */
  double device_ms;           /* device time of all row steps (CUDA events) */
  double merge_kernel_ms;     /* device time of the merge kernel (table compact or partition merge) */
  double scatter_kernel_ms;   /* device time of the expand kernel (table insert or partition scatter) */
  uint64_t merge_kernel_launches;
  uint64_t merge_kernel_bytes; /* algorithmic bytes of the dominant kernel */
  uint32_t tail_row;          /* first row contracted by the slice-tail kernel (N = none) */
  uint32_t exact_weights;     /* 1: the boundary's two u32 planes held each entry's exact 64-bit weight
                                 (low and high words) and the host derived the residues; 0: residue planes */
  uint64_t tail_items;        /* boundary entries handed to the slice-tail kernel */
  uint64_t tail_overflow;     /* of those, entries redone by the row engine */
  double tail_kernel_ms;      /* device time of the slice-tail kernel */
  uint64_t h2d_bytes;         /* host->device bytes copied by this call */
  uint64_t d2h_bytes;         /* device->host bytes copied by this call */
  uint32_t residue_primes[4];
  uint64_t count_residues[4];
} qpeps_result;

#define QPEPS_GRAIN_ROW 0  /* compiled row operator, one fused step per row */
#define QPEPS_GRAIN_SITE 1 /* explicit C, one plain launch per site */

#define QPEPS_MERGE_AUTO 0
#define QPEPS_MERGE_HASH 1      /* global open-addressing table */
#define QPEPS_MERGE_PARTITION 2 /* radix partition + shared-memory merge */

typedef struct qpeps_options {
  uint32_t struct_size;          /* sizeof(qpeps_options) */
  uint32_t granularity;          /* QPEPS_GRAIN_* */
  uint32_t merge;                /* QPEPS_MERGE_* */
  uint32_t residues;             /* 0 = shortest prime prefix with product > N!, else 1..4 */
  uint32_t key_bits;             /* 0 = narrowest that fits (64 up to N = 22, where the row key drops the
                                    two diagonal bits every row step clears), 64 or 128 to force */
  uint32_t slice_depth;          /* 0 = auto, else rows enumerated on the host (>= 1) */
  uint32_t symmetry;             /* 1 = first-row vertical-reflection orbits (reference default) */
  uint32_t collect_layers;       /* 1 = fill per-row metrics */
  uint32_t block_threads;        /* 0 = auto */
  uint32_t use_graph;            /* 1 = the first contraction with these options (and tuning) on a
                                    context records its row steps and captures them as one CUDA
                                    graph; later identical contractions replay it (one launch, one
                                    synchronisation) and check every row against the recorded run */
  uint64_t device_budget_bytes;  /* 0 = auto (a fraction of free device memory) */
  uint32_t tail_row;             /* rows >= tail_row run in the slice-tail kernel (a CTA contracts
                                    batches of boundary entries in shared memory); 0 = auto (never),
                                    >= N = never */
  uint32_t reserved;
} qpeps_options;

/* Library version string, e.g. "qpeps-gb300 0.1.0 (sm_103a)". */
const char* qpeps_version(void);

/* Fill `opt` with the defaults (reference semantics: row grain, orbits on). */
void qpeps_options_default(qpeps_options* opt);

/* Replaces `known_count` (src/lib.rs:5752-5784): Q(0..27). Returns
 * QPEPS_ERR_RANGE for N > 27. */
int qpeps_known_count(uint32_t n, qpeps_u128* out);

/* Create / destroy a context bound to one CUDA device. */
int qpeps_ctx_create(int device, void** ctx_out, char* err, size_t err_len);
void qpeps_ctx_destroy(void* ctx);

/* Replaces `contract_rows(n)` (src/lib.rs:758, via
 * contract_rows_d4_orbit_sort_reduce 784 and
 * contract_rows_sort_reduce_with_modes 5287-5415): exact count of Q(N) with
 * per-row metrics. `layers` may be NULL; otherwise it receives up to
 * `layers_cap` rows. N > 42 -> QPEPS_ERR_RANGE with the reference's message;
 * N = 0 -> count 1. */
int qpeps_contract_rows(void* ctx, uint32_t n, const qpeps_options* opt, qpeps_result* result,
                        qpeps_layer* layers, uint32_t layers_cap, char* err, size_t err_len);

/* Count completions of one board with `k` rows already placed (`prefix[r]`
 * is the queen's column in row r; NULL when k = 0). k = 0 equals
 * contract_rows(n).count. An attacked prefix gives 0. This has no single
 * reference function: it is the prefix boundary of
 * recursive_tail_successor (src/lib.rs:3139-3151) contracted like
 * contract_rows. */
int qpeps_count(void* ctx, uint32_t n, const uint32_t* prefix, uint32_t k, const qpeps_options* opt,
                qpeps_u128* count_out, qpeps_result* stats_out, char* err, size_t err_len);

/* Many independent instances in one call: instance i has board size n[i]
 * and k[i] placed rows stored at prefix_cols[prefix_offset[i] ...]. Results
 * go to counts[i]. Instances share device batches. */
int qpeps_count_batch(void* ctx, uint32_t num, const uint32_t* n, const uint32_t* k,
                      const uint32_t* prefix_offset, const uint32_t* prefix_cols,
                      const qpeps_options* opt, qpeps_u128* counts, char* err, size_t err_len);

/* Certification of the local tensor: run the equivalent of
 * CompiledRowOperator::compile (src/lib.rs:430-485) on C given as
 * `len` entries of (legs_key, value) where legs_key follows
 * src/lib.rs:159-168. Returns 0 when C is exactly the Sec. VI automaton. The
 * device kernels are only launched after this check passes on the library's
 * own C. */
int qpeps_certify_c(const uint32_t* legs, const uint64_t* values, uint32_t len, char* err, size_t err_len);

/* ---- Explicit-C generic site frontier -------------------------------------
 * Replaces contract_explicit_c_frontier (src/lib.rs:961-967, kernel
 * 1519-1711): contract the explicit C tensor one site at a time in row-major
 * or top-left-diamond order; the boundary is the values of the open virtual
 * bonds (u128 keys). N > 21 -> QPEPS_ERR_RANGE; support_limit = 0 ->
 * QPEPS_ERR_INVALID. When a site's merged boundary exceeds support_limit the
 * result is incomplete (complete = 0, count unset, contracted_sites = the
 * sites finished before it, peak_states = support_limit + 1); its tensor
 * counters then cover the whole failing site, where the reference's stop
 * inside it. */
#define QPEPS_ORDER_ROW_MAJOR 0
#define QPEPS_ORDER_TOP_LEFT_DIAMOND 1

typedef struct qpeps_explicit_result {
  uint32_t n, order, complete;
  uint32_t merge; /* the site steps' merge: QPEPS_MERGE_PARTITION (128-bit partitions) or QPEPS_MERGE_HASH */
  qpeps_u128 count;
  double elapsed_s;
  uint64_t peak_states, peak_open_bonds;
  qpeps_u128 tensor_entries_examined, tensor_entries_accepted;
  uint64_t contracted_sites;
  uint64_t peak_rss_bytes; /* device memory high-water mark of the context */
  uint64_t gpu_launches;
  double device_ms;
} qpeps_explicit_result;

int qpeps_explicit_frontier(void* ctx, uint32_t n, uint32_t order, uint64_t support_limit,
                            qpeps_explicit_result* out, char* err, size_t err_len);

/* ---- Tuning ---------------------------------------------------------------
 * No reference counterpart (the reference has one CPU code path): the knobs of
 * the partitioned merge, held per context. Every setting gives the same
 * counts and metrics; only the speed changes. */
#define QPEPS_SCATTER_SEARCH 0 /* shuffle search for each successor's parent */
#define QPEPS_SCATTER_WINDOW 1 /* per-warp shared-memory candidate window (default) */
#define QPEPS_SCATTER_TWO_LEVEL 2 /* coarse buckets, then partitions, each written as runs ordered in
                                     shared memory (16-byte candidates, up to 2^20 partitions; the
                                     window scatter elsewhere); needs about one more candidate array;
                                     exact like the others, measured slower on GB300 */
#define QPEPS_SCATTER_CLASS 3  /* class-grouped partitions: a candidate's partition follows its columns
                                  and outermost diagonal signals, so a CTA's successors go to few
                                  partitions and are written as runs (16-byte candidates; the window
                                  scatter elsewhere) */
#define QPEPS_SCATTER_DIRECT 4 /* each lane stores its own parents' successors: no shared-memory window,
                                  no shuffles */
#define QPEPS_MERGEK_SCAN 0    /* ballot/scan compaction over the whole table */
#define QPEPS_MERGEK_CLAIM 1   /* claim list + first-claimant stores (default) */

typedef struct qpeps_tuning {
  uint32_t struct_size;          /* sizeof(qpeps_tuning) */
  uint32_t scatter_kind;         /* QPEPS_SCATTER_* */
  uint32_t parents_per_lane;     /* scatter: parents per lane per warp iteration, 2 or 4 */
  uint32_t merge_kind;           /* QPEPS_MERGEK_* */
  uint32_t wide_merge;           /* 0 never, 1 always, 2 auto: 8192-slot merge CTAs, 4096-candidate partitions;
                                    3: 2048-slot merge CTAs, four per SM, 1024-candidate partitions */
  uint32_t wide_above_parts;     /* auto: 2048-candidate partition count above which merges go wide */
  uint32_t spread_cursors_below; /* partition counts up to which cursors get 32-byte spacing */
  uint32_t fold_weights;         /* 2 (default) = with the partitioned row merge and 13 <= N - k <= 21
                                    the boundary carries exact 64-bit weights (each row certified
                                    to stay below 2^63 before it runs, QPEPS_ERR_OVERFLOW
                                    otherwise); 1 = residues, but with two residues (N - k <= 20)
                                    the claim-list merge accumulates one CRT-folded 64-bit value
                                    per key; 0 = residue sums throughout */
  double partition_fill;         /* mean candidates per partition / capacity, in [0.3, 0.95] */
  double slice_margin;           /* predictive slicing: assumed slice peak / mean slice peak, >= 1 */
  uint32_t unit_target;          /* QPEPS_SCATTER_CLASS: planned candidates per partition, 256..2048 */
  uint32_t unit_sample;          /* QPEPS_SCATTER_CLASS: 1 in unit_sample parents sampled for the plan
                                    (a power of two, 1..64) */
  uint32_t batch_lanes;          /* CUDA-graph replay: independent device batches run concurrently on
                                    this many streams, each with its own buffers (1..8, default 1;
                                    lanes beyond the first only while the device budget holds their
                                    buffers, and only with the window or direct scatter) */
  uint32_t merge_compact;        /* claim-list merge: 0 (default) = compaction walks a slot list in shared
                                    memory; 1 = a key's first claimant writes the output entry from
                                    registers (exact too; measured about 7 % slower on GB300) */
  uint32_t scatter_block;        /* one-level scatters: threads per CTA, 128, 256 (default) or 512 */
  uint32_t merge_auto;           /* what QPEPS_MERGE_AUTO resolves to where both apply:
                                    QPEPS_MERGE_PARTITION (default) or QPEPS_MERGE_HASH */
  uint32_t slice_rows;           /* rows enumerated on the host before batching is decided, 1..4 */
  uint32_t reserved;
} qpeps_tuning;

/* Library defaults (what a new context starts with). */
void qpeps_tuning_default(qpeps_tuning* t);
int qpeps_ctx_get_tuning(void* ctx, qpeps_tuning* out);
/* QPEPS_ERR_INVALID for an out-of-range field (the context keeps its tuning). */
int qpeps_ctx_set_tuning(void* ctx, const qpeps_tuning* t, char* err, size_t err_len);
/* Autotuner: coordinate descent from the context's tuning over scatter kind,
 * parents per lane, scatter block size, merge kind, merge CTA shape,
 * partition fill, weight accumulator, merge strategy and batch sizing (slice
 * margin, host rows); each candidate times
 * contract_rows(n) (8 <= n <= 19) with CUDA-graph replay (device time, best
 * of `repeats` after a warm-up run; every count checked against known_count).
 * Keeps the fastest in the context and returns it. */
int qpeps_autotune(void* ctx, uint32_t n, uint32_t repeats, qpeps_tuning* best, double* best_device_ms, char* err,
                   size_t err_len);
/* Name of the context's CUDA device (for keying tuning caches). */
int qpeps_ctx_device_name(void* ctx, char* out, size_t len);

/* Device rate of the partition scatter's memory pattern, as a ceiling to
 * judge the scatter against (no reference counterpart): `candidates`
 * pseudo-random 16-byte records into `parts` partitions of 2048 slots, by
 * `mode`: QPEPS_PROBE_APPEND (one cursor atomic takes each record's slot, as
 * in the scatter), QPEPS_PROBE_STORE (stores to random slots, no atomic),
 * QPEPS_PROBE_ATOMIC (the atomics, no store), QPEPS_PROBE_STREAM (coalesced
 * stores), QPEPS_PROBE_APPEND_PLAIN (the append without the scatter's L2 keep
 * hint). `best_ms`: the best CUDA-event time of `repeats` launches after one
 * untimed launch. Needs parts * 32 KiB of free device memory. */
#define QPEPS_PROBE_APPEND 0
#define QPEPS_PROBE_STORE 1
#define QPEPS_PROBE_ATOMIC 2
#define QPEPS_PROBE_STREAM 3
#define QPEPS_PROBE_APPEND_PLAIN 4
int qpeps_probe_append(void* ctx, uint32_t mode, uint64_t candidates, uint32_t parts, uint32_t repeats,
                       double* best_ms, char* err, size_t err_len);

/* ---- Serving: continuous batching of counting requests -------------------
 * No single reference counterpart: each request is the prefix contraction of
 * qpeps_count (contract_rows, src/lib.rs:758, from a placed prefix). A server
 * owns two contexts on one device: a shared batch where admitted requests of
 * mixed N (<= 19) advance one row per step together, and a context that runs
 * requests too large for the batch one at a time; both run concurrently.
 * submit() never blocks on the GPU; poll() returns finished requests. */
typedef struct qpeps_serve_config {
  uint32_t struct_size;            /* sizeof(qpeps_serve_config) */
  uint32_t max_slots;              /* concurrent requests in the shared batch (<= 64; 0 = 64) */
  uint64_t batch_budget_bytes;     /* device memory of the shared batch (0 = 25 % of free) */
  uint64_t large_budget_bytes;     /* device memory of the large-request contexts together (0 = 60 % of free) */
  uint64_t large_threshold_states; /* estimated peak frontier above which a request runs alone (0 = auto) */
  uint32_t use_cache;              /* 1 = answer repeated (N, prefix or its mirror) from a result cache */
  uint32_t large_workers;          /* concurrent large-request contexts, each with an equal share of the
                                      large budget (0 = 2; at most 8) */
} qpeps_serve_config;

typedef struct qpeps_serve_completion {
  uint64_t tag;
  qpeps_u128 count;
  int32_t status;   /* QPEPS_OK or an error code */
  uint32_t n, k;
  uint32_t path;    /* 0 shared batch, 1 large-request context, 2 result cache, 3 host (trivial prefix),
                       4 waited on an identical request that was already queued or running */
  double latency_s; /* submit -> completion */
  double queue_s;   /* submit -> admission */
} qpeps_serve_completion;

typedef struct qpeps_serve_stats {
  uint64_t submitted, completed, batch_steps, cache_hits, large_runs;
  uint64_t batch_requeued; /* requests moved from the shared batch to the large-request context */
  uint64_t coalesced;      /* requests answered by an identical in-flight request (cache on) */
} qpeps_serve_stats;

void qpeps_serve_config_default(qpeps_serve_config* cfg);
int qpeps_serve_open(int device, const qpeps_serve_config* cfg, void** server_out, char* err, size_t err_len);
int qpeps_serve_submit(void* server, uint32_t n, const uint32_t* prefix, uint32_t k, uint64_t tag, char* err,
                       size_t err_len);
/* Copy up to `cap` completions into `out`; waits up to `wait_ms` when none is ready. */
int qpeps_serve_poll(void* server, qpeps_serve_completion* out, uint32_t cap, uint32_t* got, uint32_t wait_ms);
int qpeps_serve_stats_get(void* server, qpeps_serve_stats* out);
/* Why a server stopped: its error code and message (QPEPS_OK and "" while it
 * runs). A request that overflows the shared batch's budget does not stop the
 * server: the batch's requests move to the large-request context. */
int qpeps_serve_error(void* server, char* err, size_t err_len);
void qpeps_serve_close(void* server);

/* One row step of the partitioned merge that allocates no device memory.
 * No counterpart in the reference (its Rust driver owns all memory).
 *
 * For callers that cannot call cudaMalloc, e.g. a host framework whose
 * caching allocator owns the GPU's memory, or a serving loop that must not
 * let an allocation synchronise the device. The caller passes device
 * pointers: the boundary `keys_in[n_in]` (packed u64 keys, N <= 21) with
 * residue planes `res_in[r * n_in + i]`, and output buffers
 * `keys_out[out_cap]`, `res_out[r * out_cap + i]`; `out_cap` must be at
 * least the step's successor count (n * n_in always suffices). Scratch comes
 * from a fixed 48 MiB device array inside the library (held by every GPU that
 * loads it until exit); a step whose successors do not fit is rejected with
 * QPEPS_ERR_CAPACITY. The first call on a device looks up that array's
 * address, so make it before any stream capture. Calls share the array:
 * calls whose GPU work overlaps race and must be serialised by the caller.
 * Synchronous on `stream` (NULL = default stream). Outputs: `*out_count`
 * entries written, and per residue r the sums (mod prime r) of all written
 * residues (`weight_residues`) and of those whose columns are all set
 * (`final_residues`, the count after the last row); either may be NULL. */
int qpeps_row_step_noalloc(uint32_t n, uint32_t residues, const uint64_t* keys_in, const uint32_t* res_in,
                           uint64_t n_in, uint64_t* keys_out, uint32_t* res_out, uint64_t out_cap, void* stream,
                           uint64_t* out_count, uint64_t* weight_residues, uint64_t* final_residues, char* err,
                           size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* QPEPS_H */

// Internal interface between the host engine and the CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace qpeps {

// Explicit local tensor C in the form the site kernel reads from constant
// memory: for each 4-bit input signature (column_in | row_in<<1 |
// diag_dr_in<<2 | diag_dl_in<<3, src/lib.rs:152-157) the matching entries'
// outputs (column_out | row_out<<1 | diag_dr_out<<2 | diag_dl_out<<3) and
// their values reduced modulo each residue prime.
struct CTableDev {
  uint32_t count[16];
  uint32_t out[16][4];
  uint32_t value_mod[16][4][4];
};

// Device view of one boundary buffer (structure of arrays).
struct FrontierView {
  void* keys;          // u64[cap] or u128[cap]
  uint32_t* res;       // u32[R][cap]
  uint64_t cap;        // entries per residue plane
};

// Per-step device scalars (one cache line each to avoid false sharing).
struct StepScalars {
  unsigned long long terms;          // successor terms generated
  unsigned long long out_count;      // entries written by compaction
  unsigned long long weight_sum[4];  // sum of residues of written entries
  unsigned long long final_sum[4];   // sum of residues of entries with all columns set
  unsigned long long final_states;   // entries with all columns set
  unsigned int error;                // ErrorBits
  unsigned int next_terms_ok;        // 1: the merge counted next_terms (fixed-layout row merges)
  unsigned long long sitewise_examined;  // row count: C entries the reference's per-parent sitewise
                                         // row kernel matches over the input (sitewise_entries())
  unsigned long long plan_units;         // class-grouped partitions: units of the step's plan (graph replay)
  unsigned long long next_terms;         // successor terms of the written boundary at the next row
};

struct LaunchCfg {
  int key_bits;  // 64 or 128
  int residues;  // 1..4
  int threads;   // block size of the expand kernel
  int sms;       // SM count of the device
};

// All launchers enqueue on `stream` and return cudaGetLastError().
cudaError_t upload_c_table(const CTableDev& table, cudaStream_t stream);

// Sum over entries of popcount(free columns): the row step's successor count.
cudaError_t launch_row_count(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n,
                             StepScalars* scalars, cudaStream_t stream);

// Fused compiled-row expansion + global-table insertion.
cudaError_t launch_row_expand_insert(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n,
                                     void* table, uint64_t table_slots, StepScalars* scalars, cudaStream_t stream);

// Number of explicit-C terms produced at site `site` (mid-row key layout).
cudaError_t launch_site_count(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n, unsigned site,
                              StepScalars* scalars, cudaStream_t stream);

// Explicit-C site update (one launch per site) + global-table insertion.
cudaError_t launch_site_expand_insert(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n,
                                      unsigned site, void* table, uint64_t table_slots, StepScalars* scalars,
                                      cudaStream_t stream);

// Table -> boundary buffer; accumulates weight sums and final (v1) sums.
cudaError_t launch_compact(const LaunchCfg& cfg, const void* table, uint64_t table_slots, const FrontierView& out,
                           unsigned n, bool write_out, StepScalars* scalars, cudaStream_t stream);

// Bytes per table slot for a key width / residue count.
size_t slot_bytes(int key_bits, int residues);

// Explicit-C generic site frontier: one site step. The boundary key holds the
// values of the open virtual bonds (bit i = i-th open bond in increasing bond
// id). The bonds that stay open move to their new positions by a few masked
// shifts (the map is monotone), and every C entry allowed at the site becomes
// a transition: a key matching (req_mask, req_value) on the bonds the site
// closes yields the moved key OR `added` (the values of the bonds it opens).
constexpr int kFrontierMaxRuns = 16;
constexpr int kFrontierMaxTrans = 17;
struct FrontierStepDev {
  uint32_t n_runs, n_trans;
  int32_t run_shift[kFrontierMaxRuns];  // > 0 left, < 0 right
  unsigned __int128 run_mask[kFrontierMaxRuns];
  unsigned __int128 req_mask[kFrontierMaxTrans], req_value[kFrontierMaxTrans], added[kFrontierMaxTrans];
};

cudaError_t upload_frontier_step(const FrontierStepDev& step, cudaStream_t stream);

// Every (boundary entry, matching transition) successor into the u128-keyed
// global table; `scalars->terms` receives the number of matches.
cudaError_t launch_frontier_expand_insert(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, void* table,
                                          uint64_t table_slots, StepScalars* scalars, cudaStream_t stream);

// Partitioned merge (u64 keys): `parts` hash partitions of `cap` candidate
// slots each.
struct PartitionCfg {
  int residues;
  int sms;
  uint32_t parts;
  uint32_t cap;
  int merge_blocks_per_sm;
  uint32_t cursor_stride = 1;     // u32 slots between partition cursors (1 or 8)
  uint32_t parents_per_lane = 2;  // scatter: parents per lane per iteration (2 or 4)
  uint32_t wide = 0;              // merge CTA shape: 0 = 512 threads, 4096-slot table, 2048 candidates,
                                  // two CTAs per SM; 1 = 1024 threads, 8192 slots, 4096 candidates,
                                  // one CTA per SM (R <= 2 only: the table is 8 KiB x (8 + 8R) bytes);
                                  // 2 = 256 threads, 2048 slots, 1024 candidates, four CTAs per SM (R <= 2)
  uint32_t scatter_kind = 1;      // scatter: 0 = shuffle search for each successor's parent,
                                  // 1 = per-warp shared-memory candidate window,
                                  // 2 = two-level (coarse buckets, then partitions; runs staged and
                                  //     ordered in shared memory), where two_level_plan() accepts the step
  uint32_t merge_kind = 1;        // merge: 0 = ballot/scan compaction over the whole table,
                                  // 1 = claim list + first-claimant stores (three phases)
  uint32_t fold = 0;              // merge_kind 1, R = 2, one 64-bit accumulator plane:
                                  // 1 = CRT-folded residues, 2 = the planes hold an exact weight's
                                  // low and high words (both exact only when N! < p0 * p1, N <= 20)
  uint32_t key_bits = 64;         // 128: wide-key scatter and merge (32-byte candidates, `cap` = 1024)
  uint32_t count_next = 1;        // fixed-layout row merges: count the next row's successor terms
  uint32_t scatter_block = 256;   // one-level scatters: threads per CTA (128, 256 or 512; 256 for R > 2)
  uint32_t merge_regs = 0;        // merge_kind 1, fixed layout: first claimants write their entries from
                                  // registers (no slot list in shared memory)
  uint32_t tl_nb = 0;             // two-level scatter: coarse buckets (0 = one-level scatter)
  uint32_t tl_p2 = 0;             // two-level scatter: partitions per bucket (parts = tl_nb * tl_p2)
  uint64_t tl_bcap = 0;           // two-level scatter: candidate slots per bucket
};

size_t candidate_bytes(int residues);
// Partitioned merge with 128-bit keys: candidate slots per partition (1024),
// and its scatter and merge (window scatter; claim-list merge over residue
// planes with a 2048-slot table of 128-bit keys).
uint32_t wide_key_partition_capacity();
cudaError_t launch_wide_partition_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in, unsigned n,
                                          void* regions, uint32_t* cursors, StepScalars* scalars, cudaStream_t stream);
// With n > 0 (row keys) the merge counts the written boundary's successor
// terms at the next row; with n = 0 and `next_step` (explicit-C bond keys, a
// device copy of the next site step) it counts the boundary's matches there.
// Either count lands in scalars->next_terms with next_terms_ok set.
cudaError_t launch_wide_partition_merge(const PartitionCfg& pc, const void* regions, const uint32_t* cursors,
                                        const FrontierView& out, unsigned n, bool write_out, StepScalars* scalars,
                                        cudaStream_t stream, const FrontierStepDev* next_step = nullptr);
// Access-pattern probe (qpeps_probe_append): `total` pseudo-random 16-byte
// records into `parts` partitions of `cap` slots (cap a power of two) by mode
// 0 append (cursor atomic + store), 1 store only, 2 atomic only, 3 stream.
cudaError_t launch_append_probe(uint32_t mode, uint64_t total, uint32_t parts, uint32_t cap, void* regions,
                                uint32_t* cursors, uint32_t cursor_stride, int sms, uint64_t seed,
                                unsigned long long* sink, cudaStream_t stream);
// Explicit-C frontier step through the same 128-bit partitions: the number of
// (boundary entry, matching transition) pairs into `scalars->terms`, and
// every such pair as one candidate (merged by launch_wide_partition_merge
// with n = 0). Keys must not set all 128 bits (at most 127 open bonds).
cudaError_t launch_frontier_count(const FrontierView& in, uint64_t n_in, const FrontierStepDev& step, int sms,
                                  StepScalars* scalars, cudaStream_t stream);
cudaError_t launch_frontier_partition_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in,
                                              const FrontierStepDev& step, void* regions, uint32_t* cursors,
                                              StepScalars* scalars, cudaStream_t stream);
// Candidate slots per partition for a merge shape (PartitionCfg::wide).
uint32_t partition_capacity(uint32_t wide = 0);
// Whether the wide merge shape is available for a residue count.
bool wide_merge_supported(int residues);

// Two-level scatter plan for a step of `terms` successors and at least
// `parts` partitions: sets tl_nb, tl_p2, tl_bcap and parts (= tl_nb * tl_p2,
// rounded up from `parts`). False where it does not apply (more than 16-byte
// candidates, or more partitions than its bins address).
bool two_level_plan(uint64_t terms, uint32_t parts, int residues, PartitionCfg* pc);
// Its scratch follows the partition cursors (parts x 4 x cursor_stride bytes,
// rounded up to 256) in the same allocation: bucket cursors, then bucket slots.
size_t two_level_cursor_bytes(const PartitionCfg& pc);
size_t two_level_extra_bytes(const PartitionCfg& pc);

cudaError_t launch_partition_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in, unsigned n,
                                     void* regions, uint32_t* cursors, StepScalars* scalars, cudaStream_t stream);

// Class-grouped partitions (scatter_kind 3, 16-byte candidates). A
// candidate's class is its columns and the t outermost diagonal pairs; classes
// hash into 2^lg buckets (four sibling classes, equal but for pair 0, in
// consecutive buckets), and a plan maps each bucket to a run of "units"
// (merge partitions of `cap` slots) from a sampled histogram.
struct UnitClassPlan {
  unsigned n;   // board size
  unsigned t;   // window pairs (0: columns only); t <= n / 2
  unsigned lg;  // log2 of the bucket count (>= 3 when t >= 1)
};
struct UnitPlanArgs {
  uint32_t lg;      // log2 of the bucket count
  uint32_t sample;  // one parent block of 512 in `sample` is counted
  uint64_t target;  // planned candidates per unit
};
struct UnitPlanTotals {
  unsigned long long small_units;  // units of packed small buckets (unit ids [0, small_units))
  unsigned long long units;        // all units (the merge's partition count)
  unsigned long long small_e;      // estimated candidates of the packed buckets
  unsigned long long pad;
};
struct UnitPlanDev {
  const uint2* table = nullptr;         // per bucket {first unit, units}
  UnitPlanTotals* totals = nullptr;     // device
};
bool unit_scatter_supported(int residues);
// Device scratch of a plan with 2^lg buckets (histogram, table, scan partials, totals).
size_t unit_plan_scratch_bytes(uint32_t lg);
// Sampled histogram of the step's successors and the bucket -> units table;
// the unit count lands in out->totals (device) for the host to read.
cudaError_t launch_unit_plan(const FrontierView& in, uint64_t n_in, const UnitClassPlan& c, const UnitPlanArgs& a,
                             void* scratch, int sms, cudaStream_t stream, UnitPlanDev* out,
                             StepScalars* scalars = nullptr);
cudaError_t launch_unit_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in,
                                const UnitClassPlan& c, const uint2* table, void* regions, uint32_t* cursors,
                                StepScalars* scalars, cudaStream_t stream);

cudaError_t launch_partition_merge(const PartitionCfg& pc, const void* regions, const uint32_t* cursors,
                                   const FrontierView& out, unsigned n, bool write_out, StepScalars* scalars,
                                   cudaStream_t stream);



// Serving (slotted keys, R = 2): count, scatter and merge of a boundary
// shared by requests of different board sizes. slot_mask[s] is the board mask
// of the request in slot s; finished boards are summed into
// slot_final[s * 4 + r] and leave the boundary.
cudaError_t launch_serve_count(const FrontierView& in, uint64_t n_in, const uint64_t* slot_mask, StepScalars* sc,
                               int sms, cudaStream_t stream);
cudaError_t launch_serve_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in,
                                 const uint64_t* slot_mask, void* regions, uint32_t* cursors, StepScalars* sc,
                                 cudaStream_t stream);
cudaError_t launch_serve_merge(const PartitionCfg& pc, const void* regions, const uint32_t* cursors,
                               const FrontierView& out, const uint64_t* slot_mask, unsigned long long* slot_final,
                               StepScalars* sc, cudaStream_t stream);

// Slice-tail kernel control block (device memory). Row statistics per tail
// row q (row0 + q): [0] input states, [1] output states, [2] successor terms,
// [3 + r] output weight residue r.
constexpr int kTailMaxRows = 32;
constexpr int kTailRowFields = 7;
struct TailControl {
  unsigned long long next_item;
  unsigned long long overflow_count;
  unsigned long long overflow_cap;
  uint64_t* overflow_items;
  unsigned long long final_sum[4];
  unsigned long long row_acc[kTailMaxRows][kTailRowFields];
  unsigned int error;
  unsigned int pad[3];
};

// Contract rows [row0, n) of every boundary entry independently, one warp per
// entry, in shared memory. Entries whose frontier exceeds tail_capacity()
// states are listed in ctl->overflow_items.
uint32_t tail_capacity();
cudaError_t launch_gather_entries(int residues, const FrontierView& in, const uint64_t* idx, uint64_t m,
                                  uint64_t* out_keys, uint32_t* out_res, int sms, cudaStream_t stream);
cudaError_t launch_slice_tail(int residues, const FrontierView& in, uint64_t n_items, unsigned n, unsigned row0,
                              TailControl* ctl, int sms, cudaStream_t stream);

}  // namespace qpeps

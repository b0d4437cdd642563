// Host engine of the GB300 row-boundary contraction and the C ABI of
// include/qpeps.h.
//
// Mirrors the reference's drivers:
//   contract_rows(n)                       src/lib.rs:758 -> 784 -> 5287-5415
//   CompiledRowOperator::compile           src/lib.rs:430-485
//   top-row vertical-reflection orbits     src/lib.rs:721-749
//   known_count                            src/lib.rs:5752-5784
//   CRT certificate (product > N!)         src/lib.rs:3859-3886, 4134-4163
// with the row loop's expand/sort/reduce replaced by device kernels over an
// HBM-resident boundary store.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/qpeps.h"
#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {

// ---------------------------------------------------------------------------
// Errors

struct Failure {
  int code;
  std::string msg;
};

[[noreturn]] static void fail(int code, const std::string& msg) { throw Failure{code, msg}; }

static void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(QPEPS_ERR_OOM, std::string("device allocation failed: ") + what);
  }
  fail(QPEPS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static std::string row_msg(const char* prefix, unsigned row) {
  char buf[96];
  std::snprintf(buf, sizeof buf, "%s %u", prefix, row);
  return buf;
}

// ---------------------------------------------------------------------------
// u128 helpers

static bool add_u128(u128 a, u128 b, u128* out) {
  u128 s = a + b;
  if (s < a) return false;
  *out = s;
  return true;
}
static bool mul_u128(u128 a, u128 b, u128* out) {
  if (a == 0 || b == 0) {
    *out = 0;
    return true;
  }
  u128 p = a * b;
  if (p / a != b) return false;
  *out = p;
  return true;
}
static qpeps_u128 to_abi(u128 v) { return qpeps_u128{(uint64_t)v, (uint64_t)(v >> 64)}; }

// ---------------------------------------------------------------------------
// Local tensor C from B (Sec. VI, Eq. 16-18) and its certification.

struct Legs {
  uint8_t ci, co, ri, ro, dri, dro, dli, dlo;
};

static unsigned legs_key(const Legs& l) {
  return l.ci | (l.co << 1) | (l.ri << 2) | (l.ro << 3) | (l.dri << 4) | (l.dro << 5) | (l.dli << 6) | (l.dlo << 7);
}
static Legs legs_from_key(unsigned k) {
  return Legs{(uint8_t)(k & 1),        (uint8_t)((k >> 1) & 1), (uint8_t)((k >> 2) & 1), (uint8_t)((k >> 3) & 1),
              (uint8_t)((k >> 4) & 1), (uint8_t)((k >> 5) & 1), (uint8_t)((k >> 6) & 1), (uint8_t)((k >> 7) & 1)};
}

struct CEntryH {
  unsigned legs;  // legs_key
  u128 value;
};

// B has 16 alpha=0 identity entries (one per incoming signature) and one
// alpha=1 entry emitting 0->1 on all four channels; C sums alpha out.
static std::vector<CEntryH> build_c_sec_vi() {
  std::map<unsigned, u128> acc;
  for (unsigned sig = 0; sig < 16; ++sig) {
    uint8_t c = sig & 1, r = (sig >> 1) & 1, d = (sig >> 2) & 1, l = (sig >> 3) & 1;
    acc[legs_key(Legs{c, c, r, r, d, d, l, l})] += 1;
  }
  acc[legs_key(Legs{0, 1, 0, 1, 0, 1, 0, 1})] += 1;
  std::vector<CEntryH> out;
  for (auto& kv : acc) out.push_back(CEntryH{kv.first, kv.second});
  return out;
}

static unsigned input_signature(const Legs& l) { return l.ci | (l.ri << 1) | (l.dri << 2) | (l.dli << 3); }

// Fails closed exactly where CompiledRowOperator::compile does.
static void certify_c(const std::vector<CEntryH>& c) {
  bool pass[16] = {false};
  bool have_occ = false;
  for (const CEntryH& e : c) {
    Legs l = legs_from_key(e.legs);
    const bool is_pass = l.ci == l.co && l.ri == l.ro && l.dri == l.dro && l.dli == l.dlo;
    const bool is_occ = l.ci == 0 && l.co == 1 && l.ri == 0 && l.ro == 1 && l.dri == 0 && l.dro == 1 && l.dli == 0 &&
                        l.dlo == 1;
    if (e.value != 1) fail(QPEPS_ERR_INVALID, "compiled row operator requires unit Sec. VI coefficients");
    if (is_pass) {
      unsigned k = input_signature(l);
      if (pass[k]) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "duplicate C pass-through signature %u%u%u%u", (k >> 3) & 1, (k >> 2) & 1,
                      (k >> 1) & 1, k & 1);
        fail(QPEPS_ERR_INVALID, buf);
      }
      pass[k] = true;
    } else if (is_occ) {
      if (have_occ) fail(QPEPS_ERR_INVALID, "multiple occupied C entries");
      have_occ = true;
    } else {
      fail(QPEPS_ERR_INVALID, "C contains an entry outside the Sec. VI row automaton");
    }
  }
  for (bool p : pass)
    if (!p) fail(QPEPS_ERR_INVALID, "C is missing a pass-through signature");
  if (!have_occ) fail(QPEPS_ERR_INVALID, "C is missing the occupied entry");
}

static CTableDev c_table_for_device(const std::vector<CEntryH>& c) {
  CTableDev t;
  std::memset(&t, 0, sizeof t);
  for (const CEntryH& e : c) {
    Legs l = legs_from_key(e.legs);
    unsigned sig = input_signature(l);
    unsigned slot = t.count[sig]++;
    if (slot >= 4) fail(QPEPS_ERR_INVALID, "more than four C entries share one input signature");
    t.out[sig][slot] = l.co | (l.ro << 1) | (l.dro << 2) | (l.dlo << 3);
    for (int r = 0; r < kMaxResidues; ++r) t.value_mod[sig][slot][r] = (uint32_t)(e.value % kPrimes[r]);
  }
  return t;
}

// ---------------------------------------------------------------------------
// Known counts (OEIS A000170), CRT plan and reconstruction.

static const char* kKnown[28] = {"1",
                                 "1",
                                 "0",
                                 "0",
                                 "2",
                                 "10",
                                 "4",
                                 "40",
                                 "92",
                                 "352",
                                 "724",
                                 "2680",
                                 "14200",
                                 "73712",
                                 "365596",
                                 "2279184",
                                 "14772512",
                                 "95815104",
                                 "666090624",
                                 "4968057848",
                                 "39029188884",
                                 "314666222712",
                                 "2691008701644",
                                 "24233937684440",
                                 "227514171973736",
                                 "2207893435808352",
                                 "22317699616364044",
                                 "234907967154122528"};

static bool known_count(unsigned n, u128* out) {
  if (n >= 28) return false;
  u128 v = 0;
  for (const char* p = kKnown[n]; *p; ++p) v = v * 10 + (u128)(*p - '0');
  *out = v;
  return true;
}

static u128 factorial(unsigned n) {
  u128 f = 1;
  for (unsigned i = 2; i <= n; ++i)
    if (!mul_u128(f, i, &f)) fail(QPEPS_ERR_RANGE, "N! exactness bound does not fit u128");
  return f;
}

// Shortest prefix of the residue primes whose product exceeds N! (the count
// and every row weight are at most N!).
static int crt_plan(unsigned n) {
  u128 bound = factorial(n), prod = 1;
  for (int r = 0; r < kMaxResidues; ++r) {
    prod *= kPrimes[r];
    if (prod > bound) return r + 1;
  }
  fail(QPEPS_ERR_RANGE, "available certified CRT product does not exceed N! bound");
}

// Modular inverse by the extended Euclidean algorithm.
static u64 inv_mod(u64 a, u64 p) {
  int64_t t = 0, nt = 1;
  int64_t r = (int64_t)p, nr = (int64_t)(a % p);
  while (nr != 0) {
    int64_t q = r / nr;
    int64_t tmp = t - q * nt;
    t = nt;
    nt = tmp;
    tmp = r - q * nr;
    r = nr;
    nr = tmp;
  }
  if (t < 0) t += (int64_t)p;
  return (u64)t;
}

// Garner's mixed-radix reconstruction with checked u128 arithmetic.
static u128 crt_reconstruct(const u64* residues, int count) {
  u128 value = 0, modulus = 1;
  for (int i = 0; i < count; ++i) {
    const u64 p = kPrimes[i];
    const u64 vm = (u64)(value % p);
    const u64 rm = residues[i] % p;
    const u64 delta = rm >= vm ? rm - vm : rm + p - vm;
    const u64 step = (u64)(((u128)delta * inv_mod((u64)(modulus % p), p)) % p);
    u128 term;
    if (!mul_u128(modulus, step, &term) || !add_u128(value, term, &value))
      fail(QPEPS_ERR_OVERFLOW, "CRT reconstruction overflow");
    if (!mul_u128(modulus, p, &modulus)) fail(QPEPS_ERR_OVERFLOW, "CRT reconstruction modulus overflow");
  }
  return value;
}

// ---------------------------------------------------------------------------
// Context: one device, one stream, a grow-only pool of device buffers.

struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct Ctx {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  DevBuf front[2];  // boundary buffers (keys then residue planes)
  DevBuf table;
  StepScalars* d_sc = nullptr;
  StepScalars* h_sc = nullptr;  // pinned
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t pool_bytes = 0, peak_pool_bytes = 0;
  size_t free_at_create = 0;
  uint64_t launches = 0;
  std::vector<CEntryH> c;
  CTableDev c_dev;
  bool c_uploaded = false;
  double partition_mean = 1700.0;  // target candidates per partition (slots: 2048)
};

static void buf_release(Ctx& ctx, DevBuf& b) {
  if (b.ptr) {
    cudaFree(b.ptr);
    ctx.pool_bytes -= b.bytes;
  }
  b.ptr = nullptr;
  b.bytes = 0;
}

static void buf_reserve(Ctx& ctx, DevBuf& b, size_t bytes, size_t budget, const char* what) {
  if (b.bytes >= bytes) return;
  size_t want = bytes + bytes / 4;
  if (ctx.pool_bytes - b.bytes + want > budget) want = bytes;
  if (ctx.pool_bytes - b.bytes + want > budget)
    fail(QPEPS_ERR_CAPACITY, std::string("device budget exceeded by ") + what);
  buf_release(ctx, b);
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(QPEPS_ERR_CAPACITY, std::string("device allocation failed for ") + what);
  }
  b.bytes = want;
  ctx.pool_bytes += want;
  ctx.peak_pool_bytes = std::max(ctx.peak_pool_bytes, ctx.pool_bytes);
}

// Buffers whose contents are dead at this point (the table and the output
// boundary buffer) are released when too small, or when their oversize from an
// earlier, larger row would push the pool past the budget.
static void make_room(Ctx& ctx, DevBuf& a, size_t a_bytes, DevBuf& b, size_t b_bytes, size_t budget) {
  if (a.bytes < a_bytes) buf_release(ctx, a);
  if (b.bytes < b_bytes) buf_release(ctx, b);
  const size_t pending = (a.ptr ? 0 : a_bytes) + (b.ptr ? 0 : b_bytes);
  if (ctx.pool_bytes + pending > budget) {
    buf_release(ctx, a);
    buf_release(ctx, b);
  }
}

static void ctx_free(Ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  buf_release(*ctx, ctx->front[0]);
  buf_release(*ctx, ctx->front[1]);
  buf_release(*ctx, ctx->table);
  if (ctx->d_sc) cudaFree(ctx->d_sc);
  if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

static Ctx* ctx_create(int device) {
  int count = 0;
  cuda_check(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
  if (device < 0 || device >= count) fail(QPEPS_ERR_CUDA, "no such CUDA device");
  Ctx* ctx = new Ctx();
  try {
    ctx->device = device;
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    cuda_check(cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device), "SM count");
    cuda_check(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaMalloc(&ctx->d_sc, sizeof(StepScalars)), "step scalars");
    cuda_check(cudaMallocHost(&ctx->h_sc, sizeof(StepScalars)), "pinned step scalars");
    for (auto& e : ctx->ev) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    ctx->free_at_create = fr;
    ctx->c = build_c_sec_vi();
    certify_c(ctx->c);
    ctx->c_dev = c_table_for_device(ctx->c);
  } catch (...) {
    ctx_free(ctx);
    throw;
  }
  return ctx;
}

// ---------------------------------------------------------------------------
// Contraction driver.

struct Item {
  u128 key;     // packed boundary (reference layout)
  u128 weight;  // exact multiplicity (orbit weight)
};

struct RowAcc {
  bool used = false;
  u64 input_states = 0, output_states = 0;
  u128 candidates = 0, matched = 0, completed = 0, examined = 0, tmatched = 0;
  u128 weight_exact = 0;      // rows computed on the host
  u64 weight_res[kMaxResidues] = {0, 0, 0, 0};  // sums mod p of device rows
  bool device_row = false;
  double elapsed = 0;
};

struct RunStats {
  u64 entries_in = 0, entries_out = 0, candidates = 0, launches = 0;
  u64 peak_states = 0;
  double device_ms = 0, merge_ms = 0, scatter_ms = 0;
  u64 merge_launches = 0, merge_bytes = 0;
  u64 final_res[kMaxResidues] = {0, 0, 0, 0};
  unsigned batches = 0;
};

struct Plan {
  unsigned n;
  int R;
  int key_bits;
  int grain;
  int merge;  // QPEPS_MERGE_HASH or QPEPS_MERGE_PARTITION
  size_t budget;
  int threads;
};

static size_t entry_bytes(const Plan& p) { return (size_t)(p.key_bits / 8) + 4u * p.R; }

static FrontierView view_of(const Plan& p, DevBuf& b, u64 cap) {
  FrontierView v;
  v.keys = b.ptr;
  v.res = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(b.ptr) + (size_t)cap * (p.key_bits / 8));
  v.cap = cap;
  return v;
}

static u64 pow2_at_least(u64 x) {
  u64 p = 1;
  while (p < x) p <<= 1;
  return p;
}

static void sync_scalars(Ctx& ctx) {
  cuda_check(cudaMemcpyAsync(ctx.h_sc, ctx.d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, ctx.stream),
             "read step scalars");
  cuda_check(cudaStreamSynchronize(ctx.stream), "step synchronize");
}

// One merge step (a full row in row grain, one site in site grain).
// Input entries are in front[cur] with capacity `cap_in`; output goes to
// front[1-cur]. Returns the number of output entries.
struct StepOut {
  u64 terms, out;
  u64 weight[kMaxResidues];
  u64 final_sum[kMaxResidues];
  u64 out_cap;
};

static StepOut merge_step(Ctx& ctx, const Plan& p, int cur, u64 n_in, u64 cap_in, bool site, unsigned site_idx,
                          bool final_step, RunStats& rs, unsigned row) {
  LaunchCfg cfg{p.key_bits, p.R, p.threads, ctx.sms};
  FrontierView in = view_of(p, ctx.front[cur], cap_in);
  cuda_check(cudaMemsetAsync(ctx.d_sc, 0, sizeof(StepScalars), ctx.stream), "clear step scalars");
  if (site)
    cuda_check(launch_site_count(cfg, in, n_in, p.n, site_idx, ctx.d_sc, ctx.stream), "site count kernel");
  else
    cuda_check(launch_row_count(cfg, in, n_in, p.n, ctx.d_sc, ctx.stream), "row count kernel");
  rs.launches += 1;
  sync_scalars(ctx);
  StepOut so{};
  so.terms = ctx.h_sc->terms;
  const u64 slots = pow2_at_least(std::max<u64>(1024, so.terms * 2));
  const size_t sb = slot_bytes(p.key_bits, p.R);
  const u64 out_cap = std::max<u64>(so.terms, 1);
  // Capacity plan for this step: table + output buffer (input already held).
  const size_t table_bytes = slots * sb;
  const size_t out_bytes = final_step ? 0 : out_cap * entry_bytes(p);
  const size_t need = table_bytes + out_bytes + ctx.front[cur].bytes;
  if (need > p.budget) fail(QPEPS_ERR_CAPACITY, row_msg("device budget exceeded at row", row + 1));
  make_room(ctx, ctx.table, table_bytes, ctx.front[1 - cur], out_bytes, p.budget);
  buf_reserve(ctx, ctx.table, table_bytes, p.budget, "hash table");
  if (!final_step) buf_reserve(ctx, ctx.front[1 - cur], out_bytes, p.budget, "boundary buffer");
  cuda_check(cudaMemsetAsync(ctx.table.ptr, 0, slots * sb, ctx.stream), "clear hash table");
  FrontierView out{};
  if (!final_step) out = view_of(p, ctx.front[1 - cur], out_cap);
  cuda_check(cudaEventRecord(ctx.ev[0], ctx.stream), "event");
  if (site)
    cuda_check(launch_site_expand_insert(cfg, in, n_in, p.n, site_idx, ctx.table.ptr, slots, ctx.d_sc, ctx.stream),
               "site expand-insert kernel");
  else
    cuda_check(launch_row_expand_insert(cfg, in, n_in, p.n, ctx.table.ptr, slots, ctx.d_sc, ctx.stream),
               "row expand-insert kernel");
  cuda_check(cudaEventRecord(ctx.ev[1], ctx.stream), "event");
  cuda_check(launch_compact(cfg, ctx.table.ptr, slots, out, p.n, !final_step, ctx.d_sc, ctx.stream), "compact kernel");
  cuda_check(cudaEventRecord(ctx.ev[2], ctx.stream), "event");
  rs.launches += 2;
  sync_scalars(ctx);
  if (ctx.h_sc->error & kErrProbeLimit) fail(QPEPS_ERR_CAPACITY, row_msg("hash probe bound exceeded at row", row + 1));
  if (ctx.h_sc->error) fail(QPEPS_ERR_CAPACITY, row_msg("device capacity error at row", row + 1));
  float ms_insert = 0, ms_compact = 0;
  cudaEventElapsedTime(&ms_insert, ctx.ev[0], ctx.ev[1]);
  cudaEventElapsedTime(&ms_compact, ctx.ev[1], ctx.ev[2]);
  so.out = ctx.h_sc->out_count;
  so.out_cap = out_cap;
  for (int r = 0; r < p.R; ++r) {
    so.weight[r] = ctx.h_sc->weight_sum[r] % kPrimes[r];
    so.final_sum[r] = ctx.h_sc->final_sum[r] % kPrimes[r];
  }
  rs.device_ms += ms_insert + ms_compact;
  rs.merge_ms += ms_insert;
  rs.merge_launches += 1;
  rs.merge_bytes += n_in * entry_bytes(p) + so.out * entry_bytes(p);
  rs.entries_in += n_in;
  rs.entries_out += so.out;
  rs.candidates += so.terms;
  return so;
}

// Row step through the partitioned merge (scatter into hash partitions, then
// one shared-memory merge per partition).
static StepOut merge_step_partition(Ctx& ctx, const Plan& p, int cur, u64 n_in, u64 cap_in, bool final_step,
                                    RunStats& rs, unsigned row) {
  LaunchCfg cfg{p.key_bits, p.R, p.threads, ctx.sms};
  FrontierView in = view_of(p, ctx.front[cur], cap_in);
  cuda_check(cudaMemsetAsync(ctx.d_sc, 0, sizeof(StepScalars), ctx.stream), "clear step scalars");
  cuda_check(launch_row_count(cfg, in, n_in, p.n, ctx.d_sc, ctx.stream), "row count kernel");
  rs.launches += 1;
  sync_scalars(ctx);
  StepOut so{};
  so.terms = ctx.h_sc->terms;
  const u64 out_cap = std::max<u64>(so.terms, 1);
  const u32 cap = partition_capacity();
  const size_t cb = candidate_bytes(p.R);
  double mean = ctx.partition_mean;
  for (int attempt = 0;; ++attempt) {
    const u64 parts64 = std::max<u64>(1, (u64)((double)so.terms / mean) + 1);
    if (parts64 > 0xffffffffull) fail(QPEPS_ERR_CAPACITY, row_msg("too many partitions at row", row + 1));
    const u32 parts = (u32)parts64;
    const size_t region_bytes = (size_t)parts * cap * cb;
    const size_t cursor_bytes = ((size_t)parts * 4 + 255) / 256 * 256;
    const size_t out_bytes = final_step ? 0 : out_cap * entry_bytes(p);
    const size_t need = region_bytes + cursor_bytes + out_bytes + ctx.front[cur].bytes;
    if (need > p.budget) fail(QPEPS_ERR_CAPACITY, row_msg("device budget exceeded at row", row + 1));
    make_room(ctx, ctx.table, region_bytes + cursor_bytes, ctx.front[1 - cur], out_bytes, p.budget);
    buf_reserve(ctx, ctx.table, region_bytes + cursor_bytes, p.budget, "partition regions");
    if (!final_step) buf_reserve(ctx, ctx.front[1 - cur], out_bytes, p.budget, "boundary buffer");
    void* regions = ctx.table.ptr;
    uint32_t* cursors = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(ctx.table.ptr) + region_bytes);
    cuda_check(cudaMemsetAsync(cursors, 0, (size_t)parts * 4, ctx.stream), "clear partition cursors");
    cuda_check(cudaMemsetAsync(ctx.d_sc, 0, sizeof(StepScalars), ctx.stream), "clear step scalars");
    FrontierView out{};
    if (!final_step) out = view_of(p, ctx.front[1 - cur], out_cap);
    PartitionCfg pc{p.R, ctx.sms, parts, cap, p.R == 1 ? 3 : p.R == 2 ? 2 : 1};
    cuda_check(cudaEventRecord(ctx.ev[0], ctx.stream), "event");
    cuda_check(launch_partition_scatter(pc, in, n_in, p.n, regions, cursors, ctx.d_sc, ctx.stream),
               "partition scatter kernel");
    cuda_check(cudaEventRecord(ctx.ev[1], ctx.stream), "event");
    cuda_check(launch_partition_merge(pc, regions, cursors, out, p.n, !final_step, ctx.d_sc, ctx.stream),
               "partition merge kernel");
    cuda_check(cudaEventRecord(ctx.ev[2], ctx.stream), "event");
    rs.launches += 2;
    sync_scalars(ctx);
    if (ctx.h_sc->error & kErrOverflow) {
      // A partition received more candidates than its slots: retry with
      // smaller partitions (the scatter wrote nothing past a full partition).
      if (attempt >= 4) fail(QPEPS_ERR_CAPACITY, row_msg("partition overflow persists at row", row + 1));
      mean *= 0.6;
      continue;
    }
    if (ctx.h_sc->error) fail(QPEPS_ERR_CAPACITY, row_msg("device capacity error at row", row + 1));
    float ms_scatter = 0, ms_merge = 0;
    cudaEventElapsedTime(&ms_scatter, ctx.ev[0], ctx.ev[1]);
    cudaEventElapsedTime(&ms_merge, ctx.ev[1], ctx.ev[2]);
    so.out = ctx.h_sc->out_count;
    so.out_cap = out_cap;
    for (int r = 0; r < p.R; ++r) {
      so.weight[r] = ctx.h_sc->weight_sum[r] % kPrimes[r];
      so.final_sum[r] = ctx.h_sc->final_sum[r] % kPrimes[r];
    }
    rs.device_ms += ms_scatter + ms_merge;
    rs.merge_ms += ms_merge;
    rs.scatter_ms += ms_scatter;
    rs.merge_launches += 1;
    rs.merge_bytes += n_in * entry_bytes(p) + so.out * entry_bytes(p);
    rs.entries_in += n_in;
    rs.entries_out += so.out;
    rs.candidates += so.terms;
    return so;
  }
}

static void upload_items(Ctx& ctx, const Plan& p, const std::vector<Item>& items, size_t lo, size_t hi, int buf,
                         u64* cap_out) {
  const u64 cnt = hi - lo;
  const u64 cap = std::max<u64>(cnt, 1);
  buf_reserve(ctx, ctx.front[buf], cap * entry_bytes(p), p.budget, "boundary buffer");
  FrontierView v = view_of(p, ctx.front[buf], cap);
  std::vector<uint8_t> keys(cap * (p.key_bits / 8));
  std::vector<uint32_t> res((size_t)p.R * cap);
  for (u64 i = 0; i < cnt; ++i) {
    const Item& it = items[lo + i];
    if (p.key_bits == 64) {
      u64 k = (u64)it.key;
      std::memcpy(&keys[i * 8], &k, 8);
    } else {
      std::memcpy(&keys[i * 16], &it.key, 16);
    }
    for (int r = 0; r < p.R; ++r) res[(size_t)r * cap + i] = (uint32_t)(it.weight % kPrimes[r]);
  }
  cuda_check(cudaMemcpyAsync(v.keys, keys.data(), keys.size(), cudaMemcpyHostToDevice, ctx.stream), "upload keys");
  cuda_check(cudaMemcpyAsync(v.res, res.data(), res.size() * 4, cudaMemcpyHostToDevice, ctx.stream),
             "upload residues");
  cuda_check(cudaStreamSynchronize(ctx.stream), "upload synchronize");
  *cap_out = cap;
}

// Contract rows [row0, n) for items[lo, hi) as one merged device boundary.
// Row metrics are added into `rows` only when the whole batch succeeds.
static void run_batch(Ctx& ctx, const Plan& p, const std::vector<Item>& items, size_t lo, size_t hi, unsigned row0,
                      std::vector<RowAcc>& rows, RunStats& rs, bool collect) {
  RunStats local;
  std::vector<RowAcc> lrows(p.n);
  u64 cap = 0;
  int cur = 0;
  // Every pooled buffer is dead between batches: drop them if a previous,
  // larger call left the pool above this call's budget.
  if (ctx.pool_bytes > p.budget / 2) {
    buf_release(ctx, ctx.front[0]);
    buf_release(ctx, ctx.front[1]);
    buf_release(ctx, ctx.table);
  }
  upload_items(ctx, p, items, lo, hi, cur, &cap);
  u64 count = hi - lo;
  local.peak_states = count;
  for (unsigned row = row0; row < p.n; ++row) {
    auto t0 = std::chrono::steady_clock::now();
    const bool last_row = row + 1 == p.n;
    RowAcc& acc = lrows[row];
    acc.used = true;
    acc.device_row = true;
    acc.input_states = count;
    acc.candidates = (u128)count * p.n;
    StepOut so{};
    if (p.grain == QPEPS_GRAIN_SITE) {
      // Row-level successor count for the metrics (compiled-operator view).
      LaunchCfg cfg{p.key_bits, p.R, p.threads, ctx.sms};
      cuda_check(cudaMemsetAsync(ctx.d_sc, 0, sizeof(StepScalars), ctx.stream), "clear step scalars");
      cuda_check(launch_row_count(cfg, view_of(p, ctx.front[cur], cap), count, p.n, ctx.d_sc, ctx.stream),
                 "row count kernel");
      local.launches += 1;
      sync_scalars(ctx);
      const u64 row_terms = ctx.h_sc->terms;
      for (unsigned site = 0; site < p.n; ++site) {
        const bool fin = last_row && site + 1 == p.n;
        so = merge_step(ctx, p, cur, count, cap, true, site, fin, local, row);
        count = so.out;
        if (!fin) {
          cur = 1 - cur;
          cap = so.out_cap;
        }
      }
      acc.matched = acc.completed = row_terms;
    } else {
      so = p.merge == QPEPS_MERGE_PARTITION ? merge_step_partition(ctx, p, cur, count, cap, last_row, local, row)
                                            : merge_step(ctx, p, cur, count, cap, false, 0, last_row, local, row);
      count = so.out;
      if (!last_row) {
        cur = 1 - cur;
        cap = so.out_cap;
      }
      acc.matched = acc.completed = so.terms;
    }
    acc.output_states = count;
    for (int r = 0; r < p.R; ++r) acc.weight_res[r] = so.weight[r];
    local.peak_states = std::max<u64>(local.peak_states, count);
    if (last_row)
      for (int r = 0; r < p.R; ++r) local.final_res[r] = so.final_sum[r];
    acc.elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (count == 0 && !last_row) {
      // Empty boundary: nothing can complete; remaining rows see no input.
      for (unsigned r2 = row + 1; r2 < p.n; ++r2) {
        lrows[r2].used = true;
        lrows[r2].device_row = true;
      }
      break;
    }
  }
  (void)collect;
  // Commit.
  for (unsigned row = 0; row < p.n; ++row) {
    if (!lrows[row].used) continue;
    RowAcc& a = rows[row];
    a.used = true;
    a.device_row = a.device_row || lrows[row].device_row;
    a.input_states += lrows[row].input_states;
    a.output_states += lrows[row].output_states;
    a.candidates += lrows[row].candidates;
    a.matched += lrows[row].matched;
    a.completed += lrows[row].completed;
    for (int r = 0; r < p.R; ++r) a.weight_res[r] = (a.weight_res[r] + lrows[row].weight_res[r]) % kPrimes[r];
    a.elapsed += lrows[row].elapsed;
  }
  for (int r = 0; r < p.R; ++r) rs.final_res[r] = (rs.final_res[r] + local.final_res[r]) % kPrimes[r];
  rs.entries_in += local.entries_in;
  rs.entries_out += local.entries_out;
  rs.candidates += local.candidates;
  rs.launches += local.launches;
  rs.device_ms += local.device_ms;
  rs.merge_ms += local.merge_ms;
  rs.scatter_ms += local.scatter_ms;
  rs.merge_launches += local.merge_launches;
  rs.merge_bytes += local.merge_bytes;
  rs.peak_states = std::max(rs.peak_states, local.peak_states);
  rs.batches += 1;
}

// Host expansion of one row over a merged item list (used for the first
// row(s) that seed slices): compiled successor + optional orbit weights,
// merged by key (checked u128).
static std::vector<Item> host_expand(unsigned n, const std::vector<Item>& in, unsigned row, bool orbit, RowAcc& acc) {
  const u64 mask = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  std::map<u128, u128> next;
  acc.used = true;
  acc.input_states = in.size();
  for (const Item& it : in) {
    State s = unpack<u128>(it.key, n, mask);
    u64 fr = ~(s.cols | s.dr | s.dl) & mask;
    acc.candidates += n;
    while (fr) {
      const u64 b = fr & (~fr + 1);
      fr &= fr - 1;
      acc.matched += 1;
      u128 w = it.weight;
      if (row == 0 && orbit) {
        const unsigned c = (unsigned)__builtin_ctzll(b), mirror = n - 1 - c;
        if (c > mirror) continue;
        if (c < mirror && !mul_u128(w, 2, &w)) fail(QPEPS_ERR_OVERFLOW, "coefficient overflow in D4 orbit weighting");
      }
      acc.completed += 1;
      u128& dst = next[row_successor<u128>(s, b, n, mask)];
      if (!add_u128(dst, w, &dst)) fail(QPEPS_ERR_OVERFLOW, row_msg("coefficient overflow after row", row + 1));
    }
  }
  std::vector<Item> out;
  out.reserve(next.size());
  for (auto& kv : next) {
    out.push_back(Item{kv.first, kv.second});
    if (!add_u128(acc.weight_exact, kv.second, &acc.weight_exact))
      fail(QPEPS_ERR_OVERFLOW, row_msg("coefficient sum overflow after row", row + 1));
  }
  acc.output_states = out.size();
  return out;
}

struct Contraction {
  u128 count = 0;
  u64 peak_states = 1;
  std::vector<RowAcc> rows;
  RunStats rs;
  Plan plan{};
  unsigned slice_depth = 0;
  double elapsed = 0;
};

static Plan make_plan(Ctx& ctx, unsigned n, const qpeps_options& o) {
  Plan p;
  p.n = n;
  p.grain = o.granularity == QPEPS_GRAIN_SITE ? QPEPS_GRAIN_SITE : QPEPS_GRAIN_ROW;
  p.R = o.residues ? (int)o.residues : crt_plan(n);
  if (p.R < 1 || p.R > kMaxResidues) fail(QPEPS_ERR_INVALID, "residue count must be in 1..=4");
  if (o.residues && p.R < crt_plan(n))
    fail(QPEPS_ERR_RANGE, "forced residue count does not certify N! for this N");
  const unsigned narrow_max = p.grain == QPEPS_GRAIN_SITE ? 20 : 21;
  if (o.key_bits == 0)
    p.key_bits = n <= narrow_max ? 64 : 128;
  else if (o.key_bits == 64 || o.key_bits == 128)
    p.key_bits = (int)o.key_bits;
  else
    fail(QPEPS_ERR_INVALID, "key_bits must be 0, 64 or 128");
  if (p.key_bits == 64 && n > narrow_max) fail(QPEPS_ERR_RANGE, "packed boundary does not fit a u64 key for this N");
  if (o.device_budget_bytes)
    p.budget = (size_t)o.device_budget_bytes;
  else {
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    p.budget = (size_t)((double)(fr + ctx.pool_bytes) * 0.90);
  }
  p.threads = o.block_threads ? (int)o.block_threads : 256;
  const bool partition_ok = p.key_bits == 64 && p.grain == QPEPS_GRAIN_ROW;
  if (o.merge == QPEPS_MERGE_PARTITION && !partition_ok)
    fail(QPEPS_ERR_INVALID, "the partitioned merge needs u64 keys and row granularity");
  if (o.merge == QPEPS_MERGE_HASH)
    p.merge = QPEPS_MERGE_HASH;
  else if (o.merge == QPEPS_MERGE_PARTITION || o.merge == QPEPS_MERGE_AUTO)
    p.merge = partition_ok ? QPEPS_MERGE_PARTITION : QPEPS_MERGE_HASH;
  else
    fail(QPEPS_ERR_INVALID, "unknown merge strategy");
  return p;
}

// Contract rows from a list of seed items at depth row0 (rows already applied).
static void contract_items(Ctx& ctx, Contraction& out, std::vector<Item> items, unsigned row0) {
  const Plan& p = out.plan;
  // Batches: start with everything merged; on a capacity failure split the
  // batch in halves; a single item that still does not fit is deepened by one
  // host row into child items.
  struct Range {
    size_t lo, hi;
    unsigned depth;
    std::vector<Item>* src;
  };
  std::vector<std::vector<Item>*> owned;
  std::vector<Range> work;
  if (!items.empty()) {
    owned.push_back(new std::vector<Item>(std::move(items)));
    work.push_back(Range{0, owned.back()->size(), row0, owned.back()});
  }
  try {
    while (!work.empty()) {
      Range w = work.back();
      work.pop_back();
      if (w.depth >= p.n) {
        // Fully placed: every item is a finished board.
        const u64 mask = (p.n >= 64) ? ~0ull : ((1ull << p.n) - 1);
        for (size_t i = w.lo; i < w.hi; ++i) {
          const Item& it = (*w.src)[i];
          if (((u64)it.key & mask) == mask)
            for (int r = 0; r < p.R; ++r)
              out.rs.final_res[r] = (out.rs.final_res[r] + (u64)(it.weight % kPrimes[r])) % kPrimes[r];
        }
        continue;
      }
      try {
        run_batch(ctx, p, *w.src, w.lo, w.hi, w.depth, out.rows, out.rs, true);
      } catch (const Failure& f) {
        if (f.code != QPEPS_ERR_CAPACITY) throw;
        if (w.hi - w.lo > 1) {
          const size_t mid = w.lo + (w.hi - w.lo) / 2;
          work.push_back(Range{mid, w.hi, w.depth, w.src});
          work.push_back(Range{w.lo, mid, w.depth, w.src});
        } else {
          RowAcc scratch;
          std::vector<Item> one{(*w.src)[w.lo]};
          owned.push_back(new std::vector<Item>(host_expand(p.n, one, w.depth, false, scratch)));
          if (owned.back()->empty()) continue;
          out.slice_depth = std::max(out.slice_depth, w.depth + 1);
          // The host row is not a device row; its metrics are folded in.
          RowAcc& a = out.rows[w.depth];
          a.used = true;
          a.input_states += scratch.input_states;
          a.output_states += scratch.output_states;
          a.candidates += scratch.candidates;
          a.matched += scratch.matched;
          a.completed += scratch.completed;
          for (int r = 0; r < p.R; ++r)
            a.weight_res[r] = (a.weight_res[r] + (u64)(scratch.weight_exact % kPrimes[r])) % kPrimes[r];
          a.device_row = true;
          work.push_back(Range{0, owned.back()->size(), w.depth + 1, owned.back()});
        }
      }
    }
  } catch (...) {
    for (auto* v : owned) delete v;
    throw;
  }
  for (auto* v : owned) delete v;
}

static void contract(Ctx& ctx, unsigned n, const qpeps_options& o, const uint32_t* prefix, unsigned k,
                     Contraction& out) {
  auto t0 = std::chrono::steady_clock::now();
  if (n > 42) fail(QPEPS_ERR_RANGE, "the packed u128 virtual-boundary backend supports N <= 42");
  out.rows.assign(n, RowAcc());
  if (n == 0) {
    out.count = 1;
    out.peak_states = 1;
    return;
  }
  cuda_check(cudaSetDevice(ctx.device), "cudaSetDevice");
  certify_c(ctx.c);
  if (!ctx.c_uploaded) {
    cuda_check(upload_c_table(ctx.c_dev, ctx.stream), "upload C table");
    ctx.c_uploaded = true;
  }
  out.plan = make_plan(ctx, n, o);
  const u64 mask = (1ull << n) - 1;
  std::vector<Item> items;
  unsigned row0 = 0;
  if (k > 0) {
    if (k > n) fail(QPEPS_ERR_RANGE, "prefix longer than the board");
    State s{0, 0, 0};
    bool legal = true;
    for (unsigned r = 0; r < k; ++r) {
      if (prefix[r] >= n) fail(QPEPS_ERR_RANGE, "prefix column out of range");
      const u64 b = 1ull << prefix[r];
      if ((s.cols | s.dr | s.dl) & b) {
        legal = false;
        break;
      }
      const u128 key = row_successor<u128>(s, b, n, mask);
      s = unpack<u128>(key, n, mask);
    }
    if (!legal) {
      out.count = 0;
      out.peak_states = 1;
      return;
    }
    items.push_back(Item{pack<u128>(s.cols, s.dr, s.dl, n), 1});
    row0 = k;
  } else {
    items.push_back(Item{0, 1});
  }
  // Seed rows on the host: the first row applies the orbit weights
  // (src/lib.rs:721-749); further rows only when a slice depth is requested.
  const bool orbit = (k == 0) && o.symmetry;
  const unsigned depth = std::max<unsigned>(o.slice_depth ? o.slice_depth : 1, row0 == 0 ? 1 : row0);
  while (row0 < depth && row0 < n) {
    RowAcc& acc = out.rows[row0];
    items = host_expand(n, items, row0, orbit && row0 == 0, acc);
    acc.device_row = false;
    out.peak_states = std::max<u64>(out.peak_states, items.size());
    ++row0;
  }
  out.slice_depth = row0;
  contract_items(ctx, out, std::move(items), row0);
  out.peak_states = std::max<u64>(out.peak_states, out.rs.peak_states);
  // Count: host-finished boards plus device final sums, then CRT.
  u64 res[kMaxResidues];
  for (int r = 0; r < out.plan.R; ++r) res[r] = out.rs.final_res[r];
  out.count = crt_reconstruct(res, out.plan.R);
  if (out.count > factorial(n)) fail(QPEPS_ERR_CRT_BOUND, "CRT reconstruction exceeds certified N! count bound");
  out.elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

static u128 row_weight(const Contraction& c, const RowAcc& a) {
  if (!a.device_row) return a.weight_exact;
  u64 res[kMaxResidues];
  for (int r = 0; r < c.plan.R; ++r) res[r] = a.weight_res[r];
  return crt_reconstruct(res, c.plan.R);
}

static void fill_result(const Ctx& ctx, const Contraction& c, unsigned n, qpeps_result* r, qpeps_layer* layers,
                        uint32_t cap) {
  std::memset(r, 0, sizeof *r);
  r->n = n;
  r->count = to_abi(c.count);
  r->elapsed_s = c.elapsed;
  r->peak_states = c.peak_states;
  u128 cand = 0, matched = 0;
  uint32_t nl = 0;
  for (unsigned row = 0; row < c.rows.size(); ++row) {
    const RowAcc& a = c.rows[row];
    if (!a.used) continue;
    cand += a.candidates;
    matched += a.matched;
    if (layers && nl < cap) {
      qpeps_layer& L = layers[nl];
      std::memset(&L, 0, sizeof L);
      L.row = row;
      L.input_states = a.input_states;
      L.tensor_entries_examined = to_abi(a.examined);
      L.tensor_entries_matched = to_abi(a.tmatched);
      L.row_operator_candidates = to_abi(a.candidates);
      L.row_operator_matched = to_abi(a.matched);
      L.completed_row_terms = to_abi(a.completed);
      L.output_states = a.output_states;
      L.output_weight = to_abi(row_weight(c, a));
      L.elapsed_s = a.elapsed;
      L.peak_rss_bytes = ctx.pool_bytes;
    }
    ++nl;
  }
  r->n_layers = nl;
  r->tensor_entries_examined = to_abi(n ? 17 : 0);
  r->tensor_entries_matched = to_abi(n ? 17 : 0);
  r->row_operator_candidates = to_abi(cand);
  r->row_operator_matched = to_abi(matched);
  r->peak_rss_bytes = ctx.peak_pool_bytes;
  r->residues = n ? (uint32_t)c.plan.R : 0;
  r->key_bits = n ? (uint32_t)c.plan.key_bits : 0;
  r->slice_depth = c.slice_depth;
  r->batches = c.rs.batches;
  r->merge = n ? (uint32_t)c.plan.merge : 0;
  r->entries_in = c.rs.entries_in;
  r->entries_out = c.rs.entries_out;
  r->candidates = c.rs.candidates;
  r->gpu_launches = c.rs.launches;
  r->peak_device_bytes = ctx.peak_pool_bytes;
  r->device_ms = c.rs.device_ms;
  r->merge_kernel_ms = c.rs.merge_ms;
  r->scatter_kernel_ms = c.rs.scatter_ms;
  r->merge_kernel_launches = c.rs.merge_launches;
  r->merge_kernel_bytes = c.rs.merge_bytes;
  for (int i = 0; i < kMaxResidues; ++i) {
    r->residue_primes[i] = i < (n ? c.plan.R : 0) ? kPrimes[i] : 0;
    r->count_residues[i] = i < (n ? c.plan.R : 0) ? (uint64_t)(c.count % kPrimes[i]) : 0;
  }
}

static void set_err(char* err, size_t len, const std::string& msg) {
  if (err && len) std::snprintf(err, len, "%s", msg.c_str());
}

template <typename F>
static int guarded(char* err, size_t err_len, F&& f) {
  try {
    f();
    if (err && err_len) err[0] = 0;
    return QPEPS_OK;
  } catch (const Failure& e) {
    set_err(err, err_len, e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    set_err(err, err_len, "host allocation failed");
    return QPEPS_ERR_OOM;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return QPEPS_ERR_INVALID;
  }
}

static qpeps_options effective_options(const qpeps_options* opt) {
  qpeps_options o;
  qpeps_options_default(&o);
  if (opt) {
    if (opt->struct_size != sizeof(qpeps_options)) fail(QPEPS_ERR_INVALID, "qpeps_options.struct_size mismatch");
    o = *opt;
  }
  return o;
}

}  // namespace qpeps

using namespace qpeps;

extern "C" {

const char* qpeps_version(void) { return "qpeps-gb300 0.1.0 (sm_103a)"; }

void qpeps_options_default(qpeps_options* opt) {
  std::memset(opt, 0, sizeof *opt);
  opt->struct_size = sizeof(qpeps_options);
  opt->granularity = QPEPS_GRAIN_ROW;
  opt->merge = QPEPS_MERGE_AUTO;
  opt->symmetry = 1;
  opt->collect_layers = 1;
}

int qpeps_known_count(uint32_t n, qpeps_u128* out) {
  u128 v;
  if (!known_count(n, &v)) return QPEPS_ERR_RANGE;
  *out = to_abi(v);
  return QPEPS_OK;
}

int qpeps_ctx_create(int device, void** ctx_out, char* err, size_t err_len) {
  return guarded(err, err_len, [&] { *ctx_out = ctx_create(device); });
}

void qpeps_ctx_destroy(void* ctx) { ctx_free(static_cast<Ctx*>(ctx)); }

int qpeps_contract_rows(void* ctx, uint32_t n, const qpeps_options* opt, qpeps_result* result, qpeps_layer* layers,
                        uint32_t layers_cap, char* err, size_t err_len) {
  return guarded(err, err_len, [&] {
    if (!ctx || !result) fail(QPEPS_ERR_INVALID, "null context or result");
    Ctx& c = *static_cast<Ctx*>(ctx);
    qpeps_options o = effective_options(opt);
    Contraction con;
    contract(c, n, o, nullptr, 0, con);
    fill_result(c, con, n, result, layers, layers_cap);
  });
}

int qpeps_count(void* ctx, uint32_t n, const uint32_t* prefix, uint32_t k, const qpeps_options* opt,
                qpeps_u128* count_out, qpeps_result* stats_out, char* err, size_t err_len) {
  return guarded(err, err_len, [&] {
    if (!ctx || !count_out) fail(QPEPS_ERR_INVALID, "null context or output");
    if (k > 0 && !prefix) fail(QPEPS_ERR_INVALID, "null prefix with k > 0");
    Ctx& c = *static_cast<Ctx*>(ctx);
    qpeps_options o = effective_options(opt);
    Contraction con;
    contract(c, n, o, prefix, k, con);
    *count_out = to_abi(con.count);
    if (stats_out) fill_result(c, con, n, stats_out, nullptr, 0);
  });
}

int qpeps_count_batch(void* ctx, uint32_t num, const uint32_t* n, const uint32_t* k, const uint32_t* prefix_offset,
                      const uint32_t* prefix_cols, const qpeps_options* opt, qpeps_u128* counts, char* err,
                      size_t err_len) {
  return guarded(err, err_len, [&] {
    if (!ctx || (num && (!n || !k || !counts))) fail(QPEPS_ERR_INVALID, "null argument");
    Ctx& c = *static_cast<Ctx*>(ctx);
    qpeps_options o = effective_options(opt);
    for (uint32_t i = 0; i < num; ++i) {
      Contraction con;
      const uint32_t* pre = k[i] ? prefix_cols + prefix_offset[i] : nullptr;
      contract(c, n[i], o, pre, k[i], con);
      counts[i] = to_abi(con.count);
    }
  });
}

int qpeps_certify_c(const uint32_t* legs, const uint64_t* values, uint32_t len, char* err, size_t err_len) {
  return guarded(err, err_len, [&] {
    std::vector<CEntryH> c;
    for (uint32_t i = 0; i < len; ++i) c.push_back(CEntryH{legs[i], values[i]});
    certify_c(c);
  });
}

}  // extern "C"

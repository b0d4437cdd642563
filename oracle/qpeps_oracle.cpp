// CPU ORACLE — test infrastructure only.
//
// This file is a C++17 restatement of the reference crate's CPU algorithm for
// the exact N-Queens PEPS row-boundary contraction (Rust crate
// `nqueens-peps-naive`, file `src/lib.rs` unless noted). It exists so that the
// GPU product path can be checked against the reference's own algorithm on the
// same inputs. Only `tests/`, `__graft_entry__.smoke()` and the CPU-baseline
// leg of `bench.py` load it; the product library never links or calls it.
//
// Parity pin: the Rust reference cannot be compiled here (no cargo/rustc), so
// this restatement is pinned against the reference's own golden values:
// `known_count` (src/lib.rs:5752-5784), the per-row orbit frontier sizes in
// benchmarks/e35_frontier_audit_layers.csv, the peak-support / matched-work
// figures in benchmarks/e12_d4_orbit_slicing_release.csv,
// benchmarks/current_scaling_peps_release.csv and
// benchmarks/e36_joint_u64_release.csv, the dense per-row layers of
// benchmarks/n14_layers.csv, and the CRT known-answer test of
// src/lib.rs:6530-6545. Those values are committed as fixtures under
// tests/golden/ and checked by tests/test_oracle_golden.py.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace oracle {

using u8 = uint8_t;
using u64 = uint64_t;
using u128 = unsigned __int128;

struct Error {
  std::string msg;
};

static bool checked_add(u128 a, u128 b, u128* out) {
  u128 s = a + b;
  if (s < a) return false;
  *out = s;
  return true;
}

static bool checked_mul(u128 a, u128 b, u128* out) {
  if (a == 0 || b == 0) {
    *out = 0;
    return true;
  }
  u128 p = a * b;
  if (p / a != b) return false;
  *out = p;
  return true;
}

// ---------------------------------------------------------------------------
// Local tensors B and C (src/lib.rs:19-168).

struct VirtualLegs {
  u8 column_in, column_out, row_in, row_out, diag_dr_in, diag_dr_out, diag_dl_in, diag_dl_out;
  bool operator==(const VirtualLegs& o) const {
    return column_in == o.column_in && column_out == o.column_out && row_in == o.row_in &&
           row_out == o.row_out && diag_dr_in == o.diag_dr_in && diag_dr_out == o.diag_dr_out &&
           diag_dl_in == o.diag_dl_in && diag_dl_out == o.diag_dl_out;
  }
};

struct BEntry {
  u8 alpha;
  VirtualLegs legs;
  u128 value;
};

struct CEntry {
  VirtualLegs legs;
  u128 value;
};

// SiteTensorB::sec_vi, src/lib.rs:43-88: 16 pass-through entries with alpha=0
// (each channel in == out, signature bits column,row,dr,dl) and one occupied
// entry with alpha=1 emitting 0->1 on every channel.
static std::vector<BEntry> site_tensor_b_sec_vi() {
  std::vector<BEntry> entries;
  for (u8 signals = 0; signals < 16; ++signals) {
    u8 column = signals & 1, row = (signals >> 1) & 1, dr = (signals >> 2) & 1,
       dl = (signals >> 3) & 1;
    entries.push_back(BEntry{0, VirtualLegs{column, column, row, row, dr, dr, dl, dl}, 1});
  }
  entries.push_back(BEntry{1, VirtualLegs{0, 1, 0, 1, 0, 1, 0, 1}, 1});
  return entries;
}

// input_key, src/lib.rs:152-157.
static int input_key(u8 column_in, u8 row_in, u8 diag_dr_in, u8 diag_dl_in) {
  return column_in | (row_in << 1) | (diag_dr_in << 2) | (diag_dl_in << 3);
}

// legs_key, src/lib.rs:159-168.
static unsigned legs_key(const VirtualLegs& l) {
  return l.column_in | (l.column_out << 1) | (l.row_in << 2) | (l.row_out << 3) |
         (l.diag_dr_in << 4) | (l.diag_dr_out << 5) | (l.diag_dl_in << 6) | (l.diag_dl_out << 7);
}

struct SiteTensorC {
  std::vector<CEntry> entries;
  std::vector<CEntry> by_input[16];

  // SiteTensorC::from_b, src/lib.rs:102-131: sum B over alpha (checked),
  // order by legs_key, bucket by input signature.
  static SiteTensorC from_b(const std::vector<BEntry>& b) {
    SiteTensorC c;
    std::vector<CEntry> acc;
    for (const BEntry& e : b) {
      bool found = false;
      for (CEntry& a : acc) {
        if (a.legs == e.legs) {
          if (!checked_add(a.value, e.value, &a.value)) throw Error{"local tensor coefficient overflow"};
          found = true;
          break;
        }
      }
      if (!found) acc.push_back(CEntry{e.legs, e.value});
    }
    std::sort(acc.begin(), acc.end(),
              [](const CEntry& x, const CEntry& y) { return legs_key(x.legs) < legs_key(y.legs); });
    c.entries = acc;
    for (const CEntry& e : c.entries)
      c.by_input[input_key(e.legs.column_in, e.legs.row_in, e.legs.diag_dr_in, e.legs.diag_dl_in)]
          .push_back(e);
    return c;
  }
  static SiteTensorC sec_vi() { return from_b(site_tensor_b_sec_vi()); }
  const std::vector<CEntry>& matching(u8 ci, u8 ri, u8 dri, u8 dli) const {
    return by_input[input_key(ci, ri, dri, dli)];
  }
};

// CompiledRowOperator::compile, src/lib.rs:430-485. Fails closed unless C is
// exactly 16 identity pass-through signatures plus one all-channel 0->1 entry,
// every value 1.
struct CompiledRowOperator {
  CEntry occupied;
  static CompiledRowOperator compile(const SiteTensorC& tensor) {
    bool passthrough[16] = {false};
    bool have_occupied = false;
    CEntry occupied{};
    for (const CEntry& entry : tensor.entries) {
      const VirtualLegs& l = entry.legs;
      bool is_pass = l.column_in == l.column_out && l.row_in == l.row_out &&
                     l.diag_dr_in == l.diag_dr_out && l.diag_dl_in == l.diag_dl_out;
      bool is_occ = l.column_in == 0 && l.column_out == 1 && l.row_in == 0 && l.row_out == 1 &&
                    l.diag_dr_in == 0 && l.diag_dr_out == 1 && l.diag_dl_in == 0 &&
                    l.diag_dl_out == 1;
      if (entry.value != 1) throw Error{"compiled row operator requires unit Sec. VI coefficients"};
      if (is_pass) {
        int key = input_key(l.column_in, l.row_in, l.diag_dr_in, l.diag_dl_in);
        if (passthrough[key]) {
          char buf[64];
          std::snprintf(buf, sizeof buf, "duplicate C pass-through signature %d%d%d%d", (key >> 3) & 1,
                        (key >> 2) & 1, (key >> 1) & 1, key & 1);
          throw Error{buf};
        }
        passthrough[key] = true;
      } else if (is_occ) {
        if (have_occupied) throw Error{"multiple occupied C entries"};
        have_occupied = true;
        occupied = entry;
      } else {
        throw Error{"C contains an entry outside the Sec. VI row automaton"};
      }
    }
    for (bool p : passthrough)
      if (!p) throw Error{"C is missing a pass-through signature"};
    if (!have_occupied) throw Error{"C is missing the occupied entry"};
    return CompiledRowOperator{occupied};
  }
};

// ---------------------------------------------------------------------------
// Boundary state and packed key (src/lib.rs:170-178, 348-377).

struct BoundaryState {
  u64 columns, diag_dr, diag_dl;
  bool operator==(const BoundaryState& o) const {
    return columns == o.columns && diag_dr == o.diag_dr && diag_dl == o.diag_dl;
  }
};

// PackedBoundary: bits [0,n) columns, [n,2n) diag_dr, [2n,3n) diag_dl.
static u128 pack(const BoundaryState& s, unsigned n) {
  return (u128)s.columns | ((u128)s.diag_dr << n) | ((u128)s.diag_dl << (2 * n));
}
static BoundaryState unpack(u128 key, unsigned n) {
  u128 mask = (((u128)1) << n) - 1;
  return BoundaryState{(u64)(key & mask), (u64)((key >> n) & mask), (u64)((key >> (2 * n)) & mask)};
}
static u64 packed_columns(u128 key, unsigned n) {
  u128 mask = (((u128)1) << n) - 1;
  return (u64)(key & mask);
}

struct RowCounters {
  u128 tensor_examined = 0, tensor_matched = 0, operator_candidates = 0, operator_matched = 0;
  void add(const RowCounters& o) {
    tensor_examined += o.tensor_examined;
    tensor_matched += o.tensor_matched;
    operator_candidates += o.operator_candidates;
    operator_matched += o.operator_matched;
  }
};

static inline u8 bit(u64 mask, unsigned i) { return (u8)((mask >> i) & 1); }
static inline void set_bit(u64* mask, unsigned i, u8 v) {
  if (v == 1) *mask |= (u64)1 << i;
}
static inline u64 replace_bit(u64 mask, unsigned i, u8 v) {
  u64 sel = (u64)1 << i;
  return (mask & ~sel) | ((u64)v << i);
}

using Term = std::pair<BoundaryState, u128>;

// contract_one_row_sitewise, src/lib.rs:513-592: apply the indexed C entries
// one site at a time; the left boundary is v0 (row_in = 0), signals leaving the
// board are contracted with v2, and the right boundary keeps row_signal == 1
// (v1).
static void contract_one_row_sitewise(unsigned n, const SiteTensorC& tensor, const BoundaryState& parent,
                                      u128 parent_weight, RowCounters& counters, std::vector<Term>& out) {
  struct Partial {
    u64 co, dro, dlo;
    u8 row_signal;
    u128 weight;
  };
  std::vector<Partial> partials{Partial{0, 0, 0, 0, parent_weight}};
  std::vector<Partial> next;
  for (unsigned column = 0; column < n; ++column) {
    next.clear();
    u8 ci = bit(parent.columns, column), dri = bit(parent.diag_dr, column), dli = bit(parent.diag_dl, column);
    for (const Partial& p : partials) {
      const auto& matching = tensor.matching(ci, p.row_signal, dri, dli);
      counters.tensor_examined += matching.size();
      for (const CEntry& e : matching) {
        counters.tensor_matched += 1;
        Partial s{p.co, p.dro, p.dlo, e.legs.row_out, 0};
        if (!checked_mul(p.weight, e.value, &s.weight)) throw Error{"coefficient overflow in local C contraction"};
        set_bit(&s.co, column, e.legs.column_out);
        if (column + 1 < n) set_bit(&s.dro, column + 1, e.legs.diag_dr_out);
        if (column > 0) set_bit(&s.dlo, column - 1, e.legs.diag_dl_out);
        next.push_back(s);
      }
    }
    std::swap(partials, next);
  }
  for (const Partial& p : partials)
    if (p.row_signal == 1) out.push_back(Term{BoundaryState{p.co, p.dro, p.dlo}, p.weight});
}

// contract_one_row_compiled, src/lib.rs:600-638 (dense position scan).
static void contract_one_row_compiled(unsigned n, const CompiledRowOperator& op, const BoundaryState& parent,
                                      u128 parent_weight, RowCounters& counters, std::vector<Term>& out) {
  const VirtualLegs& legs = op.occupied.legs;
  u64 board_mask = (n == 64) ? ~(u64)0 : (((u64)1 << n) - 1);
  for (unsigned column = 0; column < n; ++column) {
    counters.operator_candidates += 1;
    if (bit(parent.columns, column) != legs.column_in || bit(parent.diag_dr, column) != legs.diag_dr_in ||
        bit(parent.diag_dl, column) != legs.diag_dl_in)
      continue;
    counters.operator_matched += 1;
    u64 columns_out = replace_bit(parent.columns, column, legs.column_out);
    u64 dr_at = replace_bit(parent.diag_dr, column, legs.diag_dr_out);
    u64 dl_at = replace_bit(parent.diag_dl, column, legs.diag_dl_out);
    u128 w;
    if (!checked_mul(parent_weight, op.occupied.value, &w)) throw Error{"coefficient overflow in compiled row operator"};
    out.push_back(Term{BoundaryState{columns_out, (dr_at << 1) & board_mask, dl_at >> 1}, w});
  }
}

// contract_one_row_compiled_sparse, src/lib.rs:640-689 (iterate set bits only).
static void contract_one_row_compiled_sparse(unsigned n, const CompiledRowOperator& op, const BoundaryState& parent,
                                             u128 parent_weight, RowCounters& counters, std::vector<Term>& out) {
  const VirtualLegs& legs = op.occupied.legs;
  if (legs.row_in != 0) throw Error{"sparse row iterator requires occupied row_in to match the left v0 boundary"};
  u64 board_mask = ((u64)1 << n) - 1;
  auto matching_bits = [&](u64 mask, u8 required) -> u64 {
    if (required == 0) return (~mask) & board_mask;
    if (required == 1) return mask & board_mask;
    throw Error{"compiled C entry contains a non-binary incoming signal"};
  };
  u64 positions = matching_bits(parent.columns, legs.column_in) & matching_bits(parent.diag_dr, legs.diag_dr_in) &
                  matching_bits(parent.diag_dl, legs.diag_dl_in);
  u128 w;
  if (!checked_mul(parent_weight, op.occupied.value, &w)) throw Error{"coefficient overflow in sparse compiled row operator"};
  while (positions) {
    u64 selected = positions & (~positions + 1);
    unsigned column = (unsigned)__builtin_ctzll(selected);
    positions &= positions - 1;
    counters.operator_candidates += 1;
    counters.operator_matched += 1;
    u64 columns_out = replace_bit(parent.columns, column, legs.column_out);
    u64 dr_at = replace_bit(parent.diag_dr, column, legs.diag_dr_out);
    u64 dl_at = replace_bit(parent.diag_dl, column, legs.diag_dl_out);
    out.push_back(Term{BoundaryState{columns_out, (dr_at << 1) & board_mask, dl_at >> 1}, w});
  }
}

enum class Position { Dense = 0, Sparse = 1 };
enum class Symmetry { None = 0, TopRowVerticalOrbits = 1 };

static void contract_one_row(unsigned n, const CompiledRowOperator& op, const BoundaryState& parent, u128 weight,
                             RowCounters& counters, Position mode, std::vector<Term>& out) {
  if (mode == Position::Dense)
    contract_one_row_compiled(n, op, parent, weight, counters, out);
  else
    contract_one_row_compiled_sparse(n, op, parent, weight, counters, out);
}

// top_row_vertical_orbit_weight, src/lib.rs:721-732: column c < mirror -> 2,
// c == mirror (odd-N centre) -> 1, c > mirror -> dropped (0).
static unsigned top_row_vertical_orbit_weight(unsigned n, const BoundaryState& successor) {
  unsigned column = (unsigned)__builtin_ctzll(successor.columns);
  unsigned mirror = n - 1 - column;
  if (column > mirror) return 0;
  if (column == mirror) return 1;
  return 2;
}

// apply_top_row_symmetry, src/lib.rs:734-749.
static void apply_top_row_symmetry(unsigned n, std::vector<Term>& terms, size_t from) {
  size_t w = from;
  for (size_t r = from; r < terms.size(); ++r) {
    unsigned m = top_row_vertical_orbit_weight(n, terms[r].first);
    if (m == 0) continue;
    u128 weighted;
    if (!checked_mul(terms[r].second, m, &weighted)) throw Error{"coefficient overflow in D4 orbit weighting"};
    terms[w++] = Term{terms[r].first, weighted};
  }
  terms.resize(w);
}

// ---------------------------------------------------------------------------
// Result types (src/lib.rs:388-415).

struct LayerMetric {
  unsigned row;
  u64 input_states;
  u128 tensor_entries_examined, tensor_entries_matched, row_operator_candidates, row_operator_matched,
      completed_row_terms;
  u64 output_states;
  u128 output_weight;
  double elapsed_s;
  u64 peak_rss_bytes;
};

struct ContractionResult {
  unsigned n;
  u128 count;
  double elapsed_s;
  u64 peak_states;
  u128 tensor_entries_examined, tensor_entries_matched, row_operator_candidates, row_operator_matched;
  u64 peak_rss_bytes;
  std::vector<LayerMetric> layers;
};

static double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

static ContractionResult empty_board_result(unsigned n) {
  ContractionResult r{};
  r.n = n;
  r.count = 1;
  r.peak_states = 1;
  return r;
}

using KV = std::pair<u128, u128>;

// In-place checked reduce of a key-sorted candidate list (src/lib.rs:5354-5367).
static void reduce_sorted(std::vector<KV>& c, unsigned row) {
  size_t write = 0;
  for (size_t read = 0; read < c.size(); ++read) {
    KV kv = c[read];
    if (write > 0 && c[write - 1].first == kv.first) {
      if (!checked_add(c[write - 1].second, kv.second, &c[write - 1].second)) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "coefficient overflow after row %u", row + 1);
        throw Error{buf};
      }
    } else {
      c[write++] = kv;
    }
  }
  c.resize(write);
}

static u128 output_weight_of(const std::vector<KV>& boundary, unsigned row) {
  u128 sum = 0;
  for (const KV& kv : boundary)
    if (!checked_add(sum, kv.second, &sum)) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "coefficient sum overflow after row %u", row + 1);
      throw Error{buf};
    }
  return sum;
}

// Final v1 (columns) / v2 (diagonals) contraction, src/lib.rs:5393-5401.
static u128 final_count(const std::vector<KV>& boundary, unsigned n) {
  u64 board_mask = ((u64)1 << n) - 1;
  u128 count = 0;
  for (const KV& kv : boundary)
    if (packed_columns(kv.first, n) == board_mask)
      if (!checked_add(count, kv.second, &count)) throw Error{"final coefficient sum overflow"};
  return count;
}

// Options shared by the row drivers. `rows` limits the contraction to the
// first `rows` rows (a bounded sample of the same workload; rows == n is the
// full contraction). `initial` replaces the empty-board boundary with the
// boundary after a placed prefix (serving requests), in which case `row0` is
// the first row still to contract.
struct DriverOptions {
  unsigned rows;
  unsigned row0 = 0;
  std::vector<KV> initial;
  std::vector<KV>* final_boundary = nullptr;  // receives the boundary after the last contracted row
};

// contract_rows_sort_reduce_with_modes, src/lib.rs:5287-5415 (the `solve` path
// when called with TopRowVerticalOrbits + Dense via contract_rows, 758/784).
static ContractionResult contract_rows_sort_reduce_with_modes(unsigned n, Symmetry sym, Position pos,
                                                              const DriverOptions& opt) {
  if (n > 42) throw Error{"the packed u128 virtual-boundary backend supports N <= 42"};
  if (n == 0) return empty_board_result(n);
  SiteTensorC tensor = SiteTensorC::sec_vi();
  CompiledRowOperator op = CompiledRowOperator::compile(tensor);
  std::vector<KV> boundary = opt.initial.empty() ? std::vector<KV>{KV{pack(BoundaryState{0, 0, 0}, n), 1}} : opt.initial;
  u64 peak_states = boundary.size();
  u128 total_cand = 0, total_matched = 0;
  ContractionResult res{};
  res.n = n;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<Term> row_terms;
  for (unsigned row = opt.row0; row < opt.rows; ++row) {
    auto lt0 = std::chrono::steady_clock::now();
    u64 input_states = boundary.size();
    RowCounters counters;
    u128 completed = 0;
    std::vector<KV> candidates;
    for (const KV& kv : boundary) {
      row_terms.clear();
      contract_one_row(n, op, unpack(kv.first, n), kv.second, counters, pos, row_terms);
      if (row == 0 && sym == Symmetry::TopRowVerticalOrbits) apply_top_row_symmetry(n, row_terms, 0);
      completed += row_terms.size();
      for (const Term& t : row_terms) candidates.push_back(KV{pack(t.first, n), t.second});
    }
    std::vector<KV>().swap(boundary);
    std::sort(candidates.begin(), candidates.end(), [](const KV& a, const KV& b) { return a.first < b.first; });
    reduce_sorted(candidates, row);
    boundary.swap(candidates);
    u128 ow = output_weight_of(boundary, row);
    peak_states = std::max<u64>(peak_states, boundary.size());
    total_cand += counters.operator_candidates;
    total_matched += counters.operator_matched;
    res.layers.push_back(LayerMetric{row, input_states, counters.tensor_examined, counters.tensor_matched,
                                     counters.operator_candidates, counters.operator_matched, completed,
                                     boundary.size(), ow, seconds_since(lt0), 0});
  }
  res.count = (opt.rows == n) ? final_count(boundary, n) : 0;
  if (opt.final_boundary) *opt.final_boundary = boundary;
  res.elapsed_s = seconds_since(t0);
  res.peak_states = peak_states;
  res.tensor_entries_examined = 17;
  res.tensor_entries_matched = 17;
  res.row_operator_candidates = total_cand;
  res.row_operator_matched = total_matched;
  return res;
}

// Parallel merge sort by key for the threaded driver: each worker sorts one
// contiguous chunk, then chunks are merged pairwise in parallel rounds. It
// gives the same sorted sequence as the reference's par_sort_unstable_by_key
// up to the order of equal keys, which the checked reduce does not observe.
static void parallel_sort_by_key(std::vector<KV>& v, unsigned threads) {
  auto less = [](const KV& a, const KV& b) { return a.first < b.first; };
  if (threads <= 1 || v.size() < 1u << 15) {
    std::sort(v.begin(), v.end(), less);
    return;
  }
  size_t parts = threads;
  std::vector<size_t> bounds(parts + 1);
  for (size_t i = 0; i <= parts; ++i) bounds[i] = v.size() * i / parts;
  {
    std::vector<std::thread> ws;
    for (size_t i = 0; i < parts; ++i)
      ws.emplace_back([&, i] { std::sort(v.begin() + bounds[i], v.begin() + bounds[i + 1], less); });
    for (auto& w : ws) w.join();
  }
  std::vector<KV> tmp(v.size());
  std::vector<KV>* src = &v;
  std::vector<KV>* dst = &tmp;
  while (bounds.size() > 2) {
    std::vector<size_t> nb;
    std::vector<std::thread> ws;
    for (size_t i = 0; i + 1 < bounds.size(); i += 2) {
      size_t a = bounds[i], b = bounds[i + 1];
      size_t c = (i + 2 < bounds.size()) ? bounds[i + 2] : b;
      nb.push_back(a);
      ws.emplace_back([=, &less] {
        if (c > b)
          std::merge(src->begin() + a, src->begin() + b, src->begin() + b, src->begin() + c, dst->begin() + a, less);
        else
          std::copy(src->begin() + a, src->begin() + b, dst->begin() + a);
      });
    }
    nb.push_back(v.size());
    for (auto& w : ws) w.join();
    bounds.swap(nb);
    std::swap(src, dst);
  }
  if (src != &v) v.swap(*src);
}

// contract_rows_parallel_sort_reduce_with_modes, src/lib.rs:5469-5626: parents
// are expanded in 4*threads contiguous slices on worker threads (rayon
// par_chunks), candidates are concatenated in slice order, sorted in
// parallel, then reduced serially with checked addition.
static ContractionResult contract_rows_parallel_sort_reduce_with_modes(unsigned n, unsigned threads, Symmetry sym,
                                                                       Position pos, const DriverOptions& opt) {
  if (threads == 0) throw Error{"parallel sort-reduce requires at least one thread"};
  if (n > 42) throw Error{"the packed u128 virtual-boundary backend supports N <= 42"};
  if (n == 0) return empty_board_result(n);
  SiteTensorC tensor = SiteTensorC::sec_vi();
  CompiledRowOperator op = CompiledRowOperator::compile(tensor);
  std::vector<KV> boundary = opt.initial.empty() ? std::vector<KV>{KV{pack(BoundaryState{0, 0, 0}, n), 1}} : opt.initial;
  u64 peak_states = boundary.size();
  u128 total_cand = 0, total_matched = 0;
  ContractionResult res{};
  res.n = n;
  auto t0 = std::chrono::steady_clock::now();
  for (unsigned row = opt.row0; row < opt.rows; ++row) {
    auto lt0 = std::chrono::steady_clock::now();
    u64 input_states = boundary.size();
    size_t target_slices = std::max<size_t>((size_t)threads * 4, 1);
    size_t chunk = std::max<size_t>((input_states + target_slices - 1) / target_slices, 1);
    size_t nchunks = (input_states + chunk - 1) / chunk;
    std::vector<std::vector<KV>> locals(nchunks);
    std::vector<RowCounters> local_counters(nchunks);
    std::vector<std::string> errors(nchunks);
    std::atomic<size_t> next{0};
    auto worker = [&] {
      std::vector<Term> terms;
      for (;;) {
        size_t ci = next.fetch_add(1);
        if (ci >= nchunks) break;
        try {
          size_t lo = ci * chunk, hi = std::min<size_t>(lo + chunk, input_states);
          for (size_t i = lo; i < hi; ++i) {
            terms.clear();
            contract_one_row(n, op, unpack(boundary[i].first, n), boundary[i].second, local_counters[ci], pos, terms);
            if (row == 0 && sym == Symmetry::TopRowVerticalOrbits) apply_top_row_symmetry(n, terms, 0);
            for (const Term& t : terms) locals[ci].push_back(KV{pack(t.first, n), t.second});
          }
        } catch (const Error& e) {
          errors[ci] = e.msg;
        }
      }
    };
    {
      unsigned nw = (unsigned)std::min<size_t>(threads, nchunks);
      std::vector<std::thread> ws;
      for (unsigned i = 1; i < nw; ++i) ws.emplace_back(worker);
      worker();
      for (auto& w : ws) w.join();
    }
    for (const std::string& e : errors)
      if (!e.empty()) throw Error{e};
    u128 completed = 0;
    for (auto& l : locals) completed += l.size();
    std::vector<KV> candidates;
    candidates.reserve((size_t)completed);
    RowCounters counters;
    for (size_t i = 0; i < nchunks; ++i) {
      candidates.insert(candidates.end(), locals[i].begin(), locals[i].end());
      std::vector<KV>().swap(locals[i]);
      counters.add(local_counters[i]);
    }
    std::vector<KV>().swap(boundary);
    parallel_sort_by_key(candidates, threads);
    reduce_sorted(candidates, row);
    boundary.swap(candidates);
    u128 ow = output_weight_of(boundary, row);
    peak_states = std::max<u64>(peak_states, boundary.size());
    total_cand += counters.operator_candidates;
    total_matched += counters.operator_matched;
    res.layers.push_back(LayerMetric{row, input_states, counters.tensor_examined, counters.tensor_matched,
                                     counters.operator_candidates, counters.operator_matched, completed,
                                     boundary.size(), ow, seconds_since(lt0), 0});
  }
  res.count = (opt.rows == n) ? final_count(boundary, n) : 0;
  if (opt.final_boundary) *opt.final_boundary = boundary;
  res.elapsed_s = seconds_since(t0);
  res.peak_states = peak_states;
  res.tensor_entries_examined = 17;
  res.tensor_entries_matched = 17;
  res.row_operator_candidates = total_cand;
  res.row_operator_matched = total_matched;
  return res;
}

struct U128Hash {
  size_t operator()(u128 k) const {
    u64 x = (u64)k ^ (u64)(k >> 64);
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return (size_t)x;
  }
};

// contract_rows_with_backend, src/lib.rs:5633-5750: the HashMap
// materialisation with the compiled (default) or sitewise row backend and no
// orbit slicing.
static ContractionResult contract_rows_with_backend(unsigned n, bool sitewise, const DriverOptions& opt) {
  if (n > 42) throw Error{"the packed u128 virtual-boundary backend supports N <= 42"};
  if (n == 0) return empty_board_result(n);
  SiteTensorC tensor = SiteTensorC::sec_vi();
  CompiledRowOperator op = CompiledRowOperator::compile(tensor);
  std::unordered_map<u128, u128, U128Hash> boundary;
  if (opt.initial.empty())
    boundary.emplace(pack(BoundaryState{0, 0, 0}, n), 1);
  else
    for (const KV& kv : opt.initial) boundary.emplace(kv.first, kv.second);
  u64 peak_states = boundary.size();
  u128 total_examined = sitewise ? 0 : 17, total_matched_t = sitewise ? 0 : 17;
  u128 total_cand = 0, total_matched = 0;
  ContractionResult res{};
  res.n = n;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<Term> terms;
  for (unsigned row = opt.row0; row < opt.rows; ++row) {
    auto lt0 = std::chrono::steady_clock::now();
    u64 input_states = boundary.size();
    RowCounters counters;
    u128 completed = 0;
    std::unordered_map<u128, u128, U128Hash> next;
    next.reserve(boundary.size() * 2);
    for (const auto& kv : boundary) {
      terms.clear();
      if (sitewise)
        contract_one_row_sitewise(n, tensor, unpack(kv.first, n), kv.second, counters, terms);
      else
        contract_one_row_compiled(n, op, unpack(kv.first, n), kv.second, counters, terms);
      for (const Term& t : terms) {
        completed += 1;
        u128& c = next[pack(t.first, n)];
        if (!checked_add(c, t.second, &c)) {
          char buf[64];
          std::snprintf(buf, sizeof buf, "coefficient overflow after row %u", row + 1);
          throw Error{buf};
        }
      }
    }
    u128 ow = 0;
    for (const auto& kv : next)
      if (!checked_add(ow, kv.second, &ow)) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "coefficient sum overflow after row %u", row + 1);
        throw Error{buf};
      }
    peak_states = std::max<u64>(peak_states, next.size());
    total_examined += counters.tensor_examined;
    total_matched_t += counters.tensor_matched;
    total_cand += counters.operator_candidates;
    total_matched += counters.operator_matched;
    res.layers.push_back(LayerMetric{row, input_states, counters.tensor_examined, counters.tensor_matched,
                                     counters.operator_candidates, counters.operator_matched, completed, next.size(),
                                     ow, seconds_since(lt0), 0});
    boundary.swap(next);
  }
  std::vector<KV> fb(boundary.begin(), boundary.end());
  res.count = (opt.rows == n) ? final_count(fb, n) : 0;
  if (opt.final_boundary) {
    std::sort(fb.begin(), fb.end(), [](const KV& a, const KV& b) { return a.first < b.first; });
    *opt.final_boundary = fb;
  }
  res.elapsed_s = seconds_since(t0);
  res.peak_states = peak_states;
  res.tensor_entries_examined = total_examined;
  res.tensor_entries_matched = total_matched_t;
  res.row_operator_candidates = total_cand;
  res.row_operator_matched = total_matched;
  return res;
}

// known_count, src/lib.rs:5752-5784 (OEIS A000170, Q(0..27)).
// ---------------------------------------------------------------------------
// Explicit-C generic site frontier (src/lib.rs:940-967, 1419-1711): contract
// the explicit C tensor one site at a time over an arbitrary site order, the
// boundary being the values of the currently open virtual bonds (bit i of a
// key = value of the i-th open bond in increasing bond id).

// A site leg: a virtual bond shared with a neighbouring site, or an open
// boundary leg whose allowed values are the set bits of `allowed`
// (FrontierLeg, src/lib.rs:1419-1491).
struct OqFrontierLeg {
  bool edge;
  unsigned id;
  u8 allowed;
};

struct OqFrontierSite {
  unsigned row, column;
  OqFrontierLeg legs[8];  // column in/out, row in/out, dr in/out, dl in/out
};

// explicit_frontier_sites, src/lib.rs:1419-1491: bond ids of the four bond
// families (row bonds, column bonds, down-right and down-left diagonal
// bonds); edge-of-board legs are open: incoming legs carry 0, outgoing column
// and row legs must carry 1 (one queen per column / row), outgoing diagonal
// legs are free.
static std::vector<OqFrontierSite> explicit_frontier_sites(unsigned n) {
  const unsigned span = n ? n - 1 : 0;
  const unsigned column_base = n * span, dr_base = column_base + n * span, dl_base = dr_base + span * span;
  auto bond = [](unsigned id) { return OqFrontierLeg{true, id, 0}; };
  auto open = [](u8 allowed) { return OqFrontierLeg{false, 0, allowed}; };
  std::vector<OqFrontierSite> sites;
  sites.reserve((size_t)n * n);
  for (unsigned r = 0; r < n; ++r)
    for (unsigned c = 0; c < n; ++c) {
      OqFrontierSite s{r, c, {}};
      s.legs[0] = r == 0 ? open(0b01) : bond(column_base + (r - 1) * n + c);
      s.legs[1] = r + 1 == n ? open(0b10) : bond(column_base + r * n + c);
      s.legs[2] = c == 0 ? open(0b01) : bond(r * span + c - 1);
      s.legs[3] = c + 1 == n ? open(0b10) : bond(r * span + c);
      s.legs[4] = (r == 0 || c == 0) ? open(0b01) : bond(dr_base + (r - 1) * span + c - 1);
      s.legs[5] = (r + 1 == n || c + 1 == n) ? open(0b11) : bond(dr_base + r * span + c);
      s.legs[6] = (r == 0 || c + 1 == n) ? open(0b01) : bond(dl_base + (r - 1) * span + c);
      s.legs[7] = (r + 1 == n || c == 0) ? open(0b11) : bond(dl_base + r * span + c - 1);
      sites.push_back(s);
    }
  return sites;
}

// explicit_frontier_order, src/lib.rs:1493-1503: row-major, or by
// (row + column, row) for the top-left diamond.
static std::vector<unsigned> explicit_frontier_order(unsigned n, unsigned order) {
  std::vector<unsigned> idx((size_t)n * n);
  for (unsigned i = 0; i < idx.size(); ++i) idx[i] = i;
  if (order == 1)
    std::sort(idx.begin(), idx.end(), [n](unsigned a, unsigned b) {
      const unsigned ra = a / n, rb = b / n, sa = ra + a % n, sb = rb + b % n;
      return sa != sb ? sa < sb : ra < rb;
    });
  return idx;
}

struct ExplicitFrontierResult {
  unsigned n = 0, order = 0;
  bool complete = false;
  u128 count = 0;
  double elapsed = 0;
  u64 peak_states = 1, peak_open_bonds = 0;
  u128 examined = 0, accepted = 0;
  u64 contracted_sites = 0;
};

// contract_explicit_c_frontier_kernel, src/lib.rs:1519-1711.
static ExplicitFrontierResult contract_explicit_c_frontier(unsigned n, unsigned order, u64 support_limit) {
  if (n > 21) throw Error{"explicit-C frontier key supports N <= 21"};
  if (support_limit == 0) throw Error{"explicit-C frontier support limit must be positive"};
  ExplicitFrontierResult res;
  res.n = n;
  res.order = order;
  if (n == 0) {
    res.complete = true;
    res.count = 1;
    return res;
  }
  const SiteTensorC tensor = SiteTensorC::sec_vi();
  if (tensor.entries.size() != 17) throw Error{"explicit-C frontier requires the Sec. VI 17-entry tensor"};
  const auto sites = explicit_frontier_sites(n);
  const auto ordering = explicit_frontier_order(n, order);
  std::unordered_map<u128, u128, U128Hash> boundary{{0, 1}};
  std::vector<unsigned> open_edges;
  const auto t0 = std::chrono::steady_clock::now();
  for (size_t step = 0; step < ordering.size(); ++step) {
    const OqFrontierSite& site = sites[ordering[step]];
    std::unordered_map<unsigned, unsigned> old_pos;
    for (unsigned i = 0; i < open_edges.size(); ++i) old_pos[open_edges[i]] = i;
    std::vector<unsigned> incident;
    for (const OqFrontierLeg& l : site.legs)
      if (l.edge) incident.push_back(l.id);
    std::vector<unsigned> next;
    for (unsigned e : open_edges)
      if (std::find(incident.begin(), incident.end(), e) == incident.end()) next.push_back(e);
    for (unsigned e : incident)
      if (!old_pos.count(e)) next.push_back(e);
    std::sort(next.begin(), next.end());
    if (next.size() > 128)
      throw Error{"explicit-C frontier exceeds 128 open bonds at site (" + std::to_string(site.row) + "," +
                  std::to_string(site.column) + ")"};
    std::unordered_map<unsigned, unsigned> next_pos;
    for (unsigned i = 0; i < next.size(); ++i) next_pos[next[i]] = i;
    std::vector<std::pair<unsigned, unsigned>> carry;  // (old position, next position)
    for (unsigned i = 0; i < open_edges.size(); ++i) {
      auto it = next_pos.find(open_edges[i]);
      if (it != next_pos.end()) carry.push_back({i, it->second});
    }
    struct Transition {
      u128 required_mask, required_value, added_value, local_value;
    };
    std::vector<Transition> transitions;
    for (const CEntry& e : tensor.entries) {
      const u8 values[8] = {e.legs.column_in,  e.legs.column_out,  e.legs.row_in,     e.legs.row_out,
                            e.legs.diag_dr_in, e.legs.diag_dr_out, e.legs.diag_dl_in, e.legs.diag_dl_out};
      Transition t{0, 0, 0, e.value};
      bool keep = true;
      for (int l = 0; l < 8 && keep; ++l) {
        const OqFrontierLeg& leg = site.legs[l];
        if (!leg.edge) {
          keep = (leg.allowed >> values[l]) & 1;
        } else {
          auto it = old_pos.find(leg.id);
          if (it != old_pos.end()) {
            t.required_mask |= (u128)1 << it->second;
            t.required_value |= (u128)values[l] << it->second;
          } else {
            t.added_value |= (u128)values[l] << next_pos[leg.id];
          }
        }
      }
      if (keep) transitions.push_back(t);
    }
    std::unordered_map<u128, u128, U128Hash> candidates;
    for (const auto& kv : boundary) {
      res.examined += 17;
      u128 carried = 0;
      for (const auto& cp : carry) carried |= ((kv.first >> cp.first) & 1) << cp.second;
      for (const Transition& t : transitions) {
        if ((kv.first & t.required_mask) != t.required_value) continue;
        res.accepted += 1;
        u128 contribution;
        if (!checked_mul(kv.second, t.local_value, &contribution))
          throw Error{"explicit-C coefficient multiplication overflow at site (" + std::to_string(site.row) + "," +
                      std::to_string(site.column) + ")"};
        u128& acc = candidates[carried | t.added_value];
        if (!checked_add(acc, contribution, &acc))
          throw Error{"explicit-C coefficient addition overflow at site (" + std::to_string(site.row) + "," +
                      std::to_string(site.column) + ")"};
        if (candidates.size() > support_limit) {
          res.peak_states = std::max<u64>(res.peak_states, candidates.size());
          res.peak_open_bonds = std::max<u64>(res.peak_open_bonds, next.size());
          res.contracted_sites = step;
          res.elapsed = seconds_since(t0);
          return res;
        }
      }
    }
    boundary.swap(candidates);
    open_edges.swap(next);
    res.peak_states = std::max<u64>(res.peak_states, boundary.size());
    res.peak_open_bonds = std::max<u64>(res.peak_open_bonds, open_edges.size());
  }
  if (!open_edges.empty()) throw Error{"explicit-C contraction ended with uncontracted virtual bonds"};
  auto it = boundary.find(0);
  res.count = it == boundary.end() ? 0 : it->second;
  res.complete = true;
  res.contracted_sites = (u64)n * n;
  res.elapsed = seconds_since(t0);
  return res;
}

static bool known_count(unsigned n, u128* out) {
  static const char* counts[28] = {"1",
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
  if (n >= 28) return false;
  u128 v = 0;
  for (const char* p = counts[n]; *p; ++p) v = v * 10 + (u128)(*p - '0');
  *out = v;
  return true;
}

// ---------------------------------------------------------------------------
// DFS bitboard oracle (src/dfs_bitmask.rs:67-340).

static u64 dfs_search(u64 board_mask, u64 columns, u64 diag_left, u64 diag_right, unsigned rows_left) {
  u64 available = board_mask & ~(columns | diag_left | diag_right);
  if (rows_left == 1) return available != 0 ? 1 : 0;
  u64 count = 0;
  while (available) {
    u64 b = available & (~available + 1);
    available ^= b;
    count += dfs_search(board_mask, columns | b, ((diag_left | b) << 1) & board_mask, (diag_right | b) >> 1,
                        rows_left - 1);
  }
  return count;
}

struct DfsTask {
  u64 columns, diag_left, diag_right;
  unsigned weight, rows_placed;
};

// seed_tasks (111-138), split_once (140-157), make_tasks (159-198), run_task
// and count_dfs_bitmask_impl (200-340).
static u128 count_dfs_bitmask(unsigned n, unsigned threads) {
  if (n > 27) throw Error{"DFS bitmask baseline supports N <= 27"};
  if (threads == 0) throw Error{"thread count must be positive"};
  if (n == 0) return 1;
  u64 board_mask = ((u64)1 << n) - 1;
  std::vector<DfsTask> tasks;
  for (unsigned c = 0; c < n / 2; ++c) {
    u64 b = (u64)1 << c;
    tasks.push_back(DfsTask{b, b << 1, b >> 1, 2, 1});
  }
  if (n % 2 == 1) {
    u64 b = (u64)1 << (n / 2);
    tasks.push_back(DfsTask{b, b << 1, b >> 1, 1, 1});
  }
  size_t target = threads == 1 ? 1 : (size_t)threads * 64;
  unsigned depth = tasks.empty() ? 0 : tasks[0].rows_placed;
  while (tasks.size() < target && depth + 1 < n) {
    std::vector<DfsTask> children;
    for (const DfsTask& t : tasks) {
      u64 avail = board_mask & ~(t.columns | t.diag_left | t.diag_right);
      while (avail) {
        u64 b = avail & (~avail + 1);
        avail ^= b;
        children.push_back(DfsTask{t.columns | b, ((t.diag_left | b) << 1) & board_mask, (t.diag_right | b) >> 1,
                                   t.weight, t.rows_placed + 1});
      }
    }
    tasks.swap(children);
    ++depth;
    if (tasks.empty()) break;
  }
  auto run = [&](const DfsTask& t) -> u128 {
    unsigned rows_left = n - t.rows_placed;
    u64 raw = rows_left == 0 ? 1 : dfs_search(board_mask, t.columns, t.diag_left, t.diag_right, rows_left);
    return (u128)raw * t.weight;
  };
  unsigned workers = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, tasks.size()));
  if (workers == 1) {
    u128 total = 0;
    for (const DfsTask& t : tasks) total += run(t);
    return total;
  }
  std::atomic<size_t> next{0};
  std::vector<u128> partial(workers, 0);
  std::vector<std::thread> ws;
  for (unsigned w = 0; w < workers; ++w)
    ws.emplace_back([&, w] {
      for (;;) {
        size_t i = next.fetch_add(1);
        if (i >= tasks.size()) break;
        partial[w] += run(tasks[i]);
      }
    });
  for (auto& w : ws) w.join();
  u128 total = 0;
  for (u128 p : partial) total += p;
  return total;
}

// brute_force_count, src/lib.rs:6161-6185 (test-only independent oracle).
static u128 brute_force_count(unsigned n) {
  if (n == 0) return 1;
  std::vector<unsigned> queens;
  u128 count = 0;
  std::function<void(unsigned)> place = [&](unsigned row) {
    if (row == n) {
      ++count;
      return;
    }
    for (unsigned column = 0; column < n; ++column) {
      bool legal = true;
      for (unsigned pr = 0; pr < queens.size(); ++pr) {
        unsigned other = queens[pr];
        unsigned dc = column > other ? column - other : other - column;
        if (other == column || row - pr == dc) {
          legal = false;
          break;
        }
      }
      if (legal) {
        queens.push_back(column);
        place(row + 1);
        queens.pop_back();
      }
    }
  };
  place(0);
  return count;
}

// ---------------------------------------------------------------------------
// Wide CRT (src/lib.rs:3767, 3834-3886, 4122-4163).

static const u64 CRT_PRIME_CANDIDATES[4] = {4294967291ULL, 4294967279ULL, 4294967231ULL, 4294967197ULL};

static bool is_prime_u32_range(u64 v) {
  if (v < 2) return false;
  if (v % 2 == 0) return v == 2;
  for (u64 d = 3; d * d <= v; d += 2)
    if (v % d == 0) return false;
  return true;
}

static u128 factorial_u128(unsigned n) {
  u128 p = 1;
  for (unsigned f = 2; f <= n; ++f)
    if (!checked_mul(p, f, &p)) throw Error{"N! exactness bound does not fit u128"};
  return p;
}

// wide_crt_plan, src/lib.rs:3859-3886: the shortest prefix of the candidate
// primes whose product exceeds N!.
static std::vector<u64> wide_crt_plan(unsigned n, u128* factorial_bound, u128* product) {
  if (n > 34) throw Error{"wide CRT backend supports N <= 34 because 35! exceeds u128"};
  *factorial_bound = factorial_u128(n);
  std::vector<u64> primes;
  u128 prod = 1;
  for (u64 p : CRT_PRIME_CANDIDATES) {
    if (!is_prime_u32_range(p)) throw Error{"CRT modulus failed deterministic primality check"};
    primes.push_back(p);
    if (!checked_mul(prod, p, &prod)) throw Error{"CRT modulus product overflow"};
    if (prod > *factorial_bound) {
      *product = prod;
      return primes;
    }
  }
  throw Error{"available certified CRT product does not exceed N! bound"};
}

static u64 mod_pow(u64 base, u64 exponent, u64 modulus) {
  u64 result = 1;
  while (exponent) {
    if (exponent & 1) result = (u64)(((u128)result * base) % modulus);
    base = (u64)(((u128)base * base) % modulus);
    exponent >>= 1;
  }
  return result;
}

// reconstruct_crt, src/lib.rs:4134-4163: incremental Garner with Fermat
// inverses and checked u128 accumulation.
static u128 reconstruct_crt(const u64* residues, const u64* primes, size_t len) {
  if (len == 0) throw Error{"CRT residue/modulus length mismatch"};
  u128 value = 0, mp = 1;
  for (size_t i = 0; i < len; ++i) {
    u64 prime = primes[i], residue = residues[i];
    u64 value_mod = (u64)(value % prime);
    u64 delta = residue >= value_mod ? residue - value_mod : residue + prime - value_mod;
    u64 product_mod = (u64)(mp % prime);
    u64 inverse = mod_pow(product_mod, prime - 2, prime);
    u64 step = (u64)(((u128)delta * inverse) % prime);
    u128 term;
    if (!checked_mul(mp, step, &term)) throw Error{"CRT reconstruction product overflow"};
    if (!checked_add(value, term, &value)) throw Error{"CRT reconstruction sum overflow"};
    if (!checked_mul(mp, prime, &mp)) throw Error{"CRT reconstruction modulus overflow"};
  }
  return value;
}

// Boundary after a placed prefix: each row's queen column is applied with the
// compiled successor (recursive_tail_successor, src/lib.rs:3139-3151). A
// column that is attacked gives an empty boundary (zero completions).
static bool prefix_boundary(unsigned n, const uint32_t* cols, unsigned k, BoundaryState* out) {
  u64 board_mask = ((u64)1 << n) - 1;
  BoundaryState s{0, 0, 0};
  for (unsigned r = 0; r < k; ++r) {
    unsigned c = cols[r];
    if (c >= n) throw Error{"prefix column out of range"};
    u64 b = (u64)1 << c;
    if ((s.columns | s.diag_dr | s.diag_dl) & b) return false;
    s = BoundaryState{s.columns | b, ((s.diag_dr | b) << 1) & board_mask, (s.diag_dl | b) >> 1};
  }
  *out = s;
  return true;
}

}  // namespace oracle

// ---------------------------------------------------------------------------
// C interface used by the Python tests (ctypes).

using namespace oracle;

extern "C" {

typedef struct {
  uint64_t lo, hi;
} oq_u128;

typedef struct {
  uint32_t row;
  uint64_t input_states;
  oq_u128 tensor_entries_examined, tensor_entries_matched, row_operator_candidates, row_operator_matched,
      completed_row_terms;
  uint64_t output_states;
  oq_u128 output_weight;
  double elapsed_s;
  uint64_t peak_rss_bytes;
} oq_layer;

typedef struct {
  uint32_t n;
  oq_u128 count;
  double elapsed_s;
  uint64_t peak_states;
  oq_u128 tensor_entries_examined, tensor_entries_matched, row_operator_candidates, row_operator_matched;
  uint64_t peak_rss_bytes;
  uint32_t n_layers;
} oq_result;

static oq_u128 to_oq(u128 v) { return oq_u128{(uint64_t)v, (uint64_t)(v >> 64)}; }
static u128 from_oq(oq_u128 v) { return ((u128)v.hi << 64) | v.lo; }

static void set_err(char* err, size_t len, const std::string& msg) {
  if (err && len) {
    std::snprintf(err, len, "%s", msg.c_str());
  }
}

static void export_result(const ContractionResult& r, oq_result* out, oq_layer* layers, uint32_t layers_cap) {
  out->n = r.n;
  out->count = to_oq(r.count);
  out->elapsed_s = r.elapsed_s;
  out->peak_states = r.peak_states;
  out->tensor_entries_examined = to_oq(r.tensor_entries_examined);
  out->tensor_entries_matched = to_oq(r.tensor_entries_matched);
  out->row_operator_candidates = to_oq(r.row_operator_candidates);
  out->row_operator_matched = to_oq(r.row_operator_matched);
  out->peak_rss_bytes = r.peak_rss_bytes;
  out->n_layers = (uint32_t)r.layers.size();
  if (layers)
    for (size_t i = 0; i < r.layers.size() && i < layers_cap; ++i) {
      const LayerMetric& l = r.layers[i];
      layers[i] = oq_layer{l.row,
                           l.input_states,
                           to_oq(l.tensor_entries_examined),
                           to_oq(l.tensor_entries_matched),
                           to_oq(l.row_operator_candidates),
                           to_oq(l.row_operator_matched),
                           to_oq(l.completed_row_terms),
                           l.output_states,
                           to_oq(l.output_weight),
                           l.elapsed_s,
                           l.peak_rss_bytes};
    }
}

// backend: 0 serial sort-reduce, 1 threaded sort-reduce, 2 HashMap compiled,
// 3 HashMap sitewise. symmetry: 0 none, 1 first-row vertical orbits.
// position: 0 dense, 1 sparse. rows: number of rows to contract (0 = all).
// prefix_cols/prefix_len: optional placed prefix (serving requests).
// boundary_keys/boundary_weights: optional output of the boundary after the
// contracted rows, sorted by packed key (lo/hi u64 pairs), capacity in entries.
int oracle_contract(uint32_t n, int backend, int symmetry, int position, uint32_t threads, uint32_t rows,
                    const uint32_t* prefix_cols, uint32_t prefix_len, oq_result* out, oq_layer* layers,
                    uint32_t layers_cap, oq_u128* boundary_keys, oq_u128* boundary_weights, uint64_t boundary_cap,
                    uint64_t* boundary_len, char* err, size_t err_len) {
  try {
    DriverOptions opt;
    opt.rows = (rows == 0 || rows > n) ? n : rows;
    std::vector<KV> fb;
    if (boundary_len) opt.final_boundary = &fb;
    if (prefix_len > 0) {
      if (prefix_len > n) throw Error{"prefix longer than the board"};
      BoundaryState s;
      if (n > 42) throw Error{"the packed u128 virtual-boundary backend supports N <= 42"};
      if (!prefix_boundary(n, prefix_cols, prefix_len, &s)) {
        ContractionResult r{};
        r.n = n;
        r.count = 0;
        export_result(r, out, layers, layers_cap);
        if (boundary_len) *boundary_len = 0;
        return 0;
      }
      opt.initial = std::vector<KV>{KV{pack(s, n), 1}};
      opt.row0 = prefix_len;
    }
    Symmetry sym = symmetry ? Symmetry::TopRowVerticalOrbits : Symmetry::None;
    Position pos = position ? Position::Sparse : Position::Dense;
    ContractionResult r;
    switch (backend) {
      case 0:
        r = contract_rows_sort_reduce_with_modes(n, sym, pos, opt);
        break;
      case 1:
        r = contract_rows_parallel_sort_reduce_with_modes(n, threads, sym, pos, opt);
        break;
      case 2:
        r = contract_rows_with_backend(n, false, opt);
        break;
      case 3:
        r = contract_rows_with_backend(n, true, opt);
        break;
      default:
        throw Error{"unknown oracle backend"};
    }
    export_result(r, out, layers, layers_cap);
    if (boundary_len) {
      *boundary_len = fb.size();
      if (boundary_keys && boundary_weights)
        for (size_t i = 0; i < fb.size() && i < boundary_cap; ++i) {
          boundary_keys[i] = to_oq(fb[i].first);
          boundary_weights[i] = to_oq(fb[i].second);
        }
    }
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  } catch (const std::bad_alloc&) {
    set_err(err, err_len, "out of host memory");
    return 2;
  }
}

// Contract rows [row0, n) from an arbitrary boundary (packed keys + weights),
// with the serial sort-reduce driver and no orbit weighting. Used to check
// slice and batch decompositions: the count of a boundary is linear in it.
int oracle_contract_from(uint32_t n, uint32_t row0, const oq_u128* keys, const oq_u128* weights, uint64_t len,
                         oq_result* out, oq_layer* layers, uint32_t layers_cap, char* err, size_t err_len) {
  try {
    if (n > 42) throw Error{"the packed u128 virtual-boundary backend supports N <= 42"};
    DriverOptions opt;
    opt.rows = n;
    opt.row0 = row0;
    for (uint64_t i = 0; i < len; ++i) opt.initial.push_back(KV{from_oq(keys[i]), from_oq(weights[i])});
    if (opt.initial.empty()) {
      ContractionResult r{};
      r.n = n;
      export_result(r, out, layers, layers_cap);
      return 0;
    }
    std::sort(opt.initial.begin(), opt.initial.end(), [](const KV& a, const KV& b) { return a.first < b.first; });
    reduce_sorted(opt.initial, row0);
    ContractionResult r = contract_rows_sort_reduce_with_modes(n, Symmetry::None, Position::Dense, opt);
    export_result(r, out, layers, layers_cap);
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  }
}

int oracle_known_count(uint32_t n, oq_u128* out) {
  u128 v;
  if (!known_count(n, &v)) return 1;
  *out = to_oq(v);
  return 0;
}

int oracle_dfs_count(uint32_t n, uint32_t threads, oq_u128* out, char* err, size_t err_len) {
  try {
    *out = to_oq(count_dfs_bitmask(n, threads));
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  }
}

int oracle_brute_force_count(uint32_t n, oq_u128* out) {
  *out = to_oq(brute_force_count(n));
  return 0;
}

int oracle_crt_plan(uint32_t n, uint64_t* primes_out, uint32_t* len_out, oq_u128* factorial_out,
                    oq_u128* product_out, char* err, size_t err_len) {
  try {
    u128 f = 0, p = 0;
    std::vector<u64> primes = wide_crt_plan(n, &f, &p);
    for (size_t i = 0; i < primes.size(); ++i) primes_out[i] = primes[i];
    *len_out = (uint32_t)primes.size();
    *factorial_out = to_oq(f);
    *product_out = to_oq(p);
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  }
}

int oracle_reconstruct_crt(const uint64_t* residues, const uint64_t* primes, uint32_t len, oq_u128* out, char* err,
                           size_t err_len) {
  try {
    *out = to_oq(reconstruct_crt(residues, primes, len));
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  }
}

// The 17 C entries in legs_key order: legs packed as legs_key, value as u128.
int oracle_c_entries(uint32_t* legs_out, oq_u128* values_out, uint32_t cap) {
  SiteTensorC c = SiteTensorC::sec_vi();
  for (size_t i = 0; i < c.entries.size() && i < cap; ++i) {
    legs_out[i] = legs_key(c.entries[i].legs);
    values_out[i] = to_oq(c.entries[i].value);
  }
  return (int)c.entries.size();
}

// The 17 B entries: alpha in bit 8, legs_key in bits 0..7.
int oracle_b_entries(uint32_t* out, oq_u128* values_out, uint32_t cap) {
  std::vector<BEntry> b = site_tensor_b_sec_vi();
  for (size_t i = 0; i < b.size() && i < cap; ++i) {
    out[i] = legs_key(b[i].legs) | ((uint32_t)b[i].alpha << 8);
    values_out[i] = to_oq(b[i].value);
  }
  return (int)b.size();
}

// Number of C entries matching one input signature (matching_entries).
int oracle_c_matching(uint32_t column_in, uint32_t row_in, uint32_t dr_in, uint32_t dl_in) {
  static SiteTensorC c = SiteTensorC::sec_vi();
  return (int)c.matching((u8)column_in, (u8)row_in, (u8)dr_in, (u8)dl_in).size();
}

// Run CompiledRowOperator::compile on an arbitrary C given as legs_key + value
// pairs; returns 0 when the table certifies, 1 with the reference's message
// otherwise.
int oracle_compile_check(const uint32_t* legs, const uint64_t* values, uint32_t len, char* err, size_t err_len) {
  try {
    SiteTensorC c;
    for (uint32_t i = 0; i < len; ++i) {
      uint32_t k = legs[i];
      VirtualLegs l{(u8)(k & 1), (u8)((k >> 1) & 1), (u8)((k >> 2) & 1), (u8)((k >> 3) & 1),
                    (u8)((k >> 4) & 1), (u8)((k >> 5) & 1), (u8)((k >> 6) & 1), (u8)((k >> 7) & 1)};
      c.entries.push_back(CEntry{l, values[i]});
    }
    CompiledRowOperator::compile(c);
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  }
}

// Packed-key helpers for tests (PackedBoundary::pack/unpack).
void oracle_pack(uint32_t n, uint64_t columns, uint64_t dr, uint64_t dl, oq_u128* out) {
  *out = to_oq(pack(BoundaryState{columns, dr, dl}, n));
}
void oracle_unpack(uint32_t n, oq_u128 key, uint64_t* columns, uint64_t* dr, uint64_t* dl) {
  BoundaryState s = unpack(from_oq(key), n);
  *columns = s.columns;
  *dr = s.diag_dr;
  *dl = s.diag_dl;
}

// Successors of one packed parent under the compiled (mode 0) or sitewise
// (mode 1) row kernel, normalised by key (for operator-equivalence tests).
int oracle_row_terms(uint32_t n, int mode, oq_u128 parent, oq_u128* keys_out, oq_u128* weights_out, uint32_t cap) {
  SiteTensorC tensor = SiteTensorC::sec_vi();
  CompiledRowOperator op = CompiledRowOperator::compile(tensor);
  RowCounters counters;
  std::vector<Term> terms;
  if (mode == 0)
    contract_one_row_compiled(n, op, unpack(from_oq(parent), n), 1, counters, terms);
  else
    contract_one_row_sitewise(n, tensor, unpack(from_oq(parent), n), 1, counters, terms);
  std::vector<KV> kv;
  for (const Term& t : terms) kv.push_back(KV{pack(t.first, n), t.second});
  std::sort(kv.begin(), kv.end(), [](const KV& a, const KV& b) { return a.first < b.first; });
  reduce_sorted(kv, 0);
  for (size_t i = 0; i < kv.size() && i < cap; ++i) {
    keys_out[i] = to_oq(kv[i].first);
    weights_out[i] = to_oq(kv[i].second);
  }
  return (int)kv.size();
}

int oracle_orbit_weight(uint32_t n, uint32_t column) {
  return (int)top_row_vertical_orbit_weight(n, BoundaryState{(u64)1 << column, 0, 0});
}

typedef struct {
  uint32_t n, order, complete, pad;
  oq_u128 count;
  double elapsed_s;
  uint64_t peak_states, peak_open_bonds;
  oq_u128 tensor_entries_examined, tensor_entries_accepted;
  uint64_t contracted_sites;
} oq_explicit;

int oracle_explicit_frontier(uint32_t n, uint32_t order, uint64_t support_limit, oq_explicit* out, char* err,
                             size_t err_len) {
  try {
    if (order > 1) throw Error{"order must be 0 (row-major) or 1 (top-left diamond)"};
    const ExplicitFrontierResult r = contract_explicit_c_frontier(n, order, support_limit);
    out->n = r.n;
    out->order = r.order;
    out->complete = r.complete;
    out->pad = 0;
    out->count = to_oq(r.count);
    out->elapsed_s = r.elapsed;
    out->peak_states = r.peak_states;
    out->peak_open_bonds = r.peak_open_bonds;
    out->tensor_entries_examined = to_oq(r.examined);
    out->tensor_entries_accepted = to_oq(r.accepted);
    out->contracted_sites = r.contracted_sites;
    return 0;
  } catch (const Error& e) {
    set_err(err, err_len, e.msg);
    return 1;
  }
}

}  // extern "C"

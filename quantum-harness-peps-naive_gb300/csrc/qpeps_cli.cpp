// qpeps — command-line drop-in for the reference's binary (src/main.rs).
//
//   qpeps solve N [--layers]
//   qpeps bench MAX_N [--min N] [--repeats R] [--csv]
//
// Same commands, flags, output lines, CSV headers and exit codes as
// src/main.rs:25-174, with the count computed by libqpeps.so on the GPU.
// `peak_rss_bytes` reports the device memory high-water mark of the context.
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "qpeps.h"

namespace {

struct CliError {
  std::string msg;
};

std::string u128s(qpeps_u128 v) {
  unsigned __int128 x = ((unsigned __int128)v.hi << 64) | v.lo;
  if (x == 0) return "0";
  std::string s;
  while (x) {
    s.insert(s.begin(), (char)('0' + (int)(x % 10)));
    x /= 10;
  }
  return s;
}

bool u128_eq(qpeps_u128 a, qpeps_u128 b) { return a.lo == b.lo && a.hi == b.hi; }

size_t parse_usize(const char* value, const std::string& label) {
  if (!value) throw CliError{"missing " + label};
  char* end = nullptr;
  errno = 0;
  const unsigned long long v = std::strtoull(value, &end, 10);
  if (!*value || *end || errno || value[0] == '-') throw CliError{"invalid " + label};
  return (size_t)v;
}

void usage() {
  std::fprintf(stderr,
               "Usage:\n  qpeps solve N [--layers]\n  qpeps bench MAX_N [--min N] [--repeats R] [--csv]\n");
}

void* make_ctx() {
  void* ctx = nullptr;
  char err[512];
  if (qpeps_ctx_create(0, &ctx, err, sizeof err) != QPEPS_OK) throw CliError{err};
  return ctx;
}

void contract(void* ctx, uint32_t n, qpeps_result* r, std::vector<qpeps_layer>* layers) {
  qpeps_options o;
  qpeps_options_default(&o);
  char err[512];
  layers->assign(std::max<uint32_t>(n, 1), qpeps_layer{});
  if (qpeps_contract_rows(ctx, n, &o, r, layers->data(), (uint32_t)layers->size(), err, sizeof err) != QPEPS_OK)
    throw CliError{err};
}

// solve, src/main.rs:25-70.
void solve(int argc, char** argv) {
  const size_t n = parse_usize(argc > 2 ? argv[2] : nullptr, "N");
  bool want_layers = false;
  for (int i = 3; i < argc; ++i)
    if (std::strcmp(argv[i], "--layers") == 0) want_layers = true;
  void* ctx = make_ctx();
  qpeps_result r;
  std::vector<qpeps_layer> layers;
  try {
    contract(ctx, (uint32_t)n, &r, &layers);
  } catch (...) {
    qpeps_ctx_destroy(ctx);
    throw;
  }
  qpeps_ctx_destroy(ctx);
  qpeps_u128 expected;
  const bool have = qpeps_known_count((uint32_t)n, &expected) == QPEPS_OK;
  const bool verified = have && u128_eq(expected, r.count);
  std::printf(
      "N=%zu Q(N)=%s elapsed_s=%.6f peak_rss_bytes=%llu peak_states=%llu tensor_entries_examined=%s "
      "tensor_entries_matched=%s row_operator_candidates=%s row_operator_matched=%s verified=%s\n",
      n, u128s(r.count).c_str(), r.elapsed_s, (unsigned long long)r.peak_rss_bytes,
      (unsigned long long)r.peak_states, u128s(r.tensor_entries_examined).c_str(),
      u128s(r.tensor_entries_matched).c_str(), u128s(r.row_operator_candidates).c_str(),
      u128s(r.row_operator_matched).c_str(), verified ? "true" : "false");
  if (want_layers) {
    std::printf(
        "row,input_states,tensor_entries_examined,tensor_entries_matched,row_operator_candidates,"
        "row_operator_matched,completed_row_terms,output_states,output_weight,elapsed_s,peak_rss_bytes\n");
    for (uint32_t i = 0; i < r.n_layers && i < layers.size(); ++i) {
      const qpeps_layer& l = layers[i];
      std::printf("%u,%llu,%s,%s,%s,%s,%s,%llu,%s,%.6f,%llu\n", l.row + 1, (unsigned long long)l.input_states,
                  u128s(l.tensor_entries_examined).c_str(), u128s(l.tensor_entries_matched).c_str(),
                  u128s(l.row_operator_candidates).c_str(), u128s(l.row_operator_matched).c_str(),
                  u128s(l.completed_row_terms).c_str(), (unsigned long long)l.output_states,
                  u128s(l.output_weight).c_str(), l.elapsed_s, (unsigned long long)l.peak_rss_bytes);
    }
  }
  std::fflush(stdout);
  if (have && !verified) throw CliError{"known-count verification failed for N=" + std::to_string(n)};
}

// bench, src/main.rs:72-152.
void bench(int argc, char** argv) {
  const size_t max_n = parse_usize(argc > 2 ? argv[2] : nullptr, "MAX_N");
  size_t min_n = 1, repeats = 3;
  bool csv = false;
  for (int i = 3; i < argc;) {
    const std::string a = argv[i];
    if (a == "--min") {
      min_n = parse_usize(i + 1 < argc ? argv[i + 1] : nullptr, "--min value");
      i += 2;
    } else if (a == "--repeats") {
      repeats = parse_usize(i + 1 < argc ? argv[i + 1] : nullptr, "--repeats value");
      i += 2;
    } else if (a == "--csv") {
      csv = true;
      i += 1;
    } else {
      throw CliError{"unknown option: " + a};
    }
  }
  if (repeats == 0) throw CliError{"--repeats must be positive"};
  if (min_n > max_n) throw CliError{"--min must not exceed MAX_N"};
  if (csv)
    std::printf(
        "N,count,known_count,verified,median_elapsed_s,min_elapsed_s,peak_rss_bytes,peak_states,"
        "tensor_entries_examined,tensor_entries_matched,row_operator_candidates,row_operator_matched,repeats\n");
  void* ctx = make_ctx();
  try {
    for (size_t n = min_n; n <= max_n; ++n) {
      std::vector<double> elapsed;
      qpeps_result r{};
      std::vector<qpeps_layer> layers;
      for (size_t i = 0; i < repeats; ++i) {
        contract(ctx, (uint32_t)n, &r, &layers);
        elapsed.push_back(r.elapsed_s);
      }
      const double minimum = *std::min_element(elapsed.begin(), elapsed.end());
      std::sort(elapsed.begin(), elapsed.end());
      const double med = elapsed[elapsed.size() / 2];
      qpeps_u128 known;
      const bool have = qpeps_known_count((uint32_t)n, &known) == QPEPS_OK;
      const bool verified = have && u128_eq(known, r.count);
      if (have && !verified) throw CliError{"known-count verification failed for N=" + std::to_string(n)};
      if (csv)
        std::printf("%zu,%s,%s,%s,%.9f,%.9f,%llu,%llu,%s,%s,%s,%s,%zu\n", n, u128s(r.count).c_str(),
                    have ? u128s(known).c_str() : "", verified ? "true" : "false", med, minimum,
                    (unsigned long long)r.peak_rss_bytes, (unsigned long long)r.peak_states,
                    u128s(r.tensor_entries_examined).c_str(), u128s(r.tensor_entries_matched).c_str(),
                    u128s(r.row_operator_candidates).c_str(), u128s(r.row_operator_matched).c_str(), repeats);
      else
        std::printf("N=%2zu Q(N)=%-10s median=%.6fs peak_rss=%.1fMiB peak_states=%-8llu verified=%s\n", n,
                    u128s(r.count).c_str(), med, (double)r.peak_rss_bytes / (1024.0 * 1024.0),
                    (unsigned long long)r.peak_states, verified ? "true" : "false");
      std::fflush(stdout);
    }
  } catch (...) {
    qpeps_ctx_destroy(ctx);
    throw;
  }
  qpeps_ctx_destroy(ctx);
}

}  // namespace

// run/main, src/main.rs:154-174: errors print "error: ..." and exit 1.
int main(int argc, char** argv) {
  try {
    if (argc > 1 && std::strcmp(argv[1], "solve") == 0) {
      solve(argc, argv);
    } else if (argc > 1 && std::strcmp(argv[1], "bench") == 0) {
      bench(argc, argv);
    } else {
      usage();
      throw CliError{"missing or invalid command"};
    }
  } catch (const CliError& e) {
    std::fprintf(stderr, "error: %s\n", e.msg.c_str());
    return 1;
  }
  return 0;
}

// Command-line front end of the CPU oracle (test infrastructure only).
//
//   oracle_cli solve N [backend] [threads]     per-row layer CSV + count
//   oracle_cli dfs N [threads]                 DFS bitboard count
//   oracle_cli prefix N c0 c1 ...              completions of a placed prefix
//
// backend: 0 serial sort-reduce (contract_rows), 1 threaded sort-reduce,
// 2 HashMap compiled, 3 HashMap sitewise.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

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
int oracle_contract(uint32_t n, int backend, int symmetry, int position, uint32_t threads, uint32_t rows,
                    const uint32_t* prefix_cols, uint32_t prefix_len, oq_result* out, oq_layer* layers,
                    uint32_t layers_cap, oq_u128* boundary_keys, oq_u128* boundary_weights, uint64_t boundary_cap,
                    uint64_t* boundary_len, char* err, size_t err_len);
int oracle_dfs_count(uint32_t n, uint32_t threads, oq_u128* out, char* err, size_t err_len);
}

static std::string u128s(oq_u128 v) {
  unsigned __int128 x = ((unsigned __int128)v.hi << 64) | v.lo;
  if (x == 0) return "0";
  std::string s;
  while (x) {
    s.insert(s.begin(), (char)('0' + (int)(x % 10)));
    x /= 10;
  }
  return s;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: oracle_cli solve N [backend] [threads] | dfs N [threads] | prefix N c...\n");
    return 2;
  }
  std::string cmd = argv[1];
  uint32_t n = (uint32_t)std::atoi(argv[2]);
  char err[256] = {0};
  if (cmd == "dfs") {
    uint32_t threads = argc > 3 ? (uint32_t)std::atoi(argv[3]) : 1;
    oq_u128 c;
    if (oracle_dfs_count(n, threads, &c, err, sizeof err)) {
      std::fprintf(stderr, "error: %s\n", err);
      return 1;
    }
    std::printf("N=%u Q(N)=%s\n", n, u128s(c).c_str());
    return 0;
  }
  int backend = 0;
  uint32_t threads = 1;
  std::vector<uint32_t> prefix;
  int symmetry = 1;
  if (cmd == "solve") {
    backend = argc > 3 ? std::atoi(argv[3]) : 0;
    threads = argc > 4 ? (uint32_t)std::atoi(argv[4]) : 1;
    if (backend >= 2) symmetry = 0;
  } else if (cmd == "prefix") {
    for (int i = 3; i < argc; ++i) prefix.push_back((uint32_t)std::atoi(argv[i]));
    symmetry = 0;
  }
  std::vector<oq_layer> layers(64);
  oq_result r;
  if (oracle_contract(n, backend, symmetry, 0, threads, 0, prefix.data(), (uint32_t)prefix.size(), &r, layers.data(),
                      64, nullptr, nullptr, 0, nullptr, err, sizeof err)) {
    std::fprintf(stderr, "error: %s\n", err);
    return 1;
  }
  std::printf("N=%u Q(N)=%s elapsed_s=%.6f peak_states=%llu row_operator_candidates=%s row_operator_matched=%s\n", n,
              u128s(r.count).c_str(), r.elapsed_s, (unsigned long long)r.peak_states,
              u128s(r.row_operator_candidates).c_str(), u128s(r.row_operator_matched).c_str());
  std::printf("row,input_states,completed_row_terms,output_states,output_weight,elapsed_s\n");
  for (uint32_t i = 0; i < r.n_layers; ++i)
    std::printf("%u,%llu,%s,%llu,%s,%.6f\n", layers[i].row + 1, (unsigned long long)layers[i].input_states,
                u128s(layers[i].completed_row_terms).c_str(), (unsigned long long)layers[i].output_states,
                u128s(layers[i].output_weight).c_str(), layers[i].elapsed_s);
  return 0;
}

// Row-step kernels of the global-table merge path.
//
// One row step of the reference's sort-reduce driver
// (src/lib.rs:5325-5391: expand every parent with the compiled row operator,
// then merge equal packed keys by checked addition) is done here as
//   row_count        -> successor count T (sizes the table),
//   expand_insert    -> every (parent, free column) successor is added into an
//                       open-addressing table keyed by the packed boundary,
//   compact          -> occupied slots become the next boundary buffer.
// The site kernels do the same for the explicit C applied at one site
// (src/lib.rs:513-592), one launch per site.
#include <cuda_runtime.h>

#include <type_traits>

#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {

__constant__ CTableDev c_table;
__constant__ FrontierStepDev c_frontier;

static_assert(sizeof(Slot<u64, 1>) == 16 && sizeof(Slot<u64, 2>) == 32 && sizeof(Slot<u64, 3>) == 32 &&
                  sizeof(Slot<u64, 4>) == 64,
              "u64 slot sizes must match slot_bytes()");
static_assert(sizeof(Slot<u128, 1>) == 32 && sizeof(Slot<u128, 2>) == 32 && sizeof(Slot<u128, 3>) == 64 &&
                  sizeof(Slot<u128, 4>) == 64,
              "u128 slot sizes must match slot_bytes()");

namespace {

constexpr u32 kFull = 0xffffffffu;
constexpr u32 kMaxProbe = 1u << 16;

__device__ __forceinline__ u64 board_mask(unsigned n) { return n >= 64 ? ~0ull : ((1ull << n) - 1); }

template <typename K>
__device__ __forceinline__ K load_key(const void* keys, u64 i) {
  return reinterpret_cast<const K*>(keys)[i];
}

__device__ __forceinline__ int warp_inclusive_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int t = __shfl_up_sync(kFull, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

// Position of the k-th (0-based) set bit of a 64-bit mask (k < popcount).
__device__ __forceinline__ unsigned nth_set_bit(u64 m, int k) {
  u32 lo = (u32)m, hi = (u32)(m >> 32);
  int plo = __popc(lo);
  return k < plo ? __fns(lo, 0, k + 1) : 32u + __fns(hi, 0, k - plo + 1);
}

template <int BLOCK>
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v) {
  __shared__ unsigned long long s_part[BLOCK / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_part[wid] = v;
  __syncthreads();
  unsigned long long t = 0;
  if (wid == 0) {
    t = lane < BLOCK / 32 ? s_part[lane] : 0ull;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(kFull, t, d);
  }
  return t;  // valid in thread 0
}

// ---------------------------------------------------------------------------
// Successor count of a row step: sum of popcount(~(cols|dr|dl) & mask).

template <typename K, int BLOCK>
__global__ void __launch_bounds__(BLOCK) row_count_kernel(const void* __restrict__ keys, u64 n_in, unsigned n,
                                                          StepScalars* __restrict__ sc) {
  const u64 mask = board_mask(n);
  unsigned long long acc = 0, sw = 0;
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in; i += (u64)gridDim.x * BLOCK) {
    State s = unpack<K>(load_key<K>(keys, i), n, mask);
    const u64 fr = ~(s.cols | s.dr | s.dl) & mask;
    acc += __popcll(fr);
    sw += sitewise_entries(fr, n);
  }
  unsigned long long t = block_sum_u64<BLOCK>(acc);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->terms, t);
  t = block_sum_u64<BLOCK>(sw);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->sitewise_examined, t);
}

// ---------------------------------------------------------------------------
// Fused compiled-row expansion and table insertion.
//
// A warp loads 32 parents (coalesced), then flattens the ragged list of
// (parent, free column) pairs so that every lane inserts one successor per
// round: lane j finds its parent by a 5-step shuffle search over the warp's
// inclusive successor counts and its column as the k-th set bit of that
// parent's free mask.

template <typename K, int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) row_expand_insert_kernel(const void* __restrict__ keys,
                                                                  const u32* __restrict__ res, u64 res_stride,
                                                                  u64 n_in, unsigned n, Slot<K, R>* __restrict__ table,
                                                                  u64 table_mask, StepScalars* __restrict__ sc) {
  constexpr int WARPS = BLOCK / 32;
  __shared__ K s_key[WARPS][32];
  __shared__ u64 s_free[WARPS][32];
  __shared__ u32 s_w[WARPS][R][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const u64 mask = board_mask(n);
  const u64 gwarp = (u64)blockIdx.x * WARPS + wid;
  const u64 nwarps = (u64)gridDim.x * WARPS;
  for (u64 base = gwarp * 32; base < n_in; base += nwarps * 32) {
    const u64 i = base + lane;
    K key = 0;
    u64 fr = 0;
    if (i < n_in) {
      key = load_key<K>(keys, i);
      State s = unpack<K>(key, n, mask);
      fr = ~(s.cols | s.dr | s.dl) & mask;
#pragma unroll
      for (int r = 0; r < R; ++r) s_w[wid][r][lane] = res[r * res_stride + i];
    }
    s_key[wid][lane] = key;
    s_free[wid][lane] = fr;
    const int cnt = __popcll(fr);
    const int incl = warp_inclusive_scan(cnt);
    const int excl = incl - cnt;
    const int total = __shfl_sync(kFull, incl, 31);
    __syncwarp();
    for (int j0 = 0; j0 < total; j0 += 32) {
      const int j = j0 + lane;
      int owner = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        int v = __shfl_sync(kFull, incl, owner + step - 1);
        if (v <= j) owner += step;
      }
      const int owner_excl = __shfl_sync(kFull, excl, owner);
      if (j < total) {
        const K pk = s_key[wid][owner];
        const unsigned col = nth_set_bit(s_free[wid][owner], j - owner_excl);
        State s = unpack<K>(pk, n, mask);
        const K child = row_successor<K>(s, 1ull << col, n, mask);
        u32 w[R];
#pragma unroll
        for (int r = 0; r < R; ++r) w[r] = s_w[wid][r][owner];
        table_insert<K, R>(table, table_mask, child, w, kMaxProbe, &sc->error);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Explicit-C site update (one launch per site).
//
// Mid-row key: the packed boundary with bit 3n holding the row signal. At
// site c the column, diag_dr and diag_dl bits at position c hold incoming
// signals before the update and outgoing signals (not yet shifted) after it,
// exactly as the compiled operator's replace_bit does (src/lib.rs:621-623).
// The last site closes the row: row signal must be 1 (v1), diagonals move to
// their next-row positions, and the row signal resets to 0 (v0).

template <typename K>
__device__ __forceinline__ u32 site_signature(K key, unsigned n, unsigned site, u32* rs_out) {
  const u32 col = (u32)(key >> site) & 1u;
  const u32 dr = (u32)(key >> (n + site)) & 1u;
  const u32 dl = (u32)(key >> (2 * n + site)) & 1u;
  const u32 rs = (u32)(key >> (3 * n)) & 1u;
  *rs_out = rs;
  return col | (rs << 1) | (dr << 2) | (dl << 3);
}

template <typename K>
__device__ __forceinline__ bool site_apply(K key, unsigned n, unsigned site, u32 out_bits, u64 mask, K* child) {
  const K one = 1;
  const K clear = ~((one << site) | (one << (n + site)) | (one << (2 * n + site)) | (one << (3 * n)));
  K k = key & clear;
  k |= (K)(out_bits & 1u) << site;
  k |= (K)((out_bits >> 2) & 1u) << (n + site);
  k |= (K)((out_bits >> 3) & 1u) << (2 * n + site);
  const u32 row_out = (out_bits >> 1) & 1u;
  if (site + 1 == n) {
    if (row_out != 1u) return false;  // right boundary v1 = (0,1)
    State s = unpack<K>(k, n, mask);
    *child = pack<K>(s.cols, (s.dr << 1) & mask, s.dl >> 1, n);
  } else {
    *child = k | ((K)row_out << (3 * n));
  }
  return true;
}

template <typename K, int BLOCK>
__global__ void __launch_bounds__(BLOCK) site_count_kernel(const void* __restrict__ keys, u64 n_in, unsigned n,
                                                           unsigned site, StepScalars* __restrict__ sc) {
  unsigned long long acc = 0;
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in; i += (u64)gridDim.x * BLOCK) {
    u32 rs;
    const u32 sig = site_signature<K>(load_key<K>(keys, i), n, site, &rs);
    acc += c_table.count[sig];
  }
  unsigned long long t = block_sum_u64<BLOCK>(acc);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->terms, t);
}

template <typename K, int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) site_expand_insert_kernel(const void* __restrict__ keys,
                                                                   const u32* __restrict__ res, u64 res_stride,
                                                                   u64 n_in, unsigned n, unsigned site,
                                                                   Slot<K, R>* __restrict__ table, u64 table_mask,
                                                                   StepScalars* __restrict__ sc) {
  const u64 mask = board_mask(n);
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in; i += (u64)gridDim.x * BLOCK) {
    const K key = load_key<K>(keys, i);
    u32 w[R];
#pragma unroll
    for (int r = 0; r < R; ++r) w[r] = res[r * res_stride + i];
    u32 rs;
    const u32 sig = site_signature<K>(key, n, site, &rs);
    const u32 cnt = c_table.count[sig];
    for (u32 e = 0; e < cnt; ++e) {
      K child;
      if (!site_apply<K>(key, n, site, c_table.out[sig][e], mask, &child)) continue;
      u32 cw[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const u32 v = c_table.value_mod[sig][e][r];
        cw[r] = v == 1u ? w[r] : mul_mod(w[r], v, prime_at(r));
      }
      table_insert<K, R>(table, table_mask, child, cw, kMaxProbe, &sc->error);
    }
  }
}

// ---------------------------------------------------------------------------
// Compaction: occupied table slots -> boundary buffer (SoA), residues reduced
// modulo their primes, plus the row's output weight (sum of residues) and the
// final v1/v2 contraction (src/lib.rs:5393-5401): entries whose columns are
// all set.

template <typename K, int R, int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) compact_kernel(const Slot<K, R>* __restrict__ table, u64 slots,
                                                        void* __restrict__ keys_out, u32* __restrict__ res_out,
                                                        u64 out_stride, unsigned n, int write_out,
                                                        StepScalars* __restrict__ sc) {
  constexpr int WARPS = BLOCK / 32;
  __shared__ u32 s_warp[ITEMS][WARPS];
  __shared__ unsigned long long s_base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const u64 mask = board_mask(n);
  const u64 chunk = (u64)BLOCK * ITEMS;
  if (*reinterpret_cast<volatile const u32*>(&sc->error)) return;  // insertion failed: leave the boundary intact
  unsigned long long wsum[R], fsum[R], fstates = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) wsum[r] = fsum[r] = 0;

  for (u64 c0 = (u64)blockIdx.x * chunk; c0 < slots; c0 += (u64)gridDim.x * chunk) {
    K nk[ITEMS];
    u32 flags = 0;
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const u64 s = c0 + (u64)it * BLOCK + threadIdx.x;
      nk[it] = s < slots ? table[s].nkey : (K)0;
      const bool occ = nk[it] != (K)0;
      flags |= (u32)occ << it;
      const u32 b = __ballot_sync(kFull, occ);
      if (lane == 0) s_warp[it][wid] = __popc(b);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      u32 run = 0;
      for (int it = 0; it < ITEMS; ++it)
        for (int w = 0; w < WARPS; ++w) {
          const u32 c = s_warp[it][w];
          s_warp[it][w] = run;
          run += c;
        }
      s_base = run ? atomicAdd(&sc->out_count, (unsigned long long)run) : 0ull;
    }
    __syncthreads();
    const unsigned long long base = s_base;
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const bool occ = (flags >> it) & 1u;
      const u32 b = __ballot_sync(kFull, occ);
      if (occ) {
        const u64 s = c0 + (u64)it * BLOCK + threadIdx.x;
        const K key = ~nk[it];
        const u64 idx = base + s_warp[it][wid] + __popc(b & ((1u << lane) - 1u));
        const bool full = ((u64)key & mask) == mask;
        if (write_out) reinterpret_cast<K*>(keys_out)[idx] = key;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const u32 v = (u32)(table[s].acc[r] % prime_at(r));
          if (write_out) res_out[r * out_stride + idx] = v;
          wsum[r] += v;
          if (full) fsum[r] += v;
        }
        fstates += full;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    unsigned long long t = block_sum_u64<BLOCK>(wsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->weight_sum[r], t);
    t = block_sum_u64<BLOCK>(fsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->final_sum[r], t);
  }
  unsigned long long t = block_sum_u64<BLOCK>(fstates);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->final_states, t);
}

constexpr int kBlock = 256;
constexpr int kCompactItems = 8;

unsigned grid_for(u64 work, int per_block, int sms, int blocks_per_sm) {
  u64 want = (work + per_block - 1) / per_block;
  u64 cap = (u64)sms * blocks_per_sm;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (unsigned)want;
}

template <typename F>
cudaError_t dispatch(const LaunchCfg& cfg, F&& f) {
  switch (cfg.residues) {
    case 1:
      return cfg.key_bits == 64 ? f((u64)0, std::integral_constant<int, 1>()) : f((u128)0, std::integral_constant<int, 1>());
    case 2:
      return cfg.key_bits == 64 ? f((u64)0, std::integral_constant<int, 2>()) : f((u128)0, std::integral_constant<int, 2>());
    case 3:
      return cfg.key_bits == 64 ? f((u64)0, std::integral_constant<int, 3>()) : f((u128)0, std::integral_constant<int, 3>());
    case 4:
      return cfg.key_bits == 64 ? f((u64)0, std::integral_constant<int, 4>()) : f((u128)0, std::integral_constant<int, 4>());
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t upload_c_table(const CTableDev& table, cudaStream_t stream) {
  return cudaMemcpyToSymbolAsync(c_table, &table, sizeof(CTableDev), 0, cudaMemcpyHostToDevice, stream);
}

size_t slot_bytes(int key_bits, int residues) {
  const int kb = key_bits == 64 ? 8 : 16;
  const int raw = kb + 8 * residues;
  return raw <= 16 ? 16 : raw <= 32 ? 32 : 64;
}

cudaError_t launch_row_count(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n,
                             StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  const unsigned grid = grid_for(n_in, kBlock * 4, cfg.sms, 8);
  if (cfg.key_bits == 64)
    row_count_kernel<u64, kBlock><<<grid, kBlock, 0, stream>>>(in.keys, n_in, n, sc);
  else
    row_count_kernel<u128, kBlock><<<grid, kBlock, 0, stream>>>(in.keys, n_in, n, sc);
  return cudaGetLastError();
}

cudaError_t launch_row_expand_insert(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n,
                                     void* table, uint64_t table_slots, StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  return dispatch(cfg, [&](auto kz, auto rz) -> cudaError_t {
    using K = decltype(kz);
    constexpr int R = decltype(rz)::value;
    const unsigned grid = grid_for(n_in, kBlock, cfg.sms, 8);
    row_expand_insert_kernel<K, R, kBlock><<<grid, kBlock, 0, stream>>>(
        in.keys, in.res, in.cap, n_in, n, reinterpret_cast<Slot<K, R>*>(table), table_slots - 1, sc);
    return cudaGetLastError();
  });
}

cudaError_t launch_site_count(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n, unsigned site,
                              StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  const unsigned grid = grid_for(n_in, kBlock * 4, cfg.sms, 8);
  if (cfg.key_bits == 64)
    site_count_kernel<u64, kBlock><<<grid, kBlock, 0, stream>>>(in.keys, n_in, n, site, sc);
  else
    site_count_kernel<u128, kBlock><<<grid, kBlock, 0, stream>>>(in.keys, n_in, n, site, sc);
  return cudaGetLastError();
}

cudaError_t launch_site_expand_insert(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, unsigned n,
                                      unsigned site, void* table, uint64_t table_slots, StepScalars* sc,
                                      cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  return dispatch(cfg, [&](auto kz, auto rz) -> cudaError_t {
    using K = decltype(kz);
    constexpr int R = decltype(rz)::value;
    const unsigned grid = grid_for(n_in, kBlock, cfg.sms, 8);
    site_expand_insert_kernel<K, R, kBlock><<<grid, kBlock, 0, stream>>>(
        in.keys, in.res, in.cap, n_in, n, site, reinterpret_cast<Slot<K, R>*>(table), table_slots - 1, sc);
    return cudaGetLastError();
  });
}

cudaError_t launch_compact(const LaunchCfg& cfg, const void* table, uint64_t table_slots, const FrontierView& out,
                           unsigned n, bool write_out, StepScalars* sc, cudaStream_t stream) {
  return dispatch(cfg, [&](auto kz, auto rz) -> cudaError_t {
    using K = decltype(kz);
    constexpr int R = decltype(rz)::value;
    const unsigned grid = grid_for(table_slots, kBlock * kCompactItems, cfg.sms, 8);
    compact_kernel<K, R, kBlock, kCompactItems><<<grid, kBlock, 0, stream>>>(
        reinterpret_cast<const Slot<K, R>*>(table), table_slots, out.keys, out.res, out.cap, n, write_out ? 1 : 0, sc);
    return cudaGetLastError();
  });
}

// ---------------------------------------------------------------------------
// Explicit-C generic site frontier (src/lib.rs:1519-1711): one site step.

namespace {

__device__ __forceinline__ u128 shift_u128(u128 v, int s) { return s >= 0 ? (v << s) : (v >> (-s)); }

template <int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) frontier_expand_insert_kernel(const u128* __restrict__ keys,
                                                                       const u32* __restrict__ res, u64 res_stride,
                                                                       u64 n_in, Slot<u128, R>* __restrict__ table,
                                                                       u64 mask, StepScalars* __restrict__ sc) {
  unsigned long long accepted = 0;
  bool failed = false;  // probe bound hit (error already flagged): stop inserting, still reach the block sum
  const u32 n_runs = c_frontier.n_runs, n_trans = c_frontier.n_trans;
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in && !failed; i += (u64)gridDim.x * BLOCK) {
    const u128 key = keys[i];
    u128 moved = 0;
    for (u32 r = 0; r < n_runs; ++r) moved |= shift_u128(key & c_frontier.run_mask[r], c_frontier.run_shift[r]);
    u32 w[R];
#pragma unroll
    for (int r = 0; r < R; ++r) w[r] = res[r * res_stride + i];
    for (u32 t = 0; t < n_trans; ++t) {
      if ((key & c_frontier.req_mask[t]) != c_frontier.req_value[t]) continue;
      ++accepted;
      if (!table_insert<u128, R>(table, mask, moved | c_frontier.added[t], w, kMaxProbe, &sc->error)) {
        failed = true;
        break;
      }
    }
  }
  const unsigned long long t = block_sum_u64<BLOCK>(accepted);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->terms, t);
}

}  // namespace

cudaError_t upload_frontier_step(const FrontierStepDev& step, cudaStream_t stream) {
  return cudaMemcpyToSymbolAsync(c_frontier, &step, sizeof step, 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t launch_frontier_expand_insert(const LaunchCfg& cfg, const FrontierView& in, uint64_t n_in, void* table,
                                          uint64_t table_slots, StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (cfg.key_bits != 128 || (table_slots & (table_slots - 1))) return cudaErrorInvalidValue;
  constexpr int kBlock = 256;
  const u64 want = (n_in + kBlock - 1) / kBlock;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)cfg.sms * 8));
  const u128* keys = reinterpret_cast<const u128*>(in.keys);
  switch (cfg.residues) {
    case 1:
      frontier_expand_insert_kernel<1, kBlock><<<grid, kBlock, 0, stream>>>(
          keys, in.res, in.cap, n_in, reinterpret_cast<Slot<u128, 1>*>(table), table_slots - 1, sc);
      break;
    case 2:
      frontier_expand_insert_kernel<2, kBlock><<<grid, kBlock, 0, stream>>>(
          keys, in.res, in.cap, n_in, reinterpret_cast<Slot<u128, 2>*>(table), table_slots - 1, sc);
      break;
    case 3:
      frontier_expand_insert_kernel<3, kBlock><<<grid, kBlock, 0, stream>>>(
          keys, in.res, in.cap, n_in, reinterpret_cast<Slot<u128, 3>*>(table), table_slots - 1, sc);
      break;
    case 4:
      frontier_expand_insert_kernel<4, kBlock><<<grid, kBlock, 0, stream>>>(
          keys, in.res, in.cap, n_in, reinterpret_cast<Slot<u128, 4>*>(table), table_slots - 1, sc);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace qpeps

// Partitioned key merge: one row step as two streaming kernels.
//
//   partition_scatter : every parent is read once (coalesced); each
//                       (parent, free column) successor is appended to one of
//                       P hash partitions (16-byte candidate = key + residues).
//                       Partition tails stay in L2, so the scattered 16-byte
//                       stores reach HBM as full sectors.
//   partition_merge   : one CTA per partition loads its candidates (coalesced)
//                       into a shared-memory open-addressing table, sums equal
//                       keys' residues with shared-memory atomics, and writes
//                       the unique entries to the next boundary buffer.
//
// This replaces the reference's `candidates.sort_unstable_by_key` + checked
// reduce (src/lib.rs:5353-5367): equal packed keys are merged by addition;
// the order of the output boundary is not observable by any metric.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {

namespace {

constexpr u32 kFullMask = 0xffffffffu;

__host__ __device__ __forceinline__ u64 pboard_mask_host(unsigned n) { return n >= 64 ? ~0ull : ((1ull << n) - 1); }

__device__ __forceinline__ int pwarp_inclusive_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int t = __shfl_up_sync(kFullMask, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

__device__ __forceinline__ unsigned pnth_set_bit(u64 m, int k) {
  u32 lo = (u32)m, hi = (u32)(m >> 32);
  int plo = __popc(lo);
  return k < plo ? __fns(lo, 0, k + 1) : 32u + __fns(hi, 0, k - plo + 1);
}

// No u64 boundary key is all ones. Up to N = 21 bit 63 is clear (3n <= 63).
// At N = 22 (compact layout, 64 live bits) all ones would need all 22 columns
// set, so the last row placed, and all 21 live dr and all 21 live dl signals
// set: 42 signals, where the queen of row i still has a dr signal on the board
// only if its column is below i and a dl signal only if its column is at least
// 22 - i, so at most 22 queens + the 10 of rows 12..21 give 32.
constexpr u64 kEmptyKey = ~0ull;

// Map a 64-bit hash uniformly onto [0, parts) (multiply-high).
__device__ __forceinline__ u32 partition_of(u64 h, u32 parts) { return (u32)(((h >> 32) * (u64)parts) >> 32); }

template <int R>
struct alignas(16) Cand {
  u64 key;
  u32 res[R];
};

// 16-byte vector moves of a candidate (one or two ulonglong2).
template <int R>
__device__ __forceinline__ void store_cand(Cand<R>* dst, const Cand<R>& c) {
  ulonglong2* d = reinterpret_cast<ulonglong2*>(dst);
  u64 w01 = (u64)c.res[0] | (R > 1 ? (u64)c.res[R > 1 ? 1 : 0] << 32 : 0ull);
  d[0] = make_ulonglong2(c.key, w01);
  if constexpr (R > 2) {
    u64 w23 = (u64)c.res[2] | (R > 3 ? (u64)c.res[R > 3 ? 3 : 2] << 32 : 0ull);
    d[1] = make_ulonglong2(w23, 0ull);
  }
}

// L2 policy that keeps lines resident in preference to others: partition
// tails are written 16 bytes at a time, and a line evicted before it is full
// costs a DRAM read-fill and a second write-back.
__device__ __forceinline__ u64 l2_keep_policy() {
  u64 policy;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(policy));
  return policy;
}

template <int R>
__device__ __forceinline__ void store_cand_keep(Cand<R>* dst, const Cand<R>& c, u64 policy) {
  u64 w01 = (u64)c.res[0] | (R > 1 ? (u64)c.res[R > 1 ? 1 : 0] << 32 : 0ull);
  asm volatile("st.global.L2::cache_hint.v2.u64 [%0], {%1, %2}, %3;" ::"l"(dst), "l"(c.key), "l"(w01), "l"(policy)
               : "memory");
  if constexpr (R > 2) {
    u64 w23 = (u64)c.res[2] | (R > 3 ? (u64)c.res[R > 3 ? 3 : 2] << 32 : 0ull);
    asm volatile("st.global.L2::cache_hint.v2.u64 [%0], {%1, %2}, %3;" ::"l"(reinterpret_cast<char*>(dst) + 16),
                 "l"(w23), "l"(0ull), "l"(policy)
                 : "memory");
  }
}

template <int R>
__device__ __forceinline__ Cand<R> load_cand(const Cand<R>* src) {
  const ulonglong2* s = reinterpret_cast<const ulonglong2*>(src);
  const ulonglong2 a = __ldcs(s);
  Cand<R> c;
  c.key = a.x;
  c.res[0] = (u32)a.y;
  if constexpr (R > 1) c.res[R > 1 ? 1 : 0] = (u32)(a.y >> 32);
  if constexpr (R > 2) {
    const ulonglong2 b = __ldcs(s + 1);
    c.res[R > 2 ? 2 : 0] = (u32)b.x;
    if constexpr (R > 3) c.res[R > 3 ? 3 : 0] = (u32)(b.x >> 32);
  }
  return c;
}

template <int BLOCK>
__device__ __forceinline__ unsigned long long pblock_sum(unsigned long long v) {
  __shared__ unsigned long long s_part[BLOCK / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFullMask, v, d);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_part[wid] = v;
  __syncthreads();
  unsigned long long t = 0;
  if (wid == 0) {
    t = lane < BLOCK / 32 ? s_part[lane] : 0ull;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(kFullMask, t, d);
  }
  return t;
}

// ---------------------------------------------------------------------------
// Scatter. Each warp takes 64 parents per iteration (two per lane; the next
// iteration's parents are loaded before this iteration's atomics are waited
// on), flattens the ragged (parent, free column) list, and for every batch of
// up to KB*32 successors issues all cursor atomics before any store, so each
// lane keeps KB atomics in flight.

constexpr int kKB = 4;  // successor rounds per atomic batch

// kPPL parents per lane per iteration (2 or 4); partition cursors are
// `cstride` u32 apart (a stride of 8 gives each cursor its own 32-byte sector,
// spreading a small cursor array over more L2 slices).
template <int R, int BLOCK, int kPPL, typename Layout>
__global__ void __launch_bounds__(BLOCK) partition_scatter_kernel(const u64* __restrict__ keys,
                                                                  const u32* __restrict__ res, u64 res_stride,
                                                                  u64 n_in, Layout L, Cand<R>* __restrict__ regions,
                                                                  u32* __restrict__ cursors, u32 cstride, u32 parts,
                                                                  u32 cap, StepScalars* __restrict__ sc) {
  constexpr int WARPS = BLOCK / 32;
  constexpr int PW = 32 * kPPL;  // parents per warp iteration
  __shared__ u64 s_key[WARPS][PW];
  __shared__ u64 s_free[WARPS][PW];
  __shared__ u32 s_w[WARPS][R][PW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const u64 gwarp = (u64)blockIdx.x * WARPS + wid;
  const u64 stride = (u64)gridDim.x * WARPS * PW;
  bool overflow = false;

  // Prefetched parents of the next iteration (registers).
  u64 nkey[kPPL];
  u32 nw[kPPL][R];
  auto fetch = [&](u64 base) {
#pragma unroll
    for (int q = 0; q < kPPL; ++q) {
      const u64 i = base + q * 32 + lane;
      nkey[q] = kEmptyKey;
      if (i < n_in) {
        nkey[q] = keys[i];
#pragma unroll
        for (int r = 0; r < R; ++r) nw[q][r] = res[r * res_stride + i];
      }
    }
  };
  u64 base = gwarp * PW;
  if (base < n_in) fetch(base);
  for (; base < n_in; base += stride) {
    int cnt = 0;
    int cum[kPPL];  // successors of this lane's parents 0..q-1
#pragma unroll
    for (int q = 0; q < kPPL; ++q) {
      u64 fr = 0;
      if (nkey[q] != kEmptyKey) {
        const State s = L.unpack(nkey[q]);
        fr = ~(s.cols | s.dr | s.dl) & L.mask_of(nkey[q]);
      }
      s_key[wid][q * 32 + lane] = nkey[q];
      s_free[wid][q * 32 + lane] = fr;
#pragma unroll
      for (int r = 0; r < R; ++r) s_w[wid][r][q * 32 + lane] = nw[q][r];
      cum[q] = cnt;
      cnt += __popcll(fr);
    }
    if (base + stride < n_in) fetch(base + stride);
    const int incl = pwarp_inclusive_scan(cnt);
    const int excl = incl - cnt;
    const int total = __shfl_sync(kFullMask, incl, 31);
    __syncwarp();
    for (int j0 = 0; j0 < total; j0 += 32 * kKB) {
      Cand<R> c[kKB];
      u32 part[kKB], pos[kKB];
#pragma unroll
      for (int k = 0; k < kKB; ++k) {
        part[k] = 0xffffffffu;
        if (j0 + k * 32 >= total) continue;  // warp-uniform: no successors left for this round
        const int j = j0 + k * 32 + lane;
        int owner = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int v = __shfl_sync(kFullMask, incl, owner + step - 1);
          if (v <= j) owner += step;
        }
        const int oex = __shfl_sync(kFullMask, excl, owner);
        int ocum[kPPL];
#pragma unroll
        for (int q = 1; q < kPPL; ++q) ocum[q] = __shfl_sync(kFullMask, cum[q], owner);
        if (j < total) {
          int t = j - oex;
          int q = 0;
#pragma unroll
          for (int qq = 1; qq < kPPL; ++qq)
            if (t >= ocum[qq]) q = qq;
          t -= q ? ocum[q] : 0;
          const int slot = q * 32 + owner;
          const u64 pkey = s_key[wid][slot];
          const State s = L.unpack(pkey);
          const unsigned col = pnth_set_bit(s_free[wid][slot], t);
          c[k].key = L.successor(pkey, s, 1ull << col);
#pragma unroll
          for (int r = 0; r < R; ++r) c[k].res[r] = s_w[wid][r][slot];
          part[k] = partition_of(fib_hash_a(c[k].key), parts);
        }
      }
#pragma unroll
      for (int k = 0; k < kKB; ++k)
        if (part[k] != 0xffffffffu) pos[k] = atomicAdd(&cursors[(u64)part[k] * cstride], 1u);
#pragma unroll
      for (int k = 0; k < kKB; ++k)
        if (part[k] != 0xffffffffu) {
          if (pos[k] < cap)
            store_cand<R>(regions + (u64)part[k] * cap + pos[k], c[k]);
          else
            overflow = true;
        }
    }
    __syncwarp();
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

// List-expansion variant of the scatter. Each lane keeps its kPPL parents in
// registers and writes its own successors, as finished 16- or 32-byte
// candidates, into a per-warp shared-memory window of kKB*32 slots (lane
// order = scan order, so the window is dense); the warp then reads the window
// back one candidate per lane and round, and issues the cursor atomics and
// stores. No shuffle search and no nth-set-bit: every successor is produced
// by the lane that owns its parent, lowest free column first. Same inputs,
// outputs and overflow rule as partition_scatter_kernel.
template <int R, int BLOCK, int kPPL, typename Layout>
__global__ void __launch_bounds__(BLOCK, (kPPL <= 2 ? 4 : 3)) partition_scatter_list_kernel(const u64* __restrict__ keys,
                                                                       const u32* __restrict__ res, u64 res_stride,
                                                                       u64 n_in, Layout L,
                                                                       Cand<R>* __restrict__ regions,
                                                                       u32* __restrict__ cursors, u32 cstride,
                                                                       u32 parts, u32 cap,
                                                                       StepScalars* __restrict__ sc) {
  constexpr int WARPS = BLOCK / 32;
  constexpr int PW = 32 * kPPL;  // parents per warp iteration
  constexpr int WIN = 32 * kKB;  // candidates per window
  __shared__ Cand<R> s_cand[WARPS][WIN];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const u64 gwarp = (u64)blockIdx.x * WARPS + wid;
  const u64 stride = (u64)gridDim.x * WARPS * PW;
  bool overflow = false;
  const u64 policy = l2_keep_policy();

  u64 nkey[kPPL], ckey[kPPL], fr[kPPL];
  u32 nw[kPPL][R], cw[kPPL][R];
  auto fetch = [&](u64 base) {
#pragma unroll
    for (int q = 0; q < kPPL; ++q) {
      const u64 i = base + q * 32 + lane;
      nkey[q] = kEmptyKey;
      if (i < n_in) {
        nkey[q] = __ldcs(keys + i);
#pragma unroll
        for (int r = 0; r < R; ++r) nw[q][r] = __ldcs(res + r * res_stride + i);
      }
    }
  };
  u64 base = gwarp * PW;
  if (base < n_in) fetch(base);
  for (; base < n_in; base += stride) {
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < kPPL; ++q) {
      ckey[q] = nkey[q];
      fr[q] = 0;
      if (ckey[q] != kEmptyKey) {
        const State s = L.unpack(ckey[q]);
        fr[q] = ~(s.cols | s.dr | s.dl) & L.mask_of(ckey[q]);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) cw[q][r] = nw[q][r];
      cnt += __popcll(fr[q]);
    }
    if (base + stride < n_in) fetch(base + stride);
    const int incl = pwarp_inclusive_scan(cnt);
    const int total = __shfl_sync(kFullMask, incl, 31);
    int g = incl - cnt;  // index of this lane's next successor
    for (int j0 = 0; j0 < total; j0 += WIN) {
      const int hi = min(incl, j0 + WIN);
#pragma unroll
      for (int q = 0; q < kPPL; ++q) {
        if (g < hi && fr[q]) {
          const State s = L.unpack(ckey[q]);
          do {
            const u64 b = fr[q] & (0ull - fr[q]);
            fr[q] ^= b;
            Cand<R> c;
            c.key = L.successor(ckey[q], s, b);
#pragma unroll
            for (int r = 0; r < R; ++r) c.res[r] = cw[q][r];
            s_cand[wid][g - j0] = c;
            ++g;
          } while (g < hi && fr[q]);
        }
      }
      __syncwarp();
      // Candidates stay in shared memory while their cursor atomics are in
      // flight (only the partition index is held in registers).
      u32 part[kKB], pos[kKB];
#pragma unroll
      for (int k = 0; k < kKB; ++k) {
        part[k] = 0xffffffffu;
        if (j0 + k * 32 + lane < total)
          part[k] = partition_of(fib_hash_a(s_cand[wid][k * 32 + lane].key), parts);
      }
#pragma unroll
      for (int k = 0; k < kKB; ++k)
        if (part[k] != 0xffffffffu) pos[k] = atomicAdd(&cursors[(u64)part[k] * cstride], 1u);
#pragma unroll
      for (int k = 0; k < kKB; ++k)
        if (part[k] != 0xffffffffu) {
          if (pos[k] < cap)
            store_cand_keep<R>(regions + (u64)part[k] * cap + pos[k], s_cand[wid][k * 32 + lane], policy);
          else
            overflow = true;
        }
      __syncwarp();
    }
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

// Direct variant of the scatter (scatter_kind 4). Each lane expands its own
// kPPL parents and issues their successors' cursor atomics and candidate
// stores itself, kDB successors per round, with no shared-memory window and
// no shuffles: per candidate the load/store pipe carries one atomic and one
// store, where the window scatter adds a shared-memory write and read. Lanes
// with fewer successors idle in the rounds the warp's busiest lane still
// needs. Same inputs, outputs and overflow rule as the other scatters.
constexpr int kDB = 4;  // successors per lane per round (atomics in flight per lane)

template <int R, int BLOCK, int kPPL, typename Layout>
__global__ void __launch_bounds__(BLOCK, (kPPL <= 2 ? 4 : 3)) partition_scatter_direct_kernel(const u64* __restrict__ keys,
                                                                          const u32* __restrict__ res, u64 res_stride,
                                                                          u64 n_in, Layout L,
                                                                          Cand<R>* __restrict__ regions,
                                                                          u32* __restrict__ cursors, u32 cstride,
                                                                          u32 parts, u32 cap,
                                                                          StepScalars* __restrict__ sc) {
  constexpr int WARPS = BLOCK / 32;
  constexpr int PW = 32 * kPPL;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const u64 gwarp = (u64)blockIdx.x * WARPS + wid;
  const u64 stride = (u64)gridDim.x * WARPS * PW;
  bool overflow = false;
  const u64 policy = l2_keep_policy();
  u64 nkey[kPPL];
  u32 nw[kPPL][R];
  auto fetch = [&](u64 base) {
#pragma unroll
    for (int q = 0; q < kPPL; ++q) {
      const u64 i = base + q * 32 + lane;
      nkey[q] = kEmptyKey;
      if (i < n_in) {
        nkey[q] = __ldcs(keys + i);
#pragma unroll
        for (int r = 0; r < R; ++r) nw[q][r] = __ldcs(res + r * res_stride + i);
      }
    }
  };
  u64 base = gwarp * PW;
  if (base < n_in) fetch(base);
  for (; base < n_in; base += stride) {
    u64 ckey[kPPL], fr[kPPL];
    u32 cw[kPPL][R];
#pragma unroll
    for (int q = 0; q < kPPL; ++q) {
      ckey[q] = nkey[q];
      fr[q] = 0;
      if (ckey[q] != kEmptyKey) {
        const State s = L.unpack(ckey[q]);
        fr[q] = ~(s.cols | s.dr | s.dl) & L.mask_of(ckey[q]);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) cw[q][r] = nw[q][r];
    }
    if (base + stride < n_in) fetch(base + stride);
    int q = 0;  // this lane's current parent
    while (q < kPPL && !fr[q]) ++q;
    while (__any_sync(kFullMask, q < kPPL)) {
      Cand<R> c[kDB];
      u32 part[kDB], pos[kDB];
#pragma unroll
      for (int k = 0; k < kDB; ++k) {
        part[k] = 0xffffffffu;
        if (q < kPPL) {
          // q < kPPL implies fr[q] != 0; the parent index is dynamic, so pick
          // its words with a small unrolled select.
          u64 pk = ckey[0], pf = fr[0];
          u32 pw[R];
#pragma unroll
          for (int r = 0; r < R; ++r) pw[r] = cw[0][r];
#pragma unroll
          for (int qq = 1; qq < kPPL; ++qq)
            if (q == qq) {
              pk = ckey[qq];
              pf = fr[qq];
#pragma unroll
              for (int r = 0; r < R; ++r) pw[r] = cw[qq][r];
            }
          const u64 b = pf & (0ull - pf);
          const State s = L.unpack(pk);
          c[k].key = L.successor(pk, s, b);
#pragma unroll
          for (int r = 0; r < R; ++r) c[k].res[r] = pw[r];
          part[k] = partition_of(fib_hash_a(c[k].key), parts);
#pragma unroll
          for (int qq = 0; qq < kPPL; ++qq)
            if (q == qq) fr[qq] ^= b;
          while (q < kPPL) {
            u64 left = fr[0];
#pragma unroll
            for (int qq = 1; qq < kPPL; ++qq)
              if (q == qq) left = fr[qq];
            if (left) break;
            ++q;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kDB; ++k)
        if (part[k] != 0xffffffffu) pos[k] = atomicAdd(&cursors[(u64)part[k] * cstride], 1u);
#pragma unroll
      for (int k = 0; k < kDB; ++k)
        if (part[k] != 0xffffffffu) {
          if (pos[k] < cap)
            store_cand_keep<R>(regions + (u64)part[k] * cap + pos[k], c[k], policy);
          else
            overflow = true;
        }
    }
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

// ---------------------------------------------------------------------------
// Merge. One CTA per partition at a time (persistent over partitions). All
// candidate loads of a partition are issued together into registers; the
// next partition's loads are issued before the current table is compacted,
// and compaction resets the slots it reads so the table needs no separate
// clearing pass.

constexpr u64 kEmpty = kEmptyKey;

// Free columns of a fixed-layout boundary key at the next row: the successor
// terms it will generate there (what row_count_kernel sums).
__device__ __forceinline__ unsigned long long next_terms_of(const FixedLayout& L, u64 key) {
  const State st = L.unpack(key);
  return (unsigned long long)__popcll(~(st.cols | st.dr | st.dl) & L.mask);
}
template <typename Layout>
__device__ __forceinline__ unsigned long long next_terms_of(const Layout&, u64) {
  return 0ull;
}

template <int R, int BLOCK, int H, int CAP, typename Layout>
__global__ void __launch_bounds__(BLOCK) partition_merge_kernel(const Cand<R>* __restrict__ regions,
                                                                const u32* __restrict__ cursors, u32 cstride,
                                                                u32 parts,
                                                                u64* __restrict__ keys_out, u32* __restrict__ res_out,
                                                                u64 out_stride, Layout L, int write_out,
                                                                StepScalars* __restrict__ sc) {
  static_assert((H & (H - 1)) == 0 && H >= 2, "merge table size must be a power of two");
  constexpr int kLogH = 31 - __builtin_clz(H);
  constexpr int WARPS = BLOCK / 32;
  constexpr int PER = H / BLOCK;    // table slots per thread
  constexpr int LPT = CAP / BLOCK;  // candidate loads per thread
  static_assert(H % BLOCK == 0 && CAP % BLOCK == 0 && PER <= 32 && (PER * WARPS) % 32 == 0, "shape");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u64* s_key = reinterpret_cast<u64*>(smem_raw);
  unsigned long long* s_acc = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(u64) * H);  // [R][H]
  __shared__ u32 s_cnt[PER * WARPS];
  __shared__ unsigned long long s_base;
  // Serving: finished boards are summed per request slot here, then flushed.
  __shared__ unsigned long long s_slot_fin[Layout::kSlotted ? kServeMaxSlots * R : 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if constexpr (Layout::kSlotted)
    for (int i = threadIdx.x; i < (int)kServeMaxSlots * R; i += BLOCK) s_slot_fin[i] = 0ull;
  // A partition overflowed in the scatter: write nothing, so the boundary
  // buffer (read by the scatter, written here in place) stays intact for the
  // host's retry with smaller partitions.
  if (*reinterpret_cast<volatile const u32*>(&sc->error)) return;
  // write_out: bit 0 writes the merged boundary, bit 1 also counts its
  // successor terms at the next row (left out of CUDA-graph replays, whose
  // sizes are recorded).
  const bool count_next = (write_out & 2) != 0;
  write_out &= 1;
  unsigned long long wsum[R], fsum[R], fstates = 0;
  unsigned long long nterms = 0;  // the written boundary's successor terms at the next row
  bool bad = false;  // an output index beyond the boundary buffer (skipped)
#pragma unroll
  for (int r = 0; r < R; ++r) wsum[r] = fsum[r] = 0;

  for (int i = threadIdx.x; i < H; i += BLOCK) {
    s_key[i] = kEmpty;
#pragma unroll
    for (int r = 0; r < R; ++r) s_acc[r * H + i] = 0ull;
  }

  Cand<R> buf[LPT];
  u32 bcnt = 0;
  auto fetch = [&](u32 part) {
    bcnt = min(cursors[(u64)part * cstride], (u32)CAP);
    const Cand<R>* src = regions + (u64)part * CAP;
#pragma unroll
    for (int l = 0; l < LPT; ++l) {
      const u32 i = l * BLOCK + threadIdx.x;
      if (i < bcnt) buf[l] = load_cand<R>(src + i);
    }
  };
  u32 part = blockIdx.x;
  if (part < parts) fetch(part);
  __syncthreads();
  for (; part < parts; part += gridDim.x) {
    // Insert the fetched candidates.
#pragma unroll
    for (int l = 0; l < LPT; ++l) {
      const u32 i = l * BLOCK + threadIdx.x;
      if (i < bcnt) {
        const Cand<R>& c = buf[l];
        u32 slot = (u32)(fib_hash_b(c.key) >> (64 - kLogH));
        for (int probe = 0; probe < H; ++probe) {
          u64 cur = s_key[slot];
          if (cur == kEmpty) {
            cur = atomicCAS(reinterpret_cast<unsigned long long*>(&s_key[slot]), kEmpty, c.key);
            if (cur == kEmpty) cur = c.key;
          }
          if (cur == c.key) {
#pragma unroll
            for (int r = 0; r < R; ++r) atomicAdd(&s_acc[r * H + slot], (unsigned long long)c.res[r]);
            break;
          }
          slot = (slot + 1) & (H - 1);
        }
      }
    }
    __syncthreads();
    // Prefetch the next partition while this one is compacted.
    const u32 next = part + gridDim.x;
    if (next < parts) fetch(next);
    // Compaction: slot it*BLOCK + tid belongs to this thread (conflict-free,
    // coalesced); one warp scans the PER x WARPS ballot counts.
    u32 flags = 0;
#pragma unroll
    for (int it = 0; it < PER; ++it) {
      bool occ = s_key[it * BLOCK + threadIdx.x] != kEmpty;
      if constexpr (Layout::kSlotted) {
        // A finished board leaves the boundary: sum it into its slot.
        const u64 key = s_key[it * BLOCK + threadIdx.x];
        if (occ && (key & L.mask_of(key)) == L.mask_of(key)) {
          const int slot = it * BLOCK + threadIdx.x;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            atomicAdd(&s_slot_fin[L.slot(key) * R + r], (unsigned long long)reduce_sum(s_acc[r * H + slot], r));
            s_acc[r * H + slot] = 0ull;
          }
          s_key[slot] = kEmpty;
          occ = false;
        }
      }
      flags |= (u32)occ << it;
      const u32 b = __ballot_sync(kFullMask, occ);
      if (lane == 0) s_cnt[it * WARPS + wid] = __popc(b);
    }
    __syncthreads();
    if (wid == 0) {
      constexpr int PL = PER * WARPS / 32;  // counts per lane
      u32 v[PL];
      u32 sum = 0;
#pragma unroll
      for (int q = 0; q < PL; ++q) {
        v[q] = s_cnt[lane * PL + q];
        sum += v[q];
      }
      const int incl = pwarp_inclusive_scan((int)sum);
      u32 run = (u32)incl - sum;
#pragma unroll
      for (int q = 0; q < PL; ++q) {
        s_cnt[lane * PL + q] = run;
        run += v[q];
      }
      const int tot = __shfl_sync(kFullMask, incl, 31);
      if (lane == 0) s_base = tot ? atomicAdd(&sc->out_count, (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    const unsigned long long base = s_base;
#pragma unroll
    for (int it = 0; it < PER; ++it) {
      const bool occ = (flags >> it) & 1u;
      const u32 b = __ballot_sync(kFullMask, occ);
      if (occ) {
        const int slot = it * BLOCK + threadIdx.x;
        const u64 key = s_key[slot];
        const u64 idx = base + s_cnt[it * WARPS + wid] + __popc(b & ((1u << lane) - 1u));
        const bool full = (key & L.mask_of(key)) == L.mask_of(key);
        const bool wr = write_out && idx < out_stride;
        bad |= write_out && !wr;
        if (wr) keys_out[idx] = key;
        if constexpr (!Layout::kSlotted)
          if (count_next) nterms += next_terms_of(L, key);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const u32 v = reduce_sum(s_acc[r * H + slot], r);
          if (wr) res_out[r * out_stride + idx] = v;
          wsum[r] += v;
          if (full) fsum[r] += v;
          s_acc[r * H + slot] = 0ull;
        }
        s_key[slot] = kEmpty;
        fstates += full;
      }
    }
    __syncthreads();
  }
  if (bad) atomicOr(&sc->error, kErrBounds);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    unsigned long long t = pblock_sum<BLOCK>(wsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->weight_sum[r], t);
    t = pblock_sum<BLOCK>(fsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->final_sum[r], t);
  }
  const unsigned long long t = pblock_sum<BLOCK>(fstates);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->final_states, t);
  if constexpr (!Layout::kSlotted) {
    if (write_out && count_next) {
      const unsigned long long nt = pblock_sum<BLOCK>(nterms);
      if (threadIdx.x == 0 && nt) atomicAdd(&sc->next_terms, nt);
      if (blockIdx.x == 0 && threadIdx.x == 0) sc->next_terms_ok = 1u;
    }
  }
  if constexpr (Layout::kSlotted) {
    __syncthreads();
    for (int i = threadIdx.x; i < (int)kServeMaxSlots * R; i += BLOCK)
      if (s_slot_fin[i]) atomicAdd(&L.slot_final[(i / R) * 4 + (i % R)], s_slot_fin[i]);
  }
}

// Listed variant of the merge, in three phases per partition:
//   1. every candidate claims or finds its key's slot with one shared-memory
//      compare-and-swap; a key's first claimant appends the slot to a list
//      (one shared atomic per warp);
//   2. (after a barrier) first claimants store their residues into the
//      accumulators, so those need no zeroing and most candidates (keys seen
//      once) cost no atomic addition;
//   3. (after a barrier) the remaining candidates add their residues.
// Compaction then walks only the listed slots, and the list index is the
// output index (no ballot/scan pass over the table). In the slotted (serving)
// layout a finished board is summed into its request slot in phase 1 and never
// enters the table. Same inputs, outputs and sums as partition_merge_kernel;
// the order of the written entries differs.
//
// kAcc selects the accumulator (R = 2 for modes 1 and 2):
//   0: R residue planes, summed per plane and reduced on output;
//   1: a candidate's residue pair is folded into the one value below p0 * p1
//      it stands for (crt_fold2), accumulated in a single 64-bit plane and
//      reduced back to residues on output;
//   2: the two planes hold the low and high words of the exact weight, which
//      is accumulated in a single 64-bit plane and written back as words.
// Mode 1 is exact while every weight and every per-key sum stays below
// p0 * p1 (about 4.6e18): a row's weights sum to at most the number of
// partial placements, at most (free rows)! (20! = 2.4e18), so the engine uses
// it for boards with at most 20 free rows. Mode 2 is exact
// while they stay below 2^63; the engine certifies that before every row from
// the exact total of the row's input (at most that total times the free
// columns), which holds for every board with at most 20 free rows and is
// checked row by row at 21.
// The one-plane accumulator value of a candidate's two u32 words.
template <int kAcc>
__device__ __forceinline__ u64 one_plane(u32 w0, u32 w1) {
  if constexpr (kAcc == 2)
    return (u64)w0 | ((u64)w1 << 32);
  else
    return crt_fold2(w0, w1);
}

// kRegs (fixed layout only): a key's first claimant keeps the key and its list
// index in registers and writes the output entry itself after the last
// barrier, reading only the accumulator from shared memory; the slot list is
// never stored or read.
template <int R, int BLOCK, int H, int CAP, typename Layout, int kAcc = 0, bool kRegs = false>
__global__ void __launch_bounds__(BLOCK) partition_merge_list_kernel(const Cand<R>* __restrict__ regions,
                                                                     const u32* __restrict__ cursors, u32 cstride,
                                                                     u32 parts, u64* __restrict__ keys_out,
                                                                     u32* __restrict__ res_out, u64 out_stride,
                                                                     Layout L, int write_out,
                                                                     StepScalars* __restrict__ sc) {
  static_assert((H & (H - 1)) == 0 && H >= 2 * CAP, "merge table size must be a power of two >= 2 CAP");
  constexpr int kLogH = 31 - __builtin_clz(H);
  constexpr int LPT = CAP / BLOCK;  // candidate loads per thread
  static_assert(CAP % BLOCK == 0, "shape");
  constexpr bool kFold = kAcc != 0;  // one 64-bit accumulator plane
  static_assert(!kFold || R == 2, "the one-plane accumulators hold a residue pair or a weight's two words");
  static_assert(kAcc != 2 || !Layout::kSlotted, "exact weights are not used by the serving layout");
  static_assert(!kRegs || !Layout::kSlotted, "register compaction is for the fixed layout");
  constexpr int AP = kFold ? 1 : R;  // accumulator planes
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u64* s_key = reinterpret_cast<u64*>(smem_raw);
  unsigned long long* s_acc = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(u64) * H);  // [AP][H]
  u32* s_list = reinterpret_cast<u32*>(smem_raw + sizeof(u64) * H * (1 + AP));                   // [CAP]
  __shared__ u32 s_nused, s_n;
  __shared__ unsigned long long s_base;
  __shared__ unsigned long long s_slot_fin[Layout::kSlotted ? kServeMaxSlots * R : 1];
  const int lane = threadIdx.x & 31;
  if constexpr (Layout::kSlotted)
    for (int i = threadIdx.x; i < (int)kServeMaxSlots * R; i += BLOCK) s_slot_fin[i] = 0ull;
  if (*reinterpret_cast<volatile const u32*>(&sc->error)) return;
  // write_out: bit 0 writes the merged boundary, bit 1 also counts its
  // successor terms at the next row (left out of CUDA-graph replays, whose
  // sizes are recorded).
  const bool count_next = (write_out & 2) != 0;
  write_out &= 1;
  unsigned long long wsum[R], fsum[R], fstates = 0;
  // The written boundary's successor terms at the next row (the next row
  // step's count, so that it needs no counting pass of its own).
  unsigned long long nterms = 0;
  constexpr bool kCountNext = !Layout::kSlotted;
  bool bad = false;  // an output index beyond the boundary buffer (skipped)
#pragma unroll
  for (int r = 0; r < R; ++r) wsum[r] = fsum[r] = 0;
  for (int i = threadIdx.x; i < H; i += BLOCK) s_key[i] = kEmpty;
  if (threadIdx.x == 0) s_nused = 0;

  Cand<R> buf[LPT];
  u32 bcnt = 0;
  // `cnt` is the partition's cursor, loaded one iteration ahead so that the
  // candidate loads need not wait for it.
  auto fetch = [&](u32 part, u32 cnt) {
    bcnt = min(cnt, (u32)CAP);
    const Cand<R>* src = regions + (u64)part * CAP;
#pragma unroll
    for (int l = 0; l < LPT; ++l) {
      const u32 i = l * BLOCK + threadIdx.x;
      if (i < bcnt) buf[l] = load_cand<R>(src + i);
    }
  };
  u32 part = blockIdx.x;
  if (part < parts) fetch(part, cursors[(u64)part * cstride]);
  __syncthreads();
  for (; part < parts; part += gridDim.x) {
    const u32 next = part + gridDim.x;
    const u32 next_cnt = next < parts ? cursors[(u64)next * cstride] : 0u;
    u32 slots[LPT];
    u32 fidx[kRegs ? LPT : 1];   // list index of a first claimant (kRegs)
    u64 fkey[kRegs ? LPT : 1];   // and its key, kept past the next partition's loads
    u32 fresh_bits = 0, dup_bits = 0;
#pragma unroll
    for (int l = 0; l < LPT; ++l) {
      const u32 i = l * BLOCK + threadIdx.x;
      bool fresh = false;
      u32 slot = 0;
      if (i < bcnt) {
        const Cand<R>& c = buf[l];
        bool finished = false;
        if constexpr (Layout::kSlotted) {
          const u64 m = L.mask_of(c.key);
          if ((c.key & m) == m) {
#pragma unroll
            for (int r = 0; r < R; ++r) atomicAdd(&s_slot_fin[L.slot(c.key) * R + r], (unsigned long long)c.res[r]);
            finished = true;
          }
        }
        if (!finished) {
          slot = (u32)(fib_hash_b(c.key) >> (64 - kLogH));
          for (int probe = 0; probe < H; ++probe) {
            const u64 cur = atomicCAS(reinterpret_cast<unsigned long long*>(&s_key[slot]), kEmpty, c.key);
            if (cur == kEmpty || cur == c.key) {
              fresh = cur == kEmpty;
              dup_bits |= (u32)(!fresh) << l;
              break;
            }
            slot = (slot + 1) & (H - 1);
          }
        }
      }
      slots[l] = slot;
      fresh_bits |= (u32)fresh << l;
      const u32 b = __ballot_sync(kFullMask, fresh);
      if (b) {
        const int leader = __ffs(b) - 1;
        u32 at = 0;
        if (lane == leader) at = atomicAdd(&s_nused, (u32)__popc(b));
        at = __shfl_sync(kFullMask, at, leader);
        if constexpr (kRegs) {
          fidx[l] = at + __popc(b & ((1u << lane) - 1u));
          fkey[l] = buf[l].key;
        } else {
          if (fresh) s_list[at + __popc(b & ((1u << lane) - 1u))] = slot;
        }
      }
    }
#pragma unroll
    for (int l = 0; l < LPT; ++l)
      if ((fresh_bits >> l) & 1u) {
        if constexpr (kFold) {
          s_acc[slots[l]] = one_plane<kAcc>(buf[l].res[0], buf[l].res[kFold ? 1 : 0]);
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) s_acc[r * H + slots[l]] = buf[l].res[r];
        }
      }
    __syncthreads();
    // The list (and s_nused) is complete since this barrier: reserve the
    // partition's output range now, so the global atomic's round trip
    // overlaps the repeated-key additions and the next partition's loads.
    u32 n_unique = 0;
    unsigned long long out_base = 0ull;
    if (threadIdx.x == 0) {
      n_unique = s_nused;
      if (n_unique) out_base = atomicAdd(&sc->out_count, (unsigned long long)n_unique);
    }
#pragma unroll
    for (int l = 0; l < LPT; ++l)
      if ((dup_bits >> l) & 1u) {
        if constexpr (kFold) {
          atomicAdd(&s_acc[slots[l]],
                    (unsigned long long)one_plane<kAcc>(buf[l].res[0], buf[l].res[kFold ? 1 : 0]));
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) atomicAdd(&s_acc[r * H + slots[l]], (unsigned long long)buf[l].res[r]);
        }
      }
    // No barrier here: the barrier below orders these additions before
    // compaction.
    if (next < parts) fetch(next, next_cnt);
    if (threadIdx.x == 0) {
      s_n = n_unique;
      s_base = out_base;
      s_nused = 0;
    }
    __syncthreads();
    const u32 n = s_n;
    const unsigned long long base = s_base;
    if constexpr (kRegs) {
#pragma unroll
      for (int l = 0; l < LPT; ++l)
        if ((fresh_bits >> l) & 1u) {
          const u32 slot = slots[l];
          const u64 key = fkey[l];
          const u64 idx = base + fidx[l];
          const bool full = (key & L.mask_of(key)) == L.mask_of(key);
          const bool wr = write_out && idx < out_stride;
          bad |= write_out && !wr;
          if (wr) keys_out[idx] = key;
          if constexpr (kCountNext)
            if (count_next) nterms += next_terms_of(L, key);
          const u64 folded = kFold ? s_acc[slot] : 0ull;
          if constexpr (kAcc == 2) {
            if (wr) {
              res_out[idx] = (u32)folded;
              res_out[out_stride + idx] = (u32)(folded >> 32);
            }
            wsum[0] += folded;
            if (full) fsum[0] += folded;
          } else {
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const u32 v = kFold ? reduce_u64(folded, r) : reduce_sum(s_acc[r * H + slot], r);
              if (wr) res_out[r * out_stride + idx] = v;
              wsum[r] += v;
              if (full) fsum[r] += v;
            }
          }
          s_key[slot] = kEmpty;
          fstates += full;
        }
      (void)n;
      __syncthreads();
      continue;
    }
    for (u32 i = threadIdx.x; i < n; i += BLOCK) {
      const u32 slot = s_list[i];
      const u64 key = s_key[slot];
      const u64 idx = base + i;
      const bool full = (key & L.mask_of(key)) == L.mask_of(key);
      const bool wr = write_out && idx < out_stride;
      bad |= write_out && !wr;
      if (wr) keys_out[idx] = key;
      if constexpr (kCountNext)
        if (count_next) nterms += next_terms_of(L, key);
      const u64 folded = kFold ? s_acc[slot] : 0ull;
      if constexpr (kAcc == 2) {
        if (wr) {
          res_out[idx] = (u32)folded;
          res_out[out_stride + idx] = (u32)(folded >> 32);
        }
        wsum[0] += folded;
        if (full) fsum[0] += folded;
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const u32 v = kFold ? reduce_u64(folded, r) : reduce_sum(s_acc[r * H + slot], r);
          if (wr) res_out[r * out_stride + idx] = v;
          wsum[r] += v;
          if (full) fsum[r] += v;
        }
      }
      s_key[slot] = kEmpty;
      fstates += full;
    }
    __syncthreads();
  }
  if (bad) atomicOr(&sc->error, kErrBounds);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    unsigned long long t = pblock_sum<BLOCK>(wsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->weight_sum[r], t);
    t = pblock_sum<BLOCK>(fsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->final_sum[r], t);
  }
  const unsigned long long t = pblock_sum<BLOCK>(fstates);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->final_states, t);
  if constexpr (kCountNext) {
    if (write_out && count_next) {
      const unsigned long long nt = pblock_sum<BLOCK>(nterms);
      if (threadIdx.x == 0 && nt) atomicAdd(&sc->next_terms, nt);
      if (blockIdx.x == 0 && threadIdx.x == 0) sc->next_terms_ok = 1u;
    }
  }
  if constexpr (Layout::kSlotted) {
    __syncthreads();
    for (int i = threadIdx.x; i < (int)kServeMaxSlots * R; i += BLOCK)
      if (s_slot_fin[i]) atomicAdd(&L.slot_final[(i / R) * 4 + (i % R)], s_slot_fin[i]);
  }
}

// Successor count of a slotted (serving) boundary.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) slot_count_kernel(const u64* __restrict__ keys, u64 n_in, SlotLayout L,
                                                           StepScalars* __restrict__ sc) {
  unsigned long long acc = 0;
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in; i += (u64)gridDim.x * BLOCK) {
    const u64 key = keys[i];
    const State s = L.unpack(key);
    acc += __popcll(~(s.cols | s.dr | s.dl) & L.mask_of(key));
  }
  const unsigned long long t = pblock_sum<BLOCK>(acc);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->terms, t);
}

// ---------------------------------------------------------------------------
// Two-level scatter (scatter_kind 2, 16-byte candidates). The one-level
// scatters store every candidate on its own to a random partition tail (one
// cursor atomic and one scattered 16-byte store each). Here a CTA stages a
// round of up to kTlNC candidates in shared memory, orders them by
// destination, reserves one range per destination with one global atomic and
// writes each destination's candidates as one contiguous run:
//   level 1 (bucket_scatter_kernel): parents -> nb coarse buckets,
//            bucket = partition / p2;
//   level 2 (bucket_split_kernel): each bucket's candidates -> its p2
//            partitions, partition = bucket * p2 + sub-bucket.
// Every candidate ends in partition_of(fib_hash_a(key), parts), the partition
// the one-level scatters give it, so the merge is unchanged. Capacity rules
// are the same: a bucket or partition never receives more than it holds, and
// the error word is set instead.
// Measured on GB300, exact Q(18) with the default tuning otherwise: level 1 +
// level 2 take 661 ms against the window scatter's 605 ms (Q(17): 54 + 35 ms
// against 80 ms). The two staging passes move every candidate twice at about
// 2.8 TB/s, which costs more than the scattered stores they replace; the
// window scatter stays the default and this one is a tuning choice.

constexpr int kTlMaxBins = 1024;  // nb and p2 limit
constexpr int kTlPPT = 2;         // level 1: parents per thread per chunk

// CTA shape: BLOCK threads stage kNC candidates a round, kMinBlocks CTAs
// per SM. (One 1024-thread CTA per SM staging 6144 candidates measured
// slower: its phases cannot overlap.)
template <int BLOCK>
struct TlShape;
template <>
struct TlShape<512> {
  static constexpr int kNC = 2560, kMinBlocks = 2;
};
constexpr int kTlBlock = 512;

template <int R, int BLOCK>
constexpr size_t tl_smem() {
  // staged (generation order) + staged (destination order) + destination of
  // each ordered slot + per-bin count, offset and reserved base
  return (size_t)TlShape<BLOCK>::kNC * (sizeof(Cand<R>) * 2 + 2) + (size_t)kTlMaxBins * 4 * 3;
}

// Exclusive scan of one u32 per thread over a BLOCK-thread CTA; *total
// receives the sum. Contains two barriers.
template <int BLOCK>
__device__ __forceinline__ u32 tl_block_scan(u32 v, u32* s_warp, u32* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  u32 incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const u32 t = __shfl_up_sync(kFullMask, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const u32 w = lane < BLOCK / 32 ? s_warp[lane] : 0u;
    u32 wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const u32 t = __shfl_up_sync(kFullMask, wi, d);
      if (lane >= d) wi += t;
    }
    s_warp[lane] = wi - w;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  return s_warp[wid] + incl - v;
}

// Order the m staged candidates by bin (fetch_of(k, i) is candidate
// i = k * BLOCK + tid, with bin[k] and rank[k]), reserve each bin's range with one atomic on
// cursors[bin_cursor(bin)], and write the runs to dst(bin) + base + rank.
// Shared by both levels; ends with a barrier, after which s_a, s_b and the
// bin arrays may be reused.
template <int R, int BLOCK, int PER, typename FetchOf, typename CursorOf, typename DestOf>
__device__ __forceinline__ void tl_order_and_write(FetchOf fetch_of, Cand<R>* s_b, unsigned short* s_bin, u32* s_cnt,
                                                   u32* s_off, u32* s_base, u32* s_warp, u32* s_total, u32 m,
                                                   u32 nbins, const u32 (&bin)[PER], const u32 (&rank)[PER],
                                                   CursorOf cursor_of, DestOf dest_of, u64 cap, u64 policy,
                                                   bool& overflow) {
  const int tid = threadIdx.x;
  __syncthreads();  // every rank is taken
  // Bins are dealt to threads in blocks of kTlMaxBins / BLOCK consecutive
  // bins, so the scan order is the bin order.
  constexpr int BPT = kTlMaxBins / BLOCK;
  static_assert(kTlMaxBins % BLOCK == 0, "bins per thread");
  u32 c[BPT];
  u32 mine = 0;
#pragma unroll
  for (int q = 0; q < BPT; ++q) {
    const u32 bn = (u32)tid * BPT + q;
    c[q] = bn < nbins ? s_cnt[bn] : 0u;
    mine += c[q];
  }
  u32 off = tl_block_scan<BLOCK>(mine, s_warp, s_total);
#pragma unroll
  for (int q = 0; q < BPT; ++q) {
    const u32 bn = (u32)tid * BPT + q;
    if (bn < nbins) {
      s_off[bn] = off;
      if (c[q]) s_base[bn] = atomicAdd(cursor_of(bn), c[q]);
      off += c[q];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const u32 i = (u32)k * BLOCK + tid;
    if (i < m) {
      const u32 j = s_off[bin[k]] + rank[k];
      s_b[j] = fetch_of(k, i);
      s_bin[j] = (unsigned short)bin[k];
    }
  }
  __syncthreads();
  for (u32 j = tid; j < m; j += BLOCK) {
    const u32 b = s_bin[j];
    const u64 pos = (u64)s_base[b] + (j - s_off[b]);
    if (pos < cap)
      store_cand_keep<R>(dest_of(b) + pos, s_b[j], policy);
    else
      overflow = true;
  }
  __syncthreads();
}

// Level 1. Parents stream through each CTA in chunks of kTlPPT * BLOCK (the
// next chunk is loaded into registers while the current one is staged); a
// chunk's successors, flattened in parent order and lowest free column first,
// fill rounds of exactly kNC staged candidates across chunk boundaries (only
// the CTA's last round is partial).
template <int R, int BLOCK, typename Layout>
__global__ void __launch_bounds__(BLOCK, TlShape<BLOCK>::kMinBlocks) bucket_scatter_kernel(
    const u64* __restrict__ keys, const u32* __restrict__ res, u64 res_stride, u64 n_in, Layout L,
    Cand<R>* __restrict__ buckets, u64 bcap, u32* __restrict__ bcur, u32 nb, u32 parts, u32 p2,
    StepScalars* __restrict__ sc) {
  constexpr int kTlNC = TlShape<BLOCK>::kNC, kTlPer = kTlNC / BLOCK;
  static_assert(kTlNC % BLOCK == 0, "two-level shape");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cand<R>* s_a = reinterpret_cast<Cand<R>*>(smem_raw);
  Cand<R>* s_b = s_a + kTlNC;
  unsigned short* s_bin = reinterpret_cast<unsigned short*>(s_b + kTlNC);
  u32* s_cnt = reinterpret_cast<u32*>(s_bin + kTlNC);
  u32* s_off = s_cnt + kTlMaxBins;
  u32* s_base = s_off + kTlMaxBins;
  __shared__ u32 s_warp[32];
  __shared__ u32 s_total;
  const int tid = threadIdx.x;
  constexpr u64 CP = (u64)kTlPPT * BLOCK;
  const u64 stride = (u64)gridDim.x * CP;
  const u64 policy = l2_keep_policy();
  bool overflow = false;

  // Current chunk (free masks computed) and the next one (raw, in flight).
  u64 ck[kTlPPT], cf[kTlPPT], nk[kTlPPT];
  u32 cw[kTlPPT][R], nw[kTlPPT][R];
  auto prefetch = [&](u64 base) {
#pragma unroll
    for (int q = 0; q < kTlPPT; ++q) {
      const u64 i = base + (u64)q * BLOCK + tid;
      nk[q] = kEmptyKey;
      if (i < n_in) {
        nk[q] = __ldcs(keys + i);
#pragma unroll
        for (int r = 0; r < R; ++r) nw[q][r] = __ldcs(res + r * res_stride + i);
      }
    }
  };
  u64 next_base = (u64)blockIdx.x * CP;
  bool more = next_base < n_in;  // a loaded chunk is waiting (uniform over the CTA)
  if (more) prefetch(next_base);
  u32 first = 0, total = 0, r0 = 0;  // this thread's first successor index; chunk total; consumed
  // Make the waiting chunk current and start loading the one after it.
  // Uniform; two barriers (the scan).
  auto advance = [&]() {
    u32 cnt = 0;
#pragma unroll
    for (int q = 0; q < kTlPPT; ++q) {
      ck[q] = nk[q];
#pragma unroll
      for (int r = 0; r < R; ++r) cw[q][r] = nw[q][r];
      cf[q] = 0;
      if (ck[q] != kEmptyKey) {
        const State s = L.unpack(ck[q]);
        cf[q] = ~(s.cols | s.dr | s.dl) & L.mask_of(ck[q]);
      }
      cnt += (u32)__popcll(cf[q]);
    }
    next_base += stride;
    more = next_base < n_in;
    if (more) prefetch(next_base);
    first = tl_block_scan<BLOCK>(cnt, s_warp, &s_total);
    total = s_total;
    r0 = 0;
  };
  // Stage successors [lo, lo + take) of the current chunk at s_a[at, at + take).
  auto stage = [&](u32 lo, u32 take, u32 at) {
    u32 g = first;
#pragma unroll
    for (int q = 0; q < kTlPPT; ++q) {
      const u32 c = (u32)__popcll(cf[q]);
      if (c && g + c > lo && g < lo + take) {
        const State s = L.unpack(ck[q]);
        u64 f = cf[q];
        u32 j = g;
        while (f) {
          const u64 b = f & (0ull - f);
          f ^= b;
          if (j >= lo && j < lo + take) {
            Cand<R> cd;
            cd.key = L.successor(ck[q], s, b);
#pragma unroll
            for (int r = 0; r < R; ++r) cd.res[r] = cw[q][r];
            s_a[at + (j - lo)] = cd;
          }
          ++j;
        }
      }
      g += c;
    }
  };
  for (;;) {
    u32 m = 0;  // staged this round (uniform)
    for (;;) {
      if (r0 == total) {
        if (!more) break;
        advance();
        continue;
      }
      const u32 take = min(total - r0, (u32)kTlNC - m);
      stage(r0, take, m);
      m += take;
      r0 += take;
      if (m == (u32)kTlNC) break;
    }
    if (m == 0) break;
    for (u32 i = tid; i < nb; i += BLOCK) s_cnt[i] = 0u;
    __syncthreads();  // staged candidates and cleared counts
    u32 bin[kTlPer], rank[kTlPer];
#pragma unroll
    for (int k = 0; k < kTlPer; ++k) {
      const u32 i = (u32)k * BLOCK + tid;
      bin[k] = 0;
      rank[k] = 0;
      if (i < m) {
        bin[k] = partition_of(fib_hash_a(s_a[i].key), parts) / p2;
        if (bin[k] >= nb) {  // cannot happen (parts = nb * p2); kept off shared memory all the same
          bin[k] = 0;
          overflow = true;
        }
        rank[k] = atomicAdd(&s_cnt[bin[k]], 1u);
      }
    }
    tl_order_and_write<R, BLOCK, kTlPer>(
        [&](int, u32 i) { return s_a[i]; }, s_b, s_bin, s_cnt, s_off, s_base, s_warp, &s_total, m, nb, bin, rank,
        [&](u32 b) { return bcur + b; }, [&](u32 b) { return buckets + (u64)b * bcap; }, bcap, policy, overflow);
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

// Level 2. Work item = (bucket, chunk of kNC candidates); the candidates
// stay in registers until they are ordered.
template <int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK, TlShape<BLOCK>::kMinBlocks) bucket_split_kernel(const Cand<R>* __restrict__ buckets, u64 bcap,
                                                                   const u32* __restrict__ bcur, u32 nb,
                                                                   u32 chunks_per_bucket, u32 parts, u32 p2,
                                                                   Cand<R>* __restrict__ regions, u32 cap,
                                                                   u32* __restrict__ cursors, u32 cstride,
                                                                   StepScalars* __restrict__ sc) {
  constexpr int kTlNC = TlShape<BLOCK>::kNC, kTlPer = kTlNC / BLOCK;
  static_assert(kTlNC % BLOCK == 0, "two-level shape");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cand<R>* s_b = reinterpret_cast<Cand<R>*>(smem_raw) + kTlNC;  // same layout as level 1
  unsigned short* s_bin = reinterpret_cast<unsigned short*>(s_b + kTlNC);
  u32* s_cnt = reinterpret_cast<u32*>(s_bin + kTlNC);
  u32* s_off = s_cnt + kTlMaxBins;
  u32* s_base = s_off + kTlMaxBins;
  __shared__ u32 s_warp[32];
  __shared__ u32 s_total;
  const int tid = threadIdx.x;
  const u64 policy = l2_keep_policy();
  bool overflow = false;
  const u64 items = (u64)nb * chunks_per_bucket;
  for (u64 it = blockIdx.x; it < items; it += gridDim.x) {
    const u32 b = (u32)(it / chunks_per_bucket);
    const u64 lo = (it % chunks_per_bucket) * (u64)kTlNC;
    const u64 nbk = min((u64)bcur[b], bcap);
    if (lo >= nbk) continue;  // uniform over the CTA
    const u32 m = (u32)min(nbk - lo, (u64)kTlNC);
    for (u32 i = tid; i < p2; i += BLOCK) s_cnt[i] = 0u;
    const Cand<R>* src = buckets + (u64)b * bcap + lo;
    Cand<R> c[kTlPer];
#pragma unroll
    for (int k = 0; k < kTlPer; ++k) {
      const u32 i = (u32)k * BLOCK + tid;
      if (i < m) c[k] = load_cand<R>(src + i);
    }
    __syncthreads();  // cleared counts
    u32 bin[kTlPer], rank[kTlPer];
#pragma unroll
    for (int k = 0; k < kTlPer; ++k) {
      const u32 i = (u32)k * BLOCK + tid;
      bin[k] = 0;
      rank[k] = 0;
      if (i < m) {
        bin[k] = partition_of(fib_hash_a(c[k].key), parts) - b * p2;
        if (bin[k] >= p2) {  // not this bucket's: cannot happen; flag it rather than index past the bins
          bin[k] = 0;
          overflow = true;
        }
        rank[k] = atomicAdd(&s_cnt[bin[k]], 1u);
      }
    }
    tl_order_and_write<R, BLOCK, kTlPer>(
        [&](int k, u32) { return c[k]; }, s_b, s_bin, s_cnt, s_off, s_base, s_warp, &s_total, m, p2, bin, rank,
        [&](u32 s) { return cursors + (u64)(b * p2 + s) * cstride; },
        [&](u32 s) { return regions + (u64)(b * p2 + s) * cap; }, (u64)cap, policy, overflow);
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

template <int R, int BLOCK, typename Layout>
cudaError_t two_level_scatter(const PartitionCfg& pc, const FrontierView& in, u64 n_in, Layout L, void* regions,
                              u32* cursors, StepScalars* sc, cudaStream_t stream) {
  char* area = reinterpret_cast<char*>(cursors) + two_level_cursor_bytes(pc);
  u32* bcur = reinterpret_cast<u32*>(area);
  Cand<R>* buckets = reinterpret_cast<Cand<R>*>(area + (((size_t)pc.tl_nb * 4 + 255) / 256) * 256);
  cudaError_t e = cudaMemsetAsync(bcur, 0, (size_t)pc.tl_nb * 4, stream);
  if (e != cudaSuccess) return e;
  constexpr int kTlNC = TlShape<BLOCK>::kNC, kMinBlocks = TlShape<BLOCK>::kMinBlocks;
  constexpr size_t smem = tl_smem<R, BLOCK>();
  auto k1 = bucket_scatter_kernel<R, BLOCK, Layout>;
  auto k2 = bucket_split_kernel<R, BLOCK>;
  if ((e = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) return e;
  const u64 chunks1 = (n_in + (u64)kTlPPT * BLOCK - 1) / ((u64)kTlPPT * BLOCK);
  const unsigned g1 = (unsigned)std::max<u64>(1, std::min<u64>(chunks1, (u64)pc.sms * kMinBlocks));
  k1<<<g1, BLOCK, smem, stream>>>(reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_in, L, buckets,
                                     pc.tl_bcap, bcur, pc.tl_nb, pc.parts, pc.tl_p2, sc);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const u32 cpb = (u32)((pc.tl_bcap + kTlNC - 1) / kTlNC);
  const u64 items = (u64)pc.tl_nb * cpb;
  const unsigned g2 = (unsigned)std::max<u64>(1, std::min<u64>(items, (u64)pc.sms * kMinBlocks));
  k2<<<g2, BLOCK, smem, stream>>>(buckets, pc.tl_bcap, bcur, pc.tl_nb, cpb, pc.parts, pc.tl_p2,
                                     reinterpret_cast<Cand<R>*>(regions), pc.cap, cursors,
                                     pc.cursor_stride ? pc.cursor_stride : 1, sc);
  return cudaGetLastError();
}

constexpr int kScatterBlock = 256;
// Merge CTA shapes: table slots H, candidate capacity H / 2.
constexpr int kMergeBlock = 512, kMergeH = 4096;
constexpr int kWideBlock = 1024, kWideH = 8192;
constexpr int kSmallBlock = 256, kSmallH = 2048;  // four CTAs per SM

template <int R, int H>
constexpr size_t merge_smem() {
  return (size_t)H * (8 + 8 * R);
}

template <int R, int PPL, int BLOCK, typename Layout>
cudaError_t scatter_shape(const PartitionCfg& pc, const FrontierView& in, u64 n_in, Layout L, void* regions,
                          u32* cursors, StepScalars* sc, cudaStream_t stream) {
  u64 want = (n_in + BLOCK * PPL - 1) / (BLOCK * PPL);
  const u64 capb = (u64)pc.sms * 8 * 256 / BLOCK;  // the same resident threads per SM for every block size
  const unsigned grid = (unsigned)std::max<u64>(1, std::min(want, capb));
  const u32 cstride = pc.cursor_stride ? pc.cursor_stride : 1;
  if (pc.scatter_kind == 4) {
    partition_scatter_direct_kernel<R, BLOCK, PPL, Layout><<<grid, BLOCK, 0, stream>>>(
        reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_in, L, reinterpret_cast<Cand<R>*>(regions), cursors,
        cstride, pc.parts, pc.cap, sc);
    return cudaGetLastError();
  }
  if (pc.scatter_kind != 0) {  // 2 without a two-level plan, or 3 where it does not apply: the window scatter
    partition_scatter_list_kernel<R, BLOCK, PPL, Layout><<<grid, BLOCK, 0, stream>>>(
        reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_in, L, reinterpret_cast<Cand<R>*>(regions), cursors,
        cstride, pc.parts, pc.cap, sc);
    return cudaGetLastError();
  }
  partition_scatter_kernel<R, BLOCK, PPL, Layout><<<grid, BLOCK, 0, stream>>>(
      reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_in, L, reinterpret_cast<Cand<R>*>(regions), cursors,
      cstride, pc.parts, pc.cap, sc);
  return cudaGetLastError();
}

// Block sizes 128 and 512 are instantiated for 16-byte candidates (R <= 2);
// wider candidates use 256.
template <int R, int PPL, typename Layout>
cudaError_t scatter_ppl(const PartitionCfg& pc, const FrontierView& in, u64 n_in, Layout L, void* regions,
                        u32* cursors, StepScalars* sc, cudaStream_t stream) {
  if constexpr (R <= 2) {
    if (pc.scatter_block == 128) return scatter_shape<R, PPL, 128, Layout>(pc, in, n_in, L, regions, cursors, sc, stream);
    if (pc.scatter_block == 512) return scatter_shape<R, PPL, 512, Layout>(pc, in, n_in, L, regions, cursors, sc, stream);
  }
  return scatter_shape<R, PPL, kScatterBlock, Layout>(pc, in, n_in, L, regions, cursors, sc, stream);
}

template <int R, typename Layout>
cudaError_t scatter_impl(const PartitionCfg& pc, const FrontierView& in, u64 n_in, Layout L, void* regions,
                         u32* cursors, StepScalars* sc, cudaStream_t stream) {
  if (pc.parents_per_lane == 4) return scatter_ppl<R, 4, Layout>(pc, in, n_in, L, regions, cursors, sc, stream);
  return scatter_ppl<R, 2, Layout>(pc, in, n_in, L, regions, cursors, sc, stream);
}

template <int R, int BLOCK, int H, typename Layout>
cudaError_t merge_shape(const PartitionCfg& pc, int blocks_per_sm, const void* regions, const u32* cursors,
                        const FrontierView& out, Layout L, bool write_out, StepScalars* sc, cudaStream_t stream) {
  if (pc.cap != (u32)(H / 2)) return cudaErrorInvalidValue;
  const bool fold = R == 2 && pc.merge_kind == 1 && pc.fold;
  const bool exact = fold && pc.fold == 2;
  if (pc.fold == 2 && !exact) return cudaErrorInvalidValue;  // exact words need the claim-list merge
  if constexpr (Layout::kSlotted)
    if (exact) return cudaErrorInvalidValue;
  constexpr bool kRegsOk = !Layout::kSlotted;
  const bool regs = kRegsOk && pc.merge_regs;
  auto kern = fold ? (exact ? (regs ? partition_merge_list_kernel<R, BLOCK, H, H / 2, Layout,
                                                                  (R == 2 && !Layout::kSlotted) ? 2 : 0, kRegsOk>
                                    : partition_merge_list_kernel<R, BLOCK, H, H / 2, Layout,
                                                                  (R == 2 && !Layout::kSlotted) ? 2 : 0>)
                            : (regs ? partition_merge_list_kernel<R, BLOCK, H, H / 2, Layout, R == 2 ? 1 : 0, kRegsOk>
                                    : partition_merge_list_kernel<R, BLOCK, H, H / 2, Layout, R == 2 ? 1 : 0>))
                   : pc.merge_kind == 1 ? (regs ? partition_merge_list_kernel<R, BLOCK, H, H / 2, Layout, 0, kRegsOk>
                                                : partition_merge_list_kernel<R, BLOCK, H, H / 2, Layout>)
                                        : partition_merge_kernel<R, BLOCK, H, H / 2, Layout>;
  const size_t smem = fold ? merge_smem<1, H>() + (size_t)(H / 2) * 4
                           : merge_smem<R, H>() + (pc.merge_kind == 1 ? (size_t)(H / 2) * 4 : 0);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const u64 capb = (u64)pc.sms * blocks_per_sm;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(pc.parts, capb));
  kern<<<grid, BLOCK, smem, stream>>>(reinterpret_cast<const Cand<R>*>(regions), cursors,
                                      pc.cursor_stride ? pc.cursor_stride : 1, pc.parts,
                                      reinterpret_cast<u64*>(out.keys), out.res, out.cap, L,
                                      (write_out ? 1 : 0) | (pc.count_next ? 2 : 0), sc);
  return cudaGetLastError();
}

template <int R, typename Layout>
cudaError_t merge_impl(const PartitionCfg& pc, const void* regions, const u32* cursors, const FrontierView& out,
                       Layout L, bool write_out, StepScalars* sc, cudaStream_t stream) {
  if constexpr (R <= 2) {
    if (pc.wide == 2)
      return merge_shape<R, kSmallBlock, kSmallH, Layout>(pc, 4, regions, cursors, out, L, write_out, sc, stream);
    if (pc.wide)
      return merge_shape<R, kWideBlock, kWideH, Layout>(pc, 1, regions, cursors, out, L, write_out, sc, stream);
  } else {
    if (pc.wide) return cudaErrorInvalidValue;
  }
  return merge_shape<R, kMergeBlock, kMergeH, Layout>(pc, pc.merge_blocks_per_sm, regions, cursors, out, L,
                                                      write_out, sc, stream);
}

}  // namespace

size_t candidate_bytes(int residues) { return residues <= 2 ? 16 : 32; }

cudaError_t launch_serve_count(const FrontierView& in, uint64_t n_in, const uint64_t* slot_mask, StepScalars* sc,
                               int sms, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  const u64 want = (n_in + 1023) / 1024;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)sms * 8));
  slot_count_kernel<256><<<grid, 256, 0, stream>>>(reinterpret_cast<const u64*>(in.keys), n_in,
                                                   SlotLayout{slot_mask, nullptr}, sc);
  return cudaGetLastError();
}

cudaError_t launch_serve_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in,
                                 const uint64_t* slot_mask, void* regions, uint32_t* cursors, StepScalars* sc,
                                 cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (pc.residues != 2) return cudaErrorInvalidValue;
  return scatter_impl<2>(pc, in, n_in, SlotLayout{slot_mask, nullptr}, regions, cursors, sc, stream);
}

cudaError_t launch_serve_merge(const PartitionCfg& pc, const void* regions, const uint32_t* cursors,
                               const FrontierView& out, const uint64_t* slot_mask, unsigned long long* slot_final,
                               StepScalars* sc, cudaStream_t stream) {
  if (pc.residues != 2) return cudaErrorInvalidValue;
  return merge_impl<2>(pc, regions, cursors, out, SlotLayout{slot_mask, slot_final}, true, sc, stream);
}
uint32_t partition_capacity(uint32_t wide) { return wide == 2 ? kSmallH / 2 : wide ? kWideH / 2 : kMergeH / 2; }
bool wide_merge_supported(int residues) { return residues >= 1 && residues <= 2; }

size_t two_level_cursor_bytes(const PartitionCfg& pc) {
  return ((size_t)pc.parts * 4 * (pc.cursor_stride ? pc.cursor_stride : 1) + 255) / 256 * 256;
}

size_t two_level_extra_bytes(const PartitionCfg& pc) {
  return ((size_t)pc.tl_nb * 4 + 255) / 256 * 256 + (size_t)pc.tl_nb * pc.tl_bcap * 16;
}

bool two_level_plan(uint64_t terms, uint32_t parts, int residues, PartitionCfg* pc) {
  if (residues > 2 || terms == 0 || parts == 0 || (u64)parts > (u64)kTlMaxBins * kTlMaxBins) return false;
  u64 nb = (u64)std::llround(std::sqrt((double)parts));
  nb = std::min<u64>(std::max<u64>(nb, 1), kTlMaxBins);
  u64 p2 = (parts + nb - 1) / nb;
  if (p2 > (u64)kTlMaxBins) {
    nb = (parts + kTlMaxBins - 1) / kTlMaxBins;
    p2 = (parts + nb - 1) / nb;
  }
  if (nb > (u64)kTlMaxBins || p2 > (u64)kTlMaxBins) return false;
  // Hash buckets: mean terms / nb, standard deviation about its square root.
  const double mean = (double)terms / (double)nb;
  const u64 bcap = (u64)(mean * 1.01 + 8.0 * std::sqrt(mean)) + 1024;
  if (bcap >= 0xffffffffull) return false;  // bucket cursors are u32
  pc->tl_nb = (u32)nb;
  pc->tl_p2 = (u32)p2;
  pc->tl_bcap = bcap;
  pc->parts = (u32)(nb * p2);
  return true;
}

cudaError_t launch_partition_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in, unsigned n,
                                     void* regions, uint32_t* cursors, StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (n_in > in.cap) return cudaErrorInvalidValue;
  if (pc.key_bits == 128) return launch_wide_partition_scatter(pc, in, n_in, n, regions, cursors, sc, stream);
  if (pc.tl_nb) {
    if (pc.tl_nb > (u32)kTlMaxBins || pc.tl_p2 > (u32)kTlMaxBins || pc.parts != pc.tl_nb * pc.tl_p2)
      return cudaErrorInvalidValue;
    const FixedLayout L{n, pboard_mask_host(n)};
    if (pc.residues == 1) return two_level_scatter<1, kTlBlock>(pc, in, n_in, L, regions, cursors, sc, stream);
    if (pc.residues == 2) return two_level_scatter<2, kTlBlock>(pc, in, n_in, L, regions, cursors, sc, stream);
    return cudaErrorInvalidValue;
  }
  switch (pc.residues) {
    case 1: return scatter_impl<1>(pc, in, n_in, FixedLayout{n, pboard_mask_host(n)}, regions, cursors, sc, stream);
    case 2: return scatter_impl<2>(pc, in, n_in, FixedLayout{n, pboard_mask_host(n)}, regions, cursors, sc, stream);
    case 3: return scatter_impl<3>(pc, in, n_in, FixedLayout{n, pboard_mask_host(n)}, regions, cursors, sc, stream);
    case 4: return scatter_impl<4>(pc, in, n_in, FixedLayout{n, pboard_mask_host(n)}, regions, cursors, sc, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_partition_merge(const PartitionCfg& pc, const void* regions, const uint32_t* cursors,
                                   const FrontierView& out, unsigned n, bool write_out, StepScalars* sc,
                                   cudaStream_t stream) {
  if (pc.key_bits == 128) return launch_wide_partition_merge(pc, regions, cursors, out, n, write_out, sc, stream);
  switch (pc.residues) {
    case 1: return merge_impl<1>(pc, regions, cursors, out, FixedLayout{n, pboard_mask_host(n)}, write_out, sc, stream);
    case 2: return merge_impl<2>(pc, regions, cursors, out, FixedLayout{n, pboard_mask_host(n)}, write_out, sc, stream);
    case 3: return merge_impl<3>(pc, regions, cursors, out, FixedLayout{n, pboard_mask_host(n)}, write_out, sc, stream);
    case 4: return merge_impl<4>(pc, regions, cursors, out, FixedLayout{n, pboard_mask_host(n)}, write_out, sc, stream);
  }
  return cudaErrorInvalidValue;
}

static_assert(sizeof(Cand<1>) == 16 && sizeof(Cand<2>) == 16 && sizeof(Cand<3>) == 32 && sizeof(Cand<4>) == 32,
              "candidate sizes must match candidate_bytes()");

}  // namespace qpeps

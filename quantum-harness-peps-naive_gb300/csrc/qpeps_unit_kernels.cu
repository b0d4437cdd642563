// Class-grouped partitions for the partitioned merge (scatter_kind 3).
//
// The one-level scatters store every successor candidate on its own into a
// hash partition drawn uniformly from all P partitions: one scattered 16-byte
// store per candidate, which bounds them at about 42 G candidates/s on GB300.
// Here the partition of a candidate is a function of its *class*: the columns
// it has filled and a window of its outermost diagonal signals,
//
//   class = (cols, pairs 0..t-1),  pair i = (diag_dr bit n-1-i, diag_dl bit i).
//
// A row step moves every diagonal signal one column towards the board edge it
// runs to, so the successor's pair i is the parent's pair i+1 (or the placed
// queen's bit) and the parent's pair 0 leaves the board. So all successors of
// one parent class fall into 4 x (free columns) classes (the parent's pair t
// is the one unknown), and a CTA that expands a few
// boundary partitions (each one or a few classes) produces runs of candidates
// for a few dozen partitions instead of one candidate for each of thousands.
// The CTA stages a round of successors in shared memory, orders them by
// destination partition, reserves each partition's run with one cursor atomic
// and writes the runs coalesced.
//
// Classes are hashed into 2^lg buckets: bucket = H(cols, pairs 1..t-1) * 4 +
// pair 0, so the four classes that differ only in pair 0 (which a row step
// drops, so their successors share every destination) sit in consecutive
// buckets. A sampled histogram (parents whose key hash falls in the lowest
// 1/sample of its range) estimates each bucket's candidates, and a plan packs runs of small consecutive buckets
// into one partition ("unit") and gives a large bucket its own units (its
// candidates split between them by a hash of the key). Each unit is a fixed
// region of `cap` candidate slots; a unit the estimate undersized overflows,
// which the merge detects (it then writes nothing) and the engine retries
// the row with more units.
//
// Every candidate still lands in exactly one unit that is a function of its
// key, so equal keys meet in one merge partition; the merge kernels are the
// ones of the hash partitions.
#include <cuda_runtime.h>

#include <algorithm>

#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {

namespace {

constexpr u32 kFull = 0xffffffffu;
constexpr u64 kNoKey = ~0ull;

__device__ __forceinline__ u64 ubucket_of(u64 key, const UnitClassPlan& c) {
  const u64 mask = (1ull << c.n) - 1;
  const u64 cols = key & mask;
  if (c.t == 0) return mix64(cols) >> (64 - c.lg);
  const u64 dr = (key >> c.n) & mask, dl = (key >> (2 * c.n)) & mask;
  const u64 wm = (1ull << (c.t - 1)) - 1;
  const u64 rest = cols | (((dr >> (c.n - c.t)) & wm) << c.n) | (((dl >> 1) & wm) << (c.n + c.t - 1));
  const u64 p0 = ((dr >> (c.n - 1)) & 1ull) | ((dl & 1ull) << 1);
  return ((mix64(rest) >> (64 - (c.lg - 2))) << 2) | p0;
}

// Unit of a candidate from its bucket's plan entry {base, m}.
__device__ __forceinline__ u32 unit_of(u64 key, uint2 e) {
  if (e.y <= 1) return e.x;
  return e.x + (u32)(((fib_hash_a(key) >> 32) * (u64)e.y) >> 32);
}

template <int BLOCK>
__device__ __forceinline__ void block_incl_scan_u64(u64& v, u64* s_warp) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const u64 t = __shfl_up_sync(kFull, v, d);
    if (lane >= d) v += t;
  }
  if (lane == 31) s_warp[wid] = v;
  __syncthreads();
  if (wid == 0) {
    u64 w = lane < BLOCK / 32 ? s_warp[lane] : 0ull;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const u64 t = __shfl_up_sync(kFull, w, d);
      if (lane >= d) w += t;
    }
    if (lane < BLOCK / 32) s_warp[lane] = w;
  }
  __syncthreads();
  if (wid > 0) v += s_warp[wid - 1];
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Sampled histogram: a parent is sampled when a hash of its key falls in the
// lowest 1/sample of its range (sample a power of two), so the sample, and
// with it the plan, depends only on the boundary's keys and not on their order
// in memory (the merge writes its partitions in a nondeterministic order, and
// a CUDA-graph replay must rebuild the recorded plan). Every successor of a
// sampled parent adds one to its bucket. Counts are aggregated per CTA in a
// small shared-memory table, flushed when it fills.

constexpr int kHistSlots = 2048;

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) unit_hist_kernel(const u64* __restrict__ keys, u64 n_in,
                                                          UnitClassPlan c, u32 sample_shift, u32* __restrict__ hist) {
  __shared__ u32 s_key[kHistSlots];
  __shared__ u32 s_cnt[kHistSlots];
  __shared__ u32 s_used;
  for (int i = threadIdx.x; i < kHistSlots; i += BLOCK) {
    s_key[i] = kFull;
    s_cnt[i] = 0;
  }
  if (threadIdx.x == 0) s_used = 0;
  __syncthreads();
  const u64 mask = (1ull << c.n) - 1;
  const u64 stride = (u64)gridDim.x * BLOCK;
  const u64 n_round = (n_in + stride - 1) / stride * stride;  // uniform trip count (barriers inside)
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_round; i += stride) {
    if (i < n_in) {
      const u64 key = __ldcs(keys + i);
      if (sample_shift == 0 || (fib_hash_b(key) >> (64 - sample_shift)) == 0) {
        const State s = unpack<u64>(key, c.n, mask);
        u64 fr = ~(s.cols | s.dr | s.dl) & mask;
        while (fr) {
          const u64 b = fr & (0ull - fr);
          fr ^= b;
          const u32 bk = (u32)ubucket_of(row_successor<u64>(s, b, c.n, mask), c);
          u32 slot = (bk * 0x9E3779B1u) >> (32 - 11);
          bool done = false;
          for (int p = 0; p < 16; ++p) {
            const u32 cur = atomicCAS(&s_key[slot], kFull, bk);
            if (cur == kFull || cur == bk) {
              if (cur == kFull) atomicAdd(&s_used, 1u);
              atomicAdd(&s_cnt[slot], 1u);
              done = true;
              break;
            }
            slot = (slot + 1) & (kHistSlots - 1);
          }
          if (!done) atomicAdd(&hist[bk], 1u);
        }
      }
    }
    __syncthreads();
    const bool last = i + stride >= n_round;
    if (s_used > kHistSlots / 2 || last) {
      for (int k = threadIdx.x; k < kHistSlots; k += BLOCK) {
        if (s_key[k] != kFull) {
          atomicAdd(&hist[s_key[k]], s_cnt[k]);
          s_key[k] = kFull;
          s_cnt[k] = 0;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) s_used = 0;
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Plan. Per bucket, estimated candidates e = sample * count + sample / 2
// (an unsampled bucket still gets a share; at least 1). Small buckets
// (e <= target / 2) are packed in bucket order: unit = floor(prefix of small
// e / target). Larger ones get m = e / target (rounded, at least 1) units of
// their own after all packed units. Three kernels: per-block sums, one CTA scanning the block sums, and
// the per-bucket table.

constexpr int kPlanBlock = 512;

// Every small bucket weighs at least 1, so the exclusive prefix of each one
// stays below the total and its unit below the packed-unit count. A packed
// unit's estimate stays below 1.5 target (its last bucket is at most half a
// target), and so does a large bucket's share (m = e / target rounded).
__device__ __forceinline__ void plan_split(u32 h, const UnitPlanArgs& a, u64& small_e, u64& own) {
  const u64 e = (u64)h * a.sample + (a.sample > 1 ? a.sample / 2 : 1);
  if (e * 2 <= a.target) {
    small_e = e;
    own = 0;
  } else {
    small_e = 0;
    own = std::min<u64>(std::max<u64>(1, (2 * e + a.target) / (2 * a.target)), 1ull << 20);
  }
}

__global__ void __launch_bounds__(kPlanBlock) unit_plan_sums_kernel(const u32* __restrict__ hist, UnitPlanArgs a,
                                                                    u64* __restrict__ block_small,
                                                                    u64* __restrict__ block_own) {
  __shared__ u64 s_warp[kPlanBlock / 32];
  const u64 nb = 1ull << a.lg;
  const u64 b = (u64)blockIdx.x * kPlanBlock + threadIdx.x;
  u64 se = 0, own = 0;
  if (b < nb) plan_split(hist[b], a, se, own);
  block_incl_scan_u64<kPlanBlock>(se, s_warp);
  block_incl_scan_u64<kPlanBlock>(own, s_warp);
  if (threadIdx.x == kPlanBlock - 1) {
    block_small[blockIdx.x] = se;
    block_own[blockIdx.x] = own;
  }
}

// One CTA: exclusive scans of the block sums (in place) and the totals.
__global__ void __launch_bounds__(1024) unit_plan_scan_kernel(u64* __restrict__ block_small, u64* __restrict__ block_own,
                                                              u32 nblocks, UnitPlanArgs a, UnitPlanTotals* __restrict__ tot,
                                                              StepScalars* __restrict__ sc) {
  __shared__ u64 s_warp[32];
  u64 carry_s = 0, carry_o = 0;
  for (u32 base = 0; base < nblocks; base += 1024) {
    const u32 i = base + threadIdx.x;
    u64 vs = i < nblocks ? block_small[i] : 0ull, vo = i < nblocks ? block_own[i] : 0ull;
    const u64 xs = vs, xo = vo;
    block_incl_scan_u64<1024>(vs, s_warp);
    block_incl_scan_u64<1024>(vo, s_warp);
    if (i < nblocks) {
      block_small[i] = carry_s + vs - xs;
      block_own[i] = carry_o + vo - xo;
    }
    __shared__ u64 s_last[2];
    if (threadIdx.x == 1023) {
      s_last[0] = vs;
      s_last[1] = vo;
    }
    __syncthreads();
    carry_s += s_last[0];
    carry_o += s_last[1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const u64 small_units = carry_s ? (carry_s - 1) / a.target + 1 : 0;
    tot->small_units = small_units;
    tot->units = small_units + carry_o;
    tot->small_e = carry_s;
    if (sc) sc->plan_units = small_units + carry_o;
  }
}

__global__ void __launch_bounds__(kPlanBlock) unit_plan_table_kernel(const u32* __restrict__ hist, UnitPlanArgs a,
                                                                     const u64* __restrict__ block_small,
                                                                     const u64* __restrict__ block_own,
                                                                     const UnitPlanTotals* __restrict__ tot,
                                                                     uint2* __restrict__ table) {
  __shared__ u64 s_warp[kPlanBlock / 32];
  const u64 nb = 1ull << a.lg;
  const u64 b = (u64)blockIdx.x * kPlanBlock + threadIdx.x;
  u64 se = 0, own = 0;
  if (b < nb) plan_split(hist[b], a, se, own);
  u64 is = se, io = own;
  block_incl_scan_u64<kPlanBlock>(is, s_warp);
  block_incl_scan_u64<kPlanBlock>(io, s_warp);
  if (b < nb) {
    uint2 e;
    if (own == 0) {
      const u64 prefix = block_small[blockIdx.x] + is - se;
      e = make_uint2((u32)(prefix / a.target), 1u);
    } else {
      const u64 prefix = block_own[blockIdx.x] + io - own;
      e = make_uint2((u32)(tot->small_units + prefix), (u32)own);
    }
    table[b] = e;
  }
}

// ---------------------------------------------------------------------------
// Scatter. Parents stream through each CTA in chunks of kUPPT * BLOCK (the
// next chunk is loaded into registers while the current one is staged); the
// chunk's successors, flattened in parent order and lowest free column first,
// fill rounds of exactly kUNC staged candidates (only the CTA's last round is
// partial). Per round: (1) every candidate looks up its unit; (2) the units
// of the round are entered in a shared-memory map and numbered 0..bins-1 (at
// most kUMaxBins; a candidate whose unit finds no bin is stored on its own);
// (3) ranks within bins, a block scan of the bin counts, one cursor atomic per
// bin; (4) the candidates are reordered by bin in shared memory and written
// as runs, consecutive threads to consecutive slots.

constexpr int kUBlock = 512;
constexpr int kUNC = 2048;      // staged candidates per round
constexpr int kUPer = kUNC / kUBlock;
constexpr int kUPPT = 2;        // parents per thread per chunk
constexpr int kUMaxBins = 1024;
constexpr int kUMapSlots = 2048;
constexpr u32 kNoBin = 0xffffu;

template <int R>
struct alignas(16) UCand {
  u64 key;
  u32 res[R];
};

template <int R>
__device__ __forceinline__ void ustore(UCand<R>* dst, const UCand<R>& c, u64 policy) {
  static_assert(R <= 2, "16-byte candidates");
  const u64 w01 = (u64)c.res[0] | (R > 1 ? (u64)c.res[R > 1 ? 1 : 0] << 32 : 0ull);
  asm volatile("st.global.L2::cache_hint.v2.u64 [%0], {%1, %2}, %3;" ::"l"(dst), "l"(c.key), "l"(w01), "l"(policy)
               : "memory");
}

__device__ __forceinline__ u64 uevict_first_policy() {
  u64 policy;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
  return policy;
}

template <int R>
constexpr size_t unit_scatter_smem() {
  // staged + reordered candidates, bin of each reordered candidate, map keys
  // and values, per-bin count / offset / base / unit
  return (size_t)kUNC * sizeof(UCand<R>) * 2 + (size_t)kUNC * 2 + (size_t)kUMapSlots * 4 + (size_t)kUMapSlots * 2 +
         (size_t)kUMaxBins * 4 * 4;
}

template <int BLOCK>
__device__ __forceinline__ u32 ublock_excl_scan(u32 v, u32* s_warp, u32* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  u32 incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const u32 t = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const u32 w = lane < BLOCK / 32 ? s_warp[lane] : 0u;
    u32 wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const u32 t = __shfl_up_sync(kFull, wi, d);
      if (lane >= d) wi += t;
    }
    s_warp[lane] = wi - w;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  return s_warp[wid] + incl - v;
}

template <int R>
__global__ void __launch_bounds__(kUBlock, 2) unit_scatter_kernel(const u64* __restrict__ keys,
                                                                  const u32* __restrict__ res, u64 res_stride,
                                                                  u64 n_in, UnitClassPlan c,
                                                                  const uint2* __restrict__ table,
                                                                  UCand<R>* __restrict__ regions, u32 cap,
                                                                  u32 units, u32* __restrict__ cursors, u32 cstride,
                                                                  StepScalars* __restrict__ sc) {
  constexpr int BLOCK = kUBlock;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  UCand<R>* s_a = reinterpret_cast<UCand<R>*>(smem_raw);
  UCand<R>* s_b = s_a + kUNC;
  unsigned short* s_bin = reinterpret_cast<unsigned short*>(s_b + kUNC);
  u32* s_mkey = reinterpret_cast<u32*>(s_bin + kUNC);
  unsigned short* s_mval = reinterpret_cast<unsigned short*>(s_mkey + kUMapSlots);
  u32* s_cnt = reinterpret_cast<u32*>(s_mval + kUMapSlots);
  u32* s_off = s_cnt + kUMaxBins;
  u32* s_base = s_off + kUMaxBins;
  u32* s_bunit = s_base + kUMaxBins;
  __shared__ u32 s_warp[32];
  __shared__ u32 s_total, s_nbins;
  const int tid = threadIdx.x;
  const u64 mask = (1ull << c.n) - 1;
  constexpr u64 CP = (u64)kUPPT * BLOCK;
  const u64 stride = (u64)gridDim.x * CP;
  const u64 policy = uevict_first_policy();
  bool overflow = false, bounds = false;

  u64 ck[kUPPT], cf[kUPPT], nk[kUPPT];
  u32 cw[kUPPT][R], nw[kUPPT][R];
  auto prefetch = [&](u64 base) {
#pragma unroll
    for (int q = 0; q < kUPPT; ++q) {
      const u64 i = base + (u64)q * BLOCK + tid;
      nk[q] = kNoKey;
      if (i < n_in) {
        nk[q] = __ldcs(keys + i);
#pragma unroll
        for (int r = 0; r < R; ++r) nw[q][r] = __ldcs(res + r * res_stride + i);
      }
    }
  };
  u64 next_base = (u64)blockIdx.x * CP;
  bool more = next_base < n_in;
  if (more) prefetch(next_base);
  u32 first = 0, total = 0, r0 = 0;
  auto advance = [&]() {
    u32 cnt = 0;
#pragma unroll
    for (int q = 0; q < kUPPT; ++q) {
      ck[q] = nk[q];
#pragma unroll
      for (int r = 0; r < R; ++r) cw[q][r] = nw[q][r];
      cf[q] = 0;
      if (ck[q] != kNoKey) {
        const State s = unpack<u64>(ck[q], c.n, mask);
        cf[q] = ~(s.cols | s.dr | s.dl) & mask;
      }
      cnt += (u32)__popcll(cf[q]);
    }
    next_base += stride;
    more = next_base < n_in;
    if (more) prefetch(next_base);
    first = ublock_excl_scan<BLOCK>(cnt, s_warp, &s_total);
    total = s_total;
    r0 = 0;
  };
  auto stage = [&](u32 lo, u32 take, u32 at) {
    u32 g = first;
#pragma unroll
    for (int q = 0; q < kUPPT; ++q) {
      const u32 k = (u32)__popcll(cf[q]);
      if (k && g + k > lo && g < lo + take) {
        const State s = unpack<u64>(ck[q], c.n, mask);
        u64 f = cf[q];
        u32 j = g;
        while (f) {
          const u64 b = f & (0ull - f);
          f ^= b;
          if (j >= lo && j < lo + take) {
            UCand<R> cd;
            cd.key = row_successor<u64>(s, b, c.n, mask);
#pragma unroll
            for (int r = 0; r < R; ++r) cd.res[r] = cw[q][r];
            s_a[at + (j - lo)] = cd;
          }
          ++j;
        }
      }
      g += k;
    }
  };
  for (;;) {
    u32 m = 0;
    for (;;) {
      if (r0 == total) {
        if (!more) break;
        advance();
        continue;
      }
      const u32 take = min(total - r0, (u32)kUNC - m);
      stage(r0, take, m);
      m += take;
      r0 += take;
      if (m == (u32)kUNC) break;
    }
    if (m == 0) break;
    for (int i = tid; i < kUMapSlots; i += BLOCK) s_mkey[i] = kFull;
    for (int i = tid; i < kUMaxBins; i += BLOCK) s_cnt[i] = 0u;
    if (tid == 0) s_nbins = 0;
    __syncthreads();  // staged candidates; cleared map and counts
    // (1)+(2a): unit of each candidate; enter it in the map.
    u32 unit[kUPer], mslot[kUPer];
#pragma unroll
    for (int k = 0; k < kUPer; ++k) {
      const u32 i = (u32)k * BLOCK + tid;
      mslot[k] = kFull;
      if (i < m) {
        const u64 key = s_a[i].key;
        const uint2 e = table[ubucket_of(key, c)];
        unit[k] = unit_of(key, e);
        if (unit[k] >= units) {  // outside the planned partitions: counted as an error, not stored
          overflow = bounds = true;
          unit[k] = kFull;
          continue;
        }
        u32 slot = (unit[k] * 0x9E3779B1u) >> (32 - 11);
        for (int p = 0; p < 32; ++p) {
          const u32 cur = atomicCAS(&s_mkey[slot], kFull, unit[k]);
          if (cur == kFull || cur == unit[k]) {
            mslot[k] = slot;
            break;
          }
          slot = (slot + 1) & (kUMapSlots - 1);
        }
      }
    }
    __syncthreads();
    // (2b): number the occupied map slots (block scan over slot order).
    {
      constexpr int SPT = kUMapSlots / BLOCK;
      u32 occ = 0;
#pragma unroll
      for (int q = 0; q < SPT; ++q) occ += s_mkey[tid * SPT + q] != kFull;
      u32 id = ublock_excl_scan<BLOCK>(occ, s_warp, &s_total);
#pragma unroll
      for (int q = 0; q < SPT; ++q) {
        const int sl = tid * SPT + q;
        if (s_mkey[sl] != kFull) {
          if (id < (u32)kUMaxBins) {
            s_mval[sl] = (unsigned short)id;
            s_bunit[id] = s_mkey[sl];
          } else {
            s_mval[sl] = (unsigned short)kNoBin;
          }
          ++id;
        }
      }
      if (tid == 0) s_nbins = min(s_total, (u32)kUMaxBins);
    }
    __syncthreads();
    // (3): bins and ranks; candidates without a bin are stored on their own.
    u32 bin[kUPer], rank[kUPer];
#pragma unroll
    for (int k = 0; k < kUPer; ++k) {
      const u32 i = (u32)k * BLOCK + tid;
      bin[k] = kNoBin;
      rank[k] = 0;
      if (i < m && unit[k] != kFull) {
        const u32 b = mslot[k] != kFull ? (u32)s_mval[mslot[k]] : kNoBin;
        if (b != kNoBin) {
          bin[k] = b;
          rank[k] = atomicAdd(&s_cnt[b], 1u);
        } else {
          const u32 pos = atomicAdd(&cursors[(u64)unit[k] * cstride], 1u);
          if (pos < cap)
            ustore<R>(regions + (u64)unit[k] * cap + pos, s_a[i], policy);
          else
            overflow = true;
        }
      }
    }
    __syncthreads();
    const u32 nbins = s_nbins;
    {
      constexpr int BPT = kUMaxBins / BLOCK;
      u32 cnt[BPT];
      u32 mine = 0;
#pragma unroll
      for (int q = 0; q < BPT; ++q) {
        const u32 bn = (u32)tid * BPT + q;
        cnt[q] = bn < nbins ? s_cnt[bn] : 0u;
        mine += cnt[q];
      }
      u32 off = ublock_excl_scan<BLOCK>(mine, s_warp, &s_total);
#pragma unroll
      for (int q = 0; q < BPT; ++q) {
        const u32 bn = (u32)tid * BPT + q;
        if (bn < nbins) {
          s_off[bn] = off;
          s_base[bn] = cnt[q] ? atomicAdd(&cursors[(u64)s_bunit[bn] * cstride], cnt[q]) : 0u;
          off += cnt[q];
        }
      }
    }
    __syncthreads();
    // (4): reorder by bin, then write the runs.
#pragma unroll
    for (int k = 0; k < kUPer; ++k) {
      const u32 i = (u32)k * BLOCK + tid;
      if (i < m && bin[k] != kNoBin) {
        const u32 j = s_off[bin[k]] + rank[k];
        s_b[j] = s_a[i];
        s_bin[j] = (unsigned short)bin[k];
      }
    }
    __syncthreads();
    const u32 placed = s_total;
    for (u32 j = tid; j < placed; j += BLOCK) {
      const u32 b = s_bin[j];
      const u32 pos = s_base[b] + (j - s_off[b]);
      if (pos < cap)
        ustore<R>(regions + (u64)s_bunit[b] * cap + pos, s_b[j], policy);
      else
        overflow = true;
    }
    __syncthreads();
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
  if (bounds) atomicOr(&sc->error, kErrBounds);
}

}  // namespace

bool unit_scatter_supported(int residues) { return residues >= 1 && residues <= 2; }

size_t unit_plan_scratch_bytes(uint32_t lg) {
  const size_t nb = (size_t)1 << lg;
  const size_t nblk = (nb + kPlanBlock - 1) / kPlanBlock;
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  return up(nb * 4) + up(nb * 8) + 2 * up(nblk * 8) + up(sizeof(UnitPlanTotals));
}

cudaError_t launch_unit_plan(const FrontierView& in, uint64_t n_in, const UnitClassPlan& c, const UnitPlanArgs& a,
                             void* scratch, int sms, cudaStream_t stream, UnitPlanDev* out, StepScalars* sc) {
  const size_t nb = (size_t)1 << a.lg;
  const size_t nblk = (nb + kPlanBlock - 1) / kPlanBlock;
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  char* p = static_cast<char*>(scratch);
  u32* hist = reinterpret_cast<u32*>(p);
  p += up(nb * 4);
  uint2* table = reinterpret_cast<uint2*>(p);
  p += up(nb * 8);
  u64* bsmall = reinterpret_cast<u64*>(p);
  p += up(nblk * 8);
  u64* bown = reinterpret_cast<u64*>(p);
  p += up(nblk * 8);
  UnitPlanTotals* tot = reinterpret_cast<UnitPlanTotals*>(p);
  out->table = table;
  out->totals = tot;
  if (n_in > in.cap) return cudaErrorInvalidValue;
  if (a.lg > 30 || nblk > 0xffffffffull || a.sample == 0 || (a.sample & (a.sample - 1)) || a.target == 0)
    return cudaErrorInvalidValue;
  if (c.t >= 1 && (a.lg < 3 || c.t > c.n / 2)) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(hist, 0, nb * 4, stream);
  if (e != cudaSuccess) return e;
  if (n_in) {
    constexpr int HB = 512;
    u32 shift = 0;
    while ((1u << shift) < a.sample) ++shift;
    const u64 blocks = (n_in + HB - 1) / HB;
    const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(blocks, (u64)sms * 4));
    unit_hist_kernel<HB><<<grid, HB, 0, stream>>>(reinterpret_cast<const u64*>(in.keys), n_in, c, shift, hist);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  unit_plan_sums_kernel<<<(unsigned)nblk, kPlanBlock, 0, stream>>>(hist, a, bsmall, bown);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  unit_plan_scan_kernel<<<1, 1024, 0, stream>>>(bsmall, bown, (u32)nblk, a, tot, sc);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  unit_plan_table_kernel<<<(unsigned)nblk, kPlanBlock, 0, stream>>>(hist, a, bsmall, bown, tot, table);
  return cudaGetLastError();
}

cudaError_t launch_unit_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in,
                                const UnitClassPlan& c, const uint2* table, void* regions, uint32_t* cursors,
                                StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (n_in > in.cap) return cudaErrorInvalidValue;
  const u64 chunks = (n_in + (u64)kUPPT * kUBlock - 1) / ((u64)kUPPT * kUBlock);
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(chunks, (u64)pc.sms * 2));
  const u32 cstride = pc.cursor_stride ? pc.cursor_stride : 1;
  cudaError_t e;
  if (pc.residues == 1) {
    constexpr size_t smem = unit_scatter_smem<1>();
    auto k = unit_scatter_kernel<1>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) return e;
    k<<<grid, kUBlock, smem, stream>>>(reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_in, c, table,
                                       reinterpret_cast<UCand<1>*>(regions), pc.cap, pc.parts, cursors, cstride, sc);
  } else if (pc.residues == 2) {
    constexpr size_t smem = unit_scatter_smem<2>();
    auto k = unit_scatter_kernel<2>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) return e;
    k<<<grid, kUBlock, smem, stream>>>(reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_in, c, table,
                                       reinterpret_cast<UCand<2>*>(regions), pc.cap, pc.parts, cursors, cstride, sc);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

static_assert(sizeof(UCand<1>) == 16 && sizeof(UCand<2>) == 16, "16-byte candidates, the layout of the merge's");

}  // namespace qpeps

// Partitioned merge for 128-bit boundary keys (boards with N >= 23, or
// key_bits = 128 forced): the same two streaming passes per row as the u64
// path, with 32-byte candidates and a shared-memory table of 128-bit keys.
//
//   wide_scatter_kernel : each warp loads kPPL parents per lane (16-byte
//                         keys, coalesced), writes its lanes' successors as
//                         finished 32-byte candidates (u128 key, R residues)
//                         into a per-warp shared-memory window, then takes a
//                         slot in partition hash(key) * P >> 64 with one
//                         cursor atomic per candidate and stores it.
//   wide_merge_kernel   : persistent CTAs, one partition of up to 1024
//                         candidates at a time: every candidate claims or
//                         finds its key's slot of a 2048-slot table with one
//                         128-bit compare-and-swap (atom.shared.cas.b128), a
//                         key's first claimant lists the slot and stores its
//                         residues, repeated keys add theirs after a barrier,
//                         and the listed slots are written out as the next
//                         boundary (list index = output index).
//
// This replaces, for wide keys, the global-table merge (a random 32-byte
// read-modify-write per successor in HBM). Same contract as the u64 kernels:
// a partition that would overflow sets kErrOverflow and the merge writes
// nothing (the boundary buffer, read by the scatter and written in place by
// the merge, stays intact for the engine's retry).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {

namespace {

constexpr u32 kWFull = 0xffffffffu;
constexpr u128 kWEmpty = ~(u128)0;  // no boundary key sets all 128 bits (3n <= 126)

template <int R>
struct alignas(32) WCand {
  u128 key;
  u32 res[R];
};

__device__ __forceinline__ int wwarp_inclusive_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(kWFull, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

__device__ __forceinline__ u32 wpartition_of(u128 key, u32 parts) {
  return (u32)(((key_hash<u128>(key) >> 32) * (u64)parts) >> 32);
}

__device__ __forceinline__ u128 wload_key(const u128* p) {
  const ulonglong2 v = __ldcs(reinterpret_cast<const ulonglong2*>(p));
  return ((u128)v.y << 64) | v.x;
}

__device__ __forceinline__ u64 wl2_keep_policy() {
  u64 policy;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(policy));
  return policy;
}

// A 32-byte candidate (key; residue words) moves as one 256-bit access
// (sm_100 and later): one scattered store fills a whole 32-byte sector, where
// two 16-byte stores would each leave it half written. Candidates sit at
// 32-byte multiples of a cudaMalloc base, so every access is aligned.
template <int R>
__device__ __forceinline__ void wstore(WCand<R>* dst, const WCand<R>& c, u64 policy) {
  const u64 lo = (u64)c.key, hi = (u64)(c.key >> 64);
  u64 w01 = c.res[0], w23 = 0;
  if constexpr (R > 1) w01 |= (u64)c.res[R > 1 ? 1 : 0] << 32;
  if constexpr (R > 2) w23 = c.res[R > 2 ? 2 : 0];
  if constexpr (R > 3) w23 |= (u64)c.res[R > 3 ? 3 : 0] << 32;
  asm volatile("st.global.L2::cache_hint.v4.b64 [%0], {%1, %2, %3, %4}, %5;" ::"l"(dst), "l"(lo), "l"(hi), "l"(w01),
               "l"(w23), "l"(policy)
               : "memory");
}

template <int R>
__device__ __forceinline__ WCand<R> wload(const WCand<R>* src) {
  u64 lo, hi, w01, w23;
  asm volatile("ld.global.cs.v4.b64 {%0, %1, %2, %3}, [%4];"
               : "=l"(lo), "=l"(hi), "=l"(w01), "=l"(w23)
               : "l"(src));
  WCand<R> c;
  c.key = ((u128)hi << 64) | lo;
  c.res[0] = (u32)w01;
  if constexpr (R > 1) c.res[R > 1 ? 1 : 0] = (u32)(w01 >> 32);
  if constexpr (R > 2) c.res[R > 2 ? 2 : 0] = (u32)w23;
  if constexpr (R > 3) c.res[R > 3 ? 3 : 0] = (u32)(w23 >> 32);
  return c;
}

// 128-bit compare-and-swap on shared memory (PTX atom.shared.cas.b128).
__device__ __forceinline__ u128 wscas(u128* addr, u128 cmp, u128 val) {
  const u64 cl = (u64)cmp, ch = (u64)(cmp >> 64), vl = (u64)val, vh = (u64)(val >> 64);
  u64 ol, oh;
  const unsigned a = (unsigned)__cvta_generic_to_shared(addr);
  asm volatile(
      "{\n\t.reg .b128 c, v, d;\n\t"
      "mov.b128 c, {%2, %3};\n\t"
      "mov.b128 v, {%4, %5};\n\t"
      "atom.shared.cas.b128 d, [%6], c, v;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(ol), "=l"(oh)
      : "l"(cl), "l"(ch), "l"(vl), "l"(vh), "r"(a)
      : "memory");
  return ((u128)oh << 64) | ol;
}

// Read after a barrier: a plain 16-byte shared-memory load.
__device__ __forceinline__ u128 wld_shared(const u128* p) {
  const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
  return ((u128)v.y << 64) | v.x;
}

template <int BLOCK>
__device__ __forceinline__ unsigned long long wblock_sum(unsigned long long v) {
  __shared__ unsigned long long s_part[BLOCK / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kWFull, v, d);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_part[wid] = v;
  __syncthreads();
  unsigned long long t = 0;
  if (wid == 0) {
    t = lane < BLOCK / 32 ? s_part[lane] : 0ull;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(kWFull, t, d);
  }
  return t;
}

// ---------------------------------------------------------------------------
// Scatter (the window scatter of the u64 path, with 128-bit keys).

constexpr int kWKB = 4;   // successor rounds per window
constexpr int kWPPL = 2;  // parents per lane per iteration

template <int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) wide_scatter_kernel(const u128* __restrict__ keys, const u32* __restrict__ res,
                                                            u64 res_stride, u64 n_in, unsigned n,
                                                            WCand<R>* __restrict__ regions,
                                                            u32* __restrict__ cursors, u32 cstride, u32 parts,
                                                            u32 cap, StepScalars* __restrict__ sc) {
  constexpr int WARPS = BLOCK / 32;
  constexpr int PW = 32 * kWPPL;
  constexpr int WIN = 32 * kWKB;
  __shared__ WCand<R> s_cand[WARPS][WIN];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const u64 gwarp = (u64)blockIdx.x * WARPS + wid;
  const u64 stride = (u64)gridDim.x * WARPS * PW;
  const u64 mask = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  const u64 policy = wl2_keep_policy();
  bool overflow = false;
  u128 nkey[kWPPL], ckey[kWPPL];
  u64 fr[kWPPL];
  u32 nw[kWPPL][R], cw[kWPPL][R];
  bool nval[kWPPL], cval[kWPPL];
  auto fetch = [&](u64 base) {
#pragma unroll
    for (int q = 0; q < kWPPL; ++q) {
      const u64 i = base + q * 32 + lane;
      nval[q] = i < n_in;
      if (nval[q]) {
        nkey[q] = wload_key(keys + i);
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
    for (int q = 0; q < kWPPL; ++q) {
      ckey[q] = nkey[q];
      cval[q] = nval[q];
      fr[q] = 0;
      if (cval[q]) {
        const State s = unpack<u128>(ckey[q], n, mask);
        fr[q] = ~(s.cols | s.dr | s.dl) & mask;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) cw[q][r] = nw[q][r];
      cnt += __popcll(fr[q]);
    }
    if (base + stride < n_in) fetch(base + stride);
    const int incl = wwarp_inclusive_scan(cnt);
    const int total = __shfl_sync(kWFull, incl, 31);
    int g = incl - cnt;
    for (int j0 = 0; j0 < total; j0 += WIN) {
      const int hi = min(incl, j0 + WIN);
#pragma unroll
      for (int q = 0; q < kWPPL; ++q) {
        if (g < hi && fr[q]) {
          const State s = unpack<u128>(ckey[q], n, mask);
          do {
            const u64 b = fr[q] & (0ull - fr[q]);
            fr[q] ^= b;
            WCand<R> c;
            c.key = row_successor<u128>(s, b, n, mask);
#pragma unroll
            for (int r = 0; r < R; ++r) c.res[r] = cw[q][r];
            s_cand[wid][g - j0] = c;
            ++g;
          } while (g < hi && fr[q]);
        }
      }
      __syncwarp();
      u32 part[kWKB], pos[kWKB];
#pragma unroll
      for (int k = 0; k < kWKB; ++k) {
        part[k] = kWFull;
        if (j0 + k * 32 + lane < total) part[k] = wpartition_of(s_cand[wid][k * 32 + lane].key, parts);
      }
#pragma unroll
      for (int k = 0; k < kWKB; ++k)
        if (part[k] != kWFull) pos[k] = atomicAdd(&cursors[(u64)part[k] * cstride], 1u);
#pragma unroll
      for (int k = 0; k < kWKB; ++k)
        if (part[k] != kWFull) {
          if (pos[k] < cap)
            wstore<R>(regions + (u64)part[k] * cap + pos[k], s_cand[wid][k * 32 + lane], policy);
          else
            overflow = true;
        }
      __syncwarp();
    }
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

// ---------------------------------------------------------------------------
// Merge: claim list with 128-bit keys (R residue planes summed per key).

constexpr int kWBlock = 512, kWH = 2048, kWCap = kWH / 2;

template <int R>
constexpr size_t wide_merge_smem() {
  return (size_t)kWH * 16 + (size_t)R * kWH * 8 + (size_t)kWCap * 4;
}

// kBond: the explicit-C frontier's instantiation, which also matches the
// written keys against the next site step's transitions (`next_step`); the
// row-key one counts free columns at the next row instead (n > 0). Both are
// held to two 512-thread CTAs per SM (64 registers): the row-key merge at one
// CTA per SM ran 1.5x slower.
template <int R, int BLOCK, int H, int CAP, bool kBond>
__global__ void __launch_bounds__(BLOCK, 2) wide_merge_kernel(const WCand<R>* __restrict__ regions,
                                                          const u32* __restrict__ cursors, u32 cstride, u32 parts,
                                                          u128* __restrict__ keys_out, u32* __restrict__ res_out,
                                                          u64 out_stride, unsigned n, int write_out,
                                                          const FrontierStepDev* __restrict__ next_step,
                                                          StepScalars* __restrict__ sc) {
  static_assert((H & (H - 1)) == 0 && H >= 2 * CAP && CAP % BLOCK == 0, "merge shape");
  constexpr int kLogH = 31 - __builtin_clz(H);
  constexpr int LPT = CAP / BLOCK;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u128* s_key = reinterpret_cast<u128*>(smem_raw);
  unsigned long long* s_acc = reinterpret_cast<unsigned long long*>(smem_raw + (size_t)H * 16);  // [R][H]
  u32* s_list = reinterpret_cast<u32*>(smem_raw + (size_t)H * 16 + (size_t)R * H * 8);            // [CAP]
  __shared__ u32 s_nused, s_n;
  __shared__ unsigned long long s_base;
  // Explicit-C frontier: the next site step's transitions, to count the
  // written boundary's matches there (its successor terms).
  __shared__ u128 s_req_mask[kBond ? kFrontierMaxTrans : 1], s_req_value[kBond ? kFrontierMaxTrans : 1];
  __shared__ u32 s_next_trans;
  const int lane = threadIdx.x & 31;
  if (*reinterpret_cast<volatile const u32*>(&sc->error)) return;
  // write_out: bit 0 writes the merged boundary, bit 1 lets the row-key
  // merge count its successor terms at the next row.
  const bool count_next = (write_out & 1) && (kBond ? next_step != nullptr : (n > 0 && (write_out & 2)));
  write_out &= 1;
  if constexpr (kBond) {
    if (threadIdx.x == 0) s_next_trans = min(next_step->n_trans, (u32)kFrontierMaxTrans);
    for (int t = threadIdx.x; t < kFrontierMaxTrans; t += BLOCK) {
      s_req_mask[t] = next_step->req_mask[t];
      s_req_value[t] = next_step->req_value[t];
    }
  }
  const u64 mask = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  unsigned long long wsum[R], fsum[R], fstates = 0;
  unsigned long long nterms = 0;  // the written boundary's successor terms at the next row (n > 0)
  bool bad = false;
#pragma unroll
  for (int r = 0; r < R; ++r) wsum[r] = fsum[r] = 0;
  for (int i = threadIdx.x; i < H; i += BLOCK) s_key[i] = kWEmpty;
  if (threadIdx.x == 0) s_nused = 0;

  WCand<R> buf[LPT];
  u32 bcnt = 0;
  auto fetch = [&](u32 part, u32 cnt) {
    bcnt = min(cnt, (u32)CAP);
    const WCand<R>* src = regions + (u64)part * CAP;
#pragma unroll
    for (int l = 0; l < LPT; ++l) {
      const u32 i = l * BLOCK + threadIdx.x;
      if (i < bcnt) buf[l] = wload<R>(src + i);
    }
  };
  u32 part = blockIdx.x;
  if (part < parts) fetch(part, cursors[(u64)part * cstride]);
  __syncthreads();
  for (; part < parts; part += gridDim.x) {
    const u32 next = part + gridDim.x;
    const u32 next_cnt = next < parts ? cursors[(u64)next * cstride] : 0u;
    u32 slots[LPT];
    u32 fresh_bits = 0, dup_bits = 0;
#pragma unroll
    for (int l = 0; l < LPT; ++l) {
      const u32 i = l * BLOCK + threadIdx.x;
      bool fresh = false;
      u32 slot = 0;
      if (i < bcnt) {
        const u128 key = buf[l].key;
        // The partition index takes the hash's top bits; the slot re-mixes
        // the whole hash so keys of one partition spread over the table.
        slot = (u32)(fib_hash_b(key_hash<u128>(key)) >> (64 - kLogH));
        for (int probe = 0; probe < H; ++probe) {
          const u128 cur = wscas(&s_key[slot], kWEmpty, key);
          if (cur == kWEmpty || cur == key) {
            fresh = cur == kWEmpty;
            dup_bits |= (u32)(!fresh) << l;
            break;
          }
          slot = (slot + 1) & (H - 1);
        }
      }
      slots[l] = slot;
      fresh_bits |= (u32)fresh << l;
      const u32 b = __ballot_sync(kWFull, fresh);
      if (b) {
        const int leader = __ffs(b) - 1;
        u32 at = 0;
        if (lane == leader) at = atomicAdd(&s_nused, (u32)__popc(b));
        at = __shfl_sync(kWFull, at, leader);
        if (fresh) s_list[at + __popc(b & ((1u << lane) - 1u))] = slot;
      }
    }
#pragma unroll
    for (int l = 0; l < LPT; ++l)
      if ((fresh_bits >> l) & 1u) {
#pragma unroll
        for (int r = 0; r < R; ++r) s_acc[r * H + slots[l]] = buf[l].res[r];
      }
    __syncthreads();
    u32 n_unique = 0;
    unsigned long long out_base = 0ull;
    if (threadIdx.x == 0) {
      n_unique = s_nused;
      if (n_unique) out_base = atomicAdd(&sc->out_count, (unsigned long long)n_unique);
    }
#pragma unroll
    for (int l = 0; l < LPT; ++l)
      if ((dup_bits >> l) & 1u) {
#pragma unroll
        for (int r = 0; r < R; ++r) atomicAdd(&s_acc[r * H + slots[l]], (unsigned long long)buf[l].res[r]);
      }
    if (next < parts) fetch(next, next_cnt);
    if (threadIdx.x == 0) {
      s_n = n_unique;
      s_base = out_base;
      s_nused = 0;
    }
    __syncthreads();
    const u32 nu = s_n;
    const unsigned long long base = s_base;
    for (u32 i = threadIdx.x; i < nu; i += BLOCK) {
      const u32 slot = s_list[i];
      const u128 key = wld_shared(&s_key[slot]);
      const u64 idx = base + i;
      const bool full = ((u64)key & mask) == mask;
      const bool wr = write_out && idx < out_stride;
      bad |= write_out && !wr;
      if (wr) {
        ulonglong2 kv;
        kv.x = (u64)key;
        kv.y = (u64)(key >> 64);
        reinterpret_cast<ulonglong2*>(keys_out)[idx] = kv;
      }
      if constexpr (kBond) {
        for (u32 t = 0; t < s_next_trans; ++t) nterms += (key & s_req_mask[t]) == s_req_value[t];
      } else if (n) {
        const State st = unpack<u128>(key, n, mask);
        nterms += __popcll(~(st.cols | st.dr | st.dl) & mask);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const u32 v = reduce_sum(s_acc[r * H + slot], r);
        if (wr) res_out[r * out_stride + idx] = v;
        wsum[r] += v;
        if (full) fsum[r] += v;
      }
      s_key[slot] = kWEmpty;
      fstates += full;
    }
    __syncthreads();
  }
  if (bad) atomicOr(&sc->error, kErrBounds);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    unsigned long long t = wblock_sum<BLOCK>(wsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->weight_sum[r], t);
    t = wblock_sum<BLOCK>(fsum[r]);
    if (threadIdx.x == 0 && t) atomicAdd(&sc->final_sum[r], t);
  }
  const unsigned long long t = wblock_sum<BLOCK>(fstates);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->final_states, t);
  if (count_next) {
    const unsigned long long nt = wblock_sum<BLOCK>(nterms);
    if (threadIdx.x == 0 && nt) atomicAdd(&sc->next_terms, nt);
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->next_terms_ok = 1u;
  }
}

// ---------------------------------------------------------------------------
// Explicit-C site frontier through the same partitions. A step's transitions
// (bond runs that move, and per matching C entry the required and added bond
// values) come as a kernel parameter; every (boundary entry, matching
// transition) pair is one candidate with the entry's residues. At most two C
// entries match a key, so a thread writes its entry's candidates directly.

__device__ __forceinline__ u128 wshift(u128 v, int s) { return s >= 0 ? (v << s) : (v >> (-s)); }

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) frontier_count_kernel(const u128* __restrict__ keys, u64 n_in,
                                                              const __grid_constant__ FrontierStepDev st,
                                                              StepScalars* __restrict__ sc) {
  unsigned long long acc = 0;
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in; i += (u64)gridDim.x * BLOCK) {
    const u128 key = keys[i];
    for (u32 t = 0; t < st.n_trans; ++t) acc += (key & st.req_mask[t]) == st.req_value[t];
  }
  const unsigned long long t = wblock_sum<BLOCK>(acc);
  if (threadIdx.x == 0 && t) atomicAdd(&sc->terms, t);
}

template <int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) frontier_scatter_kernel(const u128* __restrict__ keys,
                                                                const u32* __restrict__ res, u64 res_stride,
                                                                u64 n_in, const __grid_constant__ FrontierStepDev st,
                                                                WCand<R>* __restrict__ regions,
                                                                u32* __restrict__ cursors, u32 cstride, u32 parts,
                                                                u32 cap, StepScalars* __restrict__ sc) {
  const u64 policy = wl2_keep_policy();
  bool overflow = false;
  for (u64 i = (u64)blockIdx.x * BLOCK + threadIdx.x; i < n_in; i += (u64)gridDim.x * BLOCK) {
    const u128 key = wload_key(keys + i);
    u128 moved = 0;
    for (u32 r = 0; r < st.n_runs; ++r) moved |= wshift(key & st.run_mask[r], st.run_shift[r]);
    WCand<R> c;
#pragma unroll
    for (int r = 0; r < R; ++r) c.res[r] = __ldcs(res + r * res_stride + i);
    for (u32 t = 0; t < st.n_trans; ++t) {
      if ((key & st.req_mask[t]) != st.req_value[t]) continue;
      c.key = moved | st.added[t];
      const u32 part = wpartition_of(c.key, parts);
      const u32 pos = atomicAdd(&cursors[(u64)part * cstride], 1u);
      if (pos < cap)
        wstore<R>(regions + (u64)part * cap + pos, c, policy);
      else
        overflow = true;
    }
  }
  if (overflow) atomicOr(&sc->error, kErrOverflow);
}

constexpr int kWScatterBlock = 256;

template <int R>
cudaError_t wide_scatter(const PartitionCfg& pc, const FrontierView& in, u64 n_in, unsigned n, void* regions,
                         u32* cursors, StepScalars* sc, cudaStream_t stream) {
  const u64 want = (n_in + kWScatterBlock * kWPPL - 1) / (kWScatterBlock * kWPPL);
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)pc.sms * 8));
  wide_scatter_kernel<R, kWScatterBlock><<<grid, kWScatterBlock, 0, stream>>>(
      reinterpret_cast<const u128*>(in.keys), in.res, in.cap, n_in, n, reinterpret_cast<WCand<R>*>(regions), cursors,
      pc.cursor_stride ? pc.cursor_stride : 1, pc.parts, pc.cap, sc);
  return cudaGetLastError();
}

template <int R>
cudaError_t wide_merge(const PartitionCfg& pc, const void* regions, const u32* cursors, const FrontierView& out,
                       unsigned n, bool write_out, const FrontierStepDev* next_step, StepScalars* sc,
                       cudaStream_t stream) {
  if (pc.cap != (u32)kWCap) return cudaErrorInvalidValue;
  constexpr size_t smem = wide_merge_smem<R>();
  auto kern = next_step ? wide_merge_kernel<R, kWBlock, kWH, kWCap, true> : wide_merge_kernel<R, kWBlock, kWH, kWCap, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(pc.parts, (u64)pc.sms * 2));
  kern<<<grid, kWBlock, smem, stream>>>(reinterpret_cast<const WCand<R>*>(regions), cursors,
                                        pc.cursor_stride ? pc.cursor_stride : 1, pc.parts,
                                        reinterpret_cast<u128*>(out.keys), out.res, out.cap, n,
                                        (write_out ? 1 : 0) | (pc.count_next ? 2 : 0), next_step, sc);
  return cudaGetLastError();
}

}  // namespace

uint32_t wide_key_partition_capacity() { return kWCap; }

cudaError_t launch_wide_partition_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in, unsigned n,
                                          void* regions, uint32_t* cursors, StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (n_in > in.cap || reinterpret_cast<uintptr_t>(regions) % 32) return cudaErrorInvalidValue;
  switch (pc.residues) {
    case 1: return wide_scatter<1>(pc, in, n_in, n, regions, cursors, sc, stream);
    case 2: return wide_scatter<2>(pc, in, n_in, n, regions, cursors, sc, stream);
    case 3: return wide_scatter<3>(pc, in, n_in, n, regions, cursors, sc, stream);
    case 4: return wide_scatter<4>(pc, in, n_in, n, regions, cursors, sc, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_wide_partition_merge(const PartitionCfg& pc, const void* regions, const uint32_t* cursors,
                                        const FrontierView& out, unsigned n, bool write_out, StepScalars* sc,
                                        cudaStream_t stream, const FrontierStepDev* next_step) {
  if (reinterpret_cast<uintptr_t>(regions) % 32) return cudaErrorInvalidValue;  // 256-bit candidate loads
  if (n && next_step) return cudaErrorInvalidValue;                              // row keys or bond keys
  switch (pc.residues) {
    case 1: return wide_merge<1>(pc, regions, cursors, out, n, write_out, next_step, sc, stream);
    case 2: return wide_merge<2>(pc, regions, cursors, out, n, write_out, next_step, sc, stream);
    case 3: return wide_merge<3>(pc, regions, cursors, out, n, write_out, next_step, sc, stream);
    case 4: return wide_merge<4>(pc, regions, cursors, out, n, write_out, next_step, sc, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_frontier_count(const FrontierView& in, uint64_t n_in, const FrontierStepDev& step, int sms,
                                  StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (n_in > in.cap || step.n_trans > (uint32_t)kFrontierMaxTrans) return cudaErrorInvalidValue;
  const u64 want = (n_in + kWScatterBlock - 1) / kWScatterBlock;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)sms * 8));
  frontier_count_kernel<kWScatterBlock><<<grid, kWScatterBlock, 0, stream>>>(reinterpret_cast<const u128*>(in.keys),
                                                                             n_in, step, sc);
  return cudaGetLastError();
}

cudaError_t launch_frontier_partition_scatter(const PartitionCfg& pc, const FrontierView& in, uint64_t n_in,
                                              const FrontierStepDev& step, void* regions, uint32_t* cursors,
                                              StepScalars* sc, cudaStream_t stream) {
  if (n_in == 0) return cudaSuccess;
  if (n_in > in.cap || pc.parts == 0 || pc.cap != (u32)kWCap || step.n_trans > (uint32_t)kFrontierMaxTrans ||
      step.n_runs > (uint32_t)kFrontierMaxRuns || reinterpret_cast<uintptr_t>(regions) % 32)
    return cudaErrorInvalidValue;
  const u64 want = (n_in + kWScatterBlock - 1) / kWScatterBlock;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)pc.sms * 8));
  const u128* keys = reinterpret_cast<const u128*>(in.keys);
  const u32 cs = pc.cursor_stride ? pc.cursor_stride : 1;
  switch (pc.residues) {
#define QPEPS_FRONTIER_SCATTER(R)                                                                            \
  case R:                                                                                                   \
    frontier_scatter_kernel<R, kWScatterBlock><<<grid, kWScatterBlock, 0, stream>>>(                         \
        keys, in.res, in.cap, n_in, step, reinterpret_cast<WCand<R>*>(regions), cursors, cs, pc.parts, pc.cap, sc); \
    break;
    QPEPS_FRONTIER_SCATTER(1)
    QPEPS_FRONTIER_SCATTER(2)
    QPEPS_FRONTIER_SCATTER(3)
    QPEPS_FRONTIER_SCATTER(4)
#undef QPEPS_FRONTIER_SCATTER
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

static_assert(sizeof(WCand<1>) == 32 && sizeof(WCand<4>) == 32, "32-byte wide candidates");

}  // namespace qpeps

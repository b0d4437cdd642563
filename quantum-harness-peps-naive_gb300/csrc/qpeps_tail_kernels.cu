// Persistent slice-tail kernel: each warp contracts one boundary entry's
// remaining rows entirely in shared memory.
//
// The boundary after row k (computed and merged in HBM by the row engine) is
// a set of independent sub-boundaries: the count is linear in the boundary,
// so every entry can be contracted on its own (prefix-depth slicing; the
// reference splits work the same way into prefix tasks, src/lib.rs:3888-3956).
// Each entry's own frontier stays small (a few hundred states), so a warp
// holds it in shared memory with a private open-addressing table, applies the
// certified compiled row operator (src/lib.rs:600-638) row by row, merges
// equal keys (src/lib.rs:5353-5367), and at the last row adds the v1/v2 final
// contraction (src/lib.rs:5393-5401) directly: every successor of the last row
// has all columns set, so the completions of a parent are its weight times its
// free-column count. Entries whose frontier outgrows the warp's capacity are
// reported back (overflow list) and contracted by the HBM row engine instead.
// Warps pull entries from a global work counter, so uneven subtrees balance.
#include <cuda_runtime.h>

#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {
namespace {

constexpr u32 kFull = 0xffffffffu;
constexpr u64 kNone = ~0ull;

__device__ __forceinline__ u64 tboard_mask(unsigned n) { return (1ull << n) - 1; }

__device__ __forceinline__ int twarp_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int t = __shfl_up_sync(kFull, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

__device__ __forceinline__ unsigned tnth_set_bit(u64 m, int k) {
  u32 lo = (u32)m, hi = (u32)(m >> 32);
  int plo = __popc(lo);
  return k < plo ? __fns(lo, 0, k + 1) : 32u + __fns(hi, 0, k - plo + 1);
}

// Modular add into a shared-memory residue (compare-and-swap loop; equal keys
// inside one warp are rare, so the loop almost always runs once).
__device__ __forceinline__ void smem_add_mod(u32* a, u32 w, u32 p) {
  u32 old = *a;
  while (true) {
    const u32 nv = add_mod(old, w, p);
    const u32 prev = atomicCAS(a, old, nv);
    if (prev == old) break;
    old = prev;
  }
}

template <int R, int CAPF, int H>
struct TailSmem {
  u64 fkey[CAPF];
  u32 fres[R][CAPF];
  u64 tkey[H];
  u32 tacc[R][H];
  unsigned short used[H];                                      // occupied-slot list of the current row
  unsigned long long row_acc[kTailMaxRows][kTailRowFields];    // per-CTA row statistics
  unsigned long long batch_acc[kTailMaxRows][kTailRowFields];  // current batch's statistics
  unsigned long long fin[4];
  unsigned long long claim_base;
  u32 nused[2];  // occupied-slot counters, alternating by row
};

__device__ __forceinline__ unsigned long long twarp_sum(unsigned long long v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
  return v;
}

// A CTA takes B boundary entries at a time (claimed from the work counter)
// and contracts them together as one small merged boundary held in shared
// memory: a frontier of at most CAPF states and an H-slot open-addressing
// table whose claimed slots are appended to an occupied list, so compaction
// visits only used slots and a slot's list index is its output position. A
// row whose distinct successors exceed CAPF sends the batch to the overflow
// list (the HBM row engine contracts it instead). Row statistics: per row the
// input count, the successor terms (warp-summed popcounts), the distinct
// outputs, and the output weight = sum of parent weight * free columns (the
// merge preserves weight sums). The last two rows are finished without a
// table: a parent at row n-2 contributes weight * (free columns of each of its
// successors), every such successor completing the board.
template <int R, int BLOCK, int CAPF, int H, int B>
__global__ void __launch_bounds__(BLOCK) slice_tail_kernel(const u64* __restrict__ keys,
                                                           const u32* __restrict__ res, u64 res_stride,
                                                           u64 n_items, unsigned n, unsigned row0,
                                                           TailControl* __restrict__ ctl) {
  static_assert(CAPF >= B && (H & (H - 1)) == 0 && CAPF <= H / 2 && H <= 65536, "shape");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using S = TailSmem<R, CAPF, H>;
  S& sm = *reinterpret_cast<S*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31;
  const u64 mask = tboard_mask(n);
  const unsigned rows = n - row0;

  for (int i = tid; i < kTailMaxRows * kTailRowFields; i += BLOCK) (&sm.row_acc[0][0])[i] = 0ull;
  for (int i = tid; i < H; i += BLOCK) {
    sm.tkey[i] = kNone;
#pragma unroll
    for (int r = 0; r < R; ++r) sm.tacc[r][i] = 0u;
  }
  unsigned long long done_final[R];
#pragma unroll
  for (int r = 0; r < R; ++r) done_final[r] = 0;

  while (true) {
    __syncthreads();
    if (tid == 0) {
      sm.claim_base = atomicAdd(&ctl->next_item, (unsigned long long)B);
      sm.nused[0] = sm.nused[1] = 0;
#pragma unroll
      for (int r = 0; r < 4; ++r) sm.fin[r] = 0;
    }
    for (int i = tid; i < kTailMaxRows * kTailRowFields; i += BLOCK) (&sm.batch_acc[0][0])[i] = 0ull;
    __syncthreads();
    const unsigned long long first = sm.claim_base;
    if (first >= n_items) break;
    const int nb = (int)min((unsigned long long)B, n_items - first);
    if (tid < nb) {
      sm.fkey[tid] = keys[first + tid];
#pragma unroll
      for (int r = 0; r < R; ++r) sm.fres[r][tid] = res[r * res_stride + first + tid];
    }
    int count = nb;
    bool ok = true;
    __syncthreads();

    for (unsigned row = row0; row < n && count > 0; ++row) {
      const unsigned q = row - row0;
      unsigned long long* acc = sm.batch_acc[q];
      u32* nused = &sm.nused[q & 1];
      if (row + 2 >= n) {
        // Finish rows n-2 and n-1.
        u64 part[R], pw[R];
#pragma unroll
        for (int r = 0; r < R; ++r) part[r] = pw[r] = 0;
        unsigned long long terms = 0, terms_next = 0;
        for (int pi = tid; pi < count; pi += BLOCK) {
          const State s = unpack<u64>(sm.fkey[pi], n, mask);
          u64 fr = ~(s.cols | s.dr | s.dl) & mask;
          const u64 nfree = (u64)__popcll(fr);
          terms += nfree;
          u64 comp = nfree;
          if (row + 1 < n) {
            comp = 0;
            while (fr) {
              const u64 b = fr & (~fr + 1);
              fr ^= b;
              const State c = unpack<u64>(row_successor<u64>(s, b, n, mask), n, mask);
              comp += (u64)__popcll(~(c.cols | c.dr | c.dl) & mask);
            }
          }
          terms_next += comp;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const u64 wv = sm.fres[r][pi];
            part[r] = (part[r] + wv * comp) % prime_at(r);
            pw[r] = (pw[r] + wv * nfree) % prime_at(r);
          }
        }
        terms = twarp_sum(terms);
        terms_next = twarp_sum(terms_next);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          part[r] = twarp_sum(part[r]) % prime_at(r);
          pw[r] = twarp_sum(pw[r]) % prime_at(r);
        }
        if (lane == 0) {
          if (tid == 0) atomicAdd(&acc[0], (unsigned long long)count);
          atomicAdd(&acc[2], terms);
          atomicAdd(&acc[1], terms);  // unmerged successor terms
#pragma unroll
          for (int r = 0; r < R; ++r) {
            atomicAdd(&acc[3 + r], pw[r]);
            atomicAdd(&sm.fin[r], part[r]);
          }
          if (row + 1 < n) {
            unsigned long long* nxt = sm.batch_acc[q + 1];
            atomicAdd(&nxt[0], terms);
            atomicAdd(&nxt[1], terms_next);
            atomicAdd(&nxt[2], terms_next);
#pragma unroll
            for (int r = 0; r < R; ++r) atomicAdd(&nxt[3 + r], part[r]);
          }
        }
        break;
      }
      // Insert every successor; each thread walks its parents' free columns.
      unsigned long long terms = 0;
      u64 pwsum[R];
#pragma unroll
      for (int r = 0; r < R; ++r) pwsum[r] = 0;
      bool lane_full = false;
      for (int pi = tid; pi < count && !lane_full; pi += BLOCK) {
        const State ps = unpack<u64>(sm.fkey[pi], n, mask);
        u64 fr = ~(ps.cols | ps.dr | ps.dl) & mask;
        const u64 nfree = (u64)__popcll(fr);
        terms += nfree;
        u32 pw[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          pw[r] = sm.fres[r][pi];
          pwsum[r] += (u64)pw[r] * nfree;
        }
        while (fr) {
          const u64 b = fr & (~fr + 1);
          fr ^= b;
          const u64 child = row_successor<u64>(ps, b, n, mask);
          u32 slot = (u32)mix64(child) & (H - 1);
          bool placed = false;
          for (int probe = 0; probe < H; ++probe) {
            u64 cur = sm.tkey[slot];
            if (cur == kNone) {
              cur = atomicCAS(reinterpret_cast<unsigned long long*>(&sm.tkey[slot]), kNone, child);
              if (cur == kNone) {
                const u32 at = atomicAdd(nused, 1u);
                if (at < (u32)CAPF) sm.used[at] = (unsigned short)slot;
                cur = child;
              }
            }
            if (cur == child) {
#pragma unroll
              for (int r = 0; r < R; ++r) smem_add_mod(&sm.tacc[r][slot], pw[r], prime_at(r));
              placed = true;
              break;
            }
            slot = (slot + 1) & (H - 1);
          }
          if (!placed) {
            lane_full = true;
            break;
          }
        }
      }
      terms = twarp_sum(terms);
#pragma unroll
      for (int r = 0; r < R; ++r) pwsum[r] = twarp_sum(pwsum[r] % prime_at(r)) % prime_at(r);
      if (lane == 0) {
        atomicAdd(&acc[2], terms);
#pragma unroll
        for (int r = 0; r < R; ++r) atomicAdd(&acc[3 + r], pwsum[r]);
      }
      if (lane_full) atomicOr(nused, 0x80000000u);
      __syncthreads();
      const u32 nu = *nused;
      // The other counter is idle until the next row starts (after the
      // barrier that ends this row): clear it now for that row.
      if (tid == 0) sm.nused[(q + 1) & 1] = 0;
      // More distinct successors than the frontier holds (or a full table):
      // drop the batch. Reset every claimed slot (those beyond CAPF were not
      // listed, so clear the whole table in that case).
      if (nu > (u32)CAPF) {
        for (int i = tid; i < H; i += BLOCK) {
          sm.tkey[i] = kNone;
#pragma unroll
          for (int r = 0; r < R; ++r) sm.tacc[r][i] = 0u;
        }
        ok = false;
        break;
      }
      const int nc = (int)nu;
      for (int i = tid; i < nc; i += BLOCK) {
        const int slot = sm.used[i];
        sm.fkey[i] = sm.tkey[slot];
        sm.tkey[slot] = kNone;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          sm.fres[r][i] = sm.tacc[r][slot];
          sm.tacc[r][slot] = 0u;
        }
      }
      if (tid == 0) {
        acc[0] = (unsigned long long)count;
        acc[1] = (unsigned long long)nc;
      }
      count = nc;
      __syncthreads();
    }
    __syncthreads();
    if (!ok) {
      if (tid == 0) {
        const unsigned long long slot = atomicAdd(&ctl->overflow_count, (unsigned long long)nb);
        if (slot + nb <= ctl->overflow_cap)
          for (int i = 0; i < nb; ++i) ctl->overflow_items[slot + i] = first + i;
        else
          atomicOr(&ctl->error, kErrOverflow);
      }
      continue;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) done_final[r] = (done_final[r] + sm.fin[r] % prime_at(r)) % prime_at(r);
    for (int i = tid; i < (int)rows * kTailRowFields; i += BLOCK) {
      const int q = i / kTailRowFields, f = i % kTailRowFields;
      unsigned long long v = (&sm.batch_acc[0][0])[i];
      if (f >= 3) v %= prime_at(f - 3 < R ? f - 3 : 0);
      (&sm.row_acc[0][0])[i] += v;
      (void)q;
    }
  }
  if (tid == 0)
#pragma unroll
    for (int r = 0; r < R; ++r) atomicAdd(&ctl->final_sum[r], done_final[r]);
  __syncthreads();
  for (int i = tid; i < (int)rows * kTailRowFields; i += BLOCK) {
    const unsigned long long v = (&sm.row_acc[0][0])[i];
    if (v) atomicAdd(&ctl->row_acc[0][0] + i, v);
  }
}

// Gather the listed boundary entries (keys + residue planes) into a compact
// buffer with plane stride `m`.
__global__ void gather_entries_kernel(const u64* __restrict__ keys, const u32* __restrict__ res, u64 stride,
                                      const u64* __restrict__ idx, u64 m, int residues, u64* __restrict__ out_keys,
                                      u32* __restrict__ out_res) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (u64)gridDim.x * blockDim.x) {
    const u64 j = idx[i];
    out_keys[i] = keys[j];
    for (int r = 0; r < residues; ++r) out_res[r * m + i] = res[r * stride + j];
  }
}

constexpr int kTailBlock = 256;
constexpr int kTailCapF = 2048;
constexpr int kTailH = 4096;
constexpr int kTailBatch = 64;

template <int R>
cudaError_t tail_impl(const FrontierView& in, uint64_t n_items, unsigned n, unsigned row0, TailControl* ctl, int sms,
                      cudaStream_t stream) {
  auto kern = slice_tail_kernel<R, kTailBlock, kTailCapF, kTailH, kTailBatch>;
  const size_t smem = sizeof(TailSmem<R, kTailCapF, kTailH>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTailBlock, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const u64 want = (n_items + kTailBatch - 1) / kTailBatch;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)sms * per_sm));
  kern<<<grid, kTailBlock, smem, stream>>>(reinterpret_cast<const u64*>(in.keys), in.res, in.cap, n_items, n,
                                                row0, ctl);
  return cudaGetLastError();
}

}  // namespace

uint32_t tail_capacity() { return kTailCapF; }

cudaError_t launch_gather_entries(int residues, const FrontierView& in, const uint64_t* idx, uint64_t m,
                                  uint64_t* out_keys, uint32_t* out_res, int sms, cudaStream_t stream) {
  if (m == 0) return cudaSuccess;
  const u64 want = (m + 255) / 256;
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)sms * 8));
  gather_entries_kernel<<<grid, 256, 0, stream>>>(reinterpret_cast<const u64*>(in.keys), in.res, in.cap, idx, m,
                                                  residues, out_keys, out_res);
  return cudaGetLastError();
}

cudaError_t launch_slice_tail(int residues, const FrontierView& in, uint64_t n_items, unsigned n, unsigned row0,
                              TailControl* ctl, int sms, cudaStream_t stream) {
  if (n_items == 0) return cudaSuccess;
  if (n > 21 || row0 >= n || n - row0 > kTailMaxRows) return cudaErrorInvalidValue;
  switch (residues) {
    case 1: return tail_impl<1>(in, n_items, n, row0, ctl, sms, stream);
    case 2: return tail_impl<2>(in, n_items, n, row0, ctl, sms, stream);
    case 3: return tail_impl<3>(in, n_items, n, row0, ctl, sms, stream);
    case 4: return tail_impl<4>(in, n_items, n, row0, ctl, sms, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace qpeps

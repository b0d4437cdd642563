// Access-pattern probes: the device's own rate for the memory pattern the
// partition scatter is built on, without its boundary reads or successor
// arithmetic, so that the scatter can be judged against what the pattern
// itself reaches on this GPU.
//
//   mode 0  append: a pseudo-random 64-bit key picks one of `parts`
//           partitions; one cursor atomic per key takes a slot and the
//           16-byte (key, value) record is stored there (the scatter's inner
//           step, with the same L2 keep hint);
//   mode 1  store only: the same records to a pseudo-random slot of the same
//           partition, no atomic;
//   mode 2  atomic only: the cursor atomics of mode 0, no store;
//   mode 3  stream: the records stored in index order (coalesced);
//   mode 4  append as mode 0 with plain stores (no L2 hint).
//
// Every store lands inside `parts * cap` records: modes 0, 2 and 4 skip a slot
// at or beyond `cap` (a full partition), mode 1 masks the slot with cap - 1
// (cap a power of two), mode 3 runs only while the index is below
// parts * cap.
#include <cuda_runtime.h>

#include <algorithm>

#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {

namespace {

constexpr int kProbeBlock = 256;
constexpr int kProbeIlp = 4;  // independent keys per thread and round (atomics in flight)

__device__ __forceinline__ u64 probe_keep_policy() {
  u64 policy;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(policy));
  return policy;
}

__device__ __forceinline__ void probe_store(void* dst, u64 a, u64 b, u64 policy) {
  asm volatile("st.global.L2::cache_hint.v2.u64 [%0], {%1, %2}, %3;" ::"l"(dst), "l"(a), "l"(b), "l"(policy)
               : "memory");
}

template <int MODE>
__global__ void __launch_bounds__(kProbeBlock) append_probe_kernel(u64 total, u32 parts, u32 cap,
                                                                  ulonglong2* __restrict__ regions,
                                                                  u32* __restrict__ cursors, u32 cstride, u64 seed,
                                                                  unsigned long long* __restrict__ sink) {
  const u64 policy = probe_keep_policy();
  const u64 limit = (u64)parts * cap;
  // Record i = warp base + k * 32 + lane: a warp's k-th store instruction
  // covers 32 consecutive records (coalesced in mode 3).
  const u64 lane = threadIdx.x & 31;
  const u64 warp = ((u64)blockIdx.x * kProbeBlock + threadIdx.x) >> 5;
  const u64 stride = (u64)gridDim.x * kProbeBlock * kProbeIlp;
  unsigned long long acc = 0;
  for (u64 base = warp * 32 * kProbeIlp + lane; base < total; base += stride) {
    u64 key[kProbeIlp];
    u32 part[kProbeIlp], pos[kProbeIlp];
#pragma unroll
    for (int k = 0; k < kProbeIlp; ++k) {
      key[k] = mix64(base + 32 * k + seed);
      part[k] = (u32)(((key[k] >> 32) * (u64)parts) >> 32);
      pos[k] = 0;
    }
    if constexpr (MODE == 0 || MODE == 2 || MODE == 4) {
#pragma unroll
      for (int k = 0; k < kProbeIlp; ++k)
        if (base + 32 * k < total) pos[k] = atomicAdd(&cursors[(u64)part[k] * cstride], 1u);
    }
#pragma unroll
    for (int k = 0; k < kProbeIlp; ++k) {
      const u64 i = base + 32 * k;
      if (i >= total) continue;
      if constexpr (MODE == 0) {
        if (pos[k] < cap) probe_store(regions + (u64)part[k] * cap + pos[k], key[k], i, policy);
      } else if constexpr (MODE == 1) {
        probe_store(regions + (u64)part[k] * cap + ((u32)key[k] & (cap - 1)), key[k], i, policy);
      } else if constexpr (MODE == 2) {
        acc += pos[k];
      } else if constexpr (MODE == 4) {
        if (pos[k] < cap) regions[(u64)part[k] * cap + pos[k]] = make_ulonglong2(key[k], i);
      } else {
        if (i < limit) probe_store(regions + i, key[k], i, policy);
      }
    }
  }
  if constexpr (MODE == 2) {
    if (acc == 0x5eed5eed5eed5eedull) atomicAdd(sink, acc);  // keeps the atomics' results live
  }
}

}  // namespace

cudaError_t launch_append_probe(uint32_t mode, uint64_t total, uint32_t parts, uint32_t cap, void* regions,
                                uint32_t* cursors, uint32_t cursor_stride, int sms, uint64_t seed,
                                unsigned long long* sink, cudaStream_t stream) {
  if (parts == 0 || cap == 0 || (cap & (cap - 1)) || mode > 4 || cursor_stride == 0) return cudaErrorInvalidValue;
  if (total == 0) return cudaSuccess;
  const u64 want = (total + (u64)kProbeBlock * kProbeIlp - 1) / ((u64)kProbeBlock * kProbeIlp);
  const unsigned grid = (unsigned)std::max<u64>(1, std::min<u64>(want, (u64)sms * 8));
  ulonglong2* r = static_cast<ulonglong2*>(regions);
  switch (mode) {
    case 0: append_probe_kernel<0><<<grid, kProbeBlock, 0, stream>>>(total, parts, cap, r, cursors, cursor_stride, seed, sink); break;
    case 1: append_probe_kernel<1><<<grid, kProbeBlock, 0, stream>>>(total, parts, cap, r, cursors, cursor_stride, seed, sink); break;
    case 2: append_probe_kernel<2><<<grid, kProbeBlock, 0, stream>>>(total, parts, cap, r, cursors, cursor_stride, seed, sink); break;
    case 3: append_probe_kernel<3><<<grid, kProbeBlock, 0, stream>>>(total, parts, cap, r, cursors, cursor_stride, seed, sink); break;
    default: append_probe_kernel<4><<<grid, kProbeBlock, 0, stream>>>(total, parts, cap, r, cursors, cursor_stride, seed, sink); break;
  }
  return cudaGetLastError();
}

}  // namespace qpeps

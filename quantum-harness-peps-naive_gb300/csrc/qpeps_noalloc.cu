// One row step of the partitioned merge that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host framework whose caching
// allocator already owns the GPU's memory, or a latency-bound serving loop
// that must not let an allocation synchronise the device mid-stream. They
// hold their boundary buffers themselves and hand us device pointers; the
// merge's scratch (hash-partition slots, partition cursors and the step's
// scalar results) comes from the fixed array below instead of the context's
// pool.
//
// The array is a file-scope __device__ object, so every GPU that loads this
// library holds kNoAllocScratchBytes (48 MiB) of device memory until the
// process exits. Host code cannot use the array's name as a device address:
// the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and caches it beside the
// CUDA context that was current, so make that first call before any stream
// capture. A call made under a different context of the same device (after a
// device reset, or from a non-primary driver context) looks the address up
// again. All calls share the array and it keeps the previous call's contents,
// so each call clears the cursors and scalars it uses; calls whose GPU work
// overlaps (different streams or threads) race on it and must be serialised
// by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/qpeps.h"
#include "qpeps_device.cuh"
#include "qpeps_internal.h"

namespace qpeps {
namespace {

constexpr size_t kNoAllocScratchBytes = 48ull << 20;
constexpr int kMaxDevices = 64;
constexpr double kNoAllocMean = 1600.0;  // target candidates per partition

static __device__ __align__(256) unsigned char g_step_scratch[kNoAllocScratchBytes];

std::mutex g_addr_mutex;
void* g_addr[kMaxDevices] = {nullptr};
void* g_addr_ctx[kMaxDevices] = {nullptr};  // CUDA context current when g_addr[dev] was looked up

// The CUDA context current on this thread (driver cuCtxGetCurrent, fetched
// through the runtime so the library does not link libcuda), or null.
void* current_context() {
  using GetCurrent = int (*)(void**);
  static GetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<GetCurrent>(f);
  }();
  void* c = nullptr;
  if (!fn || fn(&c) != 0) return nullptr;
  return c;
}

int set_err(char* err, size_t len, int code, const char* msg) {
  if (err && len) std::snprintf(err, len, "%s", msg);
  return code;
}

}  // namespace
}  // namespace qpeps

using namespace qpeps;

extern "C" int qpeps_row_step_noalloc(uint32_t n, uint32_t residues, const uint64_t* keys_in, const uint32_t* res_in,
                                      uint64_t n_in, uint64_t* keys_out, uint32_t* res_out, uint64_t out_cap,
                                      void* stream, uint64_t* out_count, uint64_t* weight_residues,
                                      uint64_t* final_residues, char* err, size_t err_len) {
  char buf[256];
  if (n < 1 || n > 21) return set_err(err, err_len, QPEPS_ERR_RANGE, "row step without allocation supports 1 <= N <= 21 (u64 keys)");
  if (residues < 1 || residues > 4) return set_err(err, err_len, QPEPS_ERR_INVALID, "residue count must be in 1..=4");
  if (!out_count || (n_in && (!keys_in || !res_in))) return set_err(err, err_len, QPEPS_ERR_INVALID, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return set_err(err, err_len, QPEPS_ERR_CUDA, "no current CUDA device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    void* ctx = current_context();
    if (!g_addr[dev] || ctx != g_addr_ctx[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_step_scratch);
      if (e != cudaSuccess || !p) {
        std::snprintf(buf, sizeof buf, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        return set_err(err, err_len, QPEPS_ERR_CUDA, buf);
      }
      g_addr[dev] = p;
      g_addr_ctx[dev] = current_context();  // the lookup makes the primary context current if none was
    }
    base = g_addr[dev];
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

  // Scratch layout: [scalars | cursors | partition slots].
  char* scratch = static_cast<char*>(base);
  StepScalars* d_sc = reinterpret_cast<StepScalars*>(scratch);
  const size_t sc_bytes = (sizeof(StepScalars) + 255) / 256 * 256;
  const uint32_t cap = partition_capacity();
  const size_t cb = candidate_bytes((int)residues);
  const size_t slot_bytes_per_part = (size_t)cap * cb + 4;
  const uint64_t max_parts = (kNoAllocScratchBytes - sc_bytes - 256) / slot_bytes_per_part;
  uint32_t* cursors = reinterpret_cast<uint32_t*>(scratch + sc_bytes);
  const size_t cursor_bytes = ((size_t)max_parts * 4 + 255) / 256 * 256;
  void* regions = scratch + sc_bytes + cursor_bytes;

  StepScalars h{};
  FrontierView in{const_cast<uint64_t*>(keys_in), const_cast<uint32_t*>(res_in), n_in};
  LaunchCfg cfg{64, (int)residues, 256, sms};
  cudaError_t e = cudaMemsetAsync(d_sc, 0, sizeof(StepScalars), st);
  if (e == cudaSuccess) e = launch_row_count(cfg, in, n_in, n, d_sc, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    std::snprintf(buf, sizeof buf, "row count: %s", cudaGetErrorString(e));
    return set_err(err, err_len, QPEPS_ERR_CUDA, buf);
  }
  const uint64_t terms = h.terms;
  const uint64_t max_terms = (uint64_t)((double)max_parts * kNoAllocMean);
  if (terms > max_terms) {
    std::snprintf(buf, sizeof buf,
                  "row step has %llu successor terms; the %zu MiB no-allocation scratch holds at most %llu",
                  (unsigned long long)terms, kNoAllocScratchBytes >> 20, (unsigned long long)max_terms);
    return set_err(err, err_len, QPEPS_ERR_CAPACITY, buf);
  }
  if (terms > 0 && (!keys_out || !res_out || out_cap < terms)) {
    std::snprintf(buf, sizeof buf, "output capacity %llu is below the step's %llu successor terms",
                  (unsigned long long)out_cap, (unsigned long long)terms);
    return set_err(err, err_len, QPEPS_ERR_CAPACITY, buf);
  }
  if (terms > 0) {
    // A partition that overflows (hash skew) makes the merge write nothing,
    // so the input is intact and the step can run again with more, emptier
    // partitions while the scratch holds them.
    double mean = kNoAllocMean;
    for (int attempt = 0;; ++attempt) {
      const uint32_t parts = (uint32_t)std::min<uint64_t>(max_parts, (uint64_t)((double)terms / mean) + 1);
      PartitionCfg pc{(int)residues, sms, parts, cap, residues == 1 ? 3 : residues == 2 ? 2 : 1};
      FrontierView out{keys_out, res_out, out_cap};
      e = cudaMemsetAsync(cursors, 0, (size_t)parts * 4, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(d_sc, 0, sizeof(StepScalars), st);
      if (e == cudaSuccess) e = launch_partition_scatter(pc, in, n_in, n, regions, cursors, d_sc, st);
      if (e == cudaSuccess) e = launch_partition_merge(pc, regions, cursors, out, n, true, d_sc, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        std::snprintf(buf, sizeof buf, "row step: %s", cudaGetErrorString(e));
        return set_err(err, err_len, QPEPS_ERR_CUDA, buf);
      }
      if (!h.error) break;
      if (attempt >= 3 || parts >= max_parts)
        return set_err(err, err_len, QPEPS_ERR_CAPACITY, "a hash partition overflowed its slots");
      mean *= 0.75;
    }
  } else {
    std::memset(&h, 0, sizeof h);
  }
  *out_count = h.out_count;
  for (uint32_t r = 0; r < residues; ++r) {
    if (weight_residues) weight_residues[r] = h.weight_sum[r] % kPrimes[r];
    if (final_residues) final_residues[r] = h.final_sum[r] % kPrimes[r];
  }
  if (err && err_len) err[0] = 0;
  return QPEPS_OK;
}

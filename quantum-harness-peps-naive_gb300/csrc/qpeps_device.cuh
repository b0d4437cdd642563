// Device-side building blocks of the boundary store and the key merge.
//
// Boundary key layout (row granularity) is the reference's PackedBoundary
// (src/lib.rs:348-377): bits [0,n) columns, [n,2n) diag_dr, [2n,3n) diag_dl.
// A key is held in `uint64_t` up to N = 22 (the reference layout up to 21, a
// compact layout of the 3n - 2 live bits at 22, see pack/unpack) and in
// `unsigned __int128` otherwise (N <= 42). Mid-row (site granularity) keys
// add the row signal at bit 3n; the u64 form is used for N <= 20 there.
//
// Coefficients are residues modulo up to four primes just below 2^31, so the
// sum of two residues never wraps a u32; CRT on the host rebuilds the exact
// count.
#pragma once

#include <cstdint>

namespace qpeps {

using u32 = uint32_t;
using u64 = uint64_t;
using u128 = unsigned __int128;

constexpr int kMaxResidues = 4;

// The four largest primes below 2^31, in the order the CRT plan takes them.
__host__ __device__ constexpr u32 prime_at(int r) {
  return r == 0 ? 2147483647u : r == 1 ? 2147483629u : r == 2 ? 2147483587u : 2147483579u;
}
constexpr u32 kPrimes[kMaxResidues] = {prime_at(0), prime_at(1), prime_at(2), prime_at(3)};

__host__ __device__ __forceinline__ u32 add_mod(u32 a, u32 b, u32 p) {
  u32 s = a + b;  // a, b < p < 2^31: no wrap
  return s >= p ? s - p : s;
}

// The residue primes are 2^31 - c with c = 1, 19, 61, 69. For x < 2^52 (a sum
// of up to 2^21 residues), (x & (2^31-1)) + c * (x >> 31) is congruent to x and
// below 2p, so one conditional subtraction of p finishes the reduction.
__host__ __device__ __forceinline__ constexpr u32 prime_gap(int r) {
  return r == 0 ? 1u : r == 1 ? 19u : r == 2 ? 61u : 69u;
}
__host__ __device__ __forceinline__ u32 reduce_sum(u64 x, int r) {
  const u64 y = (x & 0x7fffffffull) + (u64)prime_gap(r) * (x >> 31);
  const u32 p = 0x80000000u - prime_gap(r);
  return (u32)(y >= p ? y - p : y);
}

// x mod prime_at(r) for any 64-bit x: two folds of the 2^31 - c form leave a
// value below 2p, then one conditional subtraction.
__host__ __device__ __forceinline__ u32 reduce_u64(u64 x, int r) {
  const u64 c = prime_gap(r);
  const u32 p = 0x80000000u - prime_gap(r);
  u64 y = (x & 0x7fffffffull) + c * (x >> 31);
  y = (y & 0x7fffffffull) + c * (y >> 31);
  return (u32)(y >= p ? y - p : y);
}

// The value below p0 * p1 (< 2^62) with residues (r0 mod p0, r1 mod p1):
// Garner's mixed-radix form of the Chinese remainder theorem,
// value = r0 + p0 * ((r1 - r0) * p0^-1 mod p1).
constexpr u32 kInvP0ModP1 = 2028178983u;
static_assert(((unsigned long long)(prime_at(0) % prime_at(1)) * kInvP0ModP1) % prime_at(1) == 1,
              "kInvP0ModP1 must invert p0 modulo p1");
__host__ __device__ __forceinline__ u64 crt_fold2(u32 r0, u32 r1) {
  constexpr u32 p1 = prime_at(1);
  const u32 r0m = r0 >= p1 ? r0 - p1 : r0;
  const u32 d = r1 >= r0m ? r1 - r0m : r1 + (p1 - r0m);
  const u32 t = reduce_u64((u64)d * kInvP0ModP1, 1);
  return (u64)r0 + (u64)prime_at(0) * t;
}

// Fibonacci hashing (Knuth, multiplicative): the high bits of key * odd
// constant. Two different multipliers give independent partition and slot
// indices.
__host__ __device__ __forceinline__ u64 fib_hash_a(u64 k) { return k * 0x9E3779B97F4A7C15ull; }
__host__ __device__ __forceinline__ u64 fib_hash_b(u64 k) { return k * 0xD6E8FEB86659FD93ull; }

__host__ __device__ __forceinline__ u32 mul_mod(u32 a, u32 b, u32 p) {
  return (u32)(((u64)a * (u64)b) % p);
}

// splitmix64 finaliser: a bijective 64-bit mixer (Steele, Lea, Flood 2014).
__host__ __device__ __forceinline__ u64 mix64(u64 x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}

template <typename K>
__host__ __device__ __forceinline__ u64 key_hash(K k);
template <>
__host__ __device__ __forceinline__ u64 key_hash<u64>(u64 k) {
  return mix64(k);
}
template <>
__host__ __device__ __forceinline__ u64 key_hash<u128>(u128 k) {
  return mix64((u64)k ^ mix64((u64)(k >> 64) + 0x9e3779b97f4a7c15ULL));
}

// ---- packed boundary -------------------------------------------------------

struct State {
  u64 cols, dr, dl;
};

// Key layouts. u128 keys and u64 keys up to N = 21 hold the reference's
// PackedBoundary layout (src/lib.rs:348-377): columns in bits [0, n), the
// down-right diagonal signals in [n, 2n), the down-left ones in [2n, 3n).
// A row step shifts the down-right signals up and the down-left ones down, so
// every boundary after a row has dr bit 0 and dl bit n - 1 clear: only 3n - 2
// bits are live. At N = 22 a u64 key holds exactly those (compact layout):
// columns [0, 22), dr bits 1..21 in [22, 43), dl bits 0..20 in [43, 64).
constexpr unsigned kRefU64MaxN = 21;  // widest board with the reference layout in a u64 key
constexpr unsigned kU64MaxN = 22;     // widest board a u64 key holds (compact layout)

// For u64 keys both layouts are one formula with c = 1 (compact) or 0
// (reference) and the same operations as the reference layout alone: the
// down-right field starts at bit n - c (its always-clear bit 0 lands on the
// top column bit and is masked off when read back) and the down-left field at
// 2n - c (its always-clear top bit leaves the word). No branch, and no extra
// operation per key, in the kernels' inner loops.
template <typename K>
__host__ __device__ __forceinline__ State unpack(K key, unsigned n, u64 mask) {
  State s;
  s.cols = (u64)key & mask;
  if constexpr (sizeof(K) == 8) {
    const unsigned c = n > kRefU64MaxN ? 1u : 0u;
    s.dr = ((u64)key >> (n - c)) & (mask & ~(u64)c);
    s.dl = ((u64)key >> (2 * n - c)) & mask;
  } else {
    s.dr = (u64)(key >> n) & mask;
    s.dl = (u64)(key >> (2 * n)) & mask;
  }
  return s;
}

// dr bit 0 and dl bit n - 1 must be clear at N = 22 with u64 keys (true of
// every boundary state: the empty one and every row successor).
template <typename K>
__host__ __device__ __forceinline__ K pack(u64 cols, u64 dr, u64 dl, unsigned n) {
  if constexpr (sizeof(K) == 8) {
    const unsigned c = n > kRefU64MaxN ? 1u : 0u;
    return (K)(cols | (dr << (n - c)) | (dl << (2 * n - c)));
  } else {
    return (K)cols | ((K)dr << n) | ((K)dl << (2 * n));
  }
}

// Compiled row successor (src/lib.rs:600-638 after certification): place the
// occupied C entry at free column `bit`, then move the diagonal signals to
// their next-row positions. Signals leaving the board are contracted with v2.
template <typename K>
__host__ __device__ __forceinline__ K row_successor(const State& s, u64 bit, unsigned n, u64 mask) {
  return pack<K>(s.cols | bit, ((s.dr | bit) << 1) & mask, (s.dl | bit) >> 1, n);
}

// C entries matched by the reference's per-parent sitewise row kernel
// (contract_one_row_sitewise, src/lib.rs:513-592, counters at 538-541) for a
// parent whose free columns are `fr`: the partial row that has placed no queen
// yet matches two entries at a free column (pass through or place) and one
// elsewhere; every partial that has placed its queen matches one entry per
// later column. Summed over the n columns: n + f + sum over free b of
// (n - 1 - b) = n + f * n - (sum of the free column indices), f = popcount.
__host__ __device__ __forceinline__ u64 sitewise_entries(u64 fr, unsigned n) {
  u64 idx_sum = 0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const u64 m = j == 0 ? 0xAAAAAAAAAAAAAAAAull : j == 1 ? 0xCCCCCCCCCCCCCCCCull : j == 2 ? 0xF0F0F0F0F0F0F0F0ull
                : j == 3 ? 0xFF00FF00FF00FF00ull : j == 4 ? 0xFFFF0000FFFF0000ull : 0xFFFFFFFF00000000ull;
#if defined(__CUDA_ARCH__)
    idx_sum += (u64)__popcll(fr & m) << j;
#else
    idx_sum += (u64)__builtin_popcountll(fr & m) << j;
#endif
  }
#if defined(__CUDA_ARCH__)
  const u64 f = (u64)__popcll(fr);
#else
  const u64 f = (u64)__builtin_popcountll(fr);
#endif
  return (u64)n + f * n - idx_sum;
}

// ---- key layouts of the partitioned merge ----------------------------------
//
// FixedLayout: one board size, the reference's PackedBoundary bit layout.
// SlotLayout: serving. Requests of different board sizes share one boundary;
// each field is 19 bits wide (N <= 19) and bits [57, 63) hold the request's
// slot, so entries of different requests never compare equal and never merge.
// Bit 63 stays clear, keeping ~0 free as the empty-slot marker.

struct FixedLayout {
  static constexpr bool kSlotted = false;
  unsigned n;
  u64 mask;
  __device__ __forceinline__ u64 mask_of(u64) const { return mask; }
  __device__ __forceinline__ State unpack(u64 key) const { return qpeps::unpack<u64>(key, n, mask); }
  __device__ __forceinline__ u64 successor(u64, const State& s, u64 bit) const {
    return row_successor<u64>(s, bit, n, mask);
  }
  __device__ __forceinline__ unsigned slot(u64) const { return 0; }
};

constexpr unsigned kServeFieldBits = 19;
constexpr unsigned kServeSlotShift = 57;
constexpr unsigned kServeMaxSlots = 64;

struct SlotLayout {
  static constexpr bool kSlotted = true;
  const u64* slot_mask;              // board mask per slot
  unsigned long long* slot_final;    // [kServeMaxSlots][4] residue sums of finished boards
  __device__ __forceinline__ u64 mask_of(u64 key) const { return slot_mask[key >> kServeSlotShift]; }
  __device__ __forceinline__ State unpack(u64 key) const {
    const u64 m = mask_of(key);
    State s;
    s.cols = key & m;
    s.dr = (key >> kServeFieldBits) & m;
    s.dl = (key >> (2 * kServeFieldBits)) & m;
    return s;
  }
  __device__ __forceinline__ u64 successor(u64 key, const State& s, u64 bit) const {
    const u64 m = mask_of(key);
    return (key & (63ull << kServeSlotShift)) | (s.cols | bit) | ((((s.dr | bit) << 1) & m) << kServeFieldBits) |
           (((s.dl | bit) >> 1) << (2 * kServeFieldBits));
  }
  __device__ __forceinline__ unsigned slot(u64 key) const { return (unsigned)(key >> kServeSlotShift); }
};

__host__ __device__ __forceinline__ u64 serve_key(unsigned slot, u64 cols, u64 dr, u64 dl) {
  return ((u64)slot << kServeSlotShift) | cols | (dr << kServeFieldBits) | (dl << (2 * kServeFieldBits));
}

// ---- hash table slots --------------------------------------------------------
//
// A slot holds the bitwise complement of the key (so an all-zero slot is empty
// and one memset clears the table; no valid key is all ones because its top
// bit is never used) and one u64 accumulator per residue. Each contribution is
// < 2^31 and at most 4N parents reach one key in a step, so an accumulator
// never wraps; it is reduced modulo its prime when the table is compacted.

template <typename K, int R>
struct SlotBytes {
  static constexpr int raw = (int)sizeof(K) + 8 * R;
  static constexpr int value = raw <= 16 ? 16 : raw <= 32 ? 32 : 64;
};

template <typename K, int R>
struct alignas(SlotBytes<K, R>::value) Slot {
  K nkey;
  u64 acc[R];
};

__device__ __forceinline__ u64 atomic_cas_key(u64* addr, u64 cmp, u64 val) {
  return (u64)atomicCAS((unsigned long long*)addr, (unsigned long long)cmp, (unsigned long long)val);
}

// 128-bit compare-and-swap (PTX atom.cas.b128, sm_90 and later).
__device__ __forceinline__ u128 atomic_cas_key(u128* addr, u128 cmp, u128 val) {
  u64 cl = (u64)cmp, ch = (u64)(cmp >> 64), vl = (u64)val, vh = (u64)(val >> 64);
  u64 ol, oh;
  asm volatile(
      "{\n\t.reg .b128 c, v, d;\n\t"
      "mov.b128 c, {%2, %3};\n\t"
      "mov.b128 v, {%4, %5};\n\t"
      "atom.global.cas.b128 d, [%6], c, v;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(ol), "=l"(oh)
      : "l"(cl), "l"(ch), "l"(vl), "l"(vh), "l"(addr)
      : "memory");
  return ((u128)oh << 64) | ol;
}

__device__ __forceinline__ u64 load_key_cg(const u64* p) { return __ldcg((const unsigned long long*)p); }
__device__ __forceinline__ u128 load_key_cg(const u128* p) {
  ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(p));
  return ((u128)v.y << 64) | v.x;
}

// Error flags written by kernels (bit set in ErrorState::flags).
enum ErrorBits : u32 {
  kErrProbeLimit = 1u,  // hash probe sequence exceeded its bound (table too full)
  kErrOverflow = 2u,    // a bounded structure overflowed its capacity
  kErrWaitLimit = 4u,   // a bounded spin-wait gave up
  kErrBounds = 8u,      // an index fell outside its buffer; the access was skipped
};

// Insert one contribution into the global table with linear probing.
// Returns false (and sets kErrProbeLimit) if `max_probe` slots were visited.
template <typename K, int R>
__device__ __forceinline__ bool table_insert(Slot<K, R>* __restrict__ table, u64 mask, K key, const u32 (&w)[R],
                                             u32 max_probe, u32* err) {
  const K nk = ~key;
  u64 pos = key_hash<K>(key) & mask;
  for (u32 probe = 0; probe < max_probe; ++probe) {
    Slot<K, R>* s = &table[pos];
    K cur = load_key_cg(&s->nkey);
    if (cur == (K)0) {
      cur = atomic_cas_key(&s->nkey, (K)0, nk);
      if (cur == (K)0) cur = nk;
    }
    if (cur == nk) {
#pragma unroll
      for (int r = 0; r < R; ++r) atomicAdd((unsigned long long*)&s->acc[r], (unsigned long long)w[r]);
      return true;
    }
    pos = (pos + 1) & mask;
  }
  atomicOr(err, kErrProbeLimit);
  return false;
}

}  // namespace qpeps

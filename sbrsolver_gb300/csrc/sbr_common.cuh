// Warp-level helpers and the device hash tables shared by the SBR kernels.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_kernels.cuh"

namespace sbr {

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated slot reservation: every active lane asks for `cnt` (0..2)
// entries; one atomicAdd per warp.
__device__ __forceinline__ unsigned long long warp_reserve(unsigned long long* ctr, unsigned cnt) {
  const unsigned mask = __activemask();
  const unsigned b1 = __ballot_sync(mask, cnt >= 1);
  const unsigned b2 = __ballot_sync(mask, cnt >= 2);
  const unsigned lt = (1u << lane_id()) - 1u;
  const unsigned before = __popc(b1 & lt) + __popc(b2 & lt);
  const unsigned total = __popc(b1) + __popc(b2);
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane_id() == unsigned(leader) && total) base = atomicAdd(ctr, (unsigned long long)total);
  base = __shfl_sync(mask, base, leader);
  return base + before;
}

// Open addressing with linear probing.  Tables are kept at most half full
// (the host grows them between solves from the occupancy counters), so a
// probe run longer than kMaxProbe means the table is too small: the insert
// reports overflow and the solve is repeated with a larger table.
constexpr uint32_t kMaxProbe = 256;

__device__ __forceinline__ uint32_t ht_insert(HashTable t, unsigned long long key, unsigned* ov,
                                              unsigned bit, unsigned long long* used,
                                              unsigned long long* lost, bool* fresh = nullptr) {
  uint32_t h = uint32_t(mix64(key)) & t.mask;
  const uint32_t lim = min(kMaxProbe, t.mask + 1);
  for (uint32_t i = 0; i < lim; ++i) {
    unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&t.keys[h]);
    if (k == key) return h;
    if (k == kEmptyKey) {
      unsigned long long old = atomicCAS(&t.keys[h], kEmptyKey, key);
      if (old == kEmptyKey) {
        atomicAdd(used, 1ull);
        if (fresh) *fresh = true;
        return h;
      }
      if (old == key) return h;
    }
    h = (h + 1) & t.mask;
  }
  atomicOr(ov, bit);
  atomicAdd(lost, 1ull);
  return 0xFFFFFFFFu;
}

// Find or claim key's slot in a table that may fill up: the slot, or
// 0xFFFFFFFF when a probe run of `limit` slots finds neither (the caller then
// works without the table).  fresh: this call claimed the slot.
__device__ __forceinline__ uint32_t ht_claim(HashTable t, unsigned long long key, uint32_t limit,
                                             bool& fresh) {
  fresh = false;
  uint32_t h = uint32_t(mix64(key)) & t.mask;
  const uint32_t lim = min(limit, t.mask + 1);
  for (uint32_t i = 0; i < lim; ++i) {
    unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&t.keys[h]);
    if (k == key) return h;
    if (k == kEmptyKey) {
      const unsigned long long old = atomicCAS(&t.keys[h], kEmptyKey, key);
      if (old == kEmptyKey) {
        fresh = true;
        return h;
      }
      if (old == key) return h;
    }
    h = (h + 1) & t.mask;
  }
  return 0xFFFFFFFFu;
}

__device__ __forceinline__ uint32_t ht_find(HashTable t, unsigned long long key) {
  uint32_t h = uint32_t(mix64(key)) & t.mask;
  const uint32_t lim = min(kMaxProbe, t.mask + 1);
  for (uint32_t i = 0; i < lim; ++i) {
    unsigned long long k = t.keys[h];
    if (k == key) return h;
    if (k == kEmptyKey) return 0xFFFFFFFFu;
    h = (h + 1) & t.mask;
  }
  return 0xFFFFFFFFu;
}

__global__ void k_fill_u64(unsigned long long* p, size_t n, unsigned long long v) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

}  // namespace sbr

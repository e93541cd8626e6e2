// Exact merging of identical rows between plain layers (SNICIT mode).
//
// Every row is computed independently of the others, in a fixed FP32 order
// (the same slots, the same FMA sequence, whatever tile or kernel instance
// holds it), so two rows that are bitwise equal after layer l stay bitwise
// equal through every later layer and end in the same category.  On the SDGC
// workloads the surviving rows collapse onto a handful of fixed points well
// before the threshold layer; SNICIT's clustering finds them at the threshold
// (zero residues), this step finds them as soon as they appear and drops all
// but one copy from the row list, with no approximation:
//
//  1. dedup_hash_kernel: one warp per listed row hashes the row's bits (two
//     32-bit streams, fixed lane order) and inserts the 64-bit key into an
//     open-addressed table (linear probing with atomicCAS; the table has at
//     least twice as many entries as rows, so a probe always ends); the
//     smallest row id per key wins the slot (atomicMin), which makes the kept
//     row -- and so everything downstream -- independent of thread timing;
//  2. dedup_verify_kernel: a row whose slot names another row compares the
//     two rows bit for bit; equal -> alias[r] = that row and r leaves the
//     list; unequal (a hash collision) -> r stays;
//  3. dedup_finish_kernel: copies the compacted list back, stores its count
//     and returns the touched table entries to empty.
//
// At the end of the inference resolve_alias_kernel points every merged row at
// the root of its chain and copies the root's category; activations and head
// outputs of merged rows are read through alias (materialize, head).
#include <cstdint>

#include "sdnn_internal.h"

namespace sdnn {

namespace {

constexpr int32_t kEmptyRep = 0x7F7F7F7F;  // byte-fill value of an idle slot_rep entry

// MurmurHash3's 32-bit finaliser (Appleby, public domain).
__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

__device__ __forceinline__ void mix_in(uint32_t& h1, uint32_t& h2, uint32_t v) {
  h1 = (h1 ^ v) * 0x9E3779B1u;
  h2 = (h2 + v) * 0x85EBCA77u;
  h2 ^= h2 >> 15;
}

__global__ void dedup_hash_kernel(const DedupArgs a) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int n = *a.count;
  if (blockIdx.x == 0 && threadIdx.x == 0) a.tmp_count[0] = 0;
  const bool vec = (a.N & 3) == 0;
  for (int i = wid; i < n; i += nw) {
    const int r = a.list[i];
    const float* row = a.y + (size_t)r * a.N;
    uint32_t h1 = 0x243F6A88u, h2 = 0xB7E15162u;
    if (vec) {
      // eight 16-byte loads in flight per lane, then the mixing (a few rows
      // alone are otherwise one memory round trip per 512 bytes)
      const uint4* p = reinterpret_cast<const uint4*>(row);
      const int n4 = a.N >> 2;
      int j = lane;
      for (; j + 7 * 32 < n4; j += 8 * 32) {
        uint4 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = __ldg(p + j + k * 32);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          mix_in(h1, h2, v[k].x);
          mix_in(h1, h2, v[k].y);
          mix_in(h1, h2, v[k].z);
          mix_in(h1, h2, v[k].w);
        }
      }
      for (; j < n4; j += 32) {
        const uint4 v = __ldg(p + j);
        mix_in(h1, h2, v.x);
        mix_in(h1, h2, v.y);
        mix_in(h1, h2, v.z);
        mix_in(h1, h2, v.w);
      }
    } else {
      const uint32_t* p = reinterpret_cast<const uint32_t*>(row);
      for (int j = lane; j < a.N; j += 32) mix_in(h1, h2, __ldg(p + j));
    }
    uint32_t v1 = fmix32(h1 + (uint32_t)lane * 0x27D4EB2Fu);
    uint32_t v2 = fmix32(h2 ^ ((uint32_t)lane * 0x165667B1u + 1u));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v1 ^= __shfl_xor_sync(0xffffffffu, v1, o);
      v2 ^= __shfl_xor_sync(0xffffffffu, v2, o);
    }
    if (lane == 0) {
      unsigned long long key = ((unsigned long long)v1 << 32) | v2;
      if (key == 0ull) key = 1ull;  // 0 marks an empty entry
      uint32_t slot = (uint32_t)(key >> 17) & a.mask;
      // at most mask + 1 probes; the table holds >= 2x the listed rows
      for (uint32_t probe = 0; probe <= a.mask; ++probe) {
        const unsigned long long old = atomicCAS(a.table + slot, 0ull, key);
        if (old == 0ull || old == key) break;
        slot = (slot + 1u) & a.mask;
      }
      a.pos_slot[i] = (int32_t)slot;
      atomicMin(a.slot_rep + slot, r);
    }
  }
}

__global__ void dedup_verify_kernel(const DedupArgs a) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int n = *a.count;
  if (blockIdx.x == 0 && threadIdx.x == 0) a.tmp_count[1] = n;
  const bool vec = (a.N & 3) == 0;
  for (int i = wid; i < n; i += nw) {
    const int r = a.list[i];
    const int rep = a.slot_rep[a.pos_slot[i]];
    bool keep = true;
    if (rep != r && rep >= 0 && rep != kEmptyRep) {
      bool same = true;
      if (vec) {
        const uint4* p = reinterpret_cast<const uint4*>(a.y + (size_t)r * a.N);
        const uint4* q = reinterpret_cast<const uint4*>(a.y + (size_t)rep * a.N);
        const int n4 = a.N >> 2;
        int j = lane;
        for (; j + 3 * 32 < n4; j += 4 * 32) {
          uint4 u[4], v[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            u[k] = __ldg(p + j + k * 32);
            v[k] = __ldg(q + j + k * 32);
          }
#pragma unroll
          for (int k = 0; k < 4; ++k)
            same &= u[k].x == v[k].x && u[k].y == v[k].y && u[k].z == v[k].z && u[k].w == v[k].w;
        }
        for (; j < n4; j += 32) {
          const uint4 u = __ldg(p + j), v = __ldg(q + j);
          same &= u.x == v.x && u.y == v.y && u.z == v.z && u.w == v.w;
        }
      } else {
        const uint32_t* p = reinterpret_cast<const uint32_t*>(a.y + (size_t)r * a.N);
        const uint32_t* q = reinterpret_cast<const uint32_t*>(a.y + (size_t)rep * a.N);
        for (int j = lane; j < a.N; j += 32) same &= __ldg(p + j) == __ldg(q + j);
      }
      if (__all_sync(0xffffffffu, same)) {
        keep = false;
        if (lane == 0) a.alias[r] = rep;
      }
    }
    if (keep && lane == 0) a.tmp_list[atomicAdd(a.tmp_count, 1)] = r;
  }
}

__global__ void dedup_finish_kernel(const DedupArgs a) {
  const int old_n = a.tmp_count[1], new_n = a.tmp_count[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < old_n; i += gridDim.x * blockDim.x) {
    const int slot = a.pos_slot[i];
    a.table[slot] = 0ull;
    a.slot_rep[slot] = kEmptyRep;
    if (i < new_n) a.list[i] = a.tmp_list[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.count = new_n;
}

__global__ void resolve_alias_kernel(const int32_t* nrows, int32_t* alias, int32_t* flags,
                                     int32_t max_depth) {
  const int n = *nrows;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    int x = alias[r];
    if (x < 0) continue;
    // chains only point at smaller row ids, one link per merge step
    for (int d = 0; d < max_depth; ++d) {
      const int y = alias[x];
      if (y < 0) break;
      x = y;
    }
    alias[r] = x;
    if (flags) flags[r] = flags[x];
  }
}

}  // namespace

void launch_dedup(const DedupArgs& a, int num_sms, cudaStream_t s) {
  const int grid = num_sms * 8;
  dedup_hash_kernel<<<grid, 256, 0, s>>>(a);
  dedup_verify_kernel<<<grid, 256, 0, s>>>(a);
  dedup_finish_kernel<<<num_sms * 2, 256, 0, s>>>(a);
}

void launch_resolve_alias(const int32_t* nrows, int32_t* alias, int32_t* flags, int32_t max_depth,
                          cudaStream_t s) {
  resolve_alias_kernel<<<264, 256, 0, s>>>(nrows, alias, flags, max_depth);
}

}  // namespace sdnn

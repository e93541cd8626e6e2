// First-layer kernel for binary inputs (the SDGC input images are 0/1).
//
// When every input of a row is 0 or 1 and the layer has one common weight
// value w, the pre-activation of output c is S(k) + b, where k is the number
// of active in-edges of c and S(k) is w added k times in FP32 -- exactly what
// the float gather (layer_kernel, which adds w * 1 or w * 0 slot by slot)
// computes.  This kernel therefore counts instead of multiplying:
//
//  * a CTA owns 32 rows; warps read the rows coalesced (16-byte loads, 8 rows
//    in flight per lane) and build, for every input j, one 32-bit word whose
//    bit t is input j of row t (shared memory, N + 32 words, the last 32 zero
//    for the padding slots; N is a multiple of 128);
//  * lane i of a warp owns output 32g + i and walks the same bank-scheduled
//    slots as layer_kernel, loading one word per slot (one wavefront per slot
//    for all 32 rows) and adding it into bit-sliced counters with a
//    Harley-Seal carry-save tree (15 full adders per 16 slots);
//  * the epilogue extracts each row's count, looks up S(k) (a 128-entry table
//    built on the host with the same FP32 additions), adds the bias, clamps,
//    stores row t coalesced and ballots survivors into the next row list.
//
// A tile holding any value other than 0 or 1 is not computed here: its rows
// go to a fallback list that the float kernel processes right after.
#include <algorithm>
#include <cstdint>
#include "layer_kernel.cuh"

namespace sdnn {

__device__ __forceinline__ void csa(uint32_t& h, uint32_t& l, uint32_t a, uint32_t b, uint32_t c) {
  const uint32_t u = a ^ b;
  h = (a & b) | (u & c);
  l = u ^ c;
}

// Bit-sliced counters c[0..6] (c[i] bit t = bit i of row t's count) plus 16,
// 8 or 4 words, each word adding 1 to the rows whose bit is set: Harley-Seal
// carry-save trees, the carry out of the tree rippled into the higher planes.
__device__ __forceinline__ void ripple(uint32_t (&c)[7], int from, uint32_t cy) {
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    if (i < from) continue;
    const uint32_t t = c[i] & cy;
    c[i] ^= cy;
    cy = t;
  }
}
__device__ __forceinline__ void add16(uint32_t (&c)[7], const uint32_t (&w)[16]) {
  uint32_t twosA, twosB, foursA, foursB, eightsA, eightsB, c16;
  csa(twosA, c[0], c[0], w[0], w[1]);
  csa(twosB, c[0], c[0], w[2], w[3]);
  csa(foursA, c[1], c[1], twosA, twosB);
  csa(twosA, c[0], c[0], w[4], w[5]);
  csa(twosB, c[0], c[0], w[6], w[7]);
  csa(foursB, c[1], c[1], twosA, twosB);
  csa(eightsA, c[2], c[2], foursA, foursB);
  csa(twosA, c[0], c[0], w[8], w[9]);
  csa(twosB, c[0], c[0], w[10], w[11]);
  csa(foursA, c[1], c[1], twosA, twosB);
  csa(twosA, c[0], c[0], w[12], w[13]);
  csa(twosB, c[0], c[0], w[14], w[15]);
  csa(foursB, c[1], c[1], twosA, twosB);
  csa(eightsB, c[2], c[2], foursA, foursB);
  csa(c16, c[3], c[3], eightsA, eightsB);
  ripple(c, 4, c16);
}
__device__ __forceinline__ void add8(uint32_t (&c)[7], const uint32_t* w) {
  uint32_t twosA, twosB, foursA, foursB, eights;
  csa(twosA, c[0], c[0], w[0], w[1]);
  csa(twosB, c[0], c[0], w[2], w[3]);
  csa(foursA, c[1], c[1], twosA, twosB);
  csa(twosA, c[0], c[0], w[4], w[5]);
  csa(twosB, c[0], c[0], w[6], w[7]);
  csa(foursB, c[1], c[1], twosA, twosB);
  csa(eights, c[2], c[2], foursA, foursB);
  ripple(c, 3, eights);
}
__device__ __forceinline__ void add4(uint32_t (&c)[7], const uint32_t* w) {
  uint32_t twosA, twosB, fours;
  csa(twosA, c[0], c[0], w[0], w[1]);
  csa(twosB, c[0], c[0], w[2], w[3]);
  csa(fours, c[1], c[1], twosA, twosB);
  ripple(c, 2, fours);
}

// Bit words of the slots of K blocks (block b0 onwards; indices ip, lane-
// strided) from the shared row `bits` (BYTES: indices are byte offsets).
template <bool BYTES, int K>
__device__ __forceinline__ void gather_words(uint32_t* w, const uint2* __restrict__ ip, int b0,
                                             const uint32_t* bits) {
  uint2 iv[K];
#pragma unroll
  for (int k = 0; k < K; ++k) iv[k] = __ldg(ip + (size_t)(b0 + k) * 32);
#pragma unroll
  for (int k = 0; k < K; ++k) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const uint32_t j = ((s < 2 ? iv[k].x : iv[k].y) >> ((s & 1) * 16)) & 0xffffu;
      w[k * 4 + s] = BYTES ? *reinterpret_cast<const uint32_t*>(
                                 reinterpret_cast<const char*>(bits) + j)
                           : bits[j];
    }
  }
}

// Adds the slots of a list of nb blocks into the counters: 4 blocks at a
// time, then 2, then 1 (no adder work on blocks past the list's end).
template <bool BYTES>
__device__ __forceinline__ void count_list(uint32_t (&c)[7], const uint2* __restrict__ ip, int nb,
                                           const uint32_t* bits) {
  int b = 0;
  for (; b + 4 <= nb; b += 4) {
    uint32_t w[16];
    gather_words<BYTES, 4>(w, ip, b, bits);
    add16(c, w);
  }
  if (b + 2 <= nb) {
    uint32_t w[8];
    gather_words<BYTES, 2>(w, ip, b, bits);
    add8(c, w);
    b += 2;
  }
  if (b < nb) {
    uint32_t w[4];
    gather_words<BYTES, 1>(w, ip, b, bits);
    add4(c, w);
  }
}

// ---- epilogue: per-row counts out of the bit-sliced counters ----------------
//
// Rows of a tile are bits of the counter planes P[0..6] (P[i] bit t = bit i of
// row t's count).  With a scalar bias the output of a row depends on its count
// only, through a 128-entry table, and the rows that survive are those whose
// count lies in an interval, so:
//  * the survivor mask of all 32 rows comes from bitwise comparisons of the
//    planes with the interval's end (no per-row vote);
//  * the counts come out four 8 x 8 bit-matrix transposes (plane bytes ->
//    row bytes; the three-step transpose of Hacker's Delight, section 7-3).

// Rows whose count is >= k0 (k0 in 0..128).
__device__ __forceinline__ uint32_t count_ge(const uint32_t (&P)[7], uint32_t k0) {
  if (k0 >= 128u) return 0u;
  uint32_t gt = 0u, eq = 0xffffffffu;
#pragma unroll
  for (int i = 6; i >= 0; --i) {
    if ((k0 >> i) & 1u) eq &= P[i];
    else gt |= eq & P[i];
  }
  return gt | eq;
}

__device__ __forceinline__ unsigned long long transpose8x8(unsigned long long x) {
  unsigned long long t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
  x = x ^ t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
  x = x ^ t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
  x = x ^ t ^ (t << 28);
  return x;
}

// Byte b of each of the planes P[0..6] (plane 7 = 0) as one 64-bit word.
__device__ __forceinline__ unsigned long long plane_bytes(const uint32_t (&P)[7], int b) {
  const uint32_t sel = (uint32_t)b | ((uint32_t)(b + 4) << 4);
  const uint32_t p01 = __byte_perm(P[0], P[1], sel), p23 = __byte_perm(P[2], P[3], sel);
  const uint32_t p45 = __byte_perm(P[4], P[5], sel), p67 = __byte_perm(P[6], 0u, sel);
  const uint32_t lo = __byte_perm(p01, p23, 0x5410), hi = __byte_perm(p45, p67, 0x5410);
  return ((unsigned long long)hi << 32) | lo;
}

// Survivor interval of the counts for a scalar bias: kind 1 = [k0, 127],
// kind 2 = [0, k1]; kind 0 = per-neuron bias or no interval (generic path).
struct CountInterval {
  int kind;
  uint32_t lo, hi;
};

__device__ CountInterval count_interval(const float* s_sum, float bias, bool per_neuron) {
  __shared__ uint32_t s_alive[4];
  __shared__ CountInterval s_iv;
  const int tid = threadIdx.x;
  if (tid < 128) {
    const uint32_t m = __ballot_sync(0xffffffffu, s_sum[tid] + bias > 0.f);
    if ((tid & 31) == 0) s_alive[tid >> 5] = m;
  }
  __syncthreads();
  if (tid == 0) {
    CountInterval iv{0, 0u, 0u};
    if (!per_neuron) {
      // alive counts as a 128-bit set; suffix [k0, 127] or prefix [0, k1]?
      int first = -1, last = -1;
      for (int k = 0; k < 128; ++k)
        if ((s_alive[k >> 5] >> (k & 31)) & 1u) {
          if (first < 0) first = k;
          last = k;
        }
      int n = 0;
      for (int w = 0; w < 4; ++w) n += __popc(s_alive[w]);
      if (first < 0) {
        iv = {1, 128u, 0u};  // nothing survives: k >= 128 never holds
      } else if (n == last - first + 1 && last == 127) {
        iv = {1, (uint32_t)first, 0u};
      } else if (n == last - first + 1 && first == 0) {
        iv = {2, 0u, (uint32_t)last};
      }
    }
    s_iv = iv;
  }
  __syncthreads();
  return s_iv;
}

// Outputs of one group for the rows of a tile from its counters.
__device__ __forceinline__ uint32_t bits_epilogue(const uint32_t (&P)[7], const Layer0Args& a,
                                                  const float* s_sum, const float* s_val,
                                                  const CountInterval& iv, const int32_t* s_rows,
                                                  int nrows, int c_out, int lane) {
  const int N = a.N;
  uint32_t m = 0;
  if (iv.kind != 0) {
    const uint32_t rows_mask = nrows >= 32 ? 0xffffffffu : ((1u << nrows) - 1u);
    uint32_t alive = iv.kind == 1 ? count_ge(P, iv.lo) : ~count_ge(P, iv.hi + 1u);
    m = __reduce_or_sync(0xffffffffu, alive & rows_mask);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      if (8 * b >= nrows) break;
      const unsigned long long x = transpose8x8(plane_bytes(P, b));
#pragma unroll
      for (int tp = 0; tp < 8; ++tp) {
        const int t = 8 * b + tp;
        if (t < nrows) {
          const uint32_t k = (uint32_t)(x >> (8 * tp)) & 0x7fu;
          a.y_out[(size_t)s_rows[t] * N + c_out] = s_val[k];
        }
      }
    }
    return m;
  }
  const float bc = a.bias_vec ? __ldg(a.bias_vec + c_out) : a.bias;
  for (int t = 0; t < nrows; ++t) {
    uint32_t k = 0;
#pragma unroll
    for (int i = 0; i < 7; ++i) k |= ((P[i] >> t) & 1u) << i;
    const float v = s_sum[k] + bc;
    a.y_out[(size_t)s_rows[t] * N + c_out] = clampf(v, a.clampv);
    if (__any_sync(0xffffffffu, v > 0.f)) m |= 1u << t;
  }
  return m;
}

// 256 threads, three CTAs per SM: the register budget that keeps three tiles'
// row loads in flight per SM (the kernel waits on those loads, not on issue)
template <int RSW>
__global__ void __launch_bounds__(256, 3) layer0_bits_kernel(const Layer0Args a) {
  extern __shared__ __align__(128) uint32_t bits[];  // RSW words
  __shared__ float s_sum[128];
  __shared__ float s_val[128];  // output of a row with count k (scalar bias)
  __shared__ int32_t s_rows[32];
  __shared__ uint32_t s_mask;
  __shared__ int32_t s_nonbin;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int N = a.N;
  const int count = *a.count_in;
  const int n_tiles = (count + 31) / 32;
  if (tid < 128) {
    s_sum[tid] = a.sums[tid];
    s_val[tid] = clampf(a.sums[tid] + a.bias, a.clampv);
  }
  for (int i = N + tid; i < RSW; i += blockDim.x) bits[i] = 0u;
  __syncthreads();
  const CountInterval iv = count_interval(s_sum, a.bias, a.bias_vec != nullptr);

  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int row0 = tile * 32;
    const int nrows = min(32, count - row0);
    __syncthreads();
    if (tid < 32) s_rows[tid] = tid < nrows ? a.list_in[row0 + tid] : -1;
    if (tid == 0) {
      s_mask = 0;
      s_nonbin = 0;
    }
    __syncthreads();
    // transpose 32 rows into per-input bit words: lane takes 4 consecutive
    // inputs (one 16-byte load per row), 8 rows of loads in flight at a time
    bool nonbin = false;
    for (int j0 = warp * 128; j0 < N; j0 += nwarps * 128) {
      const int j = j0 + lane * 4;
      uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
      for (int t0 = 0; t0 < nrows; t0 += 8) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (t0 + u < nrows)
            v[u] = __ldg(reinterpret_cast<const float4*>(a.y_in + (size_t)s_rows[t0 + u] * N + j));
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (t0 + u < nrows) {
            const float x[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
            for (int q = 0; q < 4; ++q) nonbin |= (x[q] != 0.f) && (x[q] != 1.f);
            const uint32_t bit = 1u << (t0 + u);
            w0 |= x[0] != 0.f ? bit : 0u;
            w1 |= x[1] != 0.f ? bit : 0u;
            w2 |= x[2] != 0.f ? bit : 0u;
            w3 |= x[3] != 0.f ? bit : 0u;
          }
        }
      }
      *reinterpret_cast<uint4*>(bits + j) = make_uint4(w0, w1, w2, w3);
    }
    if (__any_sync(0xffffffffu, nonbin) && lane == 0) s_nonbin = 1;
    __syncthreads();
    if (s_nonbin) {
      if (tid < nrows) {
        const int pos = atomicAdd(a.fallback_count, 1);
        a.fallback_list[pos] = s_rows[tid];
      }
      continue;
    }
    uint32_t m = 0;
    for (int g = warp; g < a.G; g += nwarps) {
      const int32_t b0 = __ldg(a.grp_blk + g);
      const int32_t b1 = __ldg(a.grp_blk + g + 1);
      const uint2* __restrict__ ip = a.idx + (size_t)b0 * 32 + lane;
      uint32_t P[7] = {0u, 0u, 0u, 0u, 0u, 0u, 0u};
      count_list<rsw_in_bytes(RSW)>(P, ip, b1 - b0, bits);
      m |= bits_epilogue(P, a, s_sum, s_val, iv, s_rows, nrows, g * 32 + lane, lane);
    }
    if (lane == 0 && m) atomicOr(&s_mask, m);
    __syncthreads();
    if (tid == 0) {
      const uint32_t mm = s_mask;
      if (mm) {
        const int base = atomicAdd(a.count_out, __popc(mm));
        int i = 0;
        for (int t = 0; t < 32; ++t)
          if (mm & (1u << t)) a.list_out[base + i++] = s_rows[t];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Input chunks (N > 16384: a row of bit words does not fit shared memory).
//
// Pass 1, bits_transpose_kernel: one CTA per 32-row tile writes the tile's N
// bit words to global memory (coalesced 16-byte stores) and flags tiles that
// hold a value other than 0 or 1 (their rows go to the fallback list).
// Pass 2, bits_count_chunked_kernel: an item is (tile, subset of groups); for
// each input chunk the CTA copies the chunk's Q words into shared memory
// (TMA bulk copy) and every warp adds the slots of its groups into bit-sliced
// counters that stay in registers across the chunks; after the last chunk the
// epilogue is the one of layer0_bits_kernel.  The rows that survive are
// published per tile through the tile mask and ticket (the last subset of a
// tile to finish appends them).
constexpr int kChunkGroupsPerWarp = 4;
constexpr int kChunkWarps = 16;

__global__ void __launch_bounds__(256) bits_transpose_kernel(const Layer0Args a) {
  __shared__ int32_t s_rows[32];
  __shared__ int32_t s_nonbin;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int N = a.N;
  const int count = *a.count_in;
  const int n_tiles = (count + 31) / 32;
  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int row0 = tile * 32;
    const int nrows = min(32, count - row0);
    __syncthreads();
    if (tid < 32) s_rows[tid] = tid < nrows ? a.list_in[row0 + tid] : -1;
    if (tid == 0) s_nonbin = 0;
    __syncthreads();
    uint32_t* out = a.bits + (size_t)tile * N;
    bool nonbin = false;
    for (int j0 = warp * 128; j0 < N; j0 += nwarps * 128) {
      const int j = j0 + lane * 4;
      uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
      for (int t0 = 0; t0 < nrows; t0 += 8) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (t0 + u < nrows)
            v[u] = __ldg(reinterpret_cast<const float4*>(a.y_in + (size_t)s_rows[t0 + u] * N + j));
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (t0 + u < nrows) {
            const float x[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
            for (int q = 0; q < 4; ++q) nonbin |= (x[q] != 0.f) && (x[q] != 1.f);
            const uint32_t bit = 1u << (t0 + u);
            w0 |= x[0] != 0.f ? bit : 0u;
            w1 |= x[1] != 0.f ? bit : 0u;
            w2 |= x[2] != 0.f ? bit : 0u;
            w3 |= x[3] != 0.f ? bit : 0u;
          }
        }
      }
      *reinterpret_cast<uint4*>(out + j) = make_uint4(w0, w1, w2, w3);
    }
    if (__any_sync(0xffffffffu, nonbin) && lane == 0) s_nonbin = 1;
    __syncthreads();
    if (tid == 0) a.tile_state[tile] = s_nonbin;
    if (s_nonbin && tid < nrows) {
      const int pos = atomicAdd(a.fallback_count, 1);
      a.fallback_list[pos] = s_rows[tid];
    }
  }
}

__global__ void __launch_bounds__(kChunkWarps * 32) bits_count_chunked_kernel(const Layer0Args a) {
  extern __shared__ __align__(128) uint32_t cbits[];  // Q + 32 words
  __shared__ __align__(8) uint64_t bar;
  __shared__ float s_sum[128];
  __shared__ int32_t s_rows[32];
  __shared__ uint32_t s_mask;
  __shared__ int32_t s_fail;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int N = a.N, Q = a.Q, nq = a.nq;
  const int count = *a.count_in;
  const int n_tiles = (count + 31) / 32;
  constexpr int per_item = kChunkWarps * kChunkGroupsPerWarp;
  const int subsets = (a.G + per_item - 1) / per_item;
  const long items = (long)n_tiles * subsets;
  __shared__ float s_val[128];
  if (tid < 128) {
    s_sum[tid] = a.sums[tid];
    s_val[tid] = clampf(a.sums[tid] + a.bias, a.clampv);
  }
  for (int i = tid; i < 32; i += blockDim.x) cbits[Q + i] = 0u;
  if (tid == 0) {
    mbar_init(&bar, 1);
    s_mask = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  const CountInterval iv = count_interval(s_sum, a.bias, a.bias_vec != nullptr);
  uint32_t phase = 0;
  for (long item = blockIdx.x; item < items; item += gridDim.x) {
    const int tile = (int)(item / subsets), sub = (int)(item % subsets);
    const int row0 = tile * 32;
    const int nrows = min(32, count - row0);
    if (a.tile_state[tile]) continue;  // non-binary tile: the float kernel runs it
    __syncthreads();
    if (tid < 32) s_rows[tid] = tid < nrows ? a.list_in[row0 + tid] : -1;
    uint32_t c[kChunkGroupsPerWarp][7];
#pragma unroll
    for (int k = 0; k < kChunkGroupsPerWarp; ++k)
#pragma unroll
      for (int i = 0; i < 7; ++i) c[k][i] = 0u;
    for (int q = 0; q < nq; ++q) {
      __syncthreads();  // every warp is done with the previous chunk
      if (tid == 0) {
        const uint32_t bytes = (uint32_t)Q * 4u;
        mbar_expect_tx(&bar, bytes);
        const char* src = reinterpret_cast<const char*>(a.bits + (size_t)tile * N + (size_t)q * Q);
        char* dst = reinterpret_cast<char*>(cbits);
        for (uint32_t off = 0; off < bytes; off += 32768u)
          bulk_g2s(dst + off, src + off, min(32768u, bytes - off), &bar);
        s_fail = mbar_wait_bounded(&bar, phase, a.err) ? 0 : 1;
      }
      __syncthreads();
      if (s_fail) return;
      mbar_try_wait(&bar, phase);
      phase ^= 1u;
#pragma unroll
      for (int k = 0; k < kChunkGroupsPerWarp; ++k) {
        const int g = sub * per_item + k * kChunkWarps + warp;
        if (g < a.G) {
          const int32_t b0 = __ldg(a.grp_blk + g * nq + q), b1 = __ldg(a.grp_blk + g * nq + q + 1);
          count_list<false>(c[k], a.idx + (size_t)b0 * 32 + lane, b1 - b0, cbits);
        }
      }
    }
    uint32_t m = 0;
#pragma unroll
    for (int k = 0; k < kChunkGroupsPerWarp; ++k) {
      const int g = sub * per_item + k * kChunkWarps + warp;
      if (g >= a.G) continue;
      m |= bits_epilogue(c[k], a, s_sum, s_val, iv, s_rows, nrows, g * 32 + lane, lane);
    }
    if (lane == 0 && m) atomicOr(&s_mask, m);
    __syncthreads();
    if (tid == 0) {
      uint32_t mm = s_mask;
      s_mask = 0;
      bool emit = true;
      if (subsets > 1) {
        atomicOr(a.tile_mask + tile, mm);
        __threadfence();
        const int tk = atomicAdd(a.tile_ticket + tile, 1);
        emit = (tk == subsets - 1);
        if (emit) {
          __threadfence();
          mm = atomicExch(a.tile_mask + tile, 0u);
          a.tile_ticket[tile] = 0;
        }
      }
      if (emit && mm) {
        const int base = atomicAdd(a.count_out, __popc(mm));
        int i = 0;
        for (int t = 0; t < 32; ++t)
          if (mm & (1u << t)) a.list_out[base + i++] = s_rows[t];
      }
    }
  }
}

bool layer0_bits_chunked_supported(int N, int Q) {
  return Q == 16384 && N % Q == 0 && N / Q > 1 && N % 128 == 0;
}

cudaError_t launch_layer0_bits_chunked(const Layer0Args& a, int num_sms, cudaStream_t s) {
  if (!layer0_bits_chunked_supported(a.N, a.Q)) return cudaErrorInvalidValue;
  bits_transpose_kernel<<<num_sms * 4, 256, 0, s>>>(a);
  cudaError_t rc = cudaGetLastError();
  if (rc != cudaSuccess) return rc;
  const void* fn = (const void*)&bits_count_chunked_kernel;
  const size_t smem = (size_t)(a.Q + 32) * 4;
  rc = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (rc != cudaSuccess) return rc;
  int per_sm = 0;
  rc = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kChunkWarps * 32, smem);
  if (rc != cudaSuccess) return rc;
  void* args[] = {const_cast<Layer0Args*>(&a)};
  return cudaLaunchKernel(fn, dim3(num_sms * std::max(1, per_sm)), dim3(kChunkWarps * 32), args,
                          smem, s);
}

template __global__ void layer0_bits_kernel<1056>(const Layer0Args);
template __global__ void layer0_bits_kernel<4128>(const Layer0Args);
template __global__ void layer0_bits_kernel<16416>(const Layer0Args);

static const void* bits_fn(int rsw) {
  switch (rsw) {
    case 1056: return (const void*)&layer0_bits_kernel<1056>;
    case 4128: return (const void*)&layer0_bits_kernel<4128>;
    case 16416: return (const void*)&layer0_bits_kernel<16416>;
    default: return nullptr;
  }
}

bool layer0_bits_supported(int N) { return bits_fn(N + 32) != nullptr; }

int layer0_bits_grid(int N, int num_sms, int threads) {
  const void* fn = bits_fn(N + 32);
  if (!fn) return 0;
  const size_t smem = (size_t)(N + 32) * 4;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n * num_sms;
}

cudaError_t launch_layer0_bits(const Layer0Args& a, int grid, int threads, cudaStream_t s) {
  const void* fn = bits_fn(a.N + 32);
  if (!fn) return cudaErrorInvalidValue;
  void* args[] = {const_cast<Layer0Args*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, (size_t)(a.N + 32) * 4, s);
}

}  // namespace sdnn

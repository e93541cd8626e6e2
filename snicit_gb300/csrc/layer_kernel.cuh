// Plain / centroid / residue layer kernel (the sparse-W x dense-Y step).
//
// Computes, for each row r of a row list and each output neuron c,
//     acc = sum over in-edges (j -> c) of w_jc * Y_in[r][j]
// and applies one of three epilogues (sdnn_internal.h).  The reference's
// forms of this step are bf_inference (src/SDGC/BF/kernel.hpp:26-89),
// snig_inference (src/SDGC/SNIG/kernel.hpp:24-114), the XY pre-threshold
// kernels (src/SDGC/XY/kernel.hpp:12-149) and post_spMM + post_minus
// (src/SDGC/SNICIT/kernel.hpp:71-136).  Those scatter Y*W into a shared row
// with shared-memory atomics; this kernel gathers instead:
//
//  * a CTA owns a tile of T rows; one thread issues 1-D TMA bulk copies
//    (cp.async.bulk + mbarrier) of the T input rows (or one input chunk of
//    them) into shared memory, row stride RS = chunk + 32 floats; the last 32
//    floats of every row are zero and serve the padding slots;
//  * warp w takes output groups of 32 neurons, lane i owns output 32g+i and
//    keeps T accumulators in registers (one per row of the tile);
//  * the in-edges of a group are pre-arranged into slots whose 32 indices hit
//    32 distinct banks, so every shared load of a slot is one wavefront;
//  * the summation order of an output is its slot order, fixed at packing
//    time, so results are bitwise reproducible (no atomics on values);
//  * bias + ReLU + clamp (or the residue update) are fused in the epilogue;
//    the CTA compacts surviving rows into the next row list with one atomic
//    per tile (a ticket when several CTAs share a tile).
#pragma once
#include "sdnn_internal.h"

namespace sdnn {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for an mbarrier phase for at most limit_ns (default 2 s); on timeout
// records DEV_TIMEOUT in the error word and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int32_t* err,
                                                  uint64_t limit_ns = 2000000000ull) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) {
      atomicExch(err, DEV_TIMEOUT);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ float clampf(float v, float hi) { return fminf(hi, fmaxf(0.f, v)); }


// Applies NB blocks of slots (indices in iv, values in vv) to acc[T].
template <int T, int RSW, bool CONSTW, int NB>
__device__ __forceinline__ void apply_blocks(float (&acc)[T], const uint2 (&iv)[NB],
                                             const float4 (&vv)[CONSTW ? 1 : NB], float wc,
                                             const float* __restrict__ ys, int RS) {
#pragma unroll
  for (int k = 0; k < NB; ++k) {
    const uint32_t words[2] = {iv[k].x, iv[k].y};
    float wv[4];
    if constexpr (!CONSTW) {
      wv[0] = vv[k].x; wv[1] = vv[k].y; wv[2] = vv[k].z; wv[3] = vv[k].w;
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const uint32_t j = (words[s >> 1] >> ((s & 1) * 16)) & 0xffffu;
      // byte offset or float index, fixed by the packer for this row stride
      const float* p = rsw_in_bytes(RSW)
                           ? reinterpret_cast<const float*>(reinterpret_cast<const char*>(ys) + j)
                           : ys + j;
      const float w = CONSTW ? wc : wv[s];
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const int off = (RSW > 0 ? RSW : RS) * t;
        acc[t] = fmaf(w, p[off], acc[t]);
      }
    }
  }
}

// Loads NB blocks starting at block b (indices and, for general layers, values).
template <bool CONSTW, int NB>
__device__ __forceinline__ void load_blocks(uint2 (&iv)[NB], float4 (&vv)[CONSTW ? 1 : NB],
                                            const uint2* __restrict__ ip,
                                            const float4* __restrict__ vp, int b) {
#pragma unroll
  for (int k = 0; k < NB; ++k) {
    iv[k] = __ldg(ip + (size_t)(b + k) * 32);
    if constexpr (!CONSTW) vv[k] = __ldg(vp + (size_t)(b + k) * 32);
  }
}

// Accumulates the in-edges of group g from input chunk q into acc[T].
// Slot blocks are fetched in batches of 8, then 2, then 1 (no predicated
// tail): all indices of a batch are in registers before the first is used,
// so a warp waits for one memory round trip per batch (the post-threshold
// launches have one warp per group and nothing else to hide that latency).
template <int T, int RSW, bool CONSTW>
__device__ __forceinline__ void accumulate_group(float (&acc)[T], const LayerDev& wl, int nq,
                                                 const float* __restrict__ ys, int RS, int g,
                                                 int q, int lane) {
  const int32_t b0 = __ldg(wl.grp_blk + g * nq + q);
  const int32_t b1 = __ldg(wl.grp_blk + g * nq + q + 1);
  const uint2* __restrict__ ip = wl.idx + (size_t)b0 * 32 + lane;
  const float4* __restrict__ vp = CONSTW ? nullptr : wl.val + (size_t)b0 * 32 + lane;
  const float wc = wl.wconst;
  const int nb = b1 - b0;
  int b = 0;
  for (; b + 8 <= nb; b += 8) {
    uint2 iv[8];
    float4 vv[CONSTW ? 1 : 8];
    load_blocks<CONSTW, 8>(iv, vv, ip, vp, b);
    apply_blocks<T, RSW, CONSTW, 8>(acc, iv, vv, wc, ys, RS);
  }
  for (; b + 2 <= nb; b += 2) {
    uint2 iv[2];
    float4 vv[CONSTW ? 1 : 2];
    load_blocks<CONSTW, 2>(iv, vv, ip, vp, b);
    apply_blocks<T, RSW, CONSTW, 2>(acc, iv, vv, wc, ys, RS);
  }
  if (b < nb) {
    uint2 iv[1];
    float4 vv[1];
    load_blocks<CONSTW, 1>(iv, vv, ip, vp, b);
    apply_blocks<T, RSW, CONSTW, 1>(acc, iv, vv, wc, ys, RS);
  }
}

// Input chunks: the KG groups of a warp (gbeg + warp + kk * nwarps) over
// chunk q.  Their lists are short (about 8 slots per lane and chunk), so
// fetching them group by group costs a memory round trip per group; here the
// KG offsets come in one load (lane kk holds group kk's), and the first
// CHUNK_NB blocks of group kk + 1 are loaded while group kk is applied.  The
// FMA order of every group is unchanged (blocks, then slots, in order).
constexpr int CHUNK_NB = 4;
template <int T, int RSW, bool CONSTW, int KG>
__device__ __forceinline__ void accumulate_chunk(float (&acc)[KG][T], const LayerDev& wl, int nq,
                                                 const float* __restrict__ ys, int RS, int gbeg,
                                                 int gend, int warp, int nwarps, int q, int lane) {
  int32_t my_b0 = 0, my_b1 = 0;
  if (lane < KG) {
    const int g = gbeg + warp + lane * nwarps;
    if (g < gend) {
      my_b0 = __ldg(wl.grp_blk + g * nq + q);
      my_b1 = __ldg(wl.grp_blk + g * nq + q + 1);
    }
  }
  const float wc = wl.wconst;
  uint2 iv[2][CHUNK_NB];
  float4 vv[2][CONSTW ? 1 : CHUNK_NB];
  auto fetch = [&](int kk, uint2 (&i)[CHUNK_NB], float4 (&v)[CONSTW ? 1 : CHUNK_NB]) {
    const int32_t b0 = __shfl_sync(0xffffffffu, my_b0, kk);
    const int nb = __shfl_sync(0xffffffffu, my_b1, kk) - b0;
    const uint2* ip = wl.idx + (size_t)b0 * 32 + lane;
#pragma unroll
    for (int k = 0; k < CHUNK_NB; ++k) {
      if (k < nb) {
        i[k] = __ldg(ip + (size_t)k * 32);
        if constexpr (!CONSTW) v[k] = __ldg(wl.val + (size_t)(b0 + k) * 32 + lane);
      }
    }
  };
  fetch(0, iv[0], vv[0]);
#pragma unroll
  for (int kk = 0; kk < KG; ++kk) {
    const int cur = kk & 1;
    if (kk + 1 < KG) fetch(kk + 1, iv[cur ^ 1], vv[cur ^ 1]);
    const int32_t b0 = __shfl_sync(0xffffffffu, my_b0, kk);
    const int nb = __shfl_sync(0xffffffffu, my_b1, kk) - b0;
    // the first CHUNK_NB blocks (prefetched), one at a time in order
#pragma unroll
    for (int k = 0; k < CHUNK_NB; ++k) {
      if (k < nb) {
        uint2 one[1] = {iv[cur][k]};
        float4 onev[1];
        if constexpr (!CONSTW) onev[0] = vv[cur][k];
        apply_blocks<T, RSW, CONSTW, 1>(acc[kk], one, onev, wc, ys, RS);
      }
    }
    // the rest of a long list, in exact-size batches
    if (nb > CHUNK_NB) {
      const uint2* ip = wl.idx + (size_t)b0 * 32 + lane;
      const float4* vp = CONSTW ? nullptr : wl.val + (size_t)b0 * 32 + lane;
      int b = CHUNK_NB;
      for (; b + 4 <= nb; b += 4) {
        uint2 i4[4];
        float4 v4[CONSTW ? 1 : 4];
        load_blocks<CONSTW, 4>(i4, v4, ip, vp, b);
        apply_blocks<T, RSW, CONSTW, 4>(acc[kk], i4, v4, wc, ys, RS);
      }
      for (; b < nb; ++b) {
        uint2 i1[1];
        float4 v1[1];
        load_blocks<CONSTW, 1>(i1, v1, ip, vp, b);
        apply_blocks<T, RSW, CONSTW, 1>(acc[kk], i1, v1, wc, ys, RS);
      }
    }
  }
}

// Epilogue of one group for the rows of the tile; returns the row mask of
// rows flagged by this warp (alive for PLAIN, non-empty for RESIDUE).
template <int T>
__device__ __forceinline__ uint32_t epilogue_group(const float (&acc)[T], const LayerArgs& a,
                                                   const int32_t* s_rows, int nrows, int g,
                                                   int lane) {
  const int c = g * 32 + lane;
  const float bc = a.w.bias_vec ? __ldg(a.w.bias_vec + c) : a.w.bias;
  const float hi = a.clampv;
  uint32_t m = 0;
#pragma unroll
  for (int t = 0; t < T; ++t) {
    if (t < nrows) {
      const int row = s_rows[t];
      float* dst = a.y_out + (size_t)row * a.N + c;
      bool flag;
      if (a.epi == EPI_PLAIN) {
        const float v = acc[t] + bc;
        *dst = clampf(v, hi);
        flag = v > 0.f;
      } else if (a.epi == EPI_CENTROID) {
        const int k = a.cslot[row];
        const float v = acc[t] + bc;
        a.pre_out[(size_t)k * a.N + c] = v;
        *dst = clampf(v, hi);
        flag = false;
      } else {
        const int k = a.cslot[row];
        const float pc = __ldg(a.pre_in + (size_t)k * a.N + c);
        const float y = clampf(pc + acc[t], hi) - clampf(pc, hi);
        *dst = y;
        flag = y != 0.f;
      }
      if (__any_sync(0xffffffffu, flag)) m |= 1u << t;
    }
  }
  return m;
}

// Issues the TMA bulk copies of the rows of one tile (one input chunk) into a
// shared buffer and arms its mbarrier; called by one thread.
__device__ __forceinline__ void load_tile(const LayerArgs& a, float* buf, int RS,
                                          const int32_t* rows, int nrows, int q, uint64_t* bar) {
  const uint32_t row_bytes = (uint32_t)a.Q * 4u;
  mbar_expect_tx(bar, row_bytes * (uint32_t)nrows);
  for (int t = 0; t < nrows; ++t) {
    const char* src =
        reinterpret_cast<const char*>(a.y_in + (size_t)rows[t] * a.N + (size_t)q * a.Q);
    char* dst = reinterpret_cast<char*>(buf + (size_t)t * RS);
    for (uint32_t off = 0; off < row_bytes; off += 32768u)
      bulk_g2s(dst + off, src + off, min(32768u, row_bytes - off), bar);
  }
}

// Work split shared by all CTAs of a launch (same count, same grid).
struct Split {
  int count, n_tiles, spl;
  long items;
};
template <int T>
__device__ __forceinline__ Split make_split(const LayerArgs& a) {
  Split sp;
  sp.count = *a.count_in;
  sp.n_tiles = (sp.count + T - 1) / T;
  int spl = sp.n_tiles > 0 ? (int)((gridDim.x + sp.n_tiles - 1) / sp.n_tiles) : 1;
  spl = max(spl, a.min_split);
  spl = min(spl, a.max_split);
  sp.spl = max(spl, 1);
  sp.items = (long)sp.n_tiles * sp.spl;
  return sp;
}

// Publishes the flagged rows of a finished item: straight to the next list,
// or through the per-tile mask and ticket when several CTAs share the tile.
template <int T>
__device__ __forceinline__ void publish_rows(const LayerArgs& a, uint32_t m, int tile, int spl,
                                             const int32_t* rows) {
  if (a.epi == EPI_CENTROID) return;
  bool emit = true;
  if (spl > 1) {
    atomicOr(a.tile_mask + tile, m);
    __threadfence();
    const int tk = atomicAdd(a.tile_ticket + tile, 1);
    emit = (tk == spl - 1);
    if (emit) {
      __threadfence();
      m = atomicExch(a.tile_mask + tile, 0u);
      a.tile_ticket[tile] = 0;
    }
  }
  if (emit && m) {
    const int base = atomicAdd(a.count_out, __popc(m));
    int i = 0;
    for (int t = 0; t < T; ++t)
      if (m & (1u << t)) a.list_out[base + i++] = rows[t];
  }
}

template <int T, int RSW, int KG, bool CONSTW>
// (instances with up to 8 groups per warp may run 1024 threads; 16 groups per
// warp keep 512 so their KG x T accumulators stay in registers)
__global__ void __launch_bounds__(KG <= 8 ? 1024 : 512) layer_kernel(const LayerArgs a) {
  extern __shared__ __align__(128) float ys[];
  __shared__ __align__(8) uint64_t bar[1];
  __shared__ int32_t s_rows[2][T];
  __shared__ int32_t s_next[T];
  __shared__ uint32_t s_mask, s_pmask;
  __shared__ int32_t s_ptile, s_pbuf;
  __shared__ int32_t s_fail;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int RS = RSW > 0 ? RSW : a.Q + 32;
  // Launched with programmatic stream serialization: the next launch may be
  // scheduled now, and this one may have started before its predecessor
  // ended -- so only CTA-local setup comes before griddepcontrol.wait, which
  // returns once the predecessor has completed and its writes are visible.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // One tile buffer, reloaded per item (and input chunk): the load of one CTA
  // overlaps the compute of the other CTAs on the SM (up to four).
  for (int i = tid; i < T * 32; i += blockDim.x) ys[(i >> 5) * RS + a.Q + (i & 31)] = 0.f;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    s_mask = 0;
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const Split sp = make_split<T>(a);
  if (sp.count <= 0 || (long)blockIdx.x >= sp.items) return;
  __syncthreads();

  // Per item: row ids of the item after it are fetched while it runs, and the
  // rows it flags are published (tile mask, ticket, list append: a chain of
  // global atomics) during the next item, while the other warps already work
  // on it -- both by the CTA's last warp (its lane 31 publishes); s_rows is
  // double-buffered, and the pending state lives in shared memory so that it
  // costs the compute warps no registers.
  const bool last_warp = warp == nwarps - 1;
  auto item_row = [&](long it, int t) -> int {
    const int r0 = (int)(it / sp.spl) * T;
    return t < min(T, sp.count - r0) ? a.list_in[r0 + t] : -1;
  };
  if (last_warp && lane < T) s_next[lane] = item_row(blockIdx.x, lane);
  if (last_warp && lane == 31) s_ptile = -1;
  uint32_t phase = 0;
  int loaded_tile = -1;
  int b = 0;
  for (long item = blockIdx.x; item < sp.items; item += gridDim.x, b ^= 1) {
    const int tile = (int)(item / sp.spl), part = (int)(item % sp.spl);
    const int row0 = tile * T;
    const int nrows = min(T, sp.count - row0);
    const int gbeg = (int)((long)a.G * part / sp.spl), gend = (int)((long)a.G * (part + 1) / sp.spl);
    __syncthreads();  // s_rows[b] is free: the item that used it was published
    if (tid < T) s_rows[b][tid] = s_next[tid];
    __syncthreads();
    if (last_warp) {
      if (lane < T && item + gridDim.x < sp.items) s_next[lane] = item_row(item + gridDim.x, lane);
      if (lane == 31 && s_ptile >= 0) {
        publish_rows<T>(a, s_pmask, s_ptile, sp.spl, s_rows[s_pbuf]);
        s_ptile = -1;
      }
    }
    uint32_t m = 0;
    if constexpr (KG == 1) {
      // one buffer, whole rows (one chunk): reloaded when the tile changes
      if (tile != loaded_tile) {
        if (tid == 0) {
          load_tile(a, ys, RS, s_rows[b], nrows, 0, &bar[0]);
          s_fail = mbar_wait_bounded(&bar[0], phase, a.err) ? 0 : 1;
        }
        __syncthreads();
        if (s_fail) return;
        mbar_try_wait(&bar[0], phase);
        phase ^= 1u;
        loaded_tile = tile;
      }
      for (int g = gbeg + warp; g < gend; g += nwarps) {
        float acc[T];
#pragma unroll
        for (int t = 0; t < T; ++t) acc[t] = 0.f;
        accumulate_group<T, RSW, CONSTW>(acc, a.w, a.nq, ys, RS, g, 0, lane);
        m |= epilogue_group<T>(acc, a, s_rows[b], nrows, g, lane);
      }
    } else {
      // input chunks (nq > 1): accumulators of KG groups per warp live across chunks
      float acc[KG][T];
#pragma unroll
      for (int kk = 0; kk < KG; ++kk)
#pragma unroll
        for (int t = 0; t < T; ++t) acc[kk][t] = 0.f;
      for (int q = 0; q < a.nq; ++q) {
        if (q > 0) __syncthreads();
        if (tid == 0) {
          load_tile(a, ys, RS, s_rows[b], nrows, q, &bar[0]);
          s_fail = mbar_wait_bounded(&bar[0], phase, a.err) ? 0 : 1;
        }
        __syncthreads();
        if (s_fail) return;
        mbar_try_wait(&bar[0], phase);
        phase ^= 1u;
        accumulate_chunk<T, RSW, CONSTW, KG>(acc, a.w, a.nq, ys, RS, gbeg, gend, warp, nwarps, q,
                                             lane);
      }
#pragma unroll
      for (int kk = 0; kk < KG; ++kk) {
        const int g = gbeg + warp + kk * nwarps;
        if (g < gend) m |= epilogue_group<T>(acc[kk], a, s_rows[b], nrows, g, lane);
      }
    }
    if (lane == 0 && m) atomicOr(&s_mask, m);
    __syncthreads();
    if (last_warp && lane == 31) {
      s_pmask = s_mask;
      s_mask = 0;
      s_ptile = tile;
      s_pbuf = b;
    }
  }
  if (last_warp && lane == 31 && s_ptile >= 0)
    publish_rows<T>(a, s_pmask, s_ptile, sp.spl, s_rows[s_pbuf]);
}

#define SDNN_LAYER_INSTANCE(T, RSW, KG, CW) template __global__ void layer_kernel<T, RSW, KG, CW>(const LayerArgs);

// Registry entry used by the dispatcher.
struct LayerInstance {
  int T, rsw, kg;
  bool constw;
  const void* fn;
};

}  // namespace sdnn

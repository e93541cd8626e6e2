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
// Waits for an mbarrier phase for at most ~2 s; on timeout records DEV_TIMEOUT.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int32_t* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > 2000000000ull) {
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

// Accumulates the in-edges of group g from input chunk q into acc[T].
// The slot indices (and values) of up to PF blocks are loaded into registers
// before any of them is used, so a warp waits for one memory round trip per
// PF blocks instead of one per block (the post-threshold launches have one
// warp per group and nothing else to hide that latency).
template <int T, int RSW, bool CONSTW>
__device__ __forceinline__ void accumulate_group(float (&acc)[T], const LayerArgs& a,
                                                 const float* __restrict__ ys, int RS, int g,
                                                 int q, int lane) {
  constexpr int PF = CONSTW ? 16 : 8;
  const int32_t b0 = __ldg(a.w.grp_blk + g * a.nq + q);
  const int32_t b1 = __ldg(a.w.grp_blk + g * a.nq + q + 1);
  const uint2* __restrict__ ip = a.w.idx + (size_t)b0 * 32 + lane;
  const float4* __restrict__ vp = CONSTW ? nullptr : a.w.val + (size_t)b0 * 32 + lane;
  const float wc = a.w.wconst;
  const int nb = b1 - b0;
  for (int bb = 0; bb < nb; bb += PF) {
    uint2 iv[PF];
    float4 vv[CONSTW ? 1 : PF];
#pragma unroll
    for (int k = 0; k < PF; ++k) {
      if (bb + k < nb) {
        iv[k] = __ldg(ip + (size_t)(bb + k) * 32);
        if constexpr (!CONSTW) vv[k] = __ldg(vp + (size_t)(bb + k) * 32);
      }
    }
#pragma unroll
    for (int k = 0; k < PF; ++k) {
      if (bb + k < nb) {
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

template <int T, int RSW, int KG, bool CONSTW>
__global__ void __launch_bounds__(512) layer_kernel(const LayerArgs a) {
  extern __shared__ __align__(128) float ys[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int32_t s_rows[T];
  __shared__ uint32_t s_mask;
  __shared__ int32_t s_fail;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int RS = RSW > 0 ? RSW : a.Q + 32;
  const int count = *a.count_in;
  if (count <= 0) return;
  const int n_tiles = (count + T - 1) / T;
  int spl = (int)((gridDim.x + n_tiles - 1) / n_tiles);
  spl = max(spl, a.min_split);
  spl = min(spl, a.max_split);
  spl = max(spl, 1);
  const long items = (long)n_tiles * spl;
  if ((long)blockIdx.x >= items) return;

  for (int i = tid; i < T * 32; i += blockDim.x) ys[(i >> 5) * RS + a.Q + (i & 31)] = 0.f;
  if (tid == 0) {
    mbar_init(&bar, 1);
    s_mask = 0;
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  uint32_t phase = 0;
  int loaded_tile = -1;
  for (long item = blockIdx.x; item < items; item += gridDim.x) {
    const int tile = (int)(item / spl), part = (int)(item % spl);
    const int row0 = tile * T;
    const int nrows = min(T, count - row0);
    const int gbeg = (int)((long)a.G * part / spl), gend = (int)((long)a.G * (part + 1) / spl);
    __syncthreads();
    if (tid < T) s_rows[tid] = tid < nrows ? a.list_in[row0 + tid] : -1;
    __syncthreads();

    if constexpr (KG == 1) {
      if (tile != loaded_tile) {
        if (tid == 0) {
          const uint32_t row_bytes = (uint32_t)a.Q * 4u;
          mbar_expect_tx(&bar, row_bytes * (uint32_t)nrows);
          for (int t = 0; t < nrows; ++t) {
            const char* src = reinterpret_cast<const char*>(a.y_in + (size_t)s_rows[t] * a.N);
            char* dst = reinterpret_cast<char*>(ys + (size_t)t * RS);
            for (uint32_t off = 0; off < row_bytes; off += 32768u)
              bulk_g2s(dst + off, src + off, min(32768u, row_bytes - off), &bar);
          }
          s_fail = mbar_wait_bounded(&bar, phase, a.err) ? 0 : 1;
        }
        __syncthreads();
        if (s_fail) return;
        mbar_try_wait(&bar, phase);
        phase ^= 1u;
        loaded_tile = tile;
      }
      uint32_t m = 0;
      for (int g = gbeg + warp; g < gend; g += nwarps) {
        float acc[T];
#pragma unroll
        for (int t = 0; t < T; ++t) acc[t] = 0.f;
        accumulate_group<T, RSW, CONSTW>(acc, a, ys, RS, g, 0, lane);
        m |= epilogue_group<T>(acc, a, s_rows, nrows, g, lane);
      }
      if (lane == 0 && m) atomicOr(&s_mask, m);
    } else {
      float acc[KG][T];
#pragma unroll
      for (int k = 0; k < KG; ++k)
#pragma unroll
        for (int t = 0; t < T; ++t) acc[k][t] = 0.f;
      for (int q = 0; q < a.nq; ++q) {
        if (q > 0) __syncthreads();
        if (tid == 0) {
          const uint32_t row_bytes = (uint32_t)a.Q * 4u;
          mbar_expect_tx(&bar, row_bytes * (uint32_t)nrows);
          for (int t = 0; t < nrows; ++t) {
            const char* src =
                reinterpret_cast<const char*>(a.y_in + (size_t)s_rows[t] * a.N + (size_t)q * a.Q);
            char* dst = reinterpret_cast<char*>(ys + (size_t)t * RS);
            for (uint32_t off = 0; off < row_bytes; off += 32768u)
              bulk_g2s(dst + off, src + off, min(32768u, row_bytes - off), &bar);
          }
          s_fail = mbar_wait_bounded(&bar, phase, a.err) ? 0 : 1;
        }
        __syncthreads();
        if (s_fail) return;
        mbar_try_wait(&bar, phase);
        phase ^= 1u;
#pragma unroll
        for (int k = 0; k < KG; ++k) {
          const int g = gbeg + warp + k * nwarps;
          if (g < gend) accumulate_group<T, RSW, CONSTW>(acc[k], a, ys, RS, g, q, lane);
        }
      }
      loaded_tile = -1;
      uint32_t m = 0;
#pragma unroll
      for (int k = 0; k < KG; ++k) {
        const int g = gbeg + warp + k * nwarps;
        if (g < gend) m |= epilogue_group<T>(acc[k], a, s_rows, nrows, g, lane);
      }
      if (lane == 0 && m) atomicOr(&s_mask, m);
    }

    __syncthreads();
    if (tid == 0) {
      uint32_t m = s_mask;
      s_mask = 0;
      if (a.epi != EPI_CENTROID) {
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
            if (m & (1u << t)) a.list_out[base + i++] = s_rows[t];
        }
      }
    }
  }
}

#define SDNN_LAYER_INSTANCE(T, RSW, KG, CW) template __global__ void layer_kernel<T, RSW, KG, CW>(const LayerArgs);

// Registry entry used by the dispatcher.
struct LayerInstance {
  int T, rsw, kg;
  bool constw;
  const void* fn;
};

}  // namespace sdnn

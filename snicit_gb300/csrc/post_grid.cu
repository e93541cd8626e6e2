// Post-threshold layers with no residue rows left, for widths whose rows do
// not fit in shared memory (the cluster chain kernels hold every centroid row
// in every CTA; at N = 65536 one row is 256 KB).
//
// One cooperative launch over the whole GPU carries the K centroid rows
// through all remaining layers:
//
//  * the rows of every layer get a fresh global buffer laid out per input
//    chunk with the 32 zero floats the padding slots point at
//    ([layers + 1][K][nq][Q + 32]): no address is written after it was read,
//    so the gathers may be cached in L1 (no stale copy can exist);
//  * warp w of the grid takes output groups w, w + W, ...; lane i owns output
//    32g + i and walks the same bank-scheduled slots in the same FP32 order
//    as layer_kernel (chunk by chunk);
//  * a grid barrier (one counter, bounded wait) separates layers; the last
//    layer writes the rows to the final activation buffer.
// Bitwise equal to the per-layer launches.
#include "layer_kernel.cuh"

namespace sdnn {

namespace {

constexpr int kGridChainThreads = 512;

// Arrive at the grid barrier and wait (bounded) until `target` CTAs have
// arrived in total.  After a timeout the error word is set and this CTA stops
// waiting at later barriers, so the kernel still runs to its end.
__device__ __forceinline__ void grid_barrier(unsigned int* ctr, unsigned int target, int32_t* err,
                                             int32_t* s_failed) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    if (!*s_failed) {
      const uint64_t t0 = global_ns();
      for (;;) {
        unsigned int v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
        if (v >= target) break;
        __nanosleep(32);  // back off: every CTA polls the same L2 line
        if (global_ns() - t0 > 2000000000ull) {
          atomicExch(err, DEV_TIMEOUT);
          *s_failed = 1;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <int KC>
__global__ void __launch_bounds__(kGridChainThreads) chain_grid_kernel(const GridChainArgs a) {
  __shared__ int32_t s_failed;
  const int tid = threadIdx.x, lane = tid & 31;
  const int N = a.N, Q = a.Q, nq = a.nq;
  const int K = min(*a.ccount, KC);
  const size_t cs = (size_t)Q + 32;        // chunk stride in the scratch rows
  const size_t rs = (size_t)nq * cs;       // row stride
  const long gtid = (long)blockIdx.x * blockDim.x + tid;
  const long gthreads = (long)gridDim.x * blockDim.x;
  const int gwarp = (int)(gtid >> 5), nwarps = (int)(gthreads >> 5);
  const bool bytes = slot_index_in_bytes(Q);
  if (tid == 0) s_failed = 0;
  unsigned int arrivals = 0;
  const int nbuf = a.last - a.first;  // buffers 0 .. nbuf - 1 (the last layer writes y_out)
  // rows into buffer 0, pad columns of every buffer zeroed
  for (long i = gtid; i < (long)K * N; i += gthreads) {
    const int t = (int)(i / N), j = (int)(i % N);
    a.scratch[t * rs + (size_t)(j / Q) * cs + (j % Q)] = a.y_in[(size_t)a.clist[t] * N + j];
  }
  for (long i = gtid; i < (long)nbuf * KC * nq * 32; i += gthreads) {
    const long row = i >> 5;  // (buffer, t, q)
    a.scratch[(size_t)row * cs + Q + (i & 31)] = 0.f;
  }
  arrivals += gridDim.x;
  grid_barrier(a.barrier, arrivals, a.err, &s_failed);

  for (int l = a.first; l < a.last; ++l) {
    const int li = l - a.first;
    const float* in = a.scratch + (size_t)li * KC * rs;
    float* out = a.scratch + (size_t)(li + 1) * KC * rs;
    const bool last = l + 1 == a.last;
    const LayerDev wl = a.layers[l];
    if (tid == 0 && l + 1 < a.last) {
      // this CTA's slot blocks of the next layer into L2 while this one runs
      const int gb = blockIdx.x * (blockDim.x >> 5);
      const int ge = min(a.G, gb + (int)(blockDim.x >> 5));
      if (gb < ge) {
        const LayerDev wn = a.layers[l + 1];
        const int32_t b0 = __ldg(wn.grp_blk + gb * nq), b1 = __ldg(wn.grp_blk + ge * nq);
        const uint32_t bytes = (uint32_t)(b1 - b0) * 32u * (uint32_t)sizeof(uint2);
        if (bytes > 0)
          asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(wn.idx + (size_t)b0 * 32),
                       "r"(bytes)
                       : "memory");
        if (wn.val && bytes > 0)
          asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(wn.val + (size_t)b0 * 32),
                       "r"(bytes * 2u)
                       : "memory");
      }
    }
    for (int g = gwarp; g < a.G; g += nwarps) {
      const int c = g * 32 + lane;
      const float bc = wl.bias_vec ? __ldg(wl.bias_vec + c) : wl.bias;
      float acc[KC];
#pragma unroll
      for (int t = 0; t < KC; ++t) acc[t] = 0.f;
      // the group's slot blocks of all chunks are consecutive: walk them as one
      // sequence (chunk-major, the layer kernel's order) in batches of NB
      // blocks -- all index loads, then all gathers, then the FMAs -- with the
      // chunk boundaries (nq + 1 offsets, nq <= 31) held by the lanes
      const int32_t bnd = lane <= nq ? __ldg(wl.grp_blk + g * nq + lane) : 0;
      const int32_t g0 = __shfl_sync(0xffffffffu, bnd, 0);
      const int nb = __shfl_sync(0xffffffffu, bnd, nq) - g0;
      const uint2* ip = wl.idx + (size_t)g0 * 32 + lane;
      const float4* vp = wl.val ? wl.val + (size_t)g0 * 32 + lane : nullptr;
      constexpr int NB = 8 / KC;  // 32 gathered operands in registers per batch
      int q = 0, qend = __shfl_sync(0xffffffffu, bnd, 1) - g0;  // chunk of block b
      for (int b = 0; b < nb; b += NB) {
        uint2 iv[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k)
          iv[k] = b + k < nb ? __ldg(ip + (size_t)(b + k) * 32) : make_uint2(0u, 0u);
        float y[NB][4][KC];
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          while (b + k >= qend && q + 1 < nq) {  // warp-uniform: next chunk
            ++q;
            qend = __shfl_sync(0xffffffffu, bnd, q + 1) - g0;
          }
          const float* base = in + (size_t)q * cs;
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            uint32_t j = ((s < 2 ? iv[k].x : iv[k].y) >> ((s & 1) * 16)) & 0xffffu;
            if (bytes) j >>= 2;
#pragma unroll
            for (int t = 0; t < KC; ++t)
              y[k][s][t] = (t < K && b + k < nb) ? base[(size_t)t * rs + j] : 0.f;
          }
        }
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          if (b + k < nb) {
            float4 wv = make_float4(wl.wconst, wl.wconst, wl.wconst, wl.wconst);
            if (vp) wv = __ldg(vp + (size_t)(b + k) * 32);
            const float w4[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
            for (int s = 0; s < 4; ++s)
#pragma unroll
              for (int t = 0; t < KC; ++t) acc[t] = fmaf(w4[s], y[k][s][t], acc[t]);
          }
        }
      }
#pragma unroll
      for (int t = 0; t < KC; ++t) {
        if (t < K) {
          const float y = clampf(acc[t] + bc, a.clampv);
          if (last)
            a.y_out[(size_t)a.clist[t] * N + c] = y;
          else
            out[(size_t)t * rs + (size_t)(c / Q) * cs + (c % Q)] = y;
        }
      }
    }
    if (!last) {
      arrivals += gridDim.x;
      grid_barrier(a.barrier, arrivals, a.err, &s_failed);
    }
  }
}

template __global__ void chain_grid_kernel<1>(const GridChainArgs);
template __global__ void chain_grid_kernel<2>(const GridChainArgs);
template __global__ void chain_grid_kernel<4>(const GridChainArgs);
template __global__ void chain_grid_kernel<8>(const GridChainArgs);

const void* grid_fn(int kc) {
  switch (kc) {
    case 1: return (const void*)&chain_grid_kernel<1>;
    case 2: return (const void*)&chain_grid_kernel<2>;
    case 4: return (const void*)&chain_grid_kernel<4>;
    case 8: return (const void*)&chain_grid_kernel<8>;
    default: return nullptr;
  }
}

}  // namespace

int grid_chain_capacity() { return 8; }

size_t grid_chain_scratch_floats(int layers, int nq, int Q) {
  return (size_t)(layers + 1) * grid_chain_capacity() * nq * ((size_t)Q + 32);
}

cudaError_t launch_grid_chain(const GridChainArgs& a, int kc_needed, int num_sms, cudaStream_t s) {
  int kc = 1;
  while (kc < kc_needed) kc *= 2;
  const void* fn = grid_fn(kc);
  if (!fn || a.nq > 31) return cudaErrorInvalidValue;  // lanes hold the nq + 1 chunk offsets
  int per_sm = 0;
  cudaError_t rc = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kGridChainThreads, 0);
  if (rc != cudaSuccess) return rc;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  // every CTA must be resident at once (cooperative launch): one per SM
  const int grid = num_sms;
  rc = cudaMemsetAsync(a.barrier, 0, sizeof(unsigned int), s);
  if (rc != cudaSuccess) return rc;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kGridChainThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {const_cast<GridChainArgs*>(&a)};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace sdnn

// Post-threshold layers once no residue row is left.
//
// After the threshold clustering, a row whose activations equal its centroid's
// has no residue and never gets one again (a zero residue updates to zero), so
// when the residue list is empty the rest of the inference is the K centroid
// rows alone, carried through the remaining layers (SNICIT's post_spMM +
// post_minus with nerow = K, src/SDGC/SNICIT/kernel.hpp:71-136).  Run as one
// launch per layer, that is 2 launches of a few microseconds each for a few
// rows.  Here one thread-block cluster runs all of those layers in one launch:
//
//  * every CTA of the cluster keeps all K rows in shared memory (two buffers,
//    this layer's input and the next layer's);
//  * CTA r computes the outputs of its share of the 32-neuron groups for all K
//    rows, with the same bank-scheduled slots and FP32 order as layer_kernel
//    (so the rows are bitwise equal to the per-layer path), applies bias and
//    clamp, and stores each output into the next-layer buffer of every CTA of
//    the cluster (distributed shared memory);
//  * a cluster barrier separates layers; after the last layer the rows go to
//    the final activation buffer for recovery.
#include <cooperative_groups.h>

#include "layer_kernel.cuh"

namespace cg = cooperative_groups;

namespace sdnn {

constexpr int kChainCluster = 8;

template <int RSW, int KC>
__global__ void __launch_bounds__(512, 1) chain_kernel(const ChainArgs a) {
  extern __shared__ __align__(128) float rows[];  // [2][KC][RSW]
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int csize = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int N = a.N;
  const int K = min(*a.ccount, KC);
  // zero columns of both buffers, then this layer's rows from the threshold buffer
  for (int i = tid; i < 2 * KC * 32; i += blockDim.x) rows[(i >> 5) * RSW + N + (i & 31)] = 0.f;
  for (int t = 0; t < K; ++t) {
    const float* src = a.y_in + (size_t)a.clist[t] * N;
    for (int j = tid; j < N; j += blockDim.x) rows[t * RSW + j] = src[j];
  }
  cluster.sync();
  const int gbeg = (int)((long)a.G * rank / csize), gend = (int)((long)a.G * (rank + 1) / csize);
  // this CTA's slot blocks of layer l are contiguous: prefetch them into L2 a
  // few layers ahead so the per-layer loads hit L2 instead of HBM
  auto prefetch = [&](int l) {
    if (tid != 0 || l >= a.last) return;
    const LayerDev wp = a.layers[l];
    const int32_t b0 = wp.grp_blk[gbeg], b1 = wp.grp_blk[gend];
    const uint32_t bytes = (uint32_t)(b1 - b0) * 32u * (uint32_t)sizeof(uint2);
    if (bytes > 0)
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(wp.idx + (size_t)b0 * 32),
                   "r"(bytes)
                   : "memory");
    if (wp.val && bytes > 0)
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(wp.val + (size_t)b0 * 32),
                   "r"(bytes * 2u)
                   : "memory");
  };
  for (int d = 0; d < 4; ++d) prefetch(a.first + d);
  for (int l = a.first; l < a.last; ++l) {
    prefetch(l + 4);
    const LayerDev wl = a.layers[l];
    const float* cur = rows + (size_t)((l - a.first) & 1) * KC * RSW;
    float* nxt = rows + (size_t)(((l - a.first) & 1) ^ 1) * KC * RSW;
    const bool last = l + 1 == a.last;
    for (int g = gbeg + warp; g < gend; g += nwarps) {
      float acc[KC];
#pragma unroll
      for (int t = 0; t < KC; ++t) acc[t] = 0.f;
      if (wl.val == nullptr)
        accumulate_group<KC, RSW, true>(acc, wl, 1, cur, RSW, g, 0, lane);
      else
        accumulate_group<KC, RSW, false>(acc, wl, 1, cur, RSW, g, 0, lane);
      const int c = g * 32 + lane;
      const float bc = wl.bias_vec ? __ldg(wl.bias_vec + c) : wl.bias;
#pragma unroll
      for (int t = 0; t < KC; ++t) {
        if (t < K) {
          const float y = clampf(acc[t] + bc, a.clampv);
          for (int p = 0; p < csize; ++p) cluster.map_shared_rank(nxt, p)[t * RSW + c] = y;
          if (last) a.y_out[(size_t)a.clist[t] * N + c] = y;
        }
      }
    }
    cluster.sync();
  }
}

template __global__ void chain_kernel<1056, 1>(const ChainArgs);
template __global__ void chain_kernel<1056, 2>(const ChainArgs);
template __global__ void chain_kernel<1056, 4>(const ChainArgs);
template __global__ void chain_kernel<1056, 8>(const ChainArgs);
template __global__ void chain_kernel<4128, 1>(const ChainArgs);
template __global__ void chain_kernel<4128, 2>(const ChainArgs);
template __global__ void chain_kernel<4128, 4>(const ChainArgs);
template __global__ void chain_kernel<16416, 1>(const ChainArgs);

static const void* chain_fn(int rsw, int kc) {
#define SDNN_PICK(R, K) \
  if (rsw == R && kc == K) return (const void*)&chain_kernel<R, K>;
  SDNN_PICK(1056, 1)
  SDNN_PICK(1056, 2)
  SDNN_PICK(1056, 4)
  SDNN_PICK(1056, 8)
  SDNN_PICK(4128, 1)
  SDNN_PICK(4128, 2)
  SDNN_PICK(4128, 4)
  SDNN_PICK(16416, 1)
#undef SDNN_PICK
  return nullptr;
}

int chain_capacity(int N) {
  const int rsw = N + 32;
  int best = 0;
  for (int kc : {1, 2, 4, 8})
    if (chain_fn(rsw, kc)) best = kc;
  return best;
}

cudaError_t launch_chain(const ChainArgs& a, int kc_needed, cudaStream_t s) {
  const int rsw = a.N + 32;
  int kc = 0;
  for (int k : {1, 2, 4, 8})
    if (k >= kc_needed && chain_fn(rsw, k)) {
      kc = k;
      break;
    }
  const void* fn = kc ? chain_fn(rsw, kc) : nullptr;
  if (!fn) return cudaErrorInvalidValue;
  const size_t smem = (size_t)2 * kc * rsw * sizeof(float);
  cudaError_t rc = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (rc != cudaSuccess) return rc;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kChainCluster);
  cfg.blockDim = dim3(512);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kChainCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {const_cast<ChainArgs*>(&a)};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace sdnn

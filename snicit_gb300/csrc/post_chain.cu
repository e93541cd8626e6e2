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
#include <algorithm>

#include <cooperative_groups.h>

#include "layer_kernel.cuh"

namespace cg = cooperative_groups;

namespace sdnn {

constexpr int kChainCluster = 8;

template <int RSW, int KC>
__global__ void __launch_bounds__(1024, 1) chain_kernel(const ChainArgs a) {
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

// ---------------------------------------------------------------------------
// chain2_kernel: the same computation with the weights streamed into shared
// memory and point-to-point row exchange.
//
//  * one producer warp (the last warp of the CTA) copies this CTA's slot
//    blocks of a layer into a shared weight buffer with a 1-D TMA bulk copy
//    (and the group offsets with plain loads), so the 16 compute warps read
//    indices from shared memory instead of waiting on L2.  With two weight
//    buffers (NWBUF = 2) it runs a layer ahead: once the inputs of layer l are
//    complete no warp reads the weights of layer l - 1 any more, and it
//    fetches layer l + 1 into their buffer.  With one buffer (the weight slice
//    of a layer is large: N = 16384) it fetches layer l + 1 as soon as the
//    local compute warps are done with layer l;
//  * outputs go to every CTA of the cluster with st.async, each signalling
//    the receiving CTA's mbarrier for its next row buffer with 4 bytes; a CTA
//    starts layer l + 1 when all N x K values of its next buffer have
//    arrived -- no cluster-wide barrier per layer;
//  * two row buffers suffice: a CTA that starts layer l has received every
//    CTA's layer l - 1 outputs, which each CTA sends only after it has read
//    all of its layer l - 1 inputs -- the buffer that layer l's outputs
//    overwrite everywhere.
// Same slots, same FMA order as layer_kernel and chain_kernel: bitwise equal.
constexpr int kChain2ComputeWarps = 16;
constexpr int kChain2MaxGroups = 64;  // groups per CTA (G / cluster size)

__device__ __forceinline__ uint32_t mapa_u32(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_async_f32(uint32_t raddr, float v, uint32_t rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(
                   raddr),
               "r"(__float_as_uint(v)), "r"(rbar)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait; after a timeout (error word set) every later wait of this
// thread is skipped so the kernel runs to its end.
__device__ __forceinline__ void chain_wait(uint64_t* bar, uint32_t parity, bool& failed,
                                           int32_t* err) {
  if (failed) return;
  if (!mbar_wait_bounded(bar, parity, err)) failed = true;
}

template <int KC, int RSW, bool CONSTW>
__device__ __forceinline__ void accumulate_smem(float (&acc)[KC], const uint2* __restrict__ sidx,
                                                const float4* __restrict__ sval, int nb, float wc,
                                                const float* __restrict__ ys, int lane) {
  int b = 0;
  for (; b + 8 <= nb; b += 8) {
    uint2 iv[8];
    float4 vv[CONSTW ? 1 : 8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      iv[k] = sidx[(b + k) * 32 + lane];
      if constexpr (!CONSTW) vv[k] = sval[(b + k) * 32 + lane];
    }
    apply_blocks<KC, RSW, CONSTW, 8>(acc, iv, vv, wc, ys, RSW);
  }
  for (; b < nb; ++b) {
    uint2 iv[1];
    float4 vv[1];
    iv[0] = sidx[b * 32 + lane];
    if constexpr (!CONSTW) vv[0] = sval[b * 32 + lane];
    apply_blocks<KC, RSW, CONSTW, 1>(acc, iv, vv, wc, ys, RSW);
  }
}

template <int RSW, int KC, int NWBUF>
__global__ void __launch_bounds__((kChain2ComputeWarps + 1) * 32, 1) chain2_kernel(const ChainArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  float* rows = reinterpret_cast<float*>(smem);  // [2][KC][RSW]
  unsigned char* wbase = smem + (size_t)2 * KC * RSW * 4;  // [NWBUF][wcap]
  __shared__ __align__(8) uint64_t rb[2];  // row buffer b complete
  __shared__ __align__(8) uint64_t wb[2];  // weight buffer b loaded
  __shared__ __align__(8) uint64_t cd;     // local compute warps done with a layer (NWBUF = 1)
  __shared__ int32_t s_gb[2][kChain2MaxGroups + 1];
  __shared__ LayerDev s_wl[2];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int csize = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool producer = warp == kChain2ComputeWarps;
  const int N = a.N;
  const int K = min(*a.ccount, KC);
  const int gbeg = (int)((long)a.G * rank / csize), gend = (int)((long)a.G * (rank + 1) / csize);
  const int ng = gend - gbeg;
  const uint32_t row_bytes = (uint32_t)K * (uint32_t)N * 4u;
  const uint32_t wcap = a.wcap;
  bool failed = false;
  int wcnt[2] = {0, 0};  // producer: copies issued into each weight buffer

  auto load_bounds = [&](int l, int32_t* dst) {  // producer warp
    const int32_t* gb = a.layers[l].grp_blk + gbeg;
    for (int i = lane; i <= ng; i += 32) dst[i] = __ldg(gb + i);
  };
  auto issue_weights = [&](int l, int buf) {  // producer lane 0, after load_bounds + syncwarp
    const LayerDev wl = a.layers[l];
    s_wl[buf] = wl;  // published to the compute warps by the arrive below
    ++wcnt[buf];
    const int32_t b0 = s_gb[buf][0], nblk = s_gb[buf][ng] - b0;
    const uint32_t bi = (uint32_t)nblk * 32u * 8u;
    const uint32_t bv = wl.val ? (uint32_t)nblk * 32u * 16u : 0u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&wb[buf], bi + bv);
    unsigned char* dst = wbase + (size_t)buf * wcap;
    if (bi) bulk_g2s(dst, wl.idx + (size_t)b0 * 32, bi, &wb[buf]);
    if (bv) bulk_g2s(dst + bi, wl.val + (size_t)b0 * 32, bv, &wb[buf]);
  };
  auto fetch_layer = [&](int l, int buf) {  // whole producer warp
    load_bounds(l, s_gb[buf]);
    __syncwarp();
    if (lane == 0) issue_weights(l, buf);
    __syncwarp();
  };
  auto prefetch_l2 = [&](int l) {  // producer lane 0
    if (l >= a.last) return;
    const LayerDev wp = a.layers[l];
    const int32_t b0 = __ldg(wp.grp_blk + gbeg), b1 = __ldg(wp.grp_blk + gend);
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

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) mbar_init(&rb[i], 1);
    for (int i = 0; i < 2; ++i) mbar_init(&wb[i], 1);
    mbar_init(&cd, kChain2ComputeWarps);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < 2 * KC * 32; i += blockDim.x) rows[(i >> 5) * RSW + N + (i & 31)] = 0.f;
  for (int t = 0; t < K; ++t) {
    const float* src = a.y_in + (size_t)a.clist[t] * N;
    for (int j = tid; j < N; j += blockDim.x) rows[t * RSW + j] = src[j];
  }
  __syncthreads();
  if (producer) {
    fetch_layer(a.first, 0);
    if (lane == 0)
      for (int d = 1; d < 4; ++d) prefetch_l2(a.first + d);
  }
  cluster.sync();  // every CTA's barriers exist before any remote store

  uint32_t rpar = 0u, wpar = 0u, cdpar = 0u;
  for (int l = a.first; l < a.last; ++l) {
    const int li = l - a.first;
    const int cur = li & 1, nxt = cur ^ 1;
    const int wcur = NWBUF == 2 ? (li & 1) : 0;
    const bool last = l + 1 == a.last;
    if (producer) {
      if constexpr (NWBUF == 2) {
        // inputs of layer l complete: the weight buffer of layer l - 1 is free
        if (li > 0) {
          chain_wait(&rb[cur], (rpar >> cur) & 1u, failed, a.err);
          rpar ^= 1u << cur;
        }
        if (!last) {
          if (lane == 0) mbar_expect_tx(&rb[nxt], row_bytes);
          fetch_layer(l + 1, wcur ^ 1);
          if (lane == 0) prefetch_l2(l + 4);
        }
      } else {
        // the single weight buffer: layer l was fetched when layer l - 1 was done
        if (!last && lane == 0) mbar_expect_tx(&rb[nxt], row_bytes);
        if (!last) {
          chain_wait(&cd, cdpar, failed, a.err);
          cdpar ^= 1u;
          fetch_layer(l + 1, 0);
          if (lane == 0) prefetch_l2(l + 3);
        }
      }
      continue;
    }
    if (li > 0) {
      chain_wait(&rb[cur], (rpar >> cur) & 1u, failed, a.err);
      rpar ^= 1u << cur;
    }
    chain_wait(&wb[wcur], (wpar >> wcur) & 1u, failed, a.err);
    wpar ^= 1u << wcur;
    const LayerDev wl = s_wl[wcur];
    const float* cur_rows = rows + (size_t)cur * KC * RSW;
    const unsigned char* wsm = wbase + (size_t)wcur * wcap;
    const int32_t gb0 = s_gb[wcur][0];
    const int32_t nblk_all = s_gb[wcur][ng] - gb0;
    const uint2* sidx = reinterpret_cast<const uint2*>(wsm);
    const float4* sval = reinterpret_cast<const float4*>(wsm + (size_t)nblk_all * 32 * 8);
    const uint32_t nbuf_base = smem_u32(rows + (size_t)nxt * KC * RSW);
    const uint32_t nbar = smem_u32(&rb[nxt]);
    for (int g = gbeg + warp; g < gend; g += kChain2ComputeWarps) {
      const int c = g * 32 + lane;
      const float bc = wl.bias_vec ? __ldg(wl.bias_vec + c) : wl.bias;
      const int32_t o = s_gb[wcur][g - gbeg] - gb0;
      const int nb = s_gb[wcur][g - gbeg + 1] - s_gb[wcur][g - gbeg];
      float acc[KC];
#pragma unroll
      for (int t = 0; t < KC; ++t) acc[t] = 0.f;
      if (wl.val == nullptr)
        accumulate_smem<KC, RSW, true>(acc, sidx + (size_t)o * 32, nullptr, nb, wl.wconst, cur_rows,
                                       lane);
      else
        accumulate_smem<KC, RSW, false>(acc, sidx + (size_t)o * 32, sval + (size_t)o * 32, nb,
                                        wl.wconst, cur_rows, lane);
#pragma unroll
      for (int t = 0; t < KC; ++t) {
        if (t < K) {
          const float y = clampf(acc[t] + bc, a.clampv);
          if (last) {
            a.y_out[(size_t)a.clist[t] * N + c] = y;
          } else {
            const uint32_t la = nbuf_base + (uint32_t)(t * RSW + c) * 4u;
            for (int p = 0; p < csize; ++p)
              st_async_f32(mapa_u32(la, (uint32_t)p), y, mapa_u32(nbar, (uint32_t)p));
          }
        }
      }
    }
    if constexpr (NWBUF == 1) {
      __syncwarp();
      if (lane == 0 && !last) mbar_arrive(&cd);
    }
  }
  if (producer && lane == 0 && *reinterpret_cast<volatile int32_t*>(a.err) != 0) {
    // after a timeout the compute warps stop waiting: let the last copy issued
    // into each buffer land before the CTA exits
    for (int b = 0; b < 2; ++b) {
      bool f2 = false;
      if (wcnt[b] > 0) chain_wait(&wb[b], (uint32_t)(wcnt[b] - 1) & 1u, f2, a.err);
    }
  }
  cluster.sync();  // no CTA leaves while another may still store into it
}

template __global__ void chain2_kernel<1056, 1, 2>(const ChainArgs);
template __global__ void chain2_kernel<1056, 2, 2>(const ChainArgs);
template __global__ void chain2_kernel<1056, 4, 2>(const ChainArgs);
template __global__ void chain2_kernel<1056, 8, 2>(const ChainArgs);
template __global__ void chain2_kernel<4128, 1, 2>(const ChainArgs);
template __global__ void chain2_kernel<4128, 2, 2>(const ChainArgs);
template __global__ void chain2_kernel<4128, 4, 2>(const ChainArgs);
template __global__ void chain2_kernel<16416, 1, 1>(const ChainArgs);

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

static const void* chain2_fn(int rsw, int kc, int nwbuf) {
#define SDNN_PICK(R, K, W) \
  if (rsw == R && kc == K && nwbuf == W) return (const void*)&chain2_kernel<R, K, W>;
  SDNN_PICK(1056, 1, 2)
  SDNN_PICK(1056, 2, 2)
  SDNN_PICK(1056, 4, 2)
  SDNN_PICK(1056, 8, 2)
  SDNN_PICK(4128, 1, 2)
  SDNN_PICK(4128, 2, 2)
  SDNN_PICK(4128, 4, 2)
  SDNN_PICK(16416, 1, 1)
#undef SDNN_PICK
  return nullptr;
}

uint32_t chain_slice_bytes(const int32_t* grp_blk, int G, bool general, int cluster) {
  uint32_t best = 0;
  for (int r = 0; r < cluster; ++r) {
    const int gb = (int)((long)G * r / cluster), ge = (int)((long)G * (r + 1) / cluster);
    const uint32_t nblk = (uint32_t)(grp_blk[ge] - grp_blk[gb]);
    best = std::max(best, nblk * 32u * (general ? 24u : 8u));
  }
  return best;
}

int chain_capacity(int N) {
  const int rsw = N + 32;
  int best = 0;
  for (int kc : {1, 2, 4, 8})
    if (chain_fn(rsw, kc)) best = kc;
  return best;
}

static int chain_kc_for(int rsw, int kc_needed) {
  for (int k : {1, 2, 4, 8})
    if (k >= kc_needed && chain_fn(rsw, k)) return k;
  return 0;
}

static size_t chain2_smem(int rsw, int kc, int nwbuf, uint32_t wcap) {
  return (size_t)2 * kc * rsw * sizeof(float) + (size_t)nwbuf * wcap;
}

// Whether a cluster of 16 CTAs (non-portable size) can run this kernel here.
static bool cluster16_ok(const void* fn, int threads, size_t smem) {
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(16);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 16;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

ChainPlan chain_plan(const ChainArgs& a, int kc_needed) {
  ChainPlan p{};
  const int rsw = a.N + 32;
  const int kc = chain_kc_for(rsw, kc_needed);
  if (!kc) return p;
  p.kc = kc;
  p.variant = 1;
  p.cluster = kChainCluster;
  p.threads = 512;
  p.smem = (size_t)2 * kc * rsw * sizeof(float);
  // wide rows (many groups per CTA): a cluster of 16 and 1024 threads, one
  // group per warp at N = 16384
  if (a.G / kChainCluster > 32 && cluster16_ok(chain_fn(rsw, kc), 1024, p.smem)) {
    p.cluster = 16;
    p.threads = 1024;
  }
  if (!a.stream) return p;
  const int threads2 = (kChain2ComputeWarps + 1) * 32;
  // streamed weights: cluster 8 with two weight buffers, else 16 with two or one
  const struct { int cluster, nwbuf; uint32_t wcap; } opts[] = {
      {8, 2, a.wcap8}, {16, 2, a.wcap16}, {16, 1, a.wcap16}, {8, 1, a.wcap8}};
  for (const auto& o : opts) {
    if (o.wcap == 0 || (a.G + o.cluster - 1) / o.cluster > kChain2MaxGroups) continue;
    const void* fn = chain2_fn(rsw, kc, o.nwbuf);
    const size_t smem = chain2_smem(rsw, kc, o.nwbuf, o.wcap);
    if (!fn || smem > 227 * 1024) continue;
    if (o.cluster == 16 && !cluster16_ok(fn, threads2, smem)) continue;
    p.variant = 2;
    p.cluster = o.cluster;
    p.nwbuf = o.nwbuf;
    p.wcap = o.wcap;
    p.threads = threads2;
    p.smem = smem;
    return p;
  }
  return p;
}

cudaError_t launch_chain(const ChainArgs& a0, int kc_needed, cudaStream_t s) {
  const ChainPlan p = chain_plan(a0, kc_needed);
  if (!p.variant) return cudaErrorInvalidValue;
  const int rsw = a0.N + 32;
  ChainArgs a = a0;
  a.wcap = p.wcap;
  const void* fn = p.variant == 2 ? chain2_fn(rsw, p.kc, p.nwbuf) : chain_fn(rsw, p.kc);
  cudaError_t rc = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
  if (rc != cudaSuccess) return rc;
  if (p.cluster > 8) {
    rc = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (rc != cudaSuccess) return rc;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.cluster);
  cfg.blockDim = dim3(p.threads);
  cfg.dynamicSmemBytes = p.smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {&a};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace sdnn

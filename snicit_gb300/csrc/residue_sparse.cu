// Sparse residue rows of the SNICIT post-threshold stage.
//
// After the threshold every live row is a centroid row or centroid + residue
// Delta (src/SDGC/SNICIT/kernel.hpp:8-69).  As rows saturate towards their
// centroid, Delta keeps only a few nonzeros; the reference's post_spMM then
// skips the zero entries of the residue (kernel.hpp:71-102, `if (val != 0)`),
// but its post_minus still walks every output (kernel.hpp:104-136).  Here a
// residue row with at most SC nonzeros (N/32, at least 32: a sparse row's
// update runs on one warp, so longer lists would stretch the layer) is kept as
// a sorted (position, value) list and its update touches only what it must:
//
//   split_residue_kernel   residue conversion: one warp per dense residue row,
//                          warp ballot / popc compaction of the nonzeros into
//                          the row's list (ascending positions), or the row
//                          stays dense when it has more than SC nonzeros;
//   sparse_residue_kernel  one warp per sparse row: W * Delta by scattering each
//                          nonzero along its input's out-edges (the transposed
//                          layer, one edge per lane, entries in ascending
//                          order, so every output adds its terms in a fixed
//                          order: deterministic, no atomics on values) into a
//                          shared-memory row with a touched-output bitmap; then
//                          Delta' = f(pre_c + W Delta) - f(pre_c) on the
//                          touched outputs only (an untouched output has
//                          W Delta = 0, so Delta' = 0 there exactly), compacted
//                          again -- or written as a dense row when it grew past
//                          SC, or dropped from the lists when it is all zero
//                          (the row has converged to its centroid);
//   densify_kernel         the final sparse rows written densely into the last
//                          layer's buffer, so recovery reads every residue row
//                          the same way.
#include "sdnn_internal.h"

namespace sdnn {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kAhead = 16;  // entries whose edges are in flight at once

__device__ __forceinline__ float clamp_hi(float v, float hi) { return fminf(hi, fmaxf(0.f, v)); }

// Launched with programmatic stream serialization (like the layer kernel):
// the next launch may be scheduled now; everything this kernel reads comes
// from its predecessors, so it waits for them before the first read.
__device__ __forceinline__ void pdl_prologue() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename... Args>
cudaError_t launch_pdl(void (*fn)(Args...), int grid, int threads, size_t smem, cudaStream_t s,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, args...);
}

__global__ void split_residue_kernel(const float* __restrict__ y, const int32_t* list,
                                     const int32_t* count, SparseRows out, int32_t* dense_list,
                                     int32_t* dense_count, int32_t* sparse_list,
                                     int32_t* sparse_count, int32_t N) {
  pdl_prologue();
  const int n = *count;
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int SC = out.cap;
  for (int i = wid; i < n; i += nw) {
    const int r = list[i];
    const float4* yr = reinterpret_cast<const float4*>(y + (size_t)r * N);
    int32_t* oi = out.idx + (size_t)r * SC;
    float* ov = out.val + (size_t)r * SC;
    int base = 0;
    // 256 entries per round: lane L holds entries j0 + 4L .. j0 + 4L + 3 of
    // each 128-entry half (both halves loaded before either is compacted);
    // a lane's nonzeros go after those of the lanes below it, so the list
    // comes out in ascending position
    for (int j0 = 0; j0 < N && base <= SC; j0 += 256) {
      float4 v[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int j = j0 + 128 * h + 4 * lane;
        v[h] = j < N ? yr[j >> 2] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float e[4] = {v[h].x, v[h].y, v[h].z, v[h].w};
        const int nz = (e[0] != 0.f) + (e[1] != 0.f) + (e[2] != 0.f) + (e[3] != 0.f);
        int incl = nz;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int u = __shfl_up_sync(kFull, incl, d);
          if (lane >= d) incl += u;
        }
        int k = base + incl - nz;
        const int j = j0 + 128 * h + 4 * lane;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (e[t] != 0.f) {
            if (k < SC) {
              oi[k] = j + t;
              ov[k] = e[t];
            }
            ++k;
          }
        }
        base += __shfl_sync(kFull, incl, 31);
      }
    }
    if (lane == 0) {
      if (base <= SC) {
        out.cnt[r] = base;
        sparse_list[atomicAdd(sparse_count, 1)] = r;
      } else {
        dense_list[atomicAdd(dense_count, 1)] = r;
      }
    }
  }
}

__global__ void sparse_residue_kernel(const SparseResArgs a) {
  extern __shared__ __align__(16) float sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpc = blockDim.x >> 5;
  const int N = a.N, nwords = N >> 5, SC = a.in.cap;
  pdl_prologue();
  const int n = *a.count_in;
  if ((int)blockIdx.x * wpc >= n) return;  // no row for this CTA (often no row at all)
  float* acc = sm + (size_t)warp * (N + nwords);
  uint32_t* bm = reinterpret_cast<uint32_t*>(acc + N);
  for (int j = lane; j < N + nwords; j += 32) acc[j] = 0.f;  // also clears the bitmap
  __syncwarp();
  const float hi = a.clampv;
  for (int i = blockIdx.x * wpc + warp; i < n; i += gridDim.x * wpc) {
    const int r = a.list_in[i];
    const int cnt = a.in.cnt[r];
    const int32_t* ei = a.in.idx + (size_t)r * SC;
    const float* ev = a.in.val + (size_t)r * SC;
    // W * Delta: entries in ascending position, each along its out-edges.
    // Lane e holds entry e0 + e and its edge range; the edges of kAhead
    // entries are loaded before the first of them is applied (the loads do not
    // depend on one another), the multiply-adds stay in entry order.
    for (int e0 = 0; e0 < cnt; e0 += 32) {
      int my_j = 0, my_t0 = 0, my_t1 = 0;
      float my_v = 0.f;
      if (e0 + lane < cnt) {
        my_j = ei[e0 + lane];
        my_v = ev[e0 + lane];
        my_t0 = __ldg(a.tr_off + my_j);
        my_t1 = __ldg(a.tr_off + my_j + 1);
      }
      const int ne = min(32, cnt - e0);
      for (int e = 0; e < ne; e += kAhead) {
        int o[kAhead];
        float w[kAhead], v[kAhead];
        int deg[kAhead], t0[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
          const int src = min(e + u, ne - 1);
          t0[u] = __shfl_sync(kFull, my_t0, src);
          deg[u] = e + u < ne ? __shfl_sync(kFull, my_t1, src) - t0[u] : 0;
          v[u] = __shfl_sync(kFull, my_v, src);
          o[u] = lane < deg[u] ? (int)__ldg(a.tr_out + t0[u] + lane) : -1;
          w[u] = a.tr_val && lane < deg[u] ? __ldg(a.tr_val + t0[u] + lane) : a.wconst;
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
          if (o[u] >= 0) {
            acc[o[u]] = fmaf(w[u], v[u], acc[o[u]]);
            atomicOr(&bm[o[u] >> 5], 1u << (o[u] & 31));
          }
          // out-degrees above 32 (general layers): the rest of the edges
          for (int t = t0[u] + 32 + lane; t < t0[u] + deg[u]; t += 32) {
            const int oo = __ldg(a.tr_out + t);
            const float ww = a.tr_val ? __ldg(a.tr_val + t) : a.wconst;
            acc[oo] = fmaf(ww, v[u], acc[oo]);
            atomicOr(&bm[oo >> 5], 1u << (oo & 31));
          }
          __syncwarp();
        }
      }
    }
    const float* pre = a.pre + (size_t)a.cslot[r] * N;
    // pass 1: nonzeros of Delta' among the touched outputs
    int total = 0;
    for (int w0 = 0; w0 < nwords; w0 += 32) {
      const int wi = w0 + lane;
      uint32_t bits = wi < nwords ? bm[wi] : 0u;
      int nz = 0;
      while (bits) {
        const int c = wi * 32 + __ffs(bits) - 1;
        bits &= bits - 1u;
        const float pc = __ldg(pre + c);
        nz += (clamp_hi(pc + acc[c], hi) - clamp_hi(pc, hi)) != 0.f;
      }
      total += __reduce_add_sync(kFull, (unsigned)nz);
    }
    if (total > SC) {
      // grew past the list capacity: a dense row (the dense epilogue's formula;
      // an untouched output gives f(pc + 0) - f(pc) = 0)
      float* dst = a.y_out + (size_t)r * N;
      for (int c = lane; c < N; c += 32) {
        const float pc = __ldg(pre + c);
        dst[c] = clamp_hi(pc + acc[c], hi) - clamp_hi(pc, hi);
        acc[c] = 0.f;
      }
      for (int wi = lane; wi < nwords; wi += 32) bm[wi] = 0u;
      if (lane == 0) a.dense_list[atomicAdd(a.dense_count, 1)] = r;
    } else {
      // pass 2: the list in ascending position; touched outputs cleared
      int32_t* oi = a.out.idx + (size_t)r * SC;
      float* ov = a.out.val + (size_t)r * SC;
      int base = 0;
      for (int w0 = 0; w0 < nwords; w0 += 32) {
        const int wi = w0 + lane;
        const uint32_t word = wi < nwords ? bm[wi] : 0u;
        uint32_t bits = word, nzbits = 0u;
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1u;
          const int c = wi * 32 + b;
          const float pc = __ldg(pre + c);
          if ((clamp_hi(pc + acc[c], hi) - clamp_hi(pc, hi)) != 0.f) nzbits |= 1u << b;
        }
        const int nz = __popc(nzbits);
        int incl = nz;  // inclusive scan over the lanes
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int u = __shfl_up_sync(kFull, incl, d);
          if (lane >= d) incl += u;
        }
        int k = base + incl - nz;
        bits = word;
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1u;
          const int c = wi * 32 + b;
          if (nzbits & (1u << b)) {
            const float pc = __ldg(pre + c);
            oi[k] = c;
            ov[k] = clamp_hi(pc + acc[c], hi) - clamp_hi(pc, hi);
            ++k;
          }
          acc[c] = 0.f;
        }
        if (wi < nwords) bm[wi] = 0u;
        base += __shfl_sync(kFull, incl, 31);
      }
      if (lane == 0 && total > 0) {
        a.out.cnt[r] = total;
        a.sparse_list[atomicAdd(a.sparse_count, 1)] = r;
      }
    }
    __syncwarp();
  }
}

__global__ void densify_kernel(const int32_t* list, const int32_t* count, SparseRows rows,
                               float* y, int32_t N) {
  pdl_prologue();
  const int n = *count;
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = wid; i < n; i += nw) {
    const int r = list[i];
    float* dst = y + (size_t)r * N;
    for (int c = lane; c < N; c += 32) dst[c] = 0.f;
    __syncwarp();
    const int cnt = rows.cnt[r];
    const int32_t* ei = rows.idx + (size_t)r * rows.cap;
    const float* ev = rows.val + (size_t)r * rows.cap;
    for (int e = lane; e < cnt; e += 32) dst[ei[e]] = ev[e];
    __syncwarp();
  }
}

}  // namespace

size_t sparse_residue_smem_per_warp(int N) { return (size_t)(N + N / 32) * sizeof(float); }

int sparse_residue_warps(int N) {
  const size_t per = sparse_residue_smem_per_warp(N);
  const size_t budget = 200 * 1024;
  int w = (int)(budget / per);
  return w < 1 ? (per <= 227 * 1024 ? 1 : 0) : (w > 8 ? 8 : w);
}

cudaError_t sparse_residue_prepare(int N) {
  const int w = sparse_residue_warps(N);
  if (w <= 0) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(sparse_residue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(w * sparse_residue_smem_per_warp(N)));
}

void launch_split_residue(const float* y, const int32_t* list, const int32_t* count,
                          const SparseRows& out, int32_t* dense_list, int32_t* dense_count,
                          int32_t* sparse_list, int32_t* sparse_count, int32_t N, int num_sms,
                          cudaStream_t s) {
  launch_pdl(split_residue_kernel, num_sms * 8, 256, 0, s, y, list, count, out, dense_list,
             dense_count, sparse_list, sparse_count, N);
}

cudaError_t launch_sparse_residue(const SparseResArgs& a, int num_sms, cudaStream_t s) {
  const int w = sparse_residue_warps(a.N);
  if (w <= 0) return cudaErrorInvalidValue;
  const size_t smem = w * sparse_residue_smem_per_warp(a.N);
  int per_sm = (int)((227 * 1024) / (smem + 1024));
  per_sm = per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm);
  return launch_pdl(sparse_residue_kernel, num_sms * per_sm, w * 32, smem, s, a);
}

void launch_densify(const int32_t* list, const int32_t* count, const SparseRows& rows, float* y,
                    int32_t N, int num_sms, cudaStream_t s) {
  launch_pdl(densify_kernel, num_sms * 4, 256, 0, s, list, count, rows, y, N);
}

}  // namespace sdnn

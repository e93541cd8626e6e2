// Row-list utilities, category identification, the SNICIT threshold stage
// (candidate pick, pruning, nearest-centroid residue conversion) and recovery.
#include <climits>
#include "sdnn_internal.h"

namespace sdnn {

__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static int grid_for(long work, int per_block, int cap = 4096) {
  long g = (work + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

// ---------------------------------------------------------------- row lists

// Rows of the current inference come from a device scalar (set just before a
// captured graph is launched), so one graph serves every row count.
__global__ void set_scalar_kernel(int32_t* p, int32_t v) { *p = v; }
void launch_set_scalar(int32_t* p, int32_t v, cudaStream_t s) { set_scalar_kernel<<<1, 1, 0, s>>>(p, v); }

__global__ void post_choice_kernel(const PostChoiceArgs a, cudaGraphConditionalHandle h) {
  const int residues = *a.rcount + (a.scount ? *a.scount : 0), centroids = *a.ccount;
  int body = 0;
  if (!a.no_chain && residues == 0 && centroids >= 1) {
    int i = 0, kc = 1;
    while (kc < centroids) {
      kc *= 2;
      ++i;
    }
    if (i < 4) {
      // the cluster kernel where the rows fit shared memory, else the grid kernel
      if (centroids <= a.chain_cap && a.has_body[1 + 2 * i]) body = 1 + 2 * i;
      else if (centroids <= a.grid_cap && a.has_body[2 + 2 * i]) body = 2 + 2 * i;
    }
  }
  cudaGraphSetConditional(h, (unsigned)body);
  *a.choice = body;
}
void launch_post_choice(const PostChoiceArgs& a, cudaGraphConditionalHandle h, cudaStream_t s) {
  post_choice_kernel<<<1, 1, 0, s>>>(a, h);
}

__global__ void sum_piece_counts_kernel(const int32_t* pc, int pieces, int stride, int layers,
                                        int32_t* counts) {
  for (int l = threadIdx.x; l < layers; l += blockDim.x) {
    int32_t t = 0;
    for (int p = 0; p < pieces; ++p) t += pc[(size_t)p * stride + l];
    counts[l] = t;
  }
}
void launch_sum_piece_counts(const int32_t* piece_counts, int pieces, int stride, int layers,
                             int32_t* counts, cudaStream_t s) {
  sum_piece_counts_kernel<<<1, 256, 0, s>>>(piece_counts, pieces, stride, layers, counts);
}

__global__ void begin_rows_kernel(const int32_t* nrows, int32_t* list, int32_t* count,
                                  int32_t* zero_a, int32_t* zero_b, int32_t* neg) {
  const int n = *nrows;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    list[i] = i;
    if (zero_a) zero_a[i] = 0;
    if (zero_b) zero_b[i] = 0;
    if (neg) neg[i] = -1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = n;
}
void launch_begin_rows(const int32_t* nrows, int32_t* list, int32_t* count, int32_t* zero_a,
                       int32_t* zero_b, int32_t* neg, cudaStream_t s) {
  begin_rows_kernel<<<264, 256, 0, s>>>(nrows, list, count, zero_a, zero_b, neg);
}

__global__ void zero_rows_kernel(const int32_t* nrows, int32_t* a, int32_t* b) {
  const int n = *nrows;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a[i] = 0;
    if (b) b[i] = 0;
  }
}
void launch_zero_rows(const int32_t* nrows, int32_t* a, int32_t* b, cudaStream_t s) {
  zero_rows_kernel<<<264, 256, 0, s>>>(nrows, a, b);
}

__global__ void copy_rows_kernel(const int32_t* nrows, const float4* src, float4* dst, int32_t n4) {
  const size_t total = (size_t)(*nrows) * (size_t)n4;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
void launch_copy_rows(const int32_t* nrows, const float* src, float* dst, int32_t N, cudaStream_t s) {
  copy_rows_kernel<<<1024, 256, 0, s>>>(nrows, reinterpret_cast<const float4*>(src),
                                        reinterpret_cast<float4*>(dst), N / 4);
}

__global__ void mark_rows_kernel(const int32_t* list, const int32_t* count, int32_t* flags,
                                 int32_t value) {
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flags[list[i]] = value;
}
void launch_mark_rows(const int32_t* list, const int32_t* count, int32_t* flags, int32_t value,
                      cudaStream_t s) {
  mark_rows_kernel<<<264, 256, 0, s>>>(list, count, flags, value);
}

// identify (src/SDGC/utility.hpp:194-212): category = 1 if the row has an
// activation > 0.  (The reference sums the row with thrust::reduce and an int
// initial value; see the oracle for that variant.)  One warp per listed row.
__global__ void identify_kernel(const float* __restrict__ y, const int32_t* list,
                                const int32_t* count, int32_t N, int32_t* flags) {
  const int n = *count;
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = wid; i < n; i += nw) {
    const int r = list[i];
    const float* row = y + (size_t)r * N;
    bool any = false;
    for (int j = lane; j < N && !any; j += 32) any = row[j] > 0.f;
    any = __any_sync(0xffffffffu, any);
    if (lane == 0) flags[r] = any ? 1 : 0;
  }
}
void launch_identify(const float* y, const int32_t* list, const int32_t* count, int32_t N,
                     int32_t* flags, cudaStream_t s) {
  identify_kernel<<<528, 256, 0, s>>>(y, list, count, N, flags);
}

// Ordered compaction: ids = sorted indices i with flags[i] != 0.  One CTA.
__global__ void __launch_bounds__(1024) flags_to_ids_kernel(const int32_t* flags, int32_t n,
                                                            int32_t* ids, int32_t* count) {
  __shared__ int wsum[32];
  __shared__ int s_total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int base = 0;
  for (int start = 0; start < n; start += 4096) {
    int f[4];
    int local = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = start + tid * 4 + u;
      f[u] = (i < n && flags[i] != 0) ? 1 : 0;
      local += f[u];
    }
    // inclusive warp scan of local
    int inc = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      int w = wsum[lane];
      int winc = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= o) winc += v;
      }
      wsum[lane] = winc - w;
      if (lane == 31) s_total = winc;
    }
    __syncthreads();
    int pos = base + wsum[warp] + inc - local;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (f[u]) ids[pos++] = start + tid * 4 + u;
    base += s_total;
    __syncthreads();
  }
  if (tid == 0) *count = base;
}
void launch_flags_to_ids(const int32_t* flags, int32_t n, int32_t* ids, int32_t* count,
                         cudaStream_t s) {
  flags_to_ids_kernel<<<1, 1024, 0, s>>>(flags, n, ids, count);
}

// ------------------------------------------------------- SNICIT threshold stage
//
// Reference: reduction + centroid_sel (src/SDGC/SNICIT/kernel.hpp:138-194),
// host y* compaction (src/SDGC/SNICIT/SNICIT.hpp:457-462), coarse_cluster
// (kernel.hpp:8-69) and the host ne_record -> rowsY pass (SNICIT.hpp:505-509).
// Differences, by design: candidates are a seeded pick of K live rows (the
// reference takes the first 32 rows of the batch); the 16 downsampling bins
// are disjoint N/16-neuron ranges for every N; the centroid pick and the
// residue list are built on the device.

constexpr int kHistBins = 4096;
constexpr int kCandCap = 2048;

__global__ void __launch_bounds__(1024) cand_select_kernel(ClusterArgs a) {
  __shared__ int hist[kHistBins];
  __shared__ unsigned long long skey[kCandCap];
  __shared__ int srow[kCandCap];
  __shared__ int s_cut, s_n;
  const int tid = threadIdx.x;
  const int n = *a.live_count;
  const int K = a.K;
  for (int i = tid; i < kHistBins; i += blockDim.x) hist[i] = 0;
  if (tid == 0) s_n = 0;
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    const uint64_t key = mix64(a.seed ^ mix64((uint64_t)a.live[i]));
    atomicAdd(&hist[key >> 52], 1);
  }
  __syncthreads();
  if (tid < 32) {
    // first bin whose cumulative count reaches K: lane i sums bins
    // [128 i, 128 i + 128), a warp scan finds the lane, that lane walks its bins
    constexpr int per = kHistBins / 32;
    int part = 0;
    for (int b = 0; b < per; ++b) part += hist[tid * per + b];
    int incl = part;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (tid >= o) incl += v;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, incl >= K);
    if (hit == 0u) {
      if (tid == 0) s_cut = kHistBins - 1;  // fewer live rows than K: all are candidates
    } else if (tid == __ffs(hit) - 1) {
      int cum = incl - part, cut = (tid + 1) * per - 1;
      for (int b = 0; b < per; ++b) {
        cum += hist[tid * per + b];
        if (cum >= K) {
          cut = tid * per + b;
          break;
        }
      }
      s_cut = cut;
    }
  }
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    const int r = a.live[i];
    const uint64_t key = mix64(a.seed ^ mix64((uint64_t)r));
    if ((int)(key >> 52) <= s_cut) {
      const int pos = atomicAdd(&s_n, 1);
      if (pos < kCandCap) {
        skey[pos] = key;
        srow[pos] = r;
      }
    }
  }
  __syncthreads();
  const int m = min(s_n, kCandCap);
  int M = 1;
  while (M < m) M <<= 1;
  for (int i = m + tid; i < M; i += blockDim.x) {
    skey[i] = ~0ull;
    srow[i] = INT_MAX;
  }
  __syncthreads();
  // bitonic sort on (key, row)
  for (int k = 2; k <= M; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < M; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const unsigned long long ki = skey[i], kj = skey[ixj];
          const int ri = srow[i], rj = srow[ixj];
          const bool gt = (ki > kj) || (ki == kj && ri > rj);
          if (gt == up) {
            skey[i] = kj;
            skey[ixj] = ki;
            srow[i] = rj;
            srow[ixj] = ri;
          }
        }
      }
      __syncthreads();
    }
  }
  const int nc = min(K, m);
  for (int i = tid; i < nc; i += blockDim.x) a.cand[i] = srow[i];
  if (tid == 0) *a.ncand = nc;
}

// 16 disjoint bin sums per candidate; one warp per bin, fixed reduction order.
__global__ void cand_bins_kernel(ClusterArgs a) {
  const int k = blockIdx.x;
  if (k >= *a.ncand) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float* row = a.y + (size_t)a.cand[k] * a.N;
  const int w = a.N / 16;
  for (int b = warp; b < 16; b += blockDim.x >> 5) {
    float s = 0.f;
    for (int j = b * w + lane; j < (b + 1) * w; j += 32) s += row[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) a.bins[k * 16 + b] = s;
  }
}

// Greedy pruning (paper Alg. 1; centroid_sel, src/SDGC/SNICIT/kernel.hpp:156-194):
// candidate k is dropped when an earlier kept candidate has every one of the 16
// bins within 0.03 (the reference drops when fewer than 16*0.03 bins differ by
// more than 0.03, i.e. when none does).
__global__ void __launch_bounds__(256) prune_kernel(ClusterArgs a) {
  __shared__ int keep[256];
  __shared__ float sb[256 * 16];
  const int tid = threadIdx.x;
  const int nc = min(*a.ncand, 256);
  for (int i = tid; i < nc * 16; i += blockDim.x) sb[i] = a.bins[i];
  if (tid < nc) keep[tid] = 1;
  __syncthreads();
  for (int k = 1; k < nc; ++k) {
    bool similar = false;
    if (tid < k && keep[tid]) {
      similar = true;
      for (int b = 0; b < 16; ++b)
        if (fabsf(sb[k * 16 + b] - sb[tid * 16 + b]) > 0.03f) {
          similar = false;
          break;
        }
    }
    const int any = __syncthreads_or(similar);
    if (tid == 0 && any) keep[k] = 0;
    __syncthreads();
  }
  if (tid == 0) {
    int ci = 0;
    for (int k = 0; k < nc; ++k) {
      if (!keep[k]) continue;
      const int r = a.cand[k];
      a.clist[ci] = r;
      a.cslot[r] = ci;
      a.is_centroid[r] = 1;
      ++ci;
    }
    *a.ccount = ci;
  }
}

// Nearest centroid by L0 distance (count of differing entries), ties to the
// lowest centroid index, residue written in place: y[r] <- y[r] - c.  Rows at
// distance 0 get no residue and are left out of the residue list.
__global__ void assign_kernel(ClusterArgs a) {
  const int n = *a.live_count;
  const int nc = *a.ccount;
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int N = a.N;
  for (int i = wid; i < n; i += nw) {
    const int r = a.live[i];
    if (a.is_centroid[r]) continue;
    float* yr = a.y + (size_t)r * N;
    const float4* yr4 = reinterpret_cast<const float4*>(yr);
    int best = INT_MAX, bk = 0;
    for (int k = 0; k < nc; ++k) {
      const float4* yc4 = reinterpret_cast<const float4*>(a.y + (size_t)a.clist[k] * N);
      int dt = 0;
      // 1024 entries per step, all 16 loads of a lane in flight before the
      // comparisons; stop as soon as this centroid cannot be nearer
      for (int j0 = 0; j0 < N; j0 += 1024) {
        float4 u[8], v[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int j = j0 + 128 * t + 4 * lane;
          u[t] = j < N ? yr4[j >> 2] : make_float4(0.f, 0.f, 0.f, 0.f);
          v[t] = j < N ? yc4[j >> 2] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        int dl = 0;
#pragma unroll
        for (int t = 0; t < 8; ++t)
          dl += (u[t].x != v[t].x) + (u[t].y != v[t].y) + (u[t].z != v[t].z) + (u[t].w != v[t].w);
        dt += (int)__reduce_add_sync(0xffffffffu, (unsigned)dl);
        if (dt >= best) break;
      }
      if (dt < best) {
        best = dt;
        bk = k;
        if (best == 0) break;
      }
    }
    if (lane == 0) a.cslot[r] = bk;
    if (best > 0) {
      const float* yc = a.y + (size_t)a.clist[bk] * N;
      for (int j = lane; j < N; j += 32) yr[j] = yr[j] - yc[j];
      if (lane == 0) {
        const int pos = atomicAdd(a.rcount, 1);
        a.rlist[pos] = r;
      }
    }
  }
}

void launch_cluster(const ClusterArgs& a, int num_sms, cudaStream_t s) {
  cand_select_kernel<<<1, 1024, 0, s>>>(a);
  cand_bins_kernel<<<a.K, 512, 0, s>>>(a);
  prune_kernel<<<1, 256, 0, s>>>(a);
  assign_kernel<<<num_sms * 4, 256, 0, s>>>(a);
}

// ------------------------------------------------------------------ recovery

// recover (src/SDGC/SNICIT/kernel.hpp:197-218): flags[r] = any((delta + c) > 0).
__global__ void recover_kernel(const float* __restrict__ y, const int32_t* live,
                               const int32_t* live_count, const int32_t* cslot,
                               const int32_t* clist, const int32_t* is_centroid,
                               const int32_t* res_flag, int32_t N, int32_t* flags) {
  const int n = *live_count;
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = wid; i < n; i += nw) {
    const int r = live[i];
    const float* yr = y + (size_t)r * N;
    bool any = false;
    if (is_centroid[r]) {
      for (int j = lane; j < N && !any; j += 32) any = yr[j] > 0.f;
    } else {
      const float* yc = y + (size_t)clist[cslot[r]] * N;
      if (res_flag[r]) {
        for (int j = lane; j < N && !any; j += 32) any = (yr[j] + yc[j]) > 0.f;
      } else {
        for (int j = lane; j < N && !any; j += 32) any = yc[j] > 0.f;
      }
    }
    any = __any_sync(0xffffffffu, any);
    if (lane == 0) flags[r] = any ? 1 : 0;
  }
}
void launch_recover(const float* y, const int32_t* live, const int32_t* live_count,
                    const int32_t* cslot, const int32_t* clist, const int32_t* is_centroid,
                    const int32_t* res_flag, int32_t N, int32_t* flags, cudaStream_t s) {
  recover_kernel<<<528, 256, 0, s>>>(y, live, live_count, cslot, clist, is_centroid, res_flag, N,
                                     flags);
}

// Final activations per row, in neuron order (out[r][c] reads position perm[c]):
// state 0 -> zeros (dead), 1 -> copy of the final buffer (plain modes),
// 2 -> SNICIT recovery (centroid, or centroid + residue).
__global__ void materialize_kernel(const float* __restrict__ y, const int32_t* state,
                                   const int32_t* cslot, const int32_t* clist,
                                   const int32_t* is_centroid, const int32_t* res_flag,
                                   const int32_t* alias, const int32_t* perm, int32_t N,
                                   int32_t rows, float* out) {
  for (int ro = blockIdx.x; ro < rows; ro += gridDim.x) {
    float* o = out + (size_t)ro * N;
    const int r = alias && alias[ro] >= 0 ? alias[ro] : ro;
    const int st = state[r];
    const float* yr = y + (size_t)r * N;
    if (st == 0) {
      for (int j = threadIdx.x; j < N; j += blockDim.x) o[j] = 0.f;
      continue;
    }
    const bool plain = st == 1 || is_centroid[r];
    const float* yc = plain ? yr : y + (size_t)clist[cslot[r]] * N;
    const bool has_res = !plain && res_flag[r];
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const int p = perm ? perm[j] : j;
      o[j] = plain ? yr[p] : (has_res ? yr[p] + yc[p] : yc[p]);
    }
  }
}

void launch_materialize(const float* y, const int32_t* state, const int32_t* cslot,
                        const int32_t* clist, const int32_t* is_centroid, const int32_t* res_flag,
                        const int32_t* alias, const int32_t* perm, int32_t N, float* out,
                        int32_t rows, cudaStream_t s) {
  materialize_kernel<<<grid_for(rows, 1, 8192), 256, 0, s>>>(y, state, cslot, clist, is_centroid,
                                                             res_flag, alias, perm, N, rows, out);
}

// Dense output head on the final activations (dense_output,
// src/beyond/general.hpp:74-102: logits = y . H + b, no activation), one warp
// per row, rows read the way materialize_kernel reads them (dead rows are
// zero, SNICIT rows are recovered).  Hp is the head stored by final position
// (Hp[p][k] = H[neuron at p][k]); lane-strided sums over positions, then a
// fixed xor-shuffle tree: deterministic.  argmax: first maximal logit.
template <int H>
__global__ void head_kernel(const float* __restrict__ y, const int32_t* state, const int32_t* cslot,
                            const int32_t* clist, const int32_t* is_centroid,
                            const int32_t* res_flag, const int32_t* alias,
                            const float* __restrict__ Hp, const float* __restrict__ hb, int32_t N,
                            int32_t rows, float* logits, int32_t* argmax) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int ro = wid; ro < rows; ro += nw) {
    float acc[H];
#pragma unroll
    for (int k = 0; k < H; ++k) acc[k] = 0.f;
    const int r = alias && alias[ro] >= 0 ? alias[ro] : ro;
    const int st = state[r];
    if (st != 0) {
      const float* yr = y + (size_t)r * N;
      const bool plain = st == 1 || is_centroid[r];
      const float* yc = plain ? yr : y + (size_t)clist[cslot[r]] * N;
      const bool has_res = !plain && res_flag[r];
      for (int p = lane; p < N; p += 32) {
        const float v = plain ? yr[p] : (has_res ? yr[p] + yc[p] : yc[p]);
        if (v != 0.f) {
#pragma unroll
          for (int k = 0; k < H; ++k) acc[k] = fmaf(v, __ldg(Hp + (size_t)p * H + k), acc[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < H; ++k) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    }
    if (lane == 0) {
      int best = 0;
      float bv = 0.f;
#pragma unroll
      for (int k = 0; k < H; ++k) {
        const float v = acc[k] + hb[k];
        logits[(size_t)ro * H + k] = v;
        if (k == 0 || v > bv) {
          bv = v;
          best = k;
        }
      }
      argmax[ro] = best;
    }
  }
}

bool launch_head(const float* y, const int32_t* state, const int32_t* cslot, const int32_t* clist,
                 const int32_t* is_centroid, const int32_t* res_flag, const int32_t* alias,
                 const float* Hp, const float* hb, int32_t H, int32_t N, int32_t rows,
                 float* logits, int32_t* argmax, cudaStream_t s) {
  const int grid = grid_for(rows, 8, 2048);
#define SDNN_HEAD(K)                                                                           \
  case K:                                                                                     \
    head_kernel<K><<<grid, 256, 0, s>>>(y, state, cslot, clist, is_centroid, res_flag, alias, Hp, \
                                        hb, N, rows, logits, argmax);                         \
    return true;
  switch (H) {
    SDNN_HEAD(1)
    SDNN_HEAD(2)
    SDNN_HEAD(4)
    SDNN_HEAD(8)
    SDNN_HEAD(10)
    SDNN_HEAD(16)
    SDNN_HEAD(32)
    default: return false;
  }
#undef SDNN_HEAD
}

}  // namespace sdnn

namespace sdnn {

// One-bit input rows (entry j in bit j % 64 of word j / 64, ceil(N / 64) words
// per row) to FP32 0/1 rows; one thread writes four consecutive entries.
__global__ void expand_bits_kernel(const unsigned long long* __restrict__ bits, int64_t rows,
                                   int32_t N, float4* out) {
  const int32_t W = (N + 63) / 64, n4 = N / 4;
  const int64_t total = rows * n4;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / n4;
    const int32_t j = (int32_t)(i % n4) * 4;
    const unsigned long long w = __ldg(bits + r * W + (j >> 6));
    const uint32_t b = (uint32_t)(w >> (j & 63)) & 15u;
    out[i] = make_float4(b & 1u ? 1.f : 0.f, b & 2u ? 1.f : 0.f, b & 4u ? 1.f : 0.f,
                         b & 8u ? 1.f : 0.f);
  }
}

void launch_expand_bits(const uint64_t* bits, int64_t rows, int32_t N, float* out, cudaStream_t s) {
  expand_bits_kernel<<<4096, 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(bits), rows,
                                          N, reinterpret_cast<float4*>(out));
}

}  // namespace sdnn

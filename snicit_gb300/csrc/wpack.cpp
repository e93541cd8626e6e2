// Weight packing: COO -> CSR (reference semantics) -> bank-scheduled slots.
//
// For each group of 32 output neurons and each input chunk, the group's
// in-edges form a bipartite multigraph between lanes (output within the
// group) and shared-memory banks (input index mod 32).  A proper edge
// colouring of that graph is a slot schedule in which every slot touches 32
// distinct banks (and each lane at most once), so the gather in the layer
// kernel never has a bank conflict.  König's theorem bounds the optimum by the
// maximum degree; greedy first-fit colouring (each edge takes the lowest slot
// free at its lane and its bank) stays within a few slots of it.
#include "wpack.h"

#include <algorithm>
#include <numeric>

namespace sdnn {

bool coo_to_host_layer(int32_t N, const int32_t* rows, const int32_t* cols, const float* vals,
                       int64_t nnz, HostLayer& out, std::string& err) {
  for (int64_t k = 0; k < nnz; ++k) {
    if (rows[k] < 0 || rows[k] >= N || cols[k] < 0 || cols[k] >= N) {
      err = "weight index out of range at entry " + std::to_string(k);
      return false;
    }
  }
  std::vector<int64_t> order(nnz);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return rows[a] != rows[b] ? rows[a] < rows[b] : cols[a] < cols[b];
  });
  out.row_off.assign(N + 1, 0);
  out.cols.clear();
  out.vals.clear();
  out.cols.reserve(nnz);
  out.vals.reserve(nnz);
  int32_t prev_r = -1, prev_c = -1;
  for (int64_t k : order) {
    const int32_t r = rows[k], c = cols[k];
    if (r == prev_r && c == prev_c) {
      out.vals.back() += vals[k];
    } else {
      out.cols.push_back(c);
      out.vals.push_back(vals[k]);
      out.row_off[r + 1]++;
      prev_r = r;
      prev_c = c;
    }
  }
  for (int32_t j = 0; j < N; ++j) out.row_off[j + 1] += out.row_off[j];
  out.present = true;
  return true;
}

namespace {

// Bitset of slot indices, grown on demand.
struct SlotSet {
  std::vector<uint64_t> w;
  void set(int s) {
    if ((size_t)(s >> 6) >= w.size()) w.resize((s >> 6) + 1, 0);
    w[s >> 6] |= 1ull << (s & 63);
  }
  uint64_t word(size_t i) const { return i < w.size() ? w[i] : 0; }
  void clear() { std::fill(w.begin(), w.end(), 0); }
};

}  // namespace

bool pack_layer(const HostLayer& h, int32_t N, int32_t Q, int32_t scale, PackedLayer& out) {
  if (Q <= 0 || Q % 32 != 0 || N % Q != 0 || (scale != 1 && scale != 4)) return false;
  if ((int64_t)(Q + 31) * scale > 65535) return false;
  const int32_t G = N / 32, nq = N / Q;
  // CSC: in-edges of every output, inputs ascending.
  std::vector<int32_t> indeg(N + 1, 0);
  for (int32_t c : h.cols) indeg[c + 1]++;
  for (int32_t c = 0; c < N; ++c) indeg[c + 1] += indeg[c];
  std::vector<int32_t> cin(h.cols.size());
  std::vector<float> cval(h.cols.size());
  {
    std::vector<int32_t> fill(indeg.begin(), indeg.end() - 1);
    for (int32_t j = 0; j < N; ++j)
      for (int32_t k = h.row_off[j]; k < h.row_off[j + 1]; ++k) {
        const int32_t p = fill[h.cols[k]]++;
        cin[p] = j;
        cval[p] = h.vals[k];
      }
  }
  out.nnz = (int64_t)h.cols.size();
  out.constw = !h.vals.empty();
  out.wconst = h.vals.empty() ? 0.f : h.vals[0];
  for (float v : h.vals)
    if (v != out.wconst) {
      out.constw = false;
      break;
    }
  out.grp_blk.assign((size_t)G * nq + 1, 0);
  out.idx.clear();
  out.val.clear();
  out.max_depth = 0;
  out.slots = 0;

  SlotSet lane_used[32], bank_used[32];
  struct Edge {
    int32_t lane, jl;
    float w;
    int32_t slot;
  };
  std::vector<Edge> edges;
  std::vector<int32_t> slot_lane_edge;  // [slot][lane] -> edge index or -1
  int64_t blk = 0;
  for (int32_t g = 0; g < G; ++g) {
    // per-lane cursor into the CSC list (inputs ascending, so chunks are contiguous)
    int32_t cur[32];
    for (int l = 0; l < 32; ++l) cur[l] = indeg[32 * g + l];
    for (int32_t q = 0; q < nq; ++q) {
      out.grp_blk[(size_t)g * nq + q] = (int32_t)blk;
      const int32_t lo = q * Q, hi = lo + Q;
      edges.clear();
      for (int l = 0; l < 32; ++l) {
        const int32_t c = 32 * g + l;
        while (cur[l] < indeg[c + 1] && cin[cur[l]] < hi) {
          const int32_t j = cin[cur[l]];
          edges.push_back({l, j - lo, cval[cur[l]], -1});
          ++cur[l];
        }
      }
      for (int l = 0; l < 32; ++l) {
        lane_used[l].clear();
        bank_used[l].clear();
      }
      int32_t depth = 0;
      for (Edge& e : edges) {
        const int bank = e.jl & 31;
        int s = -1;
        for (size_t wi = 0;; ++wi) {
          const uint64_t m = lane_used[e.lane].word(wi) | bank_used[bank].word(wi);
          if (m != ~0ull) {
            s = (int)(wi * 64 + __builtin_ctzll(~m));
            break;
          }
        }
        e.slot = s;
        lane_used[e.lane].set(s);
        bank_used[bank].set(s);
        depth = std::max(depth, s + 1);
      }
      out.max_depth = std::max(out.max_depth, depth);
      out.slots += depth;
      const int32_t nblk = (depth + 3) / 4;
      const int32_t D = nblk * 4;
      slot_lane_edge.assign((size_t)D * 32, -1);
      for (size_t k = 0; k < edges.size(); ++k)
        slot_lane_edge[(size_t)edges[k].slot * 32 + edges[k].lane] = (int32_t)k;
      const size_t base = out.idx.size();
      out.idx.resize(base + (size_t)nblk * 128);
      if (!out.constw) out.val.resize(base + (size_t)nblk * 128, 0.f);
      for (int32_t s = 0; s < D; ++s) {
        uint32_t banks_used = 0;
        for (int l = 0; l < 32; ++l) {
          const int32_t k = slot_lane_edge[(size_t)s * 32 + l];
          if (k >= 0) banks_used |= 1u << (edges[k].jl & 31);
        }
        uint32_t free_banks = ~banks_used;
        const int32_t b = s >> 2, si = s & 3;
        for (int l = 0; l < 32; ++l) {
          const int32_t k = slot_lane_edge[(size_t)s * 32 + l];
          const size_t at = base + (size_t)b * 128 + (size_t)l * 4 + si;
          if (k >= 0) {
            out.idx[at] = (uint16_t)(edges[k].jl * scale);
            if (!out.constw) out.val[at] = edges[k].w;
          } else {
            const int fb = __builtin_ctz(free_banks);
            free_banks &= free_banks - 1;
            out.idx[at] = (uint16_t)((Q + fb) * scale);  // zero column in the bank left free
            if (!out.constw) out.val[at] = 0.f;
          }
        }
      }
      blk += nblk;
    }
  }
  out.grp_blk[(size_t)G * nq] = (int32_t)blk;
  out.nblocks = blk;
  return true;
}

}  // namespace sdnn

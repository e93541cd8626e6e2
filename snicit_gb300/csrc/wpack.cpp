// Weight packing: COO -> CSR (reference semantics) -> bank-scheduled slots.
//
// For each group of 32 output neurons and each input chunk, the group's
// in-edges form a bipartite multigraph between lanes (output within the
// group) and shared-memory banks (input index mod 32).  A proper edge
// colouring of that graph is a slot schedule in which every slot touches 32
// distinct banks (and each lane at most once), so the gather in the layer
// kernel never has a bank conflict.  By König's theorem the maximum degree
// (largest lane in-degree or bank load) colours suffice; EdgeColoring reaches
// that bound with alternating-path (Kempe chain) recolouring.
#include "wpack.h"

#include <algorithm>
#include <array>
#include <climits>
#include <cstdint>
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

// Proper edge colouring of a bipartite multigraph with exactly Delta colours
// (Delta = maximum vertex degree), by Kempe-chain recolouring: an edge (u, v)
// takes a colour a free at u; if a is taken at v, the a/b alternating path
// from v (b free at v) is flipped first, which frees a at v and, the graph
// being bipartite, cannot reach u.  Vertices 0..31 are lanes, 32..63 banks.
class EdgeColoring {
 public:
  explicit EdgeColoring(int max_colors) : C_(max_colors), at_(64 * (size_t)max_colors, -1) {}
  void reset(int max_colors) {
    C_ = max_colors;
    at_.assign(64 * (size_t)C_, -1);
    colour_.clear();
    ends_.clear();
  }
  // returns the colour of the new edge
  int add(int lane, int bank) {
    const int u = lane, v = 32 + bank;
    const int e = (int)colour_.size();
    colour_.push_back(-1);
    ends_.push_back({u, v});
    const int a = first_free(u), b = first_free(v);
    int c;
    if (is_free(v, a)) {
      c = a;
    } else if (is_free(u, b)) {
      c = b;
    } else {
      flip(v, a, b);
      c = a;
    }
    set(e, c);
    return c;
  }
  int colour(int e) const { return colour_[e]; }

 private:
  int& slot(int vertex, int c) { return at_[(size_t)vertex * C_ + c]; }
  bool is_free(int vertex, int c) { return slot(vertex, c) < 0; }
  int first_free(int vertex) {
    for (int c = 0; c < C_; ++c)
      if (slot(vertex, c) < 0) return c;
    return -1;  // cannot happen: degree <= C_
  }
  void set(int e, int c) {
    colour_[e] = c;
    slot(ends_[e][0], c) = e;
    slot(ends_[e][1], c) = e;
  }
  // swaps colours a and b on the alternating path that starts at w with colour a
  void flip(int w, int a, int b) {
    path_.clear();
    int col = a;
    for (;;) {
      const int e = slot(w, col);
      if (e < 0) break;
      path_.push_back(e);
      w = ends_[e][0] == w ? ends_[e][1] : ends_[e][0];
      col = col == a ? b : a;
    }
    for (int e : path_) {
      slot(ends_[e][0], colour_[e]) = -1;
      slot(ends_[e][1], colour_[e]) = -1;
    }
    for (int e : path_) set(e, colour_[e] == a ? b : a);
  }
  int C_;
  std::vector<int> at_;  // [vertex][colour] -> edge or -1
  std::vector<int> colour_;
  std::vector<std::array<int, 2>> ends_;
  std::vector<int> path_;
};

}  // namespace

bool pack_layer_placed(const HostLayer& hin, int32_t N, int32_t Q, int32_t scale,
                       const int32_t* in_pos, const int32_t* out_pos, PackedLayer& out) {
  if (!in_pos && !out_pos) return pack_layer(hin, N, Q, scale, out);
  // relabel rows (inputs) and columns (outputs), keep per-row column order sorted
  HostLayer h;
  h.row_off.assign(N + 1, 0);
  for (int32_t j = 0; j < N; ++j) {
    const int32_t pj = in_pos ? in_pos[j] : j;
    h.row_off[pj + 1] = hin.row_off[j + 1] - hin.row_off[j];
  }
  for (int32_t j = 0; j < N; ++j) h.row_off[j + 1] += h.row_off[j];
  h.cols.resize(hin.cols.size());
  h.vals.resize(hin.vals.size());
  std::vector<std::pair<int32_t, float>> tmp;
  for (int32_t j = 0; j < N; ++j) {
    const int32_t pj = in_pos ? in_pos[j] : j;
    tmp.clear();
    for (int32_t k = hin.row_off[j]; k < hin.row_off[j + 1]; ++k)
      tmp.push_back({out_pos ? out_pos[hin.cols[k]] : hin.cols[k], hin.vals[k]});
    std::sort(tmp.begin(), tmp.end(),
              [](const std::pair<int32_t, float>& a, const std::pair<int32_t, float>& b) {
                return a.first < b.first;
              });
    for (size_t k = 0; k < tmp.size(); ++k) {
      h.cols[h.row_off[pj] + k] = tmp[k].first;
      h.vals[h.row_off[pj] + k] = tmp[k].second;
    }
  }
  h.present = true;
  return pack_layer(h, N, Q, scale, out);
}

std::vector<int32_t> degree_order(const HostLayer& h, int32_t N) {
  std::vector<int32_t> deg(N, 0), order(N);
  for (int32_t c : h.cols) deg[c]++;
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
  return order;
}

std::vector<int32_t> place_outputs(const std::vector<int32_t>& order, const HostLayer* next,
                                   const std::vector<int32_t>* next_order, int32_t N) {
  std::vector<int32_t> pos(N);
  const int32_t G = N / 32;
  if (!next || !next_order) {
    for (int32_t i = 0; i < N; ++i) pos[order[i]] = i;
    return pos;
  }
  std::vector<int32_t> gnext(N);
  for (int32_t i = 0; i < N; ++i) gnext[(*next_order)[i]] = i / 32;
  std::vector<int32_t> load((size_t)G * 32, 0);
  std::vector<int32_t> nodes(32);
  for (int32_t g = 0; g < G; ++g) {
    for (int i = 0; i < 32; ++i) nodes[i] = order[32 * g + i];
    // neurons with more out-edges first; each takes the free bank that adds the
    // least squared load to the next-layer groups it feeds
    std::stable_sort(nodes.begin(), nodes.end(), [&](int32_t a, int32_t b) {
      return next->row_off[a + 1] - next->row_off[a] > next->row_off[b + 1] - next->row_off[b];
    });
    uint32_t used = 0;
    for (int32_t n : nodes) {
      int best = -1;
      int64_t best_cost = INT64_MAX;
      for (int b = 0; b < 32; ++b) {
        if (used & (1u << b)) continue;
        int64_t cost = 0;
        for (int32_t k = next->row_off[n]; k < next->row_off[n + 1]; ++k) {
          const int64_t ld = load[(size_t)gnext[next->cols[k]] * 32 + b];
          cost += 2 * ld + 1;
        }
        if (cost < best_cost) {
          best_cost = cost;
          best = b;
        }
      }
      used |= 1u << best;
      pos[n] = 32 * g + best;
      for (int32_t k = next->row_off[n]; k < next->row_off[n + 1]; ++k)
        load[(size_t)gnext[next->cols[k]] * 32 + best]++;
    }
  }
  return pos;
}

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

  EdgeColoring coloring(64);
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
      // Delta = max(lane degree, bank load): the colouring uses exactly that many slots
      int lane_deg[32] = {0}, bank_load[32] = {0};
      for (const Edge& e : edges) {
        lane_deg[e.lane]++;
        bank_load[e.jl & 31]++;
      }
      int delta = 0;
      for (int i = 0; i < 32; ++i) delta = std::max({delta, lane_deg[i], bank_load[i]});
      coloring.reset(std::max(delta, 1));
      int32_t depth = 0;
      for (Edge& e : edges) {
        coloring.add(e.lane, e.jl & 31);
      }
      for (size_t k = 0; k < edges.size(); ++k) {
        edges[k].slot = coloring.colour((int)k);
        depth = std::max(depth, edges[k].slot + 1);
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


// ---- neuron placement for input-chunked layouts ---------------------------
//
// With input chunks a slot list belongs to one (group, chunk): it is as deep
// as the busiest lane (an output's in-edges from that chunk) or bank (the
// group's in-edges from that chunk landing in one bank).  Three steps spread
// both, each a pure function of the layers (so they run for all layers at
// once): which chunk a neuron sits in, which outputs share a group, and each
// neuron's lane inside its group.

namespace {
uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
}  // namespace

std::vector<uint8_t> chunk_assign(const HostLayer* next, int32_t N, int32_t Q, uint64_t seed) {
  const int32_t nq = N / Q;
  std::vector<uint8_t> chunk(N);
  if (!next) {
    for (int32_t n = 0; n < N; ++n) chunk[n] = (uint8_t)(n / Q);
    return chunk;
  }
  // neurons in a seeded order (Fisher-Yates on a SplitMix64 stream); each goes
  // to the chunk with room that adds the least squared count to the (output of
  // the next layer, chunk) pairs it feeds
  std::vector<int32_t> order(N);
  std::iota(order.begin(), order.end(), 0);
  for (int32_t i = N - 1; i > 0; --i) {
    const uint64_t r = mix64(seed + (uint64_t)i * 0x9E3779B97F4A7C15ull);
    std::swap(order[i], order[(int32_t)(r % (uint64_t)(i + 1))]);
  }
  std::vector<int32_t> cnt((size_t)N * nq, 0), room(nq, Q);
  for (int32_t n : order) {
    int best = -1;
    int64_t best_cost = INT64_MAX;
    for (int q = 0; q < nq; ++q) {
      if (!room[q]) continue;
      int64_t cost = 0;
      for (int32_t k = next->row_off[n]; k < next->row_off[n + 1]; ++k)
        cost += 2 * cnt[(size_t)next->cols[k] * nq + q] + 1;
      if (cost < best_cost) {
        best_cost = cost;
        best = q;
      }
    }
    chunk[n] = (uint8_t)best;
    room[best]--;
    for (int32_t k = next->row_off[n]; k < next->row_off[n + 1]; ++k)
      cnt[(size_t)next->cols[k] * nq + best]++;
  }
  return chunk;
}

std::vector<int32_t> chunk_group_order(const HostLayer& h, const uint8_t* in_chunk,
                                       const std::vector<uint8_t>& out_chunk, int32_t N,
                                       int32_t Q) {
  const int32_t nq = N / Q;
  // in-degree of every output per input chunk
  std::vector<int32_t> deg((size_t)N * nq, 0);
  for (int32_t j = 0; j < N; ++j) {
    const int q = in_chunk ? in_chunk[j] : j / Q;
    for (int32_t k = h.row_off[j]; k < h.row_off[j + 1]; ++k) deg[(size_t)h.cols[k] * nq + q]++;
  }
  auto key = [&](int32_t n) {
    int32_t mx = 0, sum = 0;
    for (int q = 0; q < nq; ++q) {
      mx = std::max(mx, deg[(size_t)n * nq + q]);
      sum += deg[(size_t)n * nq + q];
    }
    return std::make_pair(mx, sum);
  };
  std::vector<int32_t> order;
  order.reserve(N);
  for (int q = 0; q < nq; ++q) {
    std::vector<int32_t> in_q;
    for (int32_t n = 0; n < N; ++n)
      if (out_chunk[n] == q) in_q.push_back(n);
    // outputs of similar per-chunk depth share a group: largest chunk degree,
    // then total in-degree, descending
    std::stable_sort(in_q.begin(), in_q.end(), [&](int32_t a, int32_t b) { return key(a) > key(b); });
    order.insert(order.end(), in_q.begin(), in_q.end());
  }
  return order;
}

std::vector<int32_t> place_outputs_chunked(const std::vector<int32_t>& order,
                                           const std::vector<uint8_t>& out_chunk,
                                           const HostLayer* next,
                                           const std::vector<int32_t>* next_order, int32_t N,
                                           int32_t Q) {
  std::vector<int32_t> pos(N);
  const int32_t G = N / 32, nq = N / Q;
  if (!next || !next_order) {
    for (int32_t i = 0; i < N; ++i) pos[order[i]] = i;
    return pos;
  }
  std::vector<int32_t> gnext(N);
  for (int32_t i = 0; i < N; ++i) gnext[(*next_order)[i]] = i / 32;
  // bank loads of the next layer per (group, chunk, bank); the cost of a load
  // grows as 4^load so the greedy keeps the largest load of a list down
  std::vector<int32_t> load((size_t)G * nq * 32, 0);
  auto weight = [](int32_t x) -> int64_t { return (int64_t)1 << (2 * std::min(x, 28)); };
  std::vector<int32_t> nodes(32);
  for (int32_t g = 0; g < G; ++g) {
    for (int i = 0; i < 32; ++i) nodes[i] = order[32 * g + i];
    std::stable_sort(nodes.begin(), nodes.end(), [&](int32_t a, int32_t b) {
      return next->row_off[a + 1] - next->row_off[a] > next->row_off[b + 1] - next->row_off[b];
    });
    uint32_t used = 0;
    for (int32_t n : nodes) {
      const size_t q = out_chunk[n];
      int best = -1;
      int64_t best_cost = INT64_MAX;
      for (int b = 0; b < 32; ++b) {
        if (used & (1u << b)) continue;
        int64_t cost = 0;
        for (int32_t k = next->row_off[n]; k < next->row_off[n + 1]; ++k)
          cost += weight(load[((size_t)gnext[next->cols[k]] * nq + q) * 32 + b]);
        if (cost < best_cost) {
          best_cost = cost;
          best = b;
        }
      }
      used |= 1u << best;
      pos[n] = 32 * g + best;
      for (int32_t k = next->row_off[n]; k < next->row_off[n + 1]; ++k)
        load[((size_t)gnext[next->cols[k]] * nq + q) * 32 + best]++;
    }
  }
  return pos;
}

}  // namespace sdnn

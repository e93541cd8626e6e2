// Host-side weight storage and the bank-scheduled packer.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace sdnn {

// One layer as CSR by input row (row = input neuron j, col = output neuron c),
// duplicates summed in input order, columns ascending within a row.  This is
// the content of the reference's packed per-layer CSR
// (tsv_string_to_CSR_packed_array, src/SDGC/utility.hpp:85-126) without the
// N_SLAB section folding.
struct HostLayer {
  std::vector<int32_t> row_off;  // N + 1
  std::vector<int32_t> cols;
  std::vector<float> vals;
  bool present = false;
};

// Builds a HostLayer from COO triplets (0-based); duplicates are summed in
// the order given.  Returns false on out-of-range indices.
bool coo_to_host_layer(int32_t N, const int32_t* rows, const int32_t* cols, const float* vals,
                       int64_t nnz, HostLayer& out, std::string& err);

// Packed layer (see LayerDev in sdnn_internal.h).
struct PackedLayer {
  std::vector<uint16_t> idx;     // nblocks * 32 * 4
  std::vector<float> val;        // nblocks * 32 * 4 (empty when constw)
  std::vector<int32_t> grp_blk;  // G*nq + 1
  bool constw = true;
  float wconst = 0.f;
  int64_t nblocks = 0;
  int64_t nnz = 0;
  int32_t max_depth = 0;         // deepest slot list of a (group, chunk)
  int64_t slots = 0;             // total slots (sum of depths)
};

// Packs one layer for chunk size Q (N % Q == 0, Q % 32 == 0); slot indices are
// stored as (chunk-local index) * scale, scale 4 = byte offsets, 1 = floats;
// returns false when (Q + 32) * scale does not fit 16 bits or Q is invalid.
bool pack_layer(const HostLayer& h, int32_t N, int32_t Q, int32_t scale, PackedLayer& out);

// Same, with neurons placed at positions: input j of the layer is read from
// position in_pos[j] of the incoming row and output c is written to position
// out_pos[c] (nullptr = identity).
bool pack_layer_placed(const HostLayer& h, int32_t N, int32_t Q, int32_t scale,
                       const int32_t* in_pos, const int32_t* out_pos, PackedLayer& out);

// Output grouping of a layer: outputs sorted by in-degree (descending, ties by
// index); group g of the packed layout is order[32g .. 32g+31].
std::vector<int32_t> degree_order(const HostLayer& h, int32_t N);

// Positions of the outputs of a layer (whose grouping is `order`): each group
// keeps its 32 outputs, and their lanes (= shared-memory banks in the next
// layer) are chosen greedily so that every group of the next layer (grouping
// next_order, weights next) sees balanced bank loads.  next == nullptr gives
// lanes in order.
std::vector<int32_t> place_outputs(const std::vector<int32_t>& order, const HostLayer* next,
                                   const std::vector<int32_t>* next_order, int32_t N);


// Placement for input-chunked layouts (chunks of Q inputs):
//  chunk_assign: the chunk of every output neuron of a layer (Q per chunk),
//    balancing the in-edges of every output of the next layer over the chunks
//    (next == nullptr: neuron n in chunk n / Q); seeded, deterministic;
//  chunk_group_order: the layer's output groups -- chunk by chunk, outputs of
//    similar per-input-chunk in-degree together (in_chunk: chunk of each input,
//    nullptr = j / Q); group g is order[32g .. 32g+31], inside chunk 32g / Q;
//  place_outputs_chunked: each output's lane in its group, balancing the next
//    layer's (group, chunk, bank) loads.
std::vector<uint8_t> chunk_assign(const HostLayer* next, int32_t N, int32_t Q, uint64_t seed);
std::vector<int32_t> chunk_group_order(const HostLayer& h, const uint8_t* in_chunk,
                                       const std::vector<uint8_t>& out_chunk, int32_t N,
                                       int32_t Q);
std::vector<int32_t> place_outputs_chunked(const std::vector<int32_t>& order,
                                           const std::vector<uint8_t>& out_chunk,
                                           const HostLayer* next,
                                           const std::vector<int32_t>* next_order, int32_t N,
                                           int32_t Q);

}  // namespace sdnn

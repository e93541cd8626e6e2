// Internal declarations shared by the kernel translation units and the engine.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sdnn {

// Epilogue variants of the layer kernel.
//  PLAIN     y = clamp(acc + b)                       (bf_inference, src/SDGC/BF/kernel.hpp:76-85)
//  CENTROID  pre = acc + b stored; y = clamp(pre)     (post_minus centroid branch,
//                                                      src/SDGC/SNICIT/kernel.hpp:114-120)
//  RESIDUE   y = clamp(pre_c + acc) - clamp(pre_c)    (post_minus residue branch,
//                                                      src/SDGC/SNICIT/kernel.hpp:121-135)
enum Epilogue : int32_t { EPI_PLAIN = 0, EPI_CENTROID = 1, EPI_RESIDUE = 2 };

// Device error codes written to the engine's error word (0 = ok).
enum DevError : int32_t { DEV_OK = 0, DEV_TIMEOUT = 7, DEV_BAD_ROW = 1 };

// Bank-scheduled layer layout.  Outputs are taken in groups of 32 (lane i of
// the group computes output 32*g + i).  For every (group, input chunk) the
// in-edges are arranged in "slots": one edge per lane per slot, and the 32
// input indices of a slot fall in 32 distinct shared-memory banks.  Slots are
// stored in blocks of 4: block b holds, for each lane, 4 consecutive uint16
// chunk-local indices (one uint2) and, unless the layer has one common value,
// 4 floats (one float4).  Empty lanes point at a zero column (chunk + bank).
struct LayerDev {
  const uint2* idx;        // [blocks][32] uint2 (4 x u16)
  const float4* val;       // [blocks][32] float4, nullptr when const_w
  const int32_t* grp_blk;  // [G*nq + 1] block offsets, entry g*nq + q
  const float* bias_vec;   // [N] per-neuron bias or nullptr
  float bias;              // scalar bias when bias_vec == nullptr
  float wconst;            // common value when val == nullptr
};

struct LayerArgs {
  LayerDev w;
  const float* y_in;        // [rows][N]
  float* y_out;             // [rows][N]
  const int32_t* list_in;   // row ids to process
  const int32_t* count_in;  // number of ids (device scalar)
  int32_t* list_out;        // surviving ids (PLAIN) / non-empty residues (RESIDUE)
  int32_t* count_out;       // device scalar, must start at 0
  uint32_t* tile_mask;      // scratch per tile, zero between launches
  int32_t* tile_ticket;     // scratch per tile, zero between launches
  float* pre_out;           // CENTROID: [K][N] pre-activations
  const float* pre_in;      // RESIDUE:  [K][N] pre-activations of this layer
  const int32_t* cslot;     // row -> centroid slot
  int32_t* err;             // device error word
  int32_t N, nq, Q, G;
  int32_t epi;
  int32_t max_split;        // upper bound of CTAs sharing one tile
  int32_t min_split;        // lower bound (register capacity of chunked kernels)
  float clampv;
};

// Chunk sizes whose packed slot indices are byte offsets into the shared row
// (u16 holds (chunk + 32) * 4 only for chunks up to 16351 floats); the kernel
// instances with row stride chunk + 32 of these chunk sizes read them as such.
__host__ __device__ inline bool slot_index_in_bytes(int Q) { return Q == 1024 || Q == 4096; }
__host__ __device__ constexpr bool rsw_in_bytes(int rsw) { return rsw == 1056 || rsw == 4128; }

// Kernel instance selection.
struct LayerKernelKey {
  int T;       // rows per tile
  int rsw;     // compile-time smem row stride in floats (0 = runtime)
  int kg;      // groups per warp held across chunks (1 = no chunking)
  bool constw;
};

// Launches the layer kernel instance matching key; returns cudaErrorInvalidValue
// if no instance exists.  grid/threads/smem chosen by the caller.
cudaError_t launch_layer(const LayerKernelKey& key, const LayerArgs& a, int grid, int threads,
                         size_t smem, cudaStream_t s);
// Occupancy query for an instance (blocks per SM), 0 if not available.
int layer_blocks_per_sm(const LayerKernelKey& key, int threads, size_t smem);
// True if an instance exists.
bool layer_instance_exists(const LayerKernelKey& key);
// Sets the max dynamic shared memory attribute of an instance.
cudaError_t layer_prepare(const LayerKernelKey& key, size_t smem);

// First layer over binary inputs (layer0_bits.cu).
struct Layer0Args {
  const uint2* idx;          // packed slots of layer 0 (same layout as LayerDev)
  const int32_t* grp_blk;    // [G + 1]
  const float* bias_vec;     // [N] or nullptr
  float bias, clampv;
  const float* sums;         // [128]: w added k times in FP32, k = 0..127
  const float* y_in;
  float* y_out;
  const int32_t* list_in;
  const int32_t* count_in;
  int32_t* list_out;
  int32_t* count_out;
  int32_t* fallback_list;    // rows of tiles with non-binary inputs
  int32_t* fallback_count;
  int32_t N, G;
  // input chunks (N > 16384): bit words staged in global memory per tile
  int32_t nq, Q;
  uint32_t* bits;            // [tiles][N] words (bit t = input of row t of the tile)
  int32_t* tile_state;       // [tiles]: 1 = tile holds non-binary values
  uint32_t* tile_mask;       // scratch per tile, zero between launches
  int32_t* tile_ticket;      // scratch per tile, zero between launches
  int32_t* err;              // device error word (bounded waits)
};
bool layer0_bits_supported(int N);
int layer0_bits_grid(int N, int num_sms, int threads);
cudaError_t launch_layer0_bits(const Layer0Args& a, int grid, int threads, cudaStream_t s);
// Chunked variant (nq > 1, chunks of Q = 16384): a transpose pass writes each
// 32-row tile's bit words to `bits`, then the counting pass keeps bit-sliced
// counters of a subset of groups in registers across the chunks.
bool layer0_bits_chunked_supported(int N, int Q);
cudaError_t launch_layer0_bits_chunked(const Layer0Args& a, int num_sms, cudaStream_t s);

// Post-threshold layers with no residue rows left (post_chain.cu): one
// cluster carries the K centroid rows through layers [first, last).
struct ChainArgs {
  const LayerDev* layers;    // [L] device table
  int32_t first, last;
  const float* y_in;         // activations at the threshold
  float* y_out;              // final buffer (centroid rows written after `last`)
  const int32_t* clist;
  const int32_t* ccount;
  int32_t N, G;
  float clampv;
  int32_t* err;              // device error word (bounded waits)
  bool stream;               // weights may be streamed into shared memory
  uint32_t wcap8, wcap16;    // largest per-CTA weight slice, clusters of 8 / 16 CTAs
  uint32_t wcap;             // (set by launch_chain) bytes of one streamed weight buffer
};
// Bytes of the largest per-CTA weight slice of a layer when `cluster` CTAs
// split its groups (grp_blk: G + 1 block offsets; general = per-edge values).
uint32_t chain_slice_bytes(const int32_t* grp_blk, int G, bool general, int cluster);
int chain_capacity(int N);  // largest centroid count the chain kernel takes (0 = none)
// The chain launch for a centroid count: variant 0 none, 1 weights read from
// L2, 2 weights streamed into shared memory (cluster size, weight buffers).
struct ChainPlan {
  int variant, kc, cluster, nwbuf, threads;
  uint32_t wcap;
  size_t smem;
};
ChainPlan chain_plan(const ChainArgs& a, int kc_needed);
cudaError_t launch_chain(const ChainArgs& a, int kc_needed, cudaStream_t s);

// The same for any width, as one cooperative launch over the GPU with the
// rows in global scratch (post_grid.cu).
struct GridChainArgs {
  const LayerDev* layers;    // [L] device table
  int32_t first, last;
  const float* y_in;         // activations at the threshold
  float* y_out;              // final buffer
  const int32_t* clist;
  const int32_t* ccount;
  int32_t N, G, nq, Q;
  float clampv;
  float* scratch;            // [layers + 1][8][nq][Q + 32]: one buffer per layer
  unsigned int* barrier;     // grid barrier counter (zeroed by the launch)
  int32_t* err;
};
int grid_chain_capacity();
size_t grid_chain_scratch_floats(int layers, int nq, int Q);
cudaError_t launch_grid_chain(const GridChainArgs& a, int kc_needed, int num_sms, cudaStream_t s);

// ---- auxiliary kernels (aux.cu) ----
void launch_set_scalar(int32_t* p, int32_t v, cudaStream_t s);

// Post-threshold path chosen on the device, inside the inference's graph: a
// one-thread kernel reads what the clustering left and sets the value of the
// graph's SWITCH node -- body 0 the per-layer centroid/residue launches, body
// 1 + 2i the cluster chain kernel and body 2 + 2i the grid chain kernel for
// 2^i centroid rows (i < 4); bodies the engine could not build are absent
// (has_body 0) and never chosen.  The choice is also stored for the stats.
constexpr int kPostBodies = 9;
struct PostChoiceArgs {
  const int32_t* rcount;  // residue rows at the threshold (dense)
  const int32_t* scount;  // ... kept as sparse lists (nullptr: none)
  const int32_t* ccount;  // centroids kept
  int32_t* choice;        // out: the body taken
  int32_t chain_cap, grid_cap, no_chain;
  int32_t has_body[kPostBodies];
};
void launch_post_choice(const PostChoiceArgs& a, cudaGraphConditionalHandle h, cudaStream_t s);
// counts[l] = sum over pieces p of piece_counts[p * stride + l], l < layers
// (row counts of the layers run piece by piece).
void launch_sum_piece_counts(const int32_t* piece_counts, int pieces, int stride, int layers,
                             int32_t* counts, cudaStream_t s);
// list[i] = i, zero_a[i] = zero_b[i] = 0 and neg[i] = -1 for i < *nrows;
// *count = *nrows
void launch_begin_rows(const int32_t* nrows, int32_t* list, int32_t* count, int32_t* zero_a,
                       int32_t* zero_b, int32_t* neg, cudaStream_t s);
void launch_zero_rows(const int32_t* nrows, int32_t* a, int32_t* b, cudaStream_t s);
void launch_copy_rows(const int32_t* nrows, const float* src, float* dst, int32_t N, cudaStream_t s);
void launch_identify(const float* y, const int32_t* list, const int32_t* count, int32_t N,
                     int32_t* flags, cudaStream_t s);
void launch_flags_to_ids(const int32_t* flags, int32_t n, int32_t* ids, int32_t* count,
                         cudaStream_t s);
void launch_mark_rows(const int32_t* list, const int32_t* count, int32_t* flags, int32_t value,
                      cudaStream_t s);

// SNICIT threshold stage.
struct ClusterArgs {
  float* y;                 // [rows][N] activations at the threshold, rewritten to residues
  const int32_t* live;      // live rows at the threshold
  const int32_t* live_count;
  int32_t N;
  int32_t K;                // candidate count
  uint64_t seed;
  int32_t* cand;            // [K] candidate rows (seeded pick)
  int32_t* ncand;
  float* bins;              // [K][16] downsampled sums
  int32_t* clist;           // [K] kept centroid rows
  int32_t* ccount;
  int32_t* cslot;           // [rows] centroid slot of every live row
  int32_t* rlist;           // non-empty residue rows
  int32_t* rcount;
  int32_t* is_centroid;     // [rows] 1 for centroid rows
  int32_t* err;
};
void launch_cluster(const ClusterArgs& a, int num_sms, cudaStream_t s);

// Recovery (SNICIT.hpp:644 recover): flags[r] = any(c + delta > 0) for every
// live row at the threshold; rows absent from the final residue list have
// delta == 0.
void launch_recover(const float* y, const int32_t* live, const int32_t* live_count,
                    const int32_t* cslot, const int32_t* clist, const int32_t* is_centroid,
                    const int32_t* res_flag, int32_t N, int32_t* flags, cudaStream_t s);
// Final activations of every row into out[rows][N]: state 0 = dead (zeros),
// 1 = plain final row, 2 = SNICIT live row (centroid, or centroid + residue).
// perm[c] = position of neuron c in the final buffer (nullptr = identity).
// alias[r] >= 0: row r was merged into row alias[r] (read that row instead).
void launch_materialize(const float* y, const int32_t* state, const int32_t* cslot,
                        const int32_t* clist, const int32_t* is_centroid, const int32_t* res_flag,
                        const int32_t* alias, const int32_t* perm, int32_t N, float* out,
                        int32_t rows, cudaStream_t s);

// Dense output head (logits = recovered final row . H + b) for H in
// {1, 2, 4, 8, 10, 16, 32}; Hp is stored by final position.  False if H is
// not one of those.
bool launch_head(const float* y, const int32_t* state, const int32_t* cslot, const int32_t* clist,
                 const int32_t* is_centroid, const int32_t* res_flag, const int32_t* alias,
                 const float* Hp, const float* hb, int32_t H, int32_t N, int32_t rows,
                 float* logits, int32_t* argmax, cudaStream_t s);

// A bounded wait that nothing completes (selftest.cu): sets DEV_TIMEOUT.
cudaError_t launch_wait_selftest(int32_t* err, uint64_t limit_ns, cudaStream_t s);

// One-bit input rows (ceil(N / 64) words per row, N % 4 == 0) to FP32 rows.
void launch_expand_bits(const uint64_t* bits, int64_t rows, int32_t N, float* out, cudaStream_t s);

// ---- exact merging of identical rows (dedup.cu) ----
struct DedupArgs {
  const float* y;               // [rows][N] activations after the layer
  int32_t* list;                // live rows after the layer; compacted in place
  int32_t* count;               // its count; rewritten
  unsigned long long* table;    // [mask + 1] keys, 0 = empty (all empty between calls)
  int32_t* slot_rep;            // [mask + 1] smallest row per key, 0x7F7F7F7F = empty
  int32_t* pos_slot;            // [rows] table slot of each list position
  int32_t* tmp_list;            // [rows]
  int32_t* tmp_count;           // [2]: kept rows, rows listed before
  int32_t* alias;               // [rows] -1, or the row this row was merged into
  int32_t N;
  uint32_t mask;                // table entries - 1 (a power of 2 >= 2 x rows, minus 1)
};
void launch_dedup(const DedupArgs& a, int num_sms, cudaStream_t s);
// alias[r] := root of r's chain, flags[r] := flags[root] for merged rows.
void launch_resolve_alias(const int32_t* nrows, int32_t* alias, int32_t* flags, int32_t max_depth,
                          cudaStream_t s);


// ---- sparse residue rows (residue_sparse.cu) ----
// A residue row with at most `cap` nonzeros: entries [r * cap, r * cap + cnt[r])
// of idx (positions, ascending) and val.
struct SparseRows {
  int32_t* idx;
  float* val;
  int32_t* cnt;
  int32_t cap;
};
// One post-threshold layer over the sparse residue rows.
struct SparseResArgs {
  const int32_t* list_in;   // sparse rows of this layer
  const int32_t* count_in;
  SparseRows in, out;       // this layer's lists / the next layer's
  float* y_out;             // rows that grow past `cap` are written here densely
  int32_t* dense_list;      // ... and listed here (the next dense residue list)
  int32_t* dense_count;
  int32_t* sparse_list;     // the next sparse residue list
  int32_t* sparse_count;
  const int32_t* tr_off;    // transposed layer: out-edges of every input position
  const uint16_t* tr_out;   // output positions
  const float* tr_val;      // values, nullptr when the layer has one value
  float wconst;
  const float* pre;         // [K][N] centroid pre-activations of this layer (bias in)
  const int32_t* cslot;     // row -> centroid slot
  int32_t N;
  float clampv;
};
size_t sparse_residue_smem_per_warp(int N);
int sparse_residue_warps(int N);  // warps per CTA (0: rows too wide for shared memory)
cudaError_t sparse_residue_prepare(int N);
void launch_split_residue(const float* y, const int32_t* list, const int32_t* count,
                          const SparseRows& out, int32_t* dense_list, int32_t* dense_count,
                          int32_t* sparse_list, int32_t* sparse_count, int32_t N, int num_sms,
                          cudaStream_t s);
cudaError_t launch_sparse_residue(const SparseResArgs& a, int num_sms, cudaStream_t s);
void launch_densify(const int32_t* list, const int32_t* count, const SparseRows& rows, float* y,
                    int32_t N, int num_sms, cudaStream_t s);

}  // namespace sdnn

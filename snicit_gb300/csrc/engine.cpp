// The inference engine behind the C ABI (include/snicit_gb300.h).
//
// One engine = one CUDA stream + device-resident weights + row buffers.
// The layer loop is device-driven: every kernel reads its row count from
// device memory and compacts its survivors on the device, so no host
// synchronisation happens between layers (the reference synchronises and
// compacts on the host every layer, src/SDGC/SNICIT/SNICIT.hpp:548-630,
// src/SDGC/BF/BF.hpp:198-207).  In SNIG, XY and SNICIT modes the whole
// sequence is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "packfile.h"
#include "sdnn_internal.h"
#include "snicit_gb300.h"
#include "wpack.h"

namespace sdnn {
int read_weight_tsv(const std::string& path, int32_t N, HostLayer& out, std::string& err);
int write_weight_tsv(const std::string& path, const HostLayer& h, int32_t N);
void gen_row_cols(uint64_t seed, int32_t layer, int32_t row, int32_t N, int32_t nnz, int32_t* cols);
bool radixnet_shape_ok(int32_t N, int32_t block);
void radixnet_row_cols(int32_t N, int32_t block, int32_t layer, int32_t row, int32_t* cols);
}  // namespace sdnn

using namespace sdnn;

namespace {

struct DevLayer {
  uint2* idx = nullptr;
  float4* val = nullptr;
  int32_t* grp = nullptr;
  float* bias = nullptr;
  float* sums = nullptr;  // layer 0 with one common value: w added k times, k < 128
  // transposed layer for the sparse residue update: out-edges of every input
  // position (output positions, values unless the layer has one value)
  int32_t* tr_off = nullptr;
  uint16_t* tr_out = nullptr;
  float* tr_val = nullptr;
  bool constw = true;
  float wconst = 0.f;
  int64_t nnz = 0;
  int64_t slots = 0;
  int32_t max_depth = 0;
  uint32_t chain_slice8 = 0, chain_slice16 = 0;  // largest per-CTA weight slices (chain)
};

struct GraphKey {
  int64_t rows = -1;
  const float* in = nullptr;
  int32_t* flags = nullptr;
  int T = -1, K = -1, mode = -1, tile = -1, threads = -1, chain_kc = -1, start = -1;
  bool operator==(const GraphKey& o) const {
    return rows == o.rows && in == o.in && flags == o.flags && T == o.T && K == o.K &&
           mode == o.mode && tile == o.tile && threads == o.threads && chain_kc == o.chain_kc &&
           start == o.start;
  }
};

struct GraphSlot {
  cudaGraphExec_t exec = nullptr;
  GraphKey key;
  int launches = 0;
};

// Streamed ingest of host FP32 rows: at most this many copy pieces per call.
// The automatic piece holds about 96 MB of rows (0.45 ms of copy at the
// 211 GB/s host-to-device rate measured on GB300), clamped to 2048 .. 16384
// rows: each piece costs a few microseconds per layer.  Measured optimum:
// about 6000 rows at N = 4096, 16384 rows at N = 1024.
constexpr int kMaxPieces = 16;
constexpr int64_t kDefaultPieceBytes = 96ll << 20;
constexpr int64_t kMinPieceRows = 2048, kMaxPieceRows = 16384;

// One SNICIT inference as one graph: PH_PRE, the device-side choice of the
// post-threshold path (a SWITCH node over kPostBodies bodies), PH_FINISH.
struct FullGraph {
  cudaGraphExec_t exec = nullptr;
  GraphKey key;
  int launches = 0;                    // PH_PRE, the choice kernel, PH_FINISH
  int body_launches[kPostBodies] = {};
  int variant[4] = {};                 // cluster chain variant per 2^i rows (stats)
};

struct GenSpec {
  bool on = false;
  uint64_t seed = 0;
  int32_t nnz = 32;
  float value = 0.0625f;
  int32_t radix_block = 0;  // > 0: RadiX-Net layers with dense blocks of this width
};

}  // namespace

struct sdnn_engine {
  sdnn_config cfg{};
  std::string err;
  int N = 0, L = 0, dev = 0, num_sms = 0;
  cudaStream_t stream = nullptr;

  // host-side weights
  std::vector<HostLayer> hw;
  std::vector<std::vector<float>> hbias;
  GenSpec gen;
  std::shared_ptr<PackedFile> packed;  // weights from a packed-weight file
  bool weights_dirty = true;

  // kernel configuration
  int Q = 0, nq = 1, G = 0;
  LayerKernelKey key{};
  int threads = 512, grid = 0, grid_general = 0, min_split = 1;
  size_t smem = 0;

  // device weights (owned, or borrowed from weights_owner: a server's slot
  // engines read the model engine's copy; share_users counts the borrowers)
  const sdnn_engine* weights_owner = nullptr;
  std::atomic<int> share_users{0};
  std::vector<DevLayer> dl;
  int64_t total_nnz = 0;
  // neuron placement: positions of the outputs of every layer (empty = identity)
  std::vector<std::vector<int32_t>> pos;
  int32_t* d_perm_final = nullptr;  // position of neuron c after the last layer

  // device buffers
  int64_t cap = 0;
  int Kcap = 0;  // rows of the centroid buffers
  float* d_y[2] = {nullptr, nullptr};
  int32_t* d_list[2] = {nullptr, nullptr};
  int32_t* d_rlist[2] = {nullptr, nullptr};
  int32_t* d_counts = nullptr;   // [L + 2]
  int32_t* d_rcounts = nullptr;  // [L + 2]
  uint32_t* d_tmask = nullptr;
  int32_t* d_ticket = nullptr;
  int32_t* d_clist = nullptr;
  int32_t* d_ccount = nullptr;
  int32_t* d_cand = nullptr;
  int32_t* d_ncand = nullptr;
  float* d_bins = nullptr;
  int32_t* d_cslot = nullptr;
  int32_t* d_iscent = nullptr;
  int32_t* d_resflag = nullptr;
  int32_t* d_flags = nullptr;
  int32_t* d_state = nullptr;
  float* d_pre = nullptr;
  int32_t* d_err = nullptr;
  int32_t* d_ids = nullptr;
  int32_t* d_idcount = nullptr;
  float* d_in = nullptr;
  int32_t* d_rows = nullptr;      // row count of the current inference
  int32_t* d_fallback = nullptr;  // layer-0 rows of non-binary tiles
  int32_t* d_fbcount = nullptr;
  uint64_t* d_inbits = nullptr;    // one-bit host inputs, staged before expansion
  int64_t inbits_cap = 0;
  float* d_gscratch = nullptr;     // grid chain: [2][8][nq][Q + 32] centroid rows
  unsigned int* d_gbar = nullptr;  // grid chain barrier counter
  uint32_t* d_bits = nullptr;      // chunked binary first layer: bit words per 32-row tile
  int64_t bits_tile0 = 0;          // first tile of d_bits / d_tile_state the next launch uses
  int32_t* d_tile_state = nullptr;
  // merging of identical rows (SNICIT, below the threshold)
  int32_t* d_alias = nullptr;          // [cap] -1 or the row this row was merged into
  unsigned long long* d_mtable = nullptr;  // [mmask + 1]
  int32_t* d_mrep = nullptr;           // [mmask + 1]
  int32_t* d_mpos = nullptr;           // [cap]
  int32_t* d_mtmp = nullptr;           // [cap]
  int32_t* d_mcount = nullptr;         // [2]
  uint32_t mmask = 0;
  int bits_grid = 0;
  bool bits_chunked = false;

  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};

  // streamed ingest of host FP32 rows: a copy stream, one event per piece and
  // the per-piece row counts of the layers run piece by piece
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t piece_ev[kMaxPieces] = {};
  cudaEvent_t ingest_free = nullptr, lane_ev = nullptr;
  // second lane for odd pieces: its own stream, tile tickets and layer-0
  // fallback list (swapped in with swap_lane), so one piece's layers fill the
  // last partial wave of the other's
  cudaStream_t stream2 = nullptr;
  uint32_t* d_tmask2 = nullptr;
  int32_t* d_ticket2 = nullptr;
  int32_t* d_fallback2 = nullptr;
  int32_t* d_fbcount2 = nullptr;
  int32_t* d_pcounts = nullptr;  // [kMaxPieces][L + 2]
  int32_t* d_plist[2] = {nullptr, nullptr};  // [cap] row lists of the pieces' layers
  // sparse residue rows (SNICIT post layers, whole-row layouts): per post layer
  // p the dense residue rows are d_rlist[p & 1] and the sparse ones
  // d_slist[p & 1] with their entries in d_sp*[p & 1]; d_rtmp collects the
  // non-empty rows of a dense residue launch before they are split
  bool sparse_built = false;  // transposed layers and sparse lists allocated
  bool sparse_res = false;    // ... and used
  int32_t sp_cap = 0;  // entries per sparse row (N / 32, at least 32)
  int32_t* d_sp_idx[2] = {nullptr, nullptr};
  float* d_sp_val[2] = {nullptr, nullptr};
  int32_t* d_sp_cnt[2] = {nullptr, nullptr};
  int32_t* d_slist[2] = {nullptr, nullptr};
  int32_t* d_scounts = nullptr;  // [L + 4]
  int32_t* d_rtmp = nullptr;
  int32_t* d_tcounts = nullptr;  // [L + 4]
  int pipe_start = 0;            // first layer of the graphed part (0: every layer)
  int last_pieces = 0;

  // graph cache: one captured graph per phase of an inference (slots 5 and 6:
  // PH_ALL and PH_PRE starting after the layers run piece by piece)
  GraphSlot graphs[7];
  FullGraph full[2];       // SNICIT whole-inference graphs (pipe_start 0 / > 0)
  bool full_off = false;   // building one failed: the host picks the post path
  bool in_body = false;    // capturing a conditional body (no event records)
  int last_full = 0;       // 1 + slot of the whole-inference graph that ran last, 0: none
  int32_t* d_choice = nullptr;  // body taken by the last whole-inference graph
  int run_launches = 0;
  int32_t* h_counts = nullptr;  // pinned: residue rows and centroids after clustering
  int chain_cap = 0;            // centroid rows the cluster chain kernel can carry
  int chain_kc = 1;
  int chain_kind = 0;           // 1 cluster chain kernel, 2 grid chain kernel
  uint32_t chain_wcap8 = 0, chain_wcap16 = 0;  // chain kernel weight slices (bytes)
  bool last_chain = false;
  int last_post_kernel = 0;     // stats: 0 none, 1 per-layer launches, 2/3 chain kernel 1/2
  LayerDev* d_layer_table = nullptr;  // device copy of every layer's descriptor

  // last run
  int64_t last_rows = 0;
  int last_T = 0;
  int launches = 0;
  bool have_run = false;
  int pending_stats = 0;
  sdnn_stats stats{};
};

namespace {

int fail(sdnn_engine* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  return code;
}
int cuda_fail(sdnn_engine* e, cudaError_t rc, const char* what) {
  return fail(e, SDNN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(rc));
}
#define CK(call)                                             \
  do {                                                       \
    cudaError_t _rc = (call);                                \
    if (_rc != cudaSuccess) return cuda_fail(e, _rc, #call); \
  } while (0)

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

void free_weights(sdnn_engine* e) {
  if (e->weights_owner) {  // borrowed: the owner frees them
    const_cast<sdnn_engine*>(e->weights_owner)->share_users.fetch_sub(1);
    e->dl.clear();
    e->d_perm_final = nullptr;
    e->d_layer_table = nullptr;
    e->weights_owner = nullptr;
    return;
  }
  dfree(e->d_perm_final);
  dfree(e->d_layer_table);
  for (auto& d : e->dl) {
    dfree(d.idx);
    dfree(d.val);
    dfree(d.grp);
    dfree(d.bias);
    dfree(d.sums);
    dfree(d.tr_off);
    dfree(d.tr_out);
    dfree(d.tr_val);
  }
  e->dl.clear();
}

void free_buffers(sdnn_engine* e) {
  dfree(e->d_y[0]);
  dfree(e->d_y[1]);
  dfree(e->d_list[0]);
  dfree(e->d_list[1]);
  dfree(e->d_rlist[0]);
  dfree(e->d_rlist[1]);
  dfree(e->d_counts);
  dfree(e->d_rcounts);
  dfree(e->d_tmask);
  dfree(e->d_ticket);
  dfree(e->d_clist);
  dfree(e->d_ccount);
  dfree(e->d_cand);
  dfree(e->d_ncand);
  dfree(e->d_bins);
  dfree(e->d_cslot);
  dfree(e->d_iscent);
  dfree(e->d_resflag);
  dfree(e->d_flags);
  dfree(e->d_state);
  dfree(e->d_pre);
  dfree(e->d_err);
  dfree(e->d_ids);
  dfree(e->d_idcount);
  dfree(e->d_in);
  dfree(e->d_fallback);
  dfree(e->d_fbcount);
  dfree(e->d_bits);
  dfree(e->d_tile_state);
  dfree(e->d_gscratch);
  dfree(e->d_gbar);
  dfree(e->d_inbits);
  e->inbits_cap = 0;
  dfree(e->d_rows);
  dfree(e->d_alias);
  dfree(e->d_mtable);
  dfree(e->d_mrep);
  dfree(e->d_mpos);
  dfree(e->d_mtmp);
  dfree(e->d_mcount);
  dfree(e->d_pcounts);
  dfree(e->d_choice);
  dfree(e->d_plist[0]);
  dfree(e->d_plist[1]);
  dfree(e->d_tmask2);
  dfree(e->d_ticket2);
  dfree(e->d_fallback2);
  dfree(e->d_fbcount2);
  for (int i = 0; i < 2; ++i) {
    dfree(e->d_sp_idx[i]);
    dfree(e->d_sp_val[i]);
    dfree(e->d_sp_cnt[i]);
    dfree(e->d_slist[i]);
  }
  dfree(e->d_scounts);
  dfree(e->d_rtmp);
  dfree(e->d_tcounts);
  if (e->h_counts) cudaFreeHost(e->h_counts);
  e->h_counts = nullptr;
  e->cap = 0;
}

void drop_graph(sdnn_engine* e) {
  for (auto& g : e->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = GraphSlot{};
  }
  for (auto& g : e->full) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = FullGraph{};
  }
}

constexpr size_t kMaxSmem = 227 * 1024;
// threads per CTA of the binary first-layer kernel: small enough for two or
// three CTAs per SM, so one CTA's row loads overlap another's counting
#ifndef SDNN_BITS_THREADS
#define SDNN_BITS_THREADS 256
#endif
constexpr int kBitsThreads = SDNN_BITS_THREADS;
// first plain layer after which identical rows are merged (SNICIT): rows are
// still distinct in the first layers, where most of them die
constexpr int kMergeStart = 4;

// Chooses chunking, kernel instance, tile rows, threads and grid.
// Input chunking of the weight layout: whole rows up to 32768 neurons, else
// chunks of 16384 (fixed at creation; the packer and the kernel share it).
void choose_layout(sdnn_engine* e) {
  const int N = e->N;
  e->Q = N > 32768 ? 16384 : N;
  e->nq = N / e->Q;
  e->G = N / 32;
  // sparse residue rows need the whole row of one warp in shared memory
  // (the transposed layers and the lists exist whenever the layout allows
  // them, so the autotuner may switch between sparse and dense rows)
  e->sparse_built = e->nq == 1 && sparse_residue_warps(N) > 0;
  e->sparse_res = e->sparse_built && !(e->cfg.flags & SDNN_FLAG_DENSE_RESIDUE);
}

int choose_kernel(sdnn_engine* e) {
  const int N = e->N;
  const int req_T = e->cfg.tile_rows;
  int threads = e->cfg.threads > 0 ? e->cfg.threads : 512;
  if (threads != 256 && threads != 512 && threads != 1024) threads = 512;
  std::vector<LayerKernelKey> cands;
  if (e->nq == 1) {
    int rsw = e->Q == 1024 ? 1056 : e->Q == 4096 ? 4128 : e->Q == 16384 ? 16416 : 0;
    std::vector<int> Ts;
    if (rsw == 1056) Ts = {16, 12, 24, 8};
    else if (rsw == 4128) Ts = {3, 6, 4, 5, 2};
    else if (rsw == 16416) Ts = {3, 2, 1};
    else Ts = {8, 4, 2, 1};
    for (int T : Ts) cands.push_back({T, rsw, 1, true});
    // N = 1024 / 4096 store byte offsets (see slot_index_in_bytes), which only
    // the instances with that compile-time row stride read
    if (rsw == 16416)
      for (int T : {8, 4, 2, 1}) cands.push_back({T, 0, 1, true});
  } else {
    // 16 groups per warp at 512 threads, 8 at 1024 (the same groups per CTA)
    const int kg = threads == 1024 ? 8 : 16;
    if (e->Q == 16384)
      for (int T : {3, 2, 1}) cands.push_back({T, 16416, kg, true});
    cands.push_back({1, 0, 16, true});
  }
  for (const auto& k : cands) {
    if (req_T > 0 && k.T != req_T) continue;
    const size_t smem = (size_t)k.T * (size_t)(e->Q + 32) * 4;
    if (smem > kMaxSmem) continue;
    if (!layer_instance_exists(k)) continue;
    LayerKernelKey kc = k, kg = k;
    kc.constw = true;
    kg.constw = false;
    const int b1 = layer_blocks_per_sm(kc, threads, smem);
    const int b2 = layer_blocks_per_sm(kg, threads, smem);
    if (b1 <= 0 || b2 <= 0) continue;
    e->key = k;
    e->smem = smem;
    e->threads = threads;
    e->grid = e->num_sms * b1;          // layers with one common weight value
    e->grid_general = e->num_sms * b2;  // layers with per-edge values
    const int nwarps = threads / 32;
    e->min_split = k.kg > 1 ? (e->G + nwarps * k.kg - 1) / (nwarps * k.kg) : 1;
    return SDNN_OK;
  }
  return fail(e, SDNN_ERR_UNSUPPORTED,
              "no layer kernel instance fits N=" + std::to_string(N) +
                  (req_T > 0 ? " with tile_rows=" + std::to_string(req_T) : std::string()));
}

int ensure_buffers(sdnn_engine* e, int64_t rows) {
  if (e->cap >= rows && e->cap > 0) return SDNN_OK;
  free_buffers(e);
  drop_graph(e);
  const int64_t cap = std::max<int64_t>(rows, e->cfg.batch);
  const size_t N = (size_t)e->N;
  // centroid buffers sized for the autotuner's largest candidate count too,
  // so switching counts needs no reallocation
  const int K = std::max(std::max(1, e->cfg.num_centroids), 200);
  e->Kcap = K;
  auto A = [&](auto** p, size_t bytes) -> cudaError_t {
    return cudaMalloc((void**)p, std::max<size_t>(bytes, 16));
  };
  cudaError_t rc = cudaSuccess;
  auto T = [&](cudaError_t r) {
    if (rc == cudaSuccess) rc = r;
  };
  T(A(&e->d_y[0], (size_t)cap * N * 4));
  T(A(&e->d_y[1], (size_t)cap * N * 4));
  T(A(&e->d_in, (size_t)cap * N * 4));
  for (int i = 0; i < 2; ++i) {
    T(A(&e->d_list[i], (size_t)cap * 4));
    T(A(&e->d_rlist[i], (size_t)cap * 4));
  }
  T(A(&e->d_counts, (size_t)(e->L + 4) * 4));
  T(A(&e->d_rcounts, (size_t)(e->L + 4) * 4));
  T(A(&e->d_tmask, (size_t)(cap + 1) * 4));
  T(A(&e->d_ticket, (size_t)(cap + 1) * 4));
  T(A(&e->d_clist, (size_t)K * 4));
  T(A(&e->d_ccount, 16));
  T(A(&e->d_cand, (size_t)K * 4));
  T(A(&e->d_ncand, 16));
  T(A(&e->d_bins, (size_t)K * 16 * 4));
  T(A(&e->d_cslot, (size_t)cap * 4));
  T(A(&e->d_iscent, (size_t)cap * 4));
  T(A(&e->d_resflag, (size_t)cap * 4));
  T(A(&e->d_flags, (size_t)cap * 4));
  T(A(&e->d_state, (size_t)cap * 4));
  T(A(&e->d_pre, (size_t)K * N * 4));
  T(A(&e->d_err, 16));
  T(A(&e->d_ids, (size_t)cap * 4));
  T(A(&e->d_idcount, 16));
  T(A(&e->d_fallback, (size_t)cap * 4));
  if (e->sparse_built) {
    // a sparse row's update runs on one warp, entry after entry: rows with
    // more than N / 32 nonzeros stay dense (the gather kernel's throughput)
    e->sp_cap = std::max(32, e->N / 32);
    for (int i = 0; i < 2; ++i) {
      T(A(&e->d_sp_idx[i], (size_t)cap * e->sp_cap * 4));
      T(A(&e->d_sp_val[i], (size_t)cap * e->sp_cap * 4));
      T(A(&e->d_sp_cnt[i], (size_t)cap * 4));
      T(A(&e->d_slist[i], (size_t)cap * 4));
    }
    T(A(&e->d_scounts, (size_t)(e->L + 4) * 4));
    T(A(&e->d_rtmp, (size_t)cap * 4));
    T(A(&e->d_tcounts, (size_t)(e->L + 4) * 4));
  }
  // grid chain rows: a fresh buffer per layer (wide layouts only, where it runs)
  if (e->N >= 16384) T(A(&e->d_gscratch, grid_chain_scratch_floats(e->L, e->nq, e->Q) * 4));
  T(A(&e->d_gbar, 16));
  if (e->nq > 1 && layer0_bits_chunked_supported(e->N, e->Q)) {
    const size_t tiles = (size_t)(cap + 31) / 32;
    T(A(&e->d_bits, tiles * (size_t)N * 4));
    T(A(&e->d_tile_state, tiles * 4));
  }
  {
    uint64_t P = 1024;
    while (P < 2 * (uint64_t)cap) P <<= 1;
    e->mmask = (uint32_t)(P - 1);
    T(A(&e->d_alias, (size_t)cap * 4));
    T(A(&e->d_mtable, (size_t)P * 8));
    T(A(&e->d_mrep, (size_t)P * 4));
    T(A(&e->d_mpos, (size_t)cap * 4));
    T(A(&e->d_mtmp, (size_t)cap * 4));
    T(A(&e->d_mcount, 16));
    if (rc == cudaSuccess) rc = cudaMemset(e->d_mtable, 0, (size_t)P * 8);
    if (rc == cudaSuccess) rc = cudaMemset(e->d_mrep, 0x7F, (size_t)P * 4);
    if (rc == cudaSuccess) rc = cudaMemset(e->d_alias, 0xFF, (size_t)cap * 4);
  }
  T(A(&e->d_fbcount, 16));
  T(A(&e->d_rows, 16));
  T(A(&e->d_pcounts, (size_t)kMaxPieces * (e->L + 2) * 4));
  T(A(&e->d_choice, 16));
  T(A(&e->d_plist[0], (size_t)cap * 4));
  T(A(&e->d_plist[1], (size_t)cap * 4));
  T(A(&e->d_tmask2, (size_t)(cap + 1) * 4));
  T(A(&e->d_ticket2, (size_t)(cap + 1) * 4));
  T(A(&e->d_fallback2, (size_t)cap * 4));
  T(A(&e->d_fbcount2, 16));
  if (rc == cudaSuccess) T(cudaMallocHost((void**)&e->h_counts, 16));
  if (rc != cudaSuccess) {
    free_buffers(e);
    cudaGetLastError();
    return fail(e, SDNN_ERR_OOM, std::string("device allocation failed: ") + cudaGetErrorString(rc));
  }
  e->cap = cap;
  CK(cudaMemsetAsync(e->d_tmask, 0, (size_t)(cap + 1) * 4, e->stream));
  CK(cudaMemsetAsync(e->d_ticket, 0, (size_t)(cap + 1) * 4, e->stream));
  CK(cudaMemsetAsync(e->d_tmask2, 0, (size_t)(cap + 1) * 4, e->stream));
  CK(cudaMemsetAsync(e->d_ticket2, 0, (size_t)(cap + 1) * 4, e->stream));
  CK(cudaMemsetAsync(e->d_err, 0, 16, e->stream));
  return SDNN_OK;
}

// The host CSR of layer l: regenerated for synthetic weights, else stored.
const HostLayer* host_layer(sdnn_engine* e, int l, HostLayer& tmp) {
  if (!e->gen.on) return e->hw[l].present ? &e->hw[l] : nullptr;
  const int N = e->N, k = e->gen.radix_block > 0 ? 2 * e->gen.radix_block : e->gen.nnz;
  tmp.row_off.resize(N + 1);
  tmp.cols.resize((size_t)N * k);
  tmp.vals.assign((size_t)N * k, e->gen.value);
  for (int j = 0; j < N; ++j) {
    tmp.row_off[j] = j * k;
    int32_t* c = tmp.cols.data() + (size_t)j * k;
    if (e->gen.radix_block > 0) {
      radixnet_row_cols(N, e->gen.radix_block, l, j, c);
    } else {
      gen_row_cols(e->gen.seed, l, j, N, k, c);
      std::sort(c, c + k);
    }
  }
  tmp.row_off[N] = N * k;
  tmp.present = true;
  return &tmp;
}

// Packs layer l on the host with the chosen neuron placement (e->pos).
int pack_host_layer(sdnn_engine* e, int l, PackedLayer& p, int32_t& max_in_degree,
                    std::string& err) {
  HostLayer tmp;
  const HostLayer* h = host_layer(e, l, tmp);
  if (!h) {
    err = "layer " + std::to_string(l) + " has no weights";
    return SDNN_ERR_STATE;
  }
  const int32_t* in_pos = (l > 0 && !e->pos.empty()) ? e->pos[l - 1].data() : nullptr;
  const int32_t* out_pos = e->pos.empty() ? nullptr : e->pos[l].data();
  if (!pack_layer_placed(*h, e->N, e->Q, slot_index_in_bytes(e->Q) ? 4 : 1, in_pos, out_pos, p)) {
    err = "bad chunk size for packing";
    return SDNN_ERR_INVALID;
  }
  max_in_degree = 0;  // counts of the binary first layer must fit 7 bits
  if (p.constw) {
    std::vector<int32_t> deg(e->N, 0);
    for (int32_t c : h->cols) max_in_degree = std::max(max_in_degree, ++deg[c]);
  }
  return SDNN_OK;
}

PackedView view_of(const sdnn_engine* e, int l, const PackedLayer& p, int32_t max_in_degree) {
  PackedView v;
  v.grp_blk = p.grp_blk.data();
  v.idx = p.idx.data();
  v.val = p.constw ? nullptr : p.val.data();
  v.bias = l < (int)e->hbias.size() && !e->hbias[l].empty() ? e->hbias[l].data() : nullptr;
  v.pos = e->pos.empty() ? nullptr : e->pos[l].data();
  v.constw = p.constw;
  v.wconst = p.wconst;
  v.nblocks = p.nblocks;
  v.nnz = p.nnz;
  v.slots = p.slots;
  v.max_depth = p.max_depth;
  v.max_in_degree = max_in_degree;
  return v;
}

// Checks a packed layer from a file before it reaches the GPU: every slot
// index inside the shared row (chunk + 32 zero floats), positions in range.
bool check_view(const sdnn_engine* e, const PackedView& v, std::string& err) {
  const uint32_t limit = (uint32_t)(e->Q + 32) * (slot_index_in_bytes(e->Q) ? 4u : 1u);
  const size_t n = (size_t)v.nblocks * 128;
  const uint32_t step = slot_index_in_bytes(e->Q) ? 4u : 1u;
  for (size_t i = 0; i < n; ++i)
    if (v.idx[i] >= limit || v.idx[i] % step != 0) {
      err = "slot index out of range";
      return false;
    }
  if (v.pos) {
    std::vector<char> seen(e->N, 0);
    for (int c = 0; c < e->N; ++c) {
      const int32_t q = v.pos[c];
      if (q < 0 || q >= e->N || seen[q]) {
        err = "placement is not a permutation";
        return false;
      }
      seen[q] = 1;
    }
  }
  return true;
}

// Uploads one packed layer (slots, offsets, values, placed bias, first-layer sums).
int upload_layer(sdnn_engine* e, int l, const PackedView& p, std::string& err) {
  DevLayer d;
  d.constw = p.constw;
  d.wconst = p.wconst;
  d.nnz = p.nnz;
  d.slots = p.slots;
  d.max_depth = p.max_depth;
  if (e->nq == 1) {
    d.chain_slice8 = chain_slice_bytes(p.grp_blk, e->G, !p.constw, 8);
    d.chain_slice16 = chain_slice_bytes(p.grp_blk, e->G, !p.constw, 16);
  }
  const size_t nslot = (size_t)p.nblocks * 128;
  const size_t ngrp = (size_t)e->G * e->nq + 1;
  cudaError_t rc = cudaSuccess;
  auto T = [&](cudaError_t r) {
    if (rc == cudaSuccess) rc = r;
  };
  T(cudaMalloc((void**)&d.idx, std::max<size_t>(nslot * 2, 16)));
  T(cudaMalloc((void**)&d.grp, ngrp * 4));
  if (!p.constw) T(cudaMalloc((void**)&d.val, std::max<size_t>(nslot * 4, 16)));
  if (p.bias) T(cudaMalloc((void**)&d.bias, (size_t)e->N * 4));
  if (rc == cudaSuccess && nslot) T(cudaMemcpy(d.idx, p.idx, nslot * 2, cudaMemcpyHostToDevice));
  if (rc == cudaSuccess) T(cudaMemcpy(d.grp, p.grp_blk, ngrp * 4, cudaMemcpyHostToDevice));
  if (rc == cudaSuccess && d.val && nslot)
    T(cudaMemcpy(d.val, p.val, nslot * 4, cudaMemcpyHostToDevice));
  if (rc == cudaSuccess && p.bias) {
    // per-neuron bias follows its neuron to its position
    std::vector<float> b(e->N);
    for (int c = 0; c < e->N; ++c) b[p.pos ? p.pos[c] : c] = p.bias[c];
    T(cudaMemcpy(d.bias, b.data(), (size_t)e->N * 4, cudaMemcpyHostToDevice));
  }
  if (rc == cudaSuccess && l == 0 && p.constw && p.max_depth < 128 && p.max_in_degree < 128) {
    // the float kernel adds w once per active edge: reproduce those sums
    float sums[128];
    float acc = 0.f;
    for (int k = 0; k < 128; ++k) {
      sums[k] = acc;
      acc = acc + p.wconst;
    }
    T(cudaMalloc((void**)&d.sums, sizeof(sums)));
    if (rc == cudaSuccess) T(cudaMemcpy(d.sums, sums, sizeof(sums), cudaMemcpyHostToDevice));
  }
  if (rc == cudaSuccess && e->sparse_built) {
    // out-edges of every input position, from the packed slots (padding slots
    // point past the chunk and are skipped), each input's edges by output
    const int32_t scale = slot_index_in_bytes(e->Q) ? 4 : 1;
    const int32_t N = e->N, Q = e->Q;
    std::vector<int32_t> off(N + 1, 0);
    for (int32_t g = 0; g < e->G; ++g)
      for (int32_t b = p.grp_blk[g]; b < p.grp_blk[g + 1]; ++b)
        for (int k = 0; k < 128; ++k) {
          const int32_t j = p.idx[(size_t)b * 128 + k] / scale;
          if (j < Q) off[j + 1]++;
        }
    for (int32_t j = 0; j < N; ++j) off[j + 1] += off[j];
    const size_t ne = (size_t)off[N];
    std::vector<std::pair<uint16_t, float>> edges(ne);
    std::vector<int32_t> fill(off.begin(), off.end() - 1);
    for (int32_t g = 0; g < e->G; ++g)
      for (int32_t b = p.grp_blk[g]; b < p.grp_blk[g + 1]; ++b)
        for (int k = 0; k < 128; ++k) {
          const int32_t j = p.idx[(size_t)b * 128 + k] / scale;
          if (j >= Q) continue;
          const float w = p.constw ? p.wconst : p.val[(size_t)b * 128 + k];
          edges[fill[j]++] = {(uint16_t)(32 * g + (k >> 2)), w};
        }
    std::vector<uint16_t> tout(ne);
    std::vector<float> tval(p.constw ? 0 : ne);
    for (int32_t j = 0; j < N; ++j) {
      std::sort(edges.begin() + off[j], edges.begin() + off[j + 1],
                [](const std::pair<uint16_t, float>& x, const std::pair<uint16_t, float>& y) {
                  return x.first < y.first;
                });
      for (int32_t t = off[j]; t < off[j + 1]; ++t) {
        tout[t] = edges[t].first;
        if (!p.constw) tval[t] = edges[t].second;
      }
    }
    T(cudaMalloc((void**)&d.tr_off, (size_t)(N + 1) * 4));
    T(cudaMalloc((void**)&d.tr_out, std::max<size_t>(ne * 2, 16)));
    if (!p.constw) T(cudaMalloc((void**)&d.tr_val, std::max<size_t>(ne * 4, 16)));
    if (rc == cudaSuccess) T(cudaMemcpy(d.tr_off, off.data(), (size_t)(N + 1) * 4, cudaMemcpyHostToDevice));
    if (rc == cudaSuccess && ne) T(cudaMemcpy(d.tr_out, tout.data(), ne * 2, cudaMemcpyHostToDevice));
    if (rc == cudaSuccess && d.tr_val && ne)
      T(cudaMemcpy(d.tr_val, tval.data(), ne * 4, cudaMemcpyHostToDevice));
  }
  e->dl[l] = d;
  if (rc != cudaSuccess) {
    err = std::string("weight upload failed: ") + cudaGetErrorString(rc);
    return rc == cudaErrorMemoryAllocation ? SDNN_ERR_OOM : SDNN_ERR_CUDA;
  }
  return SDNN_OK;
}

// Packs layer l with the chosen neuron placement and uploads it.
int pack_upload_layer(sdnn_engine* e, int l, std::string& err) {
  PackedLayer p;
  int32_t maxdeg = 0;
  int rc = pack_host_layer(e, l, p, maxdeg, err);
  if (rc) return rc;
  return upload_layer(e, l, view_of(e, l, p, maxdeg), err);
}

// Runs fn(l, err) for every layer on a small thread pool; first error wins.
template <typename Fn>
int for_layers(sdnn_engine* e, Fn fn) {
  int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  nthreads = std::min(nthreads, e->L);
  std::atomic<int> next{0};
  std::atomic<int> status{SDNN_OK};
  std::vector<std::string> errs(nthreads);
  auto worker = [&](int id) {
    cudaSetDevice(e->dev);
    for (;;) {
      const int l = next.fetch_add(1);
      if (l >= e->L || status.load() != SDNN_OK) break;
      const int rc = fn(l, errs[id]);
      if (rc != SDNN_OK) {
        int expected = SDNN_OK;
        status.compare_exchange_strong(expected, rc);
        break;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker, i);
  for (auto& t : pool) t.join();
  if (status.load() != SDNN_OK) {
    std::string msg;
    for (auto& m : errs)
      if (!m.empty()) msg = m;
    e->err = msg;
  }
  return status.load();
}

// Neuron placement of every layer into e->pos.  Whole rows: outputs grouped
// by in-degree, lanes balancing the next layer's bank loads.  Input chunks:
// each neuron's chunk balancing the next layer's per-chunk in-degrees, groups
// of outputs with similar per-chunk in-degrees, lanes balancing the next
// layer's (group, chunk, bank) loads.
int compute_placement_chunked(sdnn_engine* e) {
  const int L = e->L;
  std::vector<std::vector<uint8_t>> chunk(L);
  int rc = for_layers(e, [&](int l, std::string&) {
    HostLayer tmp;
    const HostLayer* next = l + 1 < L ? host_layer(e, l + 1, tmp) : nullptr;
    chunk[l] = chunk_assign(next, e->N, e->Q, 0x5EED0000ull + (uint64_t)l);
    return SDNN_OK;
  });
  if (rc) return rc;
  std::vector<std::vector<int32_t>> order(L);
  rc = for_layers(e, [&](int l, std::string&) {
    HostLayer tmp;
    order[l] = chunk_group_order(*host_layer(e, l, tmp), l > 0 ? chunk[l - 1].data() : nullptr,
                                 chunk[l], e->N, e->Q);
    return SDNN_OK;
  });
  if (rc) return rc;
  e->pos.assign(L, {});
  return for_layers(e, [&](int l, std::string&) {
    HostLayer tmp;
    const HostLayer* next = l + 1 < L ? host_layer(e, l + 1, tmp) : nullptr;
    e->pos[l] = place_outputs_chunked(order[l], chunk[l], next, next ? &order[l + 1] : nullptr,
                                      e->N, e->Q);
    return SDNN_OK;
  });
}

int compute_placement(sdnn_engine* e) {
  if (e->nq > 1) return compute_placement_chunked(e);
  std::vector<std::vector<int32_t>> order(e->L);
  int rc = for_layers(e, [&](int l, std::string&) {
    HostLayer tmp;
    order[l] = degree_order(*host_layer(e, l, tmp), e->N);
    return SDNN_OK;
  });
  if (rc) return rc;
  e->pos.assign(e->L, {});
  return for_layers(e, [&](int l, std::string&) {
    HostLayer tmp;
    const HostLayer* next = l + 1 < e->L ? host_layer(e, l + 1, tmp) : nullptr;
    e->pos[l] = place_outputs(order[l], next, next ? &order[l + 1] : nullptr, e->N);
    return SDNN_OK;
  });
}

// Packs every layer.  With whole-row layouts (one chunk) the neurons of each
// layer are first placed: outputs grouped by in-degree (so the 32 lanes of a
// group have nearly equal slot lists) and given lanes that balance the bank
// loads of the next layer, which shortens the bank-scheduled slot lists.
int finalize_weights(sdnn_engine* e) {
  if (!e->weights_dirty) return SDNN_OK;
  if (!e->gen.on && !e->packed) {
    if ((int)e->hw.size() != e->L) return fail(e, SDNN_ERR_STATE, "weights not loaded");
    for (int l = 0; l < e->L; ++l)
      if (!e->hw[l].present)
        return fail(e, SDNN_ERR_STATE, "layer " + std::to_string(l) + " has no weights");
  }
  drop_graph(e);
  free_weights(e);
  e->dl.assign(e->L, DevLayer{});
  e->pos.clear();
  const bool place = !e->packed && !(e->cfg.flags & SDNN_FLAG_NO_PLACEMENT);
  int rc;
  if (e->packed) {
    // a packed-weight file: its placement and slots as they are, checked first
    if (e->packed->placed) {
      e->pos.resize(e->L);
      for (int l = 0; l < e->L; ++l)
        e->pos[l].assign(e->packed->layers[l].pos, e->packed->layers[l].pos + e->N);
    }
    rc = for_layers(e, [&](int l, std::string& err) {
      const PackedView& v = e->packed->layers[l];
      if (!check_view(e, v, err)) {
        err = "packed weights, layer " + std::to_string(l) + ": " + err;
        return (int)SDNN_ERR_FORMAT;
      }
      return upload_layer(e, l, v, err);
    });
  } else if (place) {
    if ((rc = compute_placement(e))) return rc;
  }
  if (!e->packed)
    rc = for_layers(e, [&](int l, std::string& err) { return pack_upload_layer(e, l, err); });
  if (rc) {
    free_weights(e);
    return rc;
  }
  {
    std::vector<LayerDev> table(e->L);
    for (int l = 0; l < e->L; ++l) {
      const DevLayer& d = e->dl[l];
      table[l].idx = d.idx;
      table[l].val = d.val;
      table[l].grp_blk = d.grp;
      table[l].bias_vec = d.bias;
      table[l].bias = e->cfg.bias;
      table[l].wconst = d.wconst;
    }
    CK(cudaMalloc((void**)&e->d_layer_table, sizeof(LayerDev) * e->L));
    CK(cudaMemcpy(e->d_layer_table, table.data(), sizeof(LayerDev) * e->L, cudaMemcpyHostToDevice));
  }
  e->chain_cap = e->nq == 1 ? chain_capacity(e->N) : 0;
  e->chain_wcap8 = e->chain_wcap16 = 0;
  for (const DevLayer& d : e->dl) {
    e->chain_wcap8 = std::max(e->chain_wcap8, d.chain_slice8);
    e->chain_wcap16 = std::max(e->chain_wcap16, d.chain_slice16);
  }
  if (!e->pos.empty()) {
    CK(cudaMalloc((void**)&e->d_perm_final, (size_t)e->N * 4));
    CK(cudaMemcpy(e->d_perm_final, e->pos[e->L - 1].data(), (size_t)e->N * 4,
                  cudaMemcpyHostToDevice));
  }
  e->total_nnz = 0;
  for (auto& d : e->dl) e->total_nnz += d.nnz;
  e->weights_dirty = false;
  return SDNN_OK;
}

int layer_launch(sdnn_engine* e, int l, int epi, const float* in, float* out, const int32_t* lin,
                 const int32_t* cin, int32_t* lout, int32_t* cout) {
  const DevLayer& d = e->dl[l];
  LayerArgs a{};
  a.w.idx = d.idx;
  a.w.val = d.val;
  a.w.grp_blk = d.grp;
  a.w.bias_vec = d.bias;
  a.w.bias = e->cfg.bias;
  a.w.wconst = d.wconst;
  a.y_in = in;
  a.y_out = out;
  a.list_in = lin;
  a.count_in = cin;
  a.list_out = lout;
  a.count_out = cout;
  a.tile_mask = e->d_tmask;
  a.tile_ticket = e->d_ticket;
  a.pre_out = e->d_pre;
  a.pre_in = e->d_pre;
  a.cslot = e->d_cslot;
  a.err = e->d_err;
  a.N = e->N;
  a.nq = e->nq;
  a.Q = e->Q;
  a.G = e->G;
  a.epi = epi;
  a.max_split = e->G;
  a.min_split = e->min_split;
  a.clampv = e->cfg.clamp;
  LayerKernelKey k = e->key;
  k.constw = d.constw;
  CK(launch_layer(k, a, d.constw ? e->grid : e->grid_general, e->threads, e->smem, e->stream));
  e->launches++;
  return SDNN_OK;
}

int record(sdnn_engine* e, int i, bool capturing) {
  if (e->in_body) return SDNN_OK;  // conditional bodies hold no event records
  if (capturing) {
    CK(cudaEventRecordWithFlags(e->ev[i], e->stream, cudaEventRecordExternal));
  } else {
    CK(cudaEventRecord(e->ev[i], e->stream));
  }
  return SDNN_OK;
}

int effective_threshold(const sdnn_engine* e) {
  if (e->cfg.mode != SDNN_MODE_SNICIT) return e->L;
  return std::max(0, std::min(e->cfg.threshold, e->L));
}

// Parts of one inference.  Plain modes (and thresholds at or past the last
// layer) enqueue PH_ALL.  SNICIT runs PH_PRE (plain layers below the threshold
// and the clustering), then, depending on what the clustering left (read back
// by the host once), PH_POST_CHAIN (no residue rows: the centroid rows alone,
// one cluster kernel for all remaining layers) or PH_POST_LAYERS (a centroid
// and a residue launch per layer), then PH_FINISH (recovery).
enum Phase { PH_ALL = 0, PH_PRE = 1, PH_POST_LAYERS = 2, PH_POST_CHAIN = 3, PH_FINISH = 4 };

// Merging of identical rows runs in SNICIT mode after plain layer l when
// merge_start <= l + 1 < T (the threshold clustering covers layer T - 1) and
// every merge_every layers from there.
bool merging_on(const sdnn_engine* e) {
  return e->cfg.mode == SDNN_MODE_SNICIT && !(e->cfg.flags & SDNN_FLAG_NO_MERGE);
}

bool merge_after(const sdnn_engine* e, int l, int T) {
  if (!merging_on(e)) return false;
  const int start = e->cfg.merge_start > 0 ? e->cfg.merge_start : kMergeStart;
  const int every = e->cfg.merge_every > 0 ? e->cfg.merge_every : 1;
  const int k = l + 1;
  return k >= start && k < T && (k - start) % every == 0;
}

int enqueue_merge(sdnn_engine* e, int l) {
  DedupArgs m{};
  m.y = e->d_y[l & 1];
  m.list = e->d_list[(l + 1) & 1];
  m.count = e->d_counts + l + 1;
  m.table = e->d_mtable;
  m.slot_rep = e->d_mrep;
  m.pos_slot = e->d_mpos;
  m.tmp_list = e->d_mtmp;
  m.tmp_count = e->d_mcount;
  m.alias = e->d_alias;
  m.N = e->N;
  m.mask = e->mmask;
  launch_dedup(m, e->num_sms, e->stream);
  e->launches += 3;
  CK(cudaGetLastError());
  return SDNN_OK;
}

// Enqueues plain layer l over the row list (lin, cin) into (lout, cout);
// layer 0 of 0/1 inputs takes the binary counting kernels, with the tiles that
// hold other values sent to the float kernel.
int enqueue_layer(sdnn_engine* e, int l, const float* in, const int32_t* lin, const int32_t* cin,
                  int32_t* lout, int32_t* cout) {
  const cudaStream_t s = e->stream;
  const bool bits = l == 0 && e->dl[0].sums && (e->bits_chunked || e->bits_grid > 0);
  if (!bits) return layer_launch(e, l, EPI_PLAIN, in, e->d_y[l & 1], lin, cin, lout, cout);
  CK(cudaMemsetAsync(e->d_fbcount, 0, 16, s));
  Layer0Args b{};
  b.idx = e->dl[0].idx;
  b.grp_blk = e->dl[0].grp;
  b.bias_vec = e->dl[0].bias;
  b.bias = e->cfg.bias;
  b.clampv = e->cfg.clamp;
  b.sums = e->dl[0].sums;
  b.y_in = in;
  b.y_out = e->d_y[0];
  b.list_in = lin;
  b.count_in = cin;
  b.list_out = lout;
  b.count_out = cout;
  b.fallback_list = e->d_fallback;
  b.fallback_count = e->d_fbcount;
  b.N = e->N;
  b.G = e->G;
  if (e->bits_chunked) {
    // input chunks: transpose pass + counting pass
    b.nq = e->nq;
    b.Q = e->Q;
    b.bits = e->d_bits + e->bits_tile0 * e->N;
    b.tile_state = e->d_tile_state + e->bits_tile0;
    b.tile_mask = e->d_tmask;
    b.tile_ticket = e->d_ticket;
    b.err = e->d_err;
    CK(launch_layer0_bits_chunked(b, e->num_sms, s));
    e->launches += 2;
  } else {
    CK(launch_layer0_bits(b, e->bits_grid, kBitsThreads, s));
    e->launches++;
  }
  return layer_launch(e, 0, EPI_PLAIN, in, e->d_y[0], e->d_fallback, e->d_fbcount, lout, cout);
}

// Enqueues plain layers e->pipe_start .. T - 1 over the global row lists (the
// layers below pipe_start ran piece by piece, enqueue_piece), with the merge
// steps between them.
int enqueue_plain_layers(sdnn_engine* e, const float* d_in, int T, bool capturing) {
  const int L = e->L;
  int rc;
  // XY mode splits the plain loop at the threshold for its pre/post timing
  // (src/SDGC/XY/XY.hpp:492-501); BF and SNIG time the loop as one stage.
  const int split = e->cfg.mode == SDNN_MODE_XY ? std::max(0, std::min(e->cfg.threshold, L)) : T;
  const int first = e->pipe_start;
  if (first > 0 && merge_after(e, first - 1, T) && (rc = enqueue_merge(e, first - 1))) return rc;
  for (int l = first; l < T; ++l) {
    if (l == split && T == L) {
      if ((rc = record(e, 1, capturing))) return rc;
      if ((rc = record(e, 2, capturing))) return rc;
    }
    const float* in = l == 0 ? d_in : e->d_y[(l - 1) & 1];
    if ((rc = enqueue_layer(e, l, in, e->d_list[l & 1], e->d_counts + l, e->d_list[(l + 1) & 1],
                            e->d_counts + l + 1)))
      return rc;
    if (merge_after(e, l, T) && (rc = enqueue_merge(e, l))) return rc;
  }
  if (!(split < T && T == L)) {
    if ((rc = record(e, 1, capturing))) return rc;
  }
  return SDNN_OK;
}

// Layers 0 .. m - 1 of one piece of rows (rows r0 .. r0 + n - 1 of the batch),
// enqueued eagerly once the piece's copy has landed.  Rows are independent
// until the first cross-row step (the first merge or the threshold
// clustering), so every row gets the same bits as in the whole-batch run.
// The piece keeps its row lists in its own segment [r0, r0 + n) of the piece
// list buffers (d_plist, identity rows for layer 0) with its own counters; its
// last layer appends the survivors to the global list of layer m, which no
// piece list shares memory with.
int enqueue_piece(sdnn_engine* e, int p, int64_t r0, int64_t n, int m, const float* d_in) {
  int32_t* pc = e->d_pcounts + (size_t)p * (e->L + 2);
  // an ordinary launch right after the copy's event: the layer launches that
  // follow (programmatic serialization) then wait for a completed kernel
  launch_set_scalar(pc, (int32_t)n, e->stream);
  e->launches++;
  CK(cudaGetLastError());
  // the piece's bit words (binary layer 0 with input chunks) go to its own
  // tiles of the buffer (pieces start on 32-row tiles), so both lanes may run
  e->bits_tile0 = r0 / 32;
  for (int l = 0; l < m; ++l) {
    const float* in = l == 0 ? d_in : e->d_y[(l - 1) & 1];
    const bool last = l + 1 == m;
    int32_t* lout = last ? e->d_list[m & 1] : e->d_plist[(l + 1) & 1] + r0;
    int32_t* cout = last ? e->d_counts + m : pc + l + 1;
    int rc = enqueue_layer(e, l, in, e->d_plist[l & 1] + r0, pc + l, lout, cout);
    if (rc) {
      e->bits_tile0 = 0;
      return rc;
    }
  }
  e->bits_tile0 = 0;
  return SDNN_OK;
}

SparseRows sparse_rows(const sdnn_engine* e, int b) {
  return SparseRows{e->d_sp_idx[b], e->d_sp_val[b], e->d_sp_cnt[b], e->sp_cap};
}

// Enqueues one phase of an inference of `rows` rows read from d_in.
int enqueue(sdnn_engine* e, int phase, int64_t rows, const float* d_in, int32_t* d_flags,
            bool capturing) {
  const int L = e->L;
  const int T = effective_threshold(e);
  const cudaStream_t s = e->stream;
  int rc;
  float* ybuf = e->d_y[(T - 1 + 2) & 1];  // activations at the threshold
  const int32_t* live = e->d_list[T & 1];
  const int32_t* live_count = e->d_counts + T;
  (void)rows;  // the row count is read on the device from d_rows
  if (phase == PH_ALL || phase == PH_PRE) {
    if (e->pipe_start == 0) {
      if ((rc = record(e, 0, capturing))) return rc;
      CK(cudaMemsetAsync(e->d_counts, 0, (size_t)(L + 4) * 4, s));
      launch_begin_rows(e->d_rows, e->d_list[0], e->d_counts, d_flags, e->d_state, e->d_alias, s);
      e->launches++;
    }
    if ((rc = enqueue_plain_layers(e, d_in, T, capturing))) return rc;
  }
  if (phase == PH_PRE) {
    if (T == 0) {
      launch_copy_rows(e->d_rows, d_in, ybuf, e->N, s);
      e->launches++;
    }
    CK(cudaMemsetAsync(e->d_rcounts, 0, (size_t)(L + 4) * 4, s));
    if (e->sparse_res) {
      CK(cudaMemsetAsync(e->d_scounts, 0, (size_t)(L + 4) * 4, s));
      CK(cudaMemsetAsync(e->d_tcounts, 0, (size_t)(L + 4) * 4, s));
    }
    launch_zero_rows(e->d_rows, e->d_iscent, e->d_resflag, s);
    e->launches++;
    CK(cudaMemsetAsync(e->d_ccount, 0, 16, s));
    CK(cudaMemsetAsync(e->d_ncand, 0, 16, s));
    ClusterArgs c{};
    c.y = ybuf;
    c.live = live;
    c.live_count = live_count;
    c.N = e->N;
    c.K = std::max(1, e->cfg.num_centroids);
    c.seed = e->cfg.seed;
    c.cand = e->d_cand;
    c.ncand = e->d_ncand;
    c.bins = e->d_bins;
    c.clist = e->d_clist;
    c.ccount = e->d_ccount;
    c.cslot = e->d_cslot;
    // residue rows of the clustering: straight to the dense list, or first to
    // d_rtmp to be split into dense and sparse rows
    c.rlist = e->sparse_res ? e->d_rtmp : e->d_rlist[0];
    c.rcount = e->sparse_res ? e->d_tcounts : e->d_rcounts;
    c.is_centroid = e->d_iscent;
    c.err = e->d_err;
    launch_cluster(c, e->num_sms, s);
    e->launches += 4;
    if (e->sparse_res) {
      launch_split_residue(ybuf, e->d_rtmp, e->d_tcounts, sparse_rows(e, 0), e->d_rlist[0],
                           e->d_rcounts, e->d_slist[0], e->d_scounts, e->N, e->num_sms, s);
      e->launches++;
    }
    if ((rc = record(e, 2, capturing))) return rc;
  }
  if (phase == PH_POST_LAYERS) {
    for (int l = T; l < L; ++l) {
      const int p = l - T;
      const float* in = e->d_y[(l - 1 + 2) & 1];
      float* out = e->d_y[l & 1];
      if ((rc = layer_launch(e, l, EPI_CENTROID, in, out, e->d_clist, e->d_ccount, nullptr,
                             nullptr)))
        return rc;
      if (!e->sparse_res) {
        if ((rc = layer_launch(e, l, EPI_RESIDUE, in, out, e->d_rlist[p & 1], e->d_rcounts + p,
                               e->d_rlist[(p + 1) & 1], e->d_rcounts + p + 1)))
          return rc;
        continue;
      }
      // dense residue rows: the layer kernel, then their split by nonzeros
      if ((rc = layer_launch(e, l, EPI_RESIDUE, in, out, e->d_rlist[p & 1], e->d_rcounts + p,
                             e->d_rtmp, e->d_tcounts + p + 1)))
        return rc;
      const SparseRows next = sparse_rows(e, (p + 1) & 1);
      launch_split_residue(out, e->d_rtmp, e->d_tcounts + p + 1, next, e->d_rlist[(p + 1) & 1],
                           e->d_rcounts + p + 1, e->d_slist[(p + 1) & 1], e->d_scounts + p + 1,
                           e->N, e->num_sms, s);
      // sparse residue rows: scattered along the transposed layer
      const DevLayer& d = e->dl[l];
      SparseResArgs sa{};
      sa.list_in = e->d_slist[p & 1];
      sa.count_in = e->d_scounts + p;
      sa.in = sparse_rows(e, p & 1);
      sa.out = next;
      sa.y_out = out;
      sa.dense_list = e->d_rlist[(p + 1) & 1];
      sa.dense_count = e->d_rcounts + p + 1;
      sa.sparse_list = e->d_slist[(p + 1) & 1];
      sa.sparse_count = e->d_scounts + p + 1;
      sa.tr_off = d.tr_off;
      sa.tr_out = d.tr_out;
      sa.tr_val = d.tr_val;
      sa.wconst = d.wconst;
      sa.pre = e->d_pre;
      sa.cslot = e->d_cslot;
      sa.N = e->N;
      sa.clampv = e->cfg.clamp;
      CK(launch_sparse_residue(sa, e->num_sms, s));
      e->launches += 2;
    }
    if ((rc = record(e, 3, capturing))) return rc;
  }
  if (phase == PH_POST_CHAIN && e->chain_kind == 2) {
    GridChainArgs ga{};
    ga.layers = e->d_layer_table;
    ga.first = T;
    ga.last = L;
    ga.y_in = ybuf;
    ga.y_out = e->d_y[(L - 1) & 1];
    ga.clist = e->d_clist;
    ga.ccount = e->d_ccount;
    ga.N = e->N;
    ga.G = e->G;
    ga.nq = e->nq;
    ga.Q = e->Q;
    ga.clampv = e->cfg.clamp;
    ga.scratch = e->d_gscratch;
    ga.barrier = e->d_gbar;
    ga.err = e->d_err;
    CK(launch_grid_chain(ga, e->chain_kc, e->num_sms, s));
    e->launches++;
    if ((rc = record(e, 3, capturing))) return rc;
  } else if (phase == PH_POST_CHAIN) {
    ChainArgs ca{};
    ca.layers = e->d_layer_table;
    ca.first = T;
    ca.last = L;
    ca.y_in = ybuf;
    ca.y_out = e->d_y[(L - 1) & 1];
    ca.clist = e->d_clist;
    ca.ccount = e->d_ccount;
    ca.N = e->N;
    ca.G = e->G;
    ca.clampv = e->cfg.clamp;
    ca.err = e->d_err;
    ca.stream = !(e->cfg.flags & SDNN_FLAG_NO_CHAIN_STREAM);
    ca.wcap8 = e->chain_wcap8;
    ca.wcap16 = e->chain_wcap16;
    CK(launch_chain(ca, e->chain_kc, s));
    e->launches++;
    if ((rc = record(e, 3, capturing))) return rc;
  }
  if (phase == PH_FINISH) {
    const int pf = L - T;
    launch_mark_rows(e->d_rlist[pf & 1], e->d_rcounts + pf, e->d_resflag, 1, s);
    if (e->sparse_res) {
      // the last sparse rows, written densely into the final buffer: from here
      // on every residue row reads the same way
      launch_densify(e->d_slist[pf & 1], e->d_scounts + pf, sparse_rows(e, pf & 1),
                     e->d_y[(L - 1) & 1], e->N, e->num_sms, s);
      launch_mark_rows(e->d_slist[pf & 1], e->d_scounts + pf, e->d_resflag, 1, s);
      e->launches += 2;
    }
    launch_recover(e->d_y[(L - 1) & 1], live, live_count, e->d_cslot, e->d_clist, e->d_iscent,
                   e->d_resflag, e->N, d_flags, s);
    launch_mark_rows(live, live_count, e->d_state, 2, s);
    e->launches += 3;
    if (merging_on(e)) {
      launch_resolve_alias(e->d_rows, e->d_alias, d_flags, L, s);
      e->launches++;
    }
    if ((rc = record(e, 4, capturing))) return rc;
  }
  if (phase == PH_ALL) {
    if (e->cfg.mode != SDNN_MODE_XY || std::min(e->cfg.threshold, L) >= T) {
      if ((rc = record(e, 2, capturing))) return rc;
    }
    if ((rc = record(e, 3, capturing))) return rc;
    launch_identify(e->d_y[(L - 1) & 1], e->d_list[L & 1], e->d_counts + L, e->N, d_flags, s);
    launch_mark_rows(e->d_list[L & 1], e->d_counts + L, e->d_state, 1, s);
    e->launches += 2;
    if (merging_on(e)) {  // SNICIT with the threshold at or past the last layer
      launch_resolve_alias(e->d_rows, e->d_alias, d_flags, L, s);
      e->launches++;
    }
    if ((rc = record(e, 4, capturing))) return rc;
  }
  CK(cudaGetLastError());
  return SDNN_OK;
}

// Runs one phase: eagerly in BF mode, else from a cached CUDA graph (captured
// on first use and whenever the pointers, sizes or kernel choice change).
int run_phase(sdnn_engine* e, int slot, int phase, int64_t rows, const float* d_in,
              int32_t* d_flags) {
  if (e->cfg.mode == SDNN_MODE_BF) {
    const int before = e->launches;
    e->launches = 0;
    int rc = enqueue(e, phase, rows, d_in, d_flags, false);
    e->run_launches += e->launches;
    e->launches = before;
    return rc;
  }
  const bool streamed = e->pipe_start > 0 && (phase == PH_ALL || phase == PH_PRE);
  GraphSlot& g = e->graphs[streamed ? 5 + slot : slot];
  const GraphKey key{0, d_in, d_flags, effective_threshold(e), std::max(1, e->cfg.num_centroids), e->cfg.mode,
                     e->key.T, e->threads,
                     phase == PH_POST_CHAIN ? e->chain_kc * 4 + e->chain_kind : 0,
                     streamed ? e->pipe_start : 0};
  if (!g.exec || !(g.key == key)) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    e->launches = 0;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue(e, phase, rows, d_in, d_flags, true);
    cudaGraph_t graph = nullptr;
    cudaError_t rc2 = cudaStreamEndCapture(e->stream, &graph);
    if (rc != SDNN_OK) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return rc;
    }
    if (rc2 != cudaSuccess) return cuda_fail(e, rc2, "cudaStreamEndCapture");
    cudaError_t rc3 = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (rc3 != cudaSuccess) {
      g.exec = nullptr;
      return cuda_fail(e, rc3, "cudaGraphInstantiate");
    }
    g.key = key;
    g.launches = e->launches;
  }
  CK(cudaGraphLaunch(g.exec, e->stream));
  e->run_launches += g.launches;
  return SDNN_OK;
}

// Captures one SNICIT inference into a single graph: PH_PRE, then a one-thread
// kernel that reads what the clustering left and sets a SWITCH node's value,
// the SWITCH node with one body per post-threshold path (the per-layer
// launches, and the cluster / grid chain kernel for 1, 2, 4, 8 centroid rows:
// the choices the host made after its read-back), then PH_FINISH.  No host
// synchronisation inside an inference.  The bodies are captured after the main
// capture has ended (each body graph belongs to the SWITCH node).
int build_full_graph(sdnn_engine* e, FullGraph& fg, int64_t rows, const float* d_in,
                     int32_t* d_flags) {
  cudaGraph_t graph = nullptr;
  CK(cudaGraphCreate(&graph, 0));
  int rc = SDNN_OK;
  auto give_up = [&](int code) {
    cudaGraphDestroy(graph);
    cudaGetLastError();
    e->in_body = false;
    return code;
  };
  cudaGraphConditionalHandle h{};
  cudaError_t r = cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault);
  if (r != cudaSuccess) return give_up(cuda_fail(e, r, "cudaGraphConditionalHandleCreate"));

  PostChoiceArgs pc{};
  pc.rcount = e->d_rcounts;
  pc.scount = e->sparse_res ? e->d_scounts : nullptr;
  pc.ccount = e->d_ccount;
  pc.choice = e->d_choice;
  pc.chain_cap = e->chain_cap;
  pc.grid_cap = grid_chain_capacity();
  pc.no_chain = (e->cfg.flags & SDNN_FLAG_NO_CHAIN) ? 1 : 0;
  pc.has_body[0] = 1;
  const bool grid_ok = e->d_gscratch && !(e->cfg.flags & SDNN_FLAG_NO_GRID_CHAIN);
  for (int i = 0; i < 4; ++i) {
    fg.variant[i] = 0;
    if (e->chain_cap > 0) {
      ChainArgs ca{};
      ca.N = e->N;
      ca.G = e->G;
      ca.stream = !(e->cfg.flags & SDNN_FLAG_NO_CHAIN_STREAM);
      ca.wcap8 = e->chain_wcap8;
      ca.wcap16 = e->chain_wcap16;
      fg.variant[i] = chain_plan(ca, 1 << i).variant;
    }
    pc.has_body[1 + 2 * i] = fg.variant[i] >= 1;
    pc.has_body[2 + 2 * i] = grid_ok && (1 << i) <= grid_chain_capacity();
  }

  r = cudaStreamBeginCaptureToGraph(e->stream, graph, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal);
  if (r != cudaSuccess) return give_up(cuda_fail(e, r, "cudaStreamBeginCaptureToGraph"));
  e->launches = 0;
  rc = enqueue(e, PH_PRE, rows, d_in, d_flags, true);
  cudaGraphNodeParams sw{};
  if (rc == SDNN_OK) {
    launch_post_choice(pc, h, e->stream);
    e->launches++;
    r = cudaGetLastError();
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (r == cudaSuccess) r = cudaStreamGetCaptureInfo(e->stream, &st, nullptr, &cg, &deps, nullptr, &nd);
    sw.type = cudaGraphNodeTypeConditional;
    sw.conditional.handle = h;
    sw.conditional.type = cudaGraphCondTypeSwitch;
    sw.conditional.size = kPostBodies;
    cudaGraphNode_t node = nullptr;
    if (r == cudaSuccess) r = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &sw);
    if (r == cudaSuccess)
      r = cudaStreamUpdateCaptureDependencies(e->stream, &node, nullptr, 1,
                                              cudaStreamSetCaptureDependencies);
    if (r != cudaSuccess) rc = cuda_fail(e, r, "post-threshold switch node");
  }
  if (rc == SDNN_OK) rc = record(e, 3, true);
  if (rc == SDNN_OK) rc = enqueue(e, PH_FINISH, rows, d_in, d_flags, true);
  cudaGraph_t captured = nullptr;
  r = cudaStreamEndCapture(e->stream, &captured);
  if (rc != SDNN_OK) return give_up(rc);
  if (r != cudaSuccess) return give_up(cuda_fail(e, r, "cudaStreamEndCapture"));
  fg.launches = e->launches;

  for (int b = 0; b < kPostBodies; ++b) {
    cudaGraph_t body = sw.conditional.phGraph_out[b];
    fg.body_launches[b] = 0;
    if (!pc.has_body[b]) {
      cudaGraphNode_t n;
      r = cudaGraphAddEmptyNode(&n, body, nullptr, 0);
      if (r != cudaSuccess) return give_up(cuda_fail(e, r, "cudaGraphAddEmptyNode"));
      continue;
    }
    r = cudaStreamBeginCaptureToGraph(e->stream, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return give_up(cuda_fail(e, r, "cudaStreamBeginCaptureToGraph"));
    e->in_body = true;
    e->launches = 0;
    int phase = PH_POST_LAYERS;
    if (b > 0) {
      phase = PH_POST_CHAIN;
      e->chain_kc = 1 << ((b - 1) / 2);
      e->chain_kind = (b & 1) ? 1 : 2;
    }
    rc = enqueue(e, phase, rows, d_in, d_flags, true);
    e->in_body = false;
    cudaGraph_t got = nullptr;
    r = cudaStreamEndCapture(e->stream, &got);
    if (rc != SDNN_OK) return give_up(rc);
    if (r != cudaSuccess) return give_up(cuda_fail(e, r, "cudaStreamEndCapture"));
    fg.body_launches[b] = e->launches;
  }
  r = cudaGraphInstantiate(&fg.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (r != cudaSuccess) {
    fg.exec = nullptr;
    cudaGetLastError();
    return cuda_fail(e, r, "cudaGraphInstantiate");
  }
  return SDNN_OK;
}

// Runs a SNICIT inference as one graph launch (built on first use).  Returns
// SDNN_ERR_UNSUPPORTED when the graph cannot be built (the caller then lets
// the host choose the post-threshold path, for this and every later call).
int run_full(sdnn_engine* e, int64_t rows, const float* d_in, int32_t* d_flags) {
  const int slot = e->pipe_start > 0 ? 1 : 0;
  FullGraph& fg = e->full[slot];
  const GraphKey key{0, d_in, d_flags, effective_threshold(e), std::max(1, e->cfg.num_centroids), e->cfg.mode,
                     e->key.T, e->threads, 0, e->pipe_start};
  if (!fg.exec || !(fg.key == key)) {
    if (fg.exec) cudaGraphExecDestroy(fg.exec);
    fg = FullGraph{};
    if (build_full_graph(e, fg, rows, d_in, d_flags) != SDNN_OK) return SDNN_ERR_UNSUPPORTED;
    fg.key = key;
  }
  CK(cudaGraphLaunch(fg.exec, e->stream));
  e->run_launches += fg.launches;
  e->last_full = 1 + slot;
  return SDNN_OK;
}

int run(sdnn_engine* e, int64_t rows, const float* d_in, int32_t* d_flags) {
  if (rows <= 0) return fail(e, SDNN_ERR_INVALID, "rows must be positive");
  if (rows > e->cap) return fail(e, SDNN_ERR_INVALID, "rows exceed the batch capacity");
  const int T = effective_threshold(e);
  e->last_T = T;
  e->last_rows = rows;
  e->run_launches = 0;
  if (e->pipe_start == 0) e->last_pieces = 0;
  // the graphs read the row count from d_rows (one graph for every count)
  launch_set_scalar(e->d_rows, (int32_t)rows, e->stream);
  e->run_launches++;
  int rc;
  e->last_full = 0;
  const bool full = e->cfg.mode == SDNN_MODE_SNICIT && T < e->L && !e->full_off &&
                    !(e->cfg.flags & SDNN_FLAG_HOST_POST_CHOICE);
  if (full) {
    rc = run_full(e, rows, d_in, d_flags);
    if (rc == SDNN_ERR_UNSUPPORTED) {
      // the graph could not be built here: the host chooses from now on
      e->full_off = true;
      e->err.clear();
    } else if (rc) {
      return rc;
    }
  }
  if (e->last_full) {
    // post-threshold path chosen on the device (stats read it back later)
  } else if (e->cfg.mode != SDNN_MODE_SNICIT || T >= e->L) {
    e->last_post_kernel = 0;
    if ((rc = run_phase(e, 0, PH_ALL, rows, d_in, d_flags))) return rc;
  } else {
    if ((rc = run_phase(e, 1, PH_PRE, rows, d_in, d_flags))) return rc;
    // what did the clustering leave?  (one small read-back per inference)
    CK(cudaMemcpyAsync(e->h_counts, e->d_rcounts, 4, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(e->h_counts + 1, e->d_ccount, 4, cudaMemcpyDeviceToHost, e->stream));
    e->h_counts[2] = 0;
    if (e->sparse_res)
      CK(cudaMemcpyAsync(e->h_counts + 2, e->d_scounts, 4, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    const int residues = e->h_counts[0] + e->h_counts[2], centroids = e->h_counts[1];
    // no residue left: one chain launch carries the centroid rows -- the
    // cluster kernel where the rows fit shared memory (measured faster: 1.6
    // and 7.2 us per layer at N = 4096 and 16384 against 13.8 and 11.8 for the
    // grid kernel), else the grid kernel
    int kind = 0, variant = 0;
    if (residues == 0 && centroids >= 1 && !(e->cfg.flags & SDNN_FLAG_NO_CHAIN)) {
      e->chain_kc = 1;
      while (e->chain_kc < centroids) e->chain_kc *= 2;
      if (e->chain_cap > 0 && centroids <= e->chain_cap) {
        ChainArgs ca{};
        ca.N = e->N;
        ca.G = e->G;
        ca.stream = !(e->cfg.flags & SDNN_FLAG_NO_CHAIN_STREAM);
        ca.wcap8 = e->chain_wcap8;
        ca.wcap16 = e->chain_wcap16;
        variant = chain_plan(ca, e->chain_kc).variant;
      }
      const bool grid_ok = e->d_gscratch && !(e->cfg.flags & SDNN_FLAG_NO_GRID_CHAIN) &&
                           centroids <= grid_chain_capacity();
      if (variant >= 1) kind = 1;
      else if (grid_ok) kind = 2;
    }
    e->chain_kind = kind;
    if (kind) {
      if ((rc = run_phase(e, 2, PH_POST_CHAIN, rows, d_in, d_flags))) return rc;
    } else {
      if ((rc = run_phase(e, 3, PH_POST_LAYERS, rows, d_in, d_flags))) return rc;
    }
    e->last_chain = kind != 0;
    e->last_post_kernel = kind == 1 ? 1 + variant : kind == 2 ? 4 : 1;
    if ((rc = run_phase(e, 4, PH_FINISH, rows, d_in, d_flags))) return rc;
  }
  e->launches = e->run_launches;
  e->have_run = true;
  e->pending_stats = 1;
  return SDNN_OK;
}

int ensure_cuda(sdnn_engine* e) {
  if (e->stream) {
    CK(cudaSetDevice(e->dev));
    return SDNN_OK;
  }
  CK(cudaSetDevice(e->dev));
  CK(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->dev));
  CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  for (int i = 0; i < 5; ++i) CK(cudaEventCreate(&e->ev[i]));
  return SDNN_OK;
}

int prepare(sdnn_engine* e, int64_t rows) {
  int rc = ensure_cuda(e);
  if (rc) return rc;
  rc = finalize_weights(e);
  if (rc) return rc;
  if (e->grid == 0) {
    rc = choose_kernel(e);
    if (rc) return rc;
  }
  CK(layer_prepare(LayerKernelKey{e->key.T, e->key.rsw, e->key.kg, true}, e->smem));
  CK(layer_prepare(LayerKernelKey{e->key.T, e->key.rsw, e->key.kg, false}, e->smem));
  if (e->sparse_built) CK(sparse_residue_prepare(e->N));
  e->bits_chunked = e->nq > 1 && !(e->cfg.flags & SDNN_FLAG_NO_BINARY_FIRST_LAYER) &&
                    layer0_bits_chunked_supported(e->N, e->Q);
  e->bits_grid = (e->nq == 1 && !(e->cfg.flags & SDNN_FLAG_NO_BINARY_FIRST_LAYER) &&
                  layer0_bits_supported(e->N))
                     ? layer0_bits_grid(e->N, e->num_sms, kBitsThreads)
                     : 0;
  return ensure_buffers(e, rows);
}

int check_device_error(sdnn_engine* e) {
  int32_t h = 0;
  CK(cudaMemcpyAsync(&h, e->d_err, 4, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  if (h == DEV_TIMEOUT) {
    cudaMemsetAsync(e->d_err, 0, 4, e->stream);
    cudaMemsetAsync(e->d_tmask, 0, (size_t)(e->cap + 1) * 4, e->stream);
    cudaMemsetAsync(e->d_ticket, 0, (size_t)(e->cap + 1) * 4, e->stream);
    return fail(e, SDNN_ERR_TIMEOUT, "a device-side wait timed out");
  }
  if (h != 0) return fail(e, SDNN_ERR_CUDA, "device error word " + std::to_string(h));
  return SDNN_OK;
}

int collect_stats(sdnn_engine* e) {
  if (!e->pending_stats) return SDNN_OK;
  CK(cudaStreamSynchronize(e->stream));
  const int L = e->L, T = e->last_T;
  std::vector<int32_t> counts(L + 4), rcounts(L + 4);
  int32_t ccount = 0;
  CK(cudaMemcpy(counts.data(), e->d_counts, (size_t)(L + 4) * 4, cudaMemcpyDeviceToHost));
  sdnn_stats& st = e->stats;
  std::memset(&st, 0, sizeof(st));
  float ms[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) CK(cudaEventElapsedTime(&ms[i], e->ev[i], e->ev[i + 1]));
  // ev1->ev2 covers the clustering, ev2->ev3 the post layers
  for (int i = 0; i < 4; ++i) st.stage_ms[i] = ms[i];
  CK(cudaEventElapsedTime(&st.total_ms, e->ev[0], e->ev[4]));
  st.rows_in = e->last_rows;
  int64_t pre = 0, post = 0;
  for (int l = 0; l < T; ++l) pre += counts[l];
  if (T < L) {
    CK(cudaMemcpy(rcounts.data(), e->d_rcounts, (size_t)(L + 4) * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&ccount, e->d_ccount, 4, cudaMemcpyDeviceToHost));
    std::vector<int32_t> scounts(L + 4, 0);
    if (e->sparse_res)
      CK(cudaMemcpy(scounts.data(), e->d_scounts, (size_t)(L + 4) * 4, cudaMemcpyDeviceToHost));
    int64_t sparse = 0;
    for (int p = 0; p < L - T; ++p) {
      post += ccount + rcounts[p] + scounts[p];
      sparse += scounts[p];
    }
    st.centroids = ccount;
    st.residue_rows = rcounts[0] + scounts[0];
    st.sparse_residue_rows = scounts[0];
    st.sparse_row_layers = sparse;
    st.rows_out = 0;
  } else {
    st.rows_out = counts[L];
  }
  st.pre_row_layers = pre;
  st.post_row_layers = post;
  st.row_layers = pre + post;
  st.weight_nnz = e->total_nnz;
  st.launches = e->launches;
  st.threshold = T;
  st.tile_rows = e->key.T;
  st.threads = e->threads;
  st.input_pieces = e->last_pieces;
  st.centroid_candidates = e->cfg.num_centroids;
  st.merge_start = merging_on(e) ? (e->cfg.merge_start > 0 ? e->cfg.merge_start : kMergeStart) : 0;
  st.merge_every = merging_on(e) ? std::max(1, e->cfg.merge_every) : 0;
  st.post_kernel = e->last_post_kernel;
  if (e->last_full) {
    // the device chose the post-threshold path: which body ran
    const FullGraph& fg = e->full[e->last_full - 1];
    int32_t b = 0;
    CK(cudaMemcpy(&b, e->d_choice, 4, cudaMemcpyDeviceToHost));
    if (b < 0 || b >= kPostBodies) b = 0;
    st.post_kernel = b == 0 ? 1 : (b & 1) ? 1 + fg.variant[(b - 1) / 2] : 4;
    st.launches += fg.body_launches[b];
    st.device_post_choice = 1;
  }
  e->pending_stats = 0;
  return SDNN_OK;
}

}  // namespace

// ============================================================== C ABI

extern "C" {

int sdnn_abi_version(void) { return SDNN_ABI_VERSION; }

int sdnn_abi_sizes(int32_t* out, int32_t n) {
  if (!out || n < 0) return SDNN_ERR_INVALID;
  const int32_t sizes[4] = {(int32_t)sizeof(sdnn_config), (int32_t)sizeof(sdnn_stats),
                            (int32_t)sizeof(sdnn_server_config), (int32_t)sizeof(sdnn_server_stats)};
  for (int32_t i = 0; i < n && i < 4; ++i) out[i] = sizes[i];
  return SDNN_OK;
}

const char* sdnn_status_string(int status) {
  switch (status) {
    case SDNN_OK: return "ok";
    case SDNN_ERR_INVALID: return "invalid argument";
    case SDNN_ERR_CUDA: return "CUDA error";
    case SDNN_ERR_OOM: return "out of memory";
    case SDNN_ERR_IO: return "I/O error";
    case SDNN_ERR_FORMAT: return "malformed input";
    case SDNN_ERR_STATE: return "call out of order";
    case SDNN_ERR_TIMEOUT: return "device wait timed out";
    case SDNN_ERR_UNSUPPORTED: return "unsupported";
    case SDNN_ERR_BUSY: return "busy";
    default: return "unknown status";
  }
}

float sdnn_reference_bias(int32_t n) {
  switch (n) {
    case 65536: return -0.45f;
    case 16384: return -0.4f;
    case 4096: return -0.35f;
    case 1024: return -0.3f;
    default: return 0.f;
  }
}

int sdnn_config_default(sdnn_config* c) {
  if (!c) return SDNN_ERR_INVALID;
  std::memset(c, 0, sizeof(*c));
  c->num_neurons = 1024;
  c->num_layers = 120;
  c->mode = SDNN_MODE_SNICIT;
  c->threshold = 30;
  c->batch = 60000;
  c->bias = sdnn_reference_bias(1024);
  c->clamp = 32.f;
  c->num_centroids = 32;
  c->autotune = 0;
  c->seed = 20260101ull;
  c->device = 0;
  return SDNN_OK;
}

int sdnn_create(const sdnn_config* cfg, sdnn_engine** out) {
  if (!cfg || !out) return SDNN_ERR_INVALID;
  *out = nullptr;
  if (cfg->num_neurons < 32 || cfg->num_neurons % 32 != 0) return SDNN_ERR_INVALID;
  if (cfg->num_neurons > 32768 && cfg->num_neurons % 16384 != 0) return SDNN_ERR_INVALID;
  if (cfg->num_layers < 1 || cfg->batch < 1 || cfg->batch > (int64_t)1 << 30) return SDNN_ERR_INVALID;
  if (cfg->mode < SDNN_MODE_BF || cfg->mode > SDNN_MODE_SNICIT) return SDNN_ERR_INVALID;
  if (cfg->num_centroids < 1 || cfg->num_centroids > 256) return SDNN_ERR_INVALID;
  if (!(cfg->clamp > 0.f)) return SDNN_ERR_INVALID;
  if (cfg->tile_rows < 0 || cfg->tile_rows > 32) return SDNN_ERR_INVALID;
  auto* e = new (std::nothrow) sdnn_engine();
  if (!e) return SDNN_ERR_OOM;
  e->cfg = *cfg;
  e->N = cfg->num_neurons;
  e->L = cfg->num_layers;
  e->dev = cfg->device;
  e->hw.resize(e->L);
  choose_layout(e);
  // CUDA is initialised on first device use (ensure_cuda), so weights can be
  // loaded, generated and written on a host without a GPU.
  *out = e;
  return SDNN_OK;
}

int sdnn_destroy(sdnn_engine* e) {
  if (!e) return SDNN_OK;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  if (e->stream) {
    cudaSetDevice(e->dev);
    cudaStreamSynchronize(e->stream);
  }
  drop_graph(e);
  free_weights(e);
  free_buffers(e);
  for (auto& ev : e->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : e->piece_ev)
    if (ev) cudaEventDestroy(ev);
  if (e->ingest_free) cudaEventDestroy(e->ingest_free);
  if (e->lane_ev) cudaEventDestroy(e->lane_ev);
  if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
  if (e->stream2) cudaStreamDestroy(e->stream2);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return SDNN_OK;
}

const char* sdnn_last_error(const sdnn_engine* e) { return e ? e->err.c_str() : ""; }

int sdnn_load_weights_tsv(sdnn_engine* e, const char* dir) {
  if (!e || !dir) return SDNN_ERR_INVALID;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  e->gen.on = false;
  for (int l = 0; l < e->L; ++l) {
    const std::string p = std::string(dir) + "/n" + std::to_string(e->N) + "-l" +
                          std::to_string(l + 1) + ".tsv";
    int rc = read_weight_tsv(p, e->N, e->hw[l], e->err);
    if (rc) return rc;
  }
  e->packed.reset();
  e->weights_dirty = true;
  return SDNN_OK;
}

int sdnn_set_layer_coo(sdnn_engine* e, int32_t layer, const int32_t* rows, const int32_t* cols,
                       const float* vals, int64_t nnz) {
  if (!e) return SDNN_ERR_INVALID;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  if (layer < 0 || layer >= e->L || nnz < 0 || (nnz > 0 && (!rows || !cols || !vals)))
    return fail(e, SDNN_ERR_INVALID, "bad layer or arrays");
  if (e->gen.on) {
    // switching from generated to explicit weights: materialise the others
    e->gen.on = false;
    for (auto& h : e->hw) h.present = false;
  }
  if (e->packed) {
    // switching from a packed file to explicit weights: the other layers are gone
    e->packed.reset();
    for (auto& h : e->hw) h.present = false;
  }
  if (!coo_to_host_layer(e->N, rows, cols, vals, nnz, e->hw[layer], e->err)) return SDNN_ERR_INVALID;
  e->weights_dirty = true;
  return SDNN_OK;
}

int sdnn_set_layer_bias(sdnn_engine* e, int32_t layer, const float* bias) {
  if (!e || !bias) return SDNN_ERR_INVALID;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  if (layer < 0 || layer >= e->L) return fail(e, SDNN_ERR_INVALID, "bad layer");
  if (e->packed)
    return fail(e, SDNN_ERR_STATE, "weights come from a packed file (its biases are part of it)");
  if ((int)e->hbias.size() < e->L) e->hbias.resize(e->L);
  e->hbias[layer].assign(bias, bias + e->N);
  e->weights_dirty = true;
  return SDNN_OK;
}

int sdnn_generate_weights(sdnn_engine* e, uint64_t seed, int32_t nnz_per_row, float value) {
  if (!e) return SDNN_ERR_INVALID;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  if (nnz_per_row < 1 || nnz_per_row > e->N) return fail(e, SDNN_ERR_INVALID, "bad nnz_per_row");
  e->packed.reset();
  e->gen.on = true;
  e->gen.seed = seed;
  e->gen.nnz = nnz_per_row;
  e->gen.value = value;
  e->gen.radix_block = 0;
  for (auto& h : e->hw) h = HostLayer{};
  e->weights_dirty = true;
  return SDNN_OK;
}

int sdnn_generate_radixnet_weights(sdnn_engine* e, int32_t block, float value) {
  if (!e) return SDNN_ERR_INVALID;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  if (!radixnet_shape_ok(e->N, block))
    return fail(e, SDNN_ERR_INVALID,
                "RadiX-Net needs N = block * M with M a power of two, M >= 2");
  e->packed.reset();
  e->gen.on = true;
  e->gen.seed = 0;
  e->gen.nnz = 2 * block;
  e->gen.value = value;
  e->gen.radix_block = block;
  for (auto& h : e->hw) h = HostLayer{};
  e->weights_dirty = true;
  return SDNN_OK;
}

int sdnn_finalize_weights(sdnn_engine* e) {
  if (!e) return SDNN_ERR_INVALID;
  int rc = ensure_cuda(e);
  if (rc) return rc;
  return finalize_weights(e);
}

int sdnn_infer_device(sdnn_engine* e, const float* d_Y0, int64_t rows, int32_t* d_flags,
                      void* stream) {
  if (!e || !d_Y0 || !d_flags || rows <= 0) return SDNN_ERR_INVALID;
  // rows are staged with 1-D TMA bulk copies, which need 16-byte aligned sources
  if (((uintptr_t)d_Y0 & 15u) != 0)
    return fail(e, SDNN_ERR_INVALID, "d_Y0 must be 16-byte aligned");
  int rc = prepare(e, rows);
  if (rc) return rc;
  cudaStream_t user = (cudaStream_t)stream;
  cudaEvent_t joined = nullptr;
  if (user && user != e->stream) {
    // order the engine stream after the caller's stream, then back
    CK(cudaEventCreateWithFlags(&joined, cudaEventDisableTiming));
    CK(cudaEventRecord(joined, user));
    CK(cudaStreamWaitEvent(e->stream, joined, 0));
  }
  rc = run(e, rows, d_Y0, d_flags);
  if (joined) {
    cudaEventRecord(joined, e->stream);
    cudaStreamWaitEvent(user, joined, 0);
    cudaEventDestroy(joined);
  }
  return rc;
}

// First layer of the cross-row part of an inference (a merge step in SNICIT
// mode, else the threshold clustering; L in SNIG mode): the layers before it
// may run piece by piece.  0 when host inputs are not streamed.
//
// With merging the pieces may run past the first merge layer up to a later
// scheduled one, k: the merges before k are skipped and the one after layer
// k - 1 merges everything they would have merged (rows that are equal stay
// equal, and every set of equal rows keeps its smallest row id either way), so
// from layer k on the rows, and all results, are the same bits.
int streamed_prefix(const sdnn_engine* e) {
  if (e->cfg.flags & SDNN_FLAG_NO_STREAMED_INPUT) return 0;
  if (e->cfg.mode != SDNN_MODE_SNIG && e->cfg.mode != SDNN_MODE_SNICIT) return 0;
  const int T = effective_threshold(e);
  int m = T;
  if (merging_on(e)) {
    const int start = e->cfg.merge_start > 0 ? e->cfg.merge_start : kMergeStart;
    const int every = e->cfg.merge_every > 0 ? e->cfg.merge_every : 1;
    if (start < T) {
      m = start;
      while (m + every < T && m + every <= e->cfg.input_prefix_layers) m += every;
    }
  }
  return m;
}

// Swaps the engine's stream, tile tickets and layer-0 fallback list with the
// second lane's (called in pairs around the work of an odd piece).
void swap_lane(sdnn_engine* e) {
  std::swap(e->stream, e->stream2);
  std::swap(e->d_tmask, e->d_tmask2);
  std::swap(e->d_ticket, e->d_ticket2);
  std::swap(e->d_fallback, e->d_fallback2);
  std::swap(e->d_fbcount, e->d_fbcount2);
}

// One inference of n host FP32 rows with the copy streamed in P pieces: the
// pieces are copied back to back on the copy stream, and the compute lanes
// (even and odd pieces) run layers 0 .. m - 1 of piece p as soon as its copy
// has landed (while the later pieces are still copying), then the rest of the
// inference from layer m over all rows (the graphed phases with pipe_start = m).
int run_streamed(sdnn_engine* e, const float* Y0, int64_t n, int m, int P) {
  const int64_t N = e->N;
  const cudaStream_t s = e->stream;
  if (!e->copy_stream) {
    CK(cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&e->stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&e->ingest_free, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&e->lane_ev, cudaEventDisableTiming));
    for (auto& ev : e->piece_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  // the copies overwrite d_in: only after everything enqueued so far
  CK(cudaEventRecord(e->ingest_free, s));
  CK(cudaStreamWaitEvent(e->copy_stream, e->ingest_free, 0));
  // piece boundaries on 32-row tiles; the last piece is half as large as the
  // others: its layers are the ingest work left once the final copy has landed
  int64_t bnd[kMaxPieces + 1];
  const double span = P - 0.5;
  for (int p = 0; p <= P; ++p)
    bnd[p] = p == P ? n : std::min<int64_t>(n, ((int64_t)((double)n * p / span) + 31) / 32 * 32);
  for (int p = 0; p < P; ++p) {
    const int64_t rows = bnd[p + 1] - bnd[p];
    if (rows > 0)
      CK(cudaMemcpyAsync(e->d_in + bnd[p] * N, Y0 + bnd[p] * N, (size_t)(rows * N) * 4,
                         cudaMemcpyHostToDevice, e->copy_stream));
    CK(cudaEventRecord(e->piece_ev[p], e->copy_stream));
  }
  e->launches = 0;
  int rc;
  if ((rc = record(e, 0, false))) return rc;
  launch_set_scalar(e->d_rows, (int32_t)n, s);
  CK(cudaMemsetAsync(e->d_counts, 0, (size_t)(e->L + 4) * 4, s));
  CK(cudaMemsetAsync(e->d_pcounts, 0, (size_t)P * (e->L + 2) * 4, s));  // the layers append
  // identity rows into the pieces' layer-0 lists
  launch_begin_rows(e->d_rows, e->d_plist[0], e->d_counts, e->d_flags, e->d_state, e->d_alias, s);
  e->launches += 2;
  // two lanes: even and odd pieces
  const bool two = true;
  if (two) {
    CK(cudaEventRecord(e->lane_ev, s));
    CK(cudaStreamWaitEvent(e->stream2, e->lane_ev, 0));
  }
  // Pieces of different lanes run at the same time: their rows, list segments
  // and counters are disjoint, and both append to the global list of layer m
  // with atomics.
  for (int p = 0; p < P; ++p) {
    const bool odd = two && (p & 1);
    if (odd) swap_lane(e);
    rc = SDNN_OK;
    const cudaError_t w = cudaStreamWaitEvent(e->stream, e->piece_ev[p], 0);
    if (w == cudaSuccess) rc = enqueue_piece(e, p, bnd[p], bnd[p + 1] - bnd[p], m, e->d_in);
    if (odd) swap_lane(e);
    if (w != cudaSuccess) return cuda_fail(e, w, "cudaStreamWaitEvent");
    if (rc) return rc;
  }
  if (two) {
    CK(cudaEventRecord(e->lane_ev, e->stream2));
    CK(cudaStreamWaitEvent(s, e->lane_ev, 0));
  }
  launch_sum_piece_counts(e->d_pcounts, P, e->L + 2, m, e->d_counts, s);
  e->launches++;
  CK(cudaGetLastError());
  const int prefix_launches = e->launches;
  e->pipe_start = m;
  e->last_pieces = P;
  rc = run(e, n, e->d_in, e->d_flags);
  e->pipe_start = 0;
  if (rc) return rc;
  e->launches += prefix_launches;  // run() counted its own launches only
  return SDNN_OK;
}

// Host inference over batches of cfg.batch rows; inputs as FP32 rows, or as
// one-bit rows (bits != nullptr) expanded on the device.
int infer_host(sdnn_engine* e, const float* Y0, const uint64_t* bits, int64_t rows, int32_t* flags,
               int32_t* ids, int64_t* count) {
  int rc = prepare(e, std::min<int64_t>(rows, e->cfg.batch));
  if (rc) return rc;
  const int64_t N = e->N;
  const int64_t W = (N + 63) / 64;
  if (bits && e->inbits_cap < e->cap) {
    dfree(e->d_inbits);
    CK(cudaMalloc((void**)&e->d_inbits, (size_t)e->cap * W * 8));
    e->inbits_cap = e->cap;
  }
  int64_t total = 0;
  sdnn_stats acc{};
  const int m = bits ? 0 : streamed_prefix(e);
  const int64_t piece_rows =
      e->cfg.input_piece_rows > 0 ? e->cfg.input_piece_rows
                                  : std::clamp<int64_t>(kDefaultPieceBytes / (4 * N), kMinPieceRows,
                                                        kMaxPieceRows);
  for (int64_t off = 0; off < rows; off += e->cfg.batch) {
    const int64_t n = std::min<int64_t>(e->cfg.batch, rows - off);
    const int P = m > 0 ? (int)std::min<int64_t>(kMaxPieces, (n + piece_rows - 1) / piece_rows) : 1;
    if (bits) {
      CK(cudaMemcpyAsync(e->d_inbits, bits + off * W, (size_t)(n * W) * 8, cudaMemcpyHostToDevice,
                         e->stream));
      launch_expand_bits(e->d_inbits, n, e->N, e->d_in, e->stream);
      CK(cudaGetLastError());
      rc = run(e, n, e->d_in, e->d_flags);
    } else if (P > 1) {
      rc = run_streamed(e, Y0 + off * N, n, m, P);
    } else {
      CK(cudaMemcpyAsync(e->d_in, Y0 + off * N, (size_t)(n * N) * 4, cudaMemcpyHostToDevice,
                         e->stream));
      rc = run(e, n, e->d_in, e->d_flags);
    }
    if (rc) return rc;
    if (ids || count) {
      launch_flags_to_ids(e->d_flags, (int32_t)n, e->d_ids, e->d_idcount, e->stream);
      int32_t c = 0;
      CK(cudaMemcpyAsync(&c, e->d_idcount, 4, cudaMemcpyDeviceToHost, e->stream));
      CK(cudaStreamSynchronize(e->stream));
      if (ids && c > 0) {
        CK(cudaMemcpyAsync(ids + total, e->d_ids, (size_t)c * 4, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        for (int32_t i = 0; i < c; ++i) ids[total + i] += (int32_t)off;
      }
      total += c;
    }
    if (flags)
      CK(cudaMemcpyAsync(flags + off, e->d_flags, (size_t)n * 4, cudaMemcpyDeviceToHost, e->stream));
    rc = check_device_error(e);
    if (rc) return rc;
    rc = collect_stats(e);
    if (rc) return rc;
    if (off == 0) {
      acc = e->stats;  // settings of the run (threshold, tile, merge, post path, ...)
      continue;
    }
    for (int i = 0; i < 4; ++i) acc.stage_ms[i] += e->stats.stage_ms[i];
    acc.total_ms += e->stats.total_ms;
    acc.rows_in += e->stats.rows_in;
    acc.row_layers += e->stats.row_layers;
    acc.pre_row_layers += e->stats.pre_row_layers;
    acc.post_row_layers += e->stats.post_row_layers;
    acc.centroids = e->stats.centroids;
    acc.residue_rows += e->stats.residue_rows;
    acc.launches += e->stats.launches;
  }
  acc.rows_out = total;
  e->stats = acc;
  if (count) *count = total;
  return SDNN_OK;
}

int sdnn_infer_host(sdnn_engine* e, const float* Y0, int64_t rows, int32_t* flags, int32_t* ids,
                    int64_t* count) {
  if (!e || !Y0 || rows <= 0) return SDNN_ERR_INVALID;
  return infer_host(e, Y0, nullptr, rows, flags, ids, count);
}

int sdnn_infer_host_bits(sdnn_engine* e, const uint64_t* bits, int64_t rows, int32_t* flags,
                         int32_t* ids, int64_t* count) {
  if (!e || !bits || rows <= 0) return SDNN_ERR_INVALID;
  if (e->N % 4) return fail(e, SDNN_ERR_UNSUPPORTED, "one-bit inputs need N % 4 == 0");
  return infer_host(e, nullptr, bits, rows, flags, ids, count);
}

int sdnn_infer_batches_host(sdnn_engine* e, const float* const* inputs, const int64_t* rows,
                            int32_t num_batches, int32_t* const* flags) {
  if (!e || !inputs || !rows || num_batches <= 0) return SDNN_ERR_INVALID;
  int64_t total = 0;
  for (int32_t b = 0; b < num_batches; ++b) {
    if (rows[b] < 0 || (rows[b] > 0 && !inputs[b])) return fail(e, SDNN_ERR_INVALID, "bad batch");
    total += rows[b];
  }
  if (total <= 0) return fail(e, SDNN_ERR_INVALID, "no rows");
  if (total > e->cfg.batch)
    return fail(e, SDNN_ERR_INVALID, "batches exceed the engine's batch capacity");
  int rc = prepare(e, total);
  if (rc) return rc;
  const int64_t N = e->N;
  // gather the batches back to back into the engine's input rows
  int64_t off = 0;
  for (int32_t b = 0; b < num_batches; ++b) {
    if (rows[b] > 0)
      CK(cudaMemcpyAsync(e->d_in + off * N, inputs[b], (size_t)(rows[b] * N) * 4,
                         cudaMemcpyHostToDevice, e->stream));
    off += rows[b];
  }
  rc = run(e, total, e->d_in, e->d_flags);
  if (rc) return rc;
  off = 0;
  for (int32_t b = 0; b < num_batches; ++b) {
    if (flags && flags[b] && rows[b] > 0)
      CK(cudaMemcpyAsync(flags[b], e->d_flags + off, (size_t)rows[b] * 4, cudaMemcpyDeviceToHost,
                         e->stream));
    off += rows[b];
  }
  rc = check_device_error(e);
  if (rc) return rc;
  return collect_stats(e);
}

int sdnn_infer_batches_device(sdnn_engine* e, const float* const* d_inputs, const int64_t* rows,
                              int32_t num_batches, int32_t* const* d_flags, void* stream) {
  if (!e || !d_inputs || !rows || !d_flags || num_batches <= 0) return SDNN_ERR_INVALID;
  int64_t total = 0;
  for (int32_t b = 0; b < num_batches; ++b) {
    if (rows[b] < 0 || (rows[b] > 0 && (!d_inputs[b] || !d_flags[b])))
      return fail(e, SDNN_ERR_INVALID, "bad batch");
    total += rows[b];
  }
  if (total <= 0) return fail(e, SDNN_ERR_INVALID, "no rows");
  int rc = prepare(e, total);
  if (rc) return rc;
  cudaStream_t user = (cudaStream_t)stream;
  cudaEvent_t joined = nullptr;
  if (user && user != e->stream) {
    CK(cudaEventCreateWithFlags(&joined, cudaEventDisableTiming));
    CK(cudaEventRecord(joined, user));
    CK(cudaStreamWaitEvent(e->stream, joined, 0));
  }
  const int64_t N = e->N;
  int64_t off = 0;
  for (int32_t b = 0; b < num_batches; ++b) {
    if (rows[b] > 0)
      CK(cudaMemcpyAsync(e->d_in + off * N, d_inputs[b], (size_t)(rows[b] * N) * 4,
                         cudaMemcpyDeviceToDevice, e->stream));
    off += rows[b];
  }
  rc = run(e, total, e->d_in, e->d_flags);
  if (rc == SDNN_OK) {
    off = 0;
    for (int32_t b = 0; b < num_batches; ++b) {
      if (rows[b] > 0) {
        const cudaError_t ce = cudaMemcpyAsync(d_flags[b], e->d_flags + off, (size_t)rows[b] * 4,
                                               cudaMemcpyDeviceToDevice, e->stream);
        if (ce != cudaSuccess) {
          rc = cuda_fail(e, ce, "cudaMemcpyAsync");
          break;
        }
      }
      off += rows[b];
    }
  }
  if (joined) {
    cudaEventRecord(joined, e->stream);
    cudaStreamWaitEvent(user, joined, 0);
    cudaEventDestroy(joined);
  }
  return rc;
}

int sdnn_read_activations(sdnn_engine* e, float* out, int64_t rows) {
  if (!e || !out) return SDNN_ERR_INVALID;
  if (!e->have_run) return fail(e, SDNN_ERR_STATE, "no inference has run");
  if (rows <= 0 || rows > e->last_rows)
    return fail(e, SDNN_ERR_INVALID, "rows exceed the last batch");
  cudaSetDevice(e->dev);
  const int L = e->L;
  float* scratch = e->d_y[L & 1];
  launch_materialize(e->d_y[(L - 1) & 1], e->d_state, e->d_cslot, e->d_clist, e->d_iscent,
                     e->d_resflag, e->d_alias, e->d_perm_final, e->N, scratch, (int32_t)rows,
                     e->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, scratch, (size_t)rows * e->N * 4, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  // the scratch buffer is the next inference's layer buffer; nothing to restore
  return SDNN_OK;
}

int sdnn_get_stats(const sdnn_engine* ce, sdnn_stats* out) {
  if (!ce || !out) return SDNN_ERR_INVALID;
  auto* e = const_cast<sdnn_engine*>(ce);
  if (e->pending_stats) {
    cudaSetDevice(e->dev);
    int rc = collect_stats(e);
    if (rc) return rc;
  }
  *out = e->stats;
  return SDNN_OK;
}

int sdnn_save_packed_weights(sdnn_engine* e, const char* path) {
  if (!e || !path) return SDNN_ERR_INVALID;
  const int32_t scale = slot_index_in_bytes(e->Q) ? 4 : 1;
  PackedWriter w;
  if (e->packed) {
    const PackedFile& pf = *e->packed;
    if (!w.begin(path, pf.N, pf.L, pf.Q, pf.nq, pf.G, pf.placed, pf.scale, e->err))
      return SDNN_ERR_IO;
    for (int l = 0; l < pf.L; ++l)
      if (!w.layer(pf.layers[l], pf.N, pf.G, pf.nq, pf.placed, e->err)) return SDNN_ERR_IO;
    return w.end(e->err) ? SDNN_OK : SDNN_ERR_IO;
  }
  if (!e->gen.on) {
    if ((int)e->hw.size() != e->L) return fail(e, SDNN_ERR_STATE, "weights not loaded");
    for (int l = 0; l < e->L; ++l)
      if (!e->hw[l].present)
        return fail(e, SDNN_ERR_STATE, "layer " + std::to_string(l) + " has no weights");
  }
  const bool place = !(e->cfg.flags & SDNN_FLAG_NO_PLACEMENT);
  int rc;
  if (place) {
    if ((rc = compute_placement(e))) return rc;
  } else {
    e->pos.clear();
  }
  if (!w.begin(path, e->N, e->L, e->Q, e->nq, e->G, place, scale, e->err)) return SDNN_ERR_IO;
  // pack a batch of layers in parallel, write it in order, next batch
  const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  for (int b0 = 0; b0 < e->L; b0 += nt) {
    const int b1 = std::min(e->L, b0 + nt);
    std::vector<PackedLayer> packs(b1 - b0);
    std::vector<int32_t> maxdeg(b1 - b0, 0);
    std::vector<std::string> errs(b1 - b0);
    std::vector<int> rcs(b1 - b0, SDNN_OK);
    std::vector<std::thread> pool;
    for (int l = b0; l < b1; ++l)
      pool.emplace_back([&, l] { rcs[l - b0] = pack_host_layer(e, l, packs[l - b0], maxdeg[l - b0], errs[l - b0]); });
    for (auto& t : pool) t.join();
    for (int l = b0; l < b1; ++l) {
      if (rcs[l - b0]) return fail(e, rcs[l - b0], errs[l - b0]);
      if (!w.layer(view_of(e, l, packs[l - b0], maxdeg[l - b0]), e->N, e->G, e->nq, place, e->err))
        return SDNN_ERR_IO;
    }
  }
  return w.end(e->err) ? SDNN_OK : SDNN_ERR_IO;
}

int sdnn_load_packed_weights(sdnn_engine* e, const char* path) {
  if (!e || !path) return SDNN_ERR_INVALID;
  if (e->share_users.load() > 0)
    return fail(e, SDNN_ERR_STATE, "the weights are in use by a server (destroy it first)");
  std::string err;
  std::shared_ptr<PackedFile> pf = open_packed_file(path, err);
  if (!pf) return fail(e, err.rfind("cannot", 0) == 0 ? SDNN_ERR_IO : SDNN_ERR_FORMAT, err);
  const int32_t scale = slot_index_in_bytes(e->Q) ? 4 : 1;
  if (pf->N != e->N || pf->L != e->L || pf->Q != e->Q || pf->nq != e->nq || pf->G != e->G ||
      pf->scale != scale)
    return fail(e, SDNN_ERR_FORMAT,
                std::string(path) + ": packed for N=" + std::to_string(pf->N) + ", L=" +
                    std::to_string(pf->L) + ", chunk " + std::to_string(pf->Q) +
                    ", not this engine's layout");
  e->packed = pf;
  e->gen.on = false;
  for (auto& h : e->hw) h = HostLayer{};
  e->hbias.clear();
  e->weights_dirty = true;
  return SDNN_OK;
}

int sdnn_selftest_wait_timeout(sdnn_engine* e, int64_t limit_us) {
  if (!e || limit_us <= 0 || limit_us > 10000000) return SDNN_ERR_INVALID;
  int rc = prepare(e, 1);
  if (rc) return rc;
  CK(launch_wait_selftest(e->d_err, (uint64_t)limit_us * 1000ull, e->stream));
  return check_device_error(e);  // SDNN_ERR_TIMEOUT expected; resets the error word
}

int sdnn_set_mode(sdnn_engine* e, int32_t mode, int32_t threshold) {
  if (!e || mode < SDNN_MODE_BF || mode > SDNN_MODE_SNICIT || threshold < 0) return SDNN_ERR_INVALID;
  e->cfg.mode = mode;
  e->cfg.threshold = threshold;
  drop_graph(e);
  return SDNN_OK;
}

int sdnn_set_input_streaming(sdnn_engine* e, int32_t piece_rows) {
  if (!e) return SDNN_ERR_INVALID;
  if (piece_rows < 0) {
    e->cfg.flags |= SDNN_FLAG_NO_STREAMED_INPUT;
  } else {
    e->cfg.flags &= ~SDNN_FLAG_NO_STREAMED_INPUT;
    e->cfg.input_piece_rows = piece_rows;
  }
  return SDNN_OK;
}

int sdnn_get_layer_rows(const sdnn_engine* ce, int64_t* out, int32_t num_layers) {
  if (!ce || !out || num_layers < ce->L) return SDNN_ERR_INVALID;
  auto* e = const_cast<sdnn_engine*>(ce);
  if (!e->have_run) return fail(e, SDNN_ERR_STATE, "no inference has run");
  CK(cudaSetDevice(e->dev));
  CK(cudaStreamSynchronize(e->stream));
  const int L = e->L, T = e->last_T;
  std::vector<int32_t> counts(L + 4), rcounts(L + 4);
  int32_t ccount = 0;
  CK(cudaMemcpy(counts.data(), e->d_counts, (size_t)(L + 4) * 4, cudaMemcpyDeviceToHost));
  for (int l = 0; l < T; ++l) out[l] = counts[l];
  if (T < L) {
    CK(cudaMemcpy(rcounts.data(), e->d_rcounts, (size_t)(L + 4) * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&ccount, e->d_ccount, 4, cudaMemcpyDeviceToHost));
    std::vector<int32_t> scounts(L + 4, 0);
    if (e->sparse_res)
      CK(cudaMemcpy(scounts.data(), e->d_scounts, (size_t)(L + 4) * 4, cudaMemcpyDeviceToHost));
    for (int l = T; l < L; ++l) out[l] = (int64_t)ccount + rcounts[l - T] + scounts[l - T];
  }
  return SDNN_OK;
}

int sdnn_write_weights_tsv(sdnn_engine* e, const char* dir) {
  if (!e || !dir) return SDNN_ERR_INVALID;
  for (int l = 0; l < e->L; ++l) {
    HostLayer tmp;
    const HostLayer* h = host_layer(e, l, tmp);
    if (!h) return fail(e, SDNN_ERR_STATE, "layer " + std::to_string(l) + " has no weights");
    const std::string p =
        std::string(dir) + "/n" + std::to_string(e->N) + "-l" + std::to_string(l + 1) + ".tsv";
    int rc = write_weight_tsv(p, *h, e->N);
    if (rc) return fail(e, rc, "cannot write " + p);
  }
  return SDNN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- internal hooks

// Used by the autotuner (autotune.cpp).
namespace sdnn {
int engine_set_tile(sdnn_engine* e, int tile_rows, int threads) {
  e->cfg.tile_rows = tile_rows;
  e->cfg.threads = threads;
  e->grid = 0;
  drop_graph(e);
  return choose_kernel(e);
}
void engine_set_snicit(sdnn_engine* e, int threshold, int centroids) {
  e->cfg.threshold = threshold;
  if (centroids != e->cfg.num_centroids) {
    e->cfg.num_centroids = centroids;
    if (centroids > e->Kcap) free_buffers(e);  // the centroid buffers hold Kcap rows
  }
  drop_graph(e);
}
// Sparse residue lists on or off (the layout must allow them); returns
// whether they are on.
bool engine_set_sparse(sdnn_engine* e, bool on) {
  const bool want = on && e->sparse_built;
  e->cfg.flags = on ? (e->cfg.flags & ~SDNN_FLAG_DENSE_RESIDUE)
                    : (e->cfg.flags | SDNN_FLAG_DENSE_RESIDUE);
  if (want != e->sparse_res) {
    e->sparse_res = want;
    drop_graph(e);
  }
  return e->sparse_res;
}
void engine_set_merge(sdnn_engine* e, int start, int every, bool on) {
  e->cfg.merge_start = start;
  e->cfg.merge_every = every;
  e->cfg.flags = on ? (e->cfg.flags & ~SDNN_FLAG_NO_MERGE) : (e->cfg.flags | SDNN_FLAG_NO_MERGE);
  drop_graph(e);
}
sdnn_config engine_config(const sdnn_engine* e) { return e->cfg; }

// Fills the weight/shape part of the layer-kernel arguments of `layer` and the
// launch shape, without allocating anything: the weights must already be on
// the device (sdnn_finalize_weights or an earlier inference).
int engine_layer_setup(sdnn_engine* e, int layer, LayerArgs* a, LayerKernelKey* key, int* grid,
                       int* threads, size_t* smem) {
  if (layer < 0 || layer >= e->L) return fail(e, SDNN_ERR_INVALID, "bad layer");
  if (!e->stream || e->weights_dirty || (int)e->dl.size() != e->L)
    return fail(e, SDNN_ERR_STATE, "weights are not on the device: call sdnn_finalize_weights first");
  CK(cudaSetDevice(e->dev));
  if (e->grid == 0) {
    int rc = choose_kernel(e);
    if (rc) return rc;
  }
  const DevLayer& d = e->dl[layer];
  LayerKernelKey k = e->key;
  k.constw = d.constw;
  CK(layer_prepare(k, e->smem));
  *a = LayerArgs{};
  a->w.idx = d.idx;
  a->w.val = d.val;
  a->w.grp_blk = d.grp;
  a->w.bias_vec = d.bias;
  a->w.bias = e->cfg.bias;
  a->w.wconst = d.wconst;
  a->N = e->N;
  a->nq = e->nq;
  a->Q = e->Q;
  a->G = e->G;
  a->epi = EPI_PLAIN;
  a->max_split = e->G;
  a->min_split = e->min_split;
  a->clampv = e->cfg.clamp;
  *key = k;
  *grid = d.constw ? e->grid : e->grid_general;
  *threads = e->threads;
  *smem = e->smem;
  return SDNN_OK;
}
cudaStream_t engine_stream(const sdnn_engine* e) { return e->stream; }

// ---- hooks for the serving loop (serve.cpp)
// The slot engines of a server read the model engine's device weights (one
// copy on the device for every slot): src must have its weights on the device
// and keep them (its weight setters and sdnn_destroy answer SDNN_ERR_STATE
// while share_users > 0).
int engine_share_weights(sdnn_engine* dst, sdnn_engine* src) {
  int rc = ensure_cuda(src);
  if (rc) return rc;
  if ((rc = finalize_weights(src))) return rc;
  if (dst->N != src->N || dst->L != src->L || dst->dev != src->dev)
    return fail(dst, SDNN_ERR_INVALID, "shared weights: another shape or device");
  drop_graph(dst);
  free_weights(dst);
  dst->dl = src->dl;
  dst->pos = src->pos;
  dst->d_perm_final = src->d_perm_final;
  dst->d_layer_table = src->d_layer_table;
  dst->total_nnz = src->total_nnz;
  dst->chain_cap = src->chain_cap;
  dst->chain_wcap8 = src->chain_wcap8;
  dst->chain_wcap16 = src->chain_wcap16;
  dst->weights_owner = src;
  dst->weights_dirty = false;
  src->share_users.fetch_add(1);
  return SDNN_OK;
}
int engine_prepare(sdnn_engine* e, int64_t rows) { return prepare(e, rows); }
float* engine_input(sdnn_engine* e) { return e->d_in; }
int32_t* engine_flags(sdnn_engine* e) { return e->d_flags; }
int engine_run(sdnn_engine* e, int64_t rows) { return run(e, rows, e->d_in, e->d_flags); }
int engine_check(sdnn_engine* e) { return check_device_error(e); }
// Positions of the neurons after the last layer (empty = identity).
std::vector<int32_t> engine_final_positions(const sdnn_engine* e) {
  return e->pos.empty() ? std::vector<int32_t>() : e->pos[e->L - 1];
}
bool engine_head(sdnn_engine* e, const float* Hp, const float* hb, int32_t H, int64_t rows,
                 float* logits, int32_t* argmax) {
  return launch_head(e->d_y[(e->L - 1) & 1], e->d_state, e->d_cslot, e->d_clist, e->d_iscent,
                     e->d_resflag, e->d_alias, Hp, hb, H, e->N, (int32_t)rows, logits, argmax,
                     e->stream);
}
std::string engine_error(const sdnn_engine* e) { return e->err; }
void engine_set_error(sdnn_engine* e, const std::string& msg) { e->err = msg; }
}  // namespace sdnn

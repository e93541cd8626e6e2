/*
 * snicit_gb300.h -- C ABI of the GB300 sparse-DNN inference engine.
 *
 * The engine computes the SDGC recurrence
 *     Y[l+1] = min(max(Y[l] * W[l] + b, 0), clamp)
 * over L sparse layers of N neurons, in one of the reference's four modes
 * (BF, SNIG, XY, SNICIT), and returns the category set: the ids of the
 * samples whose final row has any nonzero entry.
 *
 * Reference interfaces this ABI replaces (paths are inside IDEA-CUHK/SNICIT):
 *   - main/SDGC.cu:13-110             CLI flags -m -n -l -t -b, bias map, dispatch
 *   - src/SDGC/base.hpp:69-141        Base ctor + weight loading (packed CSR)
 *   - src/SDGC/utility.hpp:85-191     TSV -> CSR / dense input loaders
 *   - src/SDGC/BF/BF.hpp:102-124      BF::infer
 *   - src/SDGC/SNIG/SNIG.hpp:100-130  SNIG::infer
 *   - src/SDGC/XY/XY.hpp              XY::infer
 *   - src/SDGC/SNICIT/SNICIT.hpp:87-203  SNICIT::infer
 *   - src/SDGC/utility.hpp:194-212    identify (category per sample)
 * The reference exposes header-only C++ classes whose constructor takes
 * (weight_path, bias, N, L[, threshold]) and whose infer() takes
 * (input_path, golden_path, num_inputs[, batch]); errors there end the
 * process (Safe_Call -> exit) or throw.  Here every call returns an int
 * status (sdnn_status), never exits and takes no locks.  One engine owns one
 * CUDA stream and all of its buffers and must be driven by one host thread at
 * a time; separate engines may run concurrently.
 *
 * All pointers are plain host pointers unless the name says "device".
 */
#ifndef SNICIT_GB300_H
#define SNICIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDNN_ABI_VERSION 3

/* Status codes returned by every entry point. */
typedef enum sdnn_status {
  SDNN_OK = 0,
  SDNN_ERR_INVALID = 1,     /* bad argument or unsupported shape            */
  SDNN_ERR_CUDA = 2,        /* a CUDA runtime call failed                   */
  SDNN_ERR_OOM = 3,         /* device or host allocation failed             */
  SDNN_ERR_IO = 4,          /* a file could not be opened or written        */
  SDNN_ERR_FORMAT = 5,      /* malformed TSV / binary content               */
  SDNN_ERR_STATE = 6,       /* call out of order (e.g. infer before weights) */
  SDNN_ERR_TIMEOUT = 7,     /* a device-side bounded wait gave up           */
  SDNN_ERR_UNSUPPORTED = 8, /* feature not available in this build          */
  SDNN_ERR_BUSY = 9         /* serving: no slot / memory free for a request */
} sdnn_status;

/* Execution modes: the reference's -m values (main/SDGC.cu:15-20). */
typedef enum sdnn_mode {
  SDNN_MODE_BF = 0,     /* plain per-layer kernel, one launch per layer     */
  SDNN_MODE_SNIG = 1,   /* plain kernel, whole layer loop as one CUDA graph */
  SDNN_MODE_XY = 2,     /* plain kernel in a graph, pre/post timing split   */
  SDNN_MODE_SNICIT = 3  /* threshold clustering + residue update + recovery */
} sdnn_mode;

typedef struct sdnn_config {
  int32_t num_neurons;   /* -n  N (multiple of 32)                               */
  int32_t num_layers;    /* -l  L                                                */
  int32_t mode;          /* -m  sdnn_mode                                        */
  int32_t threshold;     /* -t  SNICIT threshold layer (layers < t are plain)    */
  int64_t batch;         /* -b  maximum rows per inference call                   */
  float bias;            /* scalar bias (main/SDGC.cu:49-54 bias_map)             */
  float clamp;           /* upper clamp of the activation (32 in SDGC)            */
  int32_t num_centroids; /* SNICIT centroid candidates (reference: 32)            */
  int32_t autotune;      /* 1: let sdnn_autotune choose threshold/centroids/tile  */
  uint64_t seed;         /* seed of the centroid candidate pick                   */
  int32_t device;        /* CUDA device ordinal                                   */
  int32_t tile_rows;     /* rows per CTA in the layer kernel (0 = automatic)      */
  int32_t threads;       /* threads per CTA in the layer kernel (0 = automatic)   */
  int32_t flags;         /* SDNN_FLAG_* bits (0 = all optimisations on)            */
  int32_t merge_start;   /* SNICIT: first plain layer after which identical rows
                            are merged (0 = automatic)                            */
  int32_t merge_every;   /* ... and then after every merge_every-th layer (0 = 1)  */
  int32_t input_piece_rows; /* host FP32 inputs: rows per copy piece of the streamed
                            ingest (0 = automatic: about 96 MB, 2048..16384 rows)  */
  int32_t input_prefix_layers; /* streamed ingest, SNICIT with merging: the pieces
                            run the layers up to the latest scheduled merge layer
                            <= this (their merges deferred to it; exact, same bits);
                            0 = up to the first merge layer                      */
} sdnn_config;

/* sdnn_config.flags: switch off layout optimisations (results are identical
 * either way; used to compare the paths). */
#define SDNN_FLAG_NO_BINARY_FIRST_LAYER 1  /* float kernel for layer 0 even for 0/1 inputs */
#define SDNN_FLAG_NO_PLACEMENT 2           /* keep neuron order; no degree/bank placement   */
#define SDNN_FLAG_NO_CHAIN 4               /* SNICIT: per-layer post launches even when no  */
                                           /* residue row is left                           */
#define SDNN_FLAG_NO_MERGE 8               /* SNICIT: no merging of bitwise-identical rows  */
                                           /* below the threshold (categories identical;    */
                                           /* the clustering then sees other rows, so       */
                                           /* activations agree within FP32 rounding)       */
#define SDNN_FLAG_NO_CHAIN_STREAM 16       /* chain kernel reads weights from L2 instead  */
                                           /* of streaming them into shared memory        */
#define SDNN_FLAG_NO_GRID_CHAIN 32         /* no grid-wide chain: the cluster chain (or    */
                                           /* per-layer launches where it cannot run)     */
#define SDNN_FLAG_NO_STREAMED_INPUT 64     /* host FP32 inputs: one copy of the whole batch */
                                           /* before the first layer (no piecewise ingest) */
#define SDNN_FLAG_DENSE_RESIDUE 256        /* SNICIT: every residue row stays a dense row    */
                                           /* (no sparse residue lists; categories identical,*/
                                           /* activations within FP32 rounding)            */
#define SDNN_FLAG_HOST_POST_CHOICE 128     /* SNICIT: the host reads back what the          */
                                           /* clustering left and picks the post-threshold  */
                                           /* path (a host sync mid-inference) instead of   */
                                           /* the device choosing it inside one graph       */

/* Per-call statistics (stage split of SNICIT.hpp:351-354,659-664). */
typedef struct sdnn_stats {
  float stage_ms[4];     /* pre-threshold, clustering, post-threshold, recovery */
  float total_ms;        /* device time of the whole inference                 */
  int64_t rows_in;       /* rows submitted                                     */
  int64_t rows_out;      /* size of the category set                           */
  int64_t row_layers;    /* sum over layers of rows processed (plain rows +    */
                         /* centroid + non-empty residue rows)                 */
  int32_t centroids;     /* SNICIT: centroids kept after pruning               */
  int32_t residue_rows;  /* SNICIT: non-empty residue rows at the threshold    */
  int32_t launches;      /* kernel launches of the last inference              */
  int32_t threshold;     /* threshold layer used                               */
  int32_t tile_rows;     /* tile rows used by the layer kernel                 */
  int32_t threads;       /* threads per CTA used by the layer kernel           */
  int32_t input_pieces;  /* host FP32 inputs: copy pieces of the last call (the
                            layers before the first cross-row step ran per piece
                            while later pieces were copied); 0 = not streamed     */
  int64_t pre_row_layers;   /* rows processed by the plain layers (sum)        */
  int64_t post_row_layers;  /* centroid + residue rows of the post layers      */
  int64_t weight_nnz;       /* nonzeros of all L layers                        */
  int32_t centroid_candidates; /* candidates drawn at the threshold (setting)        */
  int32_t merge_start;   /* first layer after which identical rows are merged     */
  int32_t merge_every;   /* ... and the spacing of the following merge steps      */
  int32_t post_kernel;   /* post-threshold path: 0 none, 1 a centroid and a residue
                            launch per layer, 2 cluster chain kernel (weights from
                            L2), 3 cluster chain kernel (weights streamed to shared
                            memory), 4 grid-wide chain kernel                     */
  int32_t device_post_choice; /* SNICIT: 1 when the post-threshold path was chosen on
                            the device (the whole inference one graph launch)     */
  int32_t sparse_residue_rows; /* SNICIT: residue rows at the threshold kept as sparse
                            (position, value) lists (<= max(32, N/32) nonzeros)  */
  int64_t sparse_row_layers;   /* sparse residue rows summed over the post layers   */
} sdnn_stats;

typedef struct sdnn_engine sdnn_engine;

/* ---- lifecycle ---------------------------------------------------------- */

/* Fills *cfg with the reference defaults: N=1024, L=120, mode SNICIT, t=30,
 * batch 60000, bias from the reference bias map, clamp 32, 32 candidates. */
int sdnn_config_default(sdnn_config* cfg);

/* Reference bias per neuron count (main/SDGC.cu:49-54); 0 for unknown N. */
float sdnn_reference_bias(int32_t num_neurons);

/* Replaces the engine constructors (BF.hpp BF::BF, SNICIT.hpp SNICIT::SNICIT). */
int sdnn_create(const sdnn_config* cfg, sdnn_engine** out);
int sdnn_destroy(sdnn_engine* e);

/* Human-readable text of the last error on this engine ("" if none). */
const char* sdnn_last_error(const sdnn_engine* e);
const char* sdnn_status_string(int status);
int sdnn_abi_version(void);
/* sizeof of the public structs, for a binding to check its own layouts:
 * out[0..3] = sdnn_config, sdnn_stats, sdnn_server_config, sdnn_server_stats
 * (at most n entries written).  No CUDA call.  (No counterpart in the
 * reference: its classes are used from C++ directly.) */
int sdnn_abi_sizes(int32_t* out, int32_t n);

/* ---- weights ------------------------------------------------------------ */

/* Reads dir/n{N}-l{l}.tsv for l = 1..L: one "row<TAB>col<TAB>value" line per
 * nonzero, 1-based, row = input neuron, col = output neuron; duplicate
 * entries are summed (Eigen setFromTriplets semantics).
 * Replaces read_weight / tsv_string_to_CSR_packed_array
 * (src/SDGC/utility.hpp:85-157) and Base::_load_weight (src/SDGC/base.hpp:89-141). */
int sdnn_load_weights_tsv(sdnn_engine* e, const char* dir);

/* One layer from 0-based COO triplets (row = input, col = output). */
int sdnn_set_layer_coo(sdnn_engine* e, int32_t layer, const int32_t* rows,
                       const int32_t* cols, const float* vals, int64_t nnz);

/* Per-neuron bias of one layer (the beyond nets, src/beyond/general.hpp:36-72).
 * Without this call every layer uses cfg->bias. */
int sdnn_set_layer_bias(sdnn_engine* e, int32_t layer, const float* bias);

/* Synthetic SDGC-shaped weights: every input row gets nnz_per_row distinct
 * output columns drawn uniformly without replacement, all with `value`.
 * Column draws are a counter-based SplitMix64 stream keyed by
 * (seed, layer, row). */
int sdnn_generate_weights(sdnn_engine* e, uint64_t seed, int32_t nnz_per_row, float value);

/* RadiX-Net-structured weights (Robinett and Kepner, "RadiX-Net: Structured
 * Sparse Matrices for Deep Neural Networks", 2019): a radix-2 topology on
 * M = N / block nodes (M a power of two, M >= 2) Kronecker-multiplied with
 * dense blocks of `block` neurons.  Neuron v is (dense index v / M, node
 * v % M); in layer l every output of node c reads every input of nodes c and
 * c + 2^(l mod log2 M) (mod M), all with `value`: 2 * block in-edges per
 * output and out-edges per input.  block = 16 with value 1/16 is the layout
 * the reference's SNICIT / XY kernels are written for: its HashReorder
 * (src/SDGC/reorder/hash.h:14-22, buckets = M) makes every node's 16 neurons
 * contiguous, and its layers 0 .. log2 M - 1 read node c + 16 * 2^l / 16
 * (src/SDGC/SNICIT/SNICIT.hpp:329-342, src/SDGC/XY/kernel.hpp:12-101).
 * SDNN_ERR_INVALID for other shapes. */
int sdnn_generate_radixnet_weights(sdnn_engine* e, int32_t block, float value);

/* Packs the host weights into the device layout (bank-scheduled slots) and
 * uploads them.  Called implicitly by the first inference. */
int sdnn_finalize_weights(sdnn_engine* e);

/* ---- inference ---------------------------------------------------------- */

/* Host-buffer inference: Y0 is rows x N row-major FP32 on the host.  Copies
 * in, runs the configured mode, copies the category set out.
 *   flags      (optional) rows ints, 1 if the sample survives (identify)
 *   ids        (optional) up to rows ints, sorted 0-based survivor ids
 *   count      (optional) number of survivors
 * Replaces BF::infer / SNIG::infer / XY::infer / SNICIT::infer minus the
 * golden-file check. */
int sdnn_infer_host(sdnn_engine* e, const float* Y0, int64_t rows,
                    int32_t* flags, int32_t* ids, int64_t* count);

/* The same with one-bit input rows (entry j of a row in bit j % 64 of word
 * j / 64, ceil(N / 64) words per row -- the layout of the bit-encoded input
 * files): 32x fewer bytes over the host link for 0/1 inputs such as the SDGC
 * images; the rows are expanded on the device.  N must be a multiple of 4. */
int sdnn_infer_host_bits(sdnn_engine* e, const uint64_t* bits, int64_t rows, int32_t* flags,
                         int32_t* ids, int64_t* count);

/* Device-resident inference on the engine's stream (cudaStream_t passed as
 * void*; NULL = the engine's own).  d_Y0 rows x N FP32 device pointer
 * (16-byte aligned), d_flags rows int32 device pointer.  Every mode enqueues
 * the whole inference without a host synchronisation: SNICIT is one CUDA
 * graph launch in which a one-thread kernel reads how many residue rows and
 * centroids the threshold clustering left and sets the graph's SWITCH node,
 * which picks the post-threshold kernels on the device.  (With
 * SDNN_FLAG_HOST_POST_CHOICE the host reads those counts back instead: one
 * synchronisation after the clustering.)  The call returns once the work is
 * enqueued; sdnn_get_stats waits for it. */
int sdnn_infer_device(sdnn_engine* e, const float* d_Y0, int64_t rows,
                      int32_t* d_flags, void* stream);

/* Several input batches of uneven size in one launch schedule: their rows are
 * gathered back to back and run as one inference (rows are independent, so
 * each batch gets its own category set; in SNICIT mode the clustering spans
 * all batches).  inputs[b] has rows[b] x N floats, flags[b] (optional)
 * receives rows[b] ints.  The total must not exceed cfg.batch.  Replaces the
 * reference's per-batch offset loop (src/SDGC/SNICIT/SNICIT.hpp:121-202) where
 * each batch is a separate inference. */
int sdnn_infer_batches_host(sdnn_engine* e, const float* const* inputs, const int64_t* rows,
                            int32_t num_batches, int32_t* const* flags);
/* Device-pointer variant (inputs and flags in device memory, 16-byte aligned). */
int sdnn_infer_batches_device(sdnn_engine* e, const float* const* d_inputs, const int64_t* rows,
                              int32_t num_batches, int32_t* const* d_flags, void* stream);

/* Inputs read from a reference-format TSV ("sample<TAB>feature<TAB>value",
 * 1-based), rows [row_offset, row_offset + rows) into a host buffer
 * (src/SDGC/utility.hpp:160-191,268-293). */
int sdnn_read_inputs_tsv(const char* path, int32_t num_neurons, int64_t row_offset,
                         int64_t rows, float* out);

/* Final activations of the first `rows` rows of the last inference (at most
 * its row count), rows x N, neuron order of the reference (SNICIT rows are
 * recovered: centroid + residue). */
int sdnn_read_activations(sdnn_engine* e, float* out, int64_t rows);

/* Statistics of the last inference. */
int sdnn_get_stats(const sdnn_engine* e, sdnn_stats* out);

/* Packed-weight files: the packed slot layout and neuron placement of every
 * layer, written once (packing runs on the host, no GPU needed) and loaded
 * with one mmap by later engines of the same N and L, which then skip the
 * packing (seconds per thousand layers at N = 65536).  The reference caches
 * its XY preprocessing the same way (src/SDGC/SNICIT/SNICIT.hpp:127-182).
 * Loading validates every slot index and the placement before upload. */
int sdnn_save_packed_weights(sdnn_engine* e, const char* path);
int sdnn_load_packed_weights(sdnn_engine* e, const char* path);

/* Self-test of failure detection (no reference counterpart; the reference
 * exits on errors, src/SDGC/gpu_lib/gpu_runtime.h:2-17): runs one device wait
 * that nothing completes, bounded by limit_us (<= 10 s), through the same
 * helper every kernel wait uses.  Returns SDNN_ERR_TIMEOUT when the wait ran
 * out as it must; the engine stays usable afterwards. */
int sdnn_selftest_wait_timeout(sdnn_engine* e, int64_t limit_us);

/* Switches the mode (and threshold) of an engine without repacking its
 * weights, e.g. to time the plain path and SNICIT on one resident copy of W.
 * (The reference picks the engine class once, main/SDGC.cu:104-110.) */
int sdnn_set_mode(sdnn_engine* e, int32_t mode, int32_t threshold);

/* Streamed ingest of host FP32 rows (sdnn_infer_host): piece_rows > 0 copies
 * the rows in pieces of that many rows and runs the layers before the first
 * cross-row step on each piece while the next ones copy; 0 = automatic piece
 * size; < 0 = one copy of the whole batch before the first layer.  Results
 * are bitwise the same either way.  (The reference reads the whole input
 * before its first layer, src/SDGC/SNICIT/SNICIT.hpp:298.) */
int sdnn_set_input_streaming(sdnn_engine* e, int32_t piece_rows);

/* Rows processed by every layer of the last inference (plain rows for layers
 * below the threshold -- one per set of merged identical rows in SNICIT mode
 * --, centroid + non-empty residue rows above it); out has
 * room for num_layers entries.  (The reference prints these counts only as
 * debugging output, src/SDGC/XY/XY.hpp:481.) */
int sdnn_get_layer_rows(const sdnn_engine* e, int64_t* out, int32_t num_layers);

/* One plain layer (bias + ReLU + clamp) of an engine whose weights are already
 * on the device, applied to `rows` caller-owned rows: d_y_in (rows x N FP32,
 * 16-byte aligned) -> d_y_out (rows x N), d_alive[r] = 1 if row r has an
 * output > 0, else 0.  Allocates no memory at all; has no counterpart in the
 * reference.  For callers that cannot call cudaMalloc (during CUDA-graph
 * capture, fixed-budget or real-time serving threads, hosts whose allocator
 * belongs to another framework).  Its scratch is a static device array for
 * at most 65536 rows (larger `rows` -> SDNN_ERR_INVALID), shared by all calls
 * on a device: calls that overlap on the GPU race.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); make it before
 * any stream capture.  d_y_in and d_y_out must not overlap (SDNN_ERR_INVALID):
 * the layer is not computed in place.  Rows are in the engine's storage order:
 * neuron order for layer 0's input, and for every layer when the engine was
 * created with SDNN_FLAG_NO_PLACEMENT.  Requires sdnn_finalize_weights (or an
 * inference) first; stream NULL = the engine's stream; does not synchronise;
 * the caller's current device is left as it was.  Failure on the device: if a
 * bounded device wait of the layer gives up, every d_alive entry is -1 after
 * the call's work has run (check it once the stream is synchronised). */
int sdnn_layer_noalloc(sdnn_engine* e, int32_t layer, const float* d_y_in, float* d_y_out,
                       int64_t rows, int32_t* d_alive, void* stream);

/* Self-test of sdnn_layer_noalloc's failure report (no reference counterpart):
 * runs its call sequence with the layer replaced by a device wait that nothing
 * completes (bounded by limit_us <= 10 s), so every d_alive entry (rows of
 * them) must read -1 afterwards; the engine and the scratch stay usable. */
int sdnn_selftest_noalloc_timeout(sdnn_engine* e, int32_t* d_alive, int64_t rows,
                                  int64_t limit_us, void* stream);

/* Chooses threshold, centroid count and tile shape by timing the candidates
 * on the given sample rows (host buffer) and appends one JSON line per tried
 * setting to record_path (if not NULL).  Applies the fastest setting. */
int sdnn_autotune(sdnn_engine* e, const float* Y0, int64_t rows, const char* record_path);
/* The same on device-resident sample rows (d_Y0: rows x N, 16-byte aligned);
 * SNICIT mode also sweeps the first merge layer of identical rows. */
int sdnn_autotune_device(sdnn_engine* e, const float* d_Y0, int64_t rows,
                         const char* record_path);

/* ---- serving: continuous batching of requests ---------------------------- */

typedef struct sdnn_server sdnn_server;

typedef struct sdnn_server_config {
  int32_t slots;           /* passes in flight: one engine, stream and worker each */
  int32_t head_outputs;    /* width of the dense head after the last layer (0 = none) */
  int64_t max_rows;        /* largest request and largest pass, in rows (0 = 2^20;
                              default 16384)                                        */
  double memory_fraction;  /* share of the device memory free at admission time that
                              slots may grow into (default 0.25)                    */
  int64_t max_pending;     /* queued requests before sdnn_submit answers BUSY       */
  int64_t max_delay_us;    /* batching window: a pass that is not full waits until
                              its oldest request has queued this long (default 0) */
  int32_t max_requests_per_pass; /* 0 = as many as fit; 1 = one request per pass
                                    (the per-request path, for comparison)        */
  int32_t reserved[5];
} sdnn_server_config;

typedef struct sdnn_server_stats {
  int64_t passes, rows, requests, max_rows_in_pass, queued;
  int64_t slot_rows;  /* rows the largest slot's buffers hold now */
  int32_t slots;
  int32_t reserved[7];
} sdnn_server_stats;

int sdnn_server_config_default(sdnn_server_config* cfg);

/* A request server over the network of `model` (an engine with its weights
 * set).  The slot engines read the model's device weights -- one copy on the
 * device for every slot -- so the model must outlive the server and keep its
 * weights: while a server uses them, the model's weight setters and
 * sdnn_destroy answer SDNN_ERR_STATE.  head_w is N x head_outputs (row-major,
 * by neuron), head_b has head_outputs entries: the dense output layer of the
 * beyond nets (src/beyond/general.hpp:74-102).  Requests arrive with
 * sdnn_submit at any time and are admitted, in arrival order, into the first
 * free slot while they fit: a slot takes the rows its buffers hold plus what
 * the device memory free at that moment (cudaMemGetInfo x memory_fraction,
 * less what other slots were just granted) lets it grow by; a request that
 * fits nowhere while no pass runs completes with SDNN_ERR_OOM.  Slots run
 * concurrently.  The reference has no serving loop; its beyond driver runs
 * fixed rounds (src/beyond/SNICIT/SNICIT.hpp:494-641). */
int sdnn_server_create(sdnn_engine* model, const sdnn_server_config* cfg, const float* head_w,
                       const float* head_b, sdnn_server** out);
int sdnn_server_destroy(sdnn_server* sv);
/* The largest admissible request, in rows (max_rows). */
int64_t sdnn_server_capacity(const sdnn_server* sv);
/* Queues `rows` x N host floats (copied); SDNN_ERR_BUSY when the queue is full,
 * SDNN_ERR_INVALID when rows exceed max_rows. */
int sdnn_submit(sdnn_server* sv, const float* rows_host, int64_t rows, uint64_t* request_id);
/* done = 1 when finished, then copies flags (rows), logits (rows x head),
 * argmax (rows) and the submit-to-completion latency in seconds (each
 * optional) and forgets the request. */
int sdnn_poll(sdnn_server* sv, uint64_t id, int32_t* done, int32_t* flags, float* logits,
              int32_t* argmax, double* latency_s);
/* Blocks until the request is finished; same outputs as sdnn_poll. */
int sdnn_wait(sdnn_server* sv, uint64_t id, int32_t* flags, float* logits, int32_t* argmax,
              double* latency_s);
int sdnn_server_get_stats(sdnn_server* sv, sdnn_server_stats* out);

/* ---- synthetic data and reference file formats --------------------------- */

/* Seeded binary inputs: row r has density rho_r = 0.95 * (2nd smallest of 9
 * uniform draws) (mean 0.19) and entries 1 with probability rho_r.  Rows
 * [row_offset, row_offset + rows) of the stream, written to out (rows x N). */
int sdnn_generate_inputs(int32_t num_neurons, uint64_t seed, int64_t row_offset,
                         int64_t rows, float* out);

/* The same rows generated on the current device into d_out (16-byte
 * aligned, num_neurons a multiple of 4), asynchronously on `stream` (a
 * cudaStream_t; NULL = default stream); bitwise equal to the host rows. */
int sdnn_generate_inputs_device(int32_t num_neurons, uint64_t seed, int64_t row_offset,
                                int64_t rows, float* d_out, void* stream);

/* One synthetic layer as COO (rows/cols/vals each num_neurons * nnz_per_row). */
int sdnn_generate_layer_coo(int32_t num_neurons, uint64_t seed, int32_t layer,
                            int32_t nnz_per_row, float value, int32_t* rows,
                            int32_t* cols, float* vals);

/* One RadiX-Net layer (sdnn_generate_radixnet_weights) as COO, input-major,
 * each input's outputs ascending (rows/cols/vals each num_neurons * 2 * block). */
int sdnn_generate_radixnet_layer_coo(int32_t num_neurons, int32_t block, int32_t layer,
                                     float value, int32_t* rows, int32_t* cols, float* vals);

/* Binary input files (no reference counterpart; they replace parsing the
 * input TSV, src/SDGC/utility.hpp:160-191): encoding 0 = FP32 rows, 1 = one
 * bit per entry (0/1 inputs only; SDNN_ERR_INVALID otherwise).  Reads map
 * the file and decode any row window. */
int sdnn_write_inputs_bin(const char* path, const float* Y0, int64_t rows, int32_t num_neurons,
                          int32_t encoding);
int sdnn_inputs_bin_info(const char* path, int32_t* num_neurons, int64_t* rows, int32_t* encoding);
int sdnn_read_inputs_bin(const char* path, int32_t num_neurons, int64_t row_offset, int64_t rows,
                         float* out);

/* Writers for the reference formats: weights dir/n{N}-l{l}.tsv, inputs
 * sparse-images-{N}.tsv, categories one 1-based id per line. */
int sdnn_write_weights_tsv(sdnn_engine* e, const char* dir);
int sdnn_write_inputs_tsv(const char* path, const float* Y0, int64_t rows, int32_t num_neurons);
int sdnn_write_categories_tsv(const char* path, const int32_t* ids, int64_t count);

#ifdef __cplusplus
}
#endif
#endif /* SNICIT_GB300_H */

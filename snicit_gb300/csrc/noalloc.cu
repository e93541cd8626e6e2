// sdnn_layer_noalloc: one plain layer of an existing engine, applied to
// caller-owned device buffers, with no device allocation at call time.
//
// Who needs it: callers that must not call cudaMalloc after start-up --
// code running while a CUDA graph is being captured, serving threads with a
// fixed memory budget or a real-time deadline, or hosts whose allocator is
// owned by another framework.  The engine's own inference paths allocate
// their row buffers on first use; this entry point allocates nothing: the
// caller passes the rows in and out, and the per-row scratch the layer kernel
// needs (row lists, counters, per-tile masks and tickets) lives in one
// file-scope __device__ array of fixed size, kNoAllocMaxRows rows (about
// 1 MB), held by every GPU that loads the library until the process exits.
//
// Failure report without a host read-back: if a bounded device wait of the
// layer kernel gives up, the kernel records it in the scratch's error word
// and the last kernel of the call writes -1 into every d_alive entry, so the
// caller sees the failure in its own output buffer (no synchronisation, no
// allocation).
#include <cstdint>
#include <mutex>
#include <string>

#include "sdnn_internal.h"
#include "snicit_gb300.h"

namespace sdnn {
int engine_layer_setup(sdnn_engine* e, int layer, LayerArgs* a, LayerKernelKey* key, int* grid,
                       int* threads, size_t* smem);
cudaStream_t engine_stream(const sdnn_engine* e);
void engine_set_error(sdnn_engine* e, const std::string& msg);
}  // namespace sdnn

namespace {

constexpr int kNoAllocMaxRows = 65536;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
  int32_t list_in[kNoAllocMaxRows];
  int32_t list_out[kNoAllocMaxRows];
  uint32_t tile_mask[kNoAllocMaxRows + 1];
  int32_t tile_ticket[kNoAllocMaxRows + 1];
  int32_t counts[4];  // [0] rows in, [1] survivors
  int32_t err[4];
};

// Shared by every call on a device; the last call's contents stay there.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device addresses of g_noalloc_scratch, looked up once per device.
std::mutex g_addr_mutex;
NoAllocScratch* g_addr[kMaxDevices] = {};

// Resets the parts of the scratch that must start at zero for this call and
// lists every row.
__global__ void noalloc_prepare_kernel(NoAllocScratch* s, int32_t rows, int32_t tiles) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x)
    s->list_in[i] = i;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= tiles; i += gridDim.x * blockDim.x) {
    s->tile_mask[i] = 0u;
    s->tile_ticket[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    s->counts[0] = rows;
    s->counts[1] = 0;
    s->err[0] = 0;
  }
}

// Writes the survivor flags (d_alive was zeroed before): 1 for every row the
// layer listed -- or -1 for every row when a device wait of the call gave up.
__global__ void noalloc_flags_kernel(const NoAllocScratch* s, int32_t* alive, int32_t rows) {
  const int stride = gridDim.x * blockDim.x;
  if (s->err[0] != 0) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += stride) alive[i] = -1;
    return;
  }
  const int n = s->counts[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) alive[s->list_out[i]] = 1;
}

// Restores the caller's current device when the call returns.
struct DeviceGuard {
  int saved = -1;
  DeviceGuard() {
    if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
  }
  ~DeviceGuard() {
    if (saved >= 0) cudaSetDevice(saved);
  }
};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device: the host-side symbol is only a stand-in and must never be
// passed to a kernel).
int scratch_address(sdnn_engine* e, NoAllocScratch** out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    sdnn::engine_set_error(e, "sdnn_layer_noalloc: no usable current device");
    return SDNN_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (!g_addr[dev]) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess || !p) {
      sdnn::engine_set_error(e, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce));
      return SDNN_ERR_CUDA;
    }
    g_addr[dev] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_addr[dev];
  return SDNN_OK;
}

}  // namespace

extern "C" int sdnn_layer_noalloc(sdnn_engine* e, int32_t layer, const float* d_y_in,
                                  float* d_y_out, int64_t rows, int32_t* d_alive, void* stream) {
  if (!e || !d_y_in || !d_y_out || !d_alive || rows <= 0) return SDNN_ERR_INVALID;
  if (rows > kNoAllocMaxRows) {
    sdnn::engine_set_error(e, "sdnn_layer_noalloc: rows > " + std::to_string(kNoAllocMaxRows) +
                                  " (size of its static scratch)");
    return SDNN_ERR_INVALID;
  }
  if (((uintptr_t)d_y_in & 15u) != 0) {
    sdnn::engine_set_error(e, "sdnn_layer_noalloc: d_y_in must be 16-byte aligned");
    return SDNN_ERR_INVALID;
  }
  DeviceGuard guard;  // engine_layer_setup makes the engine's device current
  sdnn::LayerArgs a;
  sdnn::LayerKernelKey key;
  int grid = 0, threads = 0;
  size_t smem = 0;
  int rc = sdnn::engine_layer_setup(e, layer, &a, &key, &grid, &threads, &smem);
  if (rc) return rc;
  // CTAs that share a tile write one row's outputs while others may still be
  // loading that row: input and output must not overlap
  const uintptr_t in0 = (uintptr_t)d_y_in, out0 = (uintptr_t)d_y_out;
  const uintptr_t bytes = (uintptr_t)rows * (uintptr_t)a.N * sizeof(float);
  if (in0 < out0 + bytes && out0 < in0 + bytes) {
    sdnn::engine_set_error(e, "sdnn_layer_noalloc: d_y_in and d_y_out overlap");
    return SDNN_ERR_INVALID;
  }
  NoAllocScratch* scratch = nullptr;
  rc = scratch_address(e, &scratch);
  if (rc) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : sdnn::engine_stream(e);
  const int tiles = (int)((rows + key.T - 1) / key.T);
  noalloc_prepare_kernel<<<64, 256, 0, s>>>(scratch, (int32_t)rows, tiles);
  a.y_in = d_y_in;
  a.y_out = d_y_out;
  a.list_in = scratch->list_in;
  a.count_in = &scratch->counts[0];
  a.list_out = scratch->list_out;
  a.count_out = &scratch->counts[1];
  a.tile_mask = scratch->tile_mask;
  a.tile_ticket = scratch->tile_ticket;
  a.err = &scratch->err[0];
  cudaError_t ce = sdnn::launch_layer(key, a, grid, threads, smem, s);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(d_alive, 0, (size_t)rows * sizeof(int32_t), s);
  if (ce == cudaSuccess) {
    noalloc_flags_kernel<<<64, 256, 0, s>>>(scratch, d_alive, (int32_t)rows);
    ce = cudaGetLastError();
  }
  if (ce != cudaSuccess) {
    sdnn::engine_set_error(e, std::string("sdnn_layer_noalloc: ") + cudaGetErrorString(ce));
    return SDNN_ERR_CUDA;
  }
  return SDNN_OK;
}

// Self-test of the failure report above: the same call sequence with the
// layer replaced by a device wait that nothing completes (bounded by
// limit_us), so the error word is set exactly as a timed-out layer sets it.
extern "C" int sdnn_selftest_noalloc_timeout(sdnn_engine* e, int32_t* d_alive, int64_t rows,
                                             int64_t limit_us, void* stream) {
  if (!e || !d_alive || rows <= 0 || rows > kNoAllocMaxRows || limit_us <= 0 ||
      limit_us > 10000000)
    return SDNN_ERR_INVALID;
  DeviceGuard guard;
  sdnn::LayerArgs a;
  sdnn::LayerKernelKey key;
  int grid = 0, threads = 0;
  size_t smem = 0;
  int rc = sdnn::engine_layer_setup(e, 0, &a, &key, &grid, &threads, &smem);  // engine's device
  if (rc) return rc;
  NoAllocScratch* scratch = nullptr;
  rc = scratch_address(e, &scratch);
  if (rc) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : sdnn::engine_stream(e);
  noalloc_prepare_kernel<<<64, 256, 0, s>>>(scratch, (int32_t)rows, 0);
  cudaError_t ce = sdnn::launch_wait_selftest(&scratch->err[0], (uint64_t)limit_us * 1000ull, s);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(d_alive, 0, (size_t)rows * sizeof(int32_t), s);
  if (ce == cudaSuccess) {
    noalloc_flags_kernel<<<64, 256, 0, s>>>(scratch, d_alive, (int32_t)rows);
    ce = cudaGetLastError();
  }
  if (ce != cudaSuccess) {
    sdnn::engine_set_error(e, std::string("sdnn_selftest_noalloc_timeout: ") + cudaGetErrorString(ce));
    return SDNN_ERR_CUDA;
  }
  return SDNN_OK;
}

// Device-side generation of the seeded binary inputs: the same SplitMix64
// streams as gen.cpp (integer arithmetic and exact IEEE double products and
// comparisons), so every row is bitwise equal to sdnn_generate_inputs' row.
// Used to place large input batches (tens of GB) on the device without a
// host copy.
#include <cstdint>

#include <cuda_runtime.h>

#include "snicit_gb300.h"

namespace sdnn {
namespace {

__device__ __forceinline__ uint64_t finalize64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;
constexpr uint64_t kKindInputs = 2;

__device__ __forceinline__ uint64_t stream_key(uint64_t seed, uint64_t kind, uint64_t a, uint64_t b) {
  uint64_t k = finalize64(seed + kGolden);
  k = finalize64(k ^ (kind * 0xD1B54A32D192ED03ull + kGolden));
  k = finalize64(k ^ (a * 0xABC98388FB8FAC03ull + kGolden));
  k = finalize64(k ^ (b * 0x8CB92BA72F3D8DD7ull + kGolden));
  return k;
}
__device__ __forceinline__ uint64_t draw(uint64_t key, uint64_t i) {
  return finalize64(key + (i + 1) * kGolden);
}

// One warp per row: lane 0 derives the row density, the warp writes the row
// with 16-byte stores (N % 4 == 0).
__global__ void gen_inputs_kernel(uint64_t seed, int64_t row_offset, int64_t rows, int32_t N,
                                  float* out) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = wid; r < rows; r += nw) {
    const uint64_t key = stream_key(seed, kKindInputs, 0, (uint64_t)(row_offset + r));
    double rho = 0.0;
    if (lane == 0) {
      uint64_t u[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) u[i] = draw(key, (uint64_t)i) >> 11;
      // second smallest of the nine
      uint64_t m1 = ~0ull, m2 = ~0ull;
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        if (u[i] < m1) {
          m2 = m1;
          m1 = u[i];
        } else if (u[i] < m2) {
          m2 = u[i];
        }
      }
      rho = __dmul_rn(0.95, __dmul_rn((double)m2, 1.0 / 9007199254740992.0));
    }
    rho = __shfl_sync(0xffffffffu, rho, 0);
    float4* o = reinterpret_cast<float4*>(out + r * (int64_t)N);
    for (int j4 = lane; j4 < (N >> 2); j4 += 32) {
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint64_t d = draw(key, 9 + (uint64_t)(4 * j4 + q));
        v[q] = __dmul_rn((double)(d >> 11), 1.0 / 9007199254740992.0) < rho ? 1.f : 0.f;
      }
      o[j4] = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
}

}  // namespace
}  // namespace sdnn

extern "C" int sdnn_generate_inputs_device(int32_t num_neurons, uint64_t seed, int64_t row_offset,
                                           int64_t rows, float* d_out, void* stream) {
  if (num_neurons <= 0 || (num_neurons & 3) || rows < 0 || row_offset < 0 || (!d_out && rows > 0) ||
      (reinterpret_cast<uintptr_t>(d_out) & 15))
    return SDNN_ERR_INVALID;
  if (rows == 0) return SDNN_OK;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return SDNN_ERR_CUDA;
  const int64_t blocks = std::min<int64_t>((rows + 7) / 8, (int64_t)sms * 16);
  sdnn::gen_inputs_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      seed, row_offset, rows, num_neurons, d_out);
  return cudaGetLastError() == cudaSuccess ? SDNN_OK : SDNN_ERR_CUDA;
}

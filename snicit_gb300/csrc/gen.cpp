// Seeded synthetic SDGC-shaped data: counter-based SplitMix64 streams
// (Steele, Lea, Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014), so any layer row or input row can be regenerated alone.
// Only integer and IEEE double arithmetic: the same bits on x86 and Arm.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include "snicit_gb300.h"

namespace sdnn {

static inline uint64_t finalize64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

// Key of stream (kind, a, b) under seed.
uint64_t stream_key(uint64_t seed, uint64_t kind, uint64_t a, uint64_t b) {
  uint64_t k = finalize64(seed + kGolden);
  k = finalize64(k ^ (kind * 0xD1B54A32D192ED03ull + kGolden));
  k = finalize64(k ^ (a * 0xABC98388FB8FAC03ull + kGolden));
  k = finalize64(k ^ (b * 0x8CB92BA72F3D8DD7ull + kGolden));
  return k;
}
// i-th 64-bit draw of a stream (SplitMix64 output i+1 from state key).
static inline uint64_t draw(uint64_t key, uint64_t i) { return finalize64(key + (i + 1) * kGolden); }
// Unbiased-enough bounded integer: high 64 bits of u * n (exact for n a power of 2).
static inline uint32_t bounded(uint64_t u, uint32_t n) {
  return (uint32_t)(((unsigned __int128)u * n) >> 64);
}
static inline double unit53(uint64_t u) { return (double)(u >> 11) * (1.0 / 9007199254740992.0); }

enum : uint64_t { kKindWeights = 1, kKindInputs = 2, kKindValues = 3 };

// Columns of input row `row` of `layer`: nnz distinct outputs, draw order.
void gen_row_cols(uint64_t seed, int32_t layer, int32_t row, int32_t N, int32_t nnz,
                  int32_t* cols) {
  const uint64_t key = stream_key(seed, kKindWeights, (uint64_t)layer, (uint64_t)row);
  int have = 0;
  for (uint64_t i = 0; have < nnz; ++i) {
    const int32_t c = (int32_t)bounded(draw(key, i), (uint32_t)N);
    bool dup = false;
    for (int k = 0; k < have; ++k)
      if (cols[k] == c) {
        dup = true;
        break;
      }
    if (!dup) cols[have++] = c;
  }
}

// Input row density: 0.95 * (2nd order statistic of 9 uniforms) ~ 0.95*Beta(2,8),
// mean 0.19, so every entry is 1 with marginal probability 0.19.
double gen_row_density(uint64_t seed, int64_t row) {
  const uint64_t key = stream_key(seed, kKindInputs, 0, (uint64_t)row);
  uint64_t u[9];
  for (int i = 0; i < 9; ++i) u[i] = draw(key, (uint64_t)i) >> 11;
  std::sort(u, u + 9);
  return 0.95 * ((double)u[1] * (1.0 / 9007199254740992.0));
}

void gen_input_row(uint64_t seed, int64_t row, int32_t N, float* out) {
  const uint64_t key = stream_key(seed, kKindInputs, 0, (uint64_t)row);
  const double rho = gen_row_density(seed, row);
  for (int32_t j = 0; j < N; ++j) out[j] = unit53(draw(key, 9 + (uint64_t)j)) < rho ? 1.f : 0.f;
}

// RadiX-Net topology (Robinett and Kepner, "RadiX-Net: Structured Sparse
// Matrices for Deep Neural Networks", IPDPS workshops 2019): a mixed-radix
// topology on M nodes, Kronecker-multiplied with dense blocks of width B, so
// N = B * M.  Here every radix is 2 (M = 2^k) and the k radix layers repeat:
// in layer l, every output of node c reads every input of nodes c and
// c + 2^(l mod k) (mod M).  Neuron v is (dense index v / M, node v % M).
bool radixnet_shape_ok(int32_t N, int32_t block) {
  if (block < 1 || N < 2 * block || N % block != 0) return false;
  const int32_t M = N / block;
  return (M & (M - 1)) == 0;
}

// Outputs fed by input `row` of RadiX-Net layer `layer`: 2 * block columns,
// ascending.
void radixnet_row_cols(int32_t N, int32_t block, int32_t layer, int32_t row, int32_t* cols) {
  const int32_t M = N / block;
  int32_t k = 0;
  while ((1 << k) < M) ++k;
  const int32_t step = 1 << (layer % k);
  const int32_t c = row % M;
  // output nodes whose inputs include node c: c itself and c - step
  int32_t lo = c, hi = (c - step + M) % M;
  if (lo > hi) std::swap(lo, hi);
  int n = 0;
  for (int32_t r = 0; r < block; ++r) {
    cols[n++] = r * M + lo;
    cols[n++] = r * M + hi;
  }
}

}  // namespace sdnn

extern "C" int sdnn_generate_radixnet_layer_coo(int32_t num_neurons, int32_t block, int32_t layer,
                                                float value, int32_t* rows, int32_t* cols,
                                                float* vals) {
  if (!sdnn::radixnet_shape_ok(num_neurons, block) || layer < 0 || !rows || !cols || !vals)
    return SDNN_ERR_INVALID;
  const int32_t k = 2 * block;
  for (int32_t j = 0; j < num_neurons; ++j) {
    const int64_t o = (int64_t)j * k;
    sdnn::radixnet_row_cols(num_neurons, block, layer, j, cols + o);
    for (int32_t i = 0; i < k; ++i) {
      rows[o + i] = j;
      vals[o + i] = value;
    }
  }
  return SDNN_OK;
}

extern "C" int sdnn_generate_inputs(int32_t num_neurons, uint64_t seed, int64_t row_offset,
                                    int64_t rows, float* out) {
  if (num_neurons <= 0 || rows < 0 || row_offset < 0 || (!out && rows > 0)) return SDNN_ERR_INVALID;
  for (int64_t r = 0; r < rows; ++r)
    sdnn::gen_input_row(seed, row_offset + r, num_neurons, out + r * (int64_t)num_neurons);
  return SDNN_OK;
}

extern "C" int sdnn_generate_layer_coo(int32_t num_neurons, uint64_t seed, int32_t layer,
                                       int32_t nnz_per_row, float value, int32_t* rows,
                                       int32_t* cols, float* vals) {
  if (num_neurons <= 0 || nnz_per_row <= 0 || nnz_per_row > num_neurons || layer < 0 || !rows ||
      !cols || !vals)
    return SDNN_ERR_INVALID;
  for (int32_t j = 0; j < num_neurons; ++j) {
    const int64_t o = (int64_t)j * nnz_per_row;
    sdnn::gen_row_cols(seed, layer, j, num_neurons, nnz_per_row, cols + o);
    for (int32_t k = 0; k < nnz_per_row; ++k) {
      rows[o + k] = j;
      vals[o + k] = value;
    }
  }
  return SDNN_OK;
}

// Packed-weight files: the bank-scheduled slot layout of every layer (and the
// neuron placement) as produced by the packer, so a network is packed once and
// later engines load it with one mmap instead of re-packing (the reference
// caches its XY preprocessing the same way, src/SDGC/SNICIT/SNICIT.hpp:127-182).
//
// Layout (little-endian, every array starting on a 64-byte boundary):
//   file header (64 B): magic "SDNNPK01", N, L, Q, nq, G, placed, index scale
//   per layer: layer header (64 B), grp_blk [G*nq+1] i32, idx [nblocks*128] u16,
//              val [nblocks*128] f32 (general layers), bias [N] f32 (neuron
//              order, if any), pos [N] i32 (placement, if placed)
#pragma once
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

namespace sdnn {

// One packed layer, pointing into a PackedLayer or a mapped file.
struct PackedView {
  const int32_t* grp_blk = nullptr;
  const uint16_t* idx = nullptr;
  const float* val = nullptr;    // nullptr when constw
  const float* bias = nullptr;   // neuron order, nullptr = the engine's scalar bias
  const int32_t* pos = nullptr;  // output positions, nullptr = identity
  bool constw = true;
  float wconst = 0.f;
  int64_t nblocks = 0, nnz = 0, slots = 0;
  int32_t max_depth = 0, max_in_degree = 0;
};

struct PackedFile {
  int32_t N = 0, L = 0, Q = 0, nq = 0, G = 0, scale = 1;
  bool placed = false;
  std::vector<PackedView> layers;
  void* base = nullptr;
  size_t size = 0;
  ~PackedFile();
};

// Maps and validates a packed-weight file; nullptr (and err) on failure.
std::shared_ptr<PackedFile> open_packed_file(const std::string& path, std::string& err);

class PackedWriter {
 public:
  bool begin(const std::string& path, int32_t N, int32_t L, int32_t Q, int32_t nq, int32_t G,
             bool placed, int32_t scale, std::string& err);
  bool layer(const PackedView& v, int32_t N, int32_t G, int32_t nq, bool placed, std::string& err);
  bool end(std::string& err);
  ~PackedWriter();

 private:
  bool put(const void* p, size_t bytes);
  FILE* f_ = nullptr;
  size_t off_ = 0;
};

}  // namespace sdnn

// Packed-weight files (layout in packfile.h).
#include "packfile.h"

#include <cstring>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

namespace sdnn {

namespace {

constexpr char kMagic[8] = {'S', 'D', 'N', 'N', 'P', 'K', '0', '1'};
constexpr size_t kAlign = 64;

struct FileHeader {
  char magic[8];
  int32_t N, L, Q, nq, G, placed, scale;
  int32_t reserved[7];
};
struct LayerHeader {
  int32_t constw;
  float wconst;
  int64_t nnz, nblocks, slots;
  int32_t max_depth, max_in_degree, has_bias;
  int32_t reserved[5];
};
static_assert(sizeof(FileHeader) == 64, "file header is 64 bytes");
static_assert(sizeof(LayerHeader) == 64, "layer header is 64 bytes");

size_t pad(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

}  // namespace

PackedFile::~PackedFile() {
  if (base) munmap(base, size);
}

std::shared_ptr<PackedFile> open_packed_file(const std::string& path, std::string& err) {
  const int fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) {
    err = "cannot open " + path;
    return nullptr;
  }
  struct stat st;
  if (fstat(fd, &st) != 0 || st.st_size < (off_t)sizeof(FileHeader)) {
    ::close(fd);
    err = path + ": not a packed-weight file";
    return nullptr;
  }
  void* base = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
  ::close(fd);
  if (base == MAP_FAILED) {
    err = "cannot map " + path;
    return nullptr;
  }
  auto pf = std::make_shared<PackedFile>();
  pf->base = base;
  pf->size = (size_t)st.st_size;
  const char* b = static_cast<const char*>(base);
  FileHeader h;
  std::memcpy(&h, b, sizeof(h));
  if (std::memcmp(h.magic, kMagic, 8) != 0 || h.N <= 0 || h.L <= 0 || h.Q <= 0 || h.nq <= 0 ||
      h.G <= 0 || (int64_t)h.Q * h.nq != h.N || h.G * 32 != h.N) {
    err = path + ": bad header";
    return nullptr;
  }
  pf->N = h.N;
  pf->L = h.L;
  pf->Q = h.Q;
  pf->nq = h.nq;
  pf->G = h.G;
  pf->placed = h.placed != 0;
  pf->scale = h.scale;
  size_t off = sizeof(FileHeader);
  auto take = [&](size_t bytes) -> const char* {
    if (off + bytes > pf->size) return nullptr;
    const char* p = b + off;
    off += pad(bytes);
    return p;
  };
  pf->layers.resize(h.L);
  for (int l = 0; l < h.L; ++l) {
    const char* lh_p = take(sizeof(LayerHeader));
    if (!lh_p) {
      err = path + ": truncated at layer " + std::to_string(l);
      return nullptr;
    }
    LayerHeader lh;
    std::memcpy(&lh, lh_p, sizeof(lh));
    if (lh.nblocks < 0 || lh.nblocks > ((int64_t)1 << 34) || lh.max_depth < 0) {
      err = path + ": bad layer header " + std::to_string(l);
      return nullptr;
    }
    PackedView& v = pf->layers[l];
    v.constw = lh.constw != 0;
    v.wconst = lh.wconst;
    v.nnz = lh.nnz;
    v.nblocks = lh.nblocks;
    v.slots = lh.slots;
    v.max_depth = lh.max_depth;
    v.max_in_degree = lh.max_in_degree;
    const size_t ngrp = (size_t)h.G * h.nq + 1;
    const size_t nslot = (size_t)lh.nblocks * 128;
    const char* g = take(ngrp * 4);
    const char* ix = take(nslot * 2);
    const char* va = v.constw ? b : take(nslot * 4);
    const char* bi = lh.has_bias ? take((size_t)h.N * 4) : b;
    const char* po = pf->placed ? take((size_t)h.N * 4) : b;
    if (!g || !ix || !va || !bi || !po) {
      err = path + ": truncated at layer " + std::to_string(l);
      return nullptr;
    }
    v.grp_blk = reinterpret_cast<const int32_t*>(g);
    v.idx = reinterpret_cast<const uint16_t*>(ix);
    v.val = v.constw ? nullptr : reinterpret_cast<const float*>(va);
    v.bias = lh.has_bias ? reinterpret_cast<const float*>(bi) : nullptr;
    v.pos = pf->placed ? reinterpret_cast<const int32_t*>(po) : nullptr;
    // the offsets must address the slot array
    if (v.grp_blk[0] != 0 || v.grp_blk[ngrp - 1] != lh.nblocks) {
      err = path + ": inconsistent group offsets in layer " + std::to_string(l);
      return nullptr;
    }
    for (size_t i = 1; i < ngrp; ++i)
      if (v.grp_blk[i] < v.grp_blk[i - 1]) {
        err = path + ": inconsistent group offsets in layer " + std::to_string(l);
        return nullptr;
      }
  }
  return pf;
}

bool PackedWriter::put(const void* p, size_t bytes) {
  if (bytes && std::fwrite(p, 1, bytes, f_) != bytes) return false;
  const size_t padded = pad(bytes);
  static const char zeros[kAlign] = {};
  if (padded > bytes && std::fwrite(zeros, 1, padded - bytes, f_) != padded - bytes) return false;
  off_ += padded;
  return true;
}

bool PackedWriter::begin(const std::string& path, int32_t N, int32_t L, int32_t Q, int32_t nq,
                         int32_t G, bool placed, int32_t scale, std::string& err) {
  f_ = std::fopen(path.c_str(), "wb");
  if (!f_) {
    err = "cannot write " + path;
    return false;
  }
  FileHeader h{};
  std::memcpy(h.magic, kMagic, 8);
  h.N = N;
  h.L = L;
  h.Q = Q;
  h.nq = nq;
  h.G = G;
  h.placed = placed ? 1 : 0;
  h.scale = scale;
  if (!put(&h, sizeof(h))) {
    err = "write failed: " + path;
    return false;
  }
  return true;
}

bool PackedWriter::layer(const PackedView& v, int32_t N, int32_t G, int32_t nq, bool placed,
                         std::string& err) {
  LayerHeader lh{};
  lh.constw = v.constw ? 1 : 0;
  lh.wconst = v.wconst;
  lh.nnz = v.nnz;
  lh.nblocks = v.nblocks;
  lh.slots = v.slots;
  lh.max_depth = v.max_depth;
  lh.max_in_degree = v.max_in_degree;
  lh.has_bias = v.bias ? 1 : 0;
  const size_t nslot = (size_t)v.nblocks * 128;
  bool ok = put(&lh, sizeof(lh)) && put(v.grp_blk, ((size_t)G * nq + 1) * 4) &&
            put(v.idx, nslot * 2);
  if (ok && !v.constw) ok = put(v.val, nslot * 4);
  if (ok && v.bias) ok = put(v.bias, (size_t)N * 4);
  if (ok && placed) ok = put(v.pos, (size_t)N * 4);
  if (!ok) err = "write failed";
  return ok;
}

bool PackedWriter::end(std::string& err) {
  const bool ok = f_ && std::fclose(f_) == 0;
  f_ = nullptr;
  if (!ok) err = "write failed";
  return ok;
}

PackedWriter::~PackedWriter() {
  if (f_) std::fclose(f_);
}

}  // namespace sdnn

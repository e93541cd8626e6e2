// Binary input files: the dense row-major FP32 matrix, or one bit per entry
// for 0/1 inputs (the SDGC images), behind a 32-byte header; read with mmap,
// any row window.  They replace parsing the input TSV
// (src/SDGC/utility.hpp:160-191, 268-293), which the reference re-reads for
// every batch.
//
// Header: magic "SDNNIN01", int32 N, int32 encoding (0 = f32, 1 = bits),
// int64 rows, int64 reserved.  Rows follow: N floats, or ceil(N / 64) uint64
// words with entry j in bit j % 64 of word j / 64.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "snicit_gb300.h"

namespace {

constexpr char kMagic[8] = {'S', 'D', 'N', 'N', 'I', 'N', '0', '1'};

struct Header {
  char magic[8];
  int32_t N, encoding;
  int64_t rows, reserved;
};
static_assert(sizeof(Header) == 32, "input header is 32 bytes");

size_t row_bytes(int32_t N, int32_t enc) {
  return enc == 1 ? (size_t)((N + 63) / 64) * 8 : (size_t)N * 4;
}

struct Mapped {
  void* base = nullptr;
  size_t size = 0;
  ~Mapped() {
    if (base) munmap(base, size);
  }
};

int map_file(const char* path, Mapped& m, Header& h) {
  const int fd = ::open(path, O_RDONLY);
  if (fd < 0) return SDNN_ERR_IO;
  struct stat st;
  if (fstat(fd, &st) != 0 || st.st_size < (off_t)sizeof(Header)) {
    ::close(fd);
    return SDNN_ERR_FORMAT;
  }
  m.base = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
  ::close(fd);
  if (m.base == MAP_FAILED) {
    m.base = nullptr;
    return SDNN_ERR_IO;
  }
  m.size = (size_t)st.st_size;
  std::memcpy(&h, m.base, sizeof(h));
  if (std::memcmp(h.magic, kMagic, 8) != 0 || h.N <= 0 || (h.encoding != 0 && h.encoding != 1) ||
      h.rows < 0 ||
      sizeof(Header) + (size_t)h.rows * row_bytes(h.N, h.encoding) > m.size)
    return SDNN_ERR_FORMAT;
  return SDNN_OK;
}

}  // namespace

extern "C" int sdnn_write_inputs_bin(const char* path, const float* Y0, int64_t rows, int32_t N,
                                     int32_t encoding) {
  if (!path || (!Y0 && rows > 0) || rows < 0 || N <= 0 || (encoding != 0 && encoding != 1))
    return SDNN_ERR_INVALID;
  if (encoding == 1)
    for (int64_t i = 0; i < rows * (int64_t)N; ++i)
      if (Y0[i] != 0.f && Y0[i] != 1.f) return SDNN_ERR_INVALID;  // bits hold 0/1 only
  FILE* f = std::fopen(path, "wb");
  if (!f) return SDNN_ERR_IO;
  Header h{};
  std::memcpy(h.magic, kMagic, 8);
  h.N = N;
  h.encoding = encoding;
  h.rows = rows;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  if (encoding == 0) {
    ok = ok && (rows == 0 || std::fwrite(Y0, sizeof(float) * N, (size_t)rows, f) == (size_t)rows);
  } else {
    const int64_t W = (N + 63) / 64;
    uint64_t* words = new uint64_t[W];
    for (int64_t r = 0; r < rows && ok; ++r) {
      std::memset(words, 0, sizeof(uint64_t) * W);
      const float* y = Y0 + r * N;
      for (int32_t j = 0; j < N; ++j)
        if (y[j] != 0.f) words[j >> 6] |= 1ull << (j & 63);
      ok = std::fwrite(words, sizeof(uint64_t), (size_t)W, f) == (size_t)W;
    }
    delete[] words;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SDNN_OK : SDNN_ERR_IO;
}

extern "C" int sdnn_inputs_bin_info(const char* path, int32_t* N, int64_t* rows, int32_t* encoding) {
  if (!path) return SDNN_ERR_INVALID;
  Mapped m;
  Header h;
  const int rc = map_file(path, m, h);
  if (rc) return rc;
  if (N) *N = h.N;
  if (rows) *rows = h.rows;
  if (encoding) *encoding = h.encoding;
  return SDNN_OK;
}

extern "C" int sdnn_read_inputs_bin(const char* path, int32_t N, int64_t row_offset, int64_t rows,
                                    float* out) {
  if (!path || (!out && rows > 0) || rows < 0 || row_offset < 0 || N <= 0) return SDNN_ERR_INVALID;
  Mapped m;
  Header h;
  const int rc = map_file(path, m, h);
  if (rc) return rc;
  if (h.N != N || row_offset + rows > h.rows) return SDNN_ERR_INVALID;
  const size_t rb = row_bytes(N, h.encoding);
  const char* data = static_cast<const char*>(m.base) + sizeof(Header);
  for (int64_t r = 0; r < rows; ++r) {
    const char* src = data + (size_t)(row_offset + r) * rb;
    float* y = out + r * (int64_t)N;
    if (h.encoding == 0) {
      std::memcpy(y, src, rb);
    } else {
      for (int32_t j = 0; j < N; ++j) {
        uint64_t w;
        std::memcpy(&w, src + (size_t)(j >> 6) * 8, 8);
        y[j] = (w >> (j & 63)) & 1ull ? 1.f : 0.f;
      }
    }
  }
  return SDNN_OK;
}

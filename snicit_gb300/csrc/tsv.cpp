// Reference file formats (src/SDGC/utility.hpp):
//   weights  dir/n{N}-l{l}.tsv          "row<TAB>col<TAB>value", 1-based, l = 1..L
//   inputs   sparse-images-{N}.tsv      "sample<TAB>feature<TAB>value", 1-based
//   golden   neuron{N}-l{L}-categories.tsv   one 1-based sample id per line
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "snicit_gb300.h"
#include "wpack.h"

namespace sdnn {

bool read_file(const std::string& path, std::string& out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  const size_t got = n > 0 ? std::fread(&out[0], 1, (size_t)n, f) : 0;
  std::fclose(f);
  return got == out.size();
}

// Parses "a<ws>b<ws>v" lines. Returns false with line number on malformed input.
static bool parse_triplets(const std::string& s, std::vector<int64_t>& a, std::vector<int64_t>& b,
                           std::vector<float>& v, std::string& err) {
  const char* p = s.c_str();
  const char* end = p + s.size();
  int64_t line = 0;
  while (p < end) {
    ++line;
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p < end && *p == '\n') {
      ++p;
      continue;
    }
    if (p >= end) break;
    char* q;
    errno = 0;
    const long long x = std::strtoll(p, &q, 10);
    if (q == p) goto bad;
    p = q;
    {
      const long long y = std::strtoll(p, &q, 10);
      if (q == p) goto bad;
      p = q;
      const float z = std::strtof(p, &q);
      if (q == p) goto bad;
      p = q;
      a.push_back(x);
      b.push_back(y);
      v.push_back(z);
    }
    while (p < end && *p != '\n') {
      if (*p != ' ' && *p != '\t' && *p != '\r') goto bad;
      ++p;
    }
    if (p < end) ++p;
    continue;
  bad:
    err = "malformed line " + std::to_string(line);
    return false;
  }
  return true;
}

// Reads one weight TSV into a HostLayer (1-based -> 0-based, duplicates summed).
int read_weight_tsv(const std::string& path, int32_t N, HostLayer& out, std::string& err) {
  std::string s;
  if (!read_file(path, s)) {
    err = "cannot open the file " + path;
    return SDNN_ERR_IO;
  }
  std::vector<int64_t> a, b;
  std::vector<float> v;
  if (!parse_triplets(s, a, b, v, err)) {
    err = path + ": " + err;
    return SDNN_ERR_FORMAT;
  }
  std::vector<int32_t> r(a.size()), c(a.size());
  for (size_t k = 0; k < a.size(); ++k) {
    if (a[k] < 1 || a[k] > N || b[k] < 1 || b[k] > N) {
      err = path + ": index out of range on entry " + std::to_string(k + 1);
      return SDNN_ERR_FORMAT;
    }
    r[k] = (int32_t)(a[k] - 1);
    c[k] = (int32_t)(b[k] - 1);
  }
  if (!coo_to_host_layer(N, r.data(), c.data(), v.data(), (int64_t)v.size(), out, err))
    return SDNN_ERR_FORMAT;
  return SDNN_OK;
}

int write_weight_tsv(const std::string& path, const HostLayer& h, int32_t N) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return SDNN_ERR_IO;
  for (int32_t j = 0; j < N; ++j)
    for (int32_t k = h.row_off[j]; k < h.row_off[j + 1]; ++k)
      std::fprintf(f, "%d\t%d\t%.9g\n", j + 1, h.cols[k] + 1, (double)h.vals[k]);
  const bool ok = std::fclose(f) == 0;
  return ok ? SDNN_OK : SDNN_ERR_IO;
}

}  // namespace sdnn

extern "C" int sdnn_read_inputs_tsv(const char* path, int32_t num_neurons, int64_t row_offset,
                                    int64_t rows, float* out) {
  if (!path || num_neurons <= 0 || rows < 0 || row_offset < 0 || (!out && rows > 0))
    return SDNN_ERR_INVALID;
  std::string s, err;
  if (!sdnn::read_file(path, s)) return SDNN_ERR_IO;
  std::vector<int64_t> a, b;
  std::vector<float> v;
  if (!sdnn::parse_triplets(s, a, b, v, err)) return SDNN_ERR_FORMAT;
  std::memset(out, 0, sizeof(float) * (size_t)rows * (size_t)num_neurons);
  for (size_t k = 0; k < a.size(); ++k) {
    if (b[k] < 1 || b[k] > num_neurons || a[k] < 1) return SDNN_ERR_FORMAT;
    const int64_t r = a[k] - 1 - row_offset;
    if (r < 0 || r >= rows) continue;
    out[r * num_neurons + (b[k] - 1)] = v[k];
  }
  return SDNN_OK;
}

extern "C" int sdnn_write_inputs_tsv(const char* path, const float* Y0, int64_t rows,
                                     int32_t num_neurons) {
  if (!path || !Y0 || rows < 0 || num_neurons <= 0) return SDNN_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) return SDNN_ERR_IO;
  for (int64_t r = 0; r < rows; ++r)
    for (int32_t j = 0; j < num_neurons; ++j) {
      const float x = Y0[r * num_neurons + j];
      if (x != 0.f) std::fprintf(f, "%lld\t%d\t%.9g\n", (long long)(r + 1), j + 1, (double)x);
    }
  return std::fclose(f) == 0 ? SDNN_OK : SDNN_ERR_IO;
}

extern "C" int sdnn_write_categories_tsv(const char* path, const int32_t* ids, int64_t count) {
  if (!path || count < 0 || (!ids && count > 0)) return SDNN_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) return SDNN_ERR_IO;
  for (int64_t i = 0; i < count; ++i) std::fprintf(f, "%d\n", ids[i] + 1);
  return std::fclose(f) == 0 ? SDNN_OK : SDNN_ERR_IO;
}

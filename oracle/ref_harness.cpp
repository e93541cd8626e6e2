// Reference-kernel harness -- TEST INFRASTRUCTURE ONLY (never linked into the
// product).  Loads the reference's own bf_inference, snig_inference and
// identify kernels (built from the reference tree by oracle/ref_build.sh into
// oracle/_ref/) and drives them exactly as the reference engines do:
//
//   BF   (src/SDGC/BF/BF.hpp:157-229):  per layer bf_inference over the
//        non-empty row list, host rebuild of the list from rlenY, memset of
//        the consumed buffer; rlenY of layer 0 memset to 1 bytes.
//   SNIG (src/SDGC/SNIG/SNIG.hpp:167-305): per layer snig_inference over the
//        grid (B, num_secs) with per-section non-empty flags (layer-0 flags
//        memset to 1).
//   identify (src/SDGC/utility.hpp:194-212) on the final buffer.
//
// The weights are packed as tsv_string_to_CSR_packed_array does
// (src/SDGC/utility.hpp:85-126): [row_off(N*N_SLAB+1) | cols(max_nnz) |
// vals(max_nnz)], virtual row = input + N * (col / sec_size).
//
// Input file (little endian): int32 N, L, B, sec_size; float bias;
//   per layer: int32 nnz; int32 row_off[N+1]; int32 cols[nnz]; float vals[nnz]
//   (CSR by input row, duplicates summed, columns ascending);
//   float Y0[B*N].
// Output file: float Ybf[B*N]; float Ysnig[B*N]; int32 id_bf[B];
//   int32 id_snig[B]; int32 alive_bf[L] (non-empty rows after each layer).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define DRV(x)                                                              \
  do {                                                                      \
    CUresult r_ = (x);                                                      \
    if (r_ != CUDA_SUCCESS) {                                               \
      const char* s_ = nullptr;                                             \
      cuGetErrorString(r_, &s_);                                            \
      std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x, s_); \
      std::exit(3);                                                         \
    }                                                                       \
  } while (0)
#define RT(x)                                                                                   \
  do {                                                                                          \
    cudaError_t r_ = (x);                                                                       \
    if (r_ != cudaSuccess) {                                                                    \
      std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(r_)); \
      std::exit(3);                                                                             \
    }                                                                                           \
  } while (0)

template <typename T>
static void rd(FILE* f, T* p, size_t n) {
  if (std::fread(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "short read\n");
    std::exit(2);
  }
}

static CUfunction find_kernel(CUmodule mod, const char* needle) {
  unsigned int n = 0;
  DRV(cuModuleGetFunctionCount(&n, mod));
  std::vector<CUfunction> fns(n);
  DRV(cuModuleEnumerateFunctions(fns.data(), n, mod));
  for (CUfunction f : fns) {
    const char* name = nullptr;
    DRV(cuFuncGetName(&name, f));
    if (name && std::strstr(name, needle)) return f;
  }
  std::fprintf(stderr, "kernel %s not found\n", needle);
  std::exit(4);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: ref_harness <module.cubin> <in.bin> <out.bin>\n");
    return 1;
  }
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) return 2;
  int32_t N, L, B, sec;
  float bias;
  rd(f, &N, 1);
  rd(f, &L, 1);
  rd(f, &B, 1);
  rd(f, &sec, 1);
  rd(f, &bias, 1);
  const int nslab = N / sec;
  std::vector<std::vector<int32_t>> ro(L), co(L);
  std::vector<std::vector<float>> vo(L);
  size_t max_nnz = 0;
  for (int l = 0; l < L; ++l) {
    int32_t nnz;
    rd(f, &nnz, 1);
    ro[l].resize(N + 1);
    co[l].resize(nnz);
    vo[l].resize(nnz);
    rd(f, ro[l].data(), N + 1);
    rd(f, co[l].data(), nnz);
    rd(f, vo[l].data(), nnz);
    max_nnz = std::max(max_nnz, (size_t)nnz);
  }
  std::vector<float> Y0((size_t)B * N);
  rd(f, Y0.data(), Y0.size());
  std::fclose(f);

  // packed layout per layer
  const size_t idx_len = (size_t)N * nslab + 1 + max_nnz;
  const size_t wlen = idx_len + max_nnz;
  std::vector<int32_t> packed(wlen * L, 0);
  for (int l = 0; l < L; ++l) {
    int32_t* arr = packed.data() + wlen * l;
    int32_t* roff = arr;
    int32_t* cols = arr + (size_t)N * nslab + 1;
    float* vals = reinterpret_cast<float*>(arr + idx_len);
    std::vector<int32_t> cnt((size_t)N * nslab + 1, 0);
    for (int j = 0; j < N; ++j)
      for (int k = ro[l][j]; k < ro[l][j + 1]; ++k) cnt[(size_t)(co[l][k] / sec) * N + j + 1]++;
    for (size_t v = 0; v < (size_t)N * nslab; ++v) cnt[v + 1] += cnt[v];
    std::memcpy(roff, cnt.data(), cnt.size() * 4);
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int s = 0; s < nslab; ++s)
      for (int j = 0; j < N; ++j)
        for (int k = ro[l][j]; k < ro[l][j + 1]; ++k) {
          if (co[l][k] / sec != s) continue;
          const int32_t p = fill[(size_t)s * N + j]++;
          cols[p] = co[l][k];
          vals[p] = vo[l][k];
        }
  }

  DRV(cuInit(0));
  CUdevice dev;
  DRV(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
  DRV(cuCtxSetCurrent(ctx));
  CUmodule mod;
  DRV(cuModuleLoad(&mod, argv[1]));
  CUfunction k_bf = find_kernel(mod, "bf_inference");
  CUfunction k_snig = find_kernel(mod, "snig_inference");
  CUfunction k_id = find_kernel(mod, "identify");

  int32_t* dW;
  RT(cudaMalloc(&dW, packed.size() * 4));
  RT(cudaMemcpy(dW, packed.data(), packed.size() * 4, cudaMemcpyHostToDevice));
  const size_t ysz = (size_t)B * N * 4;

  // ---------------- BF
  float* Y[2];
  int32_t *rows[2], *rlen[2];
  for (int i = 0; i < 2; ++i) {
    RT(cudaMalloc(&Y[i], ysz));
    RT(cudaMalloc(&rows[i], (size_t)B * 4));
    RT(cudaMalloc(&rlen[i], (size_t)B * 4));
    RT(cudaMemset(rows[i], 0, (size_t)B * 4));
  }
  RT(cudaMemcpy(Y[0], Y0.data(), ysz, cudaMemcpyHostToDevice));
  RT(cudaMemset(Y[1], 0, ysz));
  RT(cudaMemset(rlen[0], 1, (size_t)B * 4));
  RT(cudaMemset(rlen[1], 0, (size_t)B * 4));
  std::vector<int32_t> hrl(B), hrows(B);
  size_t nerows = (size_t)B;
  for (int i = 0; i < B; ++i) hrows[i] = i;
  RT(cudaMemcpy(rows[0], hrows.data(), (size_t)B * 4, cudaMemcpyHostToDevice));
  std::vector<int32_t> alive_bf(L, 0);
  for (int l = 0; l < L; ++l) {
    const int a = l % 2, b = (l + 1) % 2;
    int32_t* roffw = dW + wlen * l;
    int32_t* colsw = roffw + (size_t)N * nslab + 1;
    float* valsw = reinterpret_cast<float*>(roffw + idx_len);
    const float* y0 = Y[a];
    size_t ne = nerows, colblk = (size_t)sec, ns = (size_t)nslab, nn = (size_t)N;
    float bb = bias;
    void* args[] = {&y0, &ne, &rows[a], &rlen[a], &colblk, &ns, &nn, &roffw, &colsw, &valsw, &bb, &Y[b], &rlen[b]};
    if (nerows > 0)
      DRV(cuLaunchKernel(k_bf, (unsigned)nerows, 1, 1, 2, 512, 1, (unsigned)(sec * 4), 0, args, nullptr));
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(hrl.data(), rlen[b], (size_t)B * 4, cudaMemcpyDeviceToHost));
    nerows = 0;
    for (int i = 0; i < B; ++i)
      if (hrl[i] > 0) hrows[nerows++] = i;
    RT(cudaMemcpy(rows[b], hrows.data(), (size_t)B * 4, cudaMemcpyHostToDevice));
    RT(cudaMemset(Y[a], 0, ysz));
    alive_bf[l] = (int32_t)nerows;
  }
  std::vector<float> Ybf((size_t)B * N);
  RT(cudaMemcpy(Ybf.data(), Y[L % 2], ysz, cudaMemcpyDeviceToHost));
  int32_t* dres;
  RT(cudaMalloc(&dres, (size_t)B * 4));
  std::vector<int32_t> id_bf(B), id_snig(B);
  {
    float* yf = Y[L % 2];
    size_t bs = (size_t)B, nn = (size_t)N;
    void* args[] = {&yf, &bs, &nn, &dres};
    DRV(cuLaunchKernel(k_id, 16, 1, 1, 512, 1, 1, 0, 0, args, nullptr));
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(id_bf.data(), dres, (size_t)B * 4, cudaMemcpyDeviceToHost));
  }

  // ---------------- SNIG
  bool* nz[2];
  for (int i = 0; i < 2; ++i) RT(cudaMalloc(&nz[i], (size_t)B * nslab));
  RT(cudaMemcpy(Y[0], Y0.data(), ysz, cudaMemcpyHostToDevice));
  RT(cudaMemset(Y[1], 0, ysz));
  RT(cudaMemset(nz[0], 1, (size_t)B * nslab));
  RT(cudaMemset(nz[1], 0, (size_t)B * nslab));
  for (int l = 0; l < L; ++l) {
    const int a = l % 2, b = (l + 1) % 2;
    int32_t* roffw = dW + wlen * l;
    int32_t* colsw = roffw + (size_t)N * nslab + 1;
    float* valsw = reinterpret_cast<float*>(roffw + idx_len);
    const float* y0 = Y[a];
    const bool* nz0 = nz[a];
    size_t ss = (size_t)sec, ns = (size_t)nslab, nn = (size_t)N;
    float bb = bias;
    void* args[] = {&y0, &nz0, &ss, &ns, &nn, &roffw, &colsw, &valsw, &bb, &nz[b], &Y[b]};
    DRV(cuLaunchKernel(k_snig, (unsigned)B, (unsigned)nslab, 1, 2, 512, 1, (unsigned)(sec * 4), 0, args, nullptr));
    RT(cudaDeviceSynchronize());
  }
  std::vector<float> Ysnig((size_t)B * N);
  RT(cudaMemcpy(Ysnig.data(), Y[L % 2], ysz, cudaMemcpyDeviceToHost));
  {
    float* yf = Y[L % 2];
    size_t bs = (size_t)B, nn = (size_t)N;
    void* args[] = {&yf, &bs, &nn, &dres};
    DRV(cuLaunchKernel(k_id, 16, 1, 1, 512, 1, 1, 0, 0, args, nullptr));
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(id_snig.data(), dres, (size_t)B * 4, cudaMemcpyDeviceToHost));
  }

  FILE* o = std::fopen(argv[3], "wb");
  if (!o) return 2;
  std::fwrite(Ybf.data(), 4, Ybf.size(), o);
  std::fwrite(Ysnig.data(), 4, Ysnig.size(), o);
  std::fwrite(id_bf.data(), 4, id_bf.size(), o);
  std::fwrite(id_snig.data(), 4, id_snig.size(), o);
  std::fwrite(alive_bf.data(), 4, alive_bf.size(), o);
  std::fclose(o);
  std::printf("ok N=%d L=%d B=%d sec=%d alive_last=%d\n", N, L, B, sec, alive_bf[L - 1]);
  return 0;
}

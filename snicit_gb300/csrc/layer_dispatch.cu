// Instance registry and launcher of the layer kernel.
#include <mutex>
#include <vector>
#include "layer_kernel.cuh"

namespace sdnn {

#ifndef SDNN_LAYER_PDL
#define SDNN_LAYER_PDL 1
#endif
constexpr bool kLayerPdl = SDNN_LAYER_PDL;

void register_layer_q1024(std::vector<LayerInstance>& v);
void register_layer_q4096(std::vector<LayerInstance>& v);
void register_layer_q16384(std::vector<LayerInstance>& v);
void register_layer_generic(std::vector<LayerInstance>& v);

static const std::vector<LayerInstance>& registry() {
  static std::vector<LayerInstance> v;
  static std::once_flag once;
  std::call_once(once, [] {
    register_layer_q1024(v);
    register_layer_q4096(v);
    register_layer_q16384(v);
    register_layer_generic(v);
  });
  return v;
}

static const LayerInstance* find(const LayerKernelKey& k) {
  for (const auto& e : registry())
    if (e.T == k.T && e.rsw == k.rsw && e.kg == k.kg && e.constw == k.constw) return &e;
  return nullptr;
}

bool layer_instance_exists(const LayerKernelKey& key) { return find(key) != nullptr; }

cudaError_t layer_prepare(const LayerKernelKey& key, size_t smem) {
  const LayerInstance* e = find(key);
  if (!e) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(e->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int layer_blocks_per_sm(const LayerKernelKey& key, int threads, size_t smem) {
  const LayerInstance* e = find(key);
  if (!e) return 0;
  if (cudaFuncSetAttribute(e->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, e->fn, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

cudaError_t launch_layer(const LayerKernelKey& key, const LayerArgs& a, int grid, int threads,
                         size_t smem, cudaStream_t s) {
  const LayerInstance* e = find(key);
  if (!e) return cudaErrorInvalidValue;
  // programmatic stream serialization: this launch may be scheduled while the
  // previous kernel on the stream finishes (the kernel waits for it with
  // griddepcontrol.wait before touching its outputs)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = kLayerPdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {const_cast<LayerArgs*>(&a)};
  return cudaLaunchKernelExC(&cfg, e->fn, args);
}

}  // namespace sdnn

// Layer kernel instances (T rows per tile, smem row stride, groups per warp).
// The kernel itself lives in layer_kernel.cuh.
#include <vector>
#include "layer_kernel.cuh"

namespace sdnn {

SDNN_LAYER_INSTANCE(1, 16416, 1, false)
SDNN_LAYER_INSTANCE(1, 16416, 1, true)
SDNN_LAYER_INSTANCE(2, 16416, 1, false)
SDNN_LAYER_INSTANCE(2, 16416, 1, true)
SDNN_LAYER_INSTANCE(3, 16416, 1, false)
SDNN_LAYER_INSTANCE(3, 16416, 1, true)
SDNN_LAYER_INSTANCE(1, 16416, 16, false)
SDNN_LAYER_INSTANCE(1, 16416, 16, true)
SDNN_LAYER_INSTANCE(2, 16416, 16, false)
SDNN_LAYER_INSTANCE(2, 16416, 16, true)
SDNN_LAYER_INSTANCE(3, 16416, 16, false)
SDNN_LAYER_INSTANCE(3, 16416, 16, true)
SDNN_LAYER_INSTANCE(1, 16416, 8, false)
SDNN_LAYER_INSTANCE(1, 16416, 8, true)
SDNN_LAYER_INSTANCE(2, 16416, 8, false)
SDNN_LAYER_INSTANCE(2, 16416, 8, true)
SDNN_LAYER_INSTANCE(3, 16416, 8, false)
SDNN_LAYER_INSTANCE(3, 16416, 8, true)
SDNN_LAYER_INSTANCE(1, 32800, 16, false)
SDNN_LAYER_INSTANCE(1, 32800, 16, true)

void register_layer_q16384(std::vector<LayerInstance>& v) {
  v.push_back({1, 16416, 1, false, (const void*)&layer_kernel<1, 16416, 1, false>});
  v.push_back({1, 16416, 1, true, (const void*)&layer_kernel<1, 16416, 1, true>});
  v.push_back({2, 16416, 1, false, (const void*)&layer_kernel<2, 16416, 1, false>});
  v.push_back({2, 16416, 1, true, (const void*)&layer_kernel<2, 16416, 1, true>});
  v.push_back({3, 16416, 1, false, (const void*)&layer_kernel<3, 16416, 1, false>});
  v.push_back({3, 16416, 1, true, (const void*)&layer_kernel<3, 16416, 1, true>});
  v.push_back({1, 16416, 16, false, (const void*)&layer_kernel<1, 16416, 16, false>});
  v.push_back({1, 16416, 16, true, (const void*)&layer_kernel<1, 16416, 16, true>});
  v.push_back({2, 16416, 16, false, (const void*)&layer_kernel<2, 16416, 16, false>});
  v.push_back({2, 16416, 16, true, (const void*)&layer_kernel<2, 16416, 16, true>});
  v.push_back({3, 16416, 16, false, (const void*)&layer_kernel<3, 16416, 16, false>});
  v.push_back({3, 16416, 16, true, (const void*)&layer_kernel<3, 16416, 16, true>});
  v.push_back({1, 16416, 8, false, (const void*)&layer_kernel<1, 16416, 8, false>});
  v.push_back({1, 16416, 8, true, (const void*)&layer_kernel<1, 16416, 8, true>});
  v.push_back({2, 16416, 8, false, (const void*)&layer_kernel<2, 16416, 8, false>});
  v.push_back({2, 16416, 8, true, (const void*)&layer_kernel<2, 16416, 8, true>});
  v.push_back({3, 16416, 8, false, (const void*)&layer_kernel<3, 16416, 8, false>});
  v.push_back({3, 16416, 8, true, (const void*)&layer_kernel<3, 16416, 8, true>});
  v.push_back({1, 32800, 16, false, (const void*)&layer_kernel<1, 32800, 16, false>});
  v.push_back({1, 32800, 16, true, (const void*)&layer_kernel<1, 32800, 16, true>});
}

}  // namespace sdnn

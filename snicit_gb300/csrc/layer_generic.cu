// Layer kernel instances (T rows per tile, smem row stride, groups per warp).
// The kernel itself lives in layer_kernel.cuh.
#include <vector>
#include "layer_kernel.cuh"

namespace sdnn {

SDNN_LAYER_INSTANCE(1, 0, 1, false)
SDNN_LAYER_INSTANCE(1, 0, 1, true)
SDNN_LAYER_INSTANCE(2, 0, 1, false)
SDNN_LAYER_INSTANCE(2, 0, 1, true)
SDNN_LAYER_INSTANCE(4, 0, 1, false)
SDNN_LAYER_INSTANCE(4, 0, 1, true)
SDNN_LAYER_INSTANCE(8, 0, 1, false)
SDNN_LAYER_INSTANCE(8, 0, 1, true)
SDNN_LAYER_INSTANCE(1, 0, 16, false)
SDNN_LAYER_INSTANCE(1, 0, 16, true)

void register_layer_generic(std::vector<LayerInstance>& v) {
  v.push_back({1, 0, 1, false, (const void*)&layer_kernel<1, 0, 1, false>});
  v.push_back({1, 0, 1, true, (const void*)&layer_kernel<1, 0, 1, true>});
  v.push_back({2, 0, 1, false, (const void*)&layer_kernel<2, 0, 1, false>});
  v.push_back({2, 0, 1, true, (const void*)&layer_kernel<2, 0, 1, true>});
  v.push_back({4, 0, 1, false, (const void*)&layer_kernel<4, 0, 1, false>});
  v.push_back({4, 0, 1, true, (const void*)&layer_kernel<4, 0, 1, true>});
  v.push_back({8, 0, 1, false, (const void*)&layer_kernel<8, 0, 1, false>});
  v.push_back({8, 0, 1, true, (const void*)&layer_kernel<8, 0, 1, true>});
  v.push_back({1, 0, 16, false, (const void*)&layer_kernel<1, 0, 16, false>});
  v.push_back({1, 0, 16, true, (const void*)&layer_kernel<1, 0, 16, true>});
}

}  // namespace sdnn

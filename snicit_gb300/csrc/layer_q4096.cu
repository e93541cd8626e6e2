// Layer kernel instances (T rows per tile, smem row stride, groups per warp).
// The kernel itself lives in layer_kernel.cuh.
#include <vector>
#include "layer_kernel.cuh"

namespace sdnn {

SDNN_LAYER_INSTANCE(2, 4128, 1, false)
SDNN_LAYER_INSTANCE(2, 4128, 1, true)
SDNN_LAYER_INSTANCE(3, 4128, 1, false)
SDNN_LAYER_INSTANCE(3, 4128, 1, true)
SDNN_LAYER_INSTANCE(4, 4128, 1, false)
SDNN_LAYER_INSTANCE(4, 4128, 1, true)
SDNN_LAYER_INSTANCE(5, 4128, 1, false)
SDNN_LAYER_INSTANCE(5, 4128, 1, true)
SDNN_LAYER_INSTANCE(6, 4128, 1, false)
SDNN_LAYER_INSTANCE(6, 4128, 1, true)

void register_layer_q4096(std::vector<LayerInstance>& v) {
  v.push_back({2, 4128, 1, false, (const void*)&layer_kernel<2, 4128, 1, false>});
  v.push_back({2, 4128, 1, true, (const void*)&layer_kernel<2, 4128, 1, true>});
  v.push_back({3, 4128, 1, false, (const void*)&layer_kernel<3, 4128, 1, false>});
  v.push_back({3, 4128, 1, true, (const void*)&layer_kernel<3, 4128, 1, true>});
  v.push_back({4, 4128, 1, false, (const void*)&layer_kernel<4, 4128, 1, false>});
  v.push_back({4, 4128, 1, true, (const void*)&layer_kernel<4, 4128, 1, true>});
  v.push_back({5, 4128, 1, false, (const void*)&layer_kernel<5, 4128, 1, false>});
  v.push_back({5, 4128, 1, true, (const void*)&layer_kernel<5, 4128, 1, true>});
  v.push_back({6, 4128, 1, false, (const void*)&layer_kernel<6, 4128, 1, false>});
  v.push_back({6, 4128, 1, true, (const void*)&layer_kernel<6, 4128, 1, true>});
}

}  // namespace sdnn

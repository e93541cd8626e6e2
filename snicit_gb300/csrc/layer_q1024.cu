// Layer kernel instances (T rows per tile, smem row stride, groups per warp).
// The kernel itself lives in layer_kernel.cuh.
#include <vector>
#include "layer_kernel.cuh"

namespace sdnn {

SDNN_LAYER_INSTANCE(8, 1056, 1, false)
SDNN_LAYER_INSTANCE(8, 1056, 1, true)
SDNN_LAYER_INSTANCE(12, 1056, 1, false)
SDNN_LAYER_INSTANCE(12, 1056, 1, true)
SDNN_LAYER_INSTANCE(16, 1056, 1, false)
SDNN_LAYER_INSTANCE(16, 1056, 1, true)
SDNN_LAYER_INSTANCE(24, 1056, 1, false)
SDNN_LAYER_INSTANCE(24, 1056, 1, true)

void register_layer_q1024(std::vector<LayerInstance>& v) {
  v.push_back({8, 1056, 1, false, (const void*)&layer_kernel<8, 1056, 1, false>});
  v.push_back({8, 1056, 1, true, (const void*)&layer_kernel<8, 1056, 1, true>});
  v.push_back({12, 1056, 1, false, (const void*)&layer_kernel<12, 1056, 1, false>});
  v.push_back({12, 1056, 1, true, (const void*)&layer_kernel<12, 1056, 1, true>});
  v.push_back({16, 1056, 1, false, (const void*)&layer_kernel<16, 1056, 1, false>});
  v.push_back({16, 1056, 1, true, (const void*)&layer_kernel<16, 1056, 1, true>});
  v.push_back({24, 1056, 1, false, (const void*)&layer_kernel<24, 1056, 1, false>});
  v.push_back({24, 1056, 1, true, (const void*)&layer_kernel<24, 1056, 1, true>});
}

}  // namespace sdnn

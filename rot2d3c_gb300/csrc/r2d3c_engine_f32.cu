// FP32 engine instantiation (FP32 transforms with compensated twiddles, FP64
// reductions).
#include "r2d3c_engine_impl.cuh"

namespace r2d3c {
IEngine* make_engine_f32(int n, int device, bool full, int nb) {
  return new EngineT<float>(n, device, full, nb);
}
}  // namespace r2d3c

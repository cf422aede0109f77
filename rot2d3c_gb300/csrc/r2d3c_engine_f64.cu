// FP64 (drop-in) engine instantiation.
#include "r2d3c_engine_impl.cuh"

namespace r2d3c {
IEngine* make_engine_f64(int n, int device, bool full, int nb) {
  return new EngineT<double>(n, device, full, nb);
}
}  // namespace r2d3c

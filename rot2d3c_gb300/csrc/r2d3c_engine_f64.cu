// FP64 (drop-in) engine instantiation.
#include "r2d3c_engine_impl.cuh"

namespace r2d3c {
IEngine* make_engine_f64(int n, int device, bool full) { return new EngineT<double>(n, device, full); }
}  // namespace r2d3c

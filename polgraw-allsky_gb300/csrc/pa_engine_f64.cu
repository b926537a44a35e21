// pa_engine_f64.cu -- the all-FP64 engine (every stage in double precision),
// the comparison form of the same kernels.
#include "pa_engine.cuh"

namespace pa {
Engine* make_engine_f64(const Buffers& b) { return new EngineT<double, PM_F64>(b); }
}  // namespace pa

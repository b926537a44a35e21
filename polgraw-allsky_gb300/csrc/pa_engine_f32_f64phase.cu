// pa_engine_f32_f64phase.cu -- mixed-precision engine with the spindown
// phase evaluated in FP64 per sample.
#include "pa_engine.cuh"

namespace pa {
Engine* make_engine_f32_f64phase(const Buffers& b) { return new EngineT<float, PM_F64>(b); }
}  // namespace pa

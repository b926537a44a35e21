// pa_engine_f32_ffphase.cu -- mixed-precision engine with the compensated
// two-float spindown phase.
#include "pa_engine.cuh"

namespace pa {
Engine* make_engine_f32_ffphase(const Buffers& b) { return new EngineT<float, PM_FF>(b); }
}  // namespace pa

// pa_engine_f32.cu -- mixed-precision engines (FP32 data, FFTs and
// F-statistic; FP64 time shifts, prelude phase and spline solve), one per
// spindown-phase form.
#include "pa_engine.cuh"

namespace pa {
Engine* make_engine_f32(const Buffers& b, int phase_mode) {
  switch (phase_mode) {
    case PM_FIXED: return new EngineT<float, PM_FIXED>(b);
    case PM_FF: return new EngineT<float, PM_FF>(b);
    default: return new EngineT<float, PM_F64>(b);
  }
}
}  // namespace pa

// pa_engine_f32.cu -- mixed-precision engine (FP32 data, FFTs and
// F-statistic; FP64 time shifts, prelude phase and spline solve) with the
// fixed-point spindown phase.  The other phase forms live in their own
// translation units so that they compile in parallel.
#include <new>

#include "pa_engine.cuh"

namespace pa {
Engine* make_engine_f32_f64phase(const Buffers& b);
Engine* make_engine_f32_ffphase(const Buffers& b);

// The fixed-point-phase engine constructed in caller-provided storage (no
// allocation); returns nullptr if the storage is too small.
Engine* make_engine_f32_fixed_at(void* mem, size_t bytes, const Buffers& b) {
  if (bytes < sizeof(EngineT<float, PM_FIXED>)) return nullptr;
  return new (mem) EngineT<float, PM_FIXED>(b);
}

Engine* make_engine_f32(const Buffers& b, int phase_mode) {
  switch (phase_mode) {
    case PM_FIXED: return new EngineT<float, PM_FIXED>(b);
    case PM_FF: return make_engine_f32_ffphase(b);
    default: return make_engine_f32_f64phase(b);
  }
}
}  // namespace pa

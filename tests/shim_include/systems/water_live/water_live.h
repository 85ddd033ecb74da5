// A stand-in for the engine's systems/water_live/water_live.h that declares only what the CUDA
// binding (include/wlcuda_device_step.hpp) reads: Ops, StepOptions, WaterPartial, WaterLedger and
// Ledger, with the reference's fields, sizes and order (water_live.h:57-150). The engine's own
// header also pulls in the gfx device layer, whose generated code the reference's tree does not
// hold, so the binding's test compiles against this one. Test support only.
#pragma once

#include <core/base/types.h>

namespace engine::water_live {

enum class Ops : u8 { native = 0, fixed = 1 };

struct StepOptions {
  Ops ops = Ops::native;
  bool stored_faces = false;
};

struct WaterPartial {
  f32 speed_x = 0.0f;
  f32 speed_y = 0.0f;
  f32 source_m3 = 0.0f;
  f32 open_m3 = 0.0f;
  f32 roundoff_m3 = 0.0f;
  f32 pad[3] = {};
};

struct WaterLedger {
  f32 time_hi = 0.0f;
  f32 time_lo = 0.0f;
  f32 source_hi = 0.0f;
  f32 source_lo = 0.0f;
  f32 open_hi = 0.0f;
  f32 open_lo = 0.0f;
  f32 roundoff_hi = 0.0f;
  f32 roundoff_lo = 0.0f;
  f32 remaining_s = 0.0f;
  f32 dt = 0.0f;
  u32 steps = 0;
  u32 pad = 0;
};

struct Ledger {
  f64 source_m3 = 0.0;
  f64 open_edge_out_m3 = 0.0;
  f64 roundoff_m3 = 0.0;
  f64 time_s = 0.0;
  f64 remaining_s = 0.0;
  u64 steps = 0;
};

}  // namespace engine::water_live

// The engine-side binding of the CUDA tick: water_live::DeviceStep's method set
// (systems/water_live/include/systems/water_live/water_live.h:158-256) over the C ABI of
// wlcuda.h, so that the engine's callers change only the type they name. The engine is C++20; the
// binding is header-only and links libwlcuda.so and the CUDA runtime.
//
// What differs from the reference's class, and why:
//   - `create` takes a CUDA device index where the reference takes a gfx::Device;
//   - `record` enqueues on a CUDA stream (capture it into a CUDA graph to replay ticks) where the
//     reference records into a gfx::RenderGraph; it takes no GpuTimer;
//   - the error strings are the library's.
// The PODs it reads and writes (Ledger, WaterPartial, WaterLedger) have the C ABI's sizes and
// offsets, which the library pins with static_asserts and the reference pins in
// water_live_tests.cpp:22-36, so the casts below are layout-exact.
#pragma once

#include <domain/water_state/water_state.h>
#include <systems/water_live/water_live.h>  // Ledger, WaterPartial, WaterLedger, StepOptions, Ops

#include "wlcuda.h"

#include <span>
#include <string>

namespace engine::water_live_cuda {

class DeviceStep {
 public:
  DeviceStep() noexcept = default;
  DeviceStep(const DeviceStep&) = delete;
  DeviceStep& operator=(const DeviceStep&) = delete;
  ~DeviceStep() { destroy(); }

  bool create(int device, const water_state::Config& c, const water_live::StepOptions& o,
              std::string* error = nullptr) {
    const wl_config wc{c.nx, c.ny, c.cell_m, c.gravity, c.cfl, c.dry_depth_m,
                       u8(c.edges.west == water_state::Edge::open),
                       u8(c.edges.east == water_state::Edge::open),
                       u8(c.edges.south == water_state::Edge::open),
                       u8(c.edges.north == water_state::Edge::open), device};
    const wl_options wo{u8(o.ops == water_live::Ops::fixed), u8(o.stored_faces)};
    destroy();
    return ok(wl_create(&wc, &wo, &step_, buf_, sizeof buf_), error);
  }
  void destroy() noexcept {
    wl_destroy(step_);
    step_ = nullptr;
  }
  bool valid() const noexcept { return wl_valid(step_) != 0; }
  u32 cell_count() const noexcept { return wl_cell_count(step_); }
  u32 group_count() const noexcept { return wl_group_count(step_); }

  bool write_state(std::span<const f64> h, std::span<const f64> hu, std::span<const f64> hv,
                   std::string* error = nullptr) {
    if (hu.size() != h.size() || hv.size() != h.size()) return refuse(error);
    return ok(wl_write_state(step_, h.data(), hu.data(), hv.data(), h.size(), buf_, sizeof buf_),
              error);
  }
  bool read_state(std::span<f64> h, std::span<f64> hu, std::span<f64> hv,
                  std::string* error = nullptr) {
    if (hu.size() != h.size() || hv.size() != h.size()) return refuse(error);
    return ok(wl_read_state(step_, h.data(), hu.data(), hv.data(), h.size(), buf_, sizeof buf_),
              error);
  }
  bool read_state_bits(std::span<f32> planes, std::string* error = nullptr) {
    return ok(wl_read_state_bits(step_, planes.data(), planes.size(), buf_, sizeof buf_), error);
  }
  bool read_ledger(water_live::Ledger& out, std::string* error = nullptr) {
    static_assert(sizeof(wl_ledger) == sizeof(water_live::Ledger));
    return ok(wl_read_ledger(step_, reinterpret_cast<wl_ledger*>(&out), buf_, sizeof buf_),
              error);
  }
  bool set_bed(std::span<const f64> bed, f64 datum, std::string* error = nullptr) {
    return ok(wl_set_bed(step_, bed.data(), bed.size(), datum, buf_, sizeof buf_), error);
  }
  bool set_manning(std::span<const f64> n, std::string* error = nullptr) {
    return ok(wl_set_manning(step_, n.data(), n.size(), buf_, sizeof buf_), error);
  }
  bool set_source(std::span<const f64> s, u32 every = 1, bool compensate = false,
                  std::string* error = nullptr) {
    return ok(wl_set_source(step_, s.data(), s.size(), every, compensate ? 1 : 0, buf_,
                            sizeof buf_),
              error);
  }
  // Enqueues `count` steps on `stream` and returns at once (the reference's record).
  bool record(wl_stream stream, u32 count, f32 max_dt) {
    return wl_enqueue_steps(step_, stream, count, max_dt) == WL_OK;
  }
  bool run_steps(u32 count, f32 max_dt, std::string* error = nullptr) {
    return ok(wl_run_steps(step_, count, max_dt, buf_, sizeof buf_), error);
  }
  u64 advance(f64 duration_s, std::string* error = nullptr) {
    buf_[0] = '\0';
    const u64 steps = wl_advance(step_, duration_s, buf_, sizeof buf_);
    if (steps == 0 && error != nullptr) *error = buf_;
    return steps;
  }
  u64 state_hash(std::string* error = nullptr) {
    buf_[0] = '\0';
    const u64 h = wl_state_hash(step_, buf_, sizeof buf_);
    if (h == 0 && error != nullptr) *error = buf_;
    return h;
  }
  bool read_partials_bits(std::span<water_live::WaterPartial> out, std::string* error = nullptr) {
    static_assert(sizeof(wl_partial) == sizeof(water_live::WaterPartial));
    return ok(wl_read_partials_bits(step_, reinterpret_cast<wl_partial*>(out.data()), out.size(),
                                    buf_, sizeof buf_),
              error);
  }
  bool read_ledger_bits(water_live::WaterLedger& out, std::string* error = nullptr) {
    static_assert(sizeof(wl_ledger_bits) == sizeof(water_live::WaterLedger));
    return ok(wl_read_ledger_bits(step_, reinterpret_cast<wl_ledger_bits*>(&out), buf_,
                                  sizeof buf_),
              error);
  }
  bool run_length_pass(f32 max_dt, std::string* error = nullptr) {
    return ok(wl_run_length_pass(step_, max_dt, buf_, sizeof buf_), error);
  }
  wl_step* handle() noexcept { return step_; }

 private:
  bool ok(int rc, std::string* error) {
    if (rc != WL_OK && error != nullptr) *error = buf_;
    return rc == WL_OK;
  }
  static bool refuse(std::string* error) {
    if (error != nullptr) *error = "water_live: spans of different sizes";
    return false;
  }
  wl_step* step_ = nullptr;
  char buf_[256] = {};
};

// water_live::hash_floats (water_live.h:259): FNV-1a 64 over the floats' bytes, low byte first.
inline u64 hash_floats(std::span<const f32> v) noexcept {
  return wl_hash_floats(v.data(), v.size());
}

}  // namespace engine::water_live_cuda

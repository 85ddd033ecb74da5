// The engine-side binding of the complete FP64 step on the device: water_state::Solver
// (domain/water_state/include/domain/water_state/water_state.h:161-266) over the ws_* calls of
// wlcuda.h. Header-only; links libwlcuda.so and the CUDA runtime.
//
// water_state::Solver hands out spans of its own host arrays and takes the inputs with each step.
// On the device the state and the inputs stay there, so this binding copies in and out where the
// reference hands out spans (`write`, `read`), and uploads each input with the step (a caller
// that tracks which spans changed uploads only those, in `put`). The bytes equal the CPU Solver's,
// so a caller that held its state to the CPU Solver's hash keeps it.
#pragma once

#include <domain/water_state/water_state.h>

#include "wlcuda.h"

#include <span>

namespace engine::water_state_cuda {

class Solver {
 public:
  Solver(const water_state::Config& c, int device) {
    ws_config wc{c.nx, c.ny, c.cell_m, c.gravity, c.cfl, c.dry_depth_m, c.water_density,
                 c.carried, 0, {}, u8(c.edges.west == water_state::Edge::open),
                 u8(c.edges.east == water_state::Edge::open),
                 u8(c.edges.south == water_state::Edge::open),
                 u8(c.edges.north == water_state::Edge::open), device};
    for (u32 k = 0; k < c.carried && k < 4; ++k)
      wc.carried_config[k] = {c.carried_config[k].decay_s, c.carried_config[k].per_joule,
                              c.carried_config[k].min_speed_m_per_s};
    ws_create(&wc, &s_, err_, sizeof err_);
  }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;
  ~Solver() { ws_destroy(s_); }

  bool valid() const noexcept { return ws_valid(s_) != 0; }
  // WS_DEPTH ... WS_CARRIED.
  bool write(int field, std::span<const f64> v) {
    return ws_write_field(s_, field, v.data(), v.size(), err_, sizeof err_) == WL_OK;
  }
  // WS_DEPTH ... WS_DISSIPATION.
  bool read(int field, std::span<f64> out) {
    return ws_read_field(s_, field, out.data(), out.size(), err_, sizeof err_) == WL_OK;
  }
  f64 step(const water_state::Inputs& in, f64 max_dt) {
    put(WS_BED, in.bed_m);
    put(WS_MANNING, in.manning);
    put(WS_SOURCE, in.source_m_per_s);
    put(WS_GROUND_CONDUCTIVITY, in.ground_conductivity_m_per_s);
    put(WS_GROUND_SUCTION, in.ground_suction_m);
    put(WS_GROUND_CAPACITY, in.ground_capacity_m);
    for (u32 k = 0; k < water_state::k_max_carried; ++k) {
      put(WS_CARRIED_SOURCE + int(k), in.carried_source[k]);
      put(WS_CARRIED_EXCHANGE + int(k), in.carried_exchange[k]);
    }
    return ws_step(s_, max_dt, err_, sizeof err_);
  }
  bool read_ledger(ws_ledger& out) { return ws_read_ledger(s_, &out, err_, sizeof err_) == WL_OK; }
  u64 state_hash() { return ws_state_hash(s_, err_, sizeof err_); }
  const char* error() const noexcept { return err_; }

 private:
  void put(int slot, std::span<const f64> v) {
    ws_set_input(s_, slot, v.data(), v.size(), err_, sizeof err_);
  }
  ws_solver* s_ = nullptr;
  char err_[256] = {};
};

}  // namespace engine::water_state_cuda

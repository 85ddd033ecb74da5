// A set of water tiles on one device and the launches that step them (host side).
//
// The plain step (the reference's DeviceStep) is a set of one tile; the batched form is a set of
// many. Every device buffer of a set lives in one allocation: per tile two copies of the four
// state planes, the bed, Manning's n and the source, two record buffers; then the tiles'
// control blocks and descriptors, the work items' tile indices and the launch's work counter.
#pragma once

#include "wl_device.cuh"
#include "wl_kernels.h"

#include <cstdint>
#include <string>
#include <vector>

namespace wlc {

struct TileSpec {
  uint32_t nx = 0, ny = 0;
  double cell_m = 1.0, gravity = 9.81, cfl = 0.45, dry_depth_m = 1e-9;
  uint32_t open_edges = 0;  // kFlag*Open bits
};

class TileSet {
 public:
  TileSet() = default;
  ~TileSet();
  TileSet(const TileSet&) = delete;
  TileSet& operator=(const TileSet&) = delete;

  // Allocates and clears every buffer (a dry state over a bed of zero, empty ledgers, records of
  // that state). `order` lists the tiles in the order their work items are dealt (empty: by index).
  bool create(int device, const std::vector<TileSpec>& tiles, bool fixed_ops, BlockShape shape,
              const std::vector<uint32_t>& order, std::string* err);
  void destroy();
  bool valid() const { return base_ != nullptr; }

  // The work items in another block shape (the autotuner's knob); the state is kept.
  bool reshape(BlockShape shape, const std::vector<uint32_t>& order, std::string* err);

  // ---- asynchronous, on `s` -----------------------------------------------------------------
  // `go`: a tick queue's word that lets the launches step (null: always). A single tile of no
  // more blocks than the device holds resident CTAs steps two or more ticks in one cooperative
  // launch (the resident tick); otherwise a launch a tick.
  cudaError_t enqueue_ticks(cudaStream_t s, uint32_t count, float max_dt,
                            const uint32_t* go = nullptr);
  // Tick kernel launches enqueued since create (a diagnosis counter).
  uint64_t tick_launches() const { return tick_launches_; }
  // The march's zero-apart variant for the set's launches (TickArgs::zero_apart; the autotuner's
  // knob). The same bits either way.
  void set_zero_apart(bool on) { zero_apart_ = on; }
  bool zero_apart() const { return zero_apart_; }
  // The block shapes' staged variant (TickArgs::stage): a tile whose width is a multiple of 4
  // takes each block's cells and halo by tensor copies, a CTA's next block's while it steps this
  // one. The same bits either way. kStageOff, kStageOn (both block CTAs), or kStageAuto: a launch
  // of 256-thread CTAs with more blocks than CTAs, where each CTA's next block's copies land while
  // it steps the last and its threads would otherwise load a block in two rounds (1024 x 1024:
  // 28.0 -> 29.1 Gcell/s). A CTA of one block (512 x 512: 11.7 against 11.8 us a tick) or one of
  // 512 threads, which loads in one round (256 x 256: 7.1 against 7.5), is faster by its loads.
  static constexpr uint32_t kStageOff = 0, kStageOn = 1, kStageAuto = 2;
  void set_stage(uint32_t mode) { stage_ = mode; }
  uint32_t stage() const { return stage_; }
  // The device words wait() reads after the launches since the last wait: the resident tick's
  // barrier error word and the staged tick's fault word. A captured graph keeps the ones its
  // launches set (pending_checks after the capture) and adds them at each replay (add_checks).
  static constexpr uint32_t kCheckResident = 1, kCheckStage = 2;
  uint32_t pending_checks() const {
    return (resident_used_ ? kCheckResident : 0u) | (stage_used_ ? kCheckStage : 0u);
  }
  void add_checks(uint32_t checks) {
    resident_used_ = resident_used_ || (checks & kCheckResident) != 0u;
    stage_used_ = stage_used_ || (checks & kCheckStage) != 0u;
  }
  // Tiles with tensor maps (the staged variant's tiles), and those the set's launches stage.
  uint32_t staged_tiles() const { return staged_tiles_; }
  uint32_t staged_launch_tiles() const {
    if (shape_ != BlockShape::k32x16b) return 0u;
    const bool wide = n_items_ <= uint32_t(sms_);
    return stages(wide ? BlockShape::k32x16w : shape_, n_items_, wide ? int(n_items_) + 1 : grid_)
               ? staged_tiles_
               : 0u;
  }
  // Whether a launch of this shape, items and grid takes the staged variant.
  bool stages(BlockShape launch, uint32_t items, int grid) const {
    if (staged_tiles_ == 0u) return false;
    if (stage_ == kStageOn) return launch == BlockShape::k32x16b || launch == BlockShape::k32x16w;
    return stage_ == kStageAuto && launch == BlockShape::k32x16b && items > uint32_t(grid);
  }
  // One tile's own tick (the per-tile-launch form): only that tile's work items.
  cudaError_t enqueue_tile_tick(cudaStream_t s, uint32_t tile, float max_dt);
  cudaError_t enqueue_prime(cudaStream_t s);
  // One tile's records alone (its own items): the other tiles' pending records stay as they are.
  cudaError_t enqueue_tile_prime(cudaStream_t s, uint32_t tile);
  cudaError_t enqueue_length_pass(cudaStream_t s, uint32_t tile, float max_dt);

  // ---- synchronous uploads and read-backs (each waits on the set's stream) -----------------
  bool write_state(uint32_t tile, const double* h, const double* hu, const double* hv,
                   std::string* err);
  bool set_plane(uint32_t tile, int which, const double* v, double datum, std::string* err);
  bool set_flags(uint32_t tile, uint32_t flags, uint32_t source_every, bool reset_phase,
                 std::string* err);
  bool set_remaining(uint32_t tile, float remaining, std::string* err);
  bool read_state(uint32_t tile, double* h, double* hu, double* hv, std::string* err);
  bool read_state_bits(uint32_t tile, float* planes, std::string* err);
  bool read_ctl(uint32_t tile, TileCtl& out, std::string* err);
  bool read_partials(uint32_t tile, Partial* out, std::string* err);
  bool prime(std::string* err);
  bool length_pass(uint32_t tile, float max_dt, std::string* err);
  bool wait(std::string* err);

  // ---- whole batches: arrays of every tile's cells, tile after tile in index order ---------
  bool write_all(const double* h, const double* hu, const double* hv, std::string* err);
  // One tile's state (its ledger emptied, its records primed); the other tiles are untouched.
  bool write_tile(uint32_t tile, const double* h, const double* hu, const double* hv,
                  std::string* err);
  bool set_plane_all(int which, const double* v, double datum, std::string* err);
  bool set_flags_all(uint32_t flags_set, uint32_t flags_clear, uint32_t source_every,
                     bool reset_phase, std::string* err);
  // Every tile's current copy (four planes a tile, 4 * first_cell(t) floats before tile t).
  bool read_all_bits(float* out, std::string* err);
  bool flush_all(std::string* err);
  bool read_all_ctl(TileCtl* out, std::string* err);
  // The settled check against a steady state (doubles): of every tile, the arrays tile after tile
  // (`all`), or of tile `tile` alone, its own nx * ny cells. Per tile, the largest depth and
  // momentum deviations (f32), and settled = both within their bounds. Outputs may be null.
  bool settled(bool all, uint32_t tile, const double* h, const double* hu, const double* hv,
               float depth_bound, float momentum_bound, uint8_t* settled, float* depth_dev,
               float* momentum_dev, std::string* err);
  uint64_t first_cell(uint32_t tile) const { return first_[tile]; }
  // A copy of everything a tick changes (states, records, control blocks), and its restoration:
  // the autotuner's trial ticks leave the simulation where it was.
  bool snapshot(std::string* err);
  bool restore(std::string* err);
  void drop_snapshot();
  const std::vector<uint32_t>& order() const { return order_; }

  uint32_t tile_count() const { return uint32_t(host_.size()); }
  const TileDesc& desc(uint32_t tile) const { return host_[tile]; }
  uint64_t cells(uint32_t tile) const { return uint64_t(host_[tile].nx) * host_[tile].ny; }
  uint64_t total_cells() const { return total_cells_; }
  uint32_t items() const { return n_items_; }
  int grid() const { return grid_; }
  BlockShape shape() const { return shape_; }
  bool fixed_ops() const { return fixed_; }
  cudaStream_t stream() const { return stream_; }
  int device() const { return device_; }
  TileDesc* device_descs() const { return d_desc_; }
  float* device_state(uint32_t tile, uint32_t copy) const { return host_[tile].state[copy]; }
  bool any_manning() const;
  // No tile holds a flag of kFlagsNotPlain: the tick launches the march's plain variant.
  bool plain() const;

 private:
  bool check(cudaError_t e, std::string* err, const char* what);
  bool layout_items(BlockShape shape, const std::vector<uint32_t>& order, std::string* err);
  bool ensure_staging(size_t bytes, std::string* err);
  bool push_desc(uint32_t tile, std::string* err);

  int device_ = -1;
  bool fixed_ = false;
  BlockShape shape_ = BlockShape::k32x32;
  cudaStream_t stream_ = nullptr;
  char* base_ = nullptr;  // the one allocation
  size_t bytes_ = 0;
  std::vector<TileDesc> host_;  // the descriptors as the device holds them
  TileDesc* d_desc_ = nullptr;
  TileCtl* d_ctl_ = nullptr;
  WorkCtl* d_work_ = nullptr;
  ResidentCtl* d_res_ = nullptr;  // the resident tick's barrier words and largest speeds
  int resident_cap_[2] = {0, 0};  // resident CTAs the device holds (without, with Manning's)
  bool resident_used_ = false;      // a resident launch since the last wait()
  uint64_t tick_launches_ = 0;
  bool zero_apart_ = false;
  uint32_t stage_ = kStageOff;
  bool stage_used_ = false;  // a staged block launch since the last wait()
  uint32_t staged_tiles_ = 0;
  uint32_t* d_item_tile_ = nullptr;  // the tile of each work item (null for one tile)
  uint32_t n_items_ = 0;
  int grid_ = 0;
  int sms_ = 0;  // the device's SM count
  uint64_t total_cells_ = 0;
  std::vector<uint64_t> first_;  // each tile's first cell in the concatenated arrays
  uint64_t* d_first_ = nullptr;
  size_t mutable_bytes_ = 0;     // the leading part of the allocation a tick writes
  void* snap_ = nullptr;
  void* staging_ = nullptr;  // device staging for uploads and read-backs
  size_t staging_bytes_ = 0;
  std::vector<uint32_t> order_;
};

// Waits for a stream with a time limit (WLCUDA_WAIT_S seconds, default 300): a wait that passes it
// returns cudaErrorTimeout-like failure through `timed_out` instead of blocking forever.
cudaError_t wait_stream(cudaStream_t s, bool* timed_out);

uint64_t fnv1a_floats(const float* v, size_t n, uint64_t hash = 0xcbf29ce484222325ull);

}  // namespace wlc

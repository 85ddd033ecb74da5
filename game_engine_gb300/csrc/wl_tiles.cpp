// A set of water tiles on one device (wl_tiles.h).
#include "wl_tiles.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>

namespace wlc {

namespace {

constexpr size_t kAlign = 256;
constexpr size_t kMapBytes = 128;  // a tensor map

size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

double wait_limit_s() {
  const char* e = std::getenv("WLCUDA_WAIT_S");
  if (e != nullptr) {
    const double v = std::atof(e);
    if (v > 0.0) return v;
  }
  return 300.0;
}

}  // namespace

uint64_t fnv1a_floats(const float* v, size_t n, uint64_t hash) {
  for (size_t i = 0; i < n; ++i) {
    uint32_t bits;
    std::memcpy(&bits, v + i, 4);
    for (uint32_t b = 0; b < 4; ++b) {
      hash ^= (bits >> (8 * b)) & 0xffu;
      hash *= 0x100000001b3ull;
    }
  }
  return hash;
}

cudaError_t wait_stream(cudaStream_t s, bool* timed_out) {
  if (timed_out) *timed_out = false;
  const auto start = std::chrono::steady_clock::now();
  const double limit = wait_limit_s();
  for (uint32_t spin = 0;; ++spin) {
    const cudaError_t e = cudaStreamQuery(s);
    if (e != cudaErrorNotReady) return e;
    const double waited =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    if (waited > limit) {
      if (timed_out) *timed_out = true;
      return cudaErrorNotReady;
    }
    if (spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

TileSet::~TileSet() { destroy(); }

bool TileSet::check(cudaError_t e, std::string* err, const char* what) {
  if (e == cudaSuccess) return true;
  if (err) *err = std::string("water_live: ") + what + ": " + cudaGetErrorString(e);
  return false;
}

void TileSet::destroy() {
  if (device_ >= 0) cudaSetDevice(device_);
  if (stream_ != nullptr) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
  if (base_ != nullptr) cudaFree(base_);
  if (staging_ != nullptr) cudaFree(staging_);
  if (snap_ != nullptr) cudaFree(snap_);
  if (d_item_tile_ != nullptr) cudaFree(d_item_tile_);
  snap_ = nullptr;
  d_first_ = nullptr;
  first_.clear();
  mutable_bytes_ = 0;
  stream_ = nullptr;
  base_ = nullptr;
  staging_ = nullptr;
  staging_bytes_ = 0;
  host_.clear();
  d_desc_ = nullptr;
  d_ctl_ = nullptr;
  d_work_ = nullptr;
  d_item_tile_ = nullptr;
  n_items_ = 0;
  device_ = -1;
}

bool TileSet::any_manning() const {
  for (const TileDesc& d : host_)
    if (d.flags & kFlagManning) return true;
  return false;
}

bool TileSet::plain() const {
  for (const TileDesc& d : host_)
    if (d.flags & kFlagsNotPlain) return false;
  return true;
}

bool TileSet::create(int device, const std::vector<TileSpec>& tiles, bool fixed_ops,
                     BlockShape shape, const std::vector<uint32_t>& order, std::string* err) {
  destroy();
  if (tiles.empty()) {
    if (err) *err = "water_live: no tiles";
    return false;
  }
  for (const TileSpec& t : tiles) {
    if (t.nx == 0 || t.ny == 0) {
      if (err) *err = "water_live: an empty grid";
      return false;
    }
    if (uint64_t(t.nx) * t.ny >= (1ull << 31)) {
      if (err) *err = "water_live: a grid of 2^31 cells or more";
      return false;
    }
  }
  if (!check(cudaSetDevice(device), err, "cudaSetDevice")) return false;
  device_ = device;
  fixed_ = fixed_ops;
  if (!check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), err, "cudaStreamCreate")) {
    destroy();
    return false;
  }
  // One allocation. First what a tick writes (every tile's two state copies and two record
  // buffers, then the control blocks), so a snapshot is one copy; then the inputs (bed, Manning's
  // n, source), the descriptors, the cell offsets and the work counter.
  const size_t nt = tiles.size();
  std::vector<size_t> off_state(nt), off_inputs(nt), off_rec(nt);
  size_t total = 0;
  total_cells_ = 0;
  first_.assign(nt, 0);
  for (size_t i = 0; i < nt; ++i) {
    const size_t n = size_t(tiles[i].nx) * tiles[i].ny;
    first_[i] = total_cells_;
    total_cells_ += n;
    off_state[i] = total;
    total += 2 * align_up(kStatePlanes * n * sizeof(float));
  }
  for (size_t i = 0; i < nt; ++i) {
    const size_t groups = size_t((tiles[i].nx + 15) / 16) * ((tiles[i].ny + 15) / 16);
    off_rec[i] = total;
    total += 2 * align_up(groups * sizeof(Partial));
  }
  const size_t off_ctl = total;
  total += align_up(nt * sizeof(TileCtl));
  mutable_bytes_ = total;
  for (size_t i = 0; i < nt; ++i) {
    const size_t n = size_t(tiles[i].nx) * tiles[i].ny;
    off_inputs[i] = total;
    total += 3 * align_up(n * sizeof(float));
  }
  const size_t off_desc = total;
  total += align_up(nt * sizeof(TileDesc));
  const size_t off_first = total;
  total += align_up(nt * sizeof(uint64_t));
  // The work counters: one for launches over the whole set, one per tile for its own launches
  // (tiles launched alone may run concurrently on different streams), then the resident tick's
  // words.
  const size_t off_work = total;
  total += align_up((1 + nt) * sizeof(WorkCtl));
  const size_t off_res = total;
  total += align_up(sizeof(ResidentCtl));
  // The staged block tick's tensor maps, three of 128 bytes a tile.
  const size_t off_maps = total;
  total += align_up(nt * 3 * kMapBytes);
  if (!check(cudaMalloc(&base_, total), err, "cudaMalloc")) {
    base_ = nullptr;
    destroy();
    return false;
  }
  bytes_ = total;
  if (!check(cudaMemsetAsync(base_, 0, total, stream_), err, "cudaMemset")) {
    destroy();
    return false;
  }
  d_ctl_ = reinterpret_cast<TileCtl*>(base_ + off_ctl);
  d_desc_ = reinterpret_cast<TileDesc*>(base_ + off_desc);
  d_first_ = reinterpret_cast<uint64_t*>(base_ + off_first);
  d_work_ = reinterpret_cast<WorkCtl*>(base_ + off_work);
  d_res_ = reinterpret_cast<ResidentCtl*>(base_ + off_res);
  if (!check(cudaMemcpyAsync(d_first_, first_.data(), nt * sizeof(uint64_t),
                             cudaMemcpyHostToDevice, stream_),
             err, "upload of the cell offsets")) {
    destroy();
    return false;
  }
  host_.resize(nt);
  for (size_t i = 0; i < nt; ++i) {
    const TileSpec& t = tiles[i];
    const size_t n = size_t(t.nx) * t.ny;
    const size_t groups = size_t((t.nx + 15) / 16) * ((t.ny + 15) / 16);
    TileDesc& d = host_[i];
    std::memset(&d, 0, sizeof d);
    const size_t plane_bytes = align_up(kStatePlanes * n * sizeof(float));
    d.state[0] = reinterpret_cast<float*>(base_ + off_state[i]);
    d.state[1] = reinterpret_cast<float*>(base_ + off_state[i] + plane_bytes);
    const size_t in_bytes = align_up(n * sizeof(float));
    d.bed = reinterpret_cast<const float*>(base_ + off_inputs[i]);
    d.manning = reinterpret_cast<const float*>(base_ + off_inputs[i] + in_bytes);
    d.source = reinterpret_cast<const float*>(base_ + off_inputs[i] + 2 * in_bytes);
    const size_t rec_bytes = align_up(groups * sizeof(Partial));
    d.rec[0] = reinterpret_cast<Partial*>(base_ + off_rec[i]);
    d.rec[1] = reinterpret_cast<Partial*>(base_ + off_rec[i] + rec_bytes);
    d.ctl = d_ctl_ + i;
    d.nx = t.nx;
    d.ny = t.ny;
    d.groups_x = (t.nx + 15) / 16;
    d.groups_y = (t.ny + 15) / 16;
    d.flags = t.open_edges & 15u;
    d.source_every = 1;
    // The kernels' constants round like the reference's push constants (water_live.cpp:245-248).
    d.cell_m = static_cast<float>(t.cell_m);
    d.gravity = static_cast<float>(t.gravity);
    d.cfl = static_cast<float>(t.cfl);
    d.dry = static_cast<float>(t.dry_depth_m);
  }
  // The tensor maps of every tile whose shape allows them (encoded here, uploaded once: they
  // describe the tile's fixed allocations).
  {
    std::vector<unsigned char> maps(nt * 3 * kMapBytes + 64);
    unsigned char* h = maps.data() + ((64u - reinterpret_cast<uintptr_t>(maps.data()) % 64u) % 64u);
    char* dev = base_ + off_maps;
    staged_tiles_ = 0;
    for (size_t i = 0; i < nt; ++i) {
      TileDesc& d = host_[i];
      d.tmap = nullptr;
      if (encode_stage_maps(d, h + i * 3 * kMapBytes)) {
        d.tmap = dev + i * 3 * kMapBytes;
        ++staged_tiles_;
      }
    }
    if (!check(cudaMemcpyAsync(dev, h, nt * 3 * kMapBytes, cudaMemcpyHostToDevice, stream_), err,
               "upload of the tensor maps")) {
      destroy();
      return false;
    }
  }
  // Empty ledgers: every field zero but the time left, +inf between advances.
  std::vector<TileCtl> ctl(nt);
  for (TileCtl& c : ctl) {
    std::memset(&c, 0, sizeof c);
    c.ledger[0].remaining_s = std::numeric_limits<float>::infinity();
    c.ledger[1].remaining_s = std::numeric_limits<float>::infinity();
  }
  if (!check(cudaMemcpyAsync(d_ctl_, ctl.data(), nt * sizeof(TileCtl), cudaMemcpyHostToDevice,
                             stream_),
             err, "upload of the ledgers") ||
      !check(cudaStreamSynchronize(stream_), err, "cudaStreamSynchronize")) {
    destroy();
    return false;
  }
  for (BlockShape s : {BlockShape::k32x16, BlockShape::k32x32, BlockShape::k32x64,
                       BlockShape::k32x16s, BlockShape::k32x16b, BlockShape::k32x16w})
    for (int v = 0; v < 3; ++v)  // Manning's, the plain and the general variant
      if (tick_occupancy(s, fixed_, v == 0, v == 1) <= 0) {
        if (err) *err = "water_live: the tick kernel cannot be resident on this device";
        destroy();
        return false;
      }
  // The resident tick's capacity, taken here rather than at a launch that may be under capture.
  resident_cap_[0] = resident_capacity(fixed_, false);
  resident_cap_[1] = resident_capacity(fixed_, true);
  if (!layout_items(shape, order, err)) {
    destroy();
    return false;
  }
  return prime(err);
}

bool TileSet::layout_items(BlockShape shape, const std::vector<uint32_t>& order,
                           std::string* err) {
  uint32_t bx = 0, by = 0;
  block_dims(shape, bx, by);
  const uint32_t nt = tile_count();
  order_ = order;
  if (order_.size() != nt) {
    order_.resize(nt);
    for (uint32_t i = 0; i < nt; ++i) order_[i] = i;
  }
  std::vector<uint32_t> item_tile;
  uint64_t items = 0;
  for (uint32_t k = 0; k < nt; ++k) {
    TileDesc& d = host_[order_[k]];
    d.blocks_x = (d.nx + bx - 1) / bx;
    d.blocks_y = (d.ny + by - 1) / by;
    d.items = d.blocks_x * d.blocks_y;
    d.item_base = uint32_t(items);
    items += d.items;
  }
  if (items >= (1ull << 32)) {
    if (err) *err = "water_live: too many work items";
    return false;
  }
  n_items_ = uint32_t(items);
  if (nt > 1) {
    item_tile.resize(n_items_);
    for (uint32_t k = 0; k < nt; ++k) {
      const TileDesc& d = host_[order_[k]];
      std::fill(item_tile.begin() + d.item_base, item_tile.begin() + d.item_base + d.items,
                order_[k]);
    }
  }
  shape_ = shape;
  int sms = 0;
  if (!check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_), err,
             "cudaDeviceGetAttribute"))
    return false;
  sms_ = sms;
  const int occ = tick_occupancy(shape, fixed_, any_manning(), plain());
  grid_ = std::max(1, std::min<int>(int(n_items_), sms * std::max(1, occ)));
  // The items' tile indices: a separate small allocation, replaced on a reshape.
  static_assert(sizeof(uint32_t) == 4, "");
  if (d_item_tile_ != nullptr) {
    cudaStreamSynchronize(stream_);
    cudaFree(d_item_tile_);
    d_item_tile_ = nullptr;
  }
  if (nt > 1) {
    if (!check(cudaMalloc(&d_item_tile_, item_tile.size() * sizeof(uint32_t)), err, "cudaMalloc"))
      return false;
    if (!check(cudaMemcpyAsync(d_item_tile_, item_tile.data(), item_tile.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, stream_),
               err, "upload of the work items"))
      return false;
  }
  if (!check(cudaMemcpyAsync(d_desc_, host_.data(), nt * sizeof(TileDesc), cudaMemcpyHostToDevice,
                             stream_),
             err, "upload of the tiles"))
    return false;
  return check(cudaStreamSynchronize(stream_), err, "cudaStreamSynchronize");
}

bool TileSet::reshape(BlockShape shape, const std::vector<uint32_t>& order, std::string* err) {
  if (!valid()) return false;
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(cudaStreamSynchronize(stream_), err, "cudaStreamSynchronize")) return false;
  // The records are per 16 x 16 group whatever the block shape; only the items change.
  return layout_items(shape, order, err);
}

bool TileSet::push_desc(uint32_t tile, std::string* err) {
  if (!check(cudaMemcpyAsync(d_desc_ + tile, &host_[tile], sizeof(TileDesc),
                             cudaMemcpyHostToDevice, stream_),
             err, "upload of a tile"))
    return false;
  return check(cudaStreamSynchronize(stream_), err, "cudaStreamSynchronize");
}

cudaError_t TileSet::enqueue_ticks(cudaStream_t s, uint32_t count, float max_dt,
                                   const uint32_t* go) {
  TickArgs a;
  a.tiles = d_desc_;
  a.item_tile = d_item_tile_;
  a.work = d_work_;
  a.n_items = n_items_;
  a.max_dt = max_dt;
  a.go = go;
  a.zero_apart = zero_apart_ ? 1u : 0u;
  a.fault = &d_work_->fault;
  const bool manning = any_manning(), plain_set = plain();
  // The block shape's wide CTA where the launch holds no more blocks than the device has SMs; for
  // one tile, one CTA more folds its ledger beside the items.
  const bool wide = shape_ == BlockShape::k32x16b && n_items_ <= uint32_t(sms_);
  const BlockShape shape = wide ? BlockShape::k32x16w : shape_;
  int grid = grid_;
  if (wide && d_item_tile_ == nullptr) {
    a.fold_apart = 1u;
    grid = int(n_items_) + 1;
    if (go == nullptr && count > 1) {
      if (grid <= resident_cap_[manning ? 1 : 0]) {
        resident_used_ = true;
        ++tick_launches_;
        return launch_tick_resident(fixed_, manning, a, count, d_res_, s);
      }
    }
  }
  a.stage = stages(shape, n_items_, grid) ? 1u : 0u;
  if (a.stage != 0u) stage_used_ = true;
  for (uint32_t i = 0; i < count; ++i) {
    const cudaError_t e = launch_tick(shape, fixed_, manning, plain_set, a, grid, s);
    if (e != cudaSuccess) return e;
    ++tick_launches_;
  }
  return cudaSuccess;
}

cudaError_t TileSet::enqueue_tile_tick(cudaStream_t s, uint32_t tile, float max_dt) {
  TickArgs a;
  a.tiles = d_desc_ + tile;
  a.item_tile = nullptr;
  a.work = d_work_ + 1 + tile;
  a.n_items = host_[tile].items;
  a.max_dt = max_dt;
  a.zero_apart = zero_apart_ ? 1u : 0u;
  a.fault = &d_work_->fault;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_);
  const bool manning = (host_[tile].flags & kFlagManning) != 0u;
  const bool plain_tile = (host_[tile].flags & kFlagsNotPlain) == 0u;
  const int occ = std::max(1, tick_occupancy(shape_, fixed_, manning, plain_tile));
  const int grid = std::max(1, std::min<int>(int(a.n_items), sms * occ));
  a.stage = stages(shape_, a.n_items, grid) && host_[tile].tmap != nullptr ? 1u : 0u;
  if (a.stage != 0u) stage_used_ = true;
  return launch_tick(shape_, fixed_, manning, plain_tile, a, grid, s);
}

cudaError_t TileSet::enqueue_prime(cudaStream_t s) {
  TickArgs a;
  a.tiles = d_desc_;
  a.item_tile = d_item_tile_;
  a.work = d_work_;
  a.n_items = n_items_;
  a.max_dt = 0.0f;
  return launch_prime(shape_, fixed_, a, s);
}

cudaError_t TileSet::enqueue_tile_prime(cudaStream_t s, uint32_t tile) {
  TickArgs a;
  a.tiles = d_desc_ + tile;
  a.item_tile = nullptr;
  a.work = d_work_ + 1 + tile;
  a.n_items = host_[tile].items;
  a.max_dt = 0.0f;
  return launch_prime(shape_, fixed_, a, s);
}

bool TileSet::write_tile(uint32_t tile, const double* h, const double* hu, const double* hv,
                         std::string* err) {
  if (!write_state(tile, h, hu, hv, err)) return false;
  return check(enqueue_tile_prime(stream_, tile), err, "the tile's prime pass") && wait(err);
}

cudaError_t TileSet::enqueue_length_pass(cudaStream_t s, uint32_t tile, float max_dt) {
  return launch_length_pass(fixed_, d_desc_, tile, max_dt, s);
}

bool TileSet::wait(std::string* err) {
  bool timed_out = false;
  const cudaError_t e = wait_stream(stream_, &timed_out);
  if (timed_out) {
    if (err) *err = "water_live: the device did not finish within the wait limit";
    return false;
  }
  if (!check(e, err, "the device")) return false;
  if (resident_used_) {
    // A resident launch's barrier marks its error word where a wait gave up; the state is then
    // not the ticks' result.
    resident_used_ = false;
    uint32_t word = 0u;
    if (!check(cudaMemcpy(&word, &d_res_->error, sizeof word, cudaMemcpyDeviceToHost), err,
               "read-back of the resident tick's barrier"))
      return false;
    if (word != 0u) {
      if (err) *err = "water_live: the resident tick's grid barrier gave up (a CTA did not arrive)";
      return false;
    }
  }
  if (stage_used_) {
    // A staged block launch marks the fault word where a CTA's wait on its copies gave up; the
    // state is then not the ticks' result.
    stage_used_ = false;
    uint32_t word = 0u;
    if (!check(cudaMemcpy(&word, &d_work_->fault, sizeof word, cudaMemcpyDeviceToHost), err,
               "read-back of the staged tick's fault word"))
      return false;
    if (word != 0u) {
      if (err) *err = "water_live: the staged block tick's copies did not land (wait gave up)";
      return false;
    }
  }
  return true;
}

bool TileSet::prime(std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(enqueue_prime(stream_), err, "the prime pass")) return false;
  return wait(err);
}

bool TileSet::length_pass(uint32_t tile, float max_dt, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(enqueue_length_pass(stream_, tile, max_dt), err, "the length pass")) return false;
  return wait(err);
}

bool TileSet::ensure_staging(size_t bytes, std::string* err) {
  if (staging_bytes_ >= bytes) return true;
  if (staging_ != nullptr) {
    cudaStreamSynchronize(stream_);
    cudaFree(staging_);
    staging_ = nullptr;
    staging_bytes_ = 0;
  }
  if (!check(cudaMalloc(&staging_, bytes), err, "cudaMalloc")) {
    staging_ = nullptr;
    return false;
  }
  staging_bytes_ = bytes;
  return true;
}

bool TileSet::write_state(uint32_t tile, const double* h, const double* hu, const double* hv,
                          std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = cells(tile);
  if (!ensure_staging(3 * n * sizeof(double), err)) return false;
  double* d = static_cast<double*>(staging_);
  if (!check(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of the depth") ||
      !check(cudaMemcpyAsync(d + n, hu, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of the momentum") ||
      !check(cudaMemcpyAsync(d + 2 * n, hv, n * sizeof(double), cudaMemcpyHostToDevice, stream_),
             err, "upload of the momentum") ||
      !check(launch_write_state(d_desc_, tile, n, d, d + n, d + 2 * n, stream_), err,
             "the state's conversion"))
    return false;
  return wait(err);
}

bool TileSet::set_plane(uint32_t tile, int which, const double* v, double datum,
                        std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = cells(tile);
  if (!ensure_staging(n * sizeof(double), err)) return false;
  float* dst = nullptr;
  const TileDesc& d = host_[tile];
  if (which == 0) dst = const_cast<float*>(d.bed);
  else if (which == 1) dst = const_cast<float*>(d.manning);
  else dst = const_cast<float*>(d.source);
  double* s = static_cast<double*>(staging_);
  if (!check(cudaMemcpyAsync(s, v, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of an input") ||
      !check(launch_plane(dst, s, n, datum, stream_), err, "an input's conversion"))
    return false;
  return wait(err);
}

bool TileSet::set_flags(uint32_t tile, uint32_t flags, uint32_t source_every, bool reset_phase,
                        std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  host_[tile].flags = flags;
  host_[tile].source_every = source_every;
  if (reset_phase) {
    if (!check(cudaMemsetAsync(&d_ctl_[tile].src_phase, 0, sizeof(uint32_t), stream_), err,
               "cudaMemset"))
      return false;
  }
  if (!push_desc(tile, err)) return false;
  // The launch grid follows the variant the flags select.
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_);
  const int occ = tick_occupancy(shape_, fixed_, any_manning(), plain());
  grid_ = std::max(1, std::min<int>(int(n_items_), sms * std::max(1, occ)));
  return true;
}

bool TileSet::set_remaining(uint32_t tile, float remaining, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  // Both slots: the current one is read by the next tick, the other is rewritten from it.
  for (int k = 0; k < 2; ++k)
    if (!check(cudaMemcpyAsync(&d_ctl_[tile].ledger[k].remaining_s, &remaining, sizeof remaining,
                               cudaMemcpyHostToDevice, stream_),
               err, "upload of the time left"))
      return false;
  return wait(err);
}

bool TileSet::read_state(uint32_t tile, double* h, double* hu, double* hv, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = cells(tile);
  if (!ensure_staging(3 * n * sizeof(double), err)) return false;
  double* d = static_cast<double*>(staging_);
  if (!check(launch_read_state(d_desc_, tile, n, d, d + n, d + 2 * n, stream_), err,
             "the state's widening") ||
      !check(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), err,
             "read-back of the depth") ||
      !check(cudaMemcpyAsync(hu, d + n, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), err,
             "read-back of the momentum") ||
      !check(cudaMemcpyAsync(hv, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, stream_),
             err, "read-back of the momentum"))
    return false;
  return wait(err);
}

bool TileSet::read_state_bits(uint32_t tile, float* planes, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = cells(tile);
  if (!ensure_staging(kStatePlanes * n * sizeof(float), err)) return false;
  float* d = static_cast<float*>(staging_);
  if (!check(launch_copy_state(d_desc_, tile, n, d, stream_), err, "the state's copy") ||
      !check(cudaMemcpyAsync(planes, d, kStatePlanes * n * sizeof(float), cudaMemcpyDeviceToHost,
                             stream_),
             err, "read-back of the state"))
    return false;
  return wait(err);
}

bool TileSet::read_ctl(uint32_t tile, TileCtl& out, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(cudaMemcpyAsync(&out, d_ctl_ + tile, sizeof(TileCtl), cudaMemcpyDeviceToHost, stream_),
             err, "read-back of the ledger"))
    return false;
  return wait(err);
}

bool TileSet::read_partials(uint32_t tile, Partial* out, std::string* err) {
  TileCtl c;
  if (!read_ctl(tile, c, err)) return false;
  const TileDesc& d = host_[tile];
  const size_t groups = size_t(d.groups_x) * d.groups_y;
  if (!check(cudaMemcpyAsync(out, d.rec[c.rec & 1u], groups * sizeof(Partial),
                             cudaMemcpyDeviceToHost, stream_),
             err, "read-back of the records"))
    return false;
  return wait(err);
}

bool TileSet::write_all(const double* h, const double* hu, const double* hv, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = total_cells_;
  if (!ensure_staging(3 * n * sizeof(double), err)) return false;
  double* d = static_cast<double*>(staging_);
  if (!check(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of the depth") ||
      !check(cudaMemcpyAsync(d + n, hu, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of the momentum") ||
      !check(cudaMemcpyAsync(d + 2 * n, hv, n * sizeof(double), cudaMemcpyHostToDevice, stream_),
             err, "upload of the momentum") ||
      !check(launch_scatter_state(d_desc_, tile_count(), d_first_, n, d, d + n, d + 2 * n, stream_),
             err, "the states' conversion") ||
      !check(enqueue_prime(stream_), err, "the prime pass"))
    return false;
  return wait(err);
}

bool TileSet::settled(bool all, uint32_t tile, const double* h, const double* hu,
                      const double* hv, float depth_bound, float momentum_bound, uint8_t* out,
                      float* depth_dev, float* momentum_dev, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const uint32_t count = all ? tile_count() : 1u;
  const size_t n = all ? total_cells_ : cells(tile);
  uint64_t largest = 0;
  for (uint32_t k = 0; k < count; ++k) largest = std::max<uint64_t>(largest, cells(all ? k : tile));
  const size_t values = align_up(3 * n * sizeof(double));
  if (!ensure_staging(values + size_t(count) * 2 * sizeof(uint32_t), err)) return false;
  double* d = static_cast<double*>(staging_);
  uint32_t* dev = reinterpret_cast<uint32_t*>(static_cast<char*>(staging_) + values);
  std::vector<uint32_t> bits(size_t(count) * 2);
  if (!check(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of the steady depth") ||
      !check(cudaMemcpyAsync(d + n, hu, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of the steady momentum") ||
      !check(cudaMemcpyAsync(d + 2 * n, hv, n * sizeof(double), cudaMemcpyHostToDevice, stream_),
             err, "upload of the steady momentum") ||
      !check(launch_settled(d_desc_, all ? 0u : tile, count, all ? d_first_ : nullptr, largest, d,
                            d + n, d + 2 * n, dev, stream_),
             err, "the settled check") ||
      !check(cudaMemcpyAsync(bits.data(), dev, bits.size() * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, stream_),
             err, "read-back of the settled check") ||
      !wait(err))
    return false;
  for (uint32_t k = 0; k < count; ++k) {
    float dd, dq;
    std::memcpy(&dd, &bits[2 * k], 4);
    std::memcpy(&dq, &bits[2 * k + 1], 4);
    if (depth_dev != nullptr) depth_dev[k] = dd;
    if (momentum_dev != nullptr) momentum_dev[k] = dq;
    if (out != nullptr) out[k] = (dd <= depth_bound && dq <= momentum_bound) ? 1u : 0u;
  }
  return true;
}

bool TileSet::set_plane_all(int which, const double* v, double datum, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = total_cells_;
  if (!ensure_staging(n * sizeof(double), err)) return false;
  double* d = static_cast<double*>(staging_);
  if (!check(cudaMemcpyAsync(d, v, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
             "upload of an input") ||
      !check(launch_scatter_plane(d_desc_, tile_count(), d_first_, n, d, datum, which, stream_),
             err, "an input's conversion"))
    return false;
  return wait(err);
}

bool TileSet::set_flags_all(uint32_t flags_set, uint32_t flags_clear, uint32_t source_every,
                            bool reset_phase, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  for (TileDesc& d : host_) {
    d.flags = (d.flags & ~flags_clear) | flags_set;
    d.source_every = source_every;
  }
  if (reset_phase) {
    std::vector<TileCtl> ctl(tile_count());
    if (!check(cudaMemcpyAsync(ctl.data(), d_ctl_, ctl.size() * sizeof(TileCtl),
                               cudaMemcpyDeviceToHost, stream_),
               err, "read-back of the control blocks") ||
        !wait(err))
      return false;
    for (TileCtl& c : ctl) c.src_phase = 0u;
    if (!check(cudaMemcpyAsync(d_ctl_, ctl.data(), ctl.size() * sizeof(TileCtl),
                               cudaMemcpyHostToDevice, stream_),
               err, "upload of the control blocks"))
      return false;
  }
  if (!check(cudaMemcpyAsync(d_desc_, host_.data(), host_.size() * sizeof(TileDesc),
                             cudaMemcpyHostToDevice, stream_),
             err, "upload of the tiles"))
    return false;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_);
  const int occ = tick_occupancy(shape_, fixed_, any_manning(), plain());
  grid_ = std::max(1, std::min<int>(int(n_items_), sms * std::max(1, occ)));
  return wait(err);
}

bool TileSet::read_all_bits(float* out, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  const size_t n = total_cells_;
  if (!ensure_staging(kStatePlanes * n * sizeof(float), err)) return false;
  float* d = static_cast<float*>(staging_);
  if (!check(launch_gather_state(d_desc_, tile_count(), d_first_, n, d, stream_), err,
             "the states' gather") ||
      !check(cudaMemcpyAsync(out, d, kStatePlanes * n * sizeof(float), cudaMemcpyDeviceToHost,
                             stream_),
             err, "read-back of the states"))
    return false;
  return wait(err);
}

bool TileSet::flush_all(std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(launch_flush_all(fixed_, d_desc_, tile_count(), stream_), err, "the flush")) return false;
  return wait(err);
}

bool TileSet::read_all_ctl(TileCtl* out, std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(cudaMemcpyAsync(out, d_ctl_, tile_count() * sizeof(TileCtl), cudaMemcpyDeviceToHost,
                             stream_),
             err, "read-back of the ledgers"))
    return false;
  return wait(err);
}

bool TileSet::snapshot(std::string* err) {
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (snap_ == nullptr && !check(cudaMalloc(&snap_, mutable_bytes_), err, "cudaMalloc")) {
    snap_ = nullptr;
    return false;
  }
  if (!check(cudaMemcpyAsync(snap_, base_, mutable_bytes_, cudaMemcpyDeviceToDevice, stream_), err,
             "the snapshot"))
    return false;
  return wait(err);
}

bool TileSet::restore(std::string* err) {
  if (snap_ == nullptr) {
    if (err) *err = "water_live: no snapshot";
    return false;
  }
  if (!check(cudaSetDevice(device_), err, "cudaSetDevice")) return false;
  if (!check(cudaMemcpyAsync(base_, snap_, mutable_bytes_, cudaMemcpyDeviceToDevice, stream_), err,
             "the restore"))
    return false;
  return wait(err);
}

void TileSet::drop_snapshot() {
  if (snap_ != nullptr) {
    cudaSetDevice(device_);
    cudaStreamSynchronize(stream_);
    cudaFree(snap_);
    snap_ = nullptr;
  }
}

}  // namespace wlc

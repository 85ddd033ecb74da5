// The batched form's C ABI (include/wlcuda.h, wl_batch_*): many tiles of uneven sizes stepped by
// one persistent launch per tick, replayed from a captured CUDA graph, with the block shape and
// the order work items are dealt in chosen by timing the candidates on the batch itself.
#include "wlcuda.h"

#include "wl_adjoint.h"
#include "wl_queue.h"
#include "wl_tiles.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

using wlc::BlockShape;
using wlc::TileSet;

struct wl_batch {
  TileSet set;
  wl_config common{};
  wl_options options{};
  std::vector<wlc::TileSpec> specs;
  uint32_t flags = 0;  // the batch's Manning / source / compensate flags
  uint32_t source_every = 1;
  wl_tuning tuning{};
  wl_queue* queue = nullptr;  // a tick queue attached owns the tiles' clocks
  // The captured graph of `graph_ticks` ticks and what it was captured for.
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_ticks = 0;
  float graph_max_dt = 0.0f;
  uint64_t graph_key = 0;
  uint32_t graph_checks = 0;  // the device words its launches set (TileSet::pending_checks)
  cudaGraphExec_t tile_graph = nullptr;
  float tile_graph_max_dt = 0.0f;
  uint64_t tile_graph_key = 0;
  uint32_t tile_graph_checks = 0;
  std::vector<cudaStream_t> side_streams;  // the per-tile form's concurrent streams
  ~wl_batch() {
    if (graph != nullptr) cudaGraphExecDestroy(graph);
    if (tile_graph != nullptr) cudaGraphExecDestroy(tile_graph);
    for (cudaStream_t s : side_streams) cudaStreamDestroy(s);
  }
};

namespace {

int fail(char* err, size_t len, int code, const std::string& msg) {
  if (err != nullptr && len > 0) {
    const size_t k = msg.size() < len - 1 ? msg.size() : len - 1;
    std::memcpy(err, msg.data(), k);
    err[k] = '\0';
  }
  return code;
}

int cuda_fail(char* err, size_t len, const std::string& msg) {
  const int code = msg.find("wait limit") != std::string::npos ? WL_ERR_TIMEOUT : WL_ERR_CUDA;
  return fail(err, len, code, msg);
}

bool valid(const wl_batch* b) { return b != nullptr && b->set.valid(); }
const char* k_no_device = "water_live: no device";
const char* k_queued = "water_live: the batch's tick queue owns its clocks (destroy the queue first)";

// block_rows: the rows one warp marches (4: the 32 x 16 items split over a CTA's four warps; 1: the
// 32 x 16 items in three phases, no march).
BlockShape shape_of_rows(uint32_t rows) {
  return rows == 1    ? BlockShape::k32x16b
         : rows == 4  ? BlockShape::k32x16s
         : rows == 16 ? BlockShape::k32x16
         : rows == 64 ? BlockShape::k32x64
                      : BlockShape::k32x32;
}

// Work-item orders: 0 tiles by index, 1 the largest tiles first.
std::vector<uint32_t> item_order(const std::vector<wlc::TileSpec>& specs, uint32_t order) {
  std::vector<uint32_t> o(specs.size());
  for (uint32_t i = 0; i < o.size(); ++i) o[i] = i;
  if (order == 1)
    std::stable_sort(o.begin(), o.end(), [&](uint32_t a, uint32_t b) {
      return uint64_t(specs[a].nx) * specs[a].ny > uint64_t(specs[b].nx) * specs[b].ny;
    });
  return o;
}

// What a captured graph depends on: the block shape, the order, the launch's grid and variant.
uint64_t launch_key(const wl_batch* b) {
  return (uint64_t(b->set.shape()) << 48) ^ (uint64_t(b->tuning.order) << 40) ^
         (uint64_t(b->set.grid()) << 8) ^ (b->set.any_manning() ? 1u : 0u) ^
         (b->set.plain() ? 2u : 0u) ^ (b->set.zero_apart() ? 4u : 0u) ^ (b->set.stage() != 0u ? 8u : 0u);
}

void drop_graphs(wl_batch* b) {
  if (b->graph != nullptr) cudaGraphExecDestroy(b->graph);
  if (b->tile_graph != nullptr) cudaGraphExecDestroy(b->tile_graph);
  b->graph = nullptr;
  b->tile_graph = nullptr;
  b->graph_ticks = 0;
}

// The tuning cache: one entry per (SM count, size histogram), kept for the process and, when
// WLCUDA_TUNING_CACHE names a file, across processes.
std::mutex g_cache_mu;
std::map<std::string, wl_tuning> g_cache;

std::string histogram_key(int sms, const std::vector<wlc::TileSpec>& specs, uint8_t fixed) {
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> hist;
  for (const auto& s : specs) hist[{s.nx, s.ny}] += 1;
  std::ostringstream k;
  k << "sm" << sms << (fixed ? "/fixed" : "/native");
  for (const auto& [size, count] : hist) k << "/" << size.first << "x" << size.second << ":" << count;
  return k.str();
}

bool cache_lookup(const std::string& key, wl_tuning* out) {
  std::lock_guard<std::mutex> lock(g_cache_mu);
  auto it = g_cache.find(key);
  if (it == g_cache.end()) {
    const char* path = std::getenv("WLCUDA_TUNING_CACHE");
    if (path == nullptr) return false;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
      std::istringstream in(line);
      std::string k;
      wl_tuning t{};
      if (in >> k >> t.block_rows >> t.order >> t.us_per_tick) {
        if (!(in >> t.zero_apart)) t.zero_apart = 0;
        if (!(in >> t.stage)) t.stage = 0;
        g_cache[k] = t;
      }
    }
    it = g_cache.find(key);
    if (it == g_cache.end()) return false;
  }
  *out = it->second;
  return true;
}

void cache_store(const std::string& key, const wl_tuning& t) {
  std::lock_guard<std::mutex> lock(g_cache_mu);
  g_cache[key] = t;
  if (const char* path = std::getenv("WLCUDA_TUNING_CACHE")) {
    std::ofstream f(path, std::ios::app);
    f << key << " " << t.block_rows << " " << t.order << " " << t.us_per_tick << " "
      << t.zero_apart << " " << t.stage << "\n";
  }
}

// The untimed ticks an autotuner trial steps before it times.
constexpr uint32_t kTrialWarmTicks = 8;

bool time_ticks(wl_batch* b, uint32_t ticks, float max_dt, float* us, std::string* msg) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->set.stream());
  const cudaError_t e = b->set.enqueue_ticks(b->set.stream(), ticks, max_dt);
  cudaEventRecord(e1, b->set.stream());
  bool ok = e == cudaSuccess && b->set.wait(msg);
  float ms = 0.0f;
  if (ok) ok = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok && msg->empty()) *msg = "water_live: a trial tick failed";
  *us = ms * 1000.0f / float(ticks);
  return ok;
}

}  // namespace

extern "C" {

int wl_batch_create(const wl_config* common, const wl_options* options, const wl_tile* tiles,
                    uint32_t count, wl_batch** out, char* err, size_t err_len) {
  if (out == nullptr || common == nullptr || tiles == nullptr)
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no config or tiles");
  *out = nullptr;
  if (count == 0) return fail(err, err_len, WL_ERR_SIZE, "water_live: no tiles");
  auto* b = new (std::nothrow) wl_batch;
  if (b == nullptr) return fail(err, err_len, WL_ERR_ALLOC, "water_live: out of host memory");
  b->common = *common;
  if (options != nullptr) b->options = *options;
  b->specs.resize(count);
  for (uint32_t i = 0; i < count; ++i) {
    if (tiles[i].nx == 0 || tiles[i].ny == 0) {
      delete b;
      return fail(err, err_len, WL_ERR_SIZE, "water_live: an empty grid");
    }
    if (uint64_t(tiles[i].nx) * tiles[i].ny > wlc::kMaxTileCells) {
      delete b;
      return fail(err, err_len, WL_ERR_SIZE, "water_live: a grid of more than 2^30 cells");
    }
    wlc::TileSpec& s = b->specs[i];
    s.nx = tiles[i].nx;
    s.ny = tiles[i].ny;
    s.cell_m = common->cell_m;
    s.gravity = common->gravity;
    s.cfl = common->cfl;
    s.dry_depth_m = common->dry_depth_m;
    s.open_edges = (tiles[i].west_open ? 1u : 0u) | (tiles[i].east_open ? 2u : 0u) |
                   (tiles[i].south_open ? 4u : 0u) | (tiles[i].north_open ? 8u : 0u);
  }
  b->tuning.block_rows = 16;
  b->tuning.order = 1;
  b->tuning.us_per_tick = 0.0f;
  b->tuning.zero_apart = 0;
  b->tuning.stage = 0;
  std::string msg;
  if (!b->set.create(common->device, b->specs, b->options.ops == WL_OPS_FIXED,
                     shape_of_rows(b->tuning.block_rows), item_order(b->specs, b->tuning.order),
                     &msg)) {
    delete b;
    return cuda_fail(err, err_len, msg);
  }
  *out = b;
  return WL_OK;
}

void wl_batch_destroy(wl_batch* b) {
  if (b != nullptr && b->queue != nullptr) {
    b->queue->q.destroy();
    b->queue->owner = nullptr;
  }
  delete b;
}

uint32_t wl_batch_tile_count(const wl_batch* b) { return valid(b) ? b->set.tile_count() : 0u; }

uint64_t wl_batch_cell_count(const wl_batch* b) { return valid(b) ? b->set.total_cells() : 0u; }

uint32_t wl_batch_staged_tiles(const wl_batch* b) {
  return valid(b) ? b->set.staged_launch_tiles() : 0u;
}

uint64_t wl_batch_tile_first(const wl_batch* b, uint32_t tile) {
  return valid(b) && tile < b->set.tile_count() ? b->set.first_cell(tile) : 0u;
}

int wl_batch_write_state(wl_batch* b, const double* h, const double* hu, const double* hv,
                         size_t total, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (total != b->set.total_cells() || h == nullptr || hu == nullptr || hv == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: states that do not fit the tiles");
  std::string msg;
  if (!b->set.write_all(h, hu, hv, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_write_tile_state(wl_batch* b, uint32_t tile, const double* h, const double* hu,
                              const double* hv, size_t n, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (tile >= b->set.tile_count())
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no such tile");
  if (n != b->set.cells(tile) || h == nullptr || hu == nullptr || hv == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a state that does not fit the tile");
  std::string msg;
  if (!b->set.write_tile(tile, h, hu, hv, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_settled(wl_batch* b, const double* h, const double* hu, const double* hv,
                     size_t total, float depth_bound, float momentum_bound, uint8_t* settled,
                     float* depth_dev, float* momentum_dev, uint32_t count, char* err,
                     size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (total != b->set.total_cells() || h == nullptr || hu == nullptr || hv == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: steady states that do not fit the tiles");
  if (count != b->set.tile_count())
    return fail(err, err_len, WL_ERR_SIZE, "water_live: outputs that do not fit the tiles");
  std::string msg;
  if (!b->set.settled(true, 0, h, hu, hv, depth_bound, momentum_bound, settled, depth_dev,
                      momentum_dev, &msg))
    return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_set_bed(wl_batch* b, const double* bed, size_t total, double datum, char* err,
                     size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (total != b->set.total_cells() || bed == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: beds that do not fit the tiles");
  std::string msg;
  if (!b->set.set_plane_all(0, bed, datum, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_set_manning(wl_batch* b, const double* manning, size_t total, char* err,
                         size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  std::string msg;
  if (total == 0) {
    b->flags &= ~WL_FLAG_MANNING;
    if (!b->set.set_flags_all(0u, WL_FLAG_MANNING, b->source_every, false, &msg))
      return cuda_fail(err, err_len, msg);
    drop_graphs(b);
    return WL_OK;
  }
  if (total != b->set.total_cells() || manning == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a Manning's n that does not fit");
  if (!b->set.set_plane_all(1, manning, 0.0, &msg) ||
      !b->set.set_flags_all(WL_FLAG_MANNING, 0u, b->source_every, false, &msg))
    return cuda_fail(err, err_len, msg);
  b->flags |= WL_FLAG_MANNING;
  drop_graphs(b);
  return WL_OK;
}

int wl_batch_set_source(wl_batch* b, const double* source, size_t total, uint32_t every,
                        int compensate, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr && every > 1)
    return fail(err, err_len, WL_ERR_REFUSED,
                "water_live: a batch with a tick queue refuses a coarser source clock");
  b->source_every = every == 0 ? 1 : every;
  const uint32_t comp = compensate ? WL_FLAG_COMPENSATE : 0u;
  std::string msg;
  if (total == 0) {
    if (!b->set.set_flags_all(comp, WL_FLAG_SOURCE | (comp ? 0u : WL_FLAG_COMPENSATE),
                              b->source_every, true, &msg))
      return cuda_fail(err, err_len, msg);
    drop_graphs(b);
    return WL_OK;
  }
  if (total != b->set.total_cells() || source == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a source that does not fit");
  if (!b->set.set_plane_all(2, source, 0.0, &msg) ||
      !b->set.set_flags_all(WL_FLAG_SOURCE | comp, comp ? 0u : WL_FLAG_COMPENSATE,
                            b->source_every, true, &msg))
    return cuda_fail(err, err_len, msg);
  drop_graphs(b);
  return WL_OK;
}

int wl_batch_enqueue_ticks(wl_batch* b, wl_stream stream, uint32_t count, float max_dt) {
  if (!valid(b)) return WL_ERR_INVALID;
  if (b->queue != nullptr) return WL_ERR_REFUSED;
  if (cudaSetDevice(b->set.device()) != cudaSuccess) return WL_ERR_CUDA;
  cudaStream_t st = stream == nullptr ? b->set.stream() : reinterpret_cast<cudaStream_t>(stream);
  return b->set.enqueue_ticks(st, count, max_dt) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int wl_batch_run_ticks(wl_batch* b, uint32_t count, float max_dt, int use_graph, char* err,
                       size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (cudaSetDevice(b->set.device()) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  cudaStream_t st = b->set.stream();
  uint32_t left = count;
  if (use_graph && count > 0) {
    // One captured graph of up to 16 ticks (each a single persistent launch), replayed.
    const uint32_t g = count < 16 ? count : 16;
    const uint64_t key = launch_key(b);
    if (b->graph == nullptr || b->graph_ticks != g || b->graph_max_dt != max_dt ||
        b->graph_key != key) {
      if (b->graph != nullptr) cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaStreamBeginCapture");
      const cudaError_t e = b->set.enqueue_ticks(st, g, max_dt);
      const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
      if (e != cudaSuccess || e2 != cudaSuccess ||
          cudaGraphInstantiate(&b->graph, graph, 0) != cudaSuccess) {
        if (graph != nullptr) cudaGraphDestroy(graph);
        b->graph = nullptr;
        return fail(err, err_len, WL_ERR_CUDA, "water_live: the tick graph could not be made");
      }
      cudaGraphDestroy(graph);
      b->graph_ticks = g;
      b->graph_max_dt = max_dt;
      b->graph_key = key;
      b->graph_checks = b->set.pending_checks();
    }
    while (left >= b->graph_ticks) {
      if (cudaGraphLaunch(b->graph, st) != cudaSuccess)
        return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaGraphLaunch");
      b->set.add_checks(b->graph_checks);
      left -= b->graph_ticks;
    }
  }
  if (left > 0 && b->set.enqueue_ticks(st, left, max_dt) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: the tick");
  std::string msg;
  if (!b->set.wait(&msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_enqueue_tile_tick(wl_batch* b, wl_stream stream, uint32_t tile, float max_dt) {
  if (!valid(b)) return WL_ERR_INVALID;
  if (b->queue != nullptr) return WL_ERR_REFUSED;
  if (tile >= b->set.tile_count()) return WL_ERR_ARGUMENT;
  if (cudaSetDevice(b->set.device()) != cudaSuccess) return WL_ERR_CUDA;
  cudaStream_t st = stream == nullptr ? b->set.stream() : reinterpret_cast<cudaStream_t>(stream);
  return b->set.enqueue_tile_tick(st, tile, max_dt) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int wl_batch_run_tile_ticks(wl_batch* b, uint32_t count, float max_dt, int use_graph,
                            uint32_t streams, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (cudaSetDevice(b->set.device()) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  cudaStream_t st = b->set.stream();
  const uint32_t n = b->set.tile_count();
  if (streams > 1) {
    // Tiles dealt round-robin to concurrent streams, as independent steps with their own streams
    // would run; a tile's ticks stay in order on its stream.
    while (b->side_streams.size() < streams) {
      cudaStream_t s = nullptr;
      if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
        return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaStreamCreate");
      b->side_streams.push_back(s);
    }
    cudaEvent_t start;
    cudaEventCreateWithFlags(&start, cudaEventDisableTiming);
    cudaEventRecord(start, st);
    for (uint32_t k = 0; k < streams; ++k) cudaStreamWaitEvent(b->side_streams[k], start, 0);
    for (uint32_t k = 0; k < count; ++k)
      for (uint32_t t = 0; t < n; ++t)
        if (b->set.enqueue_tile_tick(b->side_streams[t % streams], t, max_dt) != cudaSuccess) {
          cudaEventDestroy(start);
          return fail(err, err_len, WL_ERR_CUDA, "water_live: a tile's tick");
        }
    for (uint32_t k = 0; k < streams; ++k) {
      cudaEvent_t done;
      cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
      cudaEventRecord(done, b->side_streams[k]);
      cudaStreamWaitEvent(st, done, 0);
      cudaEventDestroy(done);
    }
    cudaEventDestroy(start);
  } else if (use_graph) {
    const uint64_t key = launch_key(b);
    if (b->tile_graph == nullptr || b->tile_graph_max_dt != max_dt || b->tile_graph_key != key) {
      if (b->tile_graph != nullptr) cudaGraphExecDestroy(b->tile_graph);
      b->tile_graph = nullptr;
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaStreamBeginCapture");
      cudaError_t e = cudaSuccess;
      for (uint32_t t = 0; t < n && e == cudaSuccess; ++t) e = b->set.enqueue_tile_tick(st, t, max_dt);
      const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
      if (e != cudaSuccess || e2 != cudaSuccess ||
          cudaGraphInstantiate(&b->tile_graph, graph, 0) != cudaSuccess) {
        if (graph != nullptr) cudaGraphDestroy(graph);
        b->tile_graph = nullptr;
        return fail(err, err_len, WL_ERR_CUDA, "water_live: the per-tile graph could not be made");
      }
      cudaGraphDestroy(graph);
      b->tile_graph_max_dt = max_dt;
      b->tile_graph_key = key;
      b->tile_graph_checks = b->set.pending_checks();
    }
    for (uint32_t k = 0; k < count; ++k) {
      if (cudaGraphLaunch(b->tile_graph, st) != cudaSuccess)
        return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaGraphLaunch");
      b->set.add_checks(b->tile_graph_checks);
    }
  } else {
    for (uint32_t k = 0; k < count; ++k)
      for (uint32_t t = 0; t < n; ++t)
        if (b->set.enqueue_tile_tick(st, t, max_dt) != cudaSuccess)
          return fail(err, err_len, WL_ERR_CUDA, "water_live: a tile's tick");
  }
  std::string msg;
  if (!b->set.wait(&msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_read_tile_bits(wl_batch* b, uint32_t tile, float* planes, size_t count, char* err,
                            size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (tile >= b->set.tile_count() || planes == nullptr ||
      count != size_t(WL_STATE_PLANES) * b->set.cells(tile))
    return fail(err, err_len, WL_ERR_SIZE, "water_live: planes of the wrong size");
  std::string msg;
  if (!b->set.read_state_bits(tile, planes, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_read_all_bits(wl_batch* b, float* planes, size_t count, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (planes == nullptr || count != size_t(WL_STATE_PLANES) * b->set.total_cells())
    return fail(err, err_len, WL_ERR_SIZE, "water_live: planes of the wrong size");
  std::string msg;
  if (!b->set.read_all_bits(planes, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_batch_tile_hashes(wl_batch* b, uint64_t* out, uint32_t count, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (out == nullptr || count != b->set.tile_count())
    return fail(err, err_len, WL_ERR_SIZE, "water_live: hashes of the wrong count");
  std::vector<float> all;
  try {
    all.resize(size_t(WL_STATE_PLANES) * b->set.total_cells());
  } catch (...) {
    return fail(err, err_len, WL_ERR_ALLOC, "water_live: out of host memory");
  }
  std::string msg;
  if (!b->set.read_all_bits(all.data(), &msg)) return cuda_fail(err, err_len, msg);
  // FNV-1a is a sequence: each tile's hash is one pass; the tiles go to the host's threads.
  const uint32_t threads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (uint32_t w = 0; w < threads; ++w)
    pool.emplace_back([&, w] {
      for (uint32_t t = w; t < count; t += threads)
        out[t] = wlc::fnv1a_floats(all.data() + size_t(WL_STATE_PLANES) * b->set.first_cell(t),
                                   size_t(WL_STATE_PLANES) * b->set.cells(t));
    });
  for (auto& th : pool) th.join();
  return WL_OK;
}

uint64_t wl_batch_tile_hash(wl_batch* b, uint32_t tile, char* err, size_t err_len) {
  if (!valid(b)) {
    fail(err, err_len, WL_ERR_INVALID, k_no_device);
    return 0;
  }
  if (tile >= b->set.tile_count()) {
    fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no such tile");
    return 0;
  }
  std::vector<float> planes(size_t(WL_STATE_PLANES) * b->set.cells(tile));
  std::string msg;
  if (!b->set.read_state_bits(tile, planes.data(), &msg)) {
    cuda_fail(err, err_len, msg);
    return 0;
  }
  return wlc::fnv1a_floats(planes.data(), planes.size());
}

int wl_batch_read_ledgers(wl_batch* b, wl_ledger* out, uint32_t count, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (out == nullptr || count != b->set.tile_count())
    return fail(err, err_len, WL_ERR_SIZE, "water_live: ledgers of the wrong count");
  std::vector<wlc::TileCtl> ctl(count);
  std::string msg;
  if (!b->set.flush_all(&msg) || !b->set.read_all_ctl(ctl.data(), &msg))
    return cuda_fail(err, err_len, msg);
  for (uint32_t t = 0; t < count; ++t) {
    const wlc::LedgerBits& l = ctl[t].ledger[ctl[t].rec & 1u];
    out[t].source_m3 = double(l.source_hi) + double(l.source_lo);
    out[t].open_edge_out_m3 = double(l.open_hi) + double(l.open_lo);
    out[t].roundoff_m3 = double(l.roundoff_hi) + double(l.roundoff_lo);
    out[t].time_s = double(l.time_hi) + double(l.time_lo);
    out[t].remaining_s = double(l.remaining_s);
    out[t].steps = l.steps;
  }
  return WL_OK;
}

int wl_batch_set_tuning(wl_batch* b, const wl_tuning* t, char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (t == nullptr ||
      (t->block_rows != 1 && t->block_rows != 4 && t->block_rows != 16 && t->block_rows != 32 &&
       t->block_rows != 64) ||
      t->order > 1 || t->zero_apart > 1 || t->stage > 1)
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: a tuning out of range");
  std::string msg;
  if (!b->set.reshape(shape_of_rows(t->block_rows), item_order(b->specs, t->order), &msg))
    return cuda_fail(err, err_len, msg);
  b->set.set_zero_apart(t->zero_apart != 0);
  b->set.set_stage(t->stage != 0u ? wlc::TileSet::kStageOn : wlc::TileSet::kStageOff);
  b->tuning = *t;
  drop_graphs(b);
  return WL_OK;
}

int wl_batch_get_tuning(const wl_batch* b, wl_tuning* out) {
  if (!valid(b) || out == nullptr) return WL_ERR_INVALID;
  *out = b->tuning;
  return WL_OK;
}

int wl_batch_autotune(wl_batch* b, float max_dt, uint32_t trial_ticks, wl_tuning* chosen,
                      char* err, size_t err_len) {
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (cudaSetDevice(b->set.device()) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->set.device());
  const std::string key = histogram_key(sms, b->specs, b->options.ops);
  wl_tuning best{};
  std::string msg;
  if (!cache_lookup(key, &best)) {
    if (trial_ticks == 0) trial_ticks = 4;
    // Trials run on the batch's own state and are undone: a snapshot of everything a tick
    // writes is taken first and put back after.
    if (!b->set.snapshot(&msg)) return cuda_fail(err, err_len, msg);
    best.us_per_tick = std::numeric_limits<float>::infinity();
    // The zero-apart variant exists for the march's native plain form (16, 32, 64 rows).
    const bool zg_trial = b->options.ops != WL_OPS_FIXED && b->set.plain();
    // The staged variant exists for the three-phase blocks (1 row), where a tile takes it.
    const bool stage_trial = b->set.staged_tiles() > 0u;
    for (uint32_t rows : {1u, 4u, 16u, 32u, 64u}) {
      for (uint32_t order : {0u, 1u}) {
        for (uint32_t v : {0u, 1u}) {
          const uint32_t zg = rows >= 16u ? v : 0u, stage = rows == 1u ? v : 0u;
          if (v == 1u && !(zg_trial && rows >= 16u) && !(stage_trial && rows == 1u)) continue;
          if (!b->set.reshape(shape_of_rows(rows), item_order(b->specs, order), &msg) ||
              !b->set.restore(&msg))
            return cuda_fail(err, err_len, msg);
          b->set.set_zero_apart(zg != 0u);
          b->set.set_stage(stage != 0u ? wlc::TileSet::kStageOn : wlc::TileSet::kStageOff);
          // Each trial steps the same state past its first ticks untimed (a state as written is
          // often still: zero momenta, which flatter the zero-apart variant) and times the next
          // ones; every tuning steps to the same bytes, so each times the same ticks.
          float warm = 0.0f, us = 0.0f;
          if (!time_ticks(b, kTrialWarmTicks, max_dt, &warm, &msg) ||
              !time_ticks(b, trial_ticks, max_dt, &us, &msg))
            return cuda_fail(err, err_len, msg);
          if (us < best.us_per_tick) {
            best.block_rows = rows;
            best.order = order;
            best.us_per_tick = us;
            best.zero_apart = zg;
            best.stage = stage;
          }
        }
      }
    }
    if (!b->set.restore(&msg)) return cuda_fail(err, err_len, msg);
    b->set.drop_snapshot();
    cache_store(key, best);
  }
  if (!b->set.reshape(shape_of_rows(best.block_rows), item_order(b->specs, best.order), &msg))
    return cuda_fail(err, err_len, msg);
  b->set.set_zero_apart(best.zero_apart != 0u);
  b->set.set_stage(best.stage != 0u ? wlc::TileSet::kStageOn : wlc::TileSet::kStageOff);
  b->tuning = best;
  drop_graphs(b);
  if (chosen != nullptr) *chosen = best;
  return WL_OK;
}

wl_stream wl_batch_stream(wl_batch* b) {
  return valid(b) ? reinterpret_cast<wl_stream>(b->set.stream()) : nullptr;
}

int wl_batch_adjoint_create(wl_batch* batch, uint32_t ticks, uint32_t every,
                            const uint32_t* probe_first, const uint32_t* probes,
                            const double* targets, wl_adjoint** out, char* err, size_t err_len) {
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no handle to fill");
  *out = nullptr;
  if (!valid(batch)) return fail(err, err_len, WL_ERR_INVALID, "water_live: no batch");
  if (probe_first == nullptr)
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no probe offsets");
  if (probe_first[batch->set.tile_count()] > 0 && (probes == nullptr || targets == nullptr))
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no probes or targets");
  return wl_adjoint_create_over(&batch->set, ticks, every, probe_first, probes, targets, out, err,
                                err_len);
}

int wl_batch_queue_create(wl_batch* b, uint32_t records, uint32_t arena_values,
                          uint32_t max_events, wl_queue** out, char* err, size_t err_len) {
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no handle to fill");
  *out = nullptr;
  if (!valid(b)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (b->queue != nullptr)
    return fail(err, err_len, WL_ERR_REFUSED, "water_live: the batch has a tick queue already");
  if ((b->flags & WL_FLAG_SOURCE) != 0u && b->source_every > 1)
    return fail(err, err_len, WL_ERR_REFUSED,
                "water_live: a tick queue refuses a source on a coarser clock (set_source every > 1)");
  auto* q = new (std::nothrow) wl_queue;
  if (q == nullptr) return fail(err, err_len, WL_ERR_ALLOC, "water_live: host memory");
  std::string msg;
  if (!q->q.create(&b->set, records, arena_values, max_events, &msg)) {
    delete q;
    const int code = msg.find("holds 1 to 64") != std::string::npos ? WL_ERR_ARGUMENT : WL_ERR_CUDA;
    return fail(err, err_len, code, msg);
  }
  q->owner = &b->queue;
  b->queue = q;
  *out = q;
  return WL_OK;
}

}  // extern "C"

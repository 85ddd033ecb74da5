// The C ABI of include/wlcuda.h: water_live::DeviceStep's calls over a TileSet of one tile.
// Each function names the reference call it stands in for (systems/water_live/src/water_live.cpp).
#include "wlcuda.h"

#include "wl_adjoint.h"
#include "wl_queue.h"
#include "wl_tiles.h"

#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

using wlc::TileSet;

struct wl_step {
  TileSet set;
  wl_config config{};
  wl_options options{};
  uint32_t flags = 0;  // the reference's flags_ (water_live.h:239)
  uint32_t source_every = 1;
  uint32_t cells = 0;
  uint32_t groups = 0;
  wl_queue* queue = nullptr;  // the tick queue attached, which owns the step's clock
};


// The mirrored structs keep the reference's sizes and offsets (water_live_tests.cpp:22-36,
// size_table.cpp:8-10).
static_assert(sizeof(wl_step_params) == 120, "StepParams is 120 bytes");
static_assert(offsetof(wl_step_params, ledger) == 48, "");
static_assert(offsetof(wl_step_params, nx) == 56, "");
static_assert(offsetof(wl_step_params, flags) == 72, "");
static_assert(offsetof(wl_step_params, max_dt) == 92, "");
static_assert(offsetof(wl_step_params, source_scale) == 96, "");
static_assert(offsetof(wl_step_params, faces_x) == 104, "");
static_assert(offsetof(wl_step_params, faces_y) == 112, "");
static_assert(sizeof(wl_partial) == 32 && offsetof(wl_partial, roundoff_m3) == 16, "");
static_assert(sizeof(wl_ledger_bits) == 48, "");
static_assert(offsetof(wl_ledger_bits, remaining_s) == 32, "");
static_assert(offsetof(wl_ledger_bits, dt) == 36, "");
static_assert(offsetof(wl_ledger_bits, steps) == 40, "");
static_assert(sizeof(wl_partial) == sizeof(wlc::Partial), "");
static_assert(sizeof(wl_ledger_bits) == sizeof(wlc::LedgerBits), "");

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

bool valid(const wl_step* s) { return s != nullptr && s->set.valid(); }

const char* k_no_device = "water_live: no device";
const char* k_queued = "water_live: the step's tick queue owns its clock (destroy the queue first)";

int flush(wl_step* s, wl_ledger_bits* bits, std::string* msg) {
  if (!s->set.length_pass(0, 0.0f, msg)) return WL_ERR_CUDA;
  wlc::TileCtl c;
  if (!s->set.read_ctl(0, c, msg)) return WL_ERR_CUDA;
  std::memcpy(bits, &c.ledger[c.rec & 1u], sizeof *bits);
  return WL_OK;
}

void widen(const wl_ledger_bits& l, wl_ledger* out) {  // water_live.cpp:374-379
  out->source_m3 = double(l.source_hi) + double(l.source_lo);
  out->open_edge_out_m3 = double(l.open_hi) + double(l.open_lo);
  out->roundoff_m3 = double(l.roundoff_hi) + double(l.roundoff_lo);
  out->time_s = double(l.time_hi) + double(l.time_lo);
  out->remaining_s = double(l.remaining_s);
  out->steps = l.steps;
}

}  // namespace

extern "C" {

int wl_create(const wl_config* config, const wl_options* options, wl_step** out, char* err,
              size_t err_len) {
  if (out == nullptr || config == nullptr)
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no config");
  *out = nullptr;
  if (config->nx == 0 || config->ny == 0)  // water_live.cpp:108
    return fail(err, err_len, WL_ERR_SIZE, "water_live: an empty grid");
  if (uint64_t(config->nx) * config->ny > wlc::kMaxTileCells)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a grid of more than 2^30 cells");
  auto* s = new (std::nothrow) wl_step;
  if (s == nullptr) return fail(err, err_len, WL_ERR_ALLOC, "water_live: out of host memory");
  s->config = *config;
  if (options != nullptr) s->options = *options;
  wlc::TileSpec t;
  t.nx = config->nx;
  t.ny = config->ny;
  t.cell_m = config->cell_m;
  t.gravity = config->gravity;
  t.cfl = config->cfl;
  t.dry_depth_m = config->dry_depth_m;
  s->flags = 0;
  if (config->west_open) s->flags |= WL_FLAG_WEST_OPEN;
  if (config->east_open) s->flags |= WL_FLAG_EAST_OPEN;
  if (config->south_open) s->flags |= WL_FLAG_SOUTH_OPEN;
  if (config->north_open) s->flags |= WL_FLAG_NORTH_OPEN;
  if (s->options.stored_faces) s->flags |= WL_FLAG_STORED_FACES;
  t.open_edges = s->flags & 15u;
  // The block shape: the 32 x 16 march, or the three-phase 32 x 16 blocks where the march's
  // 32 x 32 items would leave the device short of warps (fewer than eight an SM) and for the
  // stored-faces form (the block form stores every face once, in shared memory, and gathers it:
  // slang:483-551's order of work, the same bytes); WLCUDA_BLOCK_ROWS (1, 4, 16, 32 or 64)
  // overrides.
  wlc::BlockShape shape = wlc::BlockShape::k32x16;
  {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, config->device) !=
        cudaSuccess)
      sms = 0;
    const uint64_t items32 = uint64_t((config->nx + 31u) / 32u) * ((config->ny + 31u) / 32u);
    if ((sms > 0 && items32 < uint64_t(sms) * 8u) || s->options.stored_faces)
      shape = wlc::BlockShape::k32x16b;
  }
  if (const char* rows = std::getenv("WLCUDA_BLOCK_ROWS")) {
    if (std::strcmp(rows, "1") == 0) shape = wlc::BlockShape::k32x16b;
    if (std::strcmp(rows, "4") == 0) shape = wlc::BlockShape::k32x16s;
    if (std::strcmp(rows, "16") == 0) shape = wlc::BlockShape::k32x16;
    if (std::strcmp(rows, "32") == 0) shape = wlc::BlockShape::k32x32;
    if (std::strcmp(rows, "64") == 0) shape = wlc::BlockShape::k32x64;
  }
  std::string msg;
  if (!s->set.create(config->device, {t}, s->options.ops == WL_OPS_FIXED, shape, {}, &msg)) {
    delete s;
    return cuda_fail(err, err_len, msg);
  }
  // The block shape's staged variant (a block's cells and halo by tensor copies, where the tile's
  // width is a multiple of 4): by default where a launch of 256-thread block CTAs holds more blocks
  // than CTAs; WLCUDA_STAGE=1 in every block launch, 0 in none. The same bytes either way.
  s->set.set_stage(wlc::TileSet::kStageAuto);
  if (const char* stage = std::getenv("WLCUDA_STAGE")) {
    if (std::strcmp(stage, "0") == 0) s->set.set_stage(wlc::TileSet::kStageOff);
    if (std::strcmp(stage, "1") == 0) s->set.set_stage(wlc::TileSet::kStageOn);
  }
  s->cells = config->nx * config->ny;
  s->groups = ((config->nx + 15) / 16) * ((config->ny + 15) / 16);
  *out = s;
  return WL_OK;
}

void wl_destroy(wl_step* step) {
  if (step != nullptr && step->queue != nullptr) {
    step->queue->q.destroy();
    step->queue->owner = nullptr;
  }
  delete step;
}

int wl_valid(const wl_step* step) { return valid(step) ? 1 : 0; }

uint32_t wl_cell_count(const wl_step* step) { return valid(step) ? step->cells : 0u; }

uint32_t wl_group_count(const wl_step* step) { return valid(step) ? step->groups : 0u; }

uint64_t wl_tick_launches(const wl_step* step) {
  return valid(step) ? step->set.tick_launches() : 0u;
}

uint32_t wl_staged_tiles(const wl_step* step) {
  return valid(step) ? step->set.staged_launch_tiles() : 0u;
}

int wl_write_state(wl_step* s, const double* h, const double* hu, const double* hv, size_t n,
                   char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  // A new state empties the ledger, time left included: the queue's tick in flight could not land.
  if (s->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (n != s->cells || h == nullptr || hu == nullptr || hv == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a state that does not fit the grid");
  std::string msg;
  if (!s->set.write_state(0, h, hu, hv, &msg) || !s->set.prime(&msg))
    return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_read_state(wl_step* s, double* h, double* hu, double* hv, size_t n, char* err,
                  size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (n != s->cells || h == nullptr || hu == nullptr || hv == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a state that does not fit the grid");
  std::string msg;
  if (!s->set.read_state(0, h, hu, hv, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_read_state_bits(wl_step* s, float* planes, size_t count, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (planes == nullptr || count != size_t(WL_STATE_PLANES) * s->cells)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: planes of the wrong size");
  std::string msg;
  if (!s->set.read_state_bits(0, planes, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_read_ledger(wl_step* s, wl_ledger* out, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no ledger");
  wl_ledger_bits l;
  std::string msg;
  if (flush(s, &l, &msg) != WL_OK) return cuda_fail(err, err_len, msg);
  widen(l, out);
  return WL_OK;
}

int wl_settled(wl_step* s, const double* h, const double* hu, const double* hv, size_t n,
               float depth_bound, float momentum_bound, uint8_t* settled, float* depth_dev,
               float* momentum_dev, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (n != s->cells || h == nullptr || hu == nullptr || hv == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a steady state that does not fit the grid");
  std::string msg;
  if (!s->set.settled(false, 0, h, hu, hv, depth_bound, momentum_bound, settled, depth_dev,
                      momentum_dev, &msg))
    return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_set_bed(wl_step* s, const double* bed, size_t n, double datum, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (n != s->cells || bed == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a bed that does not fit the grid");
  std::string msg;
  if (!s->set.set_plane(0, 0, bed, datum, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_set_manning(wl_step* s, const double* manning, size_t n, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  std::string msg;
  if (n == 0) {
    s->flags &= ~WL_FLAG_MANNING;
    if (!s->set.set_flags(0, s->flags, s->source_every, false, &msg))
      return cuda_fail(err, err_len, msg);
    return WL_OK;
  }
  if (n != s->cells || manning == nullptr)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a Manning's n that does not fit");
  if (!s->set.set_plane(0, 1, manning, 0.0, &msg)) return cuda_fail(err, err_len, msg);
  s->flags |= WL_FLAG_MANNING;
  if (!s->set.set_flags(0, s->flags, s->source_every, false, &msg))
    return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_set_source(wl_step* s, const double* source, size_t n, uint32_t every, int compensate,
                  char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  // A coarser source clock cannot follow the sub-steps a queue's card chooses (water_live.md:92).
  if (s->queue != nullptr && every > 1)
    return fail(err, err_len, WL_ERR_REFUSED,
                "water_live: a step with a tick queue refuses a coarser source clock");
  // water_live.cpp:465-486: the clock and the compensation change even when the source is refused.
  s->source_every = every == 0 ? 1 : every;
  if (compensate) s->flags |= WL_FLAG_COMPENSATE;
  else s->flags &= ~WL_FLAG_COMPENSATE;
  std::string msg;
  if (n == 0) {
    s->flags &= ~WL_FLAG_SOURCE;
    if (!s->set.set_flags(0, s->flags, s->source_every, true, &msg))
      return cuda_fail(err, err_len, msg);
    return WL_OK;
  }
  if (n != s->cells || source == nullptr) {
    if (!s->set.set_flags(0, s->flags, s->source_every, true, &msg))
      return cuda_fail(err, err_len, msg);
    return fail(err, err_len, WL_ERR_SIZE, "water_live: a source that does not fit");
  }
  if (!s->set.set_plane(0, 2, source, 0.0, &msg)) return cuda_fail(err, err_len, msg);
  s->flags |= WL_FLAG_SOURCE;
  if (!s->set.set_flags(0, s->flags, s->source_every, true, &msg))
    return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_enqueue_steps(wl_step* s, wl_stream stream, uint32_t count, float max_dt) {
  if (!valid(s)) return WL_ERR_INVALID;
  if (s->queue != nullptr) return WL_ERR_REFUSED;
  cudaStream_t st = stream == nullptr ? s->set.stream() : reinterpret_cast<cudaStream_t>(stream);
  if (cudaSetDevice(s->set.device()) != cudaSuccess) return WL_ERR_CUDA;
  return s->set.enqueue_ticks(st, count, max_dt) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int wl_run_steps(wl_step* s, uint32_t count, float max_dt, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (s->queue != nullptr) return fail(err, err_len, WL_ERR_REFUSED, k_queued);
  if (cudaSetDevice(s->set.device()) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  const cudaError_t e = s->set.enqueue_ticks(s->set.stream(), count, max_dt);
  if (e != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, std::string("water_live: the tick: ") + cudaGetErrorString(e));
  std::string msg;
  if (!s->set.wait(&msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

uint64_t wl_advance(wl_step* s, double duration_s, char* err, size_t err_len) {
  if (!valid(s)) {
    fail(err, err_len, WL_ERR_INVALID, k_no_device);
    return 0;
  }
  if (!(duration_s > 0.0)) return 0;
  if (s->queue != nullptr) {
    fail(err, err_len, WL_ERR_REFUSED, k_queued);
    return 0;
  }
  // water_live.cpp:600-606: a coarser source clock counts steps on the host; refused.
  if ((s->flags & WL_FLAG_SOURCE) != 0u && s->source_every > 1) {
    fail(err, err_len, WL_ERR_REFUSED,
         "water_live: advance refuses a source on a coarser clock (set_source every > 1)");
    return 0;
  }
  constexpr uint32_t k_batch = 64;
  constexpr uint32_t k_most_batches = 1u << 16;
  std::string msg;
  wl_ledger_bits start, now, end;
  if (flush(s, &start, &msg) != WL_OK ||
      !s->set.set_remaining(0, static_cast<float>(duration_s), &msg)) {
    cuda_fail(err, err_len, msg);
    return 0;
  }
  const float inf = std::numeric_limits<float>::infinity();
  bool done = false;
  for (uint32_t batch = 0; batch < k_most_batches && !done; ++batch) {
    if (s->set.enqueue_ticks(s->set.stream(), k_batch, inf) != cudaSuccess) {
      fail(err, err_len, WL_ERR_CUDA, "water_live: the tick");
      return 0;
    }
    if (flush(s, &now, &msg) != WL_OK) {
      cuda_fail(err, err_len, msg);
      return 0;
    }
    done = !(double(now.remaining_s) > 0.0);
  }
  if (flush(s, &end, &msg) != WL_OK || !s->set.set_remaining(0, inf, &msg)) {
    cuda_fail(err, err_len, msg);
    return 0;
  }
  if (!done) {
    fail(err, err_len, WL_ERR_UNFINISHED, "water_live: the advance did not finish");
    return 0;
  }
  return uint64_t(end.steps) - uint64_t(start.steps);
}

uint64_t wl_state_hash(wl_step* s, char* err, size_t err_len) {
  if (!valid(s)) {
    fail(err, err_len, WL_ERR_INVALID, k_no_device);
    return 0;
  }
  std::vector<float> planes(size_t(WL_STATE_PLANES) * s->cells);
  std::string msg;
  if (!s->set.read_state_bits(0, planes.data(), &msg)) {
    cuda_fail(err, err_len, msg);
    return 0;
  }
  return wlc::fnv1a_floats(planes.data(), planes.size());
}

int wl_read_partials_bits(wl_step* s, wl_partial* out, size_t count, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (out == nullptr || count != s->groups)
    return fail(err, err_len, WL_ERR_SIZE, "water_live: records of the wrong count");
  std::string msg;
  if (!s->set.read_partials(0, reinterpret_cast<wlc::Partial*>(out), &msg))
    return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_read_ledger_bits(wl_step* s, wl_ledger_bits* out, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no ledger");
  wlc::TileCtl c;
  std::string msg;
  if (!s->set.read_ctl(0, c, &msg)) return cuda_fail(err, err_len, msg);
  std::memcpy(out, &c.ledger[c.rec & 1u], sizeof *out);
  return WL_OK;
}

int wl_run_length_pass(wl_step* s, float max_dt, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  std::string msg;
  if (!s->set.length_pass(0, max_dt, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

uint64_t wl_hash_floats(const float* values, size_t count) {
  if (values == nullptr) count = 0;
  return wlc::fnv1a_floats(values, count);
}

int wl_resident_barrier_check(int device, uint32_t ctas, char* err, size_t err_len) {
  if (ctas < 2 || ctas > 64) return fail(err, err_len, WL_ERR_INVALID, "water_live: 2 to 64 CTAs");
  if (cudaSetDevice(device) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  wlc::ResidentCtl* rc = nullptr;
  if (cudaMalloc(&rc, sizeof(wlc::ResidentCtl)) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaMalloc");
  cudaStream_t s = nullptr;
  int rc_out = WL_OK;
  wlc::ResidentCtl word = {};
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      wlc::launch_barrier_probe(rc, ctas, s) != cudaSuccess) {
    rc_out = fail(err, err_len, WL_ERR_CUDA, std::string("water_live: the barrier probe: ") +
                                                 cudaGetErrorString(cudaGetLastError()));
  } else {
    bool timed_out = false;
    const cudaError_t e = wlc::wait_stream(s, &timed_out);
    if (timed_out || e != cudaSuccess ||
        cudaMemcpy(&word, rc, sizeof word, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc_out = fail(err, err_len, WL_ERR_CUDA, "water_live: the barrier probe did not finish");
    else if (word.error == 0u || word.arrived != ctas - 1u)
      rc_out = fail(err, err_len, WL_ERR_CUDA, "water_live: the barrier's wait did not give up");
  }
  if (s != nullptr) cudaStreamDestroy(s);
  cudaFree(rc);
  return rc_out;
}

wl_stream wl_step_stream(wl_step* s) {
  return valid(s) ? reinterpret_cast<wl_stream>(s->set.stream()) : nullptr;
}

int wl_write_state_device(wl_step* s, const float* planes, wl_stream stream) {
  if (!valid(s)) return WL_ERR_INVALID;
  if (s->queue != nullptr) return WL_ERR_REFUSED;
  if (planes == nullptr) return WL_ERR_ARGUMENT;
  if (cudaSetDevice(s->set.device()) != cudaSuccess) return WL_ERR_CUDA;
  cudaStream_t st = stream == nullptr ? s->set.stream() : reinterpret_cast<cudaStream_t>(stream);
  if (wlc::launch_write_state_f32(s->set.device_descs(), 0, s->cells, planes, st) != cudaSuccess)
    return WL_ERR_CUDA;
  return s->set.enqueue_prime(st) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int wl_device_planes(wl_step* s, float** planes, float** bed, char* err, size_t err_len) {
  if (!valid(s)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  wlc::TileCtl c;
  std::string msg;
  if (!s->set.read_ctl(0, c, &msg)) return cuda_fail(err, err_len, msg);
  if (planes) *planes = s->set.device_state(0, c.cur & 1u);
  if (bed) *bed = const_cast<float*>(s->set.desc(0).bed);
  return WL_OK;
}

int wl_adjoint_create(wl_step* step, uint32_t ticks, uint32_t every, uint32_t n_probes,
                      const uint32_t* probes, const double* targets, wl_adjoint** out, char* err,
                      size_t err_len) {
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no handle to fill");
  *out = nullptr;
  if (!valid(step)) return fail(err, err_len, WL_ERR_INVALID, "water_live: no step");
  if (n_probes > 0 && (probes == nullptr || targets == nullptr))
    return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no probes or targets");
  const uint32_t first[2] = {0u, n_probes};
  return wl_adjoint_create_over(&step->set, ticks, every, first, probes, targets, out, err,
                                err_len);
}

// ---- the tick queue (water_live.md:76-94) -----------------------------------------------------

int wl_queue_create(wl_step* step, uint32_t records, uint32_t arena_values, uint32_t max_events,
                    wl_queue** out, char* err, size_t err_len) {
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no handle to fill");
  *out = nullptr;
  if (!valid(step)) return fail(err, err_len, WL_ERR_INVALID, k_no_device);
  if (step->queue != nullptr)
    return fail(err, err_len, WL_ERR_REFUSED, "water_live: the step has a tick queue already");
  if ((step->flags & WL_FLAG_SOURCE) != 0u && step->source_every > 1)
    return fail(err, err_len, WL_ERR_REFUSED,
                "water_live: a tick queue refuses a source on a coarser clock (set_source every > 1)");
  auto* q = new (std::nothrow) wl_queue;
  if (q == nullptr) return fail(err, err_len, WL_ERR_ALLOC, "water_live: host memory");
  std::string msg;
  if (!q->q.create(&step->set, records, arena_values, max_events, &msg)) {
    delete q;
    const int code = msg.find("holds 1 to 64") != std::string::npos ? WL_ERR_ARGUMENT : WL_ERR_CUDA;
    return fail(err, err_len, code, msg);
  }
  q->owner = &step->queue;
  step->queue = q;
  *out = q;
  return WL_OK;
}

void wl_queue_destroy(wl_queue* queue) {
  if (queue == nullptr) return;
  if (queue->owner != nullptr) {
    queue->q.destroy();
    *queue->owner = nullptr;
  }
  delete queue;
}

int wl_queue_push(wl_queue* queue, uint32_t tick, float length_s, const wl_event* events,
                  uint32_t n_events, const float* values, size_t n_values, char* err,
                  size_t err_len) {
  if (queue == nullptr || queue->owner == nullptr || !queue->q.valid())
    return fail(err, err_len, WL_ERR_INVALID, "water_live: no queue");
  std::string msg;
  const int rc = queue->q.push(tick, length_s, events, n_events, values, n_values, &msg);
  return rc == WL_OK ? WL_OK : fail(err, err_len, rc, msg);
}

int wl_queue_enqueue_slots(wl_queue* queue, wl_stream stream, uint32_t slots) {
  if (queue == nullptr || queue->owner == nullptr || !queue->q.valid()) return WL_ERR_INVALID;
  cudaStream_t st = stream == nullptr ? queue->q.stream() : reinterpret_cast<cudaStream_t>(stream);
  if (cudaSetDevice(queue->q.device()) != cudaSuccess) return WL_ERR_CUDA;
  return queue->q.enqueue(st, slots) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int wl_queue_run_slots(wl_queue* queue, uint32_t slots, char* err, size_t err_len) {
  if (queue == nullptr || queue->owner == nullptr || !queue->q.valid())
    return fail(err, err_len, WL_ERR_INVALID, "water_live: no queue");
  if (cudaSetDevice(queue->q.device()) != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  const cudaError_t e = queue->q.enqueue(queue->q.stream(), slots);
  if (e != cudaSuccess)
    return fail(err, err_len, WL_ERR_CUDA, std::string("water_live: the slots: ") + cudaGetErrorString(e));
  std::string msg;
  if (!queue->q.wait(&msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_queue_status_read(wl_queue* queue, wl_queue_status* out, char* err, size_t err_len) {
  if (queue == nullptr || queue->owner == nullptr || !queue->q.valid())
    return fail(err, err_len, WL_ERR_INVALID, "water_live: no queue");
  if (out == nullptr) return fail(err, err_len, WL_ERR_ARGUMENT, "water_live: no status to fill");
  wlc::QueueCtl c;
  std::string msg;
  if (!queue->q.read_ctl(c, &msg)) return cuda_fail(err, err_len, msg);
  std::memset(out, 0, sizeof *out);
  out->pushed = c.head;
  out->begun = c.begun;
  out->landed = c.landed;
  out->active = c.active;
  out->substeps = c.substeps;
  out->dropped = c.dropped;
  out->frozen = c.frozen;
  out->freezes = c.freezes;
  return WL_OK;
}

int wl_queue_set_limits(wl_queue* queue, uint32_t lag_limit_ticks, uint32_t max_slots, char* err,
                        size_t err_len) {
  if (queue == nullptr || queue->owner == nullptr || !queue->q.valid())
    return fail(err, err_len, WL_ERR_INVALID, "water_live: no queue");
  std::string msg;
  if (!queue->q.set_limits(lag_limit_ticks, max_slots, &msg)) return cuda_fail(err, err_len, msg);
  return WL_OK;
}

int wl_queue_read_landed(wl_queue* queue, uint32_t first, uint32_t count, wl_landed* out,
                         char* err, size_t err_len) {
  if (queue == nullptr || queue->owner == nullptr || !queue->q.valid())
    return fail(err, err_len, WL_ERR_INVALID, "water_live: no queue");
  std::string msg;
  if (!queue->q.read_landed(first, count, out, &msg)) {
    const int code = msg.find("not held") != std::string::npos ? WL_ERR_ARGUMENT : WL_ERR_CUDA;
    return fail(err, err_len, code, msg);
  }
  return WL_OK;
}

uint32_t wl_queue_launches_per_slot(void) { return 2u; }

uint64_t wl_queue_device_bytes(const wl_queue* queue) {
  return queue != nullptr && queue->owner != nullptr ? queue->q.device_bytes() : 0u;
}

}  // extern "C"

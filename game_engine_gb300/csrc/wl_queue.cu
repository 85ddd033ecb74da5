// The tick queue's kernels and host side (wl_queue.h). A slot is two launches on one stream:
//
//   queue_slot_kernel   one CTA. Its thread 0 settles the last slot (counts its sub-step, lands a
//                       tick whose time left reached zero, releases the events the last slot
//                       applied), then, when no tick is in flight and one is queued, begins it by
//                       setting the step's time left to its length, and writes the slot's `go`.
//                       Then the CTA writes the begun tick's events into the step's planes, in
//                       push order.
//   the tick            the step's own persistent tick (wl_kernels.cu) with max_dt = +inf, so a
//                       sub-step is min(stable step, time left); it returns at once when `go` is 0.
//
// The time left is the reference's ledger field (WaterLedger::remaining_s, water_live.h:124-137)
// that its advance counts down (water_live.cpp:590-639), so a queued tick takes the sub-steps
// wl_advance takes for the same length. The begun tick's events write the planes before its first
// sub-step and after the last sub-step of the tick before: the tick's own boundary
// (water_live.md:86). A bed, source or Manning plane enters no record (the records hold the
// state's speeds and volumes), so such an event needs no prime; a state event (a waking tile's
// starting state) folds the tile's pending records into its ledger first and primes the records
// of what it wrote after (write_state_event).
//
// The lag control (water_live.md:90-92): a begin that finds more ticks pushed and not landed than
// the queue's lag limit freezes the domain as it stands. A frozen domain drops each tick it
// begins, one a slot: the tick's events are applied in order, it takes no sub-step (its length is
// taken as 0) and lands at once, counted and marked dropped, until the queue has drained; the
// landing that drains it thaws the domain.
#include "wl_kernels.h"
#include "wl_queue.h"

#include <algorithm>
#include <cstring>
#include <limits>
#include <vector>

namespace wlc {
namespace {

constexpr uint32_t kMaxRecords = 64;  // water_live.md:84
constexpr int kApplyThreads = 1024;

// The tick in flight's read-back record (tile 0's ledger time and step count, the drop counts and
// the lag), and the queue free for the next. A dropped landing that leaves nothing queued (`head`
// ticks pushed, all begun) thaws the domain.
__device__ void land(QueueCtl* q, const LedgerBits& l, wl_landed* landed, uint32_t records,
                     uint32_t head) {
  wl_landed r;
  r.tick = q->tick;
  r.substeps = q->substeps;
  r.shortest_s = q->substeps != 0u ? q->shortest : 0.0f;
  r.longest_s = q->longest;
  r.time_hi = l.time_hi;
  r.time_lo = l.time_lo;
  r.steps = l.steps;
  r.events = q->events;
  r.dropped = q->dropping;
  if (q->dropping != 0u) {
    q->dropped += 1u;
    if (q->begun == head) q->frozen = 0u;
  }
  r.dropped_total = q->dropped;
  r.lag = q->lag;
  r.frozen = q->frozen;
  landed[q->landed % records] = r;
  q->landed += 1u;
  q->active = 0u;
  q->dropping = 0u;
}

// A state event (WL_EVENT_STATE) by the slot kernel's CTA, in the order the reference's slot
// gives (water_live.md:86: apply, then prime where the state changed):
//   1. the tile's pending records folded into its ledger: dt_main with max_dt 0 (slang:412-479),
//      256 virtual lanes each a strided sum over the records, then the fixed tree, then the three
//      pair_adds; the records' volumes cleared;
//   2. the rectangle's h, hu, hv written into the current copy, its remainder zeroed;
//   3. the records of the groups the rectangle touches recomputed from the new state (their
//      largest |u| + c and |v| + c, as prime_main: the other groups' records already hold the
//      speeds of the state as it stands and, after step 1, no volume), and the tile's largest
//      speeds, from which the next sub-step's length is chosen, taken again over every record.
// No tick runs while a slot kernel does, so the control block's slots stand still.
__device__ void write_state_event(const TileDesc& T, const QueueEvent& ev, const float* src,
                                  int fixed, float* s_sum, uint32_t* s_ab) {
  const uint32_t t = threadIdx.x;
  TileCtl* c = T.ctl;
  const uint32_t rec = c->rec;
  Partial* recs = T.rec[rec];
  const uint32_t groups = T.groups_x * T.groups_y;
  // 1. The flush.
  if (t < kGroupCells) {
    float sv = 0.0f, ov = 0.0f, rv = 0.0f;
    for (uint32_t gi = t; gi < groups; gi += kGroupCells) {
      sv = __fadd_rn(sv, recs[gi].source_m3);
      ov = __fadd_rn(ov, recs[gi].open_m3);
      rv = __fadd_rn(rv, recs[gi].roundoff_m3);
      recs[gi].source_m3 = 0.0f;
      recs[gi].open_m3 = 0.0f;
      recs[gi].roundoff_m3 = 0.0f;
    }
    s_sum[t] = sv;
    s_sum[kGroupCells + t] = ov;
    s_sum[2 * kGroupCells + t] = rv;
  }
  __syncthreads();
  for (uint32_t stride = kGroupCells / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      s_sum[t] = __fadd_rn(s_sum[t], s_sum[t + stride]);
      s_sum[kGroupCells + t] = __fadd_rn(s_sum[kGroupCells + t], s_sum[kGroupCells + t + stride]);
      s_sum[2 * kGroupCells + t] =
          __fadd_rn(s_sum[2 * kGroupCells + t], s_sum[2 * kGroupCells + t + stride]);
    }
    __syncthreads();
  }
  if (t == 0) {
    LedgerBits l = c->ledger[rec];
    pair_add(l.source_hi, l.source_lo, s_sum[0]);
    pair_add(l.open_hi, l.open_lo, s_sum[kGroupCells]);
    pair_add(l.roundoff_hi, l.roundoff_lo, s_sum[2 * kGroupCells]);
    l.dt = 0.0f;
    c->ledger[rec] = l;
    s_ab[0] = 0u;
    s_ab[1] = 0u;
  }
  // 2. The rectangle.
  const size_t n = size_t(T.nx) * T.ny;
  float* st = T.state[c->cur];
  const uint32_t count = ev.w * ev.h;
  for (uint32_t k = t; k < count; k += blockDim.x) {
    const uint32_t y = k / ev.w, x = k - y * ev.w;
    const size_t i = size_t(ev.y0 + y) * T.nx + ev.x0 + x;
    st[i] = src[k];
    st[n + i] = src[count + k];
    st[2 * n + i] = src[2 * size_t(count) + k];
    st[3 * n + i] = 0.0f;
  }
  // 3. The touched groups' records.
  const uint32_t gx0 = ev.x0 / kGroupSide, gx1 = (ev.x0 + ev.w - 1u) / kGroupSide;
  const uint32_t gy0 = ev.y0 / kGroupSide, gy1 = (ev.y0 + ev.h - 1u) / kGroupSide;
  const uint32_t gw = gx1 - gx0 + 1u, ng = gw * (gy1 - gy0 + 1u);
  __syncthreads();
  for (uint32_t k = t; k < ng; k += blockDim.x) {
    const uint32_t g = (gy0 + k / gw) * T.groups_x + gx0 + k % gw;
    recs[g].speed_x = 0.0f;
    recs[g].speed_y = 0.0f;
  }
  __syncthreads();
  for (uint32_t k = t; k < ng * kGroupCells; k += blockDim.x) {
    const uint32_t gk = k / kGroupCells, slot = k % kGroupCells;
    const uint32_t gxk = gx0 + gk % gw, gyk = gy0 + gk / gw;
    const uint32_t x = gxk * kGroupSide + slot % kGroupSide;
    const uint32_t y = gyk * kGroupSide + slot / kGroupSide;
    if (x >= T.nx || y >= T.ny) continue;
    const size_t i = size_t(y) * T.nx + x;
    float ax, ay;
    if (fixed != 0) cell_speeds<true>(T.gravity, T.dry, st[i], st[n + i], st[2 * n + i], ax, ay);
    else cell_speeds<false>(T.gravity, T.dry, st[i], st[n + i], st[2 * n + i], ax, ay);
    Partial* p = recs + size_t(gyk) * T.groups_x + gxk;
    atomicMax(reinterpret_cast<uint32_t*>(&p->speed_x), __float_as_uint(ax));
    atomicMax(reinterpret_cast<uint32_t*>(&p->speed_y), __float_as_uint(ay));
  }
  __syncthreads();
  uint32_t a = 0u, b = 0u;
  for (uint32_t g = t; g < groups; g += blockDim.x) {
    a = max(a, __float_as_uint(recs[g].speed_x));
    b = max(b, __float_as_uint(recs[g].speed_y));
  }
  atomicMax(&s_ab[0], a);
  atomicMax(&s_ab[1], b);
  __syncthreads();
  if (t == 0) {
    c->max_a[rec] = s_ab[0];
    c->max_b[rec] = s_ab[1];
  }
}

// A slot's first launch, one CTA over the queue's tiles (a step is a set of one):
//   1. the last slot's effects: a tile whose step count moved took a sub-step (its length into
//      the tick's shortest and longest), the events the last slot applied are released, and the
//      tick in flight lands when no tile has time left;
//   2. thread 0's begin: when no tick is in flight and one is queued, every tile's time left
//      becomes its length;
//   3. the begun tick's events into the planes, one after another (a later event over the same
//      cells wins). The host checked every rectangle against its tile and every plane's presence.
// With may_begin 0 it only settles (the call's last launch, so a read-back after it sees the last
// slot's effects).
__global__ void __launch_bounds__(kApplyThreads) queue_slot_kernel(
    QueueCtl* q, const QueueRecord* ring, uint32_t records, wl_landed* landed,
    const TileDesc* tiles, uint32_t n_tiles, uint32_t* seen, int may_begin,
    const QueueEvent* events, uint32_t max_events, const float* arena, uint32_t arena_values,
    int fixed) {
  const uint32_t t = threadIdx.x;
  // This thread's first tile descriptor into L1 while the grid before finishes: events change the
  // planes' values, never a descriptor, so it is the same before the wait as after it.
  if (t < n_tiles) asm volatile("prefetch.global.L1 [%0];" ::"l"(tiles + t));
  dependent_grid_start();  // a slot between two ticks is a dependent launch like them
  __shared__ uint32_t s_left, s_stepped, s_min, s_max, s_begin, s_apply, s_head;
  __shared__ float s_len;
  __shared__ float s_sum[3 * kGroupCells];
  __shared__ uint32_t s_ab[2];
  if (t == 0) {
    s_left = 0u;
    s_stepped = 0u;
    s_min = 0x7f800000u;  // +inf: lengths are >= 0, so their bits order as they do
    s_max = 0u;
  }
  __syncthreads();
  uint32_t left = 0u, stepped = 0u, lo = 0x7f800000u, hi = 0u;
  // This thread's first tile's control block and record slot, kept for the begin below (no tick
  // runs while a slot does, so neither moves).
  TileCtl* ctl0 = nullptr;
  uint32_t rec0 = 0u;
  for (uint32_t k = t; k < n_tiles; k += blockDim.x) {
    TileCtl* c = tiles[k].ctl;
    const uint32_t rec = c->rec;
    if (k == t) {
      ctl0 = c;
      rec0 = rec;
    }
    const LedgerBits& l = c->ledger[rec];
    if (l.steps != seen[k]) {
      seen[k] = l.steps;
      stepped = 1u;
      lo = min(lo, __float_as_uint(l.dt));
      hi = max(hi, __float_as_uint(l.dt));
    }
    if (l.remaining_s > 0.0f) left = 1u;
  }
  if (left != 0u) atomicOr(&s_left, 1u);
  if (stepped != 0u) {
    atomicOr(&s_stepped, 1u);
    atomicMin(&s_min, lo);
    atomicMax(&s_max, hi);
  }
  __syncthreads();
  if (t == 0) {
    if (q->apply != 0u) {
      q->events_done = q->first_event + q->events;
      q->values_done = q->values_end;
      q->apply = 0u;
    }
    if (s_stepped != 0u) {
      q->substeps += 1u;
      q->shortest = fminf(q->shortest, __uint_as_float(s_min));
      q->longest = fmaxf(q->longest, __uint_as_float(s_max));
    }
    const uint32_t head = *static_cast<volatile uint32_t*>(&q->head);  // the host's word
    s_head = head;
    if (q->active != 0u && s_left == 0u) land(q, ctl0->ledger[rec0], landed, records, head);
    s_begin = 0u;
    if (may_begin != 0 && q->active == 0u && q->begun != head) {
      // The lag: ticks pushed and not landed, this one included. Past the limit the domain
      // freezes, and each tick begun while it is frozen is dropped.
      const uint32_t lag = head - q->landed;
      if (q->frozen == 0u && q->lag_limit != 0u && lag > q->lag_limit) {
        q->frozen = 1u;
        q->freezes += 1u;
      }
      q->dropping = q->frozen;
      q->lag = lag;
      const QueueRecord r = ring[q->begun % records];
      q->begun += 1u;
      q->tick = r.tick;
      q->events = r.events;
      q->first_event = r.first_event;
      q->values_end = r.values_end;
      q->substeps = 0u;
      q->shortest = __int_as_float(0x7f800000);
      q->longest = 0.0f;
      q->apply = r.events != 0u ? 1u : 0u;
      q->active = 1u;
      s_begin = 1u;
      s_len = (q->dropping == 0u && r.length_s > 0.0f) ? r.length_s : 0.0f;
    }
    s_apply = q->apply;
  }
  __syncthreads();
  if (s_begin != 0u) {
    for (uint32_t k = t; k < n_tiles; k += blockDim.x) {
      if (k == t) {
        ctl0->ledger[rec0].remaining_s = s_len;
      } else {
        TileCtl* c = tiles[k].ctl;
        c->ledger[c->rec].remaining_s = s_len;
      }
    }
    __syncthreads();
    // A tick of no length lands now; its events are applied below all the same.
    if (t == 0 && !(s_len > 0.0f)) land(q, ctl0->ledger[rec0], landed, records, s_head);
  }
  if (t == 0) q->go = q->active;
  if (s_apply == 0u) return;
  const uint32_t n = q->events;
  const uint64_t first = q->first_event;
  for (uint32_t e = 0; e < n; ++e) {
    const QueueEvent ev = events[(first + e) % max_events];
    const TileDesc& T = tiles[ev.tile];
    if (ev.kind == WL_EVENT_STATE) {
      write_state_event(T, ev, arena + ev.value_first % arena_values, fixed, s_sum, s_ab);
      __syncthreads();
      continue;
    }
    float* dst = const_cast<float*>(ev.kind == WL_EVENT_BED      ? T.bed
                                    : ev.kind == WL_EVENT_SOURCE ? T.source
                                                                 : T.manning);
    const float* src = arena + ev.value_first % arena_values;
    const uint32_t count = ev.w * ev.h;
    for (uint32_t k = t; k < count; k += blockDim.x) {
      const uint32_t y = k / ev.w, x = k - y * ev.w;
      dst[size_t(ev.y0 + y) * T.nx + ev.x0 + x] = src[k];
    }
    __syncthreads();
  }
}

size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

bool ok(cudaError_t e, std::string* err, const char* what) {
  if (e == cudaSuccess) return true;
  if (err) *err = std::string("water_live: ") + what + ": " + cudaGetErrorString(e);
  return false;
}

}  // namespace

bool TickQueue::create(TileSet* set, uint32_t records, uint32_t arena_values, uint32_t max_events,
                       std::string* err) {
  destroy();
  if (set == nullptr || !set->valid()) {
    if (err) *err = "water_live: no step";
    return false;
  }
  if (records == 0 || records > kMaxRecords || max_events == 0 || arena_values == 0) {
    if (err) *err = "water_live: a queue holds 1 to 64 records, and at least one event and value";
    return false;
  }
  if (!ok(cudaSetDevice(set->device()), err, "cudaSetDevice")) return false;
  const size_t b_ctl = align_up(sizeof(QueueCtl));
  const size_t b_ring = align_up(size_t(records) * sizeof(QueueRecord));
  const size_t b_events = align_up(size_t(max_events) * sizeof(QueueEvent));
  const size_t b_landed = align_up(size_t(records) * sizeof(wl_landed));
  const size_t b_arena = align_up(size_t(arena_values) * sizeof(float));
  const uint32_t n_tiles = set->tile_count();
  const size_t b_seen = align_up(size_t(n_tiles) * sizeof(uint32_t));
  bytes_ = b_ctl + b_ring + b_events + b_landed + b_arena + b_seen;
  if (!ok(cudaMalloc(reinterpret_cast<void**>(&base_), bytes_), err, "cudaMalloc of the queue")) {
    base_ = nullptr;
    return false;
  }
  d_ctl_ = reinterpret_cast<QueueCtl*>(base_);
  d_ring_ = reinterpret_cast<QueueRecord*>(base_ + b_ctl);
  d_events_ = reinterpret_cast<QueueEvent*>(base_ + b_ctl + b_ring);
  d_landed_ = reinterpret_cast<wl_landed*>(base_ + b_ctl + b_ring + b_events);
  d_arena_ = reinterpret_cast<float*>(base_ + b_ctl + b_ring + b_events + b_landed);
  d_seen_ = reinterpret_cast<uint32_t*>(base_ + b_ctl + b_ring + b_events + b_landed + b_arena);
  tiles_ = n_tiles;
  set_ = set;
  records_ = records;
  max_events_ = max_events;
  arena_ = arena_values;
  pushed_ = 0;
  events_pushed_ = 0;
  values_pushed_ = 0;
  // The settle counts sub-steps from each tile's step count as it stands now.
  std::vector<TileCtl> ctl(n_tiles);
  if (!set->read_all_ctl(ctl.data(), err)) {
    destroy();
    return false;
  }
  std::vector<uint32_t> seen(n_tiles);
  for (uint32_t k = 0; k < n_tiles; ++k) seen[k] = ctl[k].ledger[ctl[k].rec & 1u].steps;
  QueueCtl q;
  std::memset(&q, 0, sizeof q);
  if (!ok(cudaMemsetAsync(base_, 0, bytes_, set->stream()), err, "cudaMemset of the queue") ||
      !ok(cudaMemcpyAsync(d_ctl_, &q, sizeof q, cudaMemcpyHostToDevice, set->stream()), err,
          "upload of the queue") ||
      !ok(cudaMemcpyAsync(d_seen_, seen.data(), n_tiles * sizeof(uint32_t),
                          cudaMemcpyHostToDevice, set->stream()),
          err, "upload of the step counts") ||
      !set->wait(err)) {
    destroy();
    return false;
  }
  return true;
}

void TickQueue::destroy() {
  if (base_ != nullptr) {
    if (set_ != nullptr && set_->valid()) {
      cudaSetDevice(set_->device());
      cudaStreamSynchronize(set_->stream());
      // Each tile's clock back to the free-running form: no time to count down.
      std::string ignored;
      for (uint32_t k = 0; k < tiles_; ++k)
        set_->set_remaining(k, std::numeric_limits<float>::infinity(), &ignored);
    }
    cudaFree(base_);
  }
  base_ = nullptr;
  set_ = nullptr;
  bytes_ = 0;
}

bool TickQueue::read_ctl(QueueCtl& out, std::string* err) {
  if (!valid()) {
    if (err) *err = "water_live: no queue";
    return false;
  }
  if (!ok(cudaSetDevice(set_->device()), err, "cudaSetDevice") ||
      !ok(cudaMemcpyAsync(&out, d_ctl_, sizeof out, cudaMemcpyDeviceToHost, set_->stream()), err,
          "read-back of the queue"))
    return false;
  return set_->wait(err);
}

int TickQueue::push(uint32_t tick, float length_s, const wl_event* events, uint32_t n_events,
                    const float* values, size_t n_values, std::string* err) {
  if (!valid()) {
    if (err) *err = "water_live: no queue";
    return WL_ERR_INVALID;
  }
  if (!(length_s >= 0.0f) || length_s == std::numeric_limits<float>::infinity()) {
    if (err) *err = "water_live: a tick's length is finite and not negative";
    return WL_ERR_ARGUMENT;
  }
  if (n_events > 0 && events == nullptr) {
    if (err) *err = "water_live: no events";
    return WL_ERR_ARGUMENT;
  }
  uint64_t need = 0;
  for (uint32_t e = 0; e < n_events; ++e) {
    const wl_event& ev = events[e];
    if (ev.tile >= tiles_) {
      if (err) *err = "water_live: an event's tile is not in the queue's set";
      return WL_ERR_ARGUMENT;
    }
    const TileDesc& d = set_->desc(ev.tile);
    const bool plane = ev.kind == WL_EVENT_BED || ev.kind == WL_EVENT_STATE ||
                       (ev.kind == WL_EVENT_SOURCE && d.source != nullptr &&
                        (d.flags & kFlagSource) != 0u) ||
                       (ev.kind == WL_EVENT_MANNING && d.manning != nullptr &&
                        (d.flags & kFlagManning) != 0u);
    if (!plane) {
      if (err) *err = "water_live: an event's plane is not on (set the source or Manning's n first)";
      return WL_ERR_ARGUMENT;
    }
    if (ev.w == 0 || ev.h == 0 || uint64_t(ev.x0) + ev.w > d.nx || uint64_t(ev.y0) + ev.h > d.ny) {
      if (err) *err = "water_live: an event's rectangle is empty or leaves the grid";
      return WL_ERR_SIZE;
    }
    need += uint64_t(ev.w) * ev.h * (ev.kind == WL_EVENT_STATE ? 3u : 1u);
  }
  if (need != n_values || (need > 0 && values == nullptr)) {
    if (err) *err = "water_live: the values do not match the events' rectangles";
    return WL_ERR_SIZE;
  }
  if (need > arena_ || n_events > max_events_) {
    if (err) *err = "water_live: the tick's events are larger than the queue's arena or event ring";
    return WL_ERR_SIZE;
  }
  QueueCtl q;
  if (!read_ctl(q, err)) return WL_ERR_CUDA;
  // A push is whole in the arena: values that would run past its end start again at 0.
  uint64_t base = values_pushed_;
  if (base % arena_ + need > arena_) base += arena_ - base % arena_;
  const bool room = pushed_ - q.begun < records_ &&
                    events_pushed_ + n_events - q.events_done <= max_events_ &&
                    base + need - q.values_done <= arena_;
  if (!room) {
    if (err) *err = "water_live: the queue has no room yet";
    return WL_ERR_REFUSED;
  }
  cudaStream_t s = set_->stream();
  std::vector<QueueEvent> dev(n_events);
  uint64_t at = base;
  for (uint32_t e = 0; e < n_events; ++e) {
    const wl_event& ev = events[e];
    dev[e] = QueueEvent{ev.kind, ev.x0, ev.y0, ev.w, ev.h, ev.tile, at};
    at += uint64_t(ev.w) * ev.h * (ev.kind == WL_EVENT_STATE ? 3u : 1u);
  }
  // Events and values first, the record, then `head`: a slot that sees the new head finds them.
  for (uint32_t e = 0; e < n_events; ++e) {
    const uint64_t slot = (events_pushed_ + e) % max_events_;
    if (!ok(cudaMemcpyAsync(d_events_ + slot, &dev[e], sizeof(QueueEvent), cudaMemcpyHostToDevice,
                            s),
            err, "upload of an event"))
      return WL_ERR_CUDA;
  }
  if (need > 0 && !ok(cudaMemcpyAsync(d_arena_ + base % arena_, values, need * sizeof(float),
                                      cudaMemcpyHostToDevice, s),
                      err, "upload of the events' values"))
    return WL_ERR_CUDA;
  // A record releases the arena up to its own values' end; one with none, up to the values
  // pushed before it (all of them released by then, records being begun in order).
  const uint64_t values_end = need > 0 ? base + need : values_pushed_;
  QueueRecord r{tick, length_s, events_pushed_, n_events, 0u, values_end};
  const uint32_t head = pushed_ + 1u;
  if (!ok(cudaMemcpyAsync(d_ring_ + pushed_ % records_, &r, sizeof r, cudaMemcpyHostToDevice, s),
          err, "upload of a record") ||
      !ok(cudaMemcpyAsync(&d_ctl_->head, &head, sizeof head, cudaMemcpyHostToDevice, s), err,
          "upload of the queue's head") ||
      !set_->wait(err))
    return WL_ERR_CUDA;
  pushed_ = head;
  events_pushed_ += n_events;
  if (need > 0) values_pushed_ = base + need;
  return WL_OK;
}

cudaError_t TickQueue::enqueue(cudaStream_t s, uint32_t slots) {
  if (!valid()) return cudaErrorInvalidValue;
  const float inf = std::numeric_limits<float>::infinity();
  const TileDesc* tiles = set_->device_descs();
  if (max_slots_ != 0u && slots > max_slots_) slots = max_slots_;  // a frame's ceiling
  for (uint32_t k = 0; k < slots; ++k) {
    cudaError_t e = launch_dependent(queue_slot_kernel, dim3(1), dim3(kApplyThreads), 0, s, d_ctl_,
                                     (const QueueRecord*)d_ring_, records_, d_landed_, tiles,
                                     tiles_, d_seen_, 1, (const QueueEvent*)d_events_, max_events_,
                                     (const float*)d_arena_, arena_, set_->fixed_ops() ? 1 : 0);
    if (e != cudaSuccess) return e;
    e = set_->enqueue_ticks(s, 1, inf, &d_ctl_->go);
    if (e != cudaSuccess) return e;
  }
  // The last slot's effects, so a read-back after the call sees them.
  queue_slot_kernel<<<1, 32, 0, s>>>(d_ctl_, d_ring_, records_, d_landed_, tiles, tiles_, d_seen_,
                                     0, d_events_, max_events_, d_arena_, arena_,
                                     set_->fixed_ops() ? 1 : 0);
  return cudaGetLastError();
}

bool TickQueue::set_limits(uint32_t lag_limit, uint32_t max_slots, std::string* err) {
  if (!valid()) {
    if (err) *err = "water_live: no queue";
    return false;
  }
  if (!ok(cudaSetDevice(set_->device()), err, "cudaSetDevice") ||
      !ok(cudaMemcpyAsync(&d_ctl_->lag_limit, &lag_limit, sizeof lag_limit,
                          cudaMemcpyHostToDevice, set_->stream()),
          err, "upload of the lag limit") ||
      !set_->wait(err))
    return false;
  max_slots_ = max_slots;
  return true;
}

bool TickQueue::read_landed(uint32_t first, uint32_t count, wl_landed* out, std::string* err) {
  QueueCtl q;
  if (!read_ctl(q, err)) return false;
  if (count == 0) return true;
  if (out == nullptr || uint64_t(first) + count > q.landed || q.landed - first > records_) {
    if (err) *err = "water_live: those landings are not held (the last `records` are)";
    return false;
  }
  std::vector<wl_landed> all(records_);
  if (!ok(cudaMemcpyAsync(all.data(), d_landed_, records_ * sizeof(wl_landed),
                          cudaMemcpyDeviceToHost, set_->stream()),
          err, "read-back of the landings") ||
      !set_->wait(err))
    return false;
  for (uint32_t i = 0; i < count; ++i) out[i] = all[(first + i) % records_];
  return true;
}

}  // namespace wlc

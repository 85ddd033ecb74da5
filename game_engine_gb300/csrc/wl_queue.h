// The tick queue: ticks of the world's clock queued on the device and stepped by slots a caller
// enqueues or captures (wlcuda.h, "the tick queue"). The design is the reference's
// (docs/subsystems/water_live.md:76-94, ADR-0081), which the reference has not built: records of
// a tick's length and events on the card, sub-step slots that begin a tick, apply its events and
// step it by a length the card chooses from the state, and a read-back record per landed tick.
#pragma once

#include "wl_device.cuh"
#include "wl_tiles.h"
#include "wlcuda.h"

#include <cstdint>
#include <string>

namespace wlc {

// A queued tick (water_live.md:84): its number, its length, its events and where its values end.
struct QueueRecord {
  uint32_t tick;
  float length_s;
  uint64_t first_event;  // absolute index of its first event
  uint32_t events;
  uint32_t pad;
  uint64_t values_end;  // absolute arena index past its last value
};
static_assert(sizeof(QueueRecord) == 32, "QueueRecord layout");

// An event as the device holds it: a rectangle of one plane of one tile and where its values start.
struct QueueEvent {
  uint32_t kind, x0, y0, w, h, tile;
  uint64_t value_first;  // absolute arena index (the host keeps an event's values contiguous)
};
static_assert(sizeof(QueueEvent) == 32, "QueueEvent layout");

// The queue's device words. The host writes `head` after a record; the slots' one-thread kernels
// write the rest; `go` and `apply` are each one slot's decision, constant while its launches run.
struct QueueCtl {
  uint32_t head;        // records pushed
  uint32_t begun;       // records begun
  uint32_t landed;      // records landed
  uint32_t active;      // a begun tick has not landed
  uint32_t go;          // this slot's tick steps
  uint32_t apply;       // this slot's apply writes the begun tick's events
  uint32_t substeps;    // slots in which a tile of the tick in flight stepped
  uint32_t pad;
  float shortest, longest;
  uint32_t tick, events;  // the tick in flight: its number and its event count
  uint64_t first_event;   // its first event
  uint64_t values_end;    // its values' end
  uint64_t events_done;   // events whose values the device no longer reads
  uint64_t values_done;   // arena values the device no longer reads
  // The lag control (water_live.md:90-92; wl_queue_set_limits).
  uint32_t lag_limit;  // ticks pushed and not landed past which a begin freezes the domain (0: off)
  uint32_t frozen;     // the domain is frozen: each begun tick is dropped
  uint32_t dropping;   // the tick in flight is a dropped one
  uint32_t dropped;    // ticks dropped
  uint32_t freezes;    // times the domain froze
  uint32_t lag;        // the lag when the tick in flight began
};

class TickQueue {
 public:
  ~TickQueue() { destroy(); }
  // Over every tile of `set` (a step is a set of one tile). records <= 64.
  bool create(TileSet* set, uint32_t records, uint32_t arena_values, uint32_t max_events,
              std::string* err);
  void destroy();
  bool valid() const { return base_ != nullptr; }
  // WL_OK, or WL_ERR_REFUSED (no room yet), WL_ERR_ARGUMENT, WL_ERR_CUDA with `err` set.
  int push(uint32_t tick, float length_s, const wl_event* events, uint32_t n_events,
           const float* values, size_t n_values, std::string* err);
  // At most max_slots slots a call when max_slots > 0 (wl_queue_set_limits).
  cudaError_t enqueue(cudaStream_t s, uint32_t slots);
  bool set_limits(uint32_t lag_limit, uint32_t max_slots, std::string* err);
  bool read_ctl(QueueCtl& out, std::string* err);
  bool read_landed(uint32_t first, uint32_t count, wl_landed* out, std::string* err);
  uint64_t device_bytes() const { return bytes_; }
  cudaStream_t stream() const { return set_ != nullptr ? set_->stream() : nullptr; }
  int device() const { return set_ != nullptr ? set_->device() : -1; }
  bool wait(std::string* err) { return set_ != nullptr && set_->wait(err); }

 private:
  TileSet* set_ = nullptr;
  char* base_ = nullptr;
  uint64_t bytes_ = 0;
  QueueCtl* d_ctl_ = nullptr;
  QueueRecord* d_ring_ = nullptr;
  QueueEvent* d_events_ = nullptr;
  float* d_arena_ = nullptr;
  wl_landed* d_landed_ = nullptr;
  uint32_t* d_seen_ = nullptr;  // each tile's step count at the last settle
  uint32_t tiles_ = 0;
  uint32_t records_ = 0, max_events_ = 0, arena_ = 0;
  uint32_t max_slots_ = 0;  // 0: no ceiling
  uint32_t pushed_ = 0;        // records pushed
  uint64_t events_pushed_ = 0;  // events pushed
  uint64_t values_pushed_ = 0;  // arena values pushed (with the padding that keeps a push whole)
};

}  // namespace wlc

// The C ABI's queue handle (wlcuda.h), over a step's or a batch's tile set. `owner` is the owner's
// own field that points back at the handle; whichever of the two goes first clears the link.
struct wl_queue {
  wlc::TickQueue q;
  wl_queue** owner = nullptr;
};

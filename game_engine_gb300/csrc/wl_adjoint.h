// The adjoint (reverse) tick and its checkpointed sweep (host side and the kernels' interface).
//
// The reference has no adjoint. For a loss L = sum over probe cells of (h_T(p) - target_p)^2 after
// T ticks of fixed length, the sweep gives dL/d(bed) and dL/d(source) per cell:
//   1. the checkpoint pass: T forward ticks from the tile set's current state (the plain tick's
//      arithmetic to the bit, with no records), keeping the state every k ticks, each tick's
//      branch words (clamp, sink limited, wet) and each state's largest speeds;
//   2. a check that no tick's stable length was shorter than the fixed length (the plain tick would
//      have shortened it, and the gradient would be of another trajectory);
//   3. the loss in FP64 and the adjoint state of tick T;
//   4. for each segment, last first: the segment's states recomputed from its checkpoint, then the
//      reverse ticks over them, the gradients accumulated in FP64.
// Every launch of a sweep is on one stream; the sweep captures into one CUDA graph.
#pragma once

#include "wl_tiles.h"

#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <vector>

namespace wlc {

// Branch words, one bit a cell, 32 cells (a band's row) a word: the three planes of a tick.
constexpr uint32_t kBranchClamp = 0u;        // the update's depth was negative and was clamped
constexpr uint32_t kBranchSinkLimited = 1u;  // a sink took all of the cell's water
constexpr uint32_t kBranchWet = 2u;          // the cell ended the tick wet (its momenta kept)

// One tile's share of a sweep as the kernels see it. Planes are the tile's layout (cell (x, y) at
// y * nx + x); a state is three planes (h, hu, hv), 3 * nx * ny floats.
struct AdjTile {
  const float* bed;
  const float* source;  // null when the tile applies no source
  float* ckpt;          // C + 1 states: state c holds tick c * k (state C: tick T)
  float* stack;         // k - 1 states: the segment's ticks c * k + j, j = 1 .. k - 1, at j - 1
  uint32_t* bits;       // per tick, 3 planes of ny * bands words
  float* lam[2];        // the adjoint state of tick t in lam[t & 1]
  double* g_bed;        // dL/d(bed), accumulated over the ticks
  double* g_src;        // dL/d(source)
  uint32_t* speeds;     // per tick t: the largest |u| + c, |v| + c of state t (float bits)
  const uint32_t* probes;
  const double* targets;
  double* loss;
  uint32_t* limited;    // ticks the plain tick would have shortened
  uint32_t n_probes;
  uint32_t nx, ny, bands, row_blocks;
  uint32_t flags;  // edges and the source flag
  float gravity, dry, cell_m, cfl;
  uint32_t item_base, items;
};

// One launch of a sweep: the tiles, the tile of each work item (null: one tile), the launch's work
// counter, the sweep's length T and checkpoint interval k, the tick t, the fixed step length.
struct AdjArgs {
  const AdjTile* tiles;
  const uint32_t* item_tile;
  WorkCtl* work;
  uint32_t n_items;
  uint32_t ticks, every, t;
  float dt;
};

// A work item is 32 columns by 4 or 16 rows (the sweep chooses by the device's SM count).
// The resident CTAs an SM of the forward marches or (reverse) of the reverse march.
int adj_occupancy(int rows, bool reverse);
// The set's current states into checkpoint 0 (grid: max_blocks by count).
cudaError_t launch_adj_copy_in(const TileDesc* set_tiles, const AdjTile* tiles, uint32_t count,
                               uint32_t max_blocks, cudaStream_t s);
// mode 0: the checkpoint pass (writes the branch words and the speeds); 1: a segment's recompute.
cudaError_t launch_adj_forward(int mode, int rows, const AdjArgs& a, int grid, cudaStream_t s);
cudaError_t launch_adj_check(const AdjArgs& a, uint32_t count, cudaStream_t s);
cudaError_t launch_adj_seed(const AdjArgs& a, uint32_t count, cudaStream_t s);
cudaError_t launch_adj_reverse(int rows, const AdjArgs& a, int grid, cudaStream_t s);

class Adjoint {
 public:
  Adjoint() = default;
  ~Adjoint();
  Adjoint(const Adjoint&) = delete;
  Adjoint& operator=(const Adjoint&) = delete;

  // The int-returning calls give WL_OK or a WL_ERR_* code (include/wlcuda.h) and a message.
  // A sweep of `ticks` ticks with a checkpoint every `every` over the tiles of `set` (which must
  // outlive it). probe_first[t] .. probe_first[t + 1] index tile t's probes (tile-local cells)
  // and their targets.
  int create(TileSet* set, uint32_t ticks, uint32_t every, const uint32_t* probe_first,
             const uint32_t* probes, const double* targets, std::string* err);
  // The whole sweep on the set's stream (no synchronisation; graph-capturable). The tiles' flags
  // must have passed check_flags.
  cudaError_t enqueue(float dt);
  // Refuses flags the sweep does not differentiate (fixed ops, Manning, the compensated source, a
  // coarser source clock) and brings the sweep's copy of the tiles' source flags up to date.
  int check_flags(std::string* err);
  // The sweep, from a captured graph when use_graph, and a wait for it.
  int run(float dt, bool use_graph, std::string* err);
  // loss: a value a tile; g_bed, g_src: every tile's cells tile after tile; limited: a count a tile.
  int read(double* loss, double* g_bed, double* g_src, uint32_t* limited, std::string* err);
  // The state of tick T (3 planes a tile, tile after tile).
  int read_final(float* planes, std::string* err);
  // dL/d(state of tick 0), the reverse sweep's last adjoint state (3 planes a tile, tile after tile).
  int read_state_gradient(float* planes, std::string* err);
  uint32_t launches() const;
  uint64_t device_bytes() const { return bytes_; }
  int rows() const { return rows_; }

 private:
  TileSet* set_ = nullptr;
  uint32_t ticks_ = 0, every_ = 0, segments_ = 0;
  char* base_ = nullptr;
  size_t bytes_ = 0;
  std::vector<AdjTile> host_;
  AdjTile* d_tiles_ = nullptr;
  uint32_t* d_item_tile_ = nullptr;
  WorkCtl* d_work_ = nullptr;
  uint32_t n_items_ = 0;
  int grid_fwd_ = 0, grid_rev_ = 0;
  int rows_ = 16;
  // zeroed at the start of every sweep: the gradients, speeds, counts and losses
  void* zero_ = nullptr;
  size_t zero_bytes_ = 0;
  float* lam_base_[2] = {nullptr, nullptr};
  size_t lam_bytes_ = 0;
  cudaGraphExec_t graph_ = nullptr;
  float graph_dt_ = 0.0f;
};

}  // namespace wlc

// The C ABI's handle (include/wlcuda.h).
struct wl_adjoint {
  wlc::Adjoint impl;
};

// Creates a sweep over a tile set (the step's and the batch's creators call this).
int wl_adjoint_create_over(wlc::TileSet* set, uint32_t ticks, uint32_t every,
                           const uint32_t* probe_first, const uint32_t* probes,
                           const double* targets, wl_adjoint** out, char* err, size_t err_len);

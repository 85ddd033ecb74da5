// Host-side entry points of the tick's kernels (wl_kernels.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace wlc {

struct TileDesc;
struct WorkCtl;
struct ResidentCtl;

// A tick launch: the tiles, which tile each work item belongs to (null: all items of tile 0), the
// launch's work counter and the step's max_dt. `go`, when not null, is a device word read at the
// start: zero makes the launch return before it takes any item (a tick queue's idle slot).
struct TickArgs {
  const TileDesc* tiles;
  const uint32_t* item_tile;
  WorkCtl* work;
  uint32_t n_items;
  float max_dt;
  const uint32_t* go = nullptr;
  // Set by launch_tick: the 32 x 16 march takes items 0 .. n_whole - 1 a warp each and the rest
  // (fewer than its warps) a CTA each, four rows a warp.
  uint32_t n_whole = 0;
  // The block shape, one tile: the grid's last CTA folds the tile's ledger instead of item 0
  // (the launch holds one CTA more than items).
  uint32_t fold_apart = 0;
  // The march's native plain variant with zero arguments taken apart from its divisions and
  // square roots (the same bits; faster where many arguments are zero, slower where few are).
  uint32_t zero_apart = 0;
  // The block shapes' staged variant: a block's cells and halo taken by two tensor copies into
  // shared memory (tiles with tensor maps; the others load cell by cell). `fault` is the word a
  // CTA marks where its wait on the copies gave up.
  uint32_t stage = 0;
  uint32_t* fault = nullptr;
};

// The block of cells one work item steps: 32 columns by 16, 32 or 64 rows, one warp marching
// them; (k32x16s) 32 by 16 split over a CTA's four warps, four rows each, for tiles with too few
// items to fill the device; or (k32x16b) 32 by 16 by a CTA of 256 threads in three phases through
// shared memory (cells, then every face on its own thread, then the updates). The batched form's
// autotuner chooses among these five. (k32x16w) is k32x16b by a CTA of 512 threads, which a tile
// set launches in k32x16b's place when the launch holds no more blocks than the device has SMs.
enum class BlockShape : uint8_t {
  k32x16 = 0, k32x32 = 1, k32x64 = 2, k32x16s = 3, k32x16b = 4, k32x16w = 5
};

size_t tick_smem_bytes(BlockShape shape);
int tick_threads(BlockShape shape);
void block_dims(BlockShape shape, uint32_t& bx, uint32_t& by);
// Sets the kernels' shared-memory opt-in on the current device and returns the resident CTAs per
// SM (0 on an error). `manning`: some tile holds Manning's n; `plain`: no tile holds a flag of
// kFlagsNotPlain (the march's plain variant; the split and block shapes have none).
int tick_occupancy(BlockShape shape, bool fixed, bool manning, bool plain);

cudaError_t launch_tick(BlockShape shape, bool fixed, bool manning, bool plain, const TickArgs& a,
                        int grid, cudaStream_t s);
// The staged block tick's three tensor maps of tile `d` (its state pointers and sizes set) into
// `maps` (384 bytes, 64-byte aligned, host memory): false, and no maps, where its width is not a
// multiple of 4 (rows off 16-byte boundaries) or the driver offers no tensor-map encoder.
bool encode_stage_maps(const TileDesc& d, void* maps);
// The records of the states just written (one CTA a work item, the same items as the tick's).
// The resident tick: `ticks` ticks of tile 0 (the wide block tick's items) in one cooperative
// launch of a.n_items + 1 CTAs, a grid barrier between ticks. `rc` (zeroed here, on `s`, before
// the launch) holds the barrier's words; a nonzero error word after the launch means a wait gave
// up and the state is not the ticks' result.
cudaError_t launch_tick_resident(bool fixed, bool manning, const TickArgs& a, uint32_t ticks,
                                 ResidentCtl* rc, cudaStream_t s);
// The resident tick's CTAs the current device holds at once (0 on an error).
int resident_capacity(bool fixed, bool manning);
// The barrier's bounded wait alone: n CTAs, the last of which never arrives; the others give up
// after a second and set rc's error word (rc is zeroed here first).
cudaError_t launch_barrier_probe(ResidentCtl* rc, uint32_t n, cudaStream_t s);
cudaError_t launch_prime(BlockShape shape, bool fixed, const TickArgs& a, cudaStream_t s);
cudaError_t launch_length_pass(bool fixed, const TileDesc* tiles, uint32_t tile, float max_dt,
                               cudaStream_t s);
cudaError_t launch_write_state(TileDesc* tiles, uint32_t tile, size_t n, const double* h,
                               const double* hu, const double* hv, cudaStream_t s);
cudaError_t launch_write_state_f32(TileDesc* tiles, uint32_t tile, size_t n, const float* planes,
                                   cudaStream_t s);
cudaError_t launch_plane(float* dst, const double* src, size_t n, double datum, cudaStream_t s);
cudaError_t launch_read_state(const TileDesc* tiles, uint32_t tile, size_t n, double* h,
                              double* hu, double* hv, cudaStream_t s);
cudaError_t launch_copy_state(const TileDesc* tiles, uint32_t tile, size_t n, float* dst,
                              cudaStream_t s);

// Whole batches: arrays hold every tile's cells tile after tile; first[t] is tile t's first cell.
cudaError_t launch_scatter_state(TileDesc* tiles, uint32_t count, const uint64_t* first,
                                 uint64_t total, const double* h, const double* hu,
                                 const double* hv, cudaStream_t s);
// which: 0 the bed (less `datum`), 1 Manning's n, 2 the source.
cudaError_t launch_scatter_plane(TileDesc* tiles, uint32_t count, const uint64_t* first,
                                 uint64_t total, const double* v, double datum, int which,
                                 cudaStream_t s);
// Every tile's current copy, four planes a tile (4 * first[t] floats before tile t).
cudaError_t launch_gather_state(const TileDesc* tiles, uint32_t count, const uint64_t* first,
                                uint64_t total, float* dst, cudaStream_t s);
// The settled check of tiles tile0 .. tile0 + count - 1 against a steady state (device doubles,
// tile t's cells from first[t], or from 0 where `first` is null): dev[2 k] and dev[2 k + 1] get
// the bits of tile tile0 + k's largest depth and momentum deviations. `largest`: the most cells a
// tile holds.
cudaError_t launch_settled(const TileDesc* tiles, uint32_t tile0, uint32_t count,
                           const uint64_t* first, uint64_t largest, const double* h,
                           const double* hu, const double* hv, uint32_t* dev, cudaStream_t s);
// A flush (dt_main with max_dt 0) of every tile.
cudaError_t launch_flush_all(bool fixed, const TileDesc* tiles, uint32_t count, cudaStream_t s);

}  // namespace wlc

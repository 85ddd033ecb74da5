/* wlcuda — the live-water tick on a GB300 (sm_103a), behind a C ABI.
 *
 * A drop-in for the reference's GPU step, engine::water_live::DeviceStep
 * (systems/water_live/include/systems/water_live/water_live.h:158-256) and its hash
 * (water_live.h:259). The scheme is the reference's: the hydrostatic reconstruction over the
 * central-upwind flux on h, hu, hv in FP32, every operation in the reference's order with no
 * contraction, so a step's bytes equal the reference CPU restatement's bit for bit.
 *
 * Conventions (water_live.h:152-157, water_live.cpp:83-86):
 *  - Every call that moves data between host and device waits for the device; wl_enqueue_steps is
 *    the asynchronous `record` analogue and may be captured into a CUDA graph.
 *  - int-returning calls give WL_OK or a WL_ERR_* code and, when `err` is non-null, a message
 *    (truncated to err_len). uint64-returning calls give 0 on an error.
 *  - A misfit size is refused with nothing changed. A null or destroyed handle refuses everything
 *    (water_live_tests.cpp:38-47).
 *  - Input arrays are read and never kept; the step owns every device buffer.
 *  - One host thread per handle; no internal locking.
 */
#ifndef WLCUDA_H
#define WLCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t, without the CUDA headers. Null is the legacy default stream. */
typedef struct CUstream_st* wl_stream;

enum {
  WL_OK = 0,
  WL_ERR_INVALID = 1,   /* no device / a handle that was never created */
  WL_ERR_SIZE = 2,      /* an array that does not fit the grid */
  WL_ERR_CUDA = 3,      /* a CUDA call failed */
  WL_ERR_ALLOC = 4,     /* device or host memory could not be had */
  WL_ERR_REFUSED = 5,   /* a call the step's state refuses (advance with a coarser source clock) */
  WL_ERR_UNFINISHED = 6,/* advance ran its most batches without landing */
  WL_ERR_TIMEOUT = 7,   /* a wait for the device passed its limit */
  WL_ERR_ARGUMENT = 8   /* an argument out of its range */
};

/* engine::water_state::Config (domain/water_state/include/domain/water_state/water_state.h:83-99),
 * the fields the step reads: carried, water_density and rows_per_job are not read
 * (water_live.h:164-166). `device` stands in for the reference's gfx::Device. */
typedef struct wl_config {
  uint32_t nx;
  uint32_t ny;
  double cell_m;
  double gravity;
  double cfl;
  double dry_depth_m;
  uint8_t west_open;  /* water_state::Edge: 0 closed (a wall), 1 open */
  uint8_t east_open;
  uint8_t south_open;
  uint8_t north_open;
  int32_t device;
} wl_config;

/* water_live::Ops (water_live.h:62) and StepOptions (water_live.h:105-110). */
enum { WL_OPS_NATIVE = 0, WL_OPS_FIXED = 1 };
typedef struct wl_options {
  uint8_t ops;
  uint8_t stored_faces;
} wl_options;

/* water_live::StepParams (water_live.h:66-88), mirrored with its 120-byte layout and the offsets
 * the reference pins (water_live_tests.cpp:22-36). The CUDA kernels take their own argument
 * structs; this one documents and checks the contract. */
typedef struct wl_step_params {
  uint64_t state_in, state_out, bed, manning, source, partials, ledger;
  uint32_t nx, ny, groups_x, group_count, flags;
  float cell_m, gravity, cfl, dry_depth_m, max_dt, source_scale;
  uint32_t pad;
  uint64_t faces_x, faces_y;
} wl_step_params;

/* water_live.h:90-97 */
#define WL_FLAG_WEST_OPEN 1u
#define WL_FLAG_EAST_OPEN 2u
#define WL_FLAG_SOUTH_OPEN 4u
#define WL_FLAG_NORTH_OPEN 8u
#define WL_FLAG_MANNING 16u
#define WL_FLAG_SOURCE 32u
#define WL_FLAG_COMPENSATE 64u
#define WL_FLAG_STORED_FACES 128u
#define WL_STATE_PLANES 4u /* water_live.h:102: h, hu, hv, the source's remainder */
#define WL_GROUP_SIDE 16u  /* water_live.h:140 */

/* water_live::WaterPartial (water_live.h:114-121), 32 bytes: one record per 16 x 16 group. */
typedef struct wl_partial {
  float speed_x, speed_y, source_m3, open_m3, roundoff_m3, pad[3];
} wl_partial;

/* water_live::WaterLedger (water_live.h:124-137), 48 bytes, as the device holds it. */
typedef struct wl_ledger_bits {
  float time_hi, time_lo, source_hi, source_lo, open_hi, open_lo, roundoff_hi, roundoff_lo;
  float remaining_s, dt;
  uint32_t steps, pad;
} wl_ledger_bits;

/* water_live::Ledger (water_live.h:143-150). */
typedef struct wl_ledger {
  double source_m3, open_edge_out_m3, roundoff_m3, time_s, remaining_s;
  uint64_t steps;
} wl_ledger;

typedef struct wl_step wl_step;

/* ---- the plain step: water_live::DeviceStep (water_live.cpp:105-639) ---------------------- */

/* DeviceStep::create (water_live.cpp:105-210): the state dry over a bed of zero, the ledger empty.
 * An empty grid, or one of more than 2^30 cells (a tile's cells are indexed in 32 bits), is
 * refused with WL_ERR_SIZE; wl_batch_create refuses such a tile the same way. */
int wl_create(const wl_config* config, const wl_options* options, wl_step** out, char* err,
              size_t err_len);
/* DeviceStep::destroy (water_live.cpp:212-229). Null is a no-op. */
void wl_destroy(wl_step* step);
/* DeviceStep::valid (water_live.h:170). */
int wl_valid(const wl_step* step);
/* DeviceStep::cell_count / group_count (water_live.h:174-175); 0 for an invalid handle. */
uint32_t wl_cell_count(const wl_step* step);
uint32_t wl_group_count(const wl_step* step);
/* Tick kernel launches enqueued since create (no counterpart in the reference: a diagnosis
 * counter). A tile of no more 32 x 16 blocks than the device holds resident CTAs steps a call's two
 * or more ticks in one launch; other tiles take a launch a tick. 0 for an invalid handle. */
uint64_t wl_tick_launches(const wl_step* step);
/* Tiles whose 32 x 16 blocks the step's launches take by tensor copies (no counterpart in the
 * reference: a diagnosis count): 1 where the tile's width is a multiple of 4 and the step ticks in
 * three-phase blocks with more blocks than its launch's 256-thread CTAs (each CTA's next block's
 * copies issued while it steps the current one), or in any block launch with WLCUDA_STAGE=1 set
 * at create (WLCUDA_STAGE=0: in none); else 0. */
uint32_t wl_staged_tiles(const wl_step* step);

/* DeviceStep::write_state (water_live.cpp:271-314): each array n = nx * ny doubles, rounded to
 * float; plane 3 zeroed; the ledger emptied; the source clock restarted. */
int wl_write_state(wl_step* step, const double* depth, const double* momentum_x,
                   const double* momentum_y, size_t n, char* err, size_t err_len);
/* DeviceStep::read_state (water_live.cpp:334-347): widened to double. */
int wl_read_state(wl_step* step, double* depth, double* momentum_x, double* momentum_y, size_t n,
                  char* err, size_t err_len);
/* DeviceStep::read_state_bits (water_live.cpp:316-332): count = 4 * nx * ny floats, by plane. */
int wl_read_state_bits(wl_step* step, float* planes, size_t count, char* err, size_t err_len);
/* DeviceStep::read_ledger (water_live.cpp:349-381): a flush, then the pairs widened. */
int wl_read_ledger(wl_step* step, wl_ledger* out, char* err, size_t err_len);
/* The settled check of wl_batch_settled on a step (n = its cells): its largest depth and momentum
 * deviations from the steady state h*, hu*, hv*, and settled = both within the bounds. No
 * counterpart in DeviceStep (the reference designs the check, ADR-0080 decision 4, W176). */
int wl_settled(wl_step* step, const double* depth, const double* momentum_x,
               const double* momentum_y, size_t n, float depth_bound_m, float momentum_bound_m2_s,
               uint8_t* settled, float* depth_dev_m, float* momentum_dev_m2_s, char* err,
               size_t err_len);

/* DeviceStep::set_bed (water_live.cpp:439-447): bed_m - datum_m in double, rounded once. */
int wl_set_bed(wl_step* step, const double* bed_m, size_t n, double datum_m, char* err,
               size_t err_len);
/* DeviceStep::set_manning (water_live.cpp:449-463): n = 0 turns friction off. */
int wl_set_manning(wl_step* step, const double* manning, size_t n, char* err, size_t err_len);
/* DeviceStep::set_source (water_live.cpp:465-486): n = 0 turns sources off; `every` > 1 applies
 * the source on one step in `every`, `every` times over; `compensate` keeps plane 3. */
int wl_set_source(wl_step* step, const double* source_m_per_s, size_t n, uint32_t every,
                  int compensate, char* err, size_t err_len);

/* DeviceStep::record (water_live.cpp:488-568) onto a stream: `count` ticks of
 * min(stable step, max_dt, time left), one kernel launch each; nothing waits. Every per-tick
 * quantity (which copy holds the state, the step's length, the ledger, the source clock) lives on
 * the device, so a captured graph of these launches may be replayed any number of times. The
 * kernel each launch runs is chosen when it is enqueued, from the step's flags (Manning on, the
 * compensated source, open edges): a graph captured before wl_set_manning or wl_set_source changes
 * those must be captured again. Each tick is launched as a programmatic dependent of the launch
 * before it on the stream (it reads nothing before that launch has completed) and lets the launch
 * after it be scheduled at its start: a caller's own kernel launched next with programmatic stream
 * serialization must wait on its grid dependency (cudaGridDependencySynchronize) before it reads
 * the state; any other launch or copy after the ticks waits for them in full. */
int wl_enqueue_steps(wl_step* step, wl_stream stream, uint32_t count, float max_dt);
/* DeviceStep::run_steps (water_live.cpp:570-574): enqueued on the step's own stream and waited for. */
int wl_run_steps(wl_step* step, uint32_t count, float max_dt, char* err, size_t err_len);
/* DeviceStep::advance (water_live.cpp:594-632): the steps taken, 0 on an error or a refusal. */
uint64_t wl_advance(wl_step* step, double duration_s, char* err, size_t err_len);
/* DeviceStep::state_hash (water_live.cpp:634-639): FNV-1a over all four planes' floats. */
uint64_t wl_state_hash(wl_step* step, char* err, size_t err_len);

/* Diagnosis (water_live.h:214-224; water_live.cpp:383-437). */
int wl_read_partials_bits(wl_step* step, wl_partial* out, size_t count, char* err, size_t err_len);
int wl_read_ledger_bits(wl_step* step, wl_ledger_bits* out, char* err, size_t err_len);
int wl_run_length_pass(wl_step* step, float max_dt, char* err, size_t err_len);

/* water_live::hash_floats (water_live.cpp:90-101). */
uint64_t wl_hash_floats(const float* values, size_t count);

/* A check of the resident tick's grid barrier (no counterpart in the reference): `ctas` CTAs
 * (2 or more) meet at the barrier on `device` except the last, which never arrives, so the others'
 * bounded wait runs out (about a second) and marks the barrier's error word. WL_OK when every CTA
 * left and the word was marked; WL_ERR_CUDA otherwise. */
int wl_resident_barrier_check(int device, uint32_t ctas, char* err, size_t err_len);

/* The step's own stream (a cudaStream_t), for callers that order work against it. */
wl_stream wl_step_stream(wl_step* step);

/* write_state from device memory: `planes` holds 4 * nx * ny floats on the step's device (plane 3
 * is ignored and zeroed, as write_state does); the ledger is emptied, the source clock restarted and
 * the records primed, all enqueued on `stream` (null: the step's own) without waiting. For callers
 * whose inputs already live on the device. */
int wl_write_state_device(wl_step* step, const float* planes, wl_stream stream);

/* The device-resident state in place, for callers that keep their data on the device (no host
 * copy): the current copy's four planes (4 * nx * ny floats, plane by plane) and the bed. Valid
 * until the next call on the handle. */
int wl_device_planes(wl_step* step, float** planes, float** bed, char* err, size_t err_len);

/* ---- the batched form: many tiles, one persistent launch per tick -------------------------- *
 * No counterpart call in the reference, which steps one rectangle per DeviceStep; each tile here
 * is stepped exactly as a DeviceStep of its size would step it (the same bytes), and the reference's
 * designed-but-unbuilt tile system (docs/subsystems/water_live.md:74-90) is what it serves.
 * Arrays passed for the whole batch hold every tile's nx * ny cells, tile after tile in index
 * order; wl_batch_tile_first gives a tile's first cell. */

typedef struct wl_batch wl_batch;

/* One tile: its size and its edges (water_state::Edges, water_state.h:62-67). */
typedef struct wl_tile {
  uint32_t nx, ny;
  uint8_t west_open, east_open, south_open, north_open;
} wl_tile;

/* The launch's shape: the rows one warp marches down a 32-column work item (16, 32 or 64; 4, 32 x
 * 16 items split over four warps of a CTA; 1, 32 x 16 items stepped by a CTA in three phases
 * through shared memory), the order items are dealt (0 tiles by index, 1 the largest tiles
 * first), and the trial's time a tick. zero_apart (16, 32 and 64 rows, native ops, no Manning, no
 * open edge, no compensated source): 1 takes a zero argument of the march's divisions and square
 * roots apart from the IEEE intrinsic (sqrt(+-0) = +-0, 0 / b = +-0 for b > 0), the same bits
 * without the intrinsic's slow path: faster where many arguments are zero (dry land, wet/dry
 * fronts, still columns), slower where few are; the autotuner tries both. stage (block_rows 1):
 * 1 takes each 32 x 16 block's cells and halo into shared memory by two tensor copies (TMA) in
 * place of each thread's loads, for tiles whose width is a multiple of 4 (the others load cell by
 * cell); the same bits either way. */
typedef struct wl_tuning {
  uint32_t block_rows;
  uint32_t order;
  float us_per_tick;
  uint32_t zero_apart;
  uint32_t stage;
} wl_tuning;

/* `common` gives cell_m, gravity, cfl, dry_depth_m and device (its nx, ny and edges are unused). */
int wl_batch_create(const wl_config* common, const wl_options* options, const wl_tile* tiles,
                    uint32_t count, wl_batch** out, char* err, size_t err_len);
void wl_batch_destroy(wl_batch* batch);
uint32_t wl_batch_tile_count(const wl_batch* batch);
uint64_t wl_batch_cell_count(const wl_batch* batch);
/* Tiles whose 32 x 16 blocks the batch's launches take by tensor copies under its tuning (block_rows
 * 1 and stage 1: the tiles whose width is a multiple of 4; else 0). A diagnosis count. */
uint32_t wl_batch_staged_tiles(const wl_batch* batch);
uint64_t wl_batch_tile_first(const wl_batch* batch, uint32_t tile);

/* write_state / set_bed / set_manning / set_source of every tile at once (total = all cells). */
int wl_batch_write_state(wl_batch* batch, const double* depth, const double* momentum_x,
                         const double* momentum_y, size_t total, char* err, size_t err_len);
/* write_state of one tile between ticks (n = its cells): its ledger emptied and its records
 * primed, every other tile's state, records and ledger untouched. The tile-start upload of a tile
 * that wakes from the baked solve (ADR-0080:30). */
int wl_batch_write_tile_state(wl_batch* batch, uint32_t tile, const double* depth,
                              const double* momentum_x, const double* momentum_y, size_t n,
                              char* err, size_t err_len);
/* The settled check of ADR-0080 decision 4 (a tile starts from the baked answer and retires to it
 * when its state has settled back within a stated bound; the retiring write is
 * wl_batch_write_tile_state): per tile, the largest |h - h*| over its cells and the largest of
 * |hu - hu*| and |hv - hv*|, against a steady state h*, hu*, hv* given as doubles tile after tile
 * (total = all cells, as wl_batch_write_state's arrays) and rounded to f32 as the step rounds its
 * own state; settled[t] = 1 when both are within depth_bound_m and momentum_bound_m2_s. The maxima
 * are order-free: the same bytes every run. Each output (count = the tiles) may be null. The
 * reference designs the check (W176) and has not built it. Waits for the device. */
int wl_batch_settled(wl_batch* batch, const double* depth, const double* momentum_x,
                     const double* momentum_y, size_t total, float depth_bound_m,
                     float momentum_bound_m2_s, uint8_t* settled, float* depth_dev_m,
                     float* momentum_dev_m2_s, uint32_t count, char* err, size_t err_len);
int wl_batch_set_bed(wl_batch* batch, const double* bed_m, size_t total, double datum_m, char* err,
                     size_t err_len);
int wl_batch_set_manning(wl_batch* batch, const double* manning, size_t total, char* err,
                         size_t err_len);
int wl_batch_set_source(wl_batch* batch, const double* source_m_per_s, size_t total,
                        uint32_t every, int compensate, char* err, size_t err_len);

/* `count` ticks of every tile, one persistent launch each, enqueued without waiting. */
int wl_batch_enqueue_ticks(wl_batch* batch, wl_stream stream, uint32_t count, float max_dt);
/* The same on the batch's own stream, replayed from a captured CUDA graph when use_graph, and
 * waited for. */
int wl_batch_run_ticks(wl_batch* batch, uint32_t count, float max_dt, int use_graph, char* err,
                       size_t err_len);
/* The per-tile-launch form, for comparison: one launch per tile per tick, on the batch's stream
 * (captured in a graph when use_graph) or, when streams > 1, dealt round-robin to that many
 * concurrent streams as independent steps would be. */
int wl_batch_enqueue_tile_tick(wl_batch* batch, wl_stream stream, uint32_t tile, float max_dt);
int wl_batch_run_tile_ticks(wl_batch* batch, uint32_t count, float max_dt, int use_graph,
                            uint32_t streams, char* err, size_t err_len);

/* Read-backs: one tile's four planes (4 * nx * ny floats), every tile's (tile after tile), each
 * tile's FNV-1a state hash, each tile's ledger (after a flush, as read_ledger does). */
int wl_batch_read_tile_bits(wl_batch* batch, uint32_t tile, float* planes, size_t count, char* err,
                            size_t err_len);
int wl_batch_read_all_bits(wl_batch* batch, float* planes, size_t count, char* err, size_t err_len);
uint64_t wl_batch_tile_hash(wl_batch* batch, uint32_t tile, char* err, size_t err_len);
int wl_batch_tile_hashes(wl_batch* batch, uint64_t* out, uint32_t count, char* err,
                         size_t err_len);
int wl_batch_read_ledgers(wl_batch* batch, wl_ledger* out, uint32_t count, char* err,
                          size_t err_len);

/* The autotuner: times every block shape, item order and (on a plain native batch) zero_apart on
 * the batch itself, each trial stepping 8 ticks untimed and then timing `trial_ticks` (the trials
 * are undone), keeps the fastest, and caches it per (SM count, tile-size histogram) for the
 * process (and across processes in the file WLCUDA_TUNING_CACHE names). */
int wl_batch_autotune(wl_batch* batch, float max_dt, uint32_t trial_ticks, wl_tuning* chosen,
                      char* err, size_t err_len);
int wl_batch_set_tuning(wl_batch* batch, const wl_tuning* tuning, char* err, size_t err_len);
int wl_batch_get_tuning(const wl_batch* batch, wl_tuning* out);
wl_stream wl_batch_stream(wl_batch* batch);

/* ---- the adjoint (no counterpart in the reference) --------------------------------------------
 *
 * For the loss L = sum over probe cells p of (h_T(p) - target_p)^2 after T ticks of fixed length
 * max_dt from the current state, the gradients dL/d(bed) and dL/d(source_m_per_s) per cell. The
 * sweep keeps the state every `every` ticks and recomputes each segment before its reverse ticks,
 * so its device memory is (T/every + every + 2) states plus three bits a cell a tick; the
 * gradients and the loss are accumulated in FP64. The forward ticks are the plain tick's
 * arithmetic to the bit (a test holds the sweep's tick-T state to wl_run_steps's); no tick may be
 * one the plain tick would shorten (wl_adjoint_read reports how many were). The sweep refuses
 * (WL_ERR_REFUSED) fixed ops, Manning friction, the compensated source and a coarser source clock.
 * A sweep reads its step's or batch's state, bed and source when it runs and changes none of them;
 * destroy it before its step or batch. */
typedef struct wl_adjoint wl_adjoint;

/* Over a step: n_probes cells (y * nx + x) and their target depths. */
int wl_adjoint_create(wl_step* step, uint32_t ticks, uint32_t every, uint32_t n_probes,
                      const uint32_t* probes, const double* targets, wl_adjoint** out, char* err,
                      size_t err_len);
/* Over a batch: tile t's probes are probes[probe_first[t] .. probe_first[t + 1]) (tile-local cells),
 * one loss a tile. */
int wl_batch_adjoint_create(wl_batch* batch, uint32_t ticks, uint32_t every,
                            const uint32_t* probe_first, const uint32_t* probes,
                            const double* targets, wl_adjoint** out, char* err, size_t err_len);
void wl_adjoint_destroy(wl_adjoint* adjoint);
/* The whole sweep on the owner's stream (wl_step_stream / wl_batch_stream), no wait. */
int wl_adjoint_enqueue(wl_adjoint* adjoint, float max_dt);
/* The sweep (replayed from one captured CUDA graph when use_graph) and a wait for it. */
int wl_adjoint_run(wl_adjoint* adjoint, float max_dt, int use_graph, char* err, size_t err_len);
/* loss: one a tile; g_bed, g_source: every tile's cells, tile after tile (null to skip); limited:
 * one count a tile of the ticks the plain tick would have shortened. */
int wl_adjoint_read(wl_adjoint* adjoint, double* loss, double* g_bed, double* g_source,
                    uint32_t* limited, char* err, size_t err_len);
/* The state of tick T: three planes (h, hu, hv) a tile, tile after tile. */
int wl_adjoint_read_final(wl_adjoint* adjoint, float* planes, char* err, size_t err_len);
/* dL/d(starting state): three planes (dL/dh, dL/dhu, dL/dhv) a tile, tile after tile, FP32 (the
 * sweep's adjoint state after its last reverse tick). */
int wl_adjoint_read_state_gradient(wl_adjoint* adjoint, float* planes, char* err, size_t err_len);
/* Kernel launches in one sweep, and the sweep's device bytes. */
uint32_t wl_adjoint_launches(const wl_adjoint* adjoint);
uint64_t wl_adjoint_device_bytes(const wl_adjoint* adjoint);

/* ---- one tick that allocates nothing (no counterpart in the reference) ------------------------
 *
 * For callers that cannot allocate device memory (a frame loop that reserved its memory at
 * start; a real-time thread): one plain tick of a caller-owned state, the records of `planes_in`
 * first (prime_main), then one update of min(stable step, max_dt) into `planes_out`. Both hold
 * four planes of nx * ny floats (h, hu, hv, remainder) on config->device; bed, and Manning's n and
 * the source when not null (the source every step, no compensation), hold nx * ny floats there.
 * `fixed_ops` selects Ops::fixed. The bytes are wl_run_steps's for one tick after wl_write_state
 * of the same state. The scratch is a fixed device array holding at most 4096 groups of 16 x 16
 * cells (1,048,576 cells as 1024 x 1024); a larger grid is refused with WL_ERR_SIZE. The first
 * call on a device looks the array's address up (cudaGetSymbolAddress): make it before any stream
 * capture. Enqueued on `stream` (null: the legacy default stream) without waiting. Calls share the
 * array: two in flight at once on one device race, so a caller runs them one after another. */
int wl_tick_noalloc(const wl_config* config, int fixed_ops, const float* planes_in,
                    float* planes_out, const float* bed, const float* manning,
                    const float* source, float max_dt, wl_stream stream, char* err,
                    size_t err_len);

/* ---- the tick queue (designed in docs/subsystems/water_live.md:76-94, ADR-0081; the reference
 * builds none of it) ----------------------------------------------------------------------------
 *
 * Ticks of the world's clock, each a length in the state's time and the events that take effect
 * at its start, queued on the device and stepped by "slots" the caller enqueues (or captures into
 * a CUDA graph once and replays every frame). A slot has two launches:
 *   - begin and apply, one CTA: it settles the last slot (a landed tick's read-back record), and
 *     when no tick is in flight and one is queued, begins it (the step's time left becomes its
 *     length) and writes its events into the step's planes, in push order.
 *   - the tick: one sub-step of min(stable step, time left), or nothing when no tick is in flight.
 * A call adds one more launch after its slots, which settles the last of them.
 * Every sub-step's length is chosen on the device from the state alone, so the bytes are those of
 * wl_advance(length) per tick with the events applied between, however many slots each call
 * enqueues: a slot past the work changes nothing. A tick of length 0 carries its events alone.
 * While a queue is attached, wl_run_steps, wl_enqueue_steps, wl_advance, wl_write_state(_device)
 * and a coarser source clock are refused: the queue owns the step's clock (water_live.md:92). A
 * queued tick's sub-steps read the bed, Manning's n and the source as they stand, so change them
 * through events to keep a run's bytes independent of the slots. Destroy the queue before its
 * step (wl_destroy of the step also detaches it). */
typedef struct wl_queue wl_queue;

enum {
  WL_EVENT_BED = 0,     /* the bed's heights over the rectangle (metres, the step's f32 datum) */
  WL_EVENT_SOURCE = 1,  /* the source over the rectangle (m/s); the step must have a source on */
  WL_EVENT_MANNING = 2, /* Manning's n over the rectangle; the step must have Manning on */
  /* The state over the rectangle: 3 * w * h values, the depths' rectangle, then hu's, then hv's
   * (the remainder plane there becomes 0). The apply pass that writes a waking tile's starting
   * state at its tick's boundary (water_live.md:80; ADR-0080 decision 4: a tile starts from the
   * baked answer). In order: the tile's pending records are folded into its ledger (dt_main with
   * max_dt 0, the flush), the rectangle is written, and the tile's records become those of its
   * new state (prime_main, slang:373-386). */
  WL_EVENT_STATE = 3
};

/* One event: a rectangle of one plane of one tile replaced by w * h values, row by row (tile 0
 * for a step's queue; 3 * w * h for WL_EVENT_STATE). */
typedef struct wl_event {
  uint32_t kind;
  uint32_t x0, y0, w, h;
  uint32_t tile;
} wl_event;

/* What a landed tick leaves (water_live.md:94): its number, its sub-steps, its shortest and
 * longest sub-step, and the ledger's time and step count when it landed; whether it was dropped
 * (stepped by none of its sub-steps, its events applied all the same), the drops so far, the lag
 * when it began (ticks pushed and not landed, itself included) and whether the domain was frozen
 * after it landed. */
typedef struct wl_landed {
  uint32_t tick;
  uint32_t substeps;
  float shortest_s;
  float longest_s;
  float time_hi;
  float time_lo;
  uint32_t steps;
  uint32_t events;
  uint32_t dropped;
  uint32_t dropped_total;
  uint32_t lag;
  uint32_t frozen;
} wl_landed;

typedef struct wl_queue_status {
  uint32_t pushed;   /* ticks pushed since the queue was made */
  uint32_t begun;    /* ticks begun */
  uint32_t landed;   /* ticks landed (dropped ones included); pushed - landed is the lag */
  uint32_t active;   /* 1 while a begun tick has not landed */
  uint32_t substeps; /* sub-steps of the tick in flight */
  uint32_t dropped;  /* ticks dropped by a freeze */
  uint32_t frozen;   /* 1 while the domain is frozen */
  uint32_t freezes;  /* times the domain froze */
} wl_queue_status;

/* A queue of `records` ticks (at most 64 in flight: water_live.md:84) over a step, with an event
 * arena of `arena_values` floats and room for `max_events` events. */
int wl_queue_create(wl_step* step, uint32_t records, uint32_t arena_values, uint32_t max_events,
                    wl_queue** out, char* err, size_t err_len);
/* The same over a batch: the domain's tiles take every tick together, each by its own sub-steps
 * (min(its stable step, its time left)); a tick lands when every tile has; a tile that has landed
 * waits through the slots the others still take. While attached, the batch refuses its own ticks,
 * tuning, autotuning and state writes. */
int wl_batch_queue_create(wl_batch* batch, uint32_t records, uint32_t arena_values,
                          uint32_t max_events, wl_queue** out, char* err, size_t err_len);
void wl_queue_destroy(wl_queue* queue);
/* Queues one tick: its number, its length (s, >= 0) and its events with their values, in order
 * (sum of w * h values). Waits for the copy. WL_ERR_REFUSED when the ring, the event ring or the
 * arena has no room yet: the caller keeps the tick and pushes it after slots have begun others. */
int wl_queue_push(wl_queue* queue, uint32_t tick, float length_s, const wl_event* events,
                  uint32_t n_events, const float* values, size_t n_values, char* err,
                  size_t err_len);
/* The lag control of water_live.md:90-92 (0: off, the default for both):
 *   - lag_limit_ticks: when a slot begins a tick while more than this many ticks are pushed and
 *     not landed (a quarter second of ticks is the reference's bound), the domain freezes as it
 *     stands: each queued tick is then dropped, one a slot (its events applied in order, no
 *     sub-step, landed with `dropped` set), and counted, until the queue has drained; then it
 *     thaws, and the next tick pushed steps as before;
 *   - max_slots: the most slots one call enqueues (a frame's ceiling, `water_live.frame.max_slots`);
 *     a call that asks for more enqueues max_slots.
 * Waits for the device; call it between slots. */
int wl_queue_set_limits(wl_queue* queue, uint32_t lag_limit_ticks, uint32_t max_slots, char* err,
                        size_t err_len);
/* `slots` slots on `stream` (null: the step's own stream), no wait; graph-capturable. */
int wl_queue_enqueue_slots(wl_queue* queue, wl_stream stream, uint32_t slots);
/* The slots, then a wait. */
int wl_queue_run_slots(wl_queue* queue, uint32_t slots, char* err, size_t err_len);
int wl_queue_status_read(wl_queue* queue, wl_queue_status* out, char* err, size_t err_len);
/* The read-back records of landed ticks first .. first + count - 1 (the 0-based landing order);
 * the last `records` landings are kept. */
int wl_queue_read_landed(wl_queue* queue, uint32_t first, uint32_t count, wl_landed* out,
                         char* err, size_t err_len);
/* Launches a slot makes (2), and the queue's device bytes. */
uint32_t wl_queue_launches_per_slot(void);
uint64_t wl_queue_device_bytes(const wl_queue* queue);

/* ---- the complete FP64 step: engine::water_state::Solver on the device -------------------------
 *
 * domain/water_state/include/domain/water_state/water_state.h:161-266 and
 * domain/water_state/src/water_state.cpp, with every input and output the reference's CPU step
 * has and the live tick lacks: the ground's store by Green and Ampt, up to four carried
 * quantities (decay, a source from the dissipation, an outside source, an exchange with the bed),
 * the per-cell speed, bed stress and dissipation, and the whole ledger. The arithmetic is IEEE
 * double in the reference's operand order with no contraction, and its cube root and decay take
 * fdlibm's e^x and ln x as the reference's deterministic transcendentals do, so a step's bytes
 * (state, outputs, ledger) equal the reference's CPU Solver's. Inputs are held on the device
 * between steps (set once, changed with ws_set_input); the reference takes them with each step. */
typedef struct ws_solver ws_solver;

typedef struct ws_carried_config { /* water_state.h:66-78 */
  double decay_s;
  double per_joule;
  double min_speed_m_per_s;
} ws_carried_config;

typedef struct ws_config { /* water_state.h:83-99; rows_per_job is not read */
  uint32_t nx;
  uint32_t ny;
  double cell_m;
  double gravity;
  double cfl;
  double dry_depth_m;
  double water_density;
  uint32_t carried; /* carried quantities in use, at most 4 */
  uint32_t pad;
  ws_carried_config carried_config[4];
  uint8_t west_open; /* water_state::Edge: 0 closed, 1 open */
  uint8_t east_open;
  uint8_t south_open;
  uint8_t north_open;
  int32_t device;
} ws_config;

typedef struct ws_carried_ledger { /* water_state.h:124-130 */
  double source, from_dissipation, exchange, decayed, open_edge_out;
} ws_carried_ledger;

typedef struct ws_ledger { /* water_state.h:135-145 */
  double source_m3, open_edge_out_m3, ground_m3, roundoff_m3, scheme_loss_j, friction_work_j;
  double time_s;
  uint64_t steps;
  ws_carried_ledger carried[4];
} ws_ledger;

/* The fields (water_state.h:147-160): the state, then the last step's outputs (read only). */
enum {
  WS_DEPTH = 0, WS_MOMENTUM_X = 1, WS_MOMENTUM_Y = 2, WS_GROUND = 3,
  WS_CARRIED = 4, /* carried * nx * ny values, quantity after quantity */
  WS_SPEED = 5, WS_BED_STRESS_X = 6, WS_BED_STRESS_Y = 7, WS_DISSIPATION = 8
};
/* The inputs (water_state.h:103-120). */
enum {
  WS_BED = 0, WS_MANNING = 1, WS_SOURCE = 2, WS_GROUND_CONDUCTIVITY = 3, WS_GROUND_SUCTION = 4,
  WS_GROUND_CAPACITY = 5,
  WS_CARRIED_SOURCE = 6,  /* + k for quantity k */
  WS_CARRIED_EXCHANGE = 10 /* + k */
};

/* Solver::Solver (cpp:110-148): every array allocated once, the state zero, the ledger empty. */
int ws_create(const ws_config* config, ws_solver** out, char* err, size_t err_len);
void ws_destroy(ws_solver* solver);
int ws_valid(const ws_solver* solver);
uint32_t ws_cell_count(const ws_solver* solver);
/* depth() ... carried(k) (water_state.h:167-180): n = the field's size. */
int ws_write_field(ws_solver* solver, int field, const double* values, size_t n, char* err,
                   size_t err_len);
int ws_read_field(ws_solver* solver, int field, double* out, size_t n, char* err, size_t err_len);
/* One of Inputs' spans, kept on the device: n = nx * ny, or 0 for an empty span. */
int ws_set_input(ws_solver* solver, int input, const double* values, size_t n, char* err,
                 size_t err_len);
/* Solver::stable_step (cpp:211-224); 0 on an error. */
double ws_stable_step(ws_solver* solver, char* err, size_t err_len);
/* Solver::step (cpp:503-533): the length taken; 0 when the inputs do not fit (no bed, or the
 * ground's three spans not all set or all empty) or max_dt <= 0, nothing changed then. */
double ws_step(ws_solver* solver, double max_dt, char* err, size_t err_len);
/* `count` steps on `stream` (null: the solver's own), no wait; graph-capturable. WL_ERR_SIZE when
 * the inputs do not fit, WL_ERR_ARGUMENT for max_dt <= 0. */
int ws_enqueue_steps(ws_solver* solver, wl_stream stream, uint32_t count, double max_dt);
int ws_run_steps(ws_solver* solver, uint32_t count, double max_dt, char* err, size_t err_len);
/* Solver::advance (cpp:535-547): the steps taken; 0 when the inputs do not fit. */
uint64_t ws_advance(ws_solver* solver, double duration_s, char* err, size_t err_len);
int ws_read_ledger(ws_solver* solver, ws_ledger* out, char* err, size_t err_len);
int ws_reset_ledger(ws_solver* solver, char* err, size_t err_len);
/* The volumes (cpp:549-568): sums in index order times a cell's area. */
double ws_surface_volume_m3(ws_solver* solver, char* err, size_t err_len);
double ws_ground_volume_m3(ws_solver* solver, char* err, size_t err_len);
double ws_carried_total(ws_solver* solver, uint32_t k, char* err, size_t err_len);
/* Solver::state_hash (cpp:570-578). 0 on an error. */
uint64_t ws_state_hash(ws_solver* solver, char* err, size_t err_len);
wl_stream ws_stream(ws_solver* solver);
uint64_t ws_device_bytes(const ws_solver* solver);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* WLCUDA_H */

// The live-water tick's kernels for sm_103a.
//
// One persistent launch steps every tile of a batch by one tick (the plain step is a batch of one
// tile). It replaces the reference's two passes a step, the length pass `dt_main`
// (water_step.slang:412-479) and the update `update_main` (slang:555-757), with one:
//
//   - A work item is a band of one tile: 32 columns by H rows. Each warp takes items from a
//     counter and steps them alone; no item waits for another and no barrier spans warps.
//   - The item chooses the step's length itself from the tile's control block: the largest
//     speeds of the last update (kept by atomicMax on their bits, exact in any order), the time
//     left and max_dt, the same arithmetic as dt_main's thread 0.
//   - The warp that takes a tile's first item also folds the last update's records into the
//     ledger in dt_main's own order (256 lanes over the records, then a fixed tree), so the
//     ledger's bits are the reference's.
//   - The warp marches down its band, a lane a column. Each row it loads the row two ahead (the
//     loads are in flight while it computes), computes the north face of its cell and its west
//     face (the west neighbour's state by shuffle), takes its east face from the lane to its
//     right by shuffle, and updates the cell; the north face is carried up as the next row's south
//     face. Each face is computed once, so both cells of a face take the same value, which is
//     what the reference's gather computes twice. The band's side columns (the west neighbour of
//     lane 0 and the east face of the last lane) are computed first, a row a lane.
//   - Every 16 rows the warp writes the records of the two 16 x 16 groups it covers, with the
//     reference's 256-slot tree over each group's volumes.
//   - What a tick writes besides the planes goes to the other of two slots: the tile's first item
//     writes the new ledger there, and every item adds its largest speeds there by atomicMax. The
//     last item of a tile to finish flips the copy, the records and the slots, and moves the
//     source's clock. Nothing a launch writes is read in the same launch, so no item fences its
//     writes: the next launch sees them at the kernel boundary.
//
// Two other shapes share the items, the update (update_cell) and the last item's flip: the split
// march (tick_split_kernel: a 32 x 16 item by a CTA's four warps, four rows each, for small tiles)
// and the block tick (tick_block_kernel: a 32 x 16 item by 256 threads in three phases through
// shared memory; the small-tile default and the stored-faces form; its staged variant takes a
// block and its halo by two tensor copies). Every shape gives the same bytes.
//
// HBM traffic per cell-update: h, hu, hv, bed read (+ source, + Manning's n, + the remainder when
// on), h, hu, hv written (+ the remainder), a 32-byte record per 256 cells.
#include "wl_device.cuh"
#include "wl_kernels.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

namespace wlc {

namespace {

constexpr int kStrip = 32;        // an item is a warp wide
constexpr int kWarpsPerCta = 4;   // 128 threads a CTA
constexpr int kCtaThreads = 32 * kWarpsPerCta;

// A warp's shared memory: the band's side columns and a ring of 16 rows of per-cell volumes.
template <int H>
struct WarpMem {
  static constexpr size_t kBytes = 2 * H * sizeof(float4) + 3 * 16 * kStrip * sizeof(float);
  float4* west;  // H: {h, z, u, v} of the column west of lane 0, row by row
  float4* east;  // H: the east face of the band's last live lane, row by row
  float* ring;   // 3 x 16 x 32: the source, open-edge and roundoff volumes of the last 16 rows
};

template <int H>
__device__ __forceinline__ WarpMem<H> warp_mem(int warp) {
  extern __shared__ float4 smem[];
  char* base = reinterpret_cast<char*>(smem) + size_t(warp) * WarpMem<H>::kBytes;
  WarpMem<H> m;
  m.west = reinterpret_cast<float4*>(base);
  m.east = m.west + H;
  m.ring = reinterpret_cast<float*>(m.east + H);
  return m;
}

__device__ __forceinline__ uint32_t item_tile_of(const uint32_t* item_tile, uint32_t item) {
  return item_tile == nullptr ? 0u : item_tile[item];
}

// The next item of one of a persistent tick's `slots` takers (CTAs or warps), the one numbered
// `own`: its own number first, then slots + the work counter's next value. A launch of no more
// takers than items (a small tile's) reads no counter, and leaves it as it found it.
__device__ __forceinline__ uint32_t take_item(WorkCtl* w, bool first, uint32_t own, uint32_t slots,
                                              uint32_t n) {
  if (first) return own;
  if (slots >= n) return n;
  return slots + atomicAdd(&w->next, 1u);
}


// ---- the ledger ---------------------------------------------------------------------------

// dt_main's sums (slang:417-456) by one warp: virtual lane L of 256 adds records L, L + 256, ...
// in order, then the fixed 256-slot tree. Leaves the three sums in s[0], s[256], s[512].
__device__ void fold_warp(const Partial* rec, uint32_t groups, float* s) {
  const int lane = threadIdx.x & 31;
  for (int vl = lane; vl < int(kGroupCells); vl += 32) {
    float src = 0.0f, opn = 0.0f, rnd = 0.0f;
    for (uint32_t gi = vl; gi < groups; gi += kGroupCells) {
      const Partial p = rec[gi];
      src = __fadd_rn(src, p.source_m3);
      opn = __fadd_rn(opn, p.open_m3);
      rnd = __fadd_rn(rnd, p.roundoff_m3);
    }
    s[vl] = src;
    s[kGroupCells + vl] = opn;
    s[2 * kGroupCells + vl] = rnd;
  }
  __syncwarp();
  for (int stride = kGroupCells / 2; stride > 0; stride >>= 1) {
    for (int vl = lane; vl < stride; vl += 32) {
      s[vl] = __fadd_rn(s[vl], s[vl + stride]);
      s[kGroupCells + vl] = __fadd_rn(s[kGroupCells + vl], s[kGroupCells + vl + stride]);
      s[2 * kGroupCells + vl] =
          __fadd_rn(s[2 * kGroupCells + vl], s[2 * kGroupCells + vl + stride]);
    }
    __syncwarp();
  }
}

// The same by a CTA of 256 threads, a thread a virtual lane: the records of each lane in flight at
// once rather than a warp's eight lanes one after another (the block tick's first item, on a small
// tile's critical path). The same sums in the same order.
__device__ void fold_block(const Partial* rec, uint32_t groups, float* s) {
  const int t = threadIdx.x;  // threads past the 256 virtual lanes take only the barriers
  if (t < int(kGroupCells)) {
    float src = 0.0f, opn = 0.0f, rnd = 0.0f;
    for (uint32_t gi = t; gi < groups; gi += kGroupCells) {
      const Partial p = rec[gi];
      src = __fadd_rn(src, p.source_m3);
      opn = __fadd_rn(opn, p.open_m3);
      rnd = __fadd_rn(rnd, p.roundoff_m3);
    }
    s[t] = src;
    s[kGroupCells + t] = opn;
    s[2 * kGroupCells + t] = rnd;
  }
  __syncthreads();
  for (int stride = kGroupCells / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      s[t] = __fadd_rn(s[t], s[t + stride]);
      s[kGroupCells + t] = __fadd_rn(s[kGroupCells + t], s[kGroupCells + t + stride]);
      s[2 * kGroupCells + t] = __fadd_rn(s[2 * kGroupCells + t], s[2 * kGroupCells + t + stride]);
    }
    __syncthreads();
  }
}

// The same with a CTA of 256 threads, the records' sums cleared after they are read and their
// largest speeds returned (the length pass, slang:412-456).
__device__ void fold_cta(Partial* rec, uint32_t groups, float* s, uint32_t* s_ab) {
  const int t = threadIdx.x;
  if (t == 0) {
    s_ab[0] = 0u;
    s_ab[1] = 0u;
  }
  __syncthreads();
  float src = 0.0f, opn = 0.0f, rnd = 0.0f;
  uint32_t a = 0u, b = 0u;
  for (uint32_t gi = t; gi < groups; gi += kGroupCells) {
    const Partial p = rec[gi];
    src = __fadd_rn(src, p.source_m3);
    opn = __fadd_rn(opn, p.open_m3);
    rnd = __fadd_rn(rnd, p.roundoff_m3);
    a = max(a, __float_as_uint(p.speed_x));
    b = max(b, __float_as_uint(p.speed_y));
    rec[gi].source_m3 = 0.0f;
    rec[gi].open_m3 = 0.0f;
    rec[gi].roundoff_m3 = 0.0f;
  }
  s[t] = src;
  s[kGroupCells + t] = opn;
  s[2 * kGroupCells + t] = rnd;
  atomicMax(&s_ab[0], a);
  atomicMax(&s_ab[1], b);
  __syncthreads();
  for (int stride = kGroupCells / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      s[t] = __fadd_rn(s[t], s[t + stride]);
      s[kGroupCells + t] = __fadd_rn(s[kGroupCells + t], s[kGroupCells + t + stride]);
      s[2 * kGroupCells + t] = __fadd_rn(s[2 * kGroupCells + t], s[2 * kGroupCells + t + stride]);
    }
    __syncthreads();
  }
}

// dt_main's thread 0 (slang:457-478): the sums into the ledger's pairs, then the step's length.
template <bool FIXED>
__device__ void ledger_update(LedgerBits& l, float src, float opn, float rnd, float a, float b,
                              float cfl, float cell_m, float max_dt) {
  pair_add(l.source_hi, l.source_lo, src);
  pair_add(l.open_hi, l.open_lo, opn);
  pair_add(l.roundoff_hi, l.roundoff_lo, rnd);
  if (max_dt > 0.0f) {
    const float dt = choose_dt<FIXED>(a, b, cfl, cell_m, max_dt, l.remaining_s);
    l.remaining_s = __fsub_rn(l.remaining_s, dt);
    l.dt = dt;
    pair_add(l.time_hi, l.time_lo, dt);
    l.steps = l.steps + (dt > 0.0f ? 1u : 0u);
  } else {
    l.dt = 0.0f;
  }
}

// The flip of a tile's control block once every item of its launch is done: slot `rec`'s largest
// speeds cleared (every item has read them, its step's length), and for a tick the copy flipped
// and the source's clock moved; a prime flips only the records. Run by the tile's last item
// (finish_item) or by the resident tick's barrier.
__device__ void flip_tile(const TileDesc& T, uint32_t rec, bool tick) {
  volatile TileCtl* v = T.ctl;
  v->max_a[rec] = 0u;
  v->max_b[rec] = 0u;
  if (tick) {
    v->cur = v->cur ^ 1u;
    if ((T.flags & kFlagSource) != 0u && T.source_every > 1u) {
      const uint32_t p = v->src_phase + 1u;
      v->src_phase = p == T.source_every ? 0u : p;
    }
    v->ticks = v->ticks + 1u;
  }
  v->rec = rec ^ 1u;
  v->done = 0u;
}

// The end of a work item (one thread): its largest speeds into slot rec ^ 1 of the tile's maxima
// and, for the tile's last item, the flip. No fence: the item's planes, records and maxima are
// read by the next launch, and the flip reads only fields no other item writes. `extra` counts a
// CTA that folded the ledger apart from the items (1) or none (0).
__device__ void finish_item(const TileDesc& T, uint32_t rec, uint32_t amax, uint32_t bmax,
                            bool tick, uint32_t extra = 0u) {
  TileCtl* ctl = T.ctl;
  atomicMax(&ctl->max_a[rec ^ 1u], amax);
  atomicMax(&ctl->max_b[rec ^ 1u], bmax);
  const uint32_t d = atomicAdd(&ctl->done, 1u);
  if (d + 1u != T.items + extra) return;
  flip_tile(T, rec, tick);
}

// ---- the records ----------------------------------------------------------------------------

// One group's 256-slot tree (slang:346-358) by one warp: lane l holds slots l + 32 k (slot
// i = ly * 16 + lx), so strides 128, 64 and 32 are adds in registers and 16..1 are shuffles.
// `ring` holds the 16 rows x 32 lanes of one quantity; the group is columns 16 gc .. 16 gc + 15.
__device__ __forceinline__ float group_tree(const float* ring, int gc) {
  const int lane = threadIdx.x & 31;
  float v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int slot = lane + 32 * k;
    v[k] = ring[(slot >> 4) * kStrip + 16 * gc + (slot & 15)];
  }
  const float a0 = __fadd_rn(v[0], v[4]), a1 = __fadd_rn(v[1], v[5]);
  const float a2 = __fadd_rn(v[2], v[6]), a3 = __fadd_rn(v[3], v[7]);
  const float b0 = __fadd_rn(a0, a2), b1 = __fadd_rn(a1, a3);
  float c = __fadd_rn(b0, b1);
#pragma unroll
  for (int stride = 16; stride > 0; stride >>= 1) {
    const float o = __shfl_down_sync(0xffffffffu, c, stride);
    if (lane < stride) c = __fadd_rn(c, o);
  }
  return c;
}

// The records of the two groups a warp covers in one group row (slang:338-371), the groups'
// largest speeds given: (ga, gb) the west group's, (a1, b1) the east group's. The ring holds the
// volumes of the group row's 16 rows (rows past the grid's edge zero); need_* names the quantities
// some cell holds. Lane 0 writes the records and adds the two groups' speeds to ia, ib.
__device__ __forceinline__ void write_group_records(uint32_t groups_x, uint32_t groups_y,
                                                    Partial* rec_out, int X0, int group_row,
                                                    uint32_t ga, uint32_t gb, uint32_t a1,
                                                    uint32_t b1, const float* ring,
                                                    bool need_src, bool need_opn, bool need_rnd,
                                                    uint32_t& ia, uint32_t& ib) {
  const int lane = threadIdx.x & 31;
  float s0 = 0.0f, s1 = 0.0f, o0 = 0.0f, o1 = 0.0f, r0 = 0.0f, r1 = 0.0f;
  if (need_src) {
    s0 = group_tree(ring, 0);
    s1 = group_tree(ring, 1);
  }
  if (need_opn) {
    o0 = group_tree(ring + 16 * kStrip, 0);
    o1 = group_tree(ring + 16 * kStrip, 1);
  }
  if (need_rnd) {
    r0 = group_tree(ring + 32 * kStrip, 0);
    r1 = group_tree(ring + 32 * kStrip, 1);
  }
  if (lane == 0) {
    const uint32_t gyg = uint32_t(group_row);
    const uint32_t gx0 = uint32_t(X0 / 16);
    if (gyg < groups_y) {
      if (gx0 < groups_x) {
        float4* d = reinterpret_cast<float4*>(rec_out + size_t(gyg) * groups_x + gx0);
        d[0] = make_float4(__uint_as_float(ga), __uint_as_float(gb), s0, o0);
        d[1] = make_float4(r0, 0.0f, 0.0f, 0.0f);
      }
      if (gx0 + 1u < groups_x) {
        float4* d = reinterpret_cast<float4*>(rec_out + size_t(gyg) * groups_x + gx0 + 1u);
        d[0] = make_float4(__uint_as_float(a1), __uint_as_float(b1), s1, o1);
        d[1] = make_float4(r1, 0.0f, 0.0f, 0.0f);
      }
    }
    ia = max(ia, max(ga, a1));
    ib = max(ib, max(gb, b1));
  }
  __syncwarp();
}
// The same from each lane's largest speeds over the group row (lanes 0-15 the west group's,
// 16-31 the east group's).
__device__ __forceinline__ void group_records(uint32_t groups_x, uint32_t groups_y,
                                              Partial* rec_out, int X0, int group_row,
                                              uint32_t ga, uint32_t gb, const float* ring,
                                              bool need_src, bool need_opn, bool need_rnd,
                                              uint32_t& ia, uint32_t& ib) {
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    ga = max(ga, __shfl_xor_sync(0xffffffffu, ga, o));
    gb = max(gb, __shfl_xor_sync(0xffffffffu, gb, o));
  }
  const uint32_t a1 = __shfl_sync(0xffffffffu, ga, 16), b1 = __shfl_sync(0xffffffffu, gb, 16);
  write_group_records(groups_x, groups_y, rec_out, X0, group_row, ga, gb, a1, b1, ring, need_src,
                      need_opn, need_rnd, ia, ib);
}

// ---- the march ------------------------------------------------------------------------------

struct Item {
  uint32_t cur, rec, apply_source;
  float dt, scale;
  int X0, Y0;
};

// {h, z, u, v} of a cell from its loaded h, hu, hv and bed (slang:303-314).
template <bool FIXED, bool ZG = false>
__device__ __forceinline__ float4 velocities(float h, float hu, float hv, float z, float dry) {
  const bool wet = h >= dry;
  const float u = wet ? zdiv<FIXED, ZG>(hu, h) : 0.0f;
  const float v = wet ? zdiv<FIXED, ZG>(hv, h) : 0.0f;
  return make_float4(h, z, u, v);
}

template <bool FIXED, bool ZG = false>
__device__ __forceinline__ float4 load_cell(const float* ph, const float* phu, const float* phv,
                                            const float* bed, int i, float dry) {
  return velocities<FIXED, ZG>(ph[i], phu[i], phv[i], bed[i], dry);
}

// An x face between cells L and R; a y face between cells S and N (slang:274-292, 597-628).
template <bool FIXED, bool ZG = false>
__device__ __forceinline__ float4 face_x(float g, float hg, const float4& L, const float4& R) {
  return face<FIXED, ZG>(g, hg, L.x, L.y, L.z, L.w, R.x, R.y, R.z, R.w);
}
template <bool FIXED, bool ZG = false>
__device__ __forceinline__ float4 face_y(float g, float hg, const float4& S, const float4& N) {
  return face<FIXED, ZG>(g, hg, S.x, S.y, S.w, S.z, N.x, N.y, N.w, N.z);
}

__device__ __forceinline__ float4 shfl_up4(const float4& v) {
  return make_float4(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1),
                     __shfl_up_sync(0xffffffffu, v.z, 1), __shfl_up_sync(0xffffffffu, v.w, 1));
}
__device__ __forceinline__ float4 shfl_down4(const float4& v) {
  return make_float4(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1),
                     __shfl_down_sync(0xffffffffu, v.z, 1), __shfl_down_sync(0xffffffffu, v.w, 1));
}

// One tick's per-cell constants of the update.
struct UpdateCtx {
  float g, dry, lam, area, edge_volume, dt, scale;
  uint32_t flags;
  int nx, ny;
  bool src_on, comp, manning, any_open;
};

// update_main's per cell (slang:630-757): the four faces' fluxes into U' = U - dt/dx ((F_e - F_w)
// + (F_n - F_s)), the clamp, the source (plain or compensated), Manning's friction and the dry
// test. Gives h, hu, hv and the remainder, and adds the cell's source, open-edge and roundoff
// volumes. `resid_in` is the cell's plane 3 (read when compensating), `nn` its Manning's n.
template <bool FIXED>
__device__ __forceinline__ void update_cell(const UpdateCtx& u, const float4& c, float hu, float hv,
                                            float src, float resid_in, float nn, const float4& fw,
                                            const float4& fe, const float4& fs, const float4& fn,
                                            int gx, int gy, float& h, float& mu, float& mv,
                                            float& residual, float& csrc, float& copn,
                                            float& crnd) {
  using O = Ops<FIXED>;
  const uint32_t flags = u.flags;
  if (u.any_open) {
    if (gx == 0 && (flags & kFlagWestOpen)) copn = __fsub_rn(copn, __fmul_rn(fw.x, u.edge_volume));
    if (gx + 1 == u.nx && (flags & kFlagEastOpen)) copn = __fadd_rn(copn, __fmul_rn(fe.x, u.edge_volume));
    if (gy == 0 && (flags & kFlagSouthOpen)) copn = __fsub_rn(copn, __fmul_rn(fs.x, u.edge_volume));
    if (gy + 1 == u.ny && (flags & kFlagNorthOpen)) copn = __fadd_rn(copn, __fmul_rn(fn.x, u.edge_volume));
  }
  const float lam = u.lam, area = u.area, dt = u.dt, scale = u.scale;
  // U' = U - dt/dx ((F_e - F_w) + (F_n - F_s)) (slang:653-668)
  h = __fsub_rn(c.x, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.x, fw.x), __fsub_rn(fn.x, fs.x))));
  mu = __fsub_rn(hu, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.y, fw.z), __fsub_rn(fn.w, fs.w))));
  mv = __fsub_rn(hv, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.w, fw.w), __fsub_rn(fn.y, fs.z))));
  if (h < 0.0f) {
    crnd = __fsub_rn(crnd, __fmul_rn(h, area));
    h = 0.0f;
  }
  residual = 0.0f;
  if (u.comp) residual = resid_in;
  if (u.src_on && u.comp) {
    const float owed = __fmul_rn(src, dt);
    const float scaled = __fmul_rn(owed, scale);
    const float target = __fadd_rn(scaled, residual);
    float h2 = h;
    if (target >= 0.0f) {
      h2 = __fadd_rn(h, target);
    } else {
      const float want = -target;
      const float taken = want < h ? want : h;
      h2 = __fsub_rn(h, taken);
    }
    const float applied = __fsub_rn(h2, h);
    const float left = __fsub_rn(target, applied);
    residual = (h2 == 0.0f && target < 0.0f) ? 0.0f : left;
    csrc = __fadd_rn(csrc, __fmul_rn(applied, area));
    h = h2;
  } else if (u.src_on) {
    const float owed = __fmul_rn(src, dt);
    const float added = __fmul_rn(owed, scale);
    if (added >= 0.0f) {
      h = __fadd_rn(h, added);
      csrc = __fadd_rn(csrc, __fmul_rn(added, area));
    } else {
      const float want = -added;
      const float taken = want < h ? want : h;
      h = __fsub_rn(h, taken);
      csrc = __fsub_rn(csrc, __fmul_rn(taken, area));
    }
  }
  if (h >= u.dry) {
    if (u.manning) {
      // (hu)' = (hu)* / (1 + dt g n^2 |u*| / h^(4/3)) (slang:722-744)
      const float g = u.g;
      const float uu = O::div(mu, h);
      const float vv = O::div(mv, h);
      const float sp = O::sqrt(__fadd_rn(__fmul_rn(uu, uu), __fmul_rn(vv, vv)));
      const float cb = O::cbrt(h);
      const float k3 = __fmul_rn(__fmul_rn(__fmul_rn(g, nn), nn), sp);
      const float k = O::div(k3, __fmul_rn(h, cb));
      const float denom = __fadd_rn(1.0f, __fmul_rn(dt, k));
      mu = O::div(mu, denom);
      mv = O::div(mv, denom);
    }
  } else {
    mu = 0.0f;
    mv = 0.0f;
  }
}

// The end of a split march: this warp's rows past the grid's edge hold nothing in the shared ring,
// its largest speeds go to the item's two groups (s_ab: a, b of the west group, a, b of the east)
// and the quantities some cell holds to s_need (1 open-edge, 2 roundoff).
__device__ __forceinline__ void split_partials(float* ring, int ring_row0, int rows, uint32_t ga,
                                               uint32_t gb, bool opn_seen, bool rnd_seen,
                                               uint32_t* s_ab, uint32_t* s_need) {
  const int lane = threadIdx.x & 31;
  for (int r = max(rows, 0); r < 4; ++r) {
    const int slot = (ring_row0 + r) * kStrip + lane;
    ring[slot] = 0.0f;
    ring[16 * kStrip + slot] = 0.0f;
    ring[32 * kStrip + slot] = 0.0f;
  }
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    ga = max(ga, __shfl_xor_sync(0xffffffffu, ga, o));
    gb = max(gb, __shfl_xor_sync(0xffffffffu, gb, o));
  }
  const bool any_opn = __any_sync(0xffffffffu, opn_seen);
  const bool any_rnd = __any_sync(0xffffffffu, rnd_seen);
  if ((lane & 15) == 0) {
    atomicMax(&s_ab[(lane >> 4) * 2], ga);
    atomicMax(&s_ab[(lane >> 4) * 2 + 1], gb);
  }
  if (lane == 0 && (any_opn || any_rnd)) atomicOr(s_need, (any_opn ? 1u : 0u) | (any_rnd ? 2u : 0u));
}

// One item: a band of 32 columns by up to H rows of one tile, one tick. SPLIT: the warp's H rows
// are rows ring_row0 .. ring_row0 + H - 1 of a 16-row item that the CTA's warps share; their
// volumes go to the CTA's ring and the records are the CTA's (split_partials, then group_records
// after the CTA's barrier).
template <bool FIXED, bool MANNING, int H, bool SPLIT, bool PLAIN = false, bool ZG = false>
__device__ void march(const TileDesc& T, const Item& it, const WarpMem<H>& wm, float* ring,
                      int ring_row0, uint32_t* s_ab, uint32_t* s_need, uint32_t& ia,
                      uint32_t& ib) {
  using O = Ops<FIXED>;
  const int lane = threadIdx.x & 31;
  const int nx = int(T.nx), ny = int(T.ny);
  const size_t n = size_t(T.nx) * T.ny;
  const int X0 = it.X0, Y0 = it.Y0;
  const int gx = X0 + lane;
  const bool col = gx < nx;
  const int last = min(kStrip - 1, nx - 1 - X0);  // the band's last live lane
  const int rows = min(H, ny - Y0);
  if (SPLIT && rows <= 0) {  // a warp below the grid's last row
    split_partials(ring, ring_row0, 0, 0u, 0u, false, false, s_ab, s_need);
    return;
  }
  const float* in = T.state[it.cur];
  float* out = T.state[it.cur ^ 1u];
  const float* ph = in;
  const float* phu = in + n;
  const float* phv = in + 2 * n;
  float* qh = out;
  float* qhu = out + n;
  float* qhv = out + 2 * n;
  const float* bed = T.bed;
  // The row loop addresses the three state planes from one base and 32-bit offsets (a tile holds
  // at most 2^30 cells): fewer live 64-bit pointers, fewer spills in the plain variant.
  const uint32_t n32 = uint32_t(n);
  // The planes the rows read, in registers: the march's stores could alias the descriptor.
  const float* source = T.source;
  const float* manning_n = T.manning;
  const float g = T.gravity, dry = T.dry, hg = __fmul_rn(0.5f, g);
  const float dt = it.dt;
  const uint32_t flags = T.flags;
  Partial* rec_out = T.rec[it.rec ^ 1u];
  uint32_t ga = 0u, gb = 0u;

  if (!(dt > 0.0f)) {
    // A step of no length: the state as it is, to the bit (slang:576-585).
    for (int j = 0; j < rows; ++j) {
      const int gy = Y0 + j;
      if (col) {
        const int i = gy * nx + gx;
        const float h0 = ph[i], hu0 = phu[i], hv0 = phv[i];
        qh[i] = h0;
        qhu[i] = hu0;
        qhv[i] = hv0;
        out[3 * n + i] = in[3 * n + i];
        float ax, ay;
        cell_speeds<FIXED, ZG>(g, dry, h0, hu0, hv0, ax, ay);
        ga = max(ga, __float_as_uint(ax));
        gb = max(gb, __float_as_uint(ay));
      }
      if (!SPLIT && ((j & 15) == 15 || j == rows - 1)) {
        group_records(T.groups_x, T.groups_y, rec_out, X0, gy / 16, ga, gb, ring, false, false,
                      false, ia, ib);
        ga = gb = 0u;
      }
    }
    if (SPLIT) split_partials(ring, ring_row0, rows, ga, gb, false, false, s_ab, s_need);
    return;
  }

  // PLAIN: every edge closed, no compensated source, no Manning (none of kFlagsNotPlain is set).
  const float sw = (!PLAIN && (flags & kFlagWestOpen)) ? 1.0f : -1.0f;
  const float se = (!PLAIN && (flags & kFlagEastOpen)) ? 1.0f : -1.0f;
  const float ss = (!PLAIN && (flags & kFlagSouthOpen)) ? 1.0f : -1.0f;
  const float sn = (!PLAIN && (flags & kFlagNorthOpen)) ? 1.0f : -1.0f;

  // The band's side columns, a row a lane: the west neighbour of lane 0 as {h, z, u, v} (a ghost
  // at the west edge, slang:597-600), and the east face of the last live lane (against its east
  // neighbour, or its ghost at the east edge, slang:605-608).
  for (int j0 = 0; j0 < rows; j0 += 32) {
    const int j = j0 + lane;
    if (j < rows) {
      const int row = (Y0 + j) * nx;
      float4 w;
      if (X0 > 0) {
        w = load_cell<FIXED, ZG>(ph, phu, phv, bed, row + X0 - 1, dry);
      } else {
        w = load_cell<FIXED, ZG>(ph, phu, phv, bed, row, dry);
        w.z = __fmul_rn(sw, w.z);
      }
      const float4 cl = load_cell<FIXED, ZG>(ph, phu, phv, bed, row + X0 + last, dry);
      float4 e;
      if (X0 + last + 1 < nx) {
        e = load_cell<FIXED, ZG>(ph, phu, phv, bed, row + X0 + last + 1, dry);
      } else {
        e = cl;
        e.z = __fmul_rn(se, cl.z);
      }
      wm.west[j] = w;
      wm.east[j] = face_x<FIXED, ZG>(g, hg, cl, e);
    }
  }
  __syncwarp();

  // The first row, its south face, and the row above it in flight.
  const int gxc = col ? gx : 0;  // dead lanes read a live column and write nothing
  int i = Y0 * nx + gxc;
  float hu = phu[i], hv = phv[i];
  float src = it.apply_source ? source[i] : 0.0f;
  float4 c = velocities<FIXED, ZG>(ph[i], hu, hv, bed[i], dry);
  float4 fs;
  {
    float4 s;
    if (Y0 > 0) {
      s = load_cell<FIXED, ZG>(ph, phu, phv, bed, i - nx, dry);
    } else {
      s = c;
      s.w = __fmul_rn(ss, c.w);
    }
    fs = face_y<FIXED, ZG>(g, hg, s, c);
  }
  float nh = 0.0f, nhu = 0.0f, nhv = 0.0f, nz = 0.0f, nsrc = 0.0f;
  if (Y0 + 1 < ny) {
    const int k = i + nx;
    nh = ph[k];
    nhu = phu[k];
    nhv = phv[k];
    nz = bed[k];
    if (it.apply_source) nsrc = source[k];
  }

  const float cell_m = T.cell_m;
  const float area = __fmul_rn(cell_m, cell_m);
  const float lam = O::div(dt, cell_m);
  const float edge_volume = __fmul_rn(dt, cell_m);
  const bool src_on = it.apply_source != 0u;
  const bool comp = !PLAIN && (flags & kFlagCompensate) != 0u;
  const bool manning = !PLAIN && MANNING && (flags & kFlagManning) != 0u;
  const bool any_open_band = !PLAIN && (flags & 15u) != 0u;
  const float scale = it.scale;
  bool opn_seen = false, rnd_seen = false;
  const UpdateCtx uc{g, dry, lam, area, edge_volume, dt, scale, flags, nx, ny,
                     src_on, comp, manning, any_open_band};

  for (int j = 0; j < rows; ++j) {
    const int gy = Y0 + j;
    // The north cell: the row loaded last iteration, or the north ghost (slang:621-624).
    float4 nc;
    const float hu_n = nhu, hv_n = nhv, src_n = nsrc;
    if (gy + 1 < ny) {
      nc = velocities<FIXED, ZG>(nh, nhu, nhv, nz, dry);
    } else {
      nc = c;
      nc.w = __fmul_rn(sn, c.w);
    }
    // The row two ahead, in flight while this row computes.
    if (gy + 2 < ny) {
      const int k = i + 2 * nx;
      nh = in[k];
      nhu = in[n32 + uint32_t(k)];
      nhv = in[2u * n32 + uint32_t(k)];
      nz = bed[k];
      if (src_on) nsrc = source[k];
    }
    const float4 fn = face_y<FIXED, ZG>(g, hg, c, nc);
    float4 w = shfl_up4(c);
    if (lane == 0) w = wm.west[j];
    const float4 fw = face_x<FIXED, ZG>(g, hg, w, c);
    float4 fe = shfl_down4(fw);
    if (lane == last) fe = wm.east[j];

    float csrc = 0.0f, copn = 0.0f, crnd = 0.0f;
    float ax = 0.0f, ay = 0.0f;
    if (col) {
      float h, mu, mv, residual;
      update_cell<FIXED>(uc, c, hu, hv, src, comp ? in[3 * n + i] : 0.0f,
                         manning ? manning_n[i] : 0.0f, fw, fe, fs, fn, gx, gy, h, mu, mv,
                         residual, csrc, copn, crnd);
      out[i] = h;
      out[n32 + uint32_t(i)] = mu;
      out[2u * n32 + uint32_t(i)] = mv;
      if (comp) out[3 * n + i] = residual;
      cell_speeds<FIXED, ZG>(g, dry, h, mu, mv, ax, ay);
    }
    ga = max(ga, __float_as_uint(ax));
    gb = max(gb, __float_as_uint(ay));
    const int slot = ((ring_row0 + j) & 15) * kStrip + lane;
    ring[slot] = csrc;
    ring[16 * kStrip + slot] = copn;
    ring[32 * kStrip + slot] = crnd;
    opn_seen |= copn != 0.0f;
    rnd_seen |= crnd != 0.0f;
    if (!SPLIT && ((j & 15) == 15 || j == rows - 1)) {
      // The group row ends: rows past the grid's edge hold nothing, then the records.
      for (int r = (j & 15) + 1; r < 16; ++r) {
        ring[r * kStrip + lane] = 0.0f;
        ring[(16 + r) * kStrip + lane] = 0.0f;
        ring[(32 + r) * kStrip + lane] = 0.0f;
      }
      __syncwarp();
      const bool need_opn = __any_sync(0xffffffffu, opn_seen);
      const bool need_rnd = __any_sync(0xffffffffu, rnd_seen);
      group_records(T.groups_x, T.groups_y, rec_out, X0, gy / 16, ga, gb, ring, src_on, need_opn,
                    need_rnd, ia, ib);
      ga = gb = 0u;
      opn_seen = rnd_seen = false;
    }
    // Up one row.
    c = nc;
    hu = hu_n;
    hv = hv_n;
    src = src_n;
    fs = fn;
    i += nx;
  }
  if (SPLIT) split_partials(ring, ring_row0, rows, ga, gb, opn_seen, rnd_seen, s_ab, s_need);
}

// The 32 x 16 march's last items, n_whole .. n_items - 1 (fewer than the launch's warps): a CTA
// at a time, its four warps four rows each (the split march, the item's volumes in the CTA's
// shared ring, the records by warp 0 after a barrier), so that the launch's last round is a
// quarter of an item long instead of a whole one. The CTA's warps meet here when the whole items
// run out. Out of line: the whole-item march keeps its registers.
template <bool FIXED, bool MANNING, bool PLAIN, bool ZG>
__device__ __noinline__ void tail_items(TickArgs a, const WarpMem<16> wm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ uint32_t s_item, s_need;
  __shared__ uint32_t s_ab[4];
  float* ring = warp_mem<16>(0).ring;     // the item's 16 rows of volumes
  float* scratch = warp_mem<16>(1).ring;  // the ledger fold's slots
  WarpMem<4> w4;
  w4.west = wm.west;
  w4.east = wm.east;
  w4.ring = wm.ring;
  __syncthreads();  // every warp's whole items are done: warp 0's ring is the CTA's
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(&a.work->tail, 1u);
      s_need = 0u;
    }
    if (threadIdx.x < 4) s_ab[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t item = a.n_whole + s_item;
    if (item >= a.n_items) break;
    const uint32_t tile = item_tile_of(a.item_tile, item);
    const TileDesc& T = a.tiles[tile];
    const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
    const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
    const TileCtl* ctl = T.ctl;
    Item it;
    it.cur = ctl->cur;
    it.rec = ctl->rec;
    const float pa = __uint_as_float(ctl->max_a[it.rec]);
    const float pb = __uint_as_float(ctl->max_b[it.rec]);
    it.dt = choose_dt<FIXED>(pa, pb, T.cfl, T.cell_m, a.max_dt, ctl->ledger[it.rec].remaining_s);
    if (a.go != nullptr && !(ctl->ledger[it.rec].remaining_s > 0.0f)) {  // a landed tile
      __syncthreads();
      continue;
    }
    const bool src = (T.flags & kFlagSource) != 0u;
    const bool on = src && (T.source_every <= 1u || ctl->src_phase + 1u == T.source_every);
    it.apply_source = on ? 1u : 0u;
    it.scale = T.source_every > 1u ? float(T.source_every) : 1.0f;
    it.X0 = int(bx) * kStrip;
    const int Y0 = int(by) * 16;
    it.Y0 = Y0 + 4 * warp;
    if (local == 0u && warp == 1) {
      fold_warp(T.rec[it.rec], T.groups_x * T.groups_y, scratch);
      if (lane == 0) {
        LedgerBits l = ctl->ledger[it.rec];
        ledger_update<FIXED>(l, scratch[0], scratch[kGroupCells], scratch[2 * kGroupCells], pa,
                             pb, T.cfl, T.cell_m, a.max_dt);
        T.ctl->ledger[it.rec ^ 1u] = l;
      }
      __syncwarp();
    }
    uint32_t ia = 0u, ib = 0u;
    march<FIXED, MANNING, 4, true, PLAIN, ZG>(T, it, w4, ring, 4 * warp, s_ab, &s_need, ia, ib);
    __syncthreads();
    if (warp == 0) {
      const uint32_t ga = s_ab[lane < 16 ? 0 : 2], gb = s_ab[lane < 16 ? 1 : 3];
      const uint32_t need = s_need;
      group_records(T.groups_x, T.groups_y, T.rec[it.rec ^ 1u], it.X0, Y0 / 16, ga, gb, ring,
                    it.dt > 0.0f && it.apply_source != 0u, (need & 1u) != 0u, (need & 2u) != 0u,
                    ia, ib);
      if (lane == 0) finish_item(T, it.rec, ia, ib, true);
    }
    __syncthreads();
  }
}

// The persistent tick: every work item of every tile, one tick. PLAIN (no tile holds a flag of
// kFlagsNotPlain) compiles the open edges, the compensated source and Manning out of the march,
// which then fits 80 registers: six CTAs an SM instead of five. ZG takes zero arguments apart
// from the divisions and square roots (zsqrt, zdiv), a choice of the batches' autotuner.
template <bool FIXED, bool MANNING, int H, bool PLAIN, bool ZG = false>
__global__ void __launch_bounds__(kCtaThreads, PLAIN ? 6 : 5) tick_kernel(TickArgs a) {
  dependent_grid_start();
  if (a.go != nullptr && *a.go == 0u) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const WarpMem<H> wm = warp_mem<H>(warp);
  const uint32_t slots = gridDim.x * kWarpsPerCta, own = blockIdx.x * kWarpsPerCta + warp;
  for (bool first = true;; first = false) {
    uint32_t item = 0u;
    if (lane == 0) item = take_item(a.work, first, own, slots, a.n_whole);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= a.n_whole) break;
    const uint32_t tile = item_tile_of(a.item_tile, item);
    const TileDesc& T = a.tiles[tile];
    const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
    const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
    const TileCtl* ctl = T.ctl;
    Item it;
    it.cur = ctl->cur;
    it.rec = ctl->rec;
    const float pa = __uint_as_float(ctl->max_a[it.rec]);
    const float pb = __uint_as_float(ctl->max_b[it.rec]);
    it.dt = choose_dt<FIXED>(pa, pb, T.cfl, T.cell_m, a.max_dt, ctl->ledger[it.rec].remaining_s);
    // A tick queue's slot: a tile with no time left has landed and waits for the others.
    if (a.go != nullptr && !(ctl->ledger[it.rec].remaining_s > 0.0f)) continue;
    const bool src = (T.flags & kFlagSource) != 0u;
    const bool on = src && (T.source_every <= 1u || ctl->src_phase + 1u == T.source_every);
    it.apply_source = on ? 1u : 0u;
    it.scale = T.source_every > 1u ? float(T.source_every) : 1.0f;
    it.X0 = int(bx) * kStrip;
    it.Y0 = int(by) * H;
    if (local == 0u) {
      // The ledger's fold of the last update's records (dt_main, slang:417-478), in the warp's
      // ring before the march needs it.
      fold_warp(T.rec[it.rec], T.groups_x * T.groups_y, wm.ring);
      if (lane == 0) {
        LedgerBits l = ctl->ledger[it.rec];
        ledger_update<FIXED>(l, wm.ring[0], wm.ring[kGroupCells], wm.ring[2 * kGroupCells], pa,
                             pb, T.cfl, T.cell_m, a.max_dt);
        T.ctl->ledger[it.rec ^ 1u] = l;
      }
      __syncwarp();
    }
    uint32_t ia = 0u, ib = 0u;
    march<FIXED, MANNING, H, false, PLAIN, ZG>(T, it, wm, wm.ring, 0, nullptr, nullptr, ia, ib);
    __syncwarp();
    // `rec` read again rather than held through the march (a register fewer): only the tile's
    // last item flips it, after this item's count.
    if (lane == 0) finish_item(T, T.ctl->rec, ia, ib, true);
    __syncwarp();
  }
  if constexpr (H == 16) {
    if (a.n_whole < a.n_items) tail_items<FIXED, MANNING, PLAIN, ZG>(a, wm);  // the same in every CTA
  }
  if (lane == 0 && slots < a.n_items) {  // the counters were read: the last warp out resets them
    __threadfence();
    if (atomicAdd(&a.work->exited, 1u) + 1u == slots) {
      a.work->next = 0u;
      a.work->tail = 0u;
      a.work->exited = 0u;
      __threadfence();
    }
  }
}

// The split tick: a CTA steps one 32 x 16 item at a time, its four warps four rows each (more
// warps in flight where a tile has few items), the item's records from the CTA's shared ring.
// The items are the 32 x 16 shape's.
template <bool FIXED, bool MANNING>
__global__ void __launch_bounds__(kCtaThreads, 5) tick_split_kernel(TickArgs a) {
  dependent_grid_start();
  if (a.go != nullptr && *a.go == 0u) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const WarpMem<4> wm = warp_mem<4>(warp);
  float* ring = warp_mem<4>(0).ring;     // the item's 16 rows of volumes
  float* scratch = warp_mem<4>(1).ring;  // the ledger fold's slots
  __shared__ uint32_t s_item, s_need;
  __shared__ uint32_t s_ab[4];
  for (bool first = true;; first = false) {
    if (threadIdx.x == 0) {
      s_item = take_item(a.work, first, blockIdx.x, gridDim.x, a.n_items);
      s_need = 0u;
    }
    if (threadIdx.x < 4) s_ab[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= a.n_items) break;
    const uint32_t tile = item_tile_of(a.item_tile, item);
    const TileDesc& T = a.tiles[tile];
    const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
    const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
    const TileCtl* ctl = T.ctl;
    Item it;
    it.cur = ctl->cur;
    it.rec = ctl->rec;
    const float pa = __uint_as_float(ctl->max_a[it.rec]);
    const float pb = __uint_as_float(ctl->max_b[it.rec]);
    it.dt = choose_dt<FIXED>(pa, pb, T.cfl, T.cell_m, a.max_dt, ctl->ledger[it.rec].remaining_s);
    if (a.go != nullptr && !(ctl->ledger[it.rec].remaining_s > 0.0f)) {  // a landed tile
      __syncthreads();
      continue;
    }
    const bool src = (T.flags & kFlagSource) != 0u;
    const bool on = src && (T.source_every <= 1u || ctl->src_phase + 1u == T.source_every);
    it.apply_source = on ? 1u : 0u;
    it.scale = T.source_every > 1u ? float(T.source_every) : 1.0f;
    it.X0 = int(bx) * kStrip;
    const int Y0 = int(by) * 16;
    it.Y0 = Y0 + 4 * warp;
    if (local == 0u && warp == 1) {
      fold_warp(T.rec[it.rec], T.groups_x * T.groups_y, scratch);
      if (lane == 0) {
        LedgerBits l = ctl->ledger[it.rec];
        ledger_update<FIXED>(l, scratch[0], scratch[kGroupCells], scratch[2 * kGroupCells], pa,
                             pb, T.cfl, T.cell_m, a.max_dt);
        T.ctl->ledger[it.rec ^ 1u] = l;
      }
      __syncwarp();
    }
    uint32_t ia = 0u, ib = 0u;
    march<FIXED, MANNING, 4, true>(T, it, wm, ring, 4 * warp, s_ab, &s_need, ia, ib);
    __syncthreads();
    if (warp == 0) {
      const uint32_t ga = s_ab[lane < 16 ? 0 : 2], gb = s_ab[lane < 16 ? 1 : 3];
      const uint32_t need = s_need;
      group_records(T.groups_x, T.groups_y, T.rec[it.rec ^ 1u], it.X0, Y0 / 16, ga, gb, ring,
                    it.dt > 0.0f && it.apply_source != 0u, (need & 1u) != 0u, (need & 2u) != 0u,
                    ia, ib);
      if (lane == 0) finish_item(T, it.rec, ia, ib, true);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && gridDim.x < a.n_items) {  // the counter was read
    __threadfence();
    if (atomicAdd(&a.work->exited, 1u) + 1u == gridDim.x) {
      a.work->next = 0u;
      a.work->exited = 0u;
      __threadfence();
    }
  }
}

// ---- the block tick -------------------------------------------------------------------------
//
// A CTA of THREADS threads steps one 32 x 16 block (the 32 x 16 items, two 16 x 16 groups) at a
// time in three phases through shared memory:
//   1. the block's cells and a one-cell halo as {h, z, u, v} (ghosts at the tile's edges);
//   2. every face of the block, one a thread (a face on the block's boundary is computed by both
//      blocks that share it);
//   3. every cell's update from its four faces, then the block's two records.
// No thread's work waits on a row before it: a tile's faces are as many independent threads as the
// device holds, where the march's warps walk their rows one after another.
// THREADS 256 (two cells and about four faces a thread) packs four CTAs an SM; 512 (one cell and
// about two faces a thread) halves each thread's share of a block, which is what a launch of no
// more blocks than SMs (a small tile) waits for: its tick is one CTA's chain of phases.
constexpr int kBlkW = 32, kBlkH = 16, kBlkThreads = 256, kBlkWideThreads = 512;

struct BlockSmem {
  float4 cell[kBlkH + 2][kBlkW + 2];  // local (r, c) at [r + 1][c + 1]
  float4 fx[kBlkH][kBlkW + 1];        // x face f of row r: between columns f - 1 and f
  float4 fy[kBlkH + 1][kBlkW];        // y face f of column c: between rows f - 1 and f
  float ring[3 * 16 * kStrip];        // the cells' source, open-edge and roundoff volumes
  float fold[3 * kGroupCells];        // dt_main's fold (the tile's first block)
  uint32_t item, need, ab[4];
  // The staged variant: whether copies are in flight for `item`, and the next item (taken while
  // this one steps) with whether its copies were issued.
  uint32_t staged, next, next_staged;
  uint64_t bar;                       // the staged variant's copies land on this mbarrier
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- the staged block: a block's cells and halo by tensor copies ------------------------------
//
// Where a tile's width is a multiple of 4 (its rows start on 16-byte boundaries), the block tick's
// staged variant takes a 32 x 16 block's cells and one-cell halo as two tensor copies (TMA) into
// shared memory, in place of each thread's global loads: the state's {h, hu, hv} as one box of
// 40 x 18 x 3 floats and the bed as one of 40 x 18, both from column X0 - 4 and row Y0 - 1. X0 is
// a multiple of 32, so every copy starts on a 16-byte boundary; the three columns west of the halo
// are copied and not read. Cells past the tile's edges arrive as zeros and are not read either: a
// ghost is its edge cell's reflection, which is in the box. The box has a shared-memory region of
// its own after the CTA's BlockSmem. One thread issues both copies on the CTA's mbarrier; every
// thread waits on it, for at most kStageWaitNs.
//
// A CTA that steps block after block takes its next block while it steps this one: thread 0 takes
// the next item from the work counter at the item's start, and issues its copies as soon as this
// block's last read of the stage is behind a CTA barrier (phase 1's), so that they land while the
// CTA computes this block's faces and updates.
constexpr int kStageW = kBlkW + 8, kStageH = kBlkH + 2, kStageX = 4;
constexpr int kStagePlane = kStageW * kStageH;                       // floats a plane
constexpr uint32_t kStateBoxBytes = 3u * kStagePlane * 4u;           // 8640
constexpr uint32_t kBedBoxBytes = uint32_t(kStagePlane) * 4u;        // 2880
constexpr int kStageBed = int((kStateBoxBytes + 127u) / 128u * 32u);  // the bed box's float offset
constexpr size_t kStageBytes = size_t(kStageBed) * 4u + kBedBoxBytes;  // 11584
// The staged kernel's dynamic shared memory: BlockSmem, up to 127 bytes to the next 128-byte
// boundary, the stage.
constexpr size_t kStagedSmemBytes = sizeof(BlockSmem) + 128u + kStageBytes;
constexpr uint64_t kStageWaitNs = 1000000000ull;  // a second

// The stage's first float: the first 128-byte boundary past the CTA's BlockSmem.
__device__ __forceinline__ float* stage_of(BlockSmem& m) {
  char* p = reinterpret_cast<char*>(&m) + sizeof(BlockSmem);
  return reinterpret_cast<float*>(p + ((128u - (smem_u32(p) & 127u)) & 127u));
}

__device__ __forceinline__ void stage_init(BlockSmem& m) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&m.bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Thread 0: block (X0, Y0)'s boxes from state copy `cur` and the bed, on the mbarrier. A CTA
// barrier before it ended every thread's reads of the stage; the proxy fence orders the CTA's
// generic accesses before the copies' writes.
__device__ __forceinline__ void stage_issue(BlockSmem& m, const TileDesc& T, uint32_t cur, int X0,
                                            int Y0) {
  const char* maps = static_cast<const char*>(T.tmap);
  const uint32_t bar = smem_u32(&m.bar), dst = smem_u32(stage_of(m));
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
               "r"(kStateBoxBytes + kBedBoxBytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(maps + size_t(cur) * 128u), "r"(X0 - kStageX), "r"(Y0 - 1), "r"(0), "r"(bar)
      : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst + uint32_t(kStageBed) * 4u),
      "l"(maps + 256), "r"(X0 - kStageX), "r"(Y0 - 1), "r"(bar)
      : "memory");
}

// Waits for phase `phase` of the mbarrier; false where it gave up after kStageWaitNs.
__device__ __forceinline__ bool stage_wait(BlockSmem& m, uint32_t phase) {
  const uint32_t bar = smem_u32(&m.bar);
  uint64_t t0 = 0;
  for (uint32_t k = 0;; ++k) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done != 0u) return true;
    if (k == 0u) t0 = global_ns();
    else if ((k & 15u) == 0u && global_ns() - t0 > kStageWaitNs) return false;
  }
}

// Thread 0: issues item `item`'s copies where it has any (an item of the launch, of a tile with
// tensor maps, not a landed tile's in a queue's launch); returns whether it did. The item's tile
// cannot flip its copy before the item is stepped, so `cur` read now is the item's.
__device__ __forceinline__ uint32_t stage_item(const TickArgs& a, BlockSmem& m, uint32_t item) {
  if (item >= a.n_items) return 0u;
  const TileDesc& T = a.tiles[item_tile_of(a.item_tile, item)];
  if (T.tmap == nullptr) return 0u;
  const TileCtl* ctl = T.ctl;
  if (a.go != nullptr && !(ctl->ledger[ctl->rec].remaining_s > 0.0f)) return 0u;
  const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
  const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
  stage_issue(m, T, ctl->cur, int(bx) * kBlkW, int(by) * kBlkH);
  return 1u;
}

// The halo cell thread t reads (threads 0 .. 2 kBlkW + 2 kBlkH - 1; none for the others or past a
// partial block's edge): its shared-memory slot, the cell it reads, and at the tile's edge the
// ghost's sign for its normal velocity (slang:597-624).
struct HaloCell {
  float4* slot = nullptr;
  int i = 0;
  int li = 0;  // the cell's float in a staged plane
  bool ghost = false, flip_v = false;
  float sign = 1.0f;
};

__device__ __forceinline__ HaloCell halo_cell(BlockSmem& m, int t, int X0, int Y0, int rows,
                                              int cols, int nx, int ny, uint32_t flags) {
  HaloCell h;
  if (t >= 2 * kBlkW + 2 * kBlkH) return h;
  int gy, gx;
  bool need;
  if (t < kBlkW) {  // south row
    const int c = t;
    need = c < cols;
    h.ghost = Y0 == 0;
    gy = h.ghost ? Y0 : Y0 - 1;
    gx = X0 + c;
    h.sign = (flags & kFlagSouthOpen) ? 1.0f : -1.0f;
    h.flip_v = true;
    h.slot = &m.cell[0][c + 1];
  } else if (t < 2 * kBlkW) {  // north row
    const int c = t - kBlkW;
    need = c < cols;
    h.ghost = Y0 + rows >= ny;
    gy = h.ghost ? Y0 + rows - 1 : Y0 + rows;
    gx = X0 + c;
    h.sign = (flags & kFlagNorthOpen) ? 1.0f : -1.0f;
    h.flip_v = true;
    h.slot = &m.cell[rows + 1][c + 1];
  } else if (t < 2 * kBlkW + kBlkH) {  // west column
    const int r = t - 2 * kBlkW;
    need = r < rows;
    h.ghost = X0 == 0;
    gy = Y0 + r;
    gx = h.ghost ? X0 : X0 - 1;
    h.sign = (flags & kFlagWestOpen) ? 1.0f : -1.0f;
    h.slot = &m.cell[r + 1][0];
  } else {  // east column
    const int r = t - 2 * kBlkW - kBlkH;
    need = r < rows;
    h.ghost = X0 + cols >= nx;
    gy = Y0 + r;
    gx = h.ghost ? X0 + cols - 1 : X0 + cols;
    h.sign = (flags & kFlagEastOpen) ? 1.0f : -1.0f;
    h.slot = &m.cell[r + 1][cols + 1];
  }
  h.i = gy * nx + gx;
  h.li = (gy - Y0 + 1) * kStageW + gx - X0 + kStageX;
  if (!need) h.slot = nullptr;
  return h;
}

// The tile's dt_main fold of the last update's records (slang:417-478) by the whole CTA, a thread
// a virtual lane, into the ledger's next slot (`rec` is the slot the records are in).
template <bool FIXED>
__device__ __forceinline__ void fold_ledger(const TileDesc& T, BlockSmem& m, uint32_t rec,
                                            float pa, float pb, float max_dt) {
  const TileCtl* ctl = T.ctl;
  fold_block(T.rec[rec], T.groups_x * T.groups_y, m.fold);
  if (threadIdx.x == 0) {
    LedgerBits l = ctl->ledger[rec];
    ledger_update<FIXED>(l, m.fold[0], m.fold[kGroupCells], m.fold[2 * kGroupCells], pa, pb,
                         T.cfl, T.cell_m, max_dt);
    T.ctl->ledger[rec ^ 1u] = l;
  }
}

// One 32 x 16 block of one tick: the three phases and the block's two records. `cur` is the copy
// that holds the state, `rec` the record slot of the last update; pa and pb are the last update's
// largest speeds; dt, whether the source applies and its scale are the tick's. Warp 0's lane 0
// leaves the block's largest speeds in ia, ib for the caller, which counts the item. The tile's
// first block folds its ledger unless a CTA of its own does (a.fold_apart). STAGE: `staged` says
// the block's cells and halo are being copied into the stage (phase `stage_phase` of the CTA's
// mbarrier, flipped here); `after_reads` runs once every thread's reads of the stage are behind a
// CTA barrier (the caller issues the next block's copies there). Returns false (every thread
// alike) where the wait on the copies gave up: the item not stepped, the launch's fault word
// marked.
template <bool FIXED, bool MANNING, int THREADS, bool STAGE = false, class AfterReads>
__device__ __forceinline__ bool block_item(const TickArgs& a, BlockSmem& m, const TileDesc& T,
                                           uint32_t local, uint32_t cur, uint32_t rec, float pa,
                                           float pb, float dt, bool apply, float scale,
                                           uint32_t& ia, uint32_t& ib, bool staged,
                                           uint32_t& stage_phase, AfterReads after_reads) {
  constexpr int kBlkWarps = THREADS / 32;
  // The native arithmetic's zero arguments taken apart from its divisions and square roots (the
  // same bits): small tiles are mostly dry land, fronts and still water, where the intrinsics'
  // slow path on a zero argument is common (256 x 256: 8.0 -> 6.4 us a tick a launch a tick).
  constexpr bool kZeroApart = !FIXED;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
  const int X0 = int(bx) * kBlkW, Y0 = int(by) * kBlkH;
  staged = STAGE && staged;
  if (local == 0u && a.fold_apart == 0u) fold_ledger<FIXED>(T, m, rec, pa, pb, a.max_dt);
  const int nx = int(T.nx), ny = int(T.ny);
  const size_t n = size_t(T.nx) * T.ny;
  const int rows = min(kBlkH, ny - Y0), cols = min(kBlkW, nx - X0);
  const float* in = T.state[cur];
  float* out = T.state[cur ^ 1u];
  const float* bed = T.bed;
  const float g = T.gravity, dry = T.dry, hg = __fmul_rn(0.5f, g);
  const uint32_t flags = T.flags;
  // The cells this thread updates: rows warp + kBlkWarps k of column t & 31.
  constexpr int K = (kBlkH + kBlkWarps - 1) / kBlkWarps;
  const int cc = lane;
  // A thread of one cell (the 512-thread CTA) loads its bed and its halo cell with its state, so
  // that the block waits on one round of loads; the 256-thread CTA loads them in phase 1 (its two
  // cells' worth held from the start would spill).
  constexpr bool kEarly = K == 1;
  float rh[K], rhu[K], rhv[K], rz[K], rsrc[K];
  bool live[K];
  int gi[K], si[K];
  const float* st = staged ? stage_of(m) : nullptr;
  bool failed = false;
#pragma unroll
  for (int k = 0; k < K; ++k) rsrc[k] = 0.0f;
  if (staged) {
    // The source's loads in flight while the copies land, then the wait.
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int r = warp + kBlkWarps * k;
      if (K == 1 && apply && r < rows && cc < cols) rsrc[k] = T.source[(Y0 + r) * nx + X0 + cc];
    }
    failed = !stage_wait(m, stage_phase);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int r = warp + kBlkWarps * k;
    live[k] = r < rows && cc < cols;
    gi[k] = (Y0 + r) * nx + X0 + cc;
    si[k] = (r + 1) * kStageW + kStageX + cc;
    rh[k] = rhu[k] = rhv[k] = rz[k] = 0.0f;
    if (live[k]) {
      if (staged) {
        rh[k] = st[si[k]];
        rhu[k] = st[kStagePlane + si[k]];
        rhv[k] = st[2 * kStagePlane + si[k]];
        if (kEarly) rz[k] = st[kStageBed + si[k]];
      } else {
        rh[k] = in[gi[k]];
        rhu[k] = in[n + gi[k]];
        rhv[k] = in[2 * n + gi[k]];
        if (kEarly) rz[k] = bed[gi[k]];
        // A thread of one cell loads its source with its state, not after the barriers (two
        // cells' worth would cost the 256-thread CTA spills).
        if (K == 1 && apply) rsrc[k] = T.source[gi[k]];
      }
    }
  }
  HaloCell hc;
  float qh = 0.0f, qhu = 0.0f, qhv = 0.0f, qz = 0.0f;
  if (kEarly) {
    hc = halo_cell(m, t, X0, Y0, rows, cols, nx, ny, flags);
    if (hc.slot != nullptr) {
      if (staged) {
        qh = st[hc.li];
        qhu = st[kStagePlane + hc.li];
        qhv = st[2 * kStagePlane + hc.li];
        qz = st[kStageBed + hc.li];
      } else {
        qh = in[hc.i];
        qhu = in[n + hc.i];
        qhv = in[2 * n + hc.i];
        qz = bed[hc.i];
      }
    }
  }
  // A staged wait that gave up (the whole CTA agrees): the launch's fault word, a last bounded
  // wait for the copies still in flight into this CTA's shared memory, and the item not stepped.
  auto give_up = [&]() {
    if (t == 0) {
      if (a.fault != nullptr) atomicOr(a.fault, 1u);
      stage_wait(m, stage_phase);
    }
    return false;
  };
  uint32_t ga = 0u, gb = 0u;
  bool opn_seen = false, rnd_seen = false;
  if (!(dt > 0.0f)) {
    if (staged && __syncthreads_or(failed)) return give_up();
    after_reads();
    // A step of no length: the state as it is, to the bit (slang:576-585).
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (live[k]) {
        const int i = gi[k];
        out[i] = rh[k];
        out[n + i] = rhu[k];
        out[2 * n + i] = rhv[k];
        out[3 * n + i] = in[3 * n + i];
        float ax, ay;
        cell_speeds<FIXED, kZeroApart>(g, dry, rh[k], rhu[k], rhv[k], ax, ay);
        ga = max(ga, __float_as_uint(ax));
        gb = max(gb, __float_as_uint(ay));
      }
    }
  } else {
    // 1. the cells and the halo ({h, z, u, v}; a ghost's normal velocity signed by its edge)
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (live[k])
        m.cell[warp + kBlkWarps * k + 1][cc + 1] = velocities<FIXED, kZeroApart>(
            rh[k], rhu[k], rhv[k],
            kEarly ? rz[k] : (staged ? st[kStageBed + si[k]] : bed[gi[k]]), dry);
    if (!kEarly) {
      hc = halo_cell(m, t, X0, Y0, rows, cols, nx, ny, flags);
      if (hc.slot != nullptr) {
        if (staged) {
          qh = st[hc.li];
          qhu = st[kStagePlane + hc.li];
          qhv = st[2 * kStagePlane + hc.li];
          qz = st[kStageBed + hc.li];
        } else {
          qh = in[hc.i];
          qhu = in[n + hc.i];
          qhv = in[2 * n + hc.i];
          qz = bed[hc.i];
        }
      }
    }
    if (hc.slot != nullptr) {
      float4 v = velocities<FIXED, kZeroApart>(qh, qhu, qhv, qz, dry);
      if (hc.ghost) {
        if (hc.flip_v) v.w = __fmul_rn(hc.sign, v.w);
        else v.z = __fmul_rn(hc.sign, v.z);
      }
      *hc.slot = v;
    }
    // The stage's last reads end here.
    if (STAGE) {
      if (__syncthreads_or(failed)) return give_up();
      after_reads();
    } else {
      __syncthreads();
    }
    // 2. the faces
    const int nfx = rows * (cols + 1), nfy = (rows + 1) * cols;
    const bool full = cols == kBlkW;
    for (int q = t; q < nfx + nfy; q += THREADS) {
      if (q < nfx) {
        const int r = full ? q / (kBlkW + 1) : q / (cols + 1);
        const int f = q - r * (cols + 1);
        m.fx[r][f] = face_x<FIXED, kZeroApart>(g, hg, m.cell[r + 1][f], m.cell[r + 1][f + 1]);
      } else {
        const int q2 = q - nfx;
        const int f = full ? q2 / kBlkW : q2 / cols;
        const int c = q2 - f * cols;
        m.fy[f][c] = face_y<FIXED, kZeroApart>(g, hg, m.cell[f][c + 1], m.cell[f + 1][c + 1]);
      }
    }
    __syncthreads();
    // 3. the updates
    const float cell_m = T.cell_m;
    const float area = __fmul_rn(cell_m, cell_m);
    const float lam = Ops<FIXED>::div(dt, cell_m);
    const float edge_volume = __fmul_rn(dt, cell_m);
    const bool comp = (flags & kFlagCompensate) != 0u;
    const bool manning = MANNING && (flags & kFlagManning) != 0u;
    const UpdateCtx uc{g, dry, lam, area, edge_volume, dt, scale, flags, nx, ny,
                       apply, comp, manning, (flags & 15u) != 0u};
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int r = warp + kBlkWarps * k;
      if (r >= kBlkH) break;  // a warp past the block's rows (more than 512 threads)
      float csrc = 0.0f, copn = 0.0f, crnd = 0.0f;
      if (live[k]) {
        const int i = gi[k];
        float h, mu, mv, residual;
        update_cell<FIXED>(uc, m.cell[r + 1][cc + 1], rhu[k], rhv[k],
                           K == 1 ? rsrc[k] : (apply ? T.source[i] : 0.0f),
                           comp ? in[3 * n + i] : 0.0f,
                           manning ? T.manning[i] : 0.0f, m.fx[r][cc], m.fx[r][cc + 1],
                           m.fy[r][cc], m.fy[r + 1][cc], X0 + cc, Y0 + r, h, mu, mv, residual,
                           csrc, copn, crnd);
        out[i] = h;
        out[n + i] = mu;
        out[2 * n + i] = mv;
        if (comp) out[3 * n + i] = residual;
        float ax, ay;
        cell_speeds<FIXED, kZeroApart>(g, dry, h, mu, mv, ax, ay);
        ga = max(ga, __float_as_uint(ax));
        gb = max(gb, __float_as_uint(ay));
      }
      const int slot = r * kStrip + cc;
      m.ring[slot] = csrc;
      m.ring[16 * kStrip + slot] = copn;
      m.ring[32 * kStrip + slot] = crnd;
      opn_seen |= copn != 0.0f;
      rnd_seen |= crnd != 0.0f;
    }
  }
  // The block's two groups: their largest speeds and the quantities some cell holds.
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    ga = max(ga, __shfl_xor_sync(0xffffffffu, ga, o));
    gb = max(gb, __shfl_xor_sync(0xffffffffu, gb, o));
  }
  const bool any_opn = __any_sync(0xffffffffu, opn_seen);
  const bool any_rnd = __any_sync(0xffffffffu, rnd_seen);
  if ((lane & 15) == 0) {
    atomicMax(&m.ab[(lane >> 4) * 2], ga);
    atomicMax(&m.ab[(lane >> 4) * 2 + 1], gb);
  }
  if (lane == 0 && (any_opn || any_rnd))
    atomicOr(&m.need, (any_opn ? 1u : 0u) | (any_rnd ? 2u : 0u));
  __syncthreads();
  if (warp == 0) {
    const uint32_t need = m.need;
    group_records(T.groups_x, T.groups_y, T.rec[rec ^ 1u], X0, Y0 / 16, m.ab[lane < 16 ? 0 : 2],
                  m.ab[lane < 16 ? 1 : 3], m.ring, dt > 0.0f && apply, (need & 1u) != 0u,
                  (need & 2u) != 0u, ia, ib);
  }
  if (staged) stage_phase ^= 1u;
  return true;
}

// STAGE: the staged variant (a tile with tensor maps takes its blocks by tensor copies; the
// others load cell by cell).
template <bool FIXED, bool MANNING, int THREADS, bool STAGE = false>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) tick_block_kernel(TickArgs a) {
  static_assert(THREADS >= int(kGroupCells) && THREADS % 32 == 0,
                "fold_block takes a thread a virtual lane");
  static_assert(THREADS >= 2 * kBlkW + 2 * kBlkH, "a thread a halo cell");
  // The first item's tile descriptor into L1 while the grid before finishes: no tick or queue
  // slot writes a descriptor (only the host's uploads do, and a copy ends a dependent launch's
  // overlap), so it is the same before the wait as after it.
  if (threadIdx.x == 0 && blockIdx.x < a.n_items) {
    const TileDesc* d = a.tiles + item_tile_of(a.item_tile, blockIdx.x);
    asm volatile("prefetch.global.L1 [%0];" ::"l"(d));
    // The staged variant: the first item's three tensor maps into the copy engine's cache (they,
    // too, only change with the host's uploads), so its copies need no fetch of their own.
    if (STAGE) {
      const char* maps = static_cast<const char*>(d->tmap);
      if (maps != nullptr)
        for (int k = 0; k < 3; ++k)
          asm volatile("prefetch.tensormap [%0];" ::"l"(maps + 128 * k) : "memory");
    }
  }
  dependent_grid_start();
  if (a.go != nullptr && *a.go == 0u) return;
  extern __shared__ float4 smem_raw[];
  BlockSmem& m = *reinterpret_cast<BlockSmem*>(smem_raw);
  const int t = threadIdx.x;
  if (a.fold_apart != 0u && blockIdx.x + 1u == gridDim.x) {
    // The tile's dt_main fold on a CTA of its own, beside the items: a single tile's launch of
    // fewer items than SMs, whose item 0 would otherwise fold before it steps. It counts as one
    // more item, so the flip waits for its read of slot `rec`.
    const TileDesc& T = a.tiles[0];
    const TileCtl* ctl = T.ctl;
    const uint32_t rec = ctl->rec;
    if (a.go != nullptr && !(ctl->ledger[rec].remaining_s > 0.0f)) return;  // a landed tile
    const float pa = __uint_as_float(ctl->max_a[rec]), pb = __uint_as_float(ctl->max_b[rec]);
    fold_ledger<FIXED>(T, m, rec, pa, pb, a.max_dt);
    if (t == 0) finish_item(T, rec, 0u, 0u, true, 1u);
    return;
  }
  uint32_t stage_phase = 0u;
  if (STAGE && t == 0) stage_init(m);  // ordered before any wait by the loop's first barrier
  for (bool first = true;; first = false) {
    if (t == 0) {
      if (!STAGE || first) {
        m.item = take_item(a.work, first, blockIdx.x, gridDim.x, a.n_items);
        if (STAGE) m.staged = stage_item(a, m, m.item);
      } else {
        m.item = m.next;  // taken, and its copies issued, while the last item stepped
        m.staged = m.next_staged;
      }
      m.need = 0u;
    }
    if (t < 4) m.ab[t] = 0u;
    __syncthreads();
    const uint32_t item = m.item;
    if (item >= a.n_items) break;
    // STAGE: the next item is taken now (the counter's round trip runs behind this item's first
    // phase), and its copies are issued once this block's reads of the stage are done.
    uint32_t next = 0u;
    if (STAGE && t == 0) next = take_item(a.work, false, blockIdx.x, gridDim.x, a.n_items);
    auto after_reads = [&]() {
      if (STAGE && t == 0) {
        m.next = next;
        m.next_staged = stage_item(a, m, next);
      }
    };
    const uint32_t tile = item_tile_of(a.item_tile, item);
    const TileDesc& T = a.tiles[tile];
    const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
    const TileCtl* ctl = T.ctl;
    const uint32_t cur = ctl->cur, rec = ctl->rec;
    const float pa = __uint_as_float(ctl->max_a[rec]), pb = __uint_as_float(ctl->max_b[rec]);
    const float dt =
        choose_dt<FIXED>(pa, pb, T.cfl, T.cell_m, a.max_dt, ctl->ledger[rec].remaining_s);
    if (a.go != nullptr && !(ctl->ledger[rec].remaining_s > 0.0f)) {  // a landed tile
      after_reads();  // no copies were issued for it: the stage is free
      __syncthreads();
      continue;
    }
    const bool src_flag = (T.flags & kFlagSource) != 0u;
    const bool apply = src_flag && (T.source_every <= 1u || ctl->src_phase + 1u == T.source_every);
    const float scale = T.source_every > 1u ? float(T.source_every) : 1.0f;
    uint32_t ia = 0u, ib = 0u;
    if (!block_item<FIXED, MANNING, THREADS, STAGE>(a, m, T, local, cur, rec, pa, pb, dt, apply,
                                                    scale, ia, ib, STAGE && m.staged != 0u,
                                                    stage_phase, after_reads))
      break;  // a staged wait gave up: the fault word is marked
    if (t == 0) finish_item(T, rec, ia, ib, true, a.fold_apart);
    __syncthreads();
  }
  if (t == 0 && gridDim.x < a.n_items) {  // the counter was read
    __threadfence();
    if (atomicAdd(&a.work->exited, 1u) + 1u == gridDim.x) {
      a.work->next = 0u;
      a.work->exited = 0u;
      __threadfence();
    }
  }
}

// ---- the resident tick: many ticks of one small tile in one launch ----------------------------
//
// A tile of no more blocks than the device has SMs (the 256 x 256 tile's 128) steps `ticks` ticks
// in one cooperative launch: a 512-thread CTA a 32 x 16 block for the whole launch (a thread a
// cell), one CTA more for the ledger's fold (fold_ledger), and a grid barrier between ticks in
// place of the launch boundary. A tick is the block tick's three phases with the same per-cell
// functions (velocities, face_x/face_y, update_cell, the records' trees), so the arithmetic,
// records and ledger are the per-tick launch's. The block's own cells stay in registers (h, hu,
// hv, the bed, the source, plane 3) and in the shared cell array ({h, z, u, v}) from tick to tick;
// only the one-cell halo is read back, from the neighbours' output copy, after the barrier. The
// interior faces (both cells the block's own, about 90 % of them) need nothing from the
// neighbours, so a CTA computes the next tick's while it waits at the barrier.
//
// What the launches' flips would do tick by tick is kept in registers (the copy and the record
// slot follow the ticks' parity, the source's clock its count), and the tick's inputs in three
// rotating slots of the ResidentCtl: tick k reads slot k % 3 (the largest speeds of the last
// update, the ledger's time left), the blocks add their speeds to slot (k + 1) % 3 and the fold's
// CTA writes its time left there, and the fold's CTA clears slot (k + 2) % 3, read at tick k - 1;
// after the last tick CTA 0 writes the control block as the last launch's flip would have left it.
//
// The barrier: each CTA's thread 0 adds one to `arrived` with release semantics once its records
// are written (the CTA barrier before them ordered every thread's state first), and lane 0 of the
// first kPollers warps poll it with acquire semantics until it reaches the tick's count (the host
// zeroes the words before a launch). A wait is bounded: past kResidentWaitNs it marks the error
// word and the CTA leaves, and so does every CTA that then sees the mark, so the launch ends; the
// host reads the word.
constexpr uint64_t kResidentWaitNs = 1000000000ull;  // a second

// The barrier in two halves, so that a CTA works while it waits: `resident_arrive` (after a CTA
// barrier: every thread's writes of the tick are done) adds the CTA's arrival with release
// semantics; `resident_wait` polls with acquire semantics until `target` CTAs have arrived, then
// meets the CTA's threads. Returns false where the wait gave up.
__device__ __forceinline__ void resident_arrive(ResidentCtl* rc) {
  if (threadIdx.x == 0)
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&rc->arrived) : "memory");
}

// Lane 0 of the CTA's first kPollers warps poll, staggered, so that the count's last step is seen
// sooner than one poller's round trip; the first to see it tells the others through `s_seen`
// (which holds the last count seen, so it needs no reset between ticks; zeroed at the launch's
// start by resident_start).
constexpr int kPollers = 4;
__shared__ uint32_t s_seen;
__shared__ int s_fail;

__device__ __forceinline__ void resident_start() {
  if (threadIdx.x == 0) {
    s_seen = 0u;
    s_fail = 0;
  }
  __syncthreads();
}

__device__ __forceinline__ bool resident_wait(ResidentCtl* rc, uint32_t target) {
  if ((threadIdx.x & 31) == 0 && threadIdx.x < 32 * kPollers) {
    volatile uint32_t* seen = &s_seen;
    const uint64_t t0 = global_ns();
    for (uint32_t polls = 1; *seen < target; ++polls) {
      uint32_t c;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(&rc->arrived) : "memory");
      if (c >= target) {
        *seen = target;
        break;
      }
      if ((polls & 63u) == 0u) {
        const uint32_t e = static_cast<const volatile ResidentCtl*>(rc)->error;
        if (e != 0u || global_ns() - t0 > kResidentWaitNs) {
          atomicOr(&rc->error, 1u);
          s_fail = 1;
          *seen = target;  // the other pollers stop too
          break;
        }
      }
    }
  }
  __syncthreads();
  return s_fail == 0;
}

__device__ __forceinline__ bool resident_barrier(ResidentCtl* rc, uint32_t target) {
  __syncthreads();
  resident_arrive(rc);
  return resident_wait(rc, target);
}

// The faces of a 32 x 16 block whose cells are all the block's own (none on the halo): x faces
// 1 .. cols - 1 of each row and y faces 1 .. rows - 1 of each column. A CTA computes the next
// tick's while it waits at the barrier; the boundary faces need the halo, read after it.
template <bool FIXED, int THREADS, bool ZG>
__device__ __forceinline__ void interior_faces(BlockSmem& m, int rows, int cols, float g,
                                               float hg) {
  const int nfx = rows * (cols - 1), nfy = (rows - 1) * cols;
  for (int q = threadIdx.x; q < nfx + nfy; q += THREADS) {
    if (q < nfx) {
      const int r = q / (cols - 1), f = q - r * (cols - 1) + 1;
      m.fx[r][f] = face_x<FIXED, ZG>(g, hg, m.cell[r + 1][f], m.cell[r + 1][f + 1]);
    } else {
      const int q2 = q - nfx;
      const int f = q2 / cols + 1, c = q2 - (f - 1) * cols;
      m.fy[f][c] = face_y<FIXED, ZG>(g, hg, m.cell[f][c + 1], m.cell[f + 1][c + 1]);
    }
  }
}

// The faces on the block's boundary (x faces 0 and cols, y faces 0 and rows), once the halo is in.
template <bool FIXED, bool ZG>
__device__ __forceinline__ void boundary_faces(BlockSmem& m, int rows, int cols, float g,
                                               float hg) {
  const int q = threadIdx.x;
  if (q < 2 * rows) {
    const int r = q >> 1, f = (q & 1) ? cols : 0;
    m.fx[r][f] = face_x<FIXED, ZG>(g, hg, m.cell[r + 1][f], m.cell[r + 1][f + 1]);
  } else if (q < 2 * rows + 2 * cols) {
    const int q2 = q - 2 * rows;
    const int c = q2 >> 1, f = (q2 & 1) ? rows : 0;
    m.fy[f][c] = face_y<FIXED, ZG>(g, hg, m.cell[f][c + 1], m.cell[f + 1][c + 1]);
  }
}

// The resident tick's CTA: a thread a cell. (A face a thread, at 1024 threads, was slower: 5.04
// against 4.48 us a tick on the 256 x 256 tile.)
constexpr int kResThreads = 512;

template <bool FIXED, bool MANNING>
__global__ void __launch_bounds__(kResThreads, 1024 / kResThreads)
    tick_resident_kernel(TickArgs a, uint32_t ticks, ResidentCtl* rc) {
  static_assert(kResThreads >= kBlkW * kBlkH, "a thread a cell");
  static_assert(kResThreads >= int(kGroupCells) && kResThreads >= 2 * kBlkW + 2 * kBlkH,
                "a thread a virtual lane of the fold, and a boundary face");
  extern __shared__ float4 smem_raw[];
  BlockSmem& m = *reinterpret_cast<BlockSmem*>(smem_raw);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const TileDesc& T = a.tiles[0];
  TileCtl* ctl = T.ctl;
  const uint32_t cur0 = ctl->cur, rec0 = ctl->rec, ticks0 = ctl->ticks;
  uint32_t cur = cur0, rec = rec0, phase = ctl->src_phase;
  const uint32_t flags = T.flags;
  const bool src_flag = (flags & kFlagSource) != 0u;
  const uint32_t every = T.source_every;
  const float scale = every > 1u ? float(every) : 1.0f;
  const bool folder = blockIdx.x == a.n_items;
  const uint32_t n = gridDim.x;
  // The block and this thread's cell (row `warp`, column `lane`), held across the ticks: its
  // state in registers, its {h, z, u, v} in the shared cell array.
  const uint32_t local = folder ? 0u : blockIdx.x;
  const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
  const int X0 = int(bx) * kBlkW, Y0 = int(by) * kBlkH;
  const int nx = int(T.nx), ny = int(T.ny);
  const size_t nn = size_t(T.nx) * T.ny;
  const int rows = min(kBlkH, ny - Y0), cols = min(kBlkW, nx - X0);
  const bool live = !folder && warp < rows && lane < cols;
  const int gi = (Y0 + warp) * nx + X0 + lane;
  const float g = T.gravity, dry = T.dry, hg = __fmul_rn(0.5f, g);
  const bool comp = (flags & kFlagCompensate) != 0u;
  const bool manning = MANNING && (flags & kFlagManning) != 0u;
  const float cell_m = T.cell_m;
  const float area = __fmul_rn(cell_m, cell_m);
  float h = 0.0f, hu = 0.0f, hv = 0.0f, z = 0.0f, src = 0.0f, resid = 0.0f, mn = 0.0f;
  if (live) {
    const float* in = T.state[cur0];
    h = in[gi];
    hu = in[nn + gi];
    hv = in[2 * nn + gi];
    resid = comp ? in[3 * nn + gi] : 0.0f;
    z = T.bed[gi];
    if (src_flag) src = T.source[gi];
    if (manning) mn = T.manning[gi];
    m.cell[warp + 1][lane + 1] = velocities<FIXED, true>(h, hu, hv, z, dry);
  }
  resident_start();
  if (!folder) interior_faces<FIXED, kResThreads, true>(m, rows, cols, g, hg);
  uint32_t slot = 0u;  // k % 3
  for (uint32_t k = 0; k < ticks; ++k) {
    // What the last tick left: the control block's at the first tick, the rotating slot after.
    uint32_t ua, ub;
    float remaining;
    if (k == 0u) {
      ua = ctl->max_a[rec0];
      ub = ctl->max_b[rec0];
      remaining = ctl->ledger[rec0].remaining_s;
    } else {
      uint4 w;
      asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                   : "=r"(w.x), "=r"(w.y), "=r"(w.z), "=r"(w.w)
                   : "l"(&rc->slot[slot]));
      ua = w.x;
      ub = w.y;
      remaining = __uint_as_float(w.z);
    }
    const float pa = __uint_as_float(ua), pb = __uint_as_float(ub);
    const uint32_t next = slot == 2u ? 0u : slot + 1u, spare = next == 2u ? 0u : next + 1u;
    if (folder) {
      fold_ledger<FIXED>(T, m, rec, pa, pb, a.max_dt);
      if (t == 0) {
        // The new ledger (thread 0 wrote it) gives the next tick its time left.
        rc->slot[next].remaining_s =
            static_cast<const volatile TileCtl*>(ctl)->ledger[rec ^ 1u].remaining_s;
        rc->slot[spare].max_a = 0u;
        rc->slot[spare].max_b = 0u;
      }
      __syncthreads();
      resident_arrive(rc);
    } else {
      // m.need and m.ab were last read before the last barrier; the barriers below order these
      // writes before their use.
      if (t == 0) m.need = 0u;
      if (t < 4) m.ab[t] = 0u;
      const float* in = T.state[cur];
      float* out = T.state[cur ^ 1u];
      // 1. the halo (the neighbours' last tick, or a ghost of this block's own edge)
      const HaloCell hc = halo_cell(m, t, X0, Y0, rows, cols, nx, ny, flags);
      if (hc.slot != nullptr) {
        float4 v =
            velocities<FIXED, true>(in[hc.i], in[nn + hc.i], in[2 * nn + hc.i], T.bed[hc.i], dry);
        if (hc.ghost) {
          if (hc.flip_v) v.w = __fmul_rn(hc.sign, v.w);
          else v.z = __fmul_rn(hc.sign, v.z);
        }
        *hc.slot = v;
      }
      const float dt = choose_dt<FIXED>(pa, pb, T.cfl, cell_m, a.max_dt, remaining);
      const bool apply = src_flag && (every <= 1u || phase + 1u == every);
      __syncthreads();
      // 2. the boundary faces (the interior ones were taken while waiting at the last barrier)
      if (dt > 0.0f) boundary_faces<FIXED, true>(m, rows, cols, g, hg);
      __syncthreads();
      // 3. the update, its speeds, and the next tick's velocities
      uint32_t ga = 0u, gb = 0u;
      bool opn_seen = false, rnd_seen = false;
      float csrc = 0.0f, copn = 0.0f, crnd = 0.0f;
      if (live) {
        // Plane 3 (the compensated source's remainder): carried in `resid` where compensating
        // (each tick writes it); otherwise a tick leaves the output copy's as it was and a step of
        // no length copies the input copy's.
        float h2 = h, mu = hu, mv = hv, residual = resid;
        if (dt > 0.0f) {
          const float lam = Ops<FIXED>::div(dt, cell_m);
          const float edge_volume = __fmul_rn(dt, cell_m);
          const UpdateCtx uc{g, dry, lam, area, edge_volume, dt, scale, flags, nx, ny,
                             apply, comp, manning, (flags & 15u) != 0u};
          update_cell<FIXED>(uc, m.cell[warp + 1][lane + 1], hu, hv, apply ? src : 0.0f,
                             comp ? resid : 0.0f, mn, m.fx[warp][lane], m.fx[warp][lane + 1],
                             m.fy[warp][lane], m.fy[warp + 1][lane], X0 + lane, Y0 + warp, h2,
                             mu, mv, residual, csrc, copn, crnd);
          if (comp) out[3 * nn + gi] = residual;
        } else {
          out[3 * nn + gi] = comp ? resid : in[3 * nn + gi];
        }
        out[gi] = h2;
        out[nn + gi] = mu;
        out[2 * nn + gi] = mv;
        // velocities() of the new state, and the records' speeds from the same quotients
        // (cell_speeds: |u| + c and |v| + c).
        const float4 c4 = velocities<FIXED, true>(h2, mu, mv, z, dry);
        const float gh = __fmul_rn(g, h2);
        const float cc = gh == 0.0f ? gh : Ops<FIXED>::sqrt(gh);
        ga = __float_as_uint(__fadd_rn(fabsf(c4.z), cc));
        gb = __float_as_uint(__fadd_rn(fabsf(c4.w), cc));
        m.cell[warp + 1][lane + 1] = c4;
        h = h2;
        hu = mu;
        hv = mv;
        if (comp) resid = residual;
      }
      if (warp < kBlkH) {
        const int rslot = warp * kStrip + lane;
        m.ring[rslot] = csrc;
        m.ring[16 * kStrip + rslot] = copn;
        m.ring[32 * kStrip + rslot] = crnd;
      }
      opn_seen = copn != 0.0f;
      rnd_seen = crnd != 0.0f;
      // 4. the block's two records (as block_item's)
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        ga = max(ga, __shfl_xor_sync(0xffffffffu, ga, o));
        gb = max(gb, __shfl_xor_sync(0xffffffffu, gb, o));
      }
      const bool any_opn = __any_sync(0xffffffffu, opn_seen);
      const bool any_rnd = __any_sync(0xffffffffu, rnd_seen);
      if ((lane & 15) == 0) {
        atomicMax(&m.ab[(lane >> 4) * 2], ga);
        atomicMax(&m.ab[(lane >> 4) * 2 + 1], gb);
      }
      if (lane == 0 && (any_opn || any_rnd))
        atomicOr(&m.need, (any_opn ? 1u : 0u) | (any_rnd ? 2u : 0u));
      __syncthreads();
      if (warp == 0) {
        uint32_t ia = 0u, ib = 0u;
        const uint32_t need = m.need;
        write_group_records(T.groups_x, T.groups_y, T.rec[rec ^ 1u], X0, Y0 / 16, m.ab[0],
                            m.ab[1], m.ab[2], m.ab[3], m.ring, dt > 0.0f && apply,
                            (need & 1u) != 0u, (need & 2u) != 0u, ia, ib);
        if (lane == 0) {
          atomicMax(&rc->slot[next].max_a, ia);
          atomicMax(&rc->slot[next].max_b, ib);
        }
      }
      // Thread 0 wrote the records and the speeds itself and saw every other thread's state
      // through the barrier above: its release covers them, and the other warps go on.
      resident_arrive(rc);
      // The next tick's interior faces while the other CTAs finish this one.
      if (k + 1u < ticks) interior_faces<FIXED, kResThreads, true>(m, rows, cols, g, hg);
    }
    if (!resident_wait(rc, n * (k + 1u))) return;
    if (src_flag && every > 1u) phase = phase + 1u == every ? 0u : phase + 1u;
    cur ^= 1u;
    rec ^= 1u;
    slot = next;
  }
  if (blockIdx.x == 0 && t == 0 && ticks > 0u) {
    // Every CTA is past the last barrier and none reads the control block again.
    volatile TileCtl* w = ctl;
    const volatile ResidentCtl* vr = rc;
    w->max_a[rec] = vr->slot[slot].max_a;
    w->max_b[rec] = vr->slot[slot].max_b;
    w->max_a[rec ^ 1u] = 0u;
    w->max_b[rec ^ 1u] = 0u;
    w->cur = cur;
    w->rec = rec;
    w->src_phase = phase;
    w->ticks = ticks0 + ticks;
  }
}

// A check of the barrier's bounded wait alone: `n` CTAs of which the last never arrives, so the
// others give up after the bound and mark the error word. The host zeroes `rc` and reads it.
__global__ void resident_barrier_probe_kernel(ResidentCtl* rc, uint32_t n) {
  if (blockIdx.x + 1u == gridDim.x) return;  // the CTA that does not arrive
  resident_start();
  resident_barrier(rc, n);
}

// The records of a state written from the host (prime_main, slang:373-386): a warp an item. The
// records and largest speeds go to slot rec ^ 1 and the tile's last item flips `rec`, as a tick
// does; the tile's first item carries the ledger over to that slot.
template <bool FIXED, int H>
__global__ void __launch_bounds__(kCtaThreads) prime_kernel(TickArgs a) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t item = blockIdx.x * kWarpsPerCta + warp;
  if (item >= a.n_items) return;
  const WarpMem<H> wm = warp_mem<H>(warp);
  const uint32_t tile = item_tile_of(a.item_tile, item);
  const TileDesc& T = a.tiles[tile];
  const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
  const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
  const uint32_t rec = T.ctl->rec;
  if (local == 0u && lane == 0) T.ctl->ledger[rec ^ 1u] = T.ctl->ledger[rec];
  const float* in = T.state[T.ctl->cur];
  const size_t n = size_t(T.nx) * T.ny;
  const int nx = int(T.nx), ny = int(T.ny);
  const int X0 = int(bx) * kStrip, Y0 = int(by) * H;
  const int gx = X0 + lane;
  const int rows = min(H, ny - Y0);
  uint32_t ga = 0u, gb = 0u, ia = 0u, ib = 0u;
  for (int j = 0; j < rows; ++j) {
    const int gy = Y0 + j;
    if (gx < nx) {
      const int i = gy * nx + gx;
      float ax, ay;
      cell_speeds<FIXED>(T.gravity, T.dry, in[i], in[n + i], in[2 * n + i], ax, ay);
      ga = max(ga, __float_as_uint(ax));
      gb = max(gb, __float_as_uint(ay));
    }
    if ((j & 15) == 15 || j == rows - 1) {
      group_records(T.groups_x, T.groups_y, T.rec[rec ^ 1u], X0, gy / 16, ga, gb, wm.ring, false,
                    false, false, ia, ib);
      ga = gb = 0u;
    }
  }
  if (lane == 0) finish_item(T, rec, ia, ib, false);
}

// dt_main alone, on one tile (slang:412-479): a flush (max_dt 0) or the length pass. The records'
// sums are folded and cleared; the ledger is written in place.
template <bool FIXED>
__global__ void __launch_bounds__(256) length_pass_kernel(const TileDesc* tiles, uint32_t tile,
                                                          float max_dt) {
  __shared__ float s[3 * kGroupCells];
  __shared__ uint32_t s_ab[2];
  const TileDesc& T = tiles[tile];
  const uint32_t cr = T.ctl->rec;
  Partial* rec = T.rec[cr];
  fold_cta(rec, T.groups_x * T.groups_y, s, s_ab);
  if (threadIdx.x == 0) {
    LedgerBits l = T.ctl->ledger[cr];
    ledger_update<FIXED>(l, s[0], s[kGroupCells], s[2 * kGroupCells], __uint_as_float(s_ab[0]),
                         __uint_as_float(s_ab[1]), T.cfl, T.cell_m, max_dt);
    T.ctl->ledger[cr] = l;
  }
}

// ---- uploads and read-backs -------------------------------------------------------------------

__device__ __forceinline__ void reset_ledger(TileCtl* ctl) {
  LedgerBits empty = {};
  empty.remaining_s = __int_as_float(0x7f800000);
  ctl->ledger[0] = empty;
  ctl->ledger[1] = empty;
  ctl->src_phase = 0u;
}

// write_state's conversion (water_live.cpp:276-282): planes 0-2 rounded from double, plane 3 zero,
// into the copy that holds the state; the ledger emptied and the source's clock restarted.
__global__ void write_state_kernel(TileDesc* tiles, uint32_t tile, const double* h,
                                   const double* hu, const double* hv) {
  const TileDesc& T = tiles[tile];
  const size_t n = size_t(T.nx) * T.ny;
  float* p = T.state[T.ctl->cur];
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    p[i] = __double2float_rn(h[i]);
    p[n + i] = __double2float_rn(hu[i]);
    p[2 * n + i] = __double2float_rn(hv[i]);
    p[3 * n + i] = 0.0f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) reset_ledger(T.ctl);
}

// write_state from float planes already on the device (planes 0-2 copied, plane 3 zeroed).
__global__ void write_state_f32_kernel(TileDesc* tiles, uint32_t tile, const float* src) {
  const TileDesc& T = tiles[tile];
  const size_t n = size_t(T.nx) * T.ny;
  float* p = T.state[T.ctl->cur];
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    p[i] = src[i];
    p[n + i] = src[n + i];
    p[2 * n + i] = src[2 * n + i];
    p[3 * n + i] = 0.0f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) reset_ledger(T.ctl);
}

// set_bed / set_manning / set_source's conversion: (x - datum) in double, rounded once.
__global__ void plane_kernel(float* dst, const double* src, size_t n, double datum) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x)
    dst[i] = __double2float_rn(src[i] - datum);
}

// read_state's widening (water_live.cpp:341-345), from the copy that holds the state.
__global__ void read_state_kernel(const TileDesc* tiles, uint32_t tile, double* h, double* hu,
                                  double* hv) {
  const TileDesc& T = tiles[tile];
  const size_t n = size_t(T.nx) * T.ny;
  const float* p = T.state[T.ctl->cur];
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    h[i] = double(p[i]);
    hu[i] = double(p[n + i]);
    hv[i] = double(p[2 * n + i]);
  }
}

// Copies the copy that holds the state (all four planes) to a flat buffer.
__global__ void copy_state_kernel(const TileDesc* tiles, uint32_t tile, float* dst) {
  const TileDesc& T = tiles[tile];
  const size_t n4 = size_t(kStatePlanes) * T.nx * T.ny;
  const float* p = T.state[T.ctl->cur];
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n4;
       i += size_t(gridDim.x) * blockDim.x)
    dst[i] = p[i];
}

// ---- the settled check (ADR-0080 decision 4) ---------------------------------------------------

// Per tile, the largest |h - h*| and the largest of |hu - hu*| and |hv - hv*| over its cells, the
// steady state h*, hu*, hv* given as doubles and rounded to f32 as the step rounds its state.
// blockIdx.y is the tile (tile0 + y), blockIdx.x a stride over its cells; the tile's cells start at
// first[t] in the arrays (0 where `first` is null). The maxima go into dev[2 y], dev[2 y + 1] by
// atomicMax on the bits of non-negative floats: exact in any order, and a NaN's bits exceed every
// number's, so a tile holding a NaN never settles.
__global__ void __launch_bounds__(256) settled_kernel(const TileDesc* tiles, uint32_t tile0,
                                                      const uint64_t* first, const double* h,
                                                      const double* hu, const double* hv,
                                                      uint32_t* dev) {
  const uint32_t t = tile0 + blockIdx.y;
  const TileDesc& T = tiles[t];
  const size_t n = size_t(T.nx) * T.ny;
  const size_t base = first == nullptr ? 0 : size_t(first[t]);
  const float* st = T.state[T.ctl->cur];
  uint32_t dd = 0u, dq = 0u;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    const float a = fabsf(__fsub_rn(st[i], __double2float_rn(h[base + i])));
    const float b = fabsf(__fsub_rn(st[n + i], __double2float_rn(hu[base + i])));
    const float c = fabsf(__fsub_rn(st[2 * n + i], __double2float_rn(hv[base + i])));
    dd = max(dd, __float_as_uint(a));
    dq = max(dq, max(__float_as_uint(b), __float_as_uint(c)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dd = max(dd, __shfl_xor_sync(0xffffffffu, dd, o));
    dq = max(dq, __shfl_xor_sync(0xffffffffu, dq, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&dev[2 * blockIdx.y], dd);
    atomicMax(&dev[2 * blockIdx.y + 1], dq);
  }
}

// ---- whole batches: arrays of every tile's cells, tile after tile ------------------------------

// The tile holding global cell index k of the batch (first[t] = the tile's first cell).
__device__ __forceinline__ uint32_t tile_of_cell(const uint64_t* first, uint32_t count, uint64_t k) {
  uint32_t lo = 0, hi = count;
  while (hi - lo > 1u) {
    const uint32_t mid = (lo + hi) >> 1;
    if (first[mid] <= k) lo = mid;
    else hi = mid;
  }
  return lo;
}

// write_state for every tile at once from concatenated doubles (water_live.cpp:276-282).
__global__ void scatter_state_kernel(TileDesc* tiles, uint32_t count, const uint64_t* first,
                                     uint64_t total, const double* h, const double* hu,
                                     const double* hv) {
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t t = tile_of_cell(first, count, k);
    const TileDesc& T = tiles[t];
    const size_t n = size_t(T.nx) * T.ny;
    const size_t i = size_t(k - first[t]);
    float* p = T.state[T.ctl->cur];
    p[i] = __double2float_rn(h[k]);
    p[n + i] = __double2float_rn(hu[k]);
    p[2 * n + i] = __double2float_rn(hv[k]);
    p[3 * n + i] = 0.0f;
    if (i == 0) reset_ledger(T.ctl);
  }
}

// set_bed / set_manning / set_source for every tile at once: which 0 bed, 1 Manning, 2 source.
__global__ void scatter_plane_kernel(TileDesc* tiles, uint32_t count, const uint64_t* first,
                                     uint64_t total, const double* v, double datum, int which) {
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t t = tile_of_cell(first, count, k);
    const TileDesc& T = tiles[t];
    float* dst = const_cast<float*>(which == 0 ? T.bed : which == 1 ? T.manning : T.source);
    dst[k - first[t]] = __double2float_rn(v[k] - datum);
  }
}

// Every tile's current copy, all four planes, tile after tile (4 n floats a tile).
__global__ void gather_state_kernel(const TileDesc* tiles, uint32_t count, const uint64_t* first,
                                    uint64_t total, float* dst) {
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t t = tile_of_cell(first, count, k);
    const TileDesc& T = tiles[t];
    const size_t n = size_t(T.nx) * T.ny;
    const size_t i = size_t(k - first[t]);
    const float* p = T.state[T.ctl->cur];
    float* d = dst + 4 * first[t];
#pragma unroll
    for (int q = 0; q < 4; ++q) d[q * n + i] = p[q * n + i];
  }
}

// A flush of every tile at once: a CTA a tile, dt_main with max_dt 0 (slang:412-479).
template <bool FIXED>
__global__ void __launch_bounds__(256) flush_all_kernel(const TileDesc* tiles) {
  __shared__ float s[3 * kGroupCells];
  __shared__ uint32_t s_ab[2];
  const TileDesc& T = tiles[blockIdx.x];
  const uint32_t cr = T.ctl->rec;
  Partial* rec = T.rec[cr];
  fold_cta(rec, T.groups_x * T.groups_y, s, s_ab);
  if (threadIdx.x == 0) {
    LedgerBits l = T.ctl->ledger[cr];
    ledger_update<FIXED>(l, s[0], s[kGroupCells], s[2 * kGroupCells], __uint_as_float(s_ab[0]),
                         __uint_as_float(s_ab[1]), T.cfl, T.cell_m, 0.0f);
    T.ctl->ledger[cr] = l;
  }
}

const void* split_fn(bool fixed, bool manning) {
  if (fixed)
    return manning ? (const void*)tick_split_kernel<true, true>
                   : (const void*)tick_split_kernel<true, false>;
  return manning ? (const void*)tick_split_kernel<false, true>
                 : (const void*)tick_split_kernel<false, false>;
}

template <int THREADS>
const void* block_fn(bool fixed, bool manning) {
  if (fixed)
    return manning ? (const void*)tick_block_kernel<true, true, THREADS>
                   : (const void*)tick_block_kernel<true, false, THREADS>;
  return manning ? (const void*)tick_block_kernel<false, true, THREADS>
                 : (const void*)tick_block_kernel<false, false, THREADS>;
}

template <int THREADS, bool STAGE>
void (*block_kernel(bool fixed, bool manning))(TickArgs) {
  return fixed ? (manning ? tick_block_kernel<true, true, THREADS, STAGE>
                          : tick_block_kernel<true, false, THREADS, STAGE>)
               : (manning ? tick_block_kernel<false, true, THREADS, STAGE>
                          : tick_block_kernel<false, false, THREADS, STAGE>);
}

template <int THREADS>
cudaError_t block_launch(bool fixed, bool manning, const TickArgs& a, int grid, cudaStream_t s) {
  static_assert(kStagedSmemBytes <= 48u * 1024u, "the staged block tick needs no opt-in");
  if (a.stage != 0u)
    return launch_dependent(block_kernel<THREADS, true>(fixed, manning), dim3(grid),
                            dim3(THREADS), kStagedSmemBytes, s, a);
  return launch_dependent(block_kernel<THREADS, false>(fixed, manning), dim3(grid), dim3(THREADS),
                          sizeof(BlockSmem), s, a);
}

cudaError_t split_launch(bool fixed, bool manning, const TickArgs& a, int grid, cudaStream_t s) {
  const size_t smem = kWarpsPerCta * WarpMem<4>::kBytes;
  void (*k)(TickArgs) = fixed ? (manning ? tick_split_kernel<true, true> : tick_split_kernel<true, false>)
                              : (manning ? tick_split_kernel<false, true> : tick_split_kernel<false, false>);
  return launch_dependent(k, dim3(grid), dim3(kCtaThreads), smem, s, a);
}

// The march's variants: Manning's, the plain one (where `plain` and no Manning), the general one.
template <int H>
const void* tick_fn(bool fixed, bool manning, bool plain) {
  if (fixed) {
    if (manning) return (const void*)tick_kernel<true, true, H, false>;
    return plain ? (const void*)tick_kernel<true, false, H, true>
                 : (const void*)tick_kernel<true, false, H, false>;
  }
  if (manning) return (const void*)tick_kernel<false, true, H, false>;
  return plain ? (const void*)tick_kernel<false, false, H, true>
               : (const void*)tick_kernel<false, false, H, false>;
}

template <int H>
cudaError_t tick_launch(bool fixed, bool manning, bool plain, const TickArgs& a, int grid,
                        cudaStream_t s) {
  // The zero-apart variant: the native arithmetic's plain march only (the fixed form's quotient
  // and root have no slow path to skip).
  const bool zg = a.zero_apart != 0u && !fixed && !manning && plain;
  void (*k)(TickArgs) =
      fixed ? (manning ? tick_kernel<true, true, H, false>
                       : plain ? tick_kernel<true, false, H, true> : tick_kernel<true, false, H, false>)
            : (manning ? tick_kernel<false, true, H, false>
                       : plain ? (zg ? tick_kernel<false, false, H, true, true>
                                     : tick_kernel<false, false, H, true>)
                               : tick_kernel<false, false, H, false>);
  return launch_dependent(k, dim3(grid), dim3(kCtaThreads), kWarpsPerCta * WarpMem<H>::kBytes, s,
                          a);
}

template <int H>
cudaError_t prime_launch(bool fixed, const TickArgs& a, cudaStream_t s) {
  const size_t smem = kWarpsPerCta * WarpMem<H>::kBytes;
  const unsigned grid = (a.n_items + kWarpsPerCta - 1) / kWarpsPerCta;
  if (fixed) prime_kernel<true, H><<<grid, kCtaThreads, smem, s>>>(a);
  else prime_kernel<false, H><<<grid, kCtaThreads, smem, s>>>(a);
  return cudaGetLastError();
}

int grid_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return int(b < 4096 ? (b == 0 ? 1 : b) : 4096);
}

}  // namespace

// ---- host-side launchers (wl_kernels.h) ---------------------------------------------------------

cudaError_t launch_settled(const TileDesc* tiles, uint32_t tile0, uint32_t count,
                           const uint64_t* first, uint64_t largest, const double* h,
                           const double* hu, const double* hv, uint32_t* dev, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  if (cudaMemsetAsync(dev, 0, size_t(count) * 2 * sizeof(uint32_t), s) != cudaSuccess)
    return cudaGetLastError();
  const uint64_t chunks = std::min<uint64_t>((largest + 4095) / 4096, 1024);
  for (uint32_t k = 0; k < count; k += 65535u) {
    const uint32_t c = std::min<uint32_t>(65535u, count - k);
    settled_kernel<<<dim3(unsigned(std::max<uint64_t>(chunks, 1)), c), 256, 0, s>>>(
        tiles, tile0 + k, first, h, hu, hv, dev + 2 * size_t(k));
  }
  return cudaGetLastError();
}

bool encode_stage_maps(const TileDesc& d, void* maps) {
  static_assert(sizeof(CUtensorMap) == 128, "a tensor map is 128 bytes");
  // The driver's encoder, looked up once through the runtime (no link against the driver).
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  // A box's x must start on a 16-byte boundary: rows of a multiple of 4 floats, and X0 - 4 with X0
  // a multiple of 32. The planes' strides (row: 4 nx bytes, plane: 4 nx ny) are then multiples of
  // 16, as a tensor map requires, and every allocation the kernels read starts on 256 bytes.
  if (encode == nullptr || d.nx % 4u != 0u || d.nx == 0u || d.ny == 0u) return false;
  CUtensorMap* m = static_cast<CUtensorMap*>(maps);
  const cuuint64_t n = cuuint64_t(d.nx) * d.ny;
  const cuuint32_t unit[3] = {1, 1, 1};
  for (int c = 0; c < 2; ++c) {
    const cuuint64_t dims[3] = {d.nx, d.ny, 3};
    const cuuint64_t strides[2] = {cuuint64_t(d.nx) * 4u, n * 4u};
    const cuuint32_t box[3] = {kStageW, kStageH, 3};
    if (encode(&m[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, d.state[c], dims, strides, box, unit,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  const cuuint64_t dims[2] = {d.nx, d.ny};
  const cuuint64_t strides[1] = {cuuint64_t(d.nx) * 4u};
  const cuuint32_t box[2] = {kStageW, kStageH};
  return encode(&m[2], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(d.bed), dims,
                strides, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

size_t tick_smem_bytes(BlockShape shape) {
  switch (shape) {
    case BlockShape::k32x16: return kWarpsPerCta * WarpMem<16>::kBytes;
    case BlockShape::k32x32: return kWarpsPerCta * WarpMem<32>::kBytes;
    case BlockShape::k32x64: return kWarpsPerCta * WarpMem<64>::kBytes;
    case BlockShape::k32x16s: return kWarpsPerCta * WarpMem<4>::kBytes;
    case BlockShape::k32x16b:
    case BlockShape::k32x16w: return sizeof(BlockSmem);
  }
  return 0;
}

int tick_threads(BlockShape shape) {
  if (shape == BlockShape::k32x16b) return kBlkThreads;
  if (shape == BlockShape::k32x16w) return kBlkWideThreads;
  return kCtaThreads;
}

void block_dims(BlockShape shape, uint32_t& bx, uint32_t& by) {
  bx = kStrip;
  switch (shape) {
    case BlockShape::k32x16: by = 16; return;
    case BlockShape::k32x32: by = 32; return;
    case BlockShape::k32x64: by = 64; return;
    case BlockShape::k32x16s:
    case BlockShape::k32x16b:
    case BlockShape::k32x16w: by = 16; return;
  }
  by = 0;
}

int tick_occupancy(BlockShape shape, bool fixed, bool manning, bool plain) {
  const void* fn = nullptr;
  switch (shape) {
    case BlockShape::k32x16: fn = tick_fn<16>(fixed, manning, plain); break;
    case BlockShape::k32x32: fn = tick_fn<32>(fixed, manning, plain); break;
    case BlockShape::k32x64: fn = tick_fn<64>(fixed, manning, plain); break;
    case BlockShape::k32x16s: fn = split_fn(fixed, manning); break;
    case BlockShape::k32x16b: fn = block_fn<kBlkThreads>(fixed, manning); break;
    case BlockShape::k32x16w: fn = block_fn<kBlkWideThreads>(fixed, manning); break;
  }
  const size_t smem = tick_smem_bytes(shape);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
    return 0;
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, tick_threads(shape), smem) !=
      cudaSuccess)
    return 0;
  return blocks;
}

cudaError_t launch_tick(BlockShape shape, bool fixed, bool manning, bool plain,
                        const TickArgs& args, int grid, cudaStream_t s) {
  TickArgs a = args;
  a.n_whole = a.n_items;
  if (shape == BlockShape::k32x16 && grid > 0) {
    // Whole rounds of items a warp each; the remainder (fewer than the warps) a CTA each.
    const uint32_t warps = uint32_t(grid) * uint32_t(kWarpsPerCta);
    if (a.n_items > warps) a.n_whole = a.n_items - a.n_items % warps;
  }
  switch (shape) {
    case BlockShape::k32x16: return tick_launch<16>(fixed, manning, plain, a, grid, s);
    case BlockShape::k32x32: return tick_launch<32>(fixed, manning, plain, a, grid, s);
    case BlockShape::k32x64: return tick_launch<64>(fixed, manning, plain, a, grid, s);
    case BlockShape::k32x16s: return split_launch(fixed, manning, a, grid, s);
    case BlockShape::k32x16b: return block_launch<kBlkThreads>(fixed, manning, a, grid, s);
    case BlockShape::k32x16w: return block_launch<kBlkWideThreads>(fixed, manning, a, grid, s);
  }
  return cudaErrorInvalidValue;
}

namespace {
const void* resident_fn(bool fixed, bool manning) {
  if (fixed)
    return manning ? (const void*)tick_resident_kernel<true, true>
                   : (const void*)tick_resident_kernel<true, false>;
  return manning ? (const void*)tick_resident_kernel<false, true>
                 : (const void*)tick_resident_kernel<false, false>;
}
}  // namespace

int resident_capacity(bool fixed, bool manning) {
  const void* fn = resident_fn(fixed, manning);
  const int smem = int(sizeof(BlockSmem));
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return 0;
  int blocks = 0, device = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kResThreads, smem) !=
          cudaSuccess ||
      cudaGetDevice(&device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return 0;
  return blocks * sms;
}

cudaError_t launch_tick_resident(bool fixed, bool manning, const TickArgs& args, uint32_t ticks,
                                 ResidentCtl* rc, cudaStream_t s) {
  TickArgs a = args;
  a.n_whole = a.n_items;
  a.fold_apart = 1u;
  if (cudaMemsetAsync(rc, 0, sizeof(ResidentCtl), s) != cudaSuccess) return cudaGetLastError();
  void (*k)(TickArgs, uint32_t, ResidentCtl*) =
      fixed ? (manning ? tick_resident_kernel<true, true> : tick_resident_kernel<true, false>)
            : (manning ? tick_resident_kernel<false, true> : tick_resident_kernel<false, false>);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.n_items + 1u);
  cfg.blockDim = dim3(kResThreads);
  cfg.dynamicSmemBytes = sizeof(BlockSmem);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, a, ticks, rc);
}

cudaError_t launch_barrier_probe(ResidentCtl* rc, uint32_t n, cudaStream_t s) {
  if (cudaMemsetAsync(rc, 0, sizeof(ResidentCtl), s) != cudaSuccess) return cudaGetLastError();
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n);
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, resident_barrier_probe_kernel, rc, n);
}

cudaError_t launch_prime(BlockShape shape, bool fixed, const TickArgs& a, cudaStream_t s) {
  if (a.n_items == 0) return cudaSuccess;
  switch (shape) {
    case BlockShape::k32x16:
    case BlockShape::k32x16s:
    case BlockShape::k32x16b:
    case BlockShape::k32x16w: return prime_launch<16>(fixed, a, s);
    case BlockShape::k32x32: return prime_launch<32>(fixed, a, s);
    case BlockShape::k32x64: return prime_launch<64>(fixed, a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_length_pass(bool fixed, const TileDesc* tiles, uint32_t tile, float max_dt,
                               cudaStream_t s) {
  if (fixed) length_pass_kernel<true><<<1, 256, 0, s>>>(tiles, tile, max_dt);
  else length_pass_kernel<false><<<1, 256, 0, s>>>(tiles, tile, max_dt);
  return cudaGetLastError();
}

cudaError_t launch_write_state(TileDesc* tiles, uint32_t tile, size_t n, const double* h,
                               const double* hu, const double* hv, cudaStream_t s) {
  write_state_kernel<<<grid_for(n), 256, 0, s>>>(tiles, tile, h, hu, hv);
  return cudaGetLastError();
}

cudaError_t launch_write_state_f32(TileDesc* tiles, uint32_t tile, size_t n, const float* planes,
                                   cudaStream_t s) {
  write_state_f32_kernel<<<grid_for(n), 256, 0, s>>>(tiles, tile, planes);
  return cudaGetLastError();
}

cudaError_t launch_plane(float* dst, const double* src, size_t n, double datum, cudaStream_t s) {
  plane_kernel<<<grid_for(n), 256, 0, s>>>(dst, src, n, datum);
  return cudaGetLastError();
}

cudaError_t launch_read_state(const TileDesc* tiles, uint32_t tile, size_t n, double* h,
                              double* hu, double* hv, cudaStream_t s) {
  read_state_kernel<<<grid_for(n), 256, 0, s>>>(tiles, tile, h, hu, hv);
  return cudaGetLastError();
}

cudaError_t launch_copy_state(const TileDesc* tiles, uint32_t tile, size_t n, float* dst,
                              cudaStream_t s) {
  copy_state_kernel<<<grid_for(4 * n), 256, 0, s>>>(tiles, tile, dst);
  return cudaGetLastError();
}

cudaError_t launch_scatter_state(TileDesc* tiles, uint32_t count, const uint64_t* first,
                                 uint64_t total, const double* h, const double* hu,
                                 const double* hv, cudaStream_t s) {
  scatter_state_kernel<<<grid_for(total), 256, 0, s>>>(tiles, count, first, total, h, hu, hv);
  return cudaGetLastError();
}

cudaError_t launch_scatter_plane(TileDesc* tiles, uint32_t count, const uint64_t* first,
                                 uint64_t total, const double* v, double datum, int which,
                                 cudaStream_t s) {
  scatter_plane_kernel<<<grid_for(total), 256, 0, s>>>(tiles, count, first, total, v, datum, which);
  return cudaGetLastError();
}

cudaError_t launch_gather_state(const TileDesc* tiles, uint32_t count, const uint64_t* first,
                                uint64_t total, float* dst, cudaStream_t s) {
  gather_state_kernel<<<grid_for(total), 256, 0, s>>>(tiles, count, first, total, dst);
  return cudaGetLastError();
}

cudaError_t launch_flush_all(bool fixed, const TileDesc* tiles, uint32_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  if (fixed) flush_all_kernel<true><<<count, 256, 0, s>>>(tiles);
  else flush_all_kernel<false><<<count, 256, 0, s>>>(tiles);
  return cudaGetLastError();
}

}  // namespace wlc

// The live-water tick's kernels for sm_103a.
//
// One persistent launch steps every tile of a batch by one tick (the plain step is a batch of one
// tile). It replaces the reference's two passes a step, the length pass `dt_main`
// (water_step.slang:412-479) and the update `update_main` (slang:555-757), with one:
//
//   - Work items are blocks of BX x BY cells of some tile; CTAs take them in order from a counter.
//   - Each item chooses the step's length itself, from the tile's control block: the largest
//     speeds of the last update (kept by atomicMax on their bits, exact in any order), the time
//     left and max_dt, the same arithmetic as dt_main's thread 0.
//   - The item that takes a tile's first block also folds the last update's records into the
//     ledger, in dt_main's own order (256 lanes over the records, then a fixed tree), so the
//     ledger's bits are the reference's.
//   - A block stages its cells and a one-cell halo in shared memory ({h, z, u, v}, the edges' ghost
//     cells built as the reference builds them), computes each of its faces once into shared
//     memory (both cells of a face take the same value, which is what the reference's gather
//     computes twice), updates its cells, writes the three planes once, and writes one record per
//     16 x 16 group with the reference's 256-slot tree.
//   - The last item of a tile to finish commits the tick: the new ledger, the flipped copy and
//     record buffer, the new largest speeds and the source's clock.
//
// HBM traffic per cell-update: h, hu, hv, bed read (+ source, + Manning's n, + the remainder when
// on), h, hu, hv written (+ the remainder), a 32-byte record per 256 cells.
#include "wl_device.cuh"
#include "wl_kernels.h"

#include <cstdio>

namespace wlc {

namespace {

template <int BX, int BY>
struct Shape {
  static constexpr int kCellsX = BX + 2;
  static constexpr int kCells = (BX + 2) * (BY + 2);
  static constexpr int kFacesX = (BX + 1) * BY;
  static constexpr int kFacesY = BX * (BY + 1);
  static constexpr int kGroupsX = BX / 16;
  static constexpr int kGroupsY = BY / 16;
  static constexpr int kGroups = kGroupsX * kGroupsY;
  static constexpr int kRowStep = kThreads / BX;     // rows between a thread's cells
  static constexpr int kPerThread = BX * BY / kThreads;
  static constexpr size_t kSmem = sizeof(float4) * (kCells + kFacesX + kFacesY) +
                                  sizeof(float) * 3 * BX * BY;
  static_assert(BX % 32 == 0 && BY % 16 == 0, "blocks are whole warps wide and whole groups tall");
  static_assert(BX * BY >= kThreads && (BX * BY) % kThreads == 0, "whole cells per thread");
};

struct ItemInfo {
  uint32_t tile, bx, by, cur, rec, fold, apply_source;
  float dt, scale;
};

// dt_main's sums (slang:417-456): lane t adds records t, t + 256, ... in order, then the fixed
// 256-slot tree. Leaves the three sums in s[0], s[256], s[512]. When `zero`, the records' sums are
// cleared after they are read (a flush or a length pass; slang:432-435). When `maxima`, also
// returns the records' largest speeds in s_ab (the length pass reads them from the records).
__device__ void fold_sums(Partial* rec, uint32_t groups, bool zero, float* s, uint32_t* s_ab,
                          bool maxima) {
  const int t = threadIdx.x;
  float src = 0.0f, opn = 0.0f, rnd = 0.0f;
  uint32_t a = 0u, b = 0u;
  for (uint32_t gi = t; gi < groups; gi += kThreads) {
    const Partial p = rec[gi];
    src = __fadd_rn(src, p.source_m3);
    opn = __fadd_rn(opn, p.open_m3);
    rnd = __fadd_rn(rnd, p.roundoff_m3);
    a = max(a, __float_as_uint(p.speed_x));
    b = max(b, __float_as_uint(p.speed_y));
    if (zero) {
      rec[gi].source_m3 = 0.0f;
      rec[gi].open_m3 = 0.0f;
      rec[gi].roundoff_m3 = 0.0f;
    }
  }
  s[t] = src;
  s[kThreads + t] = opn;
  s[2 * kThreads + t] = rnd;
  __syncthreads();
#pragma unroll
  for (int stride = kThreads / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      s[t] = __fadd_rn(s[t], s[t + stride]);
      s[kThreads + t] = __fadd_rn(s[kThreads + t], s[kThreads + t + stride]);
      s[2 * kThreads + t] = __fadd_rn(s[2 * kThreads + t], s[2 * kThreads + t + stride]);
    }
    __syncthreads();
  }
  if (maxima) {
    if (t == 0) {
      s_ab[0] = 0u;
      s_ab[1] = 0u;
    }
    __syncthreads();
    atomicMax(&s_ab[0], a);
    atomicMax(&s_ab[1], b);
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

__device__ __forceinline__ void copy_ledger(volatile LedgerBits* dst, const volatile LedgerBits* src) {
  const volatile uint32_t* s = reinterpret_cast<const volatile uint32_t*>(src);
  volatile uint32_t* d = reinterpret_cast<volatile uint32_t*>(dst);
#pragma unroll
  for (int i = 0; i < 12; ++i) d[i] = s[i];
}

// The end of a work item (thread 0, after the block's writes were fenced): the block's largest
// speeds into the tile's running maxima, and, for the tile's last item, the commit.
__device__ void finish_item(const TileDesc& T, uint32_t amax, uint32_t bmax, bool tick) {
  TileCtl* ctl = T.ctl;
  atomicMax(&ctl->max_a, amax);
  atomicMax(&ctl->max_b, bmax);
  __threadfence();
  const uint32_t d = atomicAdd(&ctl->done, 1u);
  if (d + 1u != T.items) return;
  __threadfence();
  volatile TileCtl* v = ctl;
  v->prev_a = atomicExch(&ctl->max_a, 0u);
  v->prev_b = atomicExch(&ctl->max_b, 0u);
  if (tick) {
    copy_ledger(&v->ledger, &v->ledger_next);
    v->cur = v->cur ^ 1u;
    v->rec = v->rec ^ 1u;
    if ((T.flags & kFlagSource) != 0u && T.source_every > 1u) {
      const uint32_t p = v->src_phase + 1u;
      v->src_phase = p == T.source_every ? 0u : p;
    }
    v->ticks = v->ticks + 1u;
  }
  v->done = 0u;
  __threadfence();
}

// The records of one block from per-cell values in shared memory: the largest speeds (exact in any
// order) reduced by shuffles, and each of the three sums by the reference's 256-slot tree
// (slang:338-371) where any of its cells holds a non-zero value.
template <int BX, int BY>
__device__ void write_records(const TileDesc& T, Partial* rec_out, uint32_t bx, uint32_t by,
                              const float* s_sum, uint32_t* s_gmax, float* s_gsum,
                              const uint32_t (&amax)[BY / 16], const uint32_t (&bmax)[BY / 16],
                              bool need_src, bool need_opn, bool need_rnd, uint32_t& blk_a,
                              uint32_t& blk_b) {
  using S = Shape<BX, BY>;
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  const int c = t % BX;
  const int gc = c / 16;
  // Speeds: the 16 lanes of a half-warp hold one group's column range.
#pragma unroll
  for (int gr = 0; gr < S::kGroupsY; ++gr) {
    uint32_t a = amax[gr], b = bmax[gr];
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
      a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
      b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if ((lane & 15) == 0) {
      atomicMax(&s_gmax[2 * (gr * S::kGroupsX + gc)], a);
      atomicMax(&s_gmax[2 * (gr * S::kGroupsX + gc) + 1], b);
    }
  }
  // Sums: one warp per (group, quantity) tree. Lane l holds slots l + 32 k, k = 0..7; slot
  // i = ly * 16 + lx of the group.
  const bool need[3] = {need_src, need_opn, need_rnd};
  for (int job = warp; job < 3 * S::kGroups; job += kThreads / 32) {
    const int q = job / S::kGroups, grp = job % S::kGroups;
    float res = 0.0f;
    if (need[q]) {
      const int gr = grp / S::kGroupsX, gcc = grp % S::kGroupsX;
      const float* base = s_sum + q * BX * BY + (gr * 16) * BX + gcc * 16;
      float v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int slot = lane + 32 * k;
        v[k] = base[(slot >> 4) * BX + (slot & 15)];
      }
      // strides 128, 64, 32: slot + 128 is k + 4, + 64 is k + 2, + 32 is k + 1
      const float a0 = __fadd_rn(v[0], v[4]), a1 = __fadd_rn(v[1], v[5]);
      const float a2 = __fadd_rn(v[2], v[6]), a3 = __fadd_rn(v[3], v[7]);
      const float b0 = __fadd_rn(a0, a2), b1 = __fadd_rn(a1, a3);
      float cc = __fadd_rn(b0, b1);
#pragma unroll
      for (int stride = 16; stride > 0; stride >>= 1) {
        const float o = __shfl_down_sync(0xffffffffu, cc, stride);
        if (lane < stride) cc = __fadd_rn(cc, o);
      }
      res = cc;
    }
    if (lane == 0) s_gsum[grp * 3 + q] = res;
  }
  __syncthreads();
  if (t < S::kGroups) {
    const int gr = t / S::kGroupsX, gcc = t % S::kGroupsX;
    const uint32_t gxg = bx * S::kGroupsX + gcc, gyg = by * S::kGroupsY + gr;
    if (gxg < T.groups_x && gyg < T.groups_y) {
      float4* dst = reinterpret_cast<float4*>(rec_out + size_t(gyg) * T.groups_x + gxg);
      dst[0] = make_float4(__uint_as_float(s_gmax[2 * t]), __uint_as_float(s_gmax[2 * t + 1]),
                           s_gsum[t * 3 + 0], s_gsum[t * 3 + 1]);
      dst[1] = make_float4(s_gsum[t * 3 + 2], 0.0f, 0.0f, 0.0f);
    }
  }
  if (t == 0) {
    uint32_t a = 0u, b = 0u;
    for (int g = 0; g < S::kGroups; ++g) {
      a = max(a, s_gmax[2 * g]);
      b = max(b, s_gmax[2 * g + 1]);
    }
    blk_a = a;
    blk_b = b;
  }
}

__device__ __forceinline__ uint32_t item_tile_of(const uint32_t* item_tile, uint32_t item) {
  return item_tile == nullptr ? 0u : item_tile[item];
}

// One block of one tile, one tick.
template <bool FIXED, bool MANNING, int BX, int BY>
__device__ void step_block(const TileDesc& T, const ItemInfo& it, float max_dt, float4* s_cell,
                           float4* s_fx, float4* s_fy, float* s_sum, uint32_t* s_gmax,
                           float* s_gsum, uint32_t& blk_a, uint32_t& blk_b) {
  using S = Shape<BX, BY>;
  using O = Ops<FIXED>;
  const int t = threadIdx.x;
  const uint32_t nx = T.nx, ny = T.ny;
  const size_t n = size_t(nx) * ny;
  const int X0 = int(it.bx) * BX, Y0 = int(it.by) * BY;
  const float* in = T.state[it.cur];
  float* out = T.state[it.cur ^ 1u];
  const float g = T.gravity, dry = T.dry, half_g = __fmul_rn(0.5f, g);
  const float dt = it.dt;
  const uint32_t flags = T.flags;
  const bool stepping = dt > 0.0f;

  if (t < 2 * S::kGroups) s_gmax[t] = 0u;

  if (stepping) {
    // Stage the block and its halo: {h, z, u, v}, ghosts at the edges (slang:597-628).
    const float sw = (flags & kFlagWestOpen) ? 1.0f : -1.0f;
    const float se = (flags & kFlagEastOpen) ? 1.0f : -1.0f;
    const float ss = (flags & kFlagSouthOpen) ? 1.0f : -1.0f;
    const float sn = (flags & kFlagNorthOpen) ? 1.0f : -1.0f;
    for (int p = t; p < S::kCells; p += kThreads) {
      const int py = p / S::kCellsX, px = p - py * S::kCellsX;
      const int gx = X0 + px - 1, gy = Y0 + py - 1;
      const bool inx = gx >= 0 && gx < int(nx), iny = gy >= 0 && gy < int(ny);
      int sx = gx, sy = gy;
      int ghost = 0;  // 1: the normal is u, 2: the normal is v
      float sign = 1.0f;
      bool use = inx && iny;
      if (!use && iny) {
        if (gx == -1) { sx = 0; sign = sw; ghost = 1; use = true; }
        else if (gx == int(nx)) { sx = int(nx) - 1; sign = se; ghost = 1; use = true; }
      } else if (!use && inx) {
        if (gy == -1) { sy = 0; sign = ss; ghost = 2; use = true; }
        else if (gy == int(ny)) { sy = int(ny) - 1; sign = sn; ghost = 2; use = true; }
      }
      float4 cv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (use) {
        const size_t i = size_t(sy) * nx + sx;
        const float h = in[i];
        const bool wet = h >= dry;
        float u = wet ? O::div(in[n + i], h) : 0.0f;
        float v = wet ? O::div(in[2 * n + i], h) : 0.0f;
        if (ghost == 1) u = __fmul_rn(sign, u);
        if (ghost == 2) v = __fmul_rn(sign, v);
        cv = make_float4(h, T.bed[i], u, v);
      }
      s_cell[p] = cv;
    }
    __syncthreads();
    // Every face of the block once: x faces west of each column, y faces south of each row.
    for (int f = t; f < S::kFacesX + S::kFacesY; f += kThreads) {
      float4 res = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (f < S::kFacesX) {
        const int r = f / (BX + 1), c = f - r * (BX + 1);
        if (Y0 + r < int(ny) && X0 + c - 1 < int(nx)) {
          const float4 L = s_cell[(r + 1) * S::kCellsX + c];
          const float4 R = s_cell[(r + 1) * S::kCellsX + c + 1];
          res = face<FIXED>(g, half_g, L.x, L.y, L.z, L.w, R.x, R.y, R.z, R.w);
        }
        s_fx[f] = res;
      } else {
        const int f2 = f - S::kFacesX;
        const int r = f2 / BX, c = f2 - r * BX;
        if (X0 + c < int(nx) && Y0 + r - 1 < int(ny)) {
          const float4 Sc = s_cell[r * S::kCellsX + c + 1];
          const float4 Nc = s_cell[(r + 1) * S::kCellsX + c + 1];
          res = face<FIXED>(g, half_g, Sc.x, Sc.y, Sc.w, Sc.z, Nc.x, Nc.y, Nc.w, Nc.z);
        }
        s_fy[f2] = res;
      }
    }
    __syncthreads();
  } else {
    __syncthreads();
  }

  // The update of each cell (slang:630-753).
  const float cell_m = T.cell_m;
  const float area = __fmul_rn(cell_m, cell_m);
  const float lam = O::div(dt, cell_m);
  const float edge_volume = __fmul_rn(dt, cell_m);
  const bool src_on = it.apply_source != 0u;
  const bool comp = (flags & kFlagCompensate) != 0u;
  const bool manning = MANNING && (flags & kFlagManning) != 0u;
  const float scale = it.scale;
  const int c = t % BX, r0 = t / BX;
  const int gx = X0 + c;
  uint32_t amax[BY / 16], bmax[BY / 16];
#pragma unroll
  for (int k = 0; k < BY / 16; ++k) amax[k] = bmax[k] = 0u;
  bool any_rnd = false;
#pragma unroll
  for (int k = 0; k < S::kPerThread; ++k) {
    const int r = r0 + k * S::kRowStep;
    const int gy = Y0 + r;
    float ax = 0.0f, ay = 0.0f, csrc = 0.0f, copn = 0.0f, crnd = 0.0f;
    if (gx < int(nx) && gy < int(ny)) {
      const size_t i = size_t(gy) * nx + gx;
      if (!stepping) {
        // A step of no length: the state as it is, to the bit (slang:576-585).
        const float h0 = in[i], hu0 = in[n + i], hv0 = in[2 * n + i];
        out[i] = h0;
        out[n + i] = hu0;
        out[2 * n + i] = hv0;
        out[3 * n + i] = in[3 * n + i];
        cell_speeds<FIXED>(g, dry, h0, hu0, hv0, ax, ay);
      } else {
        const float4 fw = s_fx[r * (BX + 1) + c];
        const float4 fe = s_fx[r * (BX + 1) + c + 1];
        const float4 fs = s_fy[r * BX + c];
        const float4 fn = s_fy[(r + 1) * BX + c];
        const float h0 = s_cell[(r + 1) * S::kCellsX + c + 1].x;
        if ((flags & 15u) != 0u) {
          if (gx == 0 && (flags & kFlagWestOpen)) copn = __fsub_rn(copn, __fmul_rn(fw.x, edge_volume));
          if (gx + 1 == int(nx) && (flags & kFlagEastOpen)) copn = __fadd_rn(copn, __fmul_rn(fe.x, edge_volume));
          if (gy == 0 && (flags & kFlagSouthOpen)) copn = __fsub_rn(copn, __fmul_rn(fs.x, edge_volume));
          if (gy + 1 == int(ny) && (flags & kFlagNorthOpen)) copn = __fadd_rn(copn, __fmul_rn(fn.x, edge_volume));
        }
        // U' = U - dt/dx ((F_e - F_w) + (F_n - F_s)) (slang:653-668)
        float h = __fsub_rn(h0, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.x, fw.x), __fsub_rn(fn.x, fs.x))));
        float hu = __fsub_rn(in[n + i], __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.y, fw.z), __fsub_rn(fn.w, fs.w))));
        float hv = __fsub_rn(in[2 * n + i], __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.w, fw.w), __fsub_rn(fn.y, fs.z))));
        if (h < 0.0f) {
          crnd = __fsub_rn(crnd, __fmul_rn(h, area));
          h = 0.0f;
          any_rnd = true;
        }
        float residual = 0.0f;
        if (comp) residual = in[3 * n + i];
        if (src_on && comp) {
          const float owed = __fmul_rn(T.source[i], dt);
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
        } else if (src_on) {
          const float owed = __fmul_rn(T.source[i], dt);
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
        if (h >= dry) {
          if (manning) {
            // (hu)' = (hu)* / (1 + dt g n^2 |u*| / h^(4/3)) (slang:722-744)
            const float nn = T.manning[i];
            const float u = O::div(hu, h);
            const float v = O::div(hv, h);
            const float sp = O::sqrt(__fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)));
            const float cb = O::cbrt(h);
            const float k3 = __fmul_rn(__fmul_rn(__fmul_rn(g, nn), nn), sp);
            const float k = O::div(k3, __fmul_rn(h, cb));
            const float denom = __fadd_rn(1.0f, __fmul_rn(dt, k));
            hu = O::div(hu, denom);
            hv = O::div(hv, denom);
          }
        } else {
          hu = 0.0f;
          hv = 0.0f;
        }
        out[i] = h;
        out[n + i] = hu;
        out[2 * n + i] = hv;
        if (comp) out[3 * n + i] = residual;
        cell_speeds<FIXED>(g, dry, h, hu, hv, ax, ay);
      }
    }
    const int ci = r * BX + c;
    s_sum[ci] = csrc;
    s_sum[BX * BY + ci] = copn;
    s_sum[2 * BX * BY + ci] = crnd;
    const int gr = (k * S::kRowStep) / 16;  // r0 < kRowStep <= 16: a compile-time group row
    amax[gr] = max(amax[gr], __float_as_uint(ax));
    bmax[gr] = max(bmax[gr], __float_as_uint(ay));
  }
  const bool need_rnd = __syncthreads_or(any_rnd) != 0;
  const bool touches_open =
      ((flags & kFlagWestOpen) && X0 == 0) || ((flags & kFlagEastOpen) && X0 + BX >= int(nx)) ||
      ((flags & kFlagSouthOpen) && Y0 == 0) || ((flags & kFlagNorthOpen) && Y0 + BY >= int(ny));
  write_records<BX, BY>(T, T.rec[it.rec ^ 1u], it.bx, it.by, s_sum, s_gmax, s_gsum, amax, bmax,
                        stepping && src_on, stepping && touches_open, need_rnd, blk_a, blk_b);
}

template <int BX, int BY>
__device__ __forceinline__ void carve(float4*& s_cell, float4*& s_fx, float4*& s_fy,
                                      float*& s_sum) {
  using S = Shape<BX, BY>;
  extern __shared__ float4 smem[];
  s_cell = smem;
  s_fx = s_cell + S::kCells;
  s_fy = s_fx + S::kFacesX;
  s_sum = reinterpret_cast<float*>(s_fy + S::kFacesY);
}

// The persistent tick: every work item of every tile, one tick.
template <bool FIXED, bool MANNING, int BX, int BY>
__global__ void __launch_bounds__(kThreads) tick_kernel(TickArgs a) {
  float4 *s_cell, *s_fx, *s_fy;
  float* s_sum;
  carve<BX, BY>(s_cell, s_fx, s_fy, s_sum);
  __shared__ ItemInfo s_it;
  __shared__ uint32_t s_gmax[2 * Shape<BX, BY>::kGroups];
  __shared__ float s_gsum[3 * Shape<BX, BY>::kGroups];
  __shared__ uint32_t s_ab[2];
  const int t = threadIdx.x;
  for (;;) {
    if (t == 0) {
      const uint32_t item = atomicAdd(&a.work->next, 1u);
      s_it.tile = 0xffffffffu;
      if (item < a.n_items) {
        const uint32_t tile = item_tile_of(a.item_tile, item);
        const TileDesc& T = a.tiles[tile];
        const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
        const TileCtl* ctl = T.ctl;
        s_it.tile = tile;
        s_it.by = local / T.blocks_x;
        s_it.bx = local - s_it.by * T.blocks_x;
        s_it.cur = ctl->cur;
        s_it.rec = ctl->rec;
        s_it.fold = local == 0u ? 1u : 0u;
        const float pa = __uint_as_float(ctl->prev_a), pb = __uint_as_float(ctl->prev_b);
        s_it.dt = choose_dt<FIXED>(pa, pb, T.cfl, T.cell_m, a.max_dt, ctl->ledger.remaining_s);
        const bool src = (T.flags & kFlagSource) != 0u;
        const bool on = src && (T.source_every <= 1u || ctl->src_phase + 1u == T.source_every);
        s_it.apply_source = on ? 1u : 0u;
        s_it.scale = T.source_every > 1u ? float(T.source_every) : 1.0f;
      }
    }
    __syncthreads();
    if (s_it.tile == 0xffffffffu) break;
    const ItemInfo it = s_it;
    const TileDesc& T = a.tiles[it.tile];
    if (it.fold) {
      // The ledger's fold of the last update's records (dt_main, slang:417-478).
      fold_sums(T.rec[it.rec], T.groups_x * T.groups_y, false, s_sum, s_ab, false);
      if (t == 0) {
        LedgerBits l = T.ctl->ledger;
        ledger_update<FIXED>(l, s_sum[0], s_sum[kThreads], s_sum[2 * kThreads],
                             __uint_as_float(T.ctl->prev_a), __uint_as_float(T.ctl->prev_b),
                             T.cfl, T.cell_m, a.max_dt);
        T.ctl->ledger_next = l;
      }
      __syncthreads();
    }
    uint32_t blk_a = 0u, blk_b = 0u;
    step_block<FIXED, MANNING, BX, BY>(T, it, a.max_dt, s_cell, s_fx, s_fy, s_sum, s_gmax, s_gsum,
                                      blk_a, blk_b);
    __threadfence();
    __syncthreads();
    if (t == 0) finish_item(T, blk_a, blk_b, true);
    __syncthreads();
  }
  if (t == 0) {
    __threadfence();
    if (atomicAdd(&a.work->exited, 1u) + 1u == gridDim.x) {
      a.work->next = 0u;
      a.work->exited = 0u;
      __threadfence();
    }
  }
}

// The records of a state written from the host (prime_main, slang:373-386): one CTA a block.
template <bool FIXED, int BX, int BY>
__global__ void __launch_bounds__(kThreads) prime_kernel(TickArgs a) {
  using S = Shape<BX, BY>;
  const uint32_t item = blockIdx.x;
  if (item >= a.n_items) return;
  __shared__ uint32_t s_gmax[2 * S::kGroups];
  __shared__ float s_gsum[3 * S::kGroups];
  const int t = threadIdx.x;
  const uint32_t tile = item_tile_of(a.item_tile, item);
  const TileDesc& T = a.tiles[tile];
  const uint32_t local = a.item_tile == nullptr ? item : item - T.item_base;
  const uint32_t by = local / T.blocks_x, bx = local - by * T.blocks_x;
  const uint32_t cur = T.ctl->cur, rec = T.ctl->rec;
  const float* in = T.state[cur];
  const size_t n = size_t(T.nx) * T.ny;
  if (t < 2 * S::kGroups) s_gmax[t] = 0u;
  const int c = t % BX, r0 = t / BX;
  const int gx = int(bx) * BX + c;
  uint32_t amax[BY / 16], bmax[BY / 16];
#pragma unroll
  for (int k = 0; k < BY / 16; ++k) amax[k] = bmax[k] = 0u;
#pragma unroll
  for (int k = 0; k < S::kPerThread; ++k) {
    const int r = r0 + k * S::kRowStep;
    const int gy = int(by) * BY + r;
    float ax = 0.0f, ay = 0.0f;
    if (gx < int(T.nx) && gy < int(T.ny)) {
      const size_t i = size_t(gy) * T.nx + gx;
      cell_speeds<FIXED>(T.gravity, T.dry, in[i], in[n + i], in[2 * n + i], ax, ay);
    }
    const int gr = (k * S::kRowStep) / 16;
    amax[gr] = max(amax[gr], __float_as_uint(ax));
    bmax[gr] = max(bmax[gr], __float_as_uint(ay));
  }
  __syncthreads();
  uint32_t blk_a = 0u, blk_b = 0u;
  // The prime's records carry no sums (no tree reads the per-cell sums): they go into the buffer
  // that holds the current records.
  write_records<BX, BY>(T, T.rec[rec], bx, by, s_gsum, s_gmax, s_gsum, amax, bmax, false, false,
                        false, blk_a, blk_b);
  __threadfence();
  __syncthreads();
  if (t == 0) finish_item(T, blk_a, blk_b, false);
}

// dt_main alone, on one tile (slang:412-479): a flush (max_dt 0) or the length pass. The records'
// sums are folded and cleared; the ledger is written in place.
template <bool FIXED>
__global__ void __launch_bounds__(kThreads) length_pass_kernel(const TileDesc* tiles, uint32_t tile,
                                                              float max_dt) {
  __shared__ float s[3 * kThreads];
  __shared__ uint32_t s_ab[2];
  const TileDesc& T = tiles[tile];
  Partial* rec = T.rec[T.ctl->rec];
  fold_sums(rec, T.groups_x * T.groups_y, true, s, s_ab, true);
  if (threadIdx.x == 0) {
    LedgerBits l = T.ctl->ledger;
    ledger_update<FIXED>(l, s[0], s[kThreads], s[2 * kThreads], __uint_as_float(s_ab[0]),
                         __uint_as_float(s_ab[1]), T.cfl, T.cell_m, max_dt);
    T.ctl->ledger = l;
  }
}

// ---- uploads and read-backs -------------------------------------------------------------------

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
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    LedgerBits empty = {};
    empty.remaining_s = __int_as_float(0x7f800000);
    T.ctl->ledger = empty;
    T.ctl->src_phase = 0u;
  }
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
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    LedgerBits empty = {};
    empty.remaining_s = __int_as_float(0x7f800000);
    T.ctl->ledger = empty;
    T.ctl->src_phase = 0u;
  }
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

// The tick kernels' shared-memory opt-in is set per device by tick_occupancy(), which the host
// calls when it creates a step, before any launch or capture.
template <int BX, int BY>
struct Launch {
  template <bool FIXED, bool MANNING>
  static cudaError_t tick(const TickArgs& a, int grid, cudaStream_t s) {
    tick_kernel<FIXED, MANNING, BX, BY><<<grid, kThreads, Shape<BX, BY>::kSmem, s>>>(a);
    return cudaGetLastError();
  }
};

}  // namespace

// ---- host-side launchers (wl_kernels.h) ---------------------------------------------------------

size_t tick_smem_bytes(BlockShape shape) {
  switch (shape) {
    case BlockShape::k32x16: return Shape<32, 16>::kSmem;
    case BlockShape::k32x32: return Shape<32, 32>::kSmem;
    case BlockShape::k64x32: return Shape<64, 32>::kSmem;
  }
  return 0;
}

void block_dims(BlockShape shape, uint32_t& bx, uint32_t& by) {
  switch (shape) {
    case BlockShape::k32x16: bx = 32; by = 16; return;
    case BlockShape::k32x32: bx = 32; by = 32; return;
    case BlockShape::k64x32: bx = 64; by = 32; return;
  }
  bx = by = 0;
}

template <int BX, int BY>
static const void* tick_fn(bool fixed, bool manning) {
  if (fixed) return manning ? (const void*)tick_kernel<true, true, BX, BY> : (const void*)tick_kernel<true, false, BX, BY>;
  return manning ? (const void*)tick_kernel<false, true, BX, BY> : (const void*)tick_kernel<false, false, BX, BY>;
}

int tick_occupancy(BlockShape shape, bool fixed, bool manning) {
  const void* fn = nullptr;
  size_t smem = tick_smem_bytes(shape);
  switch (shape) {
    case BlockShape::k32x16: fn = tick_fn<32, 16>(fixed, manning); break;
    case BlockShape::k32x32: fn = tick_fn<32, 32>(fixed, manning); break;
    case BlockShape::k64x32: fn = tick_fn<64, 32>(fixed, manning); break;
  }
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
    return 0;
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kThreads, smem) != cudaSuccess)
    return 0;
  return blocks;
}

cudaError_t launch_tick(BlockShape shape, bool fixed, bool manning, const TickArgs& a, int grid,
                        cudaStream_t s) {
  switch (shape) {
#define WLC_TICK(BX, BY)                                                          \
  case BlockShape::k##BX##x##BY:                                                  \
    if (fixed) return manning ? Launch<BX, BY>::tick<true, true>(a, grid, s)      \
                              : Launch<BX, BY>::tick<true, false>(a, grid, s);    \
    return manning ? Launch<BX, BY>::tick<false, true>(a, grid, s)                \
                   : Launch<BX, BY>::tick<false, false>(a, grid, s);
    WLC_TICK(32, 16)
    WLC_TICK(32, 32)
    WLC_TICK(64, 32)
#undef WLC_TICK
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_prime(BlockShape shape, bool fixed, const TickArgs& a, cudaStream_t s) {
  if (a.n_items == 0) return cudaSuccess;
  switch (shape) {
#define WLC_PRIME(BX, BY)                                                        \
  case BlockShape::k##BX##x##BY:                                                 \
    if (fixed) prime_kernel<true, BX, BY><<<a.n_items, kThreads, 0, s>>>(a);     \
    else prime_kernel<false, BX, BY><<<a.n_items, kThreads, 0, s>>>(a);          \
    return cudaGetLastError();
    WLC_PRIME(32, 16)
    WLC_PRIME(32, 32)
    WLC_PRIME(64, 32)
#undef WLC_PRIME
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_length_pass(bool fixed, const TileDesc* tiles, uint32_t tile, float max_dt,
                               cudaStream_t s) {
  if (fixed) length_pass_kernel<true><<<1, kThreads, 0, s>>>(tiles, tile, max_dt);
  else length_pass_kernel<false><<<1, kThreads, 0, s>>>(tiles, tile, max_dt);
  return cudaGetLastError();
}

static int grid_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return int(b < 4096 ? (b == 0 ? 1 : b) : 4096);
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

}  // namespace wlc

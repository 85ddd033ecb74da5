// Device-side arithmetic and layout of the live-water tick (sm_103a).
//
// The scheme is the reference's (systems/water_live/shaders/water_step.slang, and its FP64 twin
// domain/water_state/src/water_state.cpp): the hydrostatic reconstruction over the central-upwind
// flux on h, hu, hv. Every expression below keeps the reference's operand order. The translation
// unit is compiled with --fmad=false -prec-div=true -prec-sqrt=true -ftz=false, and division and
// square root are spelled with the _rn intrinsics, so each + - * / sqrt is one correctly rounded
// IEEE operation whatever the flags, and the bytes equal the CPU restatement's.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace wlc {

constexpr uint32_t kFlagWestOpen = 1u;  // water_live.h:90-97
constexpr uint32_t kFlagEastOpen = 2u;
constexpr uint32_t kFlagSouthOpen = 4u;
constexpr uint32_t kFlagNorthOpen = 8u;
constexpr uint32_t kFlagManning = 16u;
constexpr uint32_t kFlagSource = 32u;
constexpr uint32_t kFlagCompensate = 64u;
constexpr uint32_t kFlagStoredFaces = 128u;
// The flags the march's plain variant compiles out (it runs where no tile holds one).
constexpr uint32_t kFlagsNotPlain = kFlagWestOpen | kFlagEastOpen | kFlagSouthOpen |
                                    kFlagNorthOpen | kFlagManning | kFlagCompensate;
constexpr uint32_t kGroupSide = 16u;
constexpr uint32_t kGroupCells = 256u;
constexpr uint32_t kStatePlanes = 4u;
// The largest tile: the kernels index a tile's cells, and its planes' cells, in 32 bits.
constexpr uint64_t kMaxTileCells = uint64_t(1) << 30;
constexpr int kThreads = 256;  // one CTA: 8 warps; also the length pass's 256 lanes

// water_live::WaterPartial (water_live.h:114-121).
struct Partial {
  float speed_x, speed_y, source_m3, open_m3, roundoff_m3, pad0, pad1, pad2;
};
static_assert(sizeof(Partial) == 32, "WaterPartial is 32 bytes");

// water_live::WaterLedger (water_live.h:124-137).
struct LedgerBits {
  float time_hi, time_lo, source_hi, source_lo, open_hi, open_lo, roundoff_hi, roundoff_lo;
  float remaining_s, dt;
  uint32_t steps, pad;
};
static_assert(sizeof(LedgerBits) == 48, "WaterLedger is 48 bytes");

// A tile's control block, all of a tick's state that is not a plane: the ledger as the reference
// keeps it, which copy holds the state, which record buffer holds the last update's records, the
// largest speeds of each record buffer's update (the next step's length is chosen from them), and
// the source's clock. Every launch reads it and the tile's last work item flips it, so a captured
// graph of ticks replays correctly any number of times.
//
// The ledger and the largest speeds come in two slots indexed like the record buffers. A launch
// reads slot `rec` and writes slot `rec ^ 1` (the ledger by the tile's first item, the speeds by
// every item's atomicMax), and the last item flips `rec`. Nothing a launch writes is read in the
// same launch, so no item orders its writes before its `done` count: the next launch sees them
// all at the kernel boundary. Between launches the speeds of slot `rec ^ 1` are zero; the last
// item keeps that true by clearing slot `rec` (every item of the tile has read it by then).
struct TileCtl {
  LedgerBits ledger[2];  // 0, 48: the ledger; ledger[rec] is the current one
  uint32_t cur;          // 96: the copy that holds the state
  uint32_t rec;          // 100: the record buffer that holds the last update's records
  uint32_t max_a[2];     // 104: largest |u| + c of the update whose records are rec[k] (bits)
  uint32_t max_b[2];     // 112: largest |v| + c
  uint32_t done;         // 120: work items of this tile finished in this launch
  uint32_t src_phase;    // 124: steps since the source last applied (set_source's clock)
  uint32_t error;        // 128: a device error word (0: none)
  uint32_t ticks;        // 132: launches that stepped this tile (a diagnosis counter)
  uint32_t pad[2];
};
static_assert(sizeof(TileCtl) == 144, "TileCtl layout");

// One rectangle of water as the kernels see it. The planes are the reference's layout: a copy is
// four planes of nx * ny floats (h, hu, hv, remainder), cell (x, y) at y * nx + x.
struct TileDesc {
  float* state[2];
  const float* bed;
  const float* manning;
  const float* source;
  Partial* rec[2];
  TileCtl* ctl;
  uint32_t nx, ny, groups_x, groups_y;
  uint32_t flags;         // kFlag* for this tile (edges, Manning, source, compensate)
  uint32_t source_every;  // set_source's clock
  float cell_m, gravity, cfl, dry;
  uint32_t blocks_x, blocks_y;  // work items: blocks of the launch's block shape
  uint32_t item_base, items;
  // The block tick's tensor maps (three of 128 bytes: state copy 0's and copy 1's {h, hu, hv},
  // then the bed), or null where the tile's rows do not start on 16-byte boundaries.
  const void* tmap;
};

// A launch's dynamic work counter: CTAs take work items in order; the last CTA to leave resets it.
struct WorkCtl {
  uint32_t next;    // whole items dealt
  uint32_t exited;  // warps (or CTAs) that left
  uint32_t tail;    // the 32 x 16 march's last items dealt, a CTA at a time
  uint32_t fault;   // the staged block tick: nonzero where a CTA's wait on its copies gave up
};

// The resident tick's words (one a tile set, zeroed before each resident launch): the grid
// barrier's arrivals (a CTA adds one a tick) and its error word, and three rotating slots of what a
// tick reads from the last one: the largest speeds of its update and the ledger's time left. In
// three slots nothing waits at the barrier for a slot to be cleared, and a tick reads its slot in
// one 16-byte load.
struct ResidentSlot {
  uint32_t max_a, max_b;
  float remaining_s;
  uint32_t pad;
};
struct ResidentCtl {
  uint32_t arrived;
  uint32_t error;
  uint32_t pad[2];
  ResidentSlot slot[3];
};
static_assert(sizeof(ResidentCtl) == 64, "ResidentCtl layout");

// ---- dependent launches ---------------------------------------------------------------------
//
// The tick, the queue's slot and the adjoint's sweeps are launched as programmatic dependents of
// the launch before them on their stream: their CTAs may be scheduled while that grid's last CTAs
// finish. griddepcontrol.wait returns once the grid before has completed and its writes are
// visible, so nothing such a kernel reads is read before it; the kernel then lets the grid after it
// be scheduled, which waits the same way. At most two such grids are resident at once, and a
// launch before which nothing signals (an ordinary kernel, a copy) is waited for in full.
__device__ __forceinline__ void dependent_grid_start() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... Params, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem,
                                    cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// ---- the arithmetic (water_step.slang:105-191) -------------------------------------------------

__device__ __forceinline__ float max2(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float min2(float a, float b) { return a < b ? a : b; }

// rcp_fixed (slang:112-124).
__device__ __forceinline__ float rcp_fixed(float x) {
  const uint32_t bits = __float_as_uint(x);
  if (bits >= 0x7e800000u) return 0.0f;
  if (bits < 0x00800000u) return __uint_as_float(0x7f7fffffu);
  float r = __uint_as_float(0x7ef311c3u - bits);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float t = __fmul_rn(x, r);
    const float e = __fsub_rn(2.0f, t);
    r = __fmul_rn(r, e);
  }
  return r;
}

// rsqrt_fixed (slang:128-139).
__device__ __forceinline__ float rsqrt_fixed(float x) {
  float y = __uint_as_float(0x5f375a86u - (__float_as_uint(x) >> 1));
  const float half_x = __fmul_rn(0.5f, x);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float yy = __fmul_rn(y, y);
    const float t = __fmul_rn(half_x, yy);
    const float e = __fsub_rn(1.5f, t);
    y = __fmul_rn(y, e);
  }
  return y;
}

// cbrt_fixed (slang:143-154); 1.0 / 3.0 folds to the float nearest a third.
__device__ __forceinline__ float cbrt_fixed(float h) {
  float x = __uint_as_float(__float_as_uint(h) / 3u + 709921077u);
  const float third = 0.333333343267f;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float xx = __fmul_rn(x, x);
    const float q = __fmul_rn(h, rcp_fixed(xx));
    const float twice = __fadd_rn(x, x);
    const float s = __fadd_rn(twice, q);
    x = __fmul_rn(s, third);
  }
  return x;
}

// The two forms of the arithmetic (water_live.h:57-62). Native: IEEE division and square root.
// Both forms take the cube root from the fixed construction (the shader's native log2/exp2 is not
// reproducible on any two devices, nor against a CPU).
template <bool FIXED>
struct Ops {
  static __device__ __forceinline__ float div(float a, float b) {
    if (FIXED) {
      if (a == 0.0f) return a;
      return __fmul_rn(a, rcp_fixed(b));
    }
    return __fdiv_rn(a, b);
  }
  static __device__ __forceinline__ float sqrt(float x) {
    if (FIXED) {
      if (__float_as_uint(x) < 0x00800000u) return 0.0f;
      return __fmul_rn(x, rsqrt_fixed(x));
    }
    return __fsqrt_rn(x);
  }
  static __device__ __forceinline__ float cbrt(float h) { return cbrt_fixed(h); }
};

// The quotient and the root with zero taken apart (ZG): sqrt(+-0) is +-0 and 0 / b is 0 with a's
// sign for b > 0, the same bits, without the intrinsics' slow path that a zero argument takes. A
// tick where many arguments are zero (a still column, a wet/dry front) runs faster; elsewhere the
// tests cost a little (the plain tick keeps the bare intrinsics).
template <bool FIXED, bool ZG>
__device__ __forceinline__ float zsqrt(float x) {
  if (!ZG) return Ops<FIXED>::sqrt(x);
  const float r = Ops<FIXED>::sqrt(x == 0.0f ? 1.0f : x);
  return x == 0.0f ? x : r;
}
template <bool FIXED, bool ZG>
__device__ __forceinline__ float zdiv(float a, float b) {
  if (!ZG) return Ops<FIXED>::div(a, b);
  const bool zero = a == 0.0f && b > 0.0f;
  const float q = Ops<FIXED>::div(zero ? 1.0f : a, b);
  return zero ? a : q;
}

// pressure (slang:186-191): (0.5 g) h h.
__device__ __forceinline__ float pressure(float half_g, float h) {
  return __fmul_rn(__fmul_rn(half_g, h), h);
}

// face (slang:274-292) over face_flux (slang:204-262): the face's bed the larger of the two, each
// side reconstructed against it, the central-upwind flux between them, and the normal momentum's
// flux less each side's pressure. Returns {h, nl, nr, t}.
template <bool FIXED, bool ZG = false>
__device__ __forceinline__ float4 face(float g, float half_g, float hl0, float zl, float ul,
                                       float vl, float hr0, float zr, float ur, float vr) {
  const float zf = max2(zl, zr);
  const float el = __fsub_rn(__fadd_rn(hl0, zl), zf);
  const float er = __fsub_rn(__fadd_rn(hr0, zr), zf);
  const float hl = el > 0.0f ? el : 0.0f;
  const float hr = er > 0.0f ? er : 0.0f;
  const float pl = pressure(half_g, hl);
  const float pr = pressure(half_g, hr);
  float fh, fn, ft;
  if (hl == hr && ul == ur && vl == vr) {
    const float q = __fmul_rn(hl, ul);
    fh = q;
    fn = __fadd_rn(__fmul_rn(q, ul), pl);
    ft = __fmul_rn(q, vl);
  } else {
    const float cl = zsqrt<FIXED, ZG>(__fmul_rn(g, hl));
    const float cr = zsqrt<FIXED, ZG>(__fmul_rn(g, hr));
    const float ap = max2(max2(__fadd_rn(ur, cr), __fadd_rn(ul, cl)), 0.0f);
    const float am = min2(min2(__fsub_rn(ur, cr), __fsub_rn(ul, cl)), 0.0f);
    const float span = __fsub_rn(ap, am);
    if (!(span > 0.0f)) {
      fh = 0.0f;
      fn = 0.0f;
      ft = 0.0f;
    } else {
      const float ql = __fmul_rn(hl, ul);
      const float qr = __fmul_rn(hr, ur);
      const float apam = __fmul_rn(ap, am);
      const float h6 = __fadd_rn(__fsub_rn(__fmul_rn(ap, ql), __fmul_rn(am, qr)),
                                 __fmul_rn(apam, __fsub_rn(hr, hl)));
      const float n2 = __fadd_rn(__fmul_rn(ql, ul), pl);
      const float n5 = __fadd_rn(__fmul_rn(qr, ur), pr);
      const float n10 = __fadd_rn(__fsub_rn(__fmul_rn(ap, n2), __fmul_rn(am, n5)),
                                  __fmul_rn(apam, __fsub_rn(qr, ql)));
      const float t7 = __fsub_rn(__fmul_rn(hr, vr), __fmul_rn(hl, vl));
      const float t10 = __fadd_rn(__fsub_rn(__fmul_rn(ap, __fmul_rn(ql, vl)),
                                            __fmul_rn(am, __fmul_rn(qr, vr))),
                                  __fmul_rn(apam, t7));
      fh = zdiv<FIXED, ZG>(h6, span);
      fn = zdiv<FIXED, ZG>(n10, span);
      ft = zdiv<FIXED, ZG>(t10, span);
    }
  }
  return make_float4(fh, __fsub_rn(fn, pl), __fsub_rn(fn, pr), ft);
}

// |u| + c and |v| + c (slang:317-326).
template <bool FIXED, bool ZG = false>
__device__ __forceinline__ void cell_speeds(float g, float dry, float h, float hu, float hv,
                                            float& ax, float& ay) {
  using O = Ops<FIXED>;
  const bool wet = h >= dry;
  const float u = wet ? zdiv<FIXED, ZG>(hu, h) : 0.0f;
  const float v = wet ? zdiv<FIXED, ZG>(hv, h) : 0.0f;
  // sqrt(+-0) is +-0: a dry cell's zero takes no square root (the intrinsic's special-case path
  // is its slow one, and most cells of a dry landscape are exactly zero).
  const float gh = __fmul_rn(g, h);
  const float c = gh == 0.0f ? gh : O::sqrt(gh);
  ax = __fadd_rn(fabsf(u), c);
  ay = __fadd_rn(fabsf(v), c);
}

// pair_add (slang:391-404): TwoSum, then Fast2Sum.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float sa = __fsub_rn(s, bb);
  const float da = __fsub_rn(hi, sa);
  const float db = __fsub_rn(x, bb);
  const float e = __fadd_rn(da, db);
  const float l = __fadd_rn(lo, e);
  const float h2 = __fadd_rn(s, l);
  const float back = __fsub_rn(h2, s);
  const float l2 = __fsub_rn(l, back);
  hi = h2;
  lo = l2;
}

// The step's length (slang:464-474) from the last update's largest speeds and the time left.
template <bool FIXED>
__device__ __forceinline__ float choose_dt(float a, float b, float cfl, float cell_m,
                                           float max_dt, float remaining) {
  if (!(max_dt > 0.0f)) return 0.0f;
  const float speed = __fadd_rn(a, b);
  const float reach = __fmul_rn(cfl, cell_m);
  const float stable = speed > 0.0f ? Ops<FIXED>::div(reach, speed) : __int_as_float(0x7f800000);
  float dt = min2(stable, max_dt);
  dt = min2(dt, remaining);
  return dt;
}

}  // namespace wlc

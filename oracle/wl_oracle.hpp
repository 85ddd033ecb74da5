// ORACLE — test infrastructure only. Nothing in the product links, loads or calls this code: only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the checker.
//
// A CPU restatement of the reference's live-water tick, written from the reference's sources:
//
//   RefStep<T>   the card's step, systems/water_live/shaders/water_step.slang, operation for
//                operation (T = float is the FP32 oracle the CUDA path is held to bit for bit;
//                T = double is its FP64 twin), with the host half of
//                systems/water_live/src/water_live.cpp (create, write_state, set_bed, set_source's
//                clock, record, read_ledger's flush, advance, run_length_pass, state_hash).
//   Solver64     the reference CPU tick, domain/water_state/src/water_state.cpp (Solver::step,
//                advance, state_hash), restricted to depth and momenta (no ground store, no
//                carried quantities, no per-cell outputs), rows dealt to threads like the
//                reference's JobSystem (the bytes do not depend on the thread count).
//
// Parity of the oracle itself is pinned, not assumed:
//   - Solver64 reproduces the reference's cross-toolchain pin for Stoker's dam break at 800 cells
//     (domain/water_state/tests/water_state_tests.cpp:776-789, hash 11759616244214831310), and
//     equals the reference's own compiled Solver byte for byte on the cases in
//     tests/test_oracle_ref.py (oracle/_ref, built from the reference's sources by
//     oracle/build_ref.sh, in the container that has them).
//   - RefStep<double> equals Solver64 byte for byte (Manning off: the reference's FP64 cube root
//     comes from its fdlibm port, not restated here).
//   - RefStep<float> reproduces the exact lake's published hash (557 steps, 6248193821885885893,
//     docs/subsystems/water_live.md:40) and the reference's bounded cases against Solver64.
//
// Compile with -ffp-contract=off and without -ffast-math: every + - * / and sqrt below must be one
// correctly rounded IEEE operation, as the reference's no-contraction policy requires
// (cmake/EngineFpContraction.cmake:57-62).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace wl_oracle {

using u8 = std::uint8_t;
using u32 = std::uint32_t;
using u64 = std::uint64_t;

// water_live.h:90-97
constexpr u32 k_flag_west_open = 1u;
constexpr u32 k_flag_east_open = 2u;
constexpr u32 k_flag_south_open = 4u;
constexpr u32 k_flag_north_open = 8u;
constexpr u32 k_flag_manning = 16u;
constexpr u32 k_flag_source = 32u;
constexpr u32 k_flag_compensate = 64u;
constexpr u32 k_flag_stored_faces = 128u;
constexpr u32 k_group_side = 16u;    // water_live.h:140
constexpr u32 k_group_cells = 256u;  // water_step.slang:101
constexpr u32 k_state_planes = 4u;   // water_live.h:102

constexpr u64 k_fnv_offset = 0xcbf29ce484222325ull;  // water_live.cpp:22
constexpr u64 k_fnv_prime = 0x100000001b3ull;        // water_live.cpp:23

// FNV-1a over float bytes, low byte first (water_live.cpp:90-101).
inline u64 hash_floats(const float* v, size_t n, u64 hash = k_fnv_offset) {
  for (size_t i = 0; i < n; ++i) {
    u32 bits;
    std::memcpy(&bits, v + i, 4);
    for (u32 b = 0; b < 4; ++b) {
      hash ^= (bits >> (8 * b)) & 0xffu;
      hash *= k_fnv_prime;
    }
  }
  return hash;
}

// FNV-1a over double bytes (water_state.cpp:99-109).
inline u64 hash_doubles(const double* v, size_t n, u64 hash = k_fnv_offset) {
  for (size_t i = 0; i < n; ++i) {
    u64 bits;
    std::memcpy(&bits, v + i, 8);
    for (u32 b = 0; b < 8; ++b) {
      hash ^= (bits >> (8 * b)) & 0xffu;
      hash *= k_fnv_prime;
    }
  }
  return hash;
}

// The reference's ternary maximum and minimum (water_state.cpp:41-49). The shader's max/min agree
// with them on every value the step produces (no NaN; speeds are never -0).
template <class T>
inline T max2(T a, T b) { return a > b ? a : b; }
template <class T>
inline T min2(T a, T b) { return a < b ? a : b; }

inline float asfloat(u32 b) { float f; std::memcpy(&f, &b, 4); return f; }
inline u32 asuint(float f) { u32 b; std::memcpy(&b, &f, 4); return b; }

// ---- the arithmetic (water_step.slang:105-191) -------------------------------------------------

// rcp_fixed (slang:112-124): the bits' estimate and four Newton steps.
inline float rcp_fixed(float x) {
  const u32 bits = asuint(x);
  if (bits >= 0x7e800000u) return 0.0f;
  if (bits < 0x00800000u) return asfloat(0x7f7fffffu);
  float r = asfloat(0x7ef311c3u - bits);
  for (int i = 0; i < 4; ++i) {
    const float t = x * r;
    const float e = 2.0f - t;
    r = r * e;
  }
  return r;
}

// rsqrt_fixed (slang:128-139).
inline float rsqrt_fixed(float x) {
  float y = asfloat(0x5f375a86u - (asuint(x) >> 1));
  const float half_x = 0.5f * x;
  for (int i = 0; i < 3; ++i) {
    const float yy = y * y;
    const float t = half_x * yy;
    const float e = 1.5f - t;
    y = y * e;
  }
  return y;
}

// cbrt_fixed (slang:143-154). 1.0 / 3.0 folds to the float nearest a third.
inline float cbrt_fixed(float h) {
  float x = asfloat(asuint(h) / 3u + 709921077u);
  const float third = static_cast<float>(1.0 / 3.0);
  for (int i = 0; i < 4; ++i) {
    const float xx = x * x;
    const float q = h * rcp_fixed(xx);
    const float twice = x + x;
    const float s = twice + q;
    x = s * third;
  }
  return x;
}

// The two forms of the arithmetic (water_live.h:62). `native` takes IEEE division and square root;
// its cube root is cbrt_fixed (the shader's native form takes log2/exp2, which no two devices
// round alike; the CUDA path and this oracle both take the reference's fixed construction).
template <class T>
struct Ops {
  bool fixed = false;
  T div(T a, T b) const { return a / b; }
  T sqrt(T x) const { return std::sqrt(x); }
  T cbrt(T h) const { return std::cbrt(h); }
};

template <>
struct Ops<float> {
  bool fixed = false;
  float div(float a, float b) const {
    if (fixed) {
      if (a == 0.0f) return a;
      return a * rcp_fixed(b);
    }
    return a / b;
  }
  float sqrt(float x) const {
    if (fixed) {
      if (asuint(x) < 0x00800000u) return 0.0f;
      return x * rsqrt_fixed(x);
    }
    return std::sqrt(x);
  }
  float cbrt(float h) const { return cbrt_fixed(h); }
};

template <class T>
inline T pressure(T g, T h) {  // slang:186-191, water_state.cpp:39
  const T a = T(0.5) * g;
  const T b = a * h;
  return b * h;
}

template <class T>
struct Flux { T h, n, t; };

// face_flux (slang:204-262; water_state.cpp:67-90 without the energy's component).
template <class T>
inline Flux<T> face_flux(const Ops<T>& ops, T g, T hl, T ul, T vl, T hr, T ur, T vr) {
  if (hl == hr && ul == ur && vl == vr) {
    const T q = hl * ul;
    const T qu = q * ul;
    const T n = qu + pressure(g, hl);
    const T t = q * vl;
    return {q, n, t};
  }
  const T gl = g * hl;
  const T gr = g * hr;
  const T cl = ops.sqrt(gl);
  const T cr = ops.sqrt(gr);
  const T ap = max2(max2(ur + cr, ul + cl), T(0));
  const T am = min2(min2(ur - cr, ul - cl), T(0));
  const T span = ap - am;
  if (!(span > T(0))) return {T(0), T(0), T(0)};
  const T ql = hl * ul;
  const T qr = hr * ur;
  const T apam = ap * am;
  const T h1 = ap * ql;
  const T h2 = am * qr;
  const T h3 = hr - hl;
  const T h4 = apam * h3;
  const T h5 = h1 - h2;
  const T h6 = h5 + h4;
  const T n1 = ql * ul;
  const T n2 = n1 + pressure(g, hl);
  const T n3 = ap * n2;
  const T n4 = qr * ur;
  const T n5 = n4 + pressure(g, hr);
  const T n6 = am * n5;
  const T n7 = qr - ql;
  const T n8 = apam * n7;
  const T n9 = n3 - n6;
  const T n10 = n9 + n8;
  const T t1 = ql * vl;
  const T t2 = ap * t1;
  const T t3 = qr * vr;
  const T t4 = am * t3;
  const T t5 = hr * vr;
  const T t6 = hl * vl;
  const T t7 = t5 - t6;
  const T t8 = apam * t7;
  const T t9 = t2 - t4;
  const T t10 = t9 + t8;
  return {ops.div(h6, span), ops.div(n10, span), ops.div(t10, span)};
}

template <class T>
struct Face { T h, nl, nr, t; };

// face (slang:274-292; water_state.cpp:231-257).
template <class T>
inline Face<T> face(const Ops<T>& ops, T g, T hl0, T zl, T ln, T lt, T hr0, T zr, T rn, T rt) {
  const T zf = max2(zl, zr);
  const T sl = hl0 + zl;
  const T el = sl - zf;
  const T sr = hr0 + zr;
  const T er = sr - zf;
  const T hl = el > T(0) ? el : T(0);
  const T hr = er > T(0) ? er : T(0);
  const Flux<T> f = face_flux(ops, g, hl, ln, lt, hr, rn, rt);
  return {f.h, f.n - pressure(g, hl), f.n - pressure(g, hr), f.t};
}

// ---- the card's step (water_step.slang) --------------------------------------------------------

template <class T>
struct Partial { T speed_x = 0, speed_y = 0, source_m3 = 0, open_m3 = 0, roundoff_m3 = 0, pad[3] = {0, 0, 0}; };

template <class T>
struct LedgerBits {
  T time_hi = 0, time_lo = 0, source_hi = 0, source_lo = 0, open_hi = 0, open_lo = 0,
    roundoff_hi = 0, roundoff_lo = 0;
  T remaining_s = 0;
  T dt = 0;
  u32 steps = 0;
  u32 pad = 0;
};

struct LedgerF64 {  // water_live.h:143-150
  double source_m3 = 0, open_edge_out_m3 = 0, roundoff_m3 = 0, time_s = 0, remaining_s = 0;
  u64 steps = 0;
};

// pair_add (slang:391-404): Knuth's TwoSum, then Fast2Sum.
template <class T>
inline void pair_add(T& hi, T& lo, T x) {
  const T s = hi + x;
  const T bb = s - hi;
  const T sa = s - bb;
  const T da = hi - sa;
  const T db = x - bb;
  const T e = da + db;
  const T l = lo + e;
  const T h2 = s + l;
  const T back = h2 - s;
  const T l2 = l - back;
  hi = h2;
  lo = l2;
}

struct Config {  // water_state.h:83-99, the fields the card reads
  u32 nx = 0, ny = 0;
  double cell_m = 1.0, gravity = 9.81, cfl = 0.45, dry_depth_m = 1e-9;
  u8 west_open = 0, east_open = 0, south_open = 0, north_open = 0;
};

// One rectangle on the "card": systems/water_live's DeviceStep with its shader, on the CPU.
template <class T>
class RefStep {
 public:
  struct Cell { T h, u, v, z; };

  bool create(const Config& c, bool fixed_ops) {
    if (c.nx == 0 || c.ny == 0) return false;  // water_live.cpp:108
    cfg = c;
    ops.fixed = fixed_ops;
    n = size_t(c.nx) * c.ny;
    gx = (c.nx + k_group_side - 1) / k_group_side;
    gy = (c.ny + k_group_side - 1) / k_group_side;
    flags = 0;
    if (c.west_open) flags |= k_flag_west_open;
    if (c.east_open) flags |= k_flag_east_open;
    if (c.south_open) flags |= k_flag_south_open;
    if (c.north_open) flags |= k_flag_north_open;
    for (auto& s : state) s.assign(k_state_planes * n, T(0));
    bed.assign(n, T(0));
    manning.assign(n, T(0));
    source.assign(n, T(0));
    partials.assign(size_t(gx) * gy, Partial<T>{});
    ledger = LedgerBits<T>{};
    ledger.remaining_s = std::numeric_limits<T>::infinity();
    cur = 0;
    source_every = 1;
    source_phase = 0;
    cell_m = T(c.cell_m);
    g = T(c.gravity);
    cfl = T(c.cfl);
    dry = T(c.dry_depth_m);
    prime();
    return true;
  }

  // write_state (water_live.cpp:271-314): rounded to T, plane 3 zero, ledger emptied, primed.
  void write_state(const double* h, const double* hu, const double* hv) {
    T* p = state[cur].data();
    for (size_t i = 0; i < n; ++i) {
      p[i] = T(h[i]);
      p[n + i] = T(hu[i]);
      p[2 * n + i] = T(hv[i]);
      p[3 * n + i] = T(0);
    }
    source_phase = 0;
    ledger = LedgerBits<T>{};
    ledger.remaining_s = std::numeric_limits<T>::infinity();
    prime();
  }

  // set_bed (water_live.cpp:439-447): the datum subtracted in double, rounded once.
  void set_bed(const double* b, double datum) {
    for (size_t i = 0; i < n; ++i) bed[i] = T(b[i] - datum);
  }
  void set_manning(const double* m) {  // water_live.cpp:449-463
    if (m == nullptr) { flags &= ~k_flag_manning; return; }
    for (size_t i = 0; i < n; ++i) manning[i] = T(m[i]);
    flags |= k_flag_manning;
  }
  void set_source(const double* s, u32 every, bool compensate) {  // water_live.cpp:465-486
    source_every = every == 0 ? 1 : every;
    source_phase = 0;
    if (compensate) flags |= k_flag_compensate; else flags &= ~k_flag_compensate;
    if (s == nullptr) { flags &= ~k_flag_source; return; }
    for (size_t i = 0; i < n; ++i) source[i] = T(s[i]);
    flags |= k_flag_source;
  }

  // record (water_live.cpp:488-568): per step the length pass and the update, the source's clock.
  void run_steps(u32 count, T max_dt) {
    for (u32 s = 0; s < count; ++s) {
      u32 f = flags;
      T scale = T(1);
      if ((flags & k_flag_source) != 0u && source_every > 1) {
        source_phase += 1;
        if (source_phase == source_every) {
          source_phase = 0;
          scale = T(source_every);
        } else {
          f &= ~k_flag_source;
        }
      }
      dt_main(max_dt);
      update(f, scale);
      cur ^= 1u;
    }
  }

  // read_ledger (water_live.cpp:349-381): a flush, then the pairs widened.
  LedgerF64 read_ledger() {
    dt_main(T(0));
    LedgerF64 o;
    o.source_m3 = double(ledger.source_hi) + double(ledger.source_lo);
    o.open_edge_out_m3 = double(ledger.open_hi) + double(ledger.open_lo);
    o.roundoff_m3 = double(ledger.roundoff_hi) + double(ledger.roundoff_lo);
    o.time_s = double(ledger.time_hi) + double(ledger.time_lo);
    o.remaining_s = double(ledger.remaining_s);
    o.steps = ledger.steps;
    return o;
  }

  void run_length_pass(T max_dt) { dt_main(max_dt); }  // water_live.cpp:415-437
  // prime_main (slang:373-386) of the state as it stands: the records of a state just written.
  void prime_records() { prime(); }

  // advance (water_live.cpp:594-632): batches of 64 steps of unlimited length until the time
  // kept in T has run out; the steps after it choose a length of zero.
  u64 advance(double duration_s, bool* refused = nullptr) {
    if (refused) *refused = false;
    if (!(duration_s > 0.0)) return 0;
    if ((flags & k_flag_source) != 0u && source_every > 1) {
      if (refused) *refused = true;
      return 0;
    }
    const LedgerF64 start = read_ledger();
    ledger.remaining_s = T(duration_s);
    bool done = false;
    for (u32 batch = 0; batch < (1u << 16) && !done; ++batch) {
      run_steps(64, std::numeric_limits<T>::infinity());
      const LedgerF64 now = read_ledger();
      done = !(now.remaining_s > 0.0);
    }
    const LedgerF64 end = read_ledger();
    ledger.remaining_s = std::numeric_limits<T>::infinity();
    if (!done) return 0;
    return end.steps - start.steps;
  }

  const T* planes() const { return state[cur].data(); }
  T* planes_mut() { return state[cur].data(); }
  u64 state_hash() const;  // float instantiation only

  Config cfg;
  Ops<T> ops;
  size_t n = 0;
  u32 gx = 0, gy = 0, flags = 0, cur = 0, source_every = 1, source_phase = 0;
  T cell_m = 1, g = 9.81, cfl = 0.45, dry = 1e-9;
  std::vector<T> state[2];
  std::vector<T> bed, manning, source;
  std::vector<Partial<T>> partials;
  LedgerBits<T> ledger;

 private:
  Cell load_cell(const T* s, size_t i) const {  // slang:303-314
    Cell c;
    c.h = s[i];
    const bool wet = c.h >= dry;
    c.u = wet ? ops.div(s[n + i], c.h) : T(0);
    c.v = wet ? ops.div(s[2 * n + i], c.h) : T(0);
    c.z = bed[i];
    return c;
  }

  void cell_speeds(T h, T hu, T hv, T& ax, T& ay) const {  // slang:317-326
    const bool wet = h >= dry;
    const T u = wet ? ops.div(hu, h) : T(0);
    const T v = wet ? ops.div(hv, h) : T(0);
    const T gh = g * h;
    const T c = ops.sqrt(gh);
    ax = std::fabs(u) + c;
    ay = std::fabs(v) + c;
  }

  // The records of one update or prime: a fixed 256-slot tree per 16 x 16 group (slang:338-371).
  struct Slots {
    std::vector<T> sx, sy, src, opn, rnd;
    explicit Slots(size_t groups)
        : sx(groups * k_group_cells, T(0)), sy(sx), src(sx), opn(sx), rnd(sx) {}
  };

  void write_partials(Slots& s) {
    const size_t groups = size_t(gx) * gy;
    for (size_t grp = 0; grp < groups; ++grp) {
      T* a = &s.sx[grp * k_group_cells];
      T* b = &s.sy[grp * k_group_cells];
      T* c = &s.src[grp * k_group_cells];
      T* d = &s.opn[grp * k_group_cells];
      T* e = &s.rnd[grp * k_group_cells];
      for (u32 stride = k_group_cells / 2u; stride > 0u; stride >>= 1u) {
        for (u32 l = 0; l < stride; ++l) {
          a[l] = max2(a[l], a[l + stride]);
          b[l] = max2(b[l], b[l + stride]);
          c[l] = c[l] + c[l + stride];
          d[l] = d[l] + d[l + stride];
          e[l] = e[l] + e[l + stride];
        }
      }
      Partial<T> p;
      p.speed_x = a[0];
      p.speed_y = b[0];
      p.source_m3 = c[0];
      p.open_m3 = d[0];
      p.roundoff_m3 = e[0];
      partials[grp] = p;
    }
  }

  size_t slot(u32 x, u32 y) const {
    const size_t group = size_t(y / k_group_side) * gx + x / k_group_side;
    return group * k_group_cells + (y % k_group_side) * k_group_side + (x % k_group_side);
  }

  void prime() {  // slang:373-386
    Slots s(size_t(gx) * gy);
    const T* st = state[cur].data();
    for (u32 y = 0; y < cfg.ny; ++y)
      for (u32 x = 0; x < cfg.nx; ++x) {
        const size_t i = size_t(y) * cfg.nx + x;
        T ax, ay;
        cell_speeds(st[i], st[n + i], st[2 * n + i], ax, ay);
        s.sx[slot(x, y)] = ax;
        s.sy[slot(x, y)] = ay;
      }
    write_partials(s);
  }

  // dt_main (slang:412-479): 256 lanes, each a strided pass over the records, then a fixed tree.
  void dt_main(T max_dt) {
    T a[k_group_cells], b[k_group_cells], src[k_group_cells], opn[k_group_cells],
        rnd[k_group_cells];
    const u32 groups = gx * gy;
    for (u32 t = 0; t < k_group_cells; ++t) {
      T la = 0, lb = 0, ls = 0, lo = 0, lr = 0;
      for (u32 gi = t; gi < groups; gi += k_group_cells) {
        Partial<T>& p = partials[gi];
        la = max2(la, p.speed_x);
        lb = max2(lb, p.speed_y);
        ls = ls + p.source_m3;
        lo = lo + p.open_m3;
        lr = lr + p.roundoff_m3;
        p.source_m3 = T(0);
        p.open_m3 = T(0);
        p.roundoff_m3 = T(0);
      }
      a[t] = la; b[t] = lb; src[t] = ls; opn[t] = lo; rnd[t] = lr;
    }
    for (u32 stride = k_group_cells / 2u; stride > 0u; stride >>= 1u)
      for (u32 t = 0; t < stride; ++t) {
        a[t] = max2(a[t], a[t + stride]);
        b[t] = max2(b[t], b[t + stride]);
        src[t] = src[t] + src[t + stride];
        opn[t] = opn[t] + opn[t + stride];
        rnd[t] = rnd[t] + rnd[t + stride];
      }
    LedgerBits<T>& l = ledger;
    pair_add(l.source_hi, l.source_lo, src[0]);
    pair_add(l.open_hi, l.open_lo, opn[0]);
    pair_add(l.roundoff_hi, l.roundoff_lo, rnd[0]);
    if (max_dt > T(0)) {
      const T speed = a[0] + b[0];
      const T reach = cfl * cell_m;
      const T stable = speed > T(0) ? ops.div(reach, speed) : std::numeric_limits<T>::infinity();
      T dt = min2(stable, max_dt);
      dt = min2(dt, l.remaining_s);
      const T left = l.remaining_s - dt;
      l.remaining_s = left;
      l.dt = dt;
      pair_add(l.time_hi, l.time_lo, dt);
      l.steps = l.steps + (dt > T(0) ? 1u : 0u);
    } else {
      l.dt = T(0);
    }
  }

  // update_main (slang:555-757), one cell at a time in the gather form.
  void update(u32 f, T source_scale) {
    const T* in = state[cur].data();
    T* out = state[cur ^ 1u].data();
    const u32 nx = cfg.nx, ny = cfg.ny;
    const T dt = ledger.dt;
    Slots s(size_t(gx) * gy);
    for (u32 y = 0; y < ny; ++y) {
      for (u32 x = 0; x < nx; ++x) {
        const size_t i = size_t(y) * nx + x;
        T ax = 0, ay = 0, cell_source = 0, cell_open = 0, cell_roundoff = 0;
        if (!(dt > T(0))) {
          const T h0 = in[i], hu0 = in[n + i], hv0 = in[2 * n + i];
          out[i] = h0;
          out[n + i] = hu0;
          out[2 * n + i] = hv0;
          out[3 * n + i] = in[3 * n + i];
          cell_speeds(h0, hu0, hv0, ax, ay);
        } else {
          const Cell c = load_cell(in, i);
          Face<T> fw, fe, fs, fn;
          if (x == 0u) {
            const T sign = (f & k_flag_west_open) != 0u ? T(1) : T(-1);
            const T gn = sign * c.u;
            fw = face(ops, g, c.h, c.z, gn, c.v, c.h, c.z, c.u, c.v);
          } else {
            const Cell w = load_cell(in, i - 1);
            fw = face(ops, g, w.h, w.z, w.u, w.v, c.h, c.z, c.u, c.v);
          }
          if (x + 1u == nx) {
            const T sign = (f & k_flag_east_open) != 0u ? T(1) : T(-1);
            const T gn = sign * c.u;
            fe = face(ops, g, c.h, c.z, c.u, c.v, c.h, c.z, gn, c.v);
          } else {
            const Cell e = load_cell(in, i + 1);
            fe = face(ops, g, c.h, c.z, c.u, c.v, e.h, e.z, e.u, e.v);
          }
          if (y == 0u) {
            const T sign = (f & k_flag_south_open) != 0u ? T(1) : T(-1);
            const T gn = sign * c.v;
            fs = face(ops, g, c.h, c.z, gn, c.u, c.h, c.z, c.v, c.u);
          } else {
            const Cell so = load_cell(in, i - nx);
            fs = face(ops, g, so.h, so.z, so.v, so.u, c.h, c.z, c.v, c.u);
          }
          if (y + 1u == ny) {
            const T sign = (f & k_flag_north_open) != 0u ? T(1) : T(-1);
            const T gn = sign * c.v;
            fn = face(ops, g, c.h, c.z, c.v, c.u, c.h, c.z, gn, c.u);
          } else {
            const Cell no = load_cell(in, i + nx);
            fn = face(ops, g, c.h, c.z, c.v, c.u, no.h, no.z, no.v, no.u);
          }
          const T area = cell_m * cell_m;
          const T lam = ops.div(dt, cell_m);
          const T edge_volume = dt * cell_m;
          if (x == 0u && (f & k_flag_west_open) != 0u) cell_open = cell_open - fw.h * edge_volume;
          if (x + 1u == nx && (f & k_flag_east_open) != 0u) cell_open = cell_open + fe.h * edge_volume;
          if (y == 0u && (f & k_flag_south_open) != 0u) cell_open = cell_open - fs.h * edge_volume;
          if (y + 1u == ny && (f & k_flag_north_open) != 0u) cell_open = cell_open + fn.h * edge_volume;
          const T dh1 = fe.h - fw.h;
          const T dh2 = fn.h - fs.h;
          const T dh = dh1 + dh2;
          const T lh = lam * dh;
          T h = c.h - lh;
          const T du1 = fe.nl - fw.nr;
          const T du2 = fn.t - fs.t;
          const T du = du1 + du2;
          const T lu = lam * du;
          T hu = in[n + i] - lu;
          const T dv1 = fe.t - fw.t;
          const T dv2 = fn.nl - fs.nr;
          const T dv = dv1 + dv2;
          const T lv = lam * dv;
          T hv = in[2 * n + i] - lv;
          if (h < T(0)) {
            const T lost = h * area;
            cell_roundoff = cell_roundoff - lost;
            h = T(0);
          }
          T residual = 0;
          if ((f & k_flag_compensate) != 0u) residual = in[3 * n + i];
          if ((f & k_flag_source) != 0u && (f & k_flag_compensate) != 0u) {
            const T owed = source[i] * dt;
            const T scaled = owed * source_scale;
            const T target = scaled + residual;
            T h2 = h;
            if (target >= T(0)) {
              h2 = h + target;
            } else {
              const T want = -target;
              const T taken = want < h ? want : h;
              h2 = h - taken;
            }
            const T applied = h2 - h;
            const T left = target - applied;
            residual = (h2 == T(0) && target < T(0)) ? T(0) : left;
            const T v = applied * area;
            cell_source = cell_source + v;
            h = h2;
          } else if ((f & k_flag_source) != 0u) {
            const T owed = source[i] * dt;
            const T added = owed * source_scale;
            if (added >= T(0)) {
              h = h + added;
              cell_source = cell_source + added * area;
            } else {
              const T want = -added;
              const T taken = want < h ? want : h;
              h = h - taken;
              cell_source = cell_source - taken * area;
            }
          }
          if (h >= dry) {
            if ((f & k_flag_manning) != 0u) {
              const T nn = manning[i];
              const T u = ops.div(hu, h);
              const T v = ops.div(hv, h);
              const T uu = u * u;
              const T vv = v * v;
              const T s2 = uu + vv;
              const T sp = ops.sqrt(s2);
              const T cb = ops.cbrt(h);
              const T k1 = g * nn;
              const T k2 = k1 * nn;
              const T k3 = k2 * sp;
              const T k4 = h * cb;
              const T k = ops.div(k3, k4);
              const T dk = dt * k;
              const T denom = T(1) + dk;
              hu = ops.div(hu, denom);
              hv = ops.div(hv, denom);
            }
          } else {
            hu = T(0);
            hv = T(0);
          }
          out[i] = h;
          out[n + i] = hu;
          out[2 * n + i] = hv;
          if ((f & k_flag_compensate) != 0u) out[3 * n + i] = residual;
          cell_speeds(h, hu, hv, ax, ay);
        }
        const size_t sl = slot(x, y);
        s.sx[sl] = ax;
        s.sy[sl] = ay;
        s.src[sl] = cell_source;
        s.opn[sl] = cell_open;
        s.rnd[sl] = cell_roundoff;
      }
    }
    // A step of no length leaves plane 3 as it was in the other copy too (slang:584); a step that
    // does not compensate leaves the other copy's plane 3 untouched, as the shader does.
    write_partials(s);
  }
};

template <>
inline u64 RefStep<float>::state_hash() const {
  return hash_floats(state[cur].data(), k_state_planes * n);
}

// ---- the reference CPU tick in double (water_state.cpp) ----------------------------------------

class Solver64 {
 public:
  struct Ledger {  // water_state.h:135-145, the fields this restatement keeps
    double source_m3 = 0, open_edge_out_m3 = 0, roundoff_m3 = 0, time_s = 0;
    u64 steps = 0;
  };

  explicit Solver64(const Config& c, u32 threads = 1) : cfg(c), threads_(threads ? threads : 1) {
    n = size_t(c.nx) * c.ny;
    h.assign(n, 0.0);
    hu.assign(n, 0.0);
    hv.assign(n, 0.0);
    u_.assign(n, 0.0);
    v_.assign(n, 0.0);
    row_a.assign(c.ny, 0.0);
    row_b.assign(c.ny, 0.0);
    rows.assign(c.ny, RowSums{});
    const size_t xf = size_t(c.nx + 1) * c.ny, yf = size_t(c.nx) * (c.ny + 1);
    fx_h.assign(xf, 0.0); fx_nl.assign(xf, 0.0); fx_nr.assign(xf, 0.0); fx_t.assign(xf, 0.0);
    fy_h.assign(yf, 0.0); fy_nl.assign(yf, 0.0); fy_nr.assign(yf, 0.0); fy_t.assign(yf, 0.0);
  }

  // The inputs of a step (water_state.h:103-120): bed required; manning and source optional.
  const double* bed = nullptr;
  const double* manning = nullptr;
  const double* source = nullptr;

  double stable_step() {  // water_state.cpp:211-224
    if (n == 0) return std::numeric_limits<double>::infinity();
    for_rows(cfg.ny, [this](u32 b, u32 e) { velocity_rows(b, e); });
    double a = 0.0, b = 0.0;
    for (u32 y = 0; y < cfg.ny; ++y) {
      a = row_a[y] > a ? row_a[y] : a;
      b = row_b[y] > b ? row_b[y] : b;
    }
    const double speed = a + b;
    if (!(speed > 0.0)) return std::numeric_limits<double>::infinity();
    return cfg.cfl * cfg.cell_m / speed;
  }

  double step(double max_dt) {  // water_state.cpp:503-533
    if (n == 0 || bed == nullptr || !(max_dt > 0.0)) return 0.0;
    const double stable = stable_step();
    const double dt = stable < max_dt ? stable : max_dt;
    for_rows(cfg.ny, [this](u32 b, u32 e) { x_face_rows(b, e); });
    for_rows(cfg.ny + 1, [this](u32 b, u32 e) { y_face_rows(b, e); });
    for_rows(cfg.ny, [this, dt](u32 b, u32 e) { update_rows(dt, b, e); });
    for (u32 y = 0; y < cfg.ny; ++y) {
      ledger.source_m3 += rows[y].source;
      ledger.open_edge_out_m3 += rows[y].open;
      ledger.roundoff_m3 += rows[y].roundoff;
    }
    ledger.time_s += dt;
    ledger.steps += 1;
    return dt;
  }

  u64 advance(double duration_s) {  // water_state.cpp:535-547
    if (n == 0 || bed == nullptr) return 0;
    u64 steps = 0;
    double remaining = duration_s;
    while (remaining > 0.0) {
      const double dt = step(remaining);
      if (!(dt > 0.0)) break;
      ++steps;
      if (dt == remaining) break;
      remaining -= dt;
    }
    return steps;
  }

  // FNV-1a over depth, the momenta and the ground's store (zero here) (water_state.cpp:570-578).
  u64 state_hash() const {
    u64 hash = k_fnv_offset;
    hash = hash_doubles(h.data(), n, hash);
    hash = hash_doubles(hu.data(), n, hash);
    hash = hash_doubles(hv.data(), n, hash);
    const double zero = 0.0;
    for (size_t i = 0; i < n; ++i) hash = hash_doubles(&zero, 1, hash);
    return hash;
  }

  double surface_volume_m3() const {  // water_state.cpp:549-554
    double sum = 0.0;
    for (size_t i = 0; i < n; ++i) sum += h[i];
    return sum * (cfg.cell_m * cfg.cell_m);
  }

  Config cfg;
  size_t n = 0;
  std::vector<double> h, hu, hv;
  Ledger ledger;

 private:
  struct RowSums { double source = 0, open = 0, roundoff = 0; };

  template <class F>
  void for_rows(u32 count, F&& body) {  // water_state.cpp:171-183, on plain threads
    if (threads_ <= 1 || count < 2 * threads_) { body(0u, count); return; }
    std::vector<std::thread> pool;
    const u32 chunk = (count + threads_ - 1) / threads_;
    for (u32 t = 0; t < threads_; ++t) {
      const u32 b = t * chunk, e = b + chunk < count ? b + chunk : count;
      if (b >= e) break;
      pool.emplace_back([&body, b, e] { body(b, e); });
    }
    for (auto& th : pool) th.join();
  }

  void velocity_rows(u32 begin, u32 end) {  // water_state.cpp:185-209
    const u32 nx = cfg.nx;
    const double g = cfg.gravity, dry = cfg.dry_depth_m;
    for (u32 y = begin; y < end; ++y) {
      double a = 0.0, b = 0.0;
      for (u32 x = 0; x < nx; ++x) {
        const size_t i = size_t(y) * nx + x;
        const double hh = h[i];
        const bool wet = hh >= dry;
        const double u = wet ? hu[i] / hh : 0.0;
        const double v = wet ? hv[i] / hh : 0.0;
        u_[i] = u;
        v_[i] = v;
        const double c = std::sqrt(g * hh);
        const double au = std::fabs(u) + c;
        const double av = std::fabs(v) + c;
        a = au > a ? au : a;
        b = av > b ? av : b;
      }
      row_a[y] = a;
      row_b[y] = b;
    }
  }

  void face_at(u32 l, u32 r, double ln, double lt, double rn, double rt, double* oh, double* onl,
               double* onr, double* ot, size_t idx) const {  // water_state.cpp:231-257
    const Ops<double> ops;
    const Face<double> f =
        face(ops, cfg.gravity, h[l], bed[l], ln, lt, h[r], bed[r], rn, rt);
    oh[idx] = f.h;
    onl[idx] = f.nl;
    onr[idx] = f.nr;
    ot[idx] = f.t;
  }

  void x_face_rows(u32 begin, u32 end) {  // water_state.cpp:259-279
    const u32 nx = cfg.nx;
    const double west = cfg.west_open ? 1.0 : -1.0;
    const double east = cfg.east_open ? 1.0 : -1.0;
    for (u32 y = begin; y < end; ++y) {
      const u32 row = y * nx;
      const size_t frow = size_t(y) * (nx + 1);
      face_at(row, row, west * u_[row], v_[row], u_[row], v_[row], fx_h.data(), fx_nl.data(),
              fx_nr.data(), fx_t.data(), frow);
      for (u32 f = 1; f < nx; ++f) {
        const u32 l = row + f - 1, r = row + f;
        face_at(l, r, u_[l], v_[l], u_[r], v_[r], fx_h.data(), fx_nl.data(), fx_nr.data(),
                fx_t.data(), frow + f);
      }
      const u32 last = row + nx - 1;
      face_at(last, last, u_[last], v_[last], east * u_[last], v_[last], fx_h.data(),
              fx_nl.data(), fx_nr.data(), fx_t.data(), frow + nx);
    }
  }

  void y_face_rows(u32 begin, u32 end) {  // water_state.cpp:282-308
    const u32 nx = cfg.nx, ny = cfg.ny;
    const double south = cfg.south_open ? 1.0 : -1.0;
    const double north = cfg.north_open ? 1.0 : -1.0;
    for (u32 r = begin; r < end; ++r) {
      const size_t frow = size_t(r) * nx;
      if (r == 0) {
        for (u32 x = 0; x < nx; ++x)
          face_at(x, x, south * v_[x], u_[x], v_[x], u_[x], fy_h.data(), fy_nl.data(),
                  fy_nr.data(), fy_t.data(), frow + x);
      } else if (r == ny) {
        for (u32 x = 0; x < nx; ++x) {
          const u32 c = (ny - 1) * nx + x;
          face_at(c, c, v_[c], u_[c], north * v_[c], u_[c], fy_h.data(), fy_nl.data(),
                  fy_nr.data(), fy_t.data(), frow + x);
        }
      } else {
        for (u32 x = 0; x < nx; ++x) {
          const u32 s = (r - 1) * nx + x, nn = r * nx + x;
          face_at(s, nn, v_[s], u_[s], v_[nn], u_[nn], fy_h.data(), fy_nl.data(), fy_nr.data(),
                  fy_t.data(), frow + x);
        }
      }
    }
  }

  void update_rows(double dt, u32 begin, u32 end) {  // water_state.cpp:310-501, depth and momenta
    const u32 nx = cfg.nx, ny = cfg.ny;
    const double g = cfg.gravity, dry = cfg.dry_depth_m;
    const double area = cfg.cell_m * cfg.cell_m;
    const double lam = dt / cfg.cell_m;
    const double edge_volume = dt * cfg.cell_m;
    for (u32 y = begin; y < end; ++y) {
      RowSums sums{};
      const size_t frow = size_t(y) * (nx + 1);
      if (cfg.west_open) sums.open -= fx_h[frow] * edge_volume;
      if (cfg.east_open) sums.open += fx_h[frow + nx] * edge_volume;
      if (y == 0 && cfg.south_open)
        for (u32 x = 0; x < nx; ++x) sums.open -= fy_h[x] * edge_volume;
      if (y + 1 == ny && cfg.north_open)
        for (u32 x = 0; x < nx; ++x) sums.open += fy_h[size_t(ny) * nx + x] * edge_volume;
      for (u32 x = 0; x < nx; ++x) {
        const size_t i = size_t(y) * nx + x;
        const size_t w = frow + x, e = w + 1;
        const size_t s = size_t(y) * nx + x, nn = s + nx;
        const double h0 = h[i];
        double hh = h0 - lam * ((fx_h[e] - fx_h[w]) + (fy_h[nn] - fy_h[s]));
        double hhu = hu[i] - lam * ((fx_nl[e] - fx_nr[w]) + (fy_t[nn] - fy_t[s]));
        double hhv = hv[i] - lam * ((fx_t[e] - fx_t[w]) + (fy_nl[nn] - fy_nr[s]));
        if (hh < 0.0) {
          sums.roundoff -= hh * area;
          hh = 0.0;
        }
        if (source != nullptr) {
          const double added = source[i] * dt;
          if (added >= 0.0) {
            hh += added;
            sums.source += added * area;
          } else {
            const double taken = -added < hh ? -added : hh;
            hh -= taken;
            sums.source -= taken * area;
          }
        }
        if (hh >= dry) {
          if (manning != nullptr) {
            // The reference takes h^(1/3) from its fdlibm port; this restatement's cube root is
            // the C library's, so Manning's friction is not held to the reference's bytes.
            const double nnn = manning[i];
            const double u = hhu / hh;
            const double v = hhv / hh;
            const double sp = std::sqrt(u * u + v * v);
            const double cb = std::cbrt(hh);
            const double k = g * nnn * nnn * sp / (hh * cb);
            const double denom = 1.0 + dt * k;
            hhu = hhu / denom;
            hhv = hhv / denom;
          }
        } else {
          hhu = 0.0;
          hhv = 0.0;
        }
        h[i] = hh;
        hu[i] = hhu;
        hv[i] = hhv;
      }
      rows[y] = sums;
    }
  }

  u32 threads_ = 1;
  std::vector<double> u_, v_, row_a, row_b;
  std::vector<RowSums> rows;
  std::vector<double> fx_h, fx_nl, fx_nr, fx_t, fy_h, fy_nl, fy_nr, fy_t;
};

}  // namespace wl_oracle

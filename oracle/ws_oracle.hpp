// ORACLE — test infrastructure only. Never linked into, called by or shipped with the product.
//
// The reference's complete FP64 step, domain/water_state/src/water_state.cpp (Solver::step,
// advance, stable_step, the volumes and state_hash), restated in full: depth and momenta, the
// ground's store by Green and Ampt (:400-428), up to four carried quantities riding the mass fluxes
// (:247-256, :351-357, :465-490) with their decay, their source from the dissipation, their outside
// source and their exchange with the bed, the per-cell outputs (speed, bed stress, dissipation,
// :430-461 and :491-498), the energy flux the dissipation is the residual of (:53-61, :82-87), and
// the whole ledger (:503-533). The cube root and the decay take e^x and ln x from the reference's
// deterministic transcendentals (core/math/include/core/math/deterministic.h), which are ports of
// fdlibm's e_exp.c and e_log.c; fd_exp and fd_log below restate those published algorithms.
//
// Pinned by tests/test_ws_oracle.py against the reference's own Solver built from its sources
// (oracle/_ref/libwsref.so, oracle/build_ref.sh): states, outputs and ledgers byte for byte, and
// fd_exp / fd_log against the reference's det::exp / det::log over dense argument grids.
//
// Compile with -ffp-contract=off and without -ffast-math, like the reference.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace ws_oracle {

using u32 = uint32_t;
using u64 = uint64_t;

inline double from_bits(u64 b) { double d; std::memcpy(&d, &b, 8); return d; }
inline u64 to_bits(double d) { u64 b; std::memcpy(&b, &d, 8); return b; }
inline u32 high_word(double d) { return u32(to_bits(d) >> 32); }

// ---- fdlibm's e^x and ln x (Sun Microsystems 1993/2004; netlib.org/fdlibm e_exp.c, e_log.c) ----

constexpr u64 kLn2Hi = 0x3fe62e42fee00000ull, kLn2Lo = 0x3dea39ef35793c76ull;
constexpr u64 kInvLn2 = 0x3ff71547652b82feull;
constexpr u64 kP[5] = {0x3fc555555555553eull, 0xbf66c16c16bebd93ull, 0x3f11566aaf25de2cull,
                       0xbebbbd41c5d26bf1ull, 0x3e66376972bea4d0ull};
constexpr u64 kLg[7] = {0x3fe5555555555593ull, 0x3fd999999997fa04ull, 0x3fd2492494229359ull,
                        0x3fcc71c51d8e78afull, 0x3fc7466496cb03deull, 0x3fc39a09d078c69full,
                        0x3fc2f112df3e5244ull};

inline double fd_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893383973096) return std::numeric_limits<double>::infinity();
  if (x < -745.13321910194110842) return 0.0;
  const double ln2hi = from_bits(kLn2Hi), ln2lo = from_bits(kLn2Lo);
  const u32 ax = high_word(x) & 0x7fffffffu;
  const bool neg = x < 0.0;
  double hi = 0.0, lo = 0.0;
  int k = 0;
  if (ax > 0x3fd62e42u) {  // |x| > ln2 / 2: x = k ln2 + r
    if (ax < 0x3ff0a2b2u) {
      hi = neg ? x + ln2hi : x - ln2hi;
      lo = neg ? -ln2lo : ln2lo;
      k = neg ? -1 : 1;
    } else {
      k = int(from_bits(kInvLn2) * x + (neg ? -0.5 : 0.5));
      const double t = double(k);
      hi = x - t * ln2hi;
      lo = t * ln2lo;
    }
    x = hi - lo;
  } else if (ax < 0x3e300000u) {  // |x| < 2^-28
    return 1.0 + x;
  }
  const double t = x * x;
  const double c = x - t * (from_bits(kP[0]) +
                            t * (from_bits(kP[1]) +
                                 t * (from_bits(kP[2]) + t * (from_bits(kP[3]) + t * from_bits(kP[4])))));
  if (k == 0) return 1.0 - ((x * c) / (c - 2.0) - x);
  const double y = 1.0 - ((lo - (x * c) / (2.0 - c)) - hi);
  return std::ldexp(y, k);
}

inline double fd_log(double x) {
  const double ln2hi = from_bits(kLn2Hi), ln2lo = from_bits(kLn2Lo);
  u64 b = to_bits(x);
  int32_t hx = int32_t(b >> 32);
  const u32 lx = u32(b);
  int k = 0;
  if (hx < 0x00100000) {  // below the normal range
    if (((u32(hx) & 0x7fffffffu) | lx) == 0) return -std::numeric_limits<double>::infinity();
    if (hx < 0) return std::numeric_limits<double>::quiet_NaN();
    k -= 54;
    x *= from_bits(0x4350000000000000ull);  // 2^54
    b = to_bits(x);
    hx = int32_t(b >> 32);
  }
  if (hx >= 0x7ff00000) return x + x;
  k += (hx >> 20) - 1023;
  hx &= 0x000fffff;
  const int32_t i = (hx + 0x95f64) & 0x100000;
  x = from_bits((u64(u32(hx | (i ^ 0x3ff00000))) << 32) | (b & 0xffffffffull));  // into [√2/2, √2)
  k += i >> 20;
  const double f = x - 1.0;
  if ((0x000fffff & (2 + hx)) < 3) {  // |f| < 2^-20
    if (f == 0.0) {
      if (k == 0) return 0.0;
      const double dk = double(k);
      return dk * ln2hi + dk * ln2lo;
    }
    const double r = f * f * (0.5 - 0.33333333333333333 * f);
    if (k == 0) return f - r;
    const double dk = double(k);
    return dk * ln2hi - ((r - dk * ln2lo) - f);
  }
  const double s = f / (2.0 + f);
  const double dk = double(k);
  const double z = s * s;
  int32_t ii = hx - 0x6147a;
  const double w = z * z;
  const int32_t jj = 0x6b851 - hx;
  const double t1 = w * (from_bits(kLg[1]) + w * (from_bits(kLg[3]) + w * from_bits(kLg[5])));
  const double t2 = z * (from_bits(kLg[0]) +
                         w * (from_bits(kLg[2]) + w * (from_bits(kLg[4]) + w * from_bits(kLg[6]))));
  ii |= jj;
  const double r = t2 + t1;
  if (ii > 0) {
    const double hfsq = 0.5 * f * f;
    if (k == 0) return f - (hfsq - s * (hfsq + r));
    return dk * ln2hi - ((hfsq - (s * (hfsq + r) + dk * ln2lo)) - f);
  }
  if (k == 0) return f - s * (f - r);
  return dk * ln2hi - ((s * (f - r) - dk * ln2lo) - f);
}

// ---- the full step ---------------------------------------------------------------------------

constexpr u32 kMaxCarried = 4;  // water_state.h:53

struct CarriedConfig { double decay_s = 0, per_joule = 0, min_speed = 0; };  // water_state.h:66-78

struct Config {  // water_state.h:83-99
  u32 nx = 0, ny = 0;
  double cell_m = 1, gravity = 9.81, cfl = 0.45, dry = 1e-9, rho = 1000;
  u32 carried = 0;
  CarriedConfig cc[kMaxCarried];
  bool west_open = false, east_open = false, south_open = false, north_open = false;
};

struct CarriedLedger { double source = 0, from_dissipation = 0, exchange = 0, decayed = 0, open = 0; };

struct Ledger {  // water_state.h:135-145
  double source = 0, open = 0, ground = 0, roundoff = 0, scheme_loss = 0, friction = 0, time = 0;
  u64 steps = 0;
  CarriedLedger carried[kMaxCarried];
};

// The inputs of a step (water_state.h:103-120); null where a span is empty.
struct Inputs {
  const double* bed = nullptr;
  const double* manning = nullptr;
  const double* source = nullptr;
  const double* ground_k = nullptr;
  const double* ground_s = nullptr;
  const double* ground_cap = nullptr;
  const double* carried_source[kMaxCarried] = {};
  const double* carried_exchange[kMaxCarried] = {};
};

struct Flux { double h, n, t, g; };

inline double pressure(double g, double h) { return 0.5 * g * h * h; }
inline double energy(double g, double h, double un, double ut, double z) {
  return 0.5 * h * (un * un + ut * ut) + pressure(g, h) + g * h * z;
}
inline double energy_flux(double g, double h, double un, double ut, double z) {
  return un * (0.5 * h * (un * un + ut * ut) + 2.0 * pressure(g, h) + g * h * z);
}

// water_state.cpp:67-90: Bollermann et al. (2014) (2.8) with the energy as a further component.
inline Flux face_flux(double g, double z, double hl, double ul, double vl, double hr, double ur,
                      double vr) {
  if (hl == hr && ul == ur && vl == vr) {
    const double q = hl * ul;
    return {q, q * ul + pressure(g, hl), q * vl, energy_flux(g, hl, ul, vl, z)};
  }
  const double cl = std::sqrt(g * hl), cr = std::sqrt(g * hr);
  double ap = ur + cr > ul + cl ? ur + cr : ul + cl;
  ap = ap > 0.0 ? ap : 0.0;
  double am = ur - cr < ul - cl ? ur - cr : ul - cl;
  am = am < 0.0 ? am : 0.0;
  const double span = ap - am;
  if (!(span > 0.0)) return {0, 0, 0, 0};
  const double ql = hl * ul, qr = hr * ur, apam = ap * am;
  const double fh = (ap * ql - am * qr + apam * (hr - hl)) / span;
  const double fn =
      (ap * (ql * ul + pressure(g, hl)) - am * (qr * ur + pressure(g, hr)) + apam * (qr - ql)) / span;
  const double ft = (ap * (ql * vl) - am * (qr * vr) + apam * (hr * vr - hl * vl)) / span;
  const double fg = (ap * energy_flux(g, hl, ul, vl, z) - am * energy_flux(g, hr, ur, vr, z) +
                     apam * (energy(g, hr, ur, vr, z) - energy(g, hl, ul, vl, z))) / span;
  return {fh, fn, ft, fg};
}

class SolverFull {
 public:
  explicit SolverFull(const Config& c) : cfg(c) {
    if (cfg.carried > kMaxCarried) cfg.carried = kMaxCarried;
    n = size_t(c.nx) * c.ny;
    const size_t k = cfg.carried;
    h.assign(n, 0); hu.assign(n, 0); hv.assign(n, 0); ground.assign(n, 0); carried.assign(k * n, 0);
    speed.assign(n, 0); tau_x.assign(n, 0); tau_y.assign(n, 0); dissipation.assign(n, 0);
    u_.assign(n, 0); v_.assign(n, 0);
    xf = size_t(c.nx + 1) * c.ny;
    yf = size_t(c.nx) * (c.ny + 1);
    for (auto* f : {&fx_h, &fx_nl, &fx_nr, &fx_t, &fx_g}) f->assign(xf, 0);
    for (auto* f : {&fy_h, &fy_nl, &fy_nr, &fy_t, &fy_g}) f->assign(yf, 0);
    fx_c.assign(k * xf, 0);
    fy_c.assign(k * yf, 0);
    rows.assign(c.ny, RowSums{});
  }

  double stable_step() {  // water_state.cpp:185-224
    if (n == 0) return std::numeric_limits<double>::infinity();
    const double g = cfg.gravity, dry = cfg.dry;
    double a = 0, b = 0;
    for (size_t i = 0; i < n; ++i) {  // a maximum is the same in any order
      const double hh = h[i];
      const bool wet = hh >= dry;
      const double u = wet ? hu[i] / hh : 0.0, v = wet ? hv[i] / hh : 0.0;
      u_[i] = u;
      v_[i] = v;
      const double c = std::sqrt(g * hh);
      const double au = std::fabs(u) + c, av = std::fabs(v) + c;
      a = au > a ? au : a;
      b = av > b ? av : b;
    }
    const double speed_sum = a + b;
    if (!(speed_sum > 0.0)) return std::numeric_limits<double>::infinity();
    return cfg.cfl * cfg.cell_m / speed_sum;
  }

  double step(const Inputs& in, double max_dt) {  // water_state.cpp:503-533
    if (n == 0 || in.bed == nullptr || !(max_dt > 0.0)) return 0.0;
    const double stable = stable_step();
    const double dt = stable < max_dt ? stable : max_dt;
    x_faces(in);
    y_faces(in);
    update(in, dt);
    for (u32 y = 0; y < cfg.ny; ++y) {
      const RowSums& r = rows[y];
      ledger.source += r.source;
      ledger.open += r.open;
      ledger.roundoff += r.roundoff;
      ledger.ground += r.ground;
      ledger.scheme_loss += r.scheme_loss;
      ledger.friction += r.friction;
      for (u32 k = 0; k < cfg.carried; ++k) {
        CarriedLedger& to = ledger.carried[k];
        const CarriedLedger& from = r.carried[k];
        to.source += from.source;
        to.from_dissipation += from.from_dissipation;
        to.exchange += from.exchange;
        to.decayed += from.decayed;
        to.open += from.open;
      }
    }
    ledger.time += dt;
    ledger.steps += 1;
    return dt;
  }

  u64 advance(const Inputs& in, double duration) {  // water_state.cpp:535-547
    if (n == 0 || in.bed == nullptr) return 0;
    u64 steps = 0;
    double remaining = duration;
    while (remaining > 0.0) {
      const double dt = step(in, remaining);
      if (!(dt > 0.0)) break;
      ++steps;
      if (dt == remaining) break;
      remaining -= dt;
    }
    return steps;
  }

  u64 state_hash() const {  // water_state.cpp:570-578
    u64 hash = 0xcbf29ce484222325ull;
    auto put = [&hash](const std::vector<double>& v) {
      for (double d : v) {
        const u64 bits = to_bits(d);
        for (u32 b = 0; b < 8; ++b) {
          hash ^= (bits >> (8 * b)) & 0xffu;
          hash *= 0x100000001b3ull;
        }
      }
    };
    put(h); put(hu); put(hv); put(ground); put(carried);
    return hash;
  }

  Config cfg;
  size_t n = 0, xf = 0, yf = 0;
  std::vector<double> h, hu, hv, ground, carried, speed, tau_x, tau_y, dissipation;
  Ledger ledger;

 private:
  struct RowSums {
    double source = 0, open = 0, roundoff = 0, ground = 0, scheme_loss = 0, friction = 0;
    CarriedLedger carried[kMaxCarried];
  };

  // water_state.cpp:231-257: one face between l and r (l == r at an edge's ghost).
  void face(const Inputs& in, u32 l, u32 r, double ln, double lt, double rn, double rt, bool x_dir,
            size_t idx) {
    const double g = cfg.gravity;
    const double zl = in.bed[l], zr = in.bed[r];
    const double zf = zl > zr ? zl : zr;
    const double el = h[l] + zl - zf, er = h[r] + zr - zf;
    const double hl = el > 0.0 ? el : 0.0, hr = er > 0.0 ? er : 0.0;
    const Flux f = face_flux(g, zf, hl, ln, lt, hr, rn, rt);
    (x_dir ? fx_h : fy_h)[idx] = f.h;
    (x_dir ? fx_nl : fy_nl)[idx] = f.n - pressure(g, hl);
    (x_dir ? fx_nr : fy_nr)[idx] = f.n - pressure(g, hr);
    (x_dir ? fx_t : fy_t)[idx] = f.t;
    (x_dir ? fx_g : fy_g)[idx] = f.g;
    if (cfg.carried != 0) {
      const u32 up = f.h > 0.0 ? l : r;
      const double h_up = h[up];
      const bool wet = h_up >= cfg.dry;
      std::vector<double>& oc = x_dir ? fx_c : fy_c;
      const size_t count = x_dir ? xf : yf;
      for (u32 k = 0; k < cfg.carried; ++k) {
        const double conc = wet ? carried[k * n + up] / h_up : 0.0;
        oc[k * count + idx] = f.h * conc;
      }
    }
  }

  void x_faces(const Inputs& in) {  // water_state.cpp:259-279
    const u32 nx = cfg.nx;
    const double west = cfg.west_open ? 1.0 : -1.0, east = cfg.east_open ? 1.0 : -1.0;
    for (u32 y = 0; y < cfg.ny; ++y) {
      const u32 row = y * nx;
      const size_t frow = size_t(y) * (nx + 1);
      face(in, row, row, west * u_[row], v_[row], u_[row], v_[row], true, frow);
      for (u32 f = 1; f < nx; ++f)
        face(in, row + f - 1, row + f, u_[row + f - 1], v_[row + f - 1], u_[row + f], v_[row + f],
             true, frow + f);
      const u32 last = row + nx - 1;
      face(in, last, last, u_[last], v_[last], east * u_[last], v_[last], true, frow + nx);
    }
  }

  void y_faces(const Inputs& in) {  // water_state.cpp:282-308
    const u32 nx = cfg.nx, ny = cfg.ny;
    const double south = cfg.south_open ? 1.0 : -1.0, north = cfg.north_open ? 1.0 : -1.0;
    for (u32 r = 0; r <= ny; ++r) {
      const size_t frow = size_t(r) * nx;
      for (u32 x = 0; x < nx; ++x) {
        if (r == 0) {
          face(in, x, x, south * v_[x], u_[x], v_[x], u_[x], false, frow + x);
        } else if (r == ny) {
          const u32 c = (ny - 1) * nx + x;
          face(in, c, c, v_[c], u_[c], north * v_[c], u_[c], false, frow + x);
        } else {
          const u32 s = (r - 1) * nx + x, nn = r * nx + x;
          face(in, s, nn, v_[s], u_[s], v_[nn], u_[nn], false, frow + x);
        }
      }
    }
  }

  void update(const Inputs& in, double dt) {  // water_state.cpp:310-501
    const u32 nx = cfg.nx, ny = cfg.ny, nk = cfg.carried;
    const double g = cfg.gravity, dry = cfg.dry, rho = cfg.rho;
    const double area = cfg.cell_m * cfg.cell_m;
    const double lam = dt / cfg.cell_m;
    const double edge_volume = dt * cfg.cell_m;
    double keep[kMaxCarried];
    for (u32 k = 0; k < nk; ++k) {
      const double tau = cfg.cc[k].decay_s;
      keep[k] = tau > 0.0 ? fd_exp(-dt / tau) : 1.0;
    }
    for (u32 y = 0; y < ny; ++y) {
      RowSums sums{};
      const size_t frow = size_t(y) * (nx + 1);
      if (cfg.west_open) {
        sums.open -= fx_h[frow] * edge_volume;
        for (u32 k = 0; k < nk; ++k) sums.carried[k].open -= fx_c[k * xf + frow] * edge_volume;
      }
      if (cfg.east_open) {
        sums.open += fx_h[frow + nx] * edge_volume;
        for (u32 k = 0; k < nk; ++k) sums.carried[k].open += fx_c[k * xf + frow + nx] * edge_volume;
      }
      if (y == 0 && cfg.south_open) {
        for (u32 x = 0; x < nx; ++x) {
          sums.open -= fy_h[x] * edge_volume;
          for (u32 k = 0; k < nk; ++k) sums.carried[k].open -= fy_c[k * yf + x] * edge_volume;
        }
      }
      if (y + 1 == ny && cfg.north_open) {
        for (u32 x = 0; x < nx; ++x) {
          sums.open += fy_h[size_t(ny) * nx + x] * edge_volume;
          for (u32 k = 0; k < nk; ++k)
            sums.carried[k].open += fy_c[k * yf + size_t(ny) * nx + x] * edge_volume;
        }
      }
      for (u32 x = 0; x < nx; ++x) {
        const size_t i = size_t(y) * nx + x;
        const size_t w = frow + x, e = w + 1, s = i, nn = i + nx;
        const double z = in.bed[i];
        const double h0 = h[i];
        const double energy0 = energy(g, h0, u_[i], v_[i], z);
        double hh = h0 - lam * ((fx_h[e] - fx_h[w]) + (fy_h[nn] - fy_h[s]));
        double mu = hu[i] - lam * ((fx_nl[e] - fx_nr[w]) + (fy_t[nn] - fy_t[s]));
        double mv = hv[i] - lam * ((fx_t[e] - fx_t[w]) + (fy_nl[nn] - fy_nr[s]));
        for (u32 k = 0; k < nk; ++k) {
          double& q = carried[k * n + i];
          q = q - lam * ((fx_c[k * xf + e] - fx_c[k * xf + w]) + (fy_c[k * yf + nn] - fy_c[k * yf + s]));
        }
        double scheme_loss;
        {
          const bool wet = hh >= dry;
          const double u1 = wet ? mu / hh : 0.0, v1 = wet ? mv / hh : 0.0;
          const double energy1 = energy(g, hh > 0.0 ? hh : 0.0, u1, v1, z);
          const double through = (fx_g[e] - fx_g[w]) + (fy_g[nn] - fy_g[s]);
          scheme_loss = -rho * ((energy1 - energy0) / dt + through / cfg.cell_m);
        }
        sums.scheme_loss += scheme_loss * area * dt;
        if (hh < 0.0) {
          sums.roundoff -= hh * area;
          hh = 0.0;
        }
        if (in.source != nullptr) {
          const double added = in.source[i] * dt;
          if (added >= 0.0) {
            hh += added;
            sums.source += added * area;
          } else {
            const double taken = -added < hh ? -added : hh;
            hh -= taken;
            sums.source -= taken * area;
          }
        }
        if (in.ground_k != nullptr && hh > 0.0) {
          const double stored = ground[i];
          const double room = in.ground_cap[i] - stored;
          if (room > 0.0) {
            const double kdt = in.ground_k[i] * dt;
            const double b = stored + kdt;
            const double next = 0.5 * (b + std::sqrt(b * b + 4.0 * kdt * in.ground_s[i]));
            double take = next - stored;
            take = take < hh ? take : hh;
            take = take < room ? take : room;
            if (take > 0.0) {
              hh -= take;
              ground[i] = stored + take;
              sums.ground += take * area;
            }
          }
        }
        double sp = 0, tx = 0, ty = 0, friction = 0;
        if (hh >= dry) {
          if (in.manning != nullptr) {
            const double nnn = in.manning[i];
            const double u = mu / hh, v = mv / hh;
            const double s0 = std::sqrt(u * u + v * v);
            const double cb = fd_exp(fd_log(hh) / 3.0);
            const double kk = g * nnn * nnn * s0 / (hh * cb);
            const double denom = 1.0 + dt * kk;
            mu = mu / denom;
            mv = mv / denom;
            const double u1 = mu / hh, v1 = mv / hh;
            sp = std::sqrt(u1 * u1 + v1 * v1);
            const double coeff = rho * g * nnn * nnn * sp / cb;
            tx = coeff * u1;
            ty = coeff * v1;
            friction = coeff * sp * sp;
          } else {
            const double u1 = mu / hh, v1 = mv / hh;
            sp = std::sqrt(u1 * u1 + v1 * v1);
          }
        } else {
          mu = 0.0;
          mv = 0.0;
        }
        sums.friction += friction * area * dt;
        const double diss = (scheme_loss > 0.0 ? scheme_loss : 0.0) + friction;
        for (u32 k = 0; k < nk; ++k) {
          const CarriedConfig& cc = cfg.cc[k];
          CarriedLedger& account = sums.carried[k];
          double& q = carried[k * n + i];
          if (cc.per_joule > 0.0 && sp >= cc.min_speed) {
            const double made = cc.per_joule * diss * dt;
            q += made;
            account.from_dissipation += made * area;
          }
          if (in.carried_source[k] != nullptr) {
            const double added = in.carried_source[k][i] * dt;
            q += added;
            account.source += added * area;
          }
          if (in.carried_exchange[k] != nullptr) {
            double moved = in.carried_exchange[k][i] * dt;
            if (moved < 0.0 && -moved > q) moved = -q;
            q += moved;
            account.exchange += moved * area;
          }
          if (keep[k] != 1.0) {
            const double kept = q * keep[k];
            account.decayed += (q - kept) * area;
            q = kept;
          }
        }
        h[i] = hh;
        hu[i] = mu;
        hv[i] = mv;
        speed[i] = sp;
        tau_x[i] = tx;
        tau_y[i] = ty;
        dissipation[i] = diss;
      }
      rows[y] = sums;
    }
  }

  std::vector<double> u_, v_;
  std::vector<double> fx_h, fx_nl, fx_nr, fx_t, fx_g, fx_c, fy_h, fy_nl, fy_nr, fy_t, fy_g, fy_c;
  std::vector<RowSums> rows;
};

}  // namespace ws_oracle

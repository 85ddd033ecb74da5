// The complete FP64 step's kernels, its host side and its C ABI (wlcuda.h, "the complete FP64
// step"). See ws_solver.h for the launch sequence. Every expression keeps the reference's
// operand order (domain/water_state/src/water_state.cpp); the unit compiles with --fmad=false.
#include "ws_solver.h"
#include "wlcuda.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

namespace wsc {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double bits_double(unsigned long long b) { return __longlong_as_double(b); }
__device__ __forceinline__ unsigned long long double_bits(double d) {
  return static_cast<unsigned long long>(__double_as_longlong(d));
}

// ---- e^x and ln x: fdlibm's e_exp.c and e_log.c (Sun Microsystems; netlib.org/fdlibm), which
// the reference's deterministic transcendentals port (core/math/include/core/math/deterministic.h).
// Cody-Waite reduction by ln 2 and fdlibm's minimax kernels, the coefficients by their bits.

__device__ __forceinline__ double cbits(unsigned long long b) { return __longlong_as_double(b); }

__device__ double fd_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893383973096) return __longlong_as_double(0x7ff0000000000000ll);
  if (x < -745.13321910194110842) return 0.0;
  const double ln2hi = cbits(0x3fe62e42fee00000ull), ln2lo = cbits(0x3dea39ef35793c76ull);
  const uint32_t ax = uint32_t(double_bits(x) >> 32) & 0x7fffffffu;
  const bool neg = x < 0.0;
  double hi = 0.0, lo = 0.0;
  int k = 0;
  if (ax > 0x3fd62e42u) {
    if (ax < 0x3ff0a2b2u) {
      hi = neg ? x + ln2hi : x - ln2hi;
      lo = neg ? -ln2lo : ln2lo;
      k = neg ? -1 : 1;
    } else {
      k = int(cbits(0x3ff71547652b82feull) * x + (neg ? -0.5 : 0.5));
      const double t = double(k);
      hi = x - t * ln2hi;
      lo = t * ln2lo;
    }
    x = hi - lo;
  } else if (ax < 0x3e300000u) {
    return 1.0 + x;
  }
  const double t = x * x;
  const double c =
      x - t * (cbits(0x3fc555555555553eull) +
               t * (cbits(0xbf66c16c16bebd93ull) +
                    t * (cbits(0x3f11566aaf25de2cull) +
                         t * (cbits(0xbebbbd41c5d26bf1ull) + t * cbits(0x3e66376972bea4d0ull)))));
  if (k == 0) return 1.0 - ((x * c) / (c - 2.0) - x);
  const double y = 1.0 - ((lo - (x * c) / (2.0 - c)) - hi);
  return ldexp(y, k);
}

__device__ double fd_log(double x) {
  const double ln2hi = cbits(0x3fe62e42fee00000ull), ln2lo = cbits(0x3dea39ef35793c76ull);
  unsigned long long b = double_bits(x);
  int32_t hx = int32_t(b >> 32);
  const uint32_t lx = uint32_t(b);
  int k = 0;
  if (hx < 0x00100000) {
    if (((uint32_t(hx) & 0x7fffffffu) | lx) == 0) return __longlong_as_double(0xfff0000000000000ll);
    if (hx < 0) return __longlong_as_double(0x7ff8000000000000ll);
    k -= 54;
    x *= cbits(0x4350000000000000ull);
    b = double_bits(x);
    hx = int32_t(b >> 32);
  }
  if (hx >= 0x7ff00000) return x + x;
  k += (hx >> 20) - 1023;
  hx &= 0x000fffff;
  const int32_t i = (hx + 0x95f64) & 0x100000;
  x = __longlong_as_double(
      (long long)((uint64_t(uint32_t(hx | (i ^ 0x3ff00000))) << 32) | (b & 0xffffffffull)));
  k += i >> 20;
  const double f = x - 1.0;
  if ((0x000fffff & (2 + hx)) < 3) {
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
  const double t1 = w * (cbits(0x3fd999999997fa04ull) +
                         w * (cbits(0x3fcc71c51d8e78afull) + w * cbits(0x3fc39a09d078c69full)));
  const double t2 =
      z * (cbits(0x3fe5555555555593ull) +
           w * (cbits(0x3fd2492494229359ull) +
                w * (cbits(0x3fc7466496cb03deull) + w * cbits(0x3fc2f112df3e5244ull))));
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

// ---- the scheme (water_state.cpp:33-90) ------------------------------------------------------

__device__ __forceinline__ double pressure(double g, double h) { return 0.5 * g * h * h; }
__device__ __forceinline__ double energy(double g, double h, double un, double ut, double z) {
  return 0.5 * h * (un * un + ut * ut) + pressure(g, h) + g * h * z;
}
__device__ __forceinline__ double energy_flux(double g, double h, double un, double ut, double z) {
  return un * (0.5 * h * (un * un + ut * ut) + 2.0 * pressure(g, h) + g * h * z);
}

struct Flux {
  double h, n, t, g;
};

__device__ Flux face_flux(double g, double z, double hl, double ul, double vl, double hr,
                          double ur, double vr) {
  if (hl == hr && ul == ur && vl == vr) {
    const double q = hl * ul;
    return {q, q * ul + pressure(g, hl), q * vl, energy_flux(g, hl, ul, vl, z)};
  }
  const double cl = sqrt(g * hl), cr = sqrt(g * hr);
  const double p1 = ur + cr, p2 = ul + cl;
  double ap = p1 > p2 ? p1 : p2;
  ap = ap > 0.0 ? ap : 0.0;
  const double m1 = ur - cr, m2 = ul - cl;
  double am = m1 < m2 ? m1 : m2;
  am = am < 0.0 ? am : 0.0;
  const double span = ap - am;
  if (!(span > 0.0)) return {0.0, 0.0, 0.0, 0.0};
  const double ql = hl * ul, qr = hr * ur, apam = ap * am;
  const double fh = (ap * ql - am * qr + apam * (hr - hl)) / span;
  const double fn =
      (ap * (ql * ul + pressure(g, hl)) - am * (qr * ur + pressure(g, hr)) + apam * (qr - ql)) /
      span;
  const double ft = (ap * (ql * vl) - am * (qr * vr) + apam * (hr * vr - hl * vl)) / span;
  const double fg = (ap * energy_flux(g, hl, ul, vl, z) - am * energy_flux(g, hr, ur, vr, z) +
                     apam * (energy(g, hr, ur, vr, z) - energy(g, hl, ul, vl, z))) /
                    span;
  return {fh, fn, ft, fg};
}

__device__ __forceinline__ uint32_t quantities(const Desc& d) { return 6u + 5u * d.nk; }

// ---- the kernels ---------------------------------------------------------------------------

// A run's mode: `count` steps of max_dt, or an advance of `duration`.
__global__ void ws_mode_kernel(Ctl* c, uint32_t advance, double max_dt, double duration) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->advance = advance;
  c->max_dt = max_dt;
  c->remaining = duration;
  c->active = advance != 0u ? (duration > 0.0 ? 1u : 0u) : 1u;
  c->taken = 0;
}

// velocity_rows (cpp:185-209): the velocities the faces read and the largest speeds.
__global__ void __launch_bounds__(kThreads) ws_speeds_kernel(Desc d) {
  const Ctl* c = d.ctl;
  if (c->advance != 0u && c->active == 0u) return;
  unsigned long long a = 0ull, b = 0ull;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < d.n;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const double h = d.h[i];
    const bool wet = h >= d.dry;
    const double u = wet ? d.hu[i] / h : 0.0;
    const double v = wet ? d.hv[i] / h : 0.0;
    d.u[i] = u;
    d.v[i] = v;
    const double cc = sqrt(d.g * h);
    const double au = fabs(u) + cc, av = fabs(v) + cc;
    // `a = au > a ? au : a` from 0: only a positive speed raises it (a NaN never does).
    if (au > 0.0) a = max(a, double_bits(au));
    if (av > 0.0) b = max(b, double_bits(av));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (a != 0ull) atomicMax(&d.ctl->a_bits, a);
    if (b != 0ull) atomicMax(&d.ctl->b_bits, b);
  }
}

// stable_step (cpp:211-224), the step's length (cpp:506-507, and advance's loop, cpp:535-547),
// and the decay factors (cpp:330-334). One thread.
__global__ void ws_length_kernel(Desc d, int stable_only) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Ctl* c = d.ctl;
  if (!stable_only && c->advance != 0u && c->active == 0u) {
    c->dt = 0.0;
    c->a_bits = c->b_bits = 0ull;
    return;
  }
  const double a = bits_double(c->a_bits), b = bits_double(c->b_bits);
  c->a_bits = c->b_bits = 0ull;
  const double speed = a + b;
  const double stable = speed > 0.0 ? d.cfl * d.cell_m / speed
                                    : __longlong_as_double(0x7ff0000000000000ll);
  c->stable = stable;
  if (stable_only) return;
  const double limit = c->advance != 0u ? c->remaining : c->max_dt;
  const double dt = stable < limit ? stable : limit;
  if (c->advance != 0u) {
    if (!(dt > 0.0)) {  // the advance stops without a step
      c->active = 0u;
      c->dt = 0.0;
      return;
    }
    if (dt == c->remaining) c->active = 0u;
    else c->remaining -= dt;
  }
  c->taken += 1;
  c->dt = dt;
  for (uint32_t k = 0; k < d.nk; ++k) {
    const double tau = d.cc[k].decay_s;
    c->keep[k] = tau > 0.0 ? fd_exp(-dt / tau) : 1.0;
  }
}

// A step goes on unless an advance stopped: its length is then 0.
__device__ __forceinline__ bool stepping(const Ctl* c) {
  return c->advance == 0u || c->dt > 0.0;
}

// face (cpp:231-257) over x_face_rows / y_face_rows (cpp:259-308): one thread a face.
__global__ void __launch_bounds__(kThreads) ws_faces_kernel(Desc d) {
  if (!stepping(d.ctl)) return;
  const uint32_t nx = d.nx, ny = d.ny;
  const double west = (d.open & 1u) ? 1.0 : -1.0, east = (d.open & 2u) ? 1.0 : -1.0;
  const double south = (d.open & 4u) ? 1.0 : -1.0, north = (d.open & 8u) ? 1.0 : -1.0;
  const uint64_t total = d.xf + d.yf;
  for (uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; f < total;
       f += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t l, r, idx;
    double ln, lt, rn, rt;
    const bool xdir = f < d.xf;
    if (xdir) {
      idx = f;
      const uint64_t y = f / (nx + 1), fi = f - y * (nx + 1);
      const uint64_t row = y * nx;
      if (fi == 0) {
        l = r = row;
        ln = west * d.u[row];
        lt = d.v[row];
        rn = d.u[row];
        rt = d.v[row];
      } else if (fi == nx) {
        l = r = row + nx - 1;
        ln = d.u[l];
        lt = d.v[l];
        rn = east * d.u[l];
        rt = d.v[l];
      } else {
        l = row + fi - 1;
        r = row + fi;
        ln = d.u[l];
        lt = d.v[l];
        rn = d.u[r];
        rt = d.v[r];
      }
    } else {
      idx = f - d.xf;
      const uint64_t fr = idx / nx, x = idx - fr * nx;
      if (fr == 0) {
        l = r = x;
        ln = south * d.v[x];
        lt = d.u[x];
        rn = d.v[x];
        rt = d.u[x];
      } else if (fr == ny) {
        l = r = uint64_t(ny - 1) * nx + x;
        ln = d.v[l];
        lt = d.u[l];
        rn = north * d.v[l];
        rt = d.u[l];
      } else {
        l = (fr - 1) * nx + x;
        r = fr * nx + x;
        ln = d.v[l];
        lt = d.u[l];
        rn = d.v[r];
        rt = d.u[r];
      }
    }
    const double g = d.g;
    const double zl = d.bed[l], zr = d.bed[r];
    const double zf = zl > zr ? zl : zr;
    const double el = d.h[l] + zl - zf, er = d.h[r] + zr - zf;
    const double hl = el > 0.0 ? el : 0.0, hr = er > 0.0 ? er : 0.0;
    const Flux fl = face_flux(g, zf, hl, ln, lt, hr, rn, rt);
    double* const* out = xdir ? d.fx : d.fy;
    out[0][idx] = fl.h;
    out[1][idx] = fl.n - pressure(g, hl);
    out[2][idx] = fl.n - pressure(g, hr);
    out[3][idx] = fl.t;
    out[4][idx] = fl.g;
    if (d.nk != 0u) {
      const uint64_t up = fl.h > 0.0 ? l : r;
      const double h_up = d.h[up];
      const bool wet = h_up >= d.dry;
      double* oc = xdir ? d.fxc : d.fyc;
      const uint64_t count = xdir ? d.xf : d.yf;
      for (uint32_t k = 0; k < d.nk; ++k) {
        const double conc = wet ? d.carried[k * d.n + up] / h_up : 0.0;
        oc[k * count + idx] = fl.h * conc;
      }
    }
  }
}

// update_rows' cell (cpp:364-498): the state, the outputs and the cell's shares of its row's sums.
__global__ void __launch_bounds__(kThreads) ws_update_kernel(Desc d) {
  const Ctl* c = d.ctl;
  if (!stepping(c)) return;
  const double dt = c->dt;
  const uint32_t nx = d.nx, nk = d.nk;
  const double g = d.g, dry = d.dry, rho = d.rho;
  const double area = d.cell_m * d.cell_m;
  const double lam = dt / d.cell_m;
  double* share = d.share;
  const uint64_t n = d.n;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t y = i / nx, x = i - y * nx;
    const uint64_t w = y * (nx + 1) + x, e = w + 1, s = i, nn = i + nx;
    const double z = d.bed[i];
    const double h0 = d.h[i];
    const double energy0 = energy(g, h0, d.u[i], d.v[i], z);
    double h = h0 - lam * ((d.fx[0][e] - d.fx[0][w]) + (d.fy[0][nn] - d.fy[0][s]));
    double mu = d.hu[i] - lam * ((d.fx[1][e] - d.fx[2][w]) + (d.fy[3][nn] - d.fy[3][s]));
    double mv = d.hv[i] - lam * ((d.fx[3][e] - d.fx[3][w]) + (d.fy[1][nn] - d.fy[2][s]));
    for (uint32_t k = 0; k < nk; ++k) {
      const double* fxc = d.fxc + k * d.xf;
      const double* fyc = d.fyc + k * d.yf;
      double& q = d.carried[k * n + i];
      q = q - lam * ((fxc[e] - fxc[w]) + (fyc[nn] - fyc[s]));
    }
    double loss;
    {
      const bool wet = h >= dry;
      const double u1 = wet ? mu / h : 0.0, v1 = wet ? mv / h : 0.0;
      const double energy1 = energy(g, h > 0.0 ? h : 0.0, u1, v1, z);
      const double through = (d.fx[4][e] - d.fx[4][w]) + (d.fy[4][nn] - d.fy[4][s]);
      loss = -rho * ((energy1 - energy0) / dt + through / d.cell_m);
    }
    share[kShareLoss * n + i] = loss * area * dt;
    double roundoff = 0.0;
    if (h < 0.0) {
      roundoff = -(h * area);  // sums.roundoff -= h * area
      h = 0.0;
    }
    share[kShareRoundoff * n + i] = roundoff;
    double src = 0.0;
    if (d.source != nullptr) {
      const double added = d.source[i] * dt;
      if (added >= 0.0) {
        h += added;
        src = added * area;
      } else {
        const double taken = -added < h ? -added : h;
        h -= taken;
        src = -(taken * area);
      }
    }
    share[kShareSource * n + i] = src;
    double grd = 0.0;
    if (d.gk != nullptr && h > 0.0) {
      const double stored = d.ground[i];
      const double room = d.gcap[i] - stored;
      if (room > 0.0) {
        const double kdt = d.gk[i] * dt;
        const double b = stored + kdt;
        const double next = 0.5 * (b + sqrt(b * b + 4.0 * kdt * d.gs[i]));
        double take = next - stored;
        take = take < h ? take : h;
        take = take < room ? take : room;
        if (take > 0.0) {
          h -= take;
          d.ground[i] = stored + take;
          grd = take * area;
        }
      }
    }
    share[kShareGround * n + i] = grd;
    double sp = 0.0, tx = 0.0, ty = 0.0, friction = 0.0;
    if (h >= dry) {
      if (d.manning != nullptr) {
        const double nnn = d.manning[i];
        const double u = mu / h, v = mv / h;
        const double s0 = sqrt(u * u + v * v);
        const double cb = fd_exp(fd_log(h) / 3.0);
        const double kk = g * nnn * nnn * s0 / (h * cb);
        const double denom = 1.0 + dt * kk;
        mu = mu / denom;
        mv = mv / denom;
        const double u1 = mu / h, v1 = mv / h;
        sp = sqrt(u1 * u1 + v1 * v1);
        const double coeff = rho * g * nnn * nnn * sp / cb;
        tx = coeff * u1;
        ty = coeff * v1;
        friction = coeff * sp * sp;
      } else {
        const double u1 = mu / h, v1 = mv / h;
        sp = sqrt(u1 * u1 + v1 * v1);
      }
    } else {
      mu = 0.0;
      mv = 0.0;
    }
    share[kShareFriction * n + i] = friction * area * dt;
    const double diss = (loss > 0.0 ? loss : 0.0) + friction;
    for (uint32_t k = 0; k < nk; ++k) {
      const Carried& cc = d.cc[k];
      double* sh = share + (kShareCarried + 4 * k) * n + i;
      double& q = d.carried[k * n + i];
      double made = 0.0, added = 0.0, moved_area = 0.0, decayed = 0.0;
      if (cc.per_joule > 0.0 && sp >= cc.min_speed) {
        const double m = cc.per_joule * diss * dt;
        q += m;
        made = m * area;
      }
      if (d.cs[k] != nullptr) {
        const double a = d.cs[k][i] * dt;
        q += a;
        added = a * area;
      }
      if (d.ce[k] != nullptr) {
        double moved = d.ce[k][i] * dt;
        if (moved < 0.0 && -moved > q) moved = -q;
        q += moved;
        moved_area = moved * area;
      }
      const double keep = c->keep[k];
      if (keep != 1.0) {
        const double kept = q * keep;
        decayed = (q - kept) * area;
        q = kept;
      }
      sh[0] = added;
      sh[n] = made;
      sh[2 * n] = moved_area;
      sh[3 * n] = decayed;
    }
    d.h[i] = h;
    d.hu[i] = mu;
    d.hv[i] = mv;
    d.speed[i] = sp;
    d.tau_x[i] = tx;
    d.tau_y[i] = ty;
    d.diss[i] = diss;
  }
}

// A row's sums (cpp:336-363 and the x loop's additions): one thread a row and quantity, in the
// reference's order. A cell that adds nothing to a sum holds +0, which leaves the sum as it is (a
// sum from +0 is never -0 in round-to-nearest).
__global__ void __launch_bounds__(kThreads) ws_rows_kernel(Desc d) {
  const Ctl* c = d.ctl;
  if (!stepping(c)) return;
  const uint32_t q_count = quantities(d);
  const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= uint64_t(d.ny) * q_count) return;
  const uint32_t y = uint32_t(t / q_count), q = uint32_t(t - uint64_t(y) * q_count);
  const uint32_t nx = d.nx, ny = d.ny;
  const double ev = c->dt * d.cell_m;  // edge_volume
  double s = 0.0;
  const bool carried = q >= kQCarried;
  const uint32_t k = carried ? (q - kQCarried) / 5u : 0u, j = carried ? (q - kQCarried) % 5u : 0u;
  if (q == kQOpen || (carried && j == 4u)) {
    const double* fxh = q == kQOpen ? d.fx[0] : d.fxc + k * d.xf;
    const double* fyh = q == kQOpen ? d.fy[0] : d.fyc + k * d.yf;
    const uint64_t frow = uint64_t(y) * (nx + 1);
    if (d.open & 1u) s -= fxh[frow] * ev;
    if (d.open & 2u) s += fxh[frow + nx] * ev;
    if (y == 0 && (d.open & 4u))
      for (uint32_t x = 0; x < nx; ++x) s -= fyh[x] * ev;
    if (y + 1 == ny && (d.open & 8u))
      for (uint32_t x = 0; x < nx; ++x) s += fyh[uint64_t(ny) * nx + x] * ev;
  } else {
    uint32_t plane;
    switch (q) {
      case kQSource: plane = kShareSource; break;
      case kQGround: plane = kShareGround; break;
      case kQRoundoff: plane = kShareRoundoff; break;
      case kQLoss: plane = kShareLoss; break;
      case kQFriction: plane = kShareFriction; break;
      default: plane = kShareCarried + 4u * k + j; break;  // source, from_dissipation, exchange, decayed
    }
    const double* p = d.share + plane * d.n + uint64_t(y) * nx;
    for (uint32_t x = 0; x < nx; ++x) s += p[x];
  }
  d.rows[t] = s;
}

// step's ledger (cpp:514-532): each quantity's rows in row order; the time and the step count.
__global__ void ws_ledger_kernel(Desc d) {
  Ctl* c = d.ctl;
  if (!stepping(c)) return;
  const uint32_t q_count = quantities(d);
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < q_count) {
    double s = c->ledger[q];
    for (uint32_t y = 0; y < d.ny; ++y) s += d.rows[uint64_t(y) * q_count + q];
    c->ledger[q] = s;
  } else if (q == q_count) {
    c->time_s += c->dt;
    c->steps += 1;
  }
}

size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

bool ok(cudaError_t e, std::string* err, const char* what) {
  if (e == cudaSuccess) return true;
  if (err) *err = std::string("water_state: ") + what + ": " + cudaGetErrorString(e);
  return false;
}

int grid_for(uint64_t work, int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const uint64_t blocks = (work + kThreads - 1) / kThreads;
  return int(std::max<uint64_t>(1, std::min<uint64_t>(blocks, uint64_t(sms > 0 ? sms : 1) * 8)));
}

}  // namespace

bool Solver::create(int device, const Desc& shape, std::string* err) {
  destroy();
  if (shape.nx == 0 || shape.ny == 0) {
    if (err) *err = "water_state: an empty grid";
    return false;
  }
  if (!ok(cudaSetDevice(device), err, "cudaSetDevice")) return false;
  device_ = device;
  if (!ok(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), err, "cudaStreamCreate"))
    return false;
  d_ = shape;
  d_.nk = std::min(shape.nk, kMaxCarried);
  const uint64_t n = uint64_t(shape.nx) * shape.ny;
  d_.n = n;
  d_.xf = uint64_t(shape.nx + 1) * shape.ny;
  d_.yf = uint64_t(shape.nx) * (shape.ny + 1);
  const uint32_t nk = d_.nk, q = 6 + 5 * nk;
  const size_t cell = align_up(n * sizeof(double));
  const size_t xf = align_up(d_.xf * sizeof(double)), yf = align_up(d_.yf * sizeof(double));
  // state 4 + nk, outputs 4, inputs 6 + 2 nk, velocities 2, shares 5 + 4 nk planes of cells
  const size_t cells = cell * (4 + nk + 4 + 6 + 2 * nk + 2 + 5 + 4 * nk);
  const size_t faces = (xf + yf) * (5 + nk);
  const size_t rows = align_up(size_t(shape.ny) * q * sizeof(double));
  const size_t ctl = align_up(sizeof(Ctl));
  bytes_ = cells + faces + rows + ctl;
  if (!ok(cudaMalloc(reinterpret_cast<void**>(&base_), bytes_), err, "cudaMalloc")) {
    base_ = nullptr;
    destroy();
    return false;
  }
  char* p = base_;
  auto take = [&p](size_t b) {
    char* r = p;
    p += b;
    return reinterpret_cast<double*>(r);
  };
  d_.h = take(cell);
  d_.hu = take(cell);
  d_.hv = take(cell);
  d_.ground = take(cell);
  d_.carried = take(cell * nk);
  d_.speed = take(cell);
  d_.tau_x = take(cell);
  d_.tau_y = take(cell);
  d_.diss = take(cell);
  double* in = take(cell * (6 + 2 * nk));
  d_.u = take(cell);
  d_.v = take(cell);
  d_.share = take(cell * (5 + 4 * nk));
  for (int j = 0; j < 5; ++j) d_.fx[j] = take(xf);
  for (int j = 0; j < 5; ++j) d_.fy[j] = take(yf);
  d_.fxc = take(xf * nk);
  d_.fyc = take(yf * nk);
  d_.rows = take(rows);
  d_.ctl = reinterpret_cast<Ctl*>(take(ctl));
  // Multi-plane arrays (carried, shares, carried fluxes) are indexed packed, plane * n; each
  // chunk is at least that large. The input planes are one 256-byte-aligned plane each, held for
  // set_input; the descriptor points at those with a span.
  in_base_ = in;
  in_stride_ = cell / sizeof(double);
  d_.bed = d_.manning = d_.source = d_.gk = d_.gs = d_.gcap = nullptr;
  for (uint32_t k = 0; k < kMaxCarried; ++k) d_.cs[k] = d_.ce[k] = nullptr;
  std::fill(std::begin(present_), std::end(present_), false);
  if (!ok(cudaMemsetAsync(base_, 0, bytes_, stream_), err, "cudaMemset") || !wait(err)) {
    destroy();
    return false;
  }
  return true;
}

void Solver::destroy() {
  if (device_ >= 0) cudaSetDevice(device_);
  if (stream_ != nullptr) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
  if (base_ != nullptr) cudaFree(base_);
  stream_ = nullptr;
  base_ = nullptr;
  bytes_ = 0;
}

bool Solver::wait(std::string* err) { return ok(cudaStreamSynchronize(stream_), err, "the device"); }

double* Solver::field(int which) const {
  switch (which) {
    case 0: return d_.h;
    case 1: return d_.hu;
    case 2: return d_.hv;
    case 3: return d_.ground;
    case 4: return d_.carried;
    case 5: return d_.speed;
    case 6: return d_.tau_x;
    case 7: return d_.tau_y;
    case 8: return d_.diss;
    default: return nullptr;
  }
}

size_t Solver::field_size(int which) const {
  if (which < 0 || which > 8) return 0;
  return size_t(d_.n) * (which == 4 ? d_.nk : 1u);
}

bool Solver::write_field(int which, const double* v, std::string* err) {
  if (which < 0 || which > 4) {
    if (err) *err = "water_state: only the state's fields are written";
    return false;
  }
  const size_t count = field_size(which);
  if (count == 0) return true;
  return ok(cudaSetDevice(device_), err, "cudaSetDevice") &&
         ok(cudaMemcpyAsync(field(which), v, count * sizeof(double), cudaMemcpyHostToDevice,
                            stream_),
            err, "upload of a field") &&
         wait(err);
}

bool Solver::read_field(int which, double* out, std::string* err) {
  const size_t count = field_size(which);
  if (count == 0) return true;
  return ok(cudaSetDevice(device_), err, "cudaSetDevice") &&
         ok(cudaMemcpyAsync(out, field(which), count * sizeof(double), cudaMemcpyDeviceToHost,
                            stream_),
            err, "read-back of a field") &&
         wait(err);
}

bool Solver::set_input(int which, const double* v, size_t n, std::string* err) {
  const int nk = int(d_.nk);
  const bool carried_ok = which < 6 || (which < 10 ? which - 6 < nk : which - 10 < nk);
  if (which < 0 || which >= 14 || !carried_ok) {
    if (err) *err = "water_state: no such input (a carried quantity's past the configured count)";
    return false;
  }
  // Plane index: 0-5 the named inputs, 6 .. 6 + nk - 1 carried sources, then carried exchanges.
  const int plane = which < 10 ? which : 6 + nk + (which - 10);
  double* dst = in_base_ + size_t(plane) * in_stride_;
  const double** target = nullptr;
  switch (which) {
    case 0: target = &d_.bed; break;
    case 1: target = &d_.manning; break;
    case 2: target = &d_.source; break;
    case 3: target = &d_.gk; break;
    case 4: target = &d_.gs; break;
    case 5: target = &d_.gcap; break;
    default: target = which < 10 ? &d_.cs[which - 6] : &d_.ce[which - 10]; break;
  }
  if (n == 0) {
    *target = nullptr;
    present_[which] = false;
    return true;
  }
  if (n != d_.n || v == nullptr) {
    if (err) *err = "water_state: an input that does not fit the grid";
    return false;
  }
  if (!ok(cudaSetDevice(device_), err, "cudaSetDevice") ||
      !ok(cudaMemcpyAsync(dst, v, n * sizeof(double), cudaMemcpyHostToDevice, stream_), err,
          "upload of an input") ||
      !wait(err))
    return false;
  *target = dst;
  present_[which] = true;
  return true;
}

bool Solver::inputs_fit() const {  // water_state.cpp:150-169
  if (d_.n == 0 || !present_[0]) return false;
  return present_[3] == present_[4] && present_[3] == present_[5];
}

cudaError_t Solver::enqueue_step(cudaStream_t s) {
  const uint32_t q = 6 + 5 * d_.nk;
  ws_speeds_kernel<<<grid_for(d_.n, device_), kThreads, 0, s>>>(d_);
  ws_length_kernel<<<1, 32, 0, s>>>(d_, 0);
  ws_faces_kernel<<<grid_for(d_.xf + d_.yf, device_), kThreads, 0, s>>>(d_);
  ws_update_kernel<<<grid_for(d_.n, device_), kThreads, 0, s>>>(d_);
  const uint64_t row_threads = uint64_t(d_.ny) * q;
  ws_rows_kernel<<<unsigned((row_threads + kThreads - 1) / kThreads), kThreads, 0, s>>>(d_);
  ws_ledger_kernel<<<1, ((q + 1 + 31) / 32) * 32, 0, s>>>(d_);
  return cudaGetLastError();
}

cudaError_t Solver::enqueue_steps(cudaStream_t s, uint32_t count, double max_dt) {
  ws_mode_kernel<<<1, 32, 0, s>>>(d_.ctl, 0u, max_dt, 0.0);
  for (uint32_t k = 0; k < count; ++k) {
    const cudaError_t e = enqueue_step(s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t Solver::enqueue_advance_start(cudaStream_t s, double duration) {
  ws_mode_kernel<<<1, 32, 0, s>>>(d_.ctl, 1u, 0.0, duration);
  return cudaGetLastError();
}

cudaError_t Solver::enqueue_advance_steps(cudaStream_t s, uint32_t count) {
  for (uint32_t k = 0; k < count; ++k) {
    const cudaError_t e = enqueue_step(s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t Solver::enqueue_stable_step(cudaStream_t s) {
  ws_mode_kernel<<<1, 32, 0, s>>>(d_.ctl, 0u, 0.0, 0.0);
  ws_speeds_kernel<<<grid_for(d_.n, device_), kThreads, 0, s>>>(d_);
  ws_length_kernel<<<1, 32, 0, s>>>(d_, 1);
  return cudaGetLastError();
}

bool Solver::read_ctl(Ctl& out, std::string* err) {
  return ok(cudaSetDevice(device_), err, "cudaSetDevice") &&
         ok(cudaMemcpyAsync(&out, d_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), err,
            "read-back of the ledger") &&
         wait(err);
}

bool Solver::reset_ledger(std::string* err) {
  Ctl c;
  if (!read_ctl(c, err)) return false;
  std::memset(c.ledger, 0, sizeof c.ledger);
  c.time_s = 0.0;
  c.steps = 0;
  return ok(cudaMemcpyAsync(d_.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), err,
            "upload of the ledger") &&
         wait(err);
}

}  // namespace wsc

// ---- the C ABI (wlcuda.h, "the complete FP64 step") ---------------------------------------------

static_assert(sizeof(ws_config) == 160, "ws_config layout");
static_assert(sizeof(ws_ledger) == 224, "ws_ledger layout");

struct ws_solver {
  wsc::Solver s;
  ws_config config{};
};

namespace {

int ws_fail(char* err, size_t len, int code, const std::string& msg) {
  if (err != nullptr && len > 0) {
    const size_t k = msg.size() < len - 1 ? msg.size() : len - 1;
    std::memcpy(err, msg.data(), k);
    err[k] = '\0';
  }
  return code;
}

bool ws_valid_handle(const ws_solver* s) { return s != nullptr && s->s.valid(); }
const char* k_ws_none = "water_state: no solver";

uint64_t fnv_bytes(uint64_t h, const double* v, size_t n) {  // water_state.cpp:97-107
  for (size_t i = 0; i < n; ++i) {
    uint64_t bits = 0;
    std::memcpy(&bits, v + i, sizeof bits);
    for (int b = 0; b < 8; ++b) {
      h ^= (bits >> (8 * b)) & 0xffu;
      h *= 0x100000001b3ull;
    }
  }
  return h;
}

// The sum in index order, then times a cell's area (water_state.cpp:549-568).
double volume(ws_solver* s, int which, uint32_t k, char* err, size_t len) {
  const wsc::Desc& d = s->s.desc();
  std::vector<double> v(s->s.field_size(which));
  std::string msg;
  if (!s->s.read_field(which, v.data(), &msg)) {
    ws_fail(err, len, WL_ERR_CUDA, msg);
    return 0.0;
  }
  const size_t first = which == 4 ? size_t(k) * d.n : 0, count = which == 4 ? d.n : v.size();
  double sum = 0.0;
  for (size_t i = 0; i < count; ++i) sum += v[first + i];
  return sum * (d.cell_m * d.cell_m);
}

}  // namespace

extern "C" {

int ws_create(const ws_config* c, ws_solver** out, char* err, size_t err_len) {
  if (out == nullptr) return ws_fail(err, err_len, WL_ERR_ARGUMENT, "water_state: no handle to fill");
  *out = nullptr;
  if (c == nullptr) return ws_fail(err, err_len, WL_ERR_ARGUMENT, "water_state: no config");
  if (c->nx == 0 || c->ny == 0) return ws_fail(err, err_len, WL_ERR_SIZE, "water_state: an empty grid");
  if (c->carried > wsc::kMaxCarried)
    return ws_fail(err, err_len, WL_ERR_ARGUMENT, "water_state: at most 4 carried quantities");
  wsc::Desc shape{};
  shape.nx = c->nx;
  shape.ny = c->ny;
  shape.nk = c->carried;
  shape.open = (c->west_open ? 1u : 0u) | (c->east_open ? 2u : 0u) | (c->south_open ? 4u : 0u) |
               (c->north_open ? 8u : 0u);
  shape.cell_m = c->cell_m;
  shape.g = c->gravity;
  shape.cfl = c->cfl;
  shape.dry = c->dry_depth_m;
  shape.rho = c->water_density;
  for (uint32_t k = 0; k < wsc::kMaxCarried; ++k)
    shape.cc[k] = {c->carried_config[k].decay_s, c->carried_config[k].per_joule,
                   c->carried_config[k].min_speed_m_per_s};
  auto* s = new (std::nothrow) ws_solver;
  if (s == nullptr) return ws_fail(err, err_len, WL_ERR_ALLOC, "water_state: host memory");
  std::string msg;
  if (!s->s.create(c->device, shape, &msg)) {
    delete s;
    return ws_fail(err, err_len, msg.find("cudaMalloc") != std::string::npos ? WL_ERR_ALLOC
                                                                              : WL_ERR_CUDA,
                   msg);
  }
  s->config = *c;
  *out = s;
  return WL_OK;
}

void ws_destroy(ws_solver* s) { delete s; }

int ws_valid(const ws_solver* s) { return ws_valid_handle(s) ? 1 : 0; }

uint32_t ws_cell_count(const ws_solver* s) {
  return ws_valid_handle(s) ? uint32_t(s->s.desc().n) : 0u;
}

int ws_write_field(ws_solver* s, int field, const double* v, size_t n, char* err, size_t len) {
  if (!ws_valid_handle(s)) return ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
  if (field < WS_DEPTH || field > WS_CARRIED)
    return ws_fail(err, len, WL_ERR_ARGUMENT, "water_state: only the state's fields are written");
  if (n != s->s.field_size(field) || (n > 0 && v == nullptr))
    return ws_fail(err, len, WL_ERR_SIZE, "water_state: a field that does not fit the grid");
  std::string msg;
  return s->s.write_field(field, v, &msg) ? WL_OK : ws_fail(err, len, WL_ERR_CUDA, msg);
}

int ws_read_field(ws_solver* s, int field, double* out, size_t n, char* err, size_t len) {
  if (!ws_valid_handle(s)) return ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
  if (field < WS_DEPTH || field > WS_DISSIPATION)
    return ws_fail(err, len, WL_ERR_ARGUMENT, "water_state: no such field");
  if (n != s->s.field_size(field) || (n > 0 && out == nullptr))
    return ws_fail(err, len, WL_ERR_SIZE, "water_state: a field that does not fit the grid");
  std::string msg;
  return s->s.read_field(field, out, &msg) ? WL_OK : ws_fail(err, len, WL_ERR_CUDA, msg);
}

int ws_set_input(ws_solver* s, int input, const double* v, size_t n, char* err, size_t len) {
  if (!ws_valid_handle(s)) return ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
  std::string msg;
  if (s->s.set_input(input, v, n, &msg)) return WL_OK;
  const int code = msg.find("does not fit") != std::string::npos ? WL_ERR_SIZE
                   : msg.find("no such") != std::string::npos    ? WL_ERR_ARGUMENT
                                                                 : WL_ERR_CUDA;
  return ws_fail(err, len, code, msg);
}

double ws_stable_step(ws_solver* s, char* err, size_t len) {
  if (!ws_valid_handle(s)) {
    ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
    return 0.0;
  }
  wsc::Ctl c;
  std::string msg;
  if (cudaSetDevice(s->s.device()) != cudaSuccess ||
      s->s.enqueue_stable_step(s->s.stream()) != cudaSuccess || !s->s.read_ctl(c, &msg)) {
    ws_fail(err, len, WL_ERR_CUDA, msg.empty() ? "water_state: the stable step" : msg);
    return 0.0;
  }
  return c.stable;
}

int ws_enqueue_steps(ws_solver* s, wl_stream stream, uint32_t count, double max_dt) {
  if (!ws_valid_handle(s)) return WL_ERR_INVALID;
  if (!s->s.inputs_fit()) return WL_ERR_SIZE;
  if (!(max_dt > 0.0)) return WL_ERR_ARGUMENT;
  cudaStream_t st = stream == nullptr ? s->s.stream() : reinterpret_cast<cudaStream_t>(stream);
  if (cudaSetDevice(s->s.device()) != cudaSuccess) return WL_ERR_CUDA;
  return s->s.enqueue_steps(st, count, max_dt) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int ws_run_steps(ws_solver* s, uint32_t count, double max_dt, char* err, size_t len) {
  if (!ws_valid_handle(s)) return ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
  if (!s->s.inputs_fit())
    return ws_fail(err, len, WL_ERR_SIZE, "water_state: the inputs do not fit (no bed, or a partial ground)");
  if (!(max_dt > 0.0)) return ws_fail(err, len, WL_ERR_ARGUMENT, "water_state: max_dt <= 0");
  std::string msg;
  if (cudaSetDevice(s->s.device()) != cudaSuccess ||
      s->s.enqueue_steps(s->s.stream(), count, max_dt) != cudaSuccess || !s->s.wait(&msg))
    return ws_fail(err, len, WL_ERR_CUDA, msg.empty() ? "water_state: the steps" : msg);
  return WL_OK;
}

// Solver::step (cpp:503-533): the length taken, 0 when the inputs do not fit or max_dt <= 0.
double ws_step(ws_solver* s, double max_dt, char* err, size_t len) {
  if (!ws_valid_handle(s)) {
    ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
    return 0.0;
  }
  if (!s->s.inputs_fit() || !(max_dt > 0.0)) return 0.0;
  wsc::Ctl c;
  std::string msg;
  if (cudaSetDevice(s->s.device()) != cudaSuccess ||
      s->s.enqueue_steps(s->s.stream(), 1, max_dt) != cudaSuccess || !s->s.read_ctl(c, &msg)) {
    ws_fail(err, len, WL_ERR_CUDA, msg.empty() ? "water_state: the step" : msg);
    return 0.0;
  }
  return c.dt;
}

// Solver::advance (cpp:535-547): the steps taken, 0 when the inputs do not fit. The device counts
// the time down and stops itself; the host enqueues batches until it has.
uint64_t ws_advance(ws_solver* s, double duration, char* err, size_t len) {
  if (!ws_valid_handle(s)) {
    ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
    return 0;
  }
  if (!s->s.inputs_fit()) return 0;
  constexpr uint32_t kBatch = 32;
  constexpr uint32_t kMostBatches = 1u << 20;
  std::string msg;
  wsc::Ctl c;
  if (cudaSetDevice(s->s.device()) != cudaSuccess ||
      s->s.enqueue_advance_start(s->s.stream(), duration) != cudaSuccess) {
    ws_fail(err, len, WL_ERR_CUDA, "water_state: the advance");
    return 0;
  }
  for (uint32_t b = 0; b < kMostBatches; ++b) {
    if (s->s.enqueue_advance_steps(s->s.stream(), kBatch) != cudaSuccess ||
        !s->s.read_ctl(c, &msg)) {
      ws_fail(err, len, WL_ERR_CUDA, msg.empty() ? "water_state: the advance" : msg);
      return 0;
    }
    if (c.active == 0u) return c.taken;
  }
  ws_fail(err, len, WL_ERR_UNFINISHED, "water_state: the advance did not finish");
  return 0;
}

int ws_read_ledger(ws_solver* s, ws_ledger* out, char* err, size_t len) {
  if (!ws_valid_handle(s)) return ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
  if (out == nullptr) return ws_fail(err, len, WL_ERR_ARGUMENT, "water_state: no ledger");
  wsc::Ctl c;
  std::string msg;
  if (!s->s.read_ctl(c, &msg)) return ws_fail(err, len, WL_ERR_CUDA, msg);
  std::memset(out, 0, sizeof *out);
  out->source_m3 = c.ledger[wsc::kQSource];
  out->open_edge_out_m3 = c.ledger[wsc::kQOpen];
  out->ground_m3 = c.ledger[wsc::kQGround];
  out->roundoff_m3 = c.ledger[wsc::kQRoundoff];
  out->scheme_loss_j = c.ledger[wsc::kQLoss];
  out->friction_work_j = c.ledger[wsc::kQFriction];
  out->time_s = c.time_s;
  out->steps = c.steps;
  for (uint32_t k = 0; k < s->s.desc().nk; ++k) {
    const double* q = c.ledger + wsc::kQCarried + 5 * k;
    out->carried[k] = ws_carried_ledger{q[0], q[1], q[2], q[3], q[4]};
  }
  return WL_OK;
}

int ws_reset_ledger(ws_solver* s, char* err, size_t len) {
  if (!ws_valid_handle(s)) return ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
  std::string msg;
  return s->s.reset_ledger(&msg) ? WL_OK : ws_fail(err, len, WL_ERR_CUDA, msg);
}

double ws_surface_volume_m3(ws_solver* s, char* err, size_t len) {
  if (!ws_valid_handle(s)) {
    ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
    return 0.0;
  }
  return volume(s, WS_DEPTH, 0, err, len);
}

double ws_ground_volume_m3(ws_solver* s, char* err, size_t len) {
  if (!ws_valid_handle(s)) {
    ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
    return 0.0;
  }
  return volume(s, WS_GROUND, 0, err, len);
}

double ws_carried_total(ws_solver* s, uint32_t k, char* err, size_t len) {
  if (!ws_valid_handle(s) || k >= s->s.desc().nk) {
    ws_fail(err, len, WL_ERR_INVALID, "water_state: no solver, or no such carried quantity");
    return 0.0;
  }
  return volume(s, WS_CARRIED, k, err, len);
}

// Solver::state_hash (cpp:570-578): FNV-1a over depth, the momenta, the ground, the carried.
uint64_t ws_state_hash(ws_solver* s, char* err, size_t len) {
  if (!ws_valid_handle(s)) {
    ws_fail(err, len, WL_ERR_INVALID, k_ws_none);
    return 0;
  }
  uint64_t h = 0xcbf29ce484222325ull;
  std::string msg;
  for (int f = WS_DEPTH; f <= WS_CARRIED; ++f) {
    std::vector<double> v(s->s.field_size(f));
    if (!s->s.read_field(f, v.data(), &msg)) {
      ws_fail(err, len, WL_ERR_CUDA, msg);
      return 0;
    }
    h = fnv_bytes(h, v.data(), v.size());
  }
  return h;
}

wl_stream ws_stream(ws_solver* s) {
  return ws_valid_handle(s) ? reinterpret_cast<wl_stream>(s->s.stream()) : nullptr;
}

uint64_t ws_device_bytes(const ws_solver* s) { return ws_valid_handle(s) ? s->s.device_bytes() : 0; }

}  // extern "C"

// ORACLE — test infrastructure only (see wl_oracle.hpp).
//
// The reverse (adjoint) tick of the card's step, on the CPU: the vector-Jacobian product of one
// tick of RefStep<T> (water_step.slang's update_main with a fixed step length) with respect to the
// state, the bed and the per-cell source. The reference has no adjoint; this is the FP64 reference
// gradient the GPU's reverse tick is held to, and, instantiated with float, a restatement of the
// GPU's arithmetic for its own checks.
//
// Differentiation rules (the scheme is not smooth everywhere):
//   - the face's flux is differentiated through the central-upwind formula even where the forward
//     takes the identical-state shortcut (the two agree in value, and at identical states the
//     flux does not depend on the one-sided speeds, so the choice among ties does not matter);
//   - a face whose span is not positive carries no flux and no derivative but the pressure terms;
//   - max/min and clamps pass the derivative to the argument the forward selected;
//   - sqrt at zero depth passes nothing (its derivative is infinite there);
//   - the dry test, the negative-depth clamp and a sink limited by the water pass the branch the
//     forward took;
//   - the step's length is fixed (no tick may be limited by the stability bound).
#pragma once

#include "wl_oracle.hpp"

namespace wl_oracle {

template <class T>
struct FaceIn { T hl0, zl, ln, lt, hr0, zr, rn, rt; };

// The face's vector-Jacobian product: given bars of its outputs {h, nl, nr, t}, the bars of its
// eight inputs (slang:204-292 differentiated).
template <class T>
inline FaceIn<T> face_vjp(T g, const FaceIn<T>& in, T bh, T bnl, T bnr, T bt) {
  FaceIn<T> out{0, 0, 0, 0, 0, 0, 0, 0};
  const bool pick_l = in.zl > in.zr;
  const T zf = pick_l ? in.zl : in.zr;
  const T el = (in.hl0 + in.zl) - zf;
  const T er = (in.hr0 + in.zr) - zf;
  const bool al = el > T(0), ar = er > T(0);
  const T hl = al ? el : T(0), hr = ar ? er : T(0);
  const T ul = in.ln, vl = in.lt, ur = in.rn, vr = in.rt;
  T bhl = 0, bhr = 0, bul = 0, bvl = 0, bur = 0, bvr = 0;
  // nl = Fn - pl, nr = Fn - pr, p = g/2 h^2
  const T bFn = bnl + bnr;
  bhl += -bnl * g * hl;
  bhr += -bnr * g * hr;
  const T cl = std::sqrt(g * hl), cr = std::sqrt(g * hr);
  const T a1 = ur + cr, a2 = ul + cl;
  const int ap_src = (a1 > a2 ? a1 : a2) > T(0) ? (a1 > a2 ? 1 : 2) : 0;
  const T ap = ap_src == 1 ? a1 : ap_src == 2 ? a2 : T(0);
  const T b1 = ur - cr, b2 = ul - cl;
  const int am_src = (b1 < b2 ? b1 : b2) < T(0) ? (b1 < b2 ? 1 : 2) : 0;
  const T am = am_src == 1 ? b1 : am_src == 2 ? b2 : T(0);
  const T span = ap - am;
  if (span > T(0)) {
    const T pl = T(0.5) * g * hl * hl, pr = T(0.5) * g * hr * hr;
    const T ql = hl * ul, qr = hr * ur, apam = ap * am;
    const T Al = ql * ul + pl, Ar = qr * ur + pr;
    const T Tl = ql * vl, Tr = qr * vr, D = hr * vr - hl * vl;
    const T Nh = ap * ql - am * qr + apam * (hr - hl);
    const T Nn = ap * Al - am * Ar + apam * (qr - ql);
    const T Nt = ap * Tl - am * Tr + apam * D;
    const T inv = T(1) / span;
    const T Fh = Nh * inv, Fn = Nn * inv, Ft = Nt * inv;
    const T bNh = bh * inv, bNn = bFn * inv, bNt = bt * inv;
    const T bspan = -(bh * Fh + bFn * Fn + bt * Ft) * inv;
    T bap = bspan, bam = -bspan;
    T bql = 0, bqr = 0;
    bap += bNh * (ql + am * (hr - hl));
    bam += bNh * (-qr + ap * (hr - hl));
    bql += bNh * ap;
    bqr += -bNh * am;
    bhr += bNh * apam;
    bhl += -bNh * apam;
    bap += bNn * (Al + am * (qr - ql));
    bam += bNn * (-Ar + ap * (qr - ql));
    const T bAl = bNn * ap, bAr = -bNn * am;
    bqr += bNn * apam;
    bql += -bNn * apam;
    bql += bAl * ul;
    bul += bAl * ql;
    bhl += bAl * g * hl;
    bqr += bAr * ur;
    bur += bAr * qr;
    bhr += bAr * g * hr;
    bap += bNt * (Tl + am * D);
    bam += bNt * (-Tr + ap * D);
    const T bTl = bNt * ap, bTr = -bNt * am, bD = bNt * apam;
    bql += bTl * vl;
    bvl += bTl * ql;
    bqr += bTr * vr;
    bvr += bTr * qr;
    bhr += bD * vr;
    bvr += bD * hr;
    bhl += -bD * vl;
    bvl += -bD * hl;
    bhl += bql * ul;
    bul += bql * hl;
    bhr += bqr * ur;
    bur += bqr * hr;
    T bcl = 0, bcr = 0;
    if (ap_src == 1) { bur += bap; bcr += bap; }
    if (ap_src == 2) { bul += bap; bcl += bap; }
    if (am_src == 1) { bur += bam; bcr -= bam; }
    if (am_src == 2) { bul += bam; bcl -= bam; }
    if (cl > T(0)) bhl += bcl * g / (T(2) * cl);
    if (cr > T(0)) bhr += bcr * g / (T(2) * cr);
  }
  const T bel = al ? bhl : T(0), ber = ar ? bhr : T(0);
  out.hl0 = bel;
  out.zl = bel;
  out.hr0 = ber;
  out.zr = ber;
  const T bzf = -bel - ber;
  if (pick_l) out.zl += bzf; else out.zr += bzf;
  out.ln = bul;
  out.lt = bvl;
  out.rn = bur;
  out.rt = bvr;
  return out;
}

// One tick's branch record per cell, as the forward took it: the update's depth before the clamp
// was negative; the sink took all the water; the cell ended wet.
enum : u8 { kBranchClamp = 1, kBranchSinkLimited = 2, kBranchWet = 4 };

// The forward tick at a fixed length dt (RefStep's update, the source on every step, no Manning,
// no compensation), with the branch record. `in`, `out`: 3 planes (h, hu, hv). Each face is
// computed once into a face array; the face function is deterministic, so the bytes equal the
// gather form's (which computes each interior face twice).
template <class T>
void forward_tick(const Config& c, T dt, const T* bed, const T* src, const T* in, T* out,
                  u8* branch) {
  Ops<T> ops;
  const u32 nx = c.nx, ny = c.ny;
  const size_t n = size_t(nx) * ny;
  const T g = T(c.gravity), dry = T(c.dry_depth_m), cell_m = T(c.cell_m);
  std::vector<T> u(n), v(n);
  for (size_t i = 0; i < n; ++i) {  // load_cell (slang:303-314)
    const bool wet = in[i] >= dry;
    u[i] = wet ? in[n + i] / in[i] : T(0);
    v[i] = wet ? in[2 * n + i] / in[i] : T(0);
  }
  const T sw = c.west_open ? T(1) : T(-1), se = c.east_open ? T(1) : T(-1);
  const T ss = c.south_open ? T(1) : T(-1), sn = c.north_open ? T(1) : T(-1);
  // x faces: row y, face f between columns f - 1 and f (ghosts at f = 0 and f = nx)
  std::vector<Face<T>> fx(size_t(nx + 1) * ny), fy(size_t(ny + 1) * nx);
  for (u32 y = 0; y < ny; ++y)
    for (u32 f = 0; f <= nx; ++f) {
      const size_t l = size_t(y) * nx + (f == 0 ? 0 : f - 1), r = size_t(y) * nx + (f == nx ? nx - 1 : f);
      const T ln = f == 0 ? sw * u[l] : u[l], rn = f == nx ? se * u[r] : u[r];
      fx[size_t(y) * (nx + 1) + f] = face(ops, g, in[l], bed[l], ln, v[l], in[r], bed[r], rn, v[r]);
    }
  // y faces: face row f between rows f - 1 and f
  for (u32 f = 0; f <= ny; ++f)
    for (u32 x = 0; x < nx; ++x) {
      const size_t s = size_t(f == 0 ? 0 : f - 1) * nx + x, nn = size_t(f == ny ? ny - 1 : f) * nx + x;
      const T sv = f == 0 ? ss * v[s] : v[s], nv = f == ny ? sn * v[nn] : v[nn];
      fy[size_t(f) * nx + x] = face(ops, g, in[s], bed[s], sv, u[s], in[nn], bed[nn], nv, u[nn]);
    }
  const T lam = dt / cell_m;
  for (u32 y = 0; y < ny; ++y)
    for (u32 x = 0; x < nx; ++x) {
      const size_t i = size_t(y) * nx + x;
      const Face<T>& fw = fx[size_t(y) * (nx + 1) + x];
      const Face<T>& fe = fx[size_t(y) * (nx + 1) + x + 1];
      const Face<T>& fs = fy[size_t(y) * nx + x];
      const Face<T>& fn = fy[size_t(y + 1) * nx + x];
      // slang:653-668, the reference's operand order
      T h = in[i] - lam * ((fe.h - fw.h) + (fn.h - fs.h));
      T hu = in[n + i] - lam * ((fe.nl - fw.nr) + (fn.t - fs.t));
      T hv = in[2 * n + i] - lam * ((fe.t - fw.t) + (fn.nl - fs.nr));
      u8 b = 0;
      if (h < T(0)) { h = T(0); b |= kBranchClamp; }
      if (src != nullptr) {  // slang:700-715 with every = 1 (scale 1)
        const T added = src[i] * dt;
        if (added >= T(0)) {
          h = h + added;
        } else {
          const T want = -added;
          if (!(want < h)) b |= kBranchSinkLimited;
          const T taken = want < h ? want : h;
          h = h - taken;
        }
      }
      if (h >= dry) b |= kBranchWet;
      else { hu = T(0); hv = T(0); }
      out[i] = h;
      out[n + i] = hu;
      out[2 * n + i] = hv;
      if (branch) branch[i] = b;
    }
}

// The largest |u| + c and |v| + c of a state (cell_speeds, slang:317-326, folded by max), and
// whether the step the card would choose from them (slang:464-467) is shorter than dt.
template <class T>
bool limited(const Config& c, T dt, const T* st) {
  Ops<T> ops;
  const size_t n = size_t(c.nx) * c.ny;
  const T g = T(c.gravity), dry = T(c.dry_depth_m);
  T a = 0, b = 0;
  for (size_t i = 0; i < n; ++i) {
    const bool wet = st[i] >= dry;
    const T uu = wet ? ops.div(st[n + i], st[i]) : T(0), vv = wet ? ops.div(st[2 * n + i], st[i]) : T(0);
    const T cc = ops.sqrt(g * st[i]);
    a = max2(a, T(std::fabs(uu) + cc));
    b = max2(b, T(std::fabs(vv) + cc));
  }
  const T speed = a + b;
  if (!(speed > T(0))) return false;
  const T stable = ops.div(T(c.cfl) * T(c.cell_m), speed);
  return min2(stable, dt) != dt;
}

// One reverse tick: lam_out = (dF/dU)^T lam_in at the state `in` (with the tick's branch record),
// g_bed += (dF/dz)^T lam_in, g_src += (dF/ds)^T lam_in.
template <class T>
void reverse_tick(const Config& c, T dt, const T* bed, const T* src, const T* in, const u8* branch,
                  const T* lam_in, T* lam_out, double* g_bed, double* g_src) {
  const u32 nx = c.nx, ny = c.ny;
  const size_t n = size_t(nx) * ny;
  const T g = T(c.gravity), dry = T(c.dry_depth_m), cell_m = T(c.cell_m);
  const T lam = dt / cell_m;
  std::vector<T> u(n), v(n), mh(n), mu(n), mv(n);
  std::vector<T> bh(n, T(0)), bz(n, T(0)), bu(n, T(0)), bv(n, T(0));
  for (size_t i = 0; i < n; ++i) {
    const bool wet = in[i] >= dry;
    u[i] = wet ? in[n + i] / in[i] : T(0);
    v[i] = wet ? in[2 * n + i] / in[i] : T(0);
    const u8 b = branch[i];
    const bool pass = !(b & kBranchSinkLimited);
    T m = pass ? lam_in[i] : T(0);
    if (src != nullptr && pass) g_src[i] += double(lam_in[i]) * double(dt);
    if (b & kBranchClamp) m = T(0);
    mh[i] = m;
    mu[i] = (b & kBranchWet) ? lam_in[n + i] : T(0);
    mv[i] = (b & kBranchWet) ? lam_in[2 * n + i] : T(0);
  }
  const T sw = c.west_open ? T(1) : T(-1), se = c.east_open ? T(1) : T(-1);
  const T ss = c.south_open ? T(1) : T(-1), sn = c.north_open ? T(1) : T(-1);
  // x faces: face f of row y between l = f - 1 and r = f (ghosts at f = 0 and f = nx)
  for (u32 y = 0; y < ny; ++y)
    for (u32 f = 0; f <= nx; ++f) {
      const bool west = f == 0, east = f == nx;
      const size_t l = size_t(y) * nx + (west ? 0 : f - 1), r = size_t(y) * nx + (east ? nx - 1 : f);
      FaceIn<T> fi{in[l], bed[l], west ? sw * u[l] : u[l], v[l],
                   in[r], bed[r], east ? se * u[r] : u[r], v[r]};
      // the face is l's east face (unless l is a ghost) and r's west face (unless r is a ghost)
      T fbh = 0, fbnl = 0, fbnr = 0, fbt = 0;
      if (!west) { fbh += -lam * mh[l]; fbnl += -lam * mu[l]; fbt += -lam * mv[l]; }
      if (!east) { fbh += lam * mh[r]; fbnr += lam * mu[r]; fbt += lam * mv[r]; }
      const FaceIn<T> b = face_vjp(g, fi, fbh, fbnl, fbnr, fbt);
      bh[l] += b.hl0; bz[l] += b.zl; bu[l] += west ? sw * b.ln : b.ln; bv[l] += b.lt;
      bh[r] += b.hr0; bz[r] += b.zr; bu[r] += east ? se * b.rn : b.rn; bv[r] += b.rt;
    }
  // y faces: face row f between s = row f - 1 and n = row f
  for (u32 f = 0; f <= ny; ++f)
    for (u32 x = 0; x < nx; ++x) {
      const bool south = f == 0, north = f == ny;
      const size_t s = size_t(south ? 0 : f - 1) * nx + x, nn = size_t(north ? ny - 1 : f) * nx + x;
      FaceIn<T> fi{in[s], bed[s], south ? ss * v[s] : v[s], u[s],
                   in[nn], bed[nn], north ? sn * v[nn] : v[nn], u[nn]};
      T fbh = 0, fbnl = 0, fbnr = 0, fbt = 0;
      if (!south) { fbh += -lam * mh[s]; fbt += -lam * mu[s]; fbnl += -lam * mv[s]; }
      if (!north) { fbh += lam * mh[nn]; fbt += lam * mu[nn]; fbnr += lam * mv[nn]; }
      const FaceIn<T> b = face_vjp(g, fi, fbh, fbnl, fbnr, fbt);
      bh[s] += b.hl0; bz[s] += b.zl; bv[s] += south ? ss * b.ln : b.ln; bu[s] += b.lt;
      bh[nn] += b.hr0; bz[nn] += b.zr; bv[nn] += north ? sn * b.rn : b.rn; bu[nn] += b.rt;
    }
  for (size_t i = 0; i < n; ++i) {
    const bool wet = in[i] >= dry;
    T lh = mh[i] + bh[i], lu = mu[i], lv = mv[i];
    if (wet) {
      lh = lh - (bu[i] * u[i] + bv[i] * v[i]) / in[i];
      lu = lu + bu[i] / in[i];
      lv = lv + bv[i] / in[i];
    }
    lam_out[i] = lh;
    lam_out[n + i] = lu;
    lam_out[2 * n + i] = lv;
    g_bed[i] += double(bz[i]);
  }
}

// The loss L = sum over probes (h_T(p) - target_p)^2 and the gradients with respect to the bed
// and the source after `ticks` ticks of length dt from state0 (3 planes), the whole trajectory
// kept (small cases). Returns the number of ticks whose stable length was shorter than dt (the
// card would have shortened them; the gradient then is of a different trajectory).
template <class T>
u32 adjoint(const Config& c, double dt_d, u32 ticks, const double* bed_d, const double* src_d,
             const double* state0, const u32* probes, const double* targets, u32 n_probes,
             double* loss, double* g_bed, double* g_src, double* g_state0 = nullptr) {
  const size_t n = size_t(c.nx) * c.ny;
  const T dt = T(dt_d);
  std::vector<T> bed(n), src;
  for (size_t i = 0; i < n; ++i) bed[i] = T(bed_d[i]);
  if (src_d) {
    src.resize(n);
    for (size_t i = 0; i < n; ++i) src[i] = T(src_d[i]);
  }
  std::vector<T> traj(size_t(ticks + 1) * 3 * n);
  std::vector<u8> branch(size_t(ticks) * n);
  for (size_t i = 0; i < 3 * n; ++i) traj[i] = T(state0[i]);
  u32 n_limited = 0;
  for (u32 t = 0; t < ticks; ++t) {
    const T* in = &traj[size_t(t) * 3 * n];
    if (limited<T>(c, dt, in)) ++n_limited;
    forward_tick<T>(c, dt, bed.data(), src_d ? src.data() : nullptr, in,
                    &traj[size_t(t + 1) * 3 * n], &branch[size_t(t) * n]);
  }
  const T* last = &traj[size_t(ticks) * 3 * n];
  double L = 0.0;
  std::vector<T> lam(3 * n, T(0)), lam2(3 * n, T(0));
  for (u32 p = 0; p < n_probes; ++p) {
    const double d = double(last[probes[p]]) - targets[p];
    L += d * d;
    lam[probes[p]] += T(2.0 * d);
  }
  *loss = L;
  for (size_t i = 0; i < n; ++i) { g_bed[i] = 0.0; if (g_src) g_src[i] = 0.0; }
  std::vector<double> dummy(n);
  for (u32 t = ticks; t-- > 0;) {
    reverse_tick<T>(c, dt, bed.data(), src_d ? src.data() : nullptr, &traj[size_t(t) * 3 * n],
                    &branch[size_t(t) * n], lam.data(), lam2.data(), g_bed,
                    g_src ? g_src : dummy.data());
    lam.swap(lam2);
  }
  // The adjoint state of tick 0: the gradient with respect to the starting state (h, hu, hv).
  if (g_state0 != nullptr)
    for (size_t i = 0; i < 3 * n; ++i) g_state0[i] = double(lam[i]);
  return n_limited;
}

// The FP32 forward with the FP64 reverse sweep over it (each state widened): separates the error
// the FP32 trajectory brings into the gradient from the error of FP32 reverse arithmetic.
inline u32 adjoint_mixed(const Config& c, double dt_d, u32 ticks, const double* bed_d,
                         const double* src_d, const double* state0, const u32* probes,
                         const double* targets, u32 n_probes, double* loss, double* g_bed,
                         double* g_src) {
  const size_t n = size_t(c.nx) * c.ny;
  const float dt = float(dt_d);
  std::vector<float> bed(n), src;
  std::vector<double> bedw(n), srcw;
  for (size_t i = 0; i < n; ++i) { bed[i] = float(bed_d[i]); bedw[i] = double(bed[i]); }
  if (src_d) {
    src.resize(n);
    srcw.resize(n);
    for (size_t i = 0; i < n; ++i) { src[i] = float(src_d[i]); srcw[i] = double(src[i]); }
  }
  std::vector<float> traj(size_t(ticks + 1) * 3 * n);
  std::vector<u8> branch(size_t(ticks) * n);
  for (size_t i = 0; i < 3 * n; ++i) traj[i] = float(state0[i]);
  u32 n_limited = 0;
  for (u32 t = 0; t < ticks; ++t) {
    const float* in = &traj[size_t(t) * 3 * n];
    if (limited<float>(c, dt, in)) ++n_limited;
    forward_tick<float>(c, dt, bed.data(), src_d ? src.data() : nullptr, in,
                        &traj[size_t(t + 1) * 3 * n], &branch[size_t(t) * n]);
  }
  const float* last = &traj[size_t(ticks) * 3 * n];
  double L = 0.0;
  std::vector<double> lam(3 * n, 0.0), lam2(3 * n, 0.0), st(3 * n);
  for (u32 p = 0; p < n_probes; ++p) {
    const double d = double(last[probes[p]]) - targets[p];
    L += d * d;
    lam[probes[p]] += 2.0 * d;
  }
  *loss = L;
  for (size_t i = 0; i < n; ++i) { g_bed[i] = 0.0; g_src[i] = 0.0; }
  for (u32 t = ticks; t-- > 0;) {
    const float* in = &traj[size_t(t) * 3 * n];
    for (size_t i = 0; i < 3 * n; ++i) st[i] = double(in[i]);
    reverse_tick<double>(c, double(dt), bedw.data(), src_d ? srcw.data() : nullptr, st.data(),
                         &branch[size_t(t) * n], lam.data(), lam2.data(), g_bed, g_src);
    lam.swap(lam2);
  }
  return n_limited;
}

// The loss alone, in double: for finite differences (the FP64 replay).
inline double loss_fp64(const Config& c, double dt, u32 ticks, const double* bed,
                        const double* src, const double* state0, const u32* probes,
                        const double* targets, u32 n_probes) {
  const size_t n = size_t(c.nx) * c.ny;
  std::vector<double> a(state0, state0 + 3 * n), b(3 * n);
  for (u32 t = 0; t < ticks; ++t) {
    forward_tick<double>(c, dt, bed, src, a.data(), b.data(), nullptr);
    a.swap(b);
  }
  double L = 0.0;
  for (u32 p = 0; p < n_probes; ++p) {
    const double d = a[probes[p]] - targets[p];
    L += d * d;
  }
  return L;
}

}  // namespace wl_oracle

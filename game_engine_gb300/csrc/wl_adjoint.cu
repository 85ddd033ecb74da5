// The adjoint's kernels and its sweep (sm_103a).
//
// The forward march here is the plain tick's update (water_step.slang:555-757 through wl_device.cuh's
// face) at a fixed step length, with every operation spelled as a correctly rounded intrinsic, so
// its bytes equal the plain tick's whatever the contraction flag; it keeps no records and writes
// into the sweep's checkpoints and segment stack instead of the tile's two copies.
//
// The reverse march is the vector-Jacobian product of that update, and is not bit-held to anything:
// it is the FP32 derivative of the FP32 forward, with the gradients accumulated in FP64. It takes
// the forward's reconstruction (velocities, one-sided speeds) with the forward's IEEE operations so
// that its branches are the forward's, and the derivative-only quantities with fast reciprocals and
// contraction. Differentiation rules, matching the oracle's:
//   - the face's flux is differentiated through the central-upwind formula even where the forward
//     took the identical-state shortcut (equal in value there; the choice among ties is immaterial);
//   - a face with no positive span passes nothing; max/min and clamps pass to what they selected;
//   - sqrt at zero depth passes nothing;
//   - the clamp, a sink that took all the water and the dry test pass the branch the forward took,
//     read from the checkpoint pass's branch words.
#include "wl_adjoint.h"
#include "wl_device.cuh"
#include "wlcuda.h"

#include <algorithm>
#include <cstring>
#include <numeric>

namespace wlc {

namespace {

constexpr int kStrip = 32;
constexpr int kWarps = 4;
constexpr int kCta = 32 * kWarps;
constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ uint32_t tile_of_item(const uint32_t* item_tile, uint32_t item) {
  return item_tile == nullptr ? 0u : item_tile[item];
}

// {h, z, u, v} of a cell (slang:303-314), with the forward's IEEE division.
__device__ __forceinline__ float4 cell_state(float h, float hu, float hv, float z, float dry) {
  const bool wet = h >= dry;
  return make_float4(h, z, wet ? __fdiv_rn(hu, h) : 0.0f, wet ? __fdiv_rn(hv, h) : 0.0f);
}

__device__ __forceinline__ float4 shfl_up4(const float4& v) {
  return make_float4(__shfl_up_sync(kFull, v.x, 1), __shfl_up_sync(kFull, v.y, 1),
                     __shfl_up_sync(kFull, v.z, 1), __shfl_up_sync(kFull, v.w, 1));
}
__device__ __forceinline__ float4 shfl_down4(const float4& v) {
  return make_float4(__shfl_down_sync(kFull, v.x, 1), __shfl_down_sync(kFull, v.y, 1),
                     __shfl_down_sync(kFull, v.z, 1), __shfl_down_sync(kFull, v.w, 1));
}

__device__ __forceinline__ uint32_t warp_max(uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// The state planes of tick t within the sweep: the checkpoint at a segment's first tick, else the
// segment stack.
__device__ __forceinline__ const float* state_of(const AdjTile& A, uint32_t t, uint32_t every,
                                                 size_t n3) {
  const uint32_t c = t / every, j = t - c * every;
  return j == 0u ? A.ckpt + size_t(c) * n3 : A.stack + size_t(j - 1u) * n3;
}

// ---- the forward march -----------------------------------------------------------------------

// One item (32 columns by up to H rows) of one fixed-length tick from `in` into `out`. MODE 0 also
// writes the tick's branch words and the output's largest speeds.
template <int MODE, int H>
__device__ void forward_march(const AdjTile& A, const float* in, float* out, uint32_t* bits,
                              uint32_t* speeds, float dt, int X0, int Y0, int band, float4* west,
                              float4* east) {
  const int lane = threadIdx.x & 31;
  const int nx = int(A.nx), ny = int(A.ny);
  const size_t n = size_t(A.nx) * A.ny;
  const int gx = X0 + lane;
  const bool col = gx < nx;
  const int last = min(kStrip - 1, nx - 1 - X0);
  const int rows = min(H, ny - Y0);
  const float* ph = in;
  const float* phu = in + n;
  const float* phv = in + 2 * n;
  const float* bed = A.bed;
  const float* source = A.source;
  const float g = A.gravity, dry = A.dry, hg = __fmul_rn(0.5f, g);
  const uint32_t flags = A.flags;
  const float sw = (flags & kFlagWestOpen) ? 1.0f : -1.0f;
  const float se = (flags & kFlagEastOpen) ? 1.0f : -1.0f;
  const float ss = (flags & kFlagSouthOpen) ? 1.0f : -1.0f;
  const float sn = (flags & kFlagNorthOpen) ? 1.0f : -1.0f;
  auto load = [&](int i) { return cell_state(ph[i], phu[i], phv[i], bed[i], dry); };

  for (int j0 = 0; j0 < rows; j0 += 32) {
    const int j = j0 + lane;
    if (j < rows) {
      const int row = (Y0 + j) * nx;
      float4 w;
      if (X0 > 0) {
        w = load(row + X0 - 1);
      } else {
        w = load(row);
        w.z = __fmul_rn(sw, w.z);
      }
      const float4 cl = load(row + X0 + last);
      float4 e;
      if (X0 + last + 1 < nx) {
        e = load(row + X0 + last + 1);
      } else {
        e = cl;
        e.z = __fmul_rn(se, cl.z);
      }
      west[j] = w;
      east[j] = face<false>(g, hg, cl.x, cl.y, cl.z, cl.w, e.x, e.y, e.z, e.w);
    }
  }
  __syncwarp();

  const int gxc = col ? gx : X0;  // dead lanes read a live column and write nothing
  int i = Y0 * nx + gxc;
  float hu = phu[i], hv = phv[i];
  float src = source != nullptr ? source[i] : 0.0f;
  float4 c = cell_state(ph[i], hu, hv, bed[i], dry);
  float4 fs;
  {
    float4 s;
    if (Y0 > 0) {
      s = load(i - nx);
    } else {
      s = c;
      s.w = __fmul_rn(ss, c.w);
    }
    fs = face<false>(g, hg, s.x, s.y, s.w, s.z, c.x, c.y, c.w, c.z);
  }
  float nh = 0.0f, nhu = 0.0f, nhv = 0.0f, nz = 0.0f, nsrc = 0.0f;
  if (Y0 + 1 < ny) {
    const int k = i + nx;
    nh = ph[k];
    nhu = phu[k];
    nhv = phv[k];
    nz = bed[k];
    if (source != nullptr) nsrc = source[k];
  }
  const float lam = __fdiv_rn(dt, A.cell_m);
  uint32_t ga = 0u, gb = 0u;

  for (int j = 0; j < rows; ++j) {
    const int gy = Y0 + j;
    float4 nc;
    const float hu_n = nhu, hv_n = nhv, src_n = nsrc;
    if (gy + 1 < ny) {
      nc = cell_state(nh, nhu, nhv, nz, dry);
    } else {
      nc = c;
      nc.w = __fmul_rn(sn, c.w);
    }
    if (gy + 2 < ny) {
      const int k = i + 2 * nx;
      nh = ph[k];
      nhu = phu[k];
      nhv = phv[k];
      nz = bed[k];
      if (source != nullptr) nsrc = source[k];
    }
    const float4 fn = face<false>(g, hg, c.x, c.y, c.w, c.z, nc.x, nc.y, nc.w, nc.z);
    float4 w = shfl_up4(c);
    if (lane == 0) w = west[j];
    const float4 fw = face<false>(g, hg, w.x, w.y, w.z, w.w, c.x, c.y, c.z, c.w);
    float4 fe = shfl_down4(fw);
    if (lane == last) fe = east[j];

    bool clamp = false, sink = false, wet = false;
    if (col) {
      // U' = U - dt/dx ((F_e - F_w) + (F_n - F_s)) (slang:653-668)
      float h = __fsub_rn(c.x, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.x, fw.x), __fsub_rn(fn.x, fs.x))));
      float mu = __fsub_rn(hu, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.y, fw.z), __fsub_rn(fn.w, fs.w))));
      float mv = __fsub_rn(hv, __fmul_rn(lam, __fadd_rn(__fsub_rn(fe.w, fw.w), __fsub_rn(fn.y, fs.z))));
      if (h < 0.0f) {
        h = 0.0f;
        clamp = true;
      }
      if (source != nullptr) {  // slang:700-715, every step (scale 1)
        const float added = __fmul_rn(src, dt);
        if (added >= 0.0f) {
          h = __fadd_rn(h, added);
        } else {
          const float want = -added;
          sink = !(want < h);
          const float taken = want < h ? want : h;
          h = __fsub_rn(h, taken);
        }
      }
      wet = h >= dry;
      if (!wet) {
        mu = 0.0f;
        mv = 0.0f;
      }
      out[i] = h;
      out[n + i] = mu;
      out[2 * n + i] = mv;
      if (MODE == 0) {
        float ax, ay;
        cell_speeds<false>(g, dry, h, mu, mv, ax, ay);
        ga = max(ga, __float_as_uint(ax));
        gb = max(gb, __float_as_uint(ay));
      }
    }
    if (MODE == 0) {
      const uint32_t wc = __ballot_sync(kFull, clamp);
      const uint32_t ws = __ballot_sync(kFull, sink);
      const uint32_t ww = __ballot_sync(kFull, wet);
      if (lane < 3) {
        const uint32_t v = lane == 0 ? wc : (lane == 1 ? ws : ww);
        bits[(size_t(lane) * ny + gy) * A.bands + band] = v;
      }
    }
    c = nc;
    hu = hu_n;
    hv = hv_n;
    src = src_n;
    fs = fn;
    i += nx;
  }
  if (MODE == 0) {
    ga = warp_max(ga);
    gb = warp_max(gb);
    if (lane == 0) {
      atomicMax(speeds, ga);
      atomicMax(speeds + 1, gb);
    }
  }
}

// ---- the reverse march -----------------------------------------------------------------------

__device__ __forceinline__ float rcp_fast(float x) { return __fdividef(1.0f, x); }

// The face's vector-Jacobian product (the oracle's face_vjp): the sides as {h, z, normal,
// tangential}, the bars of the face's outputs {h, nl, nr, t}; out: each side's bars in the same
// order as its inputs.
__device__ __forceinline__ void face_vjp(float g, float hl0, float zl, float ul, float vl,
                                         float hr0, float zr, float ur, float vr, float bh,
                                         float bnl, float bnr, float bt, float4& bL, float4& bR) {
  const bool pick_l = zl > zr;
  const float zf = pick_l ? zl : zr;
  const float el = __fsub_rn(__fadd_rn(hl0, zl), zf);
  const float er = __fsub_rn(__fadd_rn(hr0, zr), zf);
  const float hl = el > 0.0f ? el : 0.0f;
  const float hr = er > 0.0f ? er : 0.0f;
  float bhl = -bnl * g * hl;
  float bhr = -bnr * g * hr;
  float bul = 0.0f, bvl = 0.0f, bur = 0.0f, bvr = 0.0f;
  const float cl = __fsqrt_rn(__fmul_rn(g, hl));
  const float cr = __fsqrt_rn(__fmul_rn(g, hr));
  const float a1 = __fadd_rn(ur, cr), a2 = __fadd_rn(ul, cl);
  const float b1 = __fsub_rn(ur, cr), b2 = __fsub_rn(ul, cl);
  const bool p1 = a1 > a2;
  const float apx = p1 ? a1 : a2;
  const bool ap_on = apx > 0.0f;
  const float ap = ap_on ? apx : 0.0f;
  const bool m1 = b1 < b2;
  const float amx = m1 ? b1 : b2;
  const bool am_on = amx < 0.0f;
  const float am = am_on ? amx : 0.0f;
  const float span = __fsub_rn(ap, am);
  if (span > 0.0f) {
    const float inv = rcp_fast(span);
    const float hg = 0.5f * g;
    const float pl = hg * hl * hl, pr = hg * hr * hr;
    const float ql = hl * ul, qr = hr * ur, apam = ap * am;
    const float Al = ql * ul + pl, Ar = qr * ur + pr;
    const float Tl = ql * vl, Tr = qr * vr;
    const float dh = hr - hl, dq = qr - ql, D = hr * vr - hl * vl;
    const float Fh = (ap * ql - am * qr + apam * dh) * inv;
    const float Fn = (ap * Al - am * Ar + apam * dq) * inv;
    const float Ft = (ap * Tl - am * Tr + apam * D) * inv;
    const float bFn = bnl + bnr;
    const float bNh = bh * inv, bNn = bFn * inv, bNt = bt * inv;
    const float bspan = -(bh * Fh + bFn * Fn + bt * Ft) * inv;
    const float bap = bspan + bNh * (ql + am * dh) + bNn * (Al + am * dq) + bNt * (Tl + am * D);
    const float bam = -bspan + bNh * (ap * dh - qr) + bNn * (ap * dq - Ar) + bNt * (ap * D - Tr);
    const float bAl = bNn * ap, bAr = -bNn * am, bTl = bNt * ap, bTr = -bNt * am;
    const float bD = bNt * apam;
    const float bql = bNh * ap - bNn * apam + bAl * ul + bTl * vl;
    const float bqr = -bNh * am + bNn * apam + bAr * ur + bTr * vr;
    bhl += -bNh * apam + bAl * g * hl - bD * vl + bql * ul;
    bhr += bNh * apam + bAr * g * hr + bD * vr + bqr * ur;
    bul += bAl * ql + bql * hl;
    bur += bAr * qr + bqr * hr;
    bvl += bTl * ql - bD * hl;
    bvr += bTr * qr + bD * hr;
    float bcl = 0.0f, bcr = 0.0f;
    if (ap_on) {
      if (p1) { bur += bap; bcr += bap; } else { bul += bap; bcl += bap; }
    }
    if (am_on) {
      if (m1) { bur += bam; bcr -= bam; } else { bul += bam; bcl -= bam; }
    }
    if (cl > 0.0f) bhl += bcl * hg * rcp_fast(cl);
    if (cr > 0.0f) bhr += bcr * hg * rcp_fast(cr);
  }
  const float bel = el > 0.0f ? bhl : 0.0f;
  const float ber = er > 0.0f ? bhr : 0.0f;
  const float bzf = -bel - ber;
  bL = make_float4(bel, pick_l ? bel + bzf : bel, bul, bvl);
  bR = make_float4(ber, pick_l ? ber : ber + bzf, bur, bvr);
}

// The bars of a cell's update outputs by the tick's branches: {h, hu, hv, source}, from the
// adjoint state of the next tick and the cell's branch bits.
__device__ __forceinline__ float4 masked(float lh, float lu, float lv, uint32_t wc, uint32_t ws,
                                         uint32_t ww, int bit) {
  const bool clamp = (wc >> bit) & 1u, sink = (ws >> bit) & 1u, wet = (ww >> bit) & 1u;
  return make_float4((clamp || sink) ? 0.0f : lh, wet ? lu : 0.0f, wet ? lv : 0.0f,
                     sink ? 0.0f : lh);
}

// One item of one reverse tick: lam_out = (dU'/dU)^T lam_in, and the bed's and source's bars
// added to the gradients.
template <int H>
__device__ void reverse_march(const AdjTile& A, const float* U, const float* lam_in,
                              float* lam_out, const uint32_t* bits, float dt, int X0, int Y0,
                              int band, float4* wst, float4* wmk, float4* east) {
  const int lane = threadIdx.x & 31;
  const int nx = int(A.nx), ny = int(A.ny);
  const size_t n = size_t(A.nx) * A.ny;
  const int bands = int(A.bands);
  const int gx = X0 + lane;
  const bool col = gx < nx;
  const int last = min(kStrip - 1, nx - 1 - X0);
  const int rows = min(H, ny - Y0);
  const float* bed = A.bed;
  const float g = A.gravity, dry = A.dry;
  const uint32_t flags = A.flags;
  const float sw = (flags & kFlagWestOpen) ? 1.0f : -1.0f;
  const float se = (flags & kFlagEastOpen) ? 1.0f : -1.0f;
  const float ss = (flags & kFlagSouthOpen) ? 1.0f : -1.0f;
  const float sn = (flags & kFlagNorthOpen) ? 1.0f : -1.0f;
  const float lam = __fdiv_rn(dt, A.cell_m);
  const size_t plane_words = size_t(ny) * bands;
  auto state = [&](int i) { return cell_state(U[i], U[n + i], U[2 * n + i], bed[i], dry); };
  auto mark = [&](int i, int gy, int b, int bit) {
    const size_t w = size_t(gy) * bands + b;
    return masked(lam_in[i], lam_in[n + i], lam_in[2 * n + i], bits[w], bits[plane_words + w],
                  bits[2 * plane_words + w], bit);
  };

  // The band's sides: the west neighbour of lane 0 (state and bars; a ghost at the west edge), and
  // the bars the last live lane's cell takes from its east face.
  for (int j0 = 0; j0 < rows; j0 += 32) {
    const int j = j0 + lane;
    if (j < rows) {
      const int gy = Y0 + j;
      const int row = gy * nx;
      if (X0 > 0) {
        wst[j] = state(row + X0 - 1);
        wmk[j] = mark(row + X0 - 1, gy, band - 1, 31);
      } else {
        float4 s = state(row);
        s.z = __fmul_rn(sw, s.z);
        wst[j] = s;
        wmk[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
      const int ic = row + X0 + last;
      const float4 c = state(ic);
      const float4 mc = mark(ic, gy, band, last);
      const bool ghost = X0 + last + 1 >= nx;
      float4 e, me = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (!ghost) {
        e = state(ic + 1);
        me = mark(ic + 1, gy, band + 1, 0);
      } else {
        e = c;
        e.z = __fmul_rn(se, c.z);
      }
      float4 bL, bR;
      face_vjp(g, c.x, c.y, c.z, c.w, e.x, e.y, e.z, e.w, lam * (me.x - mc.x), -lam * mc.y,
               lam * me.y, lam * (me.z - mc.z), bL, bR);
      if (ghost) {
        bL.x += bR.x;
        bL.y += bR.y;
        bL.z += se * bR.z;
        bL.w += bR.w;
      }
      east[j] = bL;
    }
  }
  __syncwarp();

  const int gxc = col ? gx : X0;
  const int bit = col ? lane : 0;
  int i = Y0 * nx + gxc;
  float4 c = state(i);
  float4 cm = mark(i, Y0, band, bit);
  // The bars the current row takes from its south face.
  float4 carry;
  {
    const bool ghost = Y0 == 0;
    float4 s, sm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!ghost) {
      s = state(i - nx);
      sm = mark(i - nx, Y0 - 1, band, bit);
    } else {
      s = c;
      s.w = __fmul_rn(ss, c.w);
    }
    float4 bS, bN;
    face_vjp(g, s.x, s.y, s.w, s.z, c.x, c.y, c.w, c.z, lam * (cm.x - sm.x), -lam * sm.z,
             lam * cm.z, lam * (cm.y - sm.y), bS, bN);
    carry = make_float4(bN.x, bN.y, bN.w, bN.z);
    if (ghost) {
      carry.x += bS.x;
      carry.y += bS.y;
      carry.z += bS.w;
      carry.w += ss * bS.z;
    }
  }
  // The next row's inputs, loaded a row ahead.
  float nh = 0.0f, nhu = 0.0f, nhv = 0.0f, nz = 0.0f, nl0 = 0.0f, nl1 = 0.0f, nl2 = 0.0f;
  uint32_t nb0 = 0u, nb1 = 0u, nb2 = 0u;
  auto fetch = [&](int k, int gy) {
    nh = U[k];
    nhu = U[n + k];
    nhv = U[2 * n + k];
    nz = bed[k];
    nl0 = lam_in[k];
    nl1 = lam_in[n + k];
    nl2 = lam_in[2 * n + k];
    const size_t w = size_t(gy) * bands + band;
    nb0 = bits[w];
    nb1 = bits[plane_words + w];
    nb2 = bits[2 * plane_words + w];
  };
  if (Y0 + 1 < ny) fetch(i + nx, Y0 + 1);
  const double ddt = double(dt);

  for (int j = 0; j < rows; ++j) {
    const int gy = Y0 + j;
    const bool nghost = gy + 1 >= ny;
    // This row's running gradients, read now so the read is in flight while the row computes.
    double gbed = 0.0, gsrc = 0.0;
    if (col) {
      gbed = A.g_bed[i];
      gsrc = A.g_src[i];
    }
    float4 nc, nm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!nghost) {
      nc = cell_state(nh, nhu, nhv, nz, dry);
      nm = masked(nl0, nl1, nl2, nb0, nb1, nb2, bit);
    } else {
      nc = c;
      nc.w = __fmul_rn(sn, c.w);
    }
    if (gy + 2 < ny) fetch(i + 2 * nx, gy + 2);

    // The north face: the south side's bars stay, the north side's go up a row.
    float4 bS, bN;
    face_vjp(g, c.x, c.y, c.w, c.z, nc.x, nc.y, nc.w, nc.z, lam * (nm.x - cm.x), -lam * cm.z,
             lam * nm.z, lam * (nm.y - cm.y), bS, bN);
    float4 acc = make_float4(carry.x + bS.x, carry.y + bS.y, carry.z + bS.w, carry.w + bS.z);
    carry = make_float4(bN.x, bN.y, bN.w, bN.z);
    if (nghost) {
      acc.x += bN.x;
      acc.y += bN.y;
      acc.z += bN.w;
      acc.w += sn * bN.z;
    }
    // The west face: the east side's bars stay, the west side's go to the lane on the west.
    float4 w = shfl_up4(c);
    float4 wm = shfl_up4(cm);
    if (lane == 0) {
      w = wst[j];
      wm = wmk[j];
    }
    float4 bW, bC;
    face_vjp(g, w.x, w.y, w.z, w.w, c.x, c.y, c.z, c.w, lam * (cm.x - wm.x), -lam * wm.y,
             lam * cm.y, lam * (cm.z - wm.z), bW, bC);
    acc.x += bC.x;
    acc.y += bC.y;
    acc.z += bC.z;
    acc.w += bC.w;
    if (lane == 0 && X0 == 0) {
      acc.x += bW.x;
      acc.y += bW.y;
      acc.z += sw * bW.z;
      acc.w += bW.w;
    }
    float4 from_e = shfl_down4(bW);
    if (lane == last) from_e = east[j];
    acc.x += from_e.x;
    acc.y += from_e.y;
    acc.z += from_e.z;
    acc.w += from_e.w;

    if (col) {
      // Through the velocities u = hu / h, v = hv / h of a wet cell.
      float lh = cm.x + acc.x, lu = cm.y, lv = cm.z;
      if (c.x >= dry) {
        const float r = rcp_fast(c.x);
        lh -= (acc.z * c.z + acc.w * c.w) * r;
        lu += acc.z * r;
        lv += acc.w * r;
      }
      lam_out[i] = lh;
      lam_out[n + i] = lu;
      lam_out[2 * n + i] = lv;
      A.g_bed[i] = gbed + double(acc.y);
      A.g_src[i] = gsrc + double(cm.w) * ddt;
    }
    c = nc;
    cm = nm;
    i += nx;
  }
}

// ---- the kernels -----------------------------------------------------------------------------

struct ItemPos {
  const AdjTile* A;
  int X0, Y0, band;
};

template <int H>
// A warp's next item: its own number first, then the warps' count + the work counter's next
// value; a launch of no more warps than items reads no counter.
__device__ __forceinline__ bool next_item(const AdjArgs& a, ItemPos& p, bool first) {
  const int lane = threadIdx.x & 31;
  const uint32_t slots = gridDim.x * kWarps;
  uint32_t item = 0u;
  if (first) {
    item = blockIdx.x * kWarps + (threadIdx.x >> 5);
  } else if (slots >= a.n_items) {
    item = a.n_items;
  } else {
    if (lane == 0) item = slots + atomicAdd(&a.work->next, 1u);
    item = __shfl_sync(kFull, item, 0);
  }
  if (item >= a.n_items) return false;
  const AdjTile& A = a.tiles[tile_of_item(a.item_tile, item)];
  const uint32_t local = item - A.item_base;
  const uint32_t by = local / A.bands, bx = local - by * A.bands;
  p.A = &A;
  p.X0 = int(bx) * kStrip;
  p.Y0 = int(by) * H;
  p.band = int(bx);
  return true;
}

__device__ __forceinline__ void leave(const AdjArgs& a) {
  if ((threadIdx.x & 31) == 0 && gridDim.x * kWarps < a.n_items) {  // the counter was read
    __threadfence();
    if (atomicAdd(&a.work->exited, 1u) + 1u == gridDim.x * kWarps) {
      a.work->next = 0u;
      a.work->exited = 0u;
      __threadfence();
    }
  }
}

template <int MODE, int H>
// 16-row items (a sweep with items enough for every warp) at 80 registers and six CTAs an SM;
// 4-row items (a small tile, one item a warp) at the registers that keep a warp's chain short.
__global__ void __launch_bounds__(kCta, H == 16 ? 6 : 4) adj_forward_kernel(AdjArgs a) {
  dependent_grid_start();
  __shared__ float4 side[kWarps][2][H];
  const int warp = threadIdx.x >> 5;
  const uint32_t t = a.t, k = a.every;
  const uint32_t c = t / k, j = t - c * k;
  const uint32_t seg_end = min((c + 1u) * k, a.ticks);
  ItemPos p;
  for (bool first = true; next_item<H>(a, p, first); first = false) {
    const AdjTile& A = *p.A;
    const size_t n3 = 3 * size_t(A.nx) * A.ny;
    const float* in = state_of(A, t, k, n3);
    float* out = (t + 1u == seg_end) ? A.ckpt + size_t(c + 1u) * n3 : A.stack + size_t(j) * n3;
    uint32_t* bits = A.bits + size_t(t) * 3 * A.ny * A.bands;
    forward_march<MODE, H>(A, in, out, bits, A.speeds + 2 * size_t(t + 1u), a.dt, p.X0, p.Y0,
                        p.band, side[warp][0], side[warp][1]);
    __syncwarp();
  }
  leave(a);
}

template <int H>
__global__ void __launch_bounds__(kCta, 4) adj_reverse_kernel(AdjArgs a) {
  dependent_grid_start();
  __shared__ float4 side[kWarps][3][H];
  const int warp = threadIdx.x >> 5;
  const uint32_t t = a.t, k = a.every;
  ItemPos p;
  for (bool first = true; next_item<H>(a, p, first); first = false) {
    const AdjTile& A = *p.A;
    const size_t n3 = 3 * size_t(A.nx) * A.ny;
    const float* U = state_of(A, t, k, n3);
    const uint32_t* bits = A.bits + size_t(t) * 3 * A.ny * A.bands;
    reverse_march<H>(A, U, A.lam[(t + 1u) & 1u], A.lam[t & 1u], bits, a.dt, p.X0, p.Y0, p.band,
                  side[warp][0], side[warp][1], side[warp][2]);
    __syncwarp();
  }
  leave(a);
}

// The set's current state into checkpoint 0, and its largest speeds into speeds[0]. Grid: x over
// a tile's cells, y over the tiles.
__global__ void __launch_bounds__(256) adj_copy_in_kernel(const TileDesc* set,
                                                          const AdjTile* tiles) {
  const TileDesc& T = set[blockIdx.y];
  const AdjTile& A = tiles[blockIdx.y];
  const size_t n = size_t(A.nx) * A.ny;
  const float* src = T.state[T.ctl->cur];
  uint32_t am = 0u, bm = 0u;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    const float h = src[i], hu = src[n + i], hv = src[2 * n + i];
    A.ckpt[i] = h;
    A.ckpt[n + i] = hu;
    A.ckpt[2 * n + i] = hv;
    float ax, ay;
    cell_speeds<false>(A.gravity, A.dry, h, hu, hv, ax, ay);
    am = max(am, __float_as_uint(ax));
    bm = max(bm, __float_as_uint(ay));
  }
  am = warp_max(am);
  bm = warp_max(bm);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(A.speeds, am);
    atomicMax(A.speeds + 1, bm);
  }
}

// Counts the ticks whose step the plain tick would have chosen shorter than dt (slang:464-474).
__global__ void __launch_bounds__(256) adj_check_kernel(AdjArgs a) {
  const AdjTile& A = a.tiles[blockIdx.x];
  uint32_t count = 0u;
  for (uint32_t t = threadIdx.x; t < a.ticks; t += blockDim.x) {
    const float sa = __uint_as_float(A.speeds[2 * t]), sb = __uint_as_float(A.speeds[2 * t + 1]);
    const float d = choose_dt<false>(sa, sb, A.cfl, A.cell_m, a.dt, __int_as_float(0x7f800000));
    if (d != a.dt) ++count;
  }
  if (count != 0u) atomicAdd(A.limited, count);
}

// The loss (FP64, the probes in order) and the adjoint state of tick T: 2 (h_T(p) - target_p) on
// the depth plane at each probe.
__global__ void adj_seed_kernel(AdjArgs a) {
  if (threadIdx.x != 0) return;
  const AdjTile& A = a.tiles[blockIdx.x];
  const size_t n3 = 3 * size_t(A.nx) * A.ny;
  const uint32_t segments = (a.ticks + a.every - 1u) / a.every;
  const float* fin = A.ckpt + size_t(segments) * n3;
  float* lam = A.lam[a.ticks & 1u];
  double loss = 0.0;
  for (uint32_t p = 0; p < A.n_probes; ++p) {
    const uint32_t cell = A.probes[p];
    const double d = double(fin[cell]) - A.targets[p];
    loss += d * d;
    lam[cell] += float(2.0 * d);
  }
  *A.loss = loss;
}

}  // namespace

// ---- launchers -------------------------------------------------------------------------------

template <int H>
int occupancy_of(bool reverse) {
  int a = 0, b = 0;
  if (reverse)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, adj_reverse_kernel<H>, kCta, 0) ==
                   cudaSuccess
               ? a
               : 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, adj_forward_kernel<0, H>, kCta, 0) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, adj_forward_kernel<1, H>, kCta, 0) !=
      cudaSuccess)
    return 0;
  return std::min(a, b);
}

int adj_occupancy(int rows, bool reverse) {
  return rows == 4 ? occupancy_of<4>(reverse) : occupancy_of<16>(reverse);
}

cudaError_t launch_adj_copy_in(const TileDesc* set_tiles, const AdjTile* tiles, uint32_t count,
                               uint32_t max_blocks, cudaStream_t s) {
  adj_copy_in_kernel<<<dim3(std::max(1u, max_blocks), count), 256, 0, s>>>(set_tiles, tiles);
  return cudaGetLastError();
}

// The sweep's marches are launched as programmatic dependents (dependent_grid_start).
cudaError_t launch_adj_forward(int mode, int rows, const AdjArgs& a, int grid, cudaStream_t s) {
  void (*k)(AdjArgs) = rows == 4 ? (mode == 0 ? adj_forward_kernel<0, 4> : adj_forward_kernel<1, 4>)
                                 : (mode == 0 ? adj_forward_kernel<0, 16> : adj_forward_kernel<1, 16>);
  return launch_dependent(k, dim3(unsigned(grid)), dim3(kCta), 0, s, a);
}

cudaError_t launch_adj_check(const AdjArgs& a, uint32_t count, cudaStream_t s) {
  adj_check_kernel<<<count, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_seed(const AdjArgs& a, uint32_t count, cudaStream_t s) {
  adj_seed_kernel<<<count, 32, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_reverse(int rows, const AdjArgs& a, int grid, cudaStream_t s) {
  void (*k)(AdjArgs) = rows == 4 ? adj_reverse_kernel<4> : adj_reverse_kernel<16>;
  return launch_dependent(k, dim3(unsigned(grid)), dim3(kCta), 0, s, a);
}

// ---- the sweep -------------------------------------------------------------------------------

namespace {

size_t align256(size_t b) { return (b + 255u) & ~size_t(255u); }

void set_err(std::string* err, const std::string& what) {
  if (err) *err = what;
}

}  // namespace

Adjoint::~Adjoint() {
  if (graph_ != nullptr) cudaGraphExecDestroy(graph_);
  if (base_ != nullptr) cudaFree(base_);
}

int Adjoint::check_flags(std::string* err) {
  if (set_->fixed_ops()) {
    set_err(err, "water_live: the adjoint takes the native arithmetic (Ops::native)");
    return WL_ERR_REFUSED;
  }
  bool changed = false;
  for (uint32_t t = 0; t < set_->tile_count(); ++t) {
    const TileDesc& d = set_->desc(t);
    if (d.flags & (kFlagManning | kFlagCompensate)) {
      set_err(err, "water_live: tile " + std::to_string(t) +
                       ": the adjoint takes no Manning friction and no compensated source");
      return WL_ERR_REFUSED;
    }
    const bool src = (d.flags & kFlagSource) != 0u;
    if (src && d.source_every > 1u) {
      set_err(err, "water_live: tile " + std::to_string(t) +
                       ": the adjoint takes a source applied every step");
      return WL_ERR_REFUSED;
    }
    const float* want = src ? d.source : nullptr;
    const uint32_t flags = d.flags & (15u | kFlagSource);
    if (host_[t].source != want || host_[t].flags != flags) {
      host_[t].source = want;
      host_[t].flags = flags;
      changed = true;
    }
  }
  if (changed) {
    const cudaError_t e = cudaMemcpyAsync(d_tiles_, host_.data(), host_.size() * sizeof(AdjTile),
                                          cudaMemcpyHostToDevice, set_->stream());
    if (e != cudaSuccess) {
      set_err(err, std::string("water_live: descriptor upload: ") + cudaGetErrorString(e));
      return WL_ERR_CUDA;
    }
  }
  return WL_OK;
}

int Adjoint::create(TileSet* set, uint32_t ticks, uint32_t every, const uint32_t* probe_first,
                     const uint32_t* probes, const double* targets, std::string* err) {
  if (set == nullptr || !set->valid()) {
    set_err(err, "water_live: no tile set");
    return WL_ERR_INVALID;
  }
  if (ticks == 0u || every == 0u) {
    set_err(err, "water_live: the sweep needs ticks > 0 and a checkpoint interval > 0");
    return WL_ERR_ARGUMENT;
  }
  set_ = set;
  ticks_ = ticks;
  every_ = std::min(every, ticks);
  segments_ = (ticks_ + every_ - 1u) / every_;
  const uint32_t nt = set->tile_count();
  host_.assign(nt, AdjTile{});
  if (cudaSetDevice(set->device()) != cudaSuccess) {
    set_err(err, "water_live: cudaSetDevice failed");
    return WL_ERR_CUDA;
  }
  // Sizes, kind by kind and tile after tile.
  std::vector<uint64_t> cells(nt), words(nt);
  uint64_t total = 0, total_words = 0;
  for (uint32_t t = 0; t < nt; ++t) {
    const TileDesc& d = set->desc(t);
    cells[t] = uint64_t(d.nx) * d.ny;
    const uint64_t bands = (d.nx + kStrip - 1u) / kStrip;
    words[t] = uint64_t(ticks_) * 3u * d.ny * bands;
    total += cells[t];
    total_words += words[t];
    const uint32_t pf = probe_first[t], pl = probe_first[t + 1];
    if (pl < pf) {
      set_err(err, "water_live: probe_first must not decrease");
      return WL_ERR_ARGUMENT;
    }
    for (uint32_t p = pf; p < pl; ++p)
      if (probes[p] >= cells[t]) {
        set_err(err, "water_live: tile " + std::to_string(t) + ": probe " +
                         std::to_string(probes[p]) + " is outside the tile");
        return WL_ERR_ARGUMENT;
      }
  }
  const uint32_t n_probes = probe_first[nt];
  const size_t b_ckpt = align256(size_t(segments_ + 1u) * 3u * total * sizeof(float));
  const size_t b_stack = align256(size_t(every_ - 1u) * 3u * total * sizeof(float));
  const size_t b_bits = align256(size_t(total_words) * sizeof(uint32_t));
  const size_t b_lam = align256(3u * total * sizeof(float));
  const size_t b_grad = align256(total * sizeof(double));
  const size_t b_speeds = align256(size_t(nt) * (ticks_ + 1u) * 2u * sizeof(uint32_t));
  const size_t b_limited = align256(size_t(nt) * sizeof(uint32_t));
  const size_t b_loss = align256(size_t(nt) * sizeof(double));
  const size_t b_probes = align256(size_t(n_probes) * sizeof(uint32_t) + 4u);
  const size_t b_targets = align256(size_t(n_probes) * sizeof(double) + 8u);
  const size_t b_tiles = align256(size_t(nt) * sizeof(AdjTile));
  // The rows of a work item: 16, or 4 where 16-row items would leave the device short of warps
  // (each warp marches its rows one after another; a short march is more warps in flight).
  int dev_sms = 0;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, set->device());
  {
    uint64_t items16 = 0;
    for (uint32_t t = 0; t < nt; ++t) {
      const TileDesc& d = set->desc(t);
      items16 += uint64_t((d.nx + kStrip - 1u) / kStrip) * ((d.ny + 15u) / 16u);
    }
    rows_ = items16 < uint64_t(std::max(dev_sms, 1)) * 8u ? 4 : 16;
  }
  const uint32_t H = uint32_t(rows_);
  // work items, largest tiles first
  std::vector<uint32_t> order(nt);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return cells[a] > cells[b]; });
  uint64_t items = 0;
  for (uint32_t t : order) {
    const TileDesc& d = set->desc(t);
    host_[t].bands = (d.nx + kStrip - 1u) / kStrip;
    host_[t].row_blocks = (d.ny + H - 1u) / H;
    host_[t].items = host_[t].bands * host_[t].row_blocks;
    host_[t].item_base = uint32_t(items);
    items += host_[t].items;
  }
  if (items >= (1ull << 31)) {
    set_err(err, "water_live: too many work items");
    return WL_ERR_SIZE;
  }
  n_items_ = uint32_t(items);
  const size_t b_items = align256((nt > 1 ? n_items_ : 1u) * sizeof(uint32_t));
  const size_t b_work = align256(sizeof(WorkCtl));
  bytes_ = b_ckpt + b_stack + b_bits + 2 * b_lam + 2 * b_grad + b_speeds + b_limited + b_loss +
           b_probes + b_targets + b_tiles + b_items + b_work;
  if (cudaMalloc(&base_, bytes_) != cudaSuccess) {
    base_ = nullptr;
    cudaGetLastError();
    set_err(err, "water_live: out of device memory for the sweep (" + std::to_string(bytes_) +
                     " bytes)");
    return WL_ERR_ALLOC;
  }
  char* p = base_;
  float* ckpt = reinterpret_cast<float*>(p); p += b_ckpt;
  float* stack = reinterpret_cast<float*>(p); p += b_stack;
  uint32_t* bits = reinterpret_cast<uint32_t*>(p); p += b_bits;
  lam_base_[0] = reinterpret_cast<float*>(p); p += b_lam;
  lam_base_[1] = reinterpret_cast<float*>(p); p += b_lam;
  lam_bytes_ = 3u * total * sizeof(float);
  zero_ = p;
  double* g_bed = reinterpret_cast<double*>(p); p += b_grad;
  double* g_src = reinterpret_cast<double*>(p); p += b_grad;
  uint32_t* speeds = reinterpret_cast<uint32_t*>(p); p += b_speeds;
  uint32_t* limited = reinterpret_cast<uint32_t*>(p); p += b_limited;
  double* loss = reinterpret_cast<double*>(p); p += b_loss;
  zero_bytes_ = size_t(p - static_cast<char*>(zero_));
  uint32_t* d_probes = reinterpret_cast<uint32_t*>(p); p += b_probes;
  double* d_targets = reinterpret_cast<double*>(p); p += b_targets;
  d_tiles_ = reinterpret_cast<AdjTile*>(p); p += b_tiles;
  d_item_tile_ = reinterpret_cast<uint32_t*>(p); p += b_items;
  d_work_ = reinterpret_cast<WorkCtl*>(p);

  uint64_t first = 0, first_word = 0;
  for (uint32_t t = 0; t < nt; ++t) {
    const TileDesc& d = set->desc(t);
    AdjTile& A = host_[t];
    A.bed = d.bed;
    A.source = nullptr;
    A.ckpt = ckpt + size_t(segments_ + 1u) * 3u * first;
    A.stack = stack + size_t(every_ - 1u) * 3u * first;
    A.bits = bits + first_word;
    A.lam[0] = lam_base_[0] + 3u * first;
    A.lam[1] = lam_base_[1] + 3u * first;
    A.g_bed = g_bed + first;
    A.g_src = g_src + first;
    A.speeds = speeds + size_t(t) * (ticks_ + 1u) * 2u;
    A.probes = d_probes + probe_first[t];
    A.targets = d_targets + probe_first[t];
    A.loss = loss + t;
    A.limited = limited + t;
    A.n_probes = probe_first[t + 1] - probe_first[t];
    A.nx = d.nx;
    A.ny = d.ny;
    A.flags = d.flags & 15u;
    A.gravity = d.gravity;
    A.dry = d.dry;
    A.cell_m = d.cell_m;
    A.cfl = d.cfl;
    first += cells[t];
    first_word += words[t];
  }
  std::vector<uint32_t> item_tile;
  if (nt > 1) {
    item_tile.resize(n_items_);
    for (uint32_t t = 0; t < nt; ++t)
      std::fill(item_tile.begin() + host_[t].item_base,
                item_tile.begin() + host_[t].item_base + host_[t].items, t);
  }
  const cudaStream_t s = set->stream();
  cudaError_t e = cudaSuccess;
  if (n_probes > 0) {
    e = cudaMemcpyAsync(d_probes, probes, n_probes * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_targets, targets, n_probes * sizeof(double), cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess && nt > 1)
    e = cudaMemcpyAsync(d_item_tile_, item_tile.data(), n_items_ * sizeof(uint32_t),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_work_, 0, sizeof(WorkCtl), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_tiles_, host_.data(), nt * sizeof(AdjTile), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_err(err, std::string("water_live: sweep setup: ") + cudaGetErrorString(e));
    return WL_ERR_CUDA;
  }
  // The forward marches and the reverse march each get the grid their own residency allows.
  const int occ_fwd = adj_occupancy(rows_, false), occ_rev = adj_occupancy(rows_, true);
  if (occ_fwd <= 0 || occ_rev <= 0 || dev_sms <= 0) {
    set_err(err, "water_live: the adjoint's kernels cannot be resident on this device");
    return WL_ERR_CUDA;
  }
  const uint64_t warps_needed = (n_items_ + kWarps - 1u) / kWarps;
  grid_fwd_ = int(std::min<uint64_t>(warps_needed, uint64_t(dev_sms) * occ_fwd));
  grid_rev_ = int(std::min<uint64_t>(warps_needed, uint64_t(dev_sms) * occ_rev));
  return check_flags(err);
}

uint32_t Adjoint::launches() const {
  // copy-in, the checkpoint pass, the check, the seed, the recompute, the reverse ticks
  return 3u + ticks_ + (ticks_ - segments_) + ticks_;
}

cudaError_t Adjoint::enqueue(float dt) {
  const cudaStream_t s = set_->stream();
  const uint32_t nt = set_->tile_count();
  cudaError_t e = cudaMemsetAsync(zero_, 0, zero_bytes_, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(lam_base_[ticks_ & 1u], 0, lam_bytes_, s);
  if (e != cudaSuccess) return e;
  uint64_t largest = 0;
  for (uint32_t t = 0; t < nt; ++t)
    largest = std::max<uint64_t>(largest, uint64_t(host_[t].nx) * host_[t].ny);
  const uint32_t copy_blocks = uint32_t(std::min<uint64_t>((largest + 255u) / 256u, 1024u));
  e = launch_adj_copy_in(set_->device_descs(), d_tiles_, nt, copy_blocks, s);
  if (e != cudaSuccess) return e;
  AdjArgs a{d_tiles_, nt > 1 ? d_item_tile_ : nullptr, d_work_, n_items_, ticks_, every_, 0u, dt};
  for (uint32_t t = 0; t < ticks_; ++t) {
    a.t = t;
    if ((e = launch_adj_forward(0, rows_, a, grid_fwd_, s)) != cudaSuccess) return e;
  }
  if ((e = launch_adj_check(a, nt, s)) != cudaSuccess) return e;
  if ((e = launch_adj_seed(a, nt, s)) != cudaSuccess) return e;
  for (uint32_t c = segments_; c-- > 0u;) {
    const uint32_t start = c * every_, end = std::min(start + every_, ticks_);
    for (uint32_t t = start; t + 1u < end; ++t) {
      a.t = t;
      if ((e = launch_adj_forward(1, rows_, a, grid_fwd_, s)) != cudaSuccess) return e;
    }
    for (uint32_t t = end; t-- > start;) {
      a.t = t;
      if ((e = launch_adj_reverse(rows_, a, grid_rev_, s)) != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

int Adjoint::run(float dt, bool use_graph, std::string* err) {
  if (cudaSetDevice(set_->device()) != cudaSuccess) {
    set_err(err, "water_live: cudaSetDevice failed");
    return WL_ERR_CUDA;
  }
  if (!(dt > 0.0f)) {
    set_err(err, "water_live: the sweep needs a step length > 0");
    return WL_ERR_ARGUMENT;
  }
  const int fc = check_flags(err);
  if (fc != WL_OK) return fc;
  const cudaStream_t s = set_->stream();
  cudaError_t e = cudaSuccess;
  if (!use_graph) {
    e = enqueue(dt);
  } else {
    if (graph_ == nullptr || graph_dt_ != dt) {
      if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
      }
      cudaGraph_t g = nullptr;
      e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const cudaError_t q = enqueue(dt);
        e = cudaStreamEndCapture(s, &g);
        if (q != cudaSuccess) e = q;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
      if (g != nullptr) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        graph_ = nullptr;
        set_err(err, std::string("water_live: sweep capture: ") + cudaGetErrorString(e));
        return WL_ERR_CUDA;
      }
      graph_dt_ = dt;
    }
    e = cudaGraphLaunch(graph_, s);
  }
  if (e != cudaSuccess) {
    set_err(err, std::string("water_live: sweep launch: ") + cudaGetErrorString(e));
    return WL_ERR_CUDA;
  }
  bool timed_out = false;
  e = wait_stream(s, &timed_out);
  if (timed_out) {
    set_err(err, "water_live: the sweep passed the wait limit");
    return WL_ERR_TIMEOUT;
  }
  if (e != cudaSuccess) {
    set_err(err, std::string("water_live: sweep: ") + cudaGetErrorString(e));
    return WL_ERR_CUDA;
  }
  return WL_OK;
}

int Adjoint::read(double* loss, double* g_bed, double* g_src, uint32_t* limited,
                   std::string* err) {
  const uint32_t nt = set_->tile_count();
  const uint64_t total = set_->total_cells();
  const char* z = static_cast<const char*>(zero_);
  const size_t b_grad = align256(total * sizeof(double));
  const size_t b_speeds = align256(size_t(nt) * (ticks_ + 1u) * 2u * sizeof(uint32_t));
  const size_t b_limited = align256(size_t(nt) * sizeof(uint32_t));
  cudaError_t e = cudaSuccess;
  if (g_bed) e = cudaMemcpy(g_bed, z, total * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && g_src)
    e = cudaMemcpy(g_src, z + b_grad, total * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && limited)
    e = cudaMemcpy(limited, z + 2 * b_grad + b_speeds, nt * sizeof(uint32_t),
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss)
    e = cudaMemcpy(loss, z + 2 * b_grad + b_speeds + b_limited, nt * sizeof(double),
                   cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_err(err, std::string("water_live: read-back: ") + cudaGetErrorString(e));
    return WL_ERR_CUDA;
  }
  return WL_OK;
}

int Adjoint::read_final(float* planes, std::string* err) {
  uint64_t first = 0;
  for (uint32_t t = 0; t < set_->tile_count(); ++t) {
    const size_t n3 = 3u * size_t(host_[t].nx) * host_[t].ny;
    const cudaError_t e = cudaMemcpy(planes + first, host_[t].ckpt + size_t(segments_) * n3,
                                     n3 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      set_err(err, std::string("water_live: read-back: ") + cudaGetErrorString(e));
      return WL_ERR_CUDA;
    }
    first += n3;
  }
  return WL_OK;
}

int Adjoint::read_state_gradient(float* planes, std::string* err) {
  // Reverse tick t writes lam[t & 1], so tick 0's adjoint state is in lam_base_[0], laid out as
  // the tiles' states are (3 planes a tile, tile after tile).
  const cudaError_t e = cudaMemcpy(planes, lam_base_[0], lam_bytes_, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_err(err, std::string("water_live: read-back: ") + cudaGetErrorString(e));
    return WL_ERR_CUDA;
  }
  return WL_OK;
}

}  // namespace wlc

// ---- the C ABI (include/wlcuda.h) ------------------------------------------------------------

namespace {

int put(char* err, size_t len, int code, const std::string& msg) {
  if (code != WL_OK && err != nullptr && len > 0) {
    const size_t k = msg.size() < len - 1 ? msg.size() : len - 1;
    std::memcpy(err, msg.data(), k);
    err[k] = '\0';
  }
  return code;
}

}  // namespace

// The two creators over a step and over a batch live beside those handles (wl_api.cpp,
// wl_batch.cpp) and call this.
int wl_adjoint_create_over(wlc::TileSet* set, uint32_t ticks, uint32_t every,
                           const uint32_t* probe_first, const uint32_t* probes,
                           const double* targets, wl_adjoint** out, char* err, size_t err_len) {
  *out = nullptr;
  auto* a = new (std::nothrow) wl_adjoint;
  if (a == nullptr) return put(err, err_len, WL_ERR_ALLOC, "water_live: out of host memory");
  std::string msg;
  const int code = a->impl.create(set, ticks, every, probe_first, probes, targets, &msg);
  if (code != WL_OK) {
    delete a;
    return put(err, err_len, code, msg);
  }
  *out = a;
  return WL_OK;
}

extern "C" {

void wl_adjoint_destroy(wl_adjoint* a) { delete a; }

int wl_adjoint_enqueue(wl_adjoint* a, float max_dt) {
  if (a == nullptr) return WL_ERR_INVALID;
  if (!(max_dt > 0.0f)) return WL_ERR_ARGUMENT;
  const int fc = a->impl.check_flags(nullptr);
  if (fc != WL_OK) return fc;
  return a->impl.enqueue(max_dt) == cudaSuccess ? WL_OK : WL_ERR_CUDA;
}

int wl_adjoint_run(wl_adjoint* a, float max_dt, int use_graph, char* err, size_t err_len) {
  if (a == nullptr) return put(err, err_len, WL_ERR_INVALID, "water_live: no sweep");
  std::string msg;
  return put(err, err_len, a->impl.run(max_dt, use_graph != 0, &msg), msg);
}

int wl_adjoint_read(wl_adjoint* a, double* loss, double* g_bed, double* g_source,
                    uint32_t* limited, char* err, size_t err_len) {
  if (a == nullptr) return put(err, err_len, WL_ERR_INVALID, "water_live: no sweep");
  std::string msg;
  return put(err, err_len, a->impl.read(loss, g_bed, g_source, limited, &msg), msg);
}

int wl_adjoint_read_final(wl_adjoint* a, float* planes, char* err, size_t err_len) {
  if (a == nullptr) return put(err, err_len, WL_ERR_INVALID, "water_live: no sweep");
  if (planes == nullptr) return put(err, err_len, WL_ERR_ARGUMENT, "water_live: no buffer");
  std::string msg;
  return put(err, err_len, a->impl.read_final(planes, &msg), msg);
}

int wl_adjoint_read_state_gradient(wl_adjoint* a, float* planes, char* err, size_t err_len) {
  if (a == nullptr) return put(err, err_len, WL_ERR_INVALID, "water_live: no sweep");
  if (planes == nullptr) return put(err, err_len, WL_ERR_ARGUMENT, "water_live: no buffer");
  std::string msg;
  return put(err, err_len, a->impl.read_state_gradient(planes, &msg), msg);
}

uint32_t wl_adjoint_launches(const wl_adjoint* a) { return a ? a->impl.launches() : 0u; }

uint64_t wl_adjoint_device_bytes(const wl_adjoint* a) { return a ? a->impl.device_bytes() : 0u; }

}  // extern "C"

// Seeded synthetic terrain for the benchmark configurations (include/wlcuda_util.h): the same
// doubles as game_engine_gb300/workloads.py's fbm, operation for operation, on the host's threads.
#include "wlcuda_util.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

// The reference's integer hash (water_live_device_tests.cpp:50-56) on 32-bit words.
inline uint32_t mix(uint32_t x, uint32_t y) {
  uint32_t h = (x * 0x9e3779b1u) ^ ((y + 0x7f4a7c15u) * 0x85ebca77u);
  h ^= h >> 15;
  h *= 0x2c1b3c6du;
  h ^= h >> 12;
  return h;
}

inline double lattice(uint64_t ix, uint64_t iy, uint64_t salt) {
  const uint32_t x = uint32_t(ix + (salt & 0xffffffffull));
  const uint32_t y = uint32_t(iy ^ ((salt >> 32) & 0xffffffffull));
  return double(mix(x, y)) / 4294967296.0;
}

}  // namespace

extern "C" int wl_util_fbm(double* out, uint32_t nx, uint32_t ny, double height, uint64_t seed,
                           uint32_t octaves) {
  if (out == nullptr || nx == 0 || ny == 0) return 1;
  const double side = double(nx > ny ? nx : ny);
  const double base = side / 4.0 > 1.0 ? side / 4.0 : 1.0;
  const size_t n = size_t(nx) * ny;
  const unsigned threads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  auto rows = [&](uint32_t y0, uint32_t y1) {
    for (uint32_t y = y0; y < y1; ++y)
      for (uint32_t x = 0; x < nx; ++x) out[size_t(y) * nx + x] = 0.0;
    double amp = 1.0, period = base;
    for (uint32_t o = 0; o < octaves; ++o) {
      const uint64_t salt = seed * uint64_t(o + 1) * 0x9e3779b97f4a7c15ull + o;
      for (uint32_t y = y0; y < y1; ++y) {
        const double fy = double(y) / period;
        const double iyf = std::floor(fy);
        const double ty = fy - iyf;
        const double sy = ty * ty * (3.0 - 2.0 * ty);
        const uint64_t iy = uint64_t(iyf);
        for (uint32_t x = 0; x < nx; ++x) {
          const double fx = double(x) / period;
          const double ixf = std::floor(fx);
          const double tx = fx - ixf;
          const double sx = tx * tx * (3.0 - 2.0 * tx);
          const uint64_t ix = uint64_t(ixf);
          const double v00 = lattice(ix, iy, salt), v10 = lattice(ix + 1, iy, salt);
          const double v01 = lattice(ix, iy + 1, salt), v11 = lattice(ix + 1, iy + 1, salt);
          const double a = v00 + (v10 - v00) * sx;
          const double b = v01 + (v11 - v01) * sx;
          out[size_t(y) * nx + x] += amp * (a + (b - a) * sy);
        }
      }
      amp *= 0.5;
      period = period / 2.0 > 1.0 ? period / 2.0 : 1.0;
    }
  };
  std::vector<std::thread> pool;
  const uint32_t chunk = (ny + threads - 1) / threads;
  for (unsigned t = 0; t < threads; ++t) {
    const uint32_t y0 = t * chunk, y1 = std::min<uint32_t>(ny, y0 + chunk);
    if (y0 < y1) pool.emplace_back(rows, y0, y1);
  }
  for (auto& th : pool) th.join();
  double lo = out[0], hi = out[0];
  for (size_t i = 1; i < n; ++i) {
    lo = out[i] < lo ? out[i] : lo;
    hi = out[i] > hi ? out[i] : hi;
  }
  const double span = hi > lo ? hi - lo : 1.0;
  for (size_t i = 0; i < n; ++i) out[i] = (out[i] - lo) / span * height;
  return 0;
}

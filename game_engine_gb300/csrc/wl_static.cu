// One plain tick of a caller-owned state that allocates nothing: its scratch (the tile's
// descriptor, control block, work counter and two record buffers) is a file-scope device array of
// a fixed size, so the call makes no cudaMalloc, cudaFree or other allocating call.
//
// The callers that cannot allocate: an engine frame loop that reserves its device memory at start
// and must not allocate mid-frame (an allocation may synchronise the device, and may fail under a
// fixed budget), and host code that must not touch the allocator for any other reason (a
// real-time thread, a caller holding its own pool). The arithmetic is the plain tick's kernels
// unchanged (wl_kernels.cu): the same launches a wl_step makes for a prime and one tick.
#include "wl_device.cuh"
#include "wl_kernels.h"
#include "wlcuda.h"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

namespace wlc {
namespace {

// The largest grid the scratch holds: 4096 groups of 16 x 16 cells (1,048,576 cells, 1024 x 1024
// when both sides are multiples of 16). The scratch is 262,528 bytes of device memory.
constexpr uint32_t kStaticMaxGroups = 4096u;
constexpr int kMaxDevices = 64;

struct StaticScratch {
  Partial rec[2][kStaticMaxGroups];
  TileDesc desc;
  TileCtl ctl;
  WorkCtl work;
};

// One per process per device. Every call rewrites all of it that a tick reads (the descriptor,
// the control block, the work counter) before its launches; the records are written by the
// prime before the tick reads them. Two calls in flight at once on one device (on two streams, or
// from two host threads) share it and race: a caller runs them one after another.
static __device__ __align__(256) StaticScratch g_scratch;

// The descriptor in, the control block emptied (the ledger with no time left to count down, as
// write_state leaves it), every word of the work counter at zero.
__global__ void static_init_kernel(StaticScratch* s, TileDesc d) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  s->desc = d;
  TileCtl c = {};
  c.ledger[0].remaining_s = __int_as_float(0x7f800000);
  c.ledger[1] = c.ledger[0];
  s->ctl = c;
  s->work.next = 0u;
  s->work.exited = 0u;
  s->work.tail = 0u;
  s->work.fault = 0u;
}

std::mutex g_mu;
StaticScratch* g_addr[kMaxDevices] = {};

int put(char* err, size_t len, int code, const std::string& msg) {
  if (code != WL_OK && err != nullptr && len > 0) {
    const size_t k = msg.size() < len - 1 ? msg.size() : len - 1;
    std::memcpy(err, msg.data(), k);
    err[k] = '\0';
  }
  return code;
}

// The scratch's device address, looked up once per device with that device current.
StaticScratch* scratch_for(int device, std::string* msg) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_addr[device] != nullptr) return g_addr[device];
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) {
    *msg = std::string("water_live: the static scratch's address: ") + cudaGetErrorString(e);
    return nullptr;
  }
  g_addr[device] = static_cast<StaticScratch*>(p);
  return g_addr[device];
}

}  // namespace
}  // namespace wlc

extern "C" int wl_tick_noalloc(const wl_config* config, int fixed_ops, const float* planes_in,
                               float* planes_out, const float* bed, const float* manning,
                               const float* source, float max_dt, wl_stream stream, char* err,
                               size_t err_len) {
  using namespace wlc;
  if (config == nullptr || planes_in == nullptr || planes_out == nullptr || bed == nullptr)
    return put(err, err_len, WL_ERR_ARGUMENT, "water_live: no config, state or bed");
  if (planes_in == planes_out)
    return put(err, err_len, WL_ERR_ARGUMENT, "water_live: the tick reads one copy, writes another");
  if (config->nx == 0 || config->ny == 0)
    return put(err, err_len, WL_ERR_SIZE, "water_live: an empty grid");
  const uint32_t gx = (config->nx + 15u) / 16u, gy = (config->ny + 15u) / 16u;
  if (uint64_t(gx) * gy > kStaticMaxGroups)
    return put(err, err_len, WL_ERR_SIZE,
               "water_live: the grid has " + std::to_string(uint64_t(gx) * gy) +
                   " groups of 16 x 16; the allocation-free tick holds at most " +
                   std::to_string(kStaticMaxGroups) + " (1,048,576 cells as 1024 x 1024)");
  if (config->device < 0 || config->device >= kMaxDevices)
    return put(err, err_len, WL_ERR_ARGUMENT, "water_live: a device index out of range");
  if (cudaSetDevice(config->device) != cudaSuccess)
    return put(err, err_len, WL_ERR_CUDA, "water_live: cudaSetDevice");
  std::string msg;
  StaticScratch* s = scratch_for(config->device, &msg);
  if (s == nullptr) return put(err, err_len, WL_ERR_CUDA, msg);

  // The same shape rule as wl_create: three-phase blocks where the march's 32 x 32 items would
  // leave the device short of warps, else the 32 x 16 march.
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, config->device) != cudaSuccess)
    return put(err, err_len, WL_ERR_CUDA, "water_live: the SM count");
  const uint64_t items32 = uint64_t((config->nx + 31u) / 32u) * ((config->ny + 31u) / 32u);
  const BlockShape shape = items32 < uint64_t(sms) * 8u ? BlockShape::k32x16b : BlockShape::k32x16;
  uint32_t bx = 0, by = 0;
  block_dims(shape, bx, by);

  TileDesc d;
  std::memset(&d, 0, sizeof(d));
  d.state[0] = const_cast<float*>(planes_in);  // read only: the tick writes the other copy
  d.state[1] = planes_out;
  d.bed = bed;
  d.manning = manning;
  d.source = source;
  d.rec[0] = s->rec[0];
  d.rec[1] = s->rec[1];
  d.ctl = &s->ctl;
  d.nx = config->nx;
  d.ny = config->ny;
  d.groups_x = gx;
  d.groups_y = gy;
  d.flags = (config->west_open ? kFlagWestOpen : 0u) | (config->east_open ? kFlagEastOpen : 0u) |
            (config->south_open ? kFlagSouthOpen : 0u) |
            (config->north_open ? kFlagNorthOpen : 0u) | (manning ? kFlagManning : 0u) |
            (source ? kFlagSource : 0u);
  d.source_every = 1;
  d.cell_m = static_cast<float>(config->cell_m);
  d.gravity = static_cast<float>(config->gravity);
  d.cfl = static_cast<float>(config->cfl);
  d.dry = static_cast<float>(config->dry_depth_m);
  d.blocks_x = (config->nx + bx - 1u) / bx;
  d.blocks_y = (config->ny + by - 1u) / by;
  d.item_base = 0;
  d.items = d.blocks_x * d.blocks_y;

  const bool fixed = fixed_ops != 0, with_manning = manning != nullptr;
  const bool plain = (d.flags & kFlagsNotPlain) == 0u;
  const int occ = tick_occupancy(shape, fixed, with_manning, plain);
  if (occ <= 0) return put(err, err_len, WL_ERR_CUDA, "water_live: the tick cannot be resident");
  const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  static_init_kernel<<<1, 32, 0, st>>>(s, d);
  cudaError_t e = cudaGetLastError();
  TickArgs a{&s->desc, nullptr, &s->work, d.items, 0.0f};
  if (e == cudaSuccess) e = launch_prime(shape, fixed, a, st);  // the input's records
  a.max_dt = max_dt;
  const int grid = int(std::min<uint64_t>(d.items, uint64_t(sms) * occ));
  if (e == cudaSuccess) e = launch_tick(shape, fixed, with_manning, plain, a, grid, st);
  if (e != cudaSuccess)
    return put(err, err_len, WL_ERR_CUDA, std::string("water_live: ") + cudaGetErrorString(e));
  return WL_OK;
}

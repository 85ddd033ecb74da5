// The reference's complete FP64 step on the device: engine::water_state::Solver
// (domain/water_state/include/domain/water_state/water_state.h:161-266,
// domain/water_state/src/water_state.cpp) with every input and output, byte for byte.
//
// A step is six launches on the solver's stream (ws_solver.cu):
//   speeds   u = hu/h, v = hv/h (0 below the dry depth) and the largest |u| + c, |v| + c
//            (velocity_rows, cpp:185-209; a maximum is the same in any order, so atomicMax);
//   length   one thread: the stable step (cpp:211-224), this step's length, the carried
//            quantities' decay factors (cpp:330-334);
//   faces    every x and y face once (cpp:231-308), with the energy flux and the carried fluxes;
//   update   every cell (cpp:310-501): the state, the outputs, and each cell's share of the rows'
//            sums written to a plane;
//   rows     one thread a row and quantity: the row's sums in the reference's x order, the open
//            edges' terms first (cpp:337-363), so each row sum is the reference's to the bit;
//   ledger   one thread a quantity: the rows added in row order (cpp:514-531).
// The arithmetic is IEEE double with no contraction (the unit compiles with --fmad=false; double
// division and square root are correctly rounded), every expression in the reference's order, so
// the bytes equal the reference's CPU step at any grid.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <string>

namespace wsc {

constexpr uint32_t kMaxCarried = 4;  // water_state.h:53

struct Carried {
  double decay_s, per_joule, min_speed;  // water_state.h:66-78
};

// The per-cell shares of the rows' sums, one plane each: 5 + 4 a carried quantity.
enum Share : uint32_t { kShareSource = 0, kShareRoundoff, kShareGround, kShareLoss, kShareFriction,
                        kShareCarried };  // then per quantity: source, from_dissipation, exchange,
                                          // decayed
// The ledger's quantities in order: 6 + 5 a carried quantity (water_state.h:135-145).
enum LedgerQ : uint32_t { kQSource = 0, kQOpen, kQGround, kQRoundoff, kQLoss, kQFriction, kQCarried };

struct Ctl {
  unsigned long long a_bits, b_bits;  // the running maxima of |u| + c, |v| + c (bits of >= 0)
  double dt;                          // this step's length; 0: the step does nothing
  double max_dt;                      // a run of steps: each min(stable, max_dt)
  double remaining;                   // an advance: the time left
  double stable;                      // the last stable step (stable_step)
  uint32_t advance;                   // 1: the run is an advance
  uint32_t active;                    // an advance still going
  uint64_t taken;                     // steps taken in this run
  double keep[kMaxCarried];           // this step's decay factors
  double ledger[6 + 5 * kMaxCarried];
  double time_s;
  uint64_t steps;
};

struct Desc {
  uint32_t nx, ny, nk, open;  // open: west 1, east 2, south 4, north 8
  uint64_t n, xf, yf;         // cells, x faces ((nx + 1) ny), y faces (nx (ny + 1))
  double cell_m, g, cfl, dry, rho;
  Carried cc[kMaxCarried];
  double *h, *hu, *hv, *ground, *carried;                // the state
  double *speed, *tau_x, *tau_y, *diss;                  // the outputs
  const double *bed, *manning, *source, *gk, *gs, *gcap;  // the inputs (null: empty)
  const double* cs[kMaxCarried];
  const double* ce[kMaxCarried];
  double *u, *v;
  double *fx[5], *fy[5];  // h, nl, nr, t, g of every face
  double *fxc, *fyc;      // carried fluxes: nk planes of xf, of yf
  double* share;          // (5 + 4 nk) planes of n
  double* rows;           // ny x (6 + 5 nk)
  Ctl* ctl;
};

class Solver {
 public:
  ~Solver() { destroy(); }
  bool create(int device, const Desc& shape, std::string* err);
  void destroy();
  bool valid() const { return base_ != nullptr; }
  const Desc& desc() const { return d_; }
  cudaStream_t stream() const { return stream_; }
  int device() const { return device_; }

  // field: 0 depth, 1 momentum x, 2 momentum y, 3 ground, 4 carried (nk planes), 5 speed, 6 bed
  // stress x, 7 bed stress y, 8 dissipation.
  double* field(int which) const;
  size_t field_size(int which) const;
  bool write_field(int which, const double* v, std::string* err);
  bool read_field(int which, double* out, std::string* err);
  // input: 0 bed, 1 manning, 2 source, 3 ground conductivity, 4 suction, 5 capacity,
  // 6 + k carried source k, 10 + k carried exchange k. n = 0 empties it.
  bool set_input(int which, const double* v, size_t n, std::string* err);
  bool inputs_fit() const;  // water_state.cpp:150-169
  // `count` steps of min(stable, max_dt), or (advance) steps until `duration` has passed.
  cudaError_t enqueue_steps(cudaStream_t s, uint32_t count, double max_dt);
  cudaError_t enqueue_advance_start(cudaStream_t s, double duration);
  cudaError_t enqueue_advance_steps(cudaStream_t s, uint32_t count);
  cudaError_t enqueue_stable_step(cudaStream_t s);
  bool read_ctl(Ctl& out, std::string* err);
  bool reset_ledger(std::string* err);
  bool wait(std::string* err);
  uint64_t device_bytes() const { return bytes_; }

 private:
  cudaError_t enqueue_step(cudaStream_t s);
  int device_ = -1;
  cudaStream_t stream_ = nullptr;
  char* base_ = nullptr;
  uint64_t bytes_ = 0;
  Desc d_{};
  bool present_[14] = {};  // which inputs hold a span
  double* in_base_ = nullptr;  // the input planes: 6 named, then carried sources, then exchanges
  size_t in_stride_ = 0;       // doubles from one input plane to the next
};

}  // namespace wsc

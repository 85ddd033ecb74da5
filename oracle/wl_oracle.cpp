// ORACLE — test infrastructure only (see wl_oracle.hpp). A flat C ABI over the restatement, for
// the tests' ctypes bindings (tests/oracle.py) and bench.py's CPU-baseline leg.
#include "wl_oracle.hpp"
#include "wl_adjoint.hpp"

#include <atomic>
#include <chrono>
#include <cstdlib>
#include <new>

using namespace wl_oracle;

namespace {

struct StepHandle {
  bool is64 = false;
  RefStep<float> f32;
  RefStep<double> f64;
};

struct SolverHandle {
  Solver64 solver;
  std::vector<double> bed, manning, source;
  SolverHandle(const Config& c, u32 threads) : solver(c, threads) {}
};

Config make_config(u32 nx, u32 ny, double cell_m, double gravity, double cfl, double dry,
                   u32 open_edges) {
  Config c;
  c.nx = nx;
  c.ny = ny;
  c.cell_m = cell_m;
  c.gravity = gravity;
  c.cfl = cfl;
  c.dry_depth_m = dry;
  c.west_open = (open_edges & 1u) ? 1 : 0;
  c.east_open = (open_edges & 2u) ? 1 : 0;
  c.south_open = (open_edges & 4u) ? 1 : 0;
  c.north_open = (open_edges & 8u) ? 1 : 0;
  return c;
}

template <class T>
void ledger_out(const LedgerF64& l, double* out) {
  out[0] = l.source_m3;
  out[1] = l.open_edge_out_m3;
  out[2] = l.roundoff_m3;
  out[3] = l.time_s;
  out[4] = l.remaining_s;
  out[5] = double(l.steps);
}

}  // namespace

extern "C" {

uint64_t oracle_hash_floats(const float* v, size_t n) { return hash_floats(v, n); }

// ---- the card's step -------------------------------------------------------------------------

void* oracle_step_create(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                         double dry, uint32_t open_edges, int fixed_ops, int precision64) {
  auto* h = new (std::nothrow) StepHandle;
  if (h == nullptr) return nullptr;
  h->is64 = precision64 != 0;
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  const bool ok = h->is64 ? h->f64.create(c, fixed_ops != 0) : h->f32.create(c, fixed_ops != 0);
  if (!ok) {
    delete h;
    return nullptr;
  }
  return h;
}

void oracle_step_destroy(void* p) { delete static_cast<StepHandle*>(p); }

void oracle_step_write_state(void* p, const double* h, const double* hu, const double* hv) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.write_state(h, hu, hv); else s->f32.write_state(h, hu, hv);
}

void oracle_step_set_bed(void* p, const double* bed, double datum) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.set_bed(bed, datum); else s->f32.set_bed(bed, datum);
}

void oracle_step_set_manning(void* p, const double* m) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.set_manning(m); else s->f32.set_manning(m);
}

void oracle_step_set_source(void* p, const double* src, uint32_t every, int compensate) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.set_source(src, every, compensate != 0);
  else s->f32.set_source(src, every, compensate != 0);
}

void oracle_step_run_steps(void* p, uint32_t count, double max_dt) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.run_steps(count, max_dt);
  else s->f32.run_steps(count, static_cast<float>(max_dt));
}

void oracle_step_run_length_pass(void* p, double max_dt) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.run_length_pass(max_dt);
  else s->f32.run_length_pass(static_cast<float>(max_dt));
}

void oracle_step_read_ledger(void* p, double* out6) {
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) ledger_out<double>(s->f64.read_ledger(), out6);
  else ledger_out<float>(s->f32.read_ledger(), out6);
}

uint64_t oracle_step_advance(void* p, double duration, int* refused) {
  auto* s = static_cast<StepHandle*>(p);
  bool r = false;
  const uint64_t steps = s->is64 ? s->f64.advance(duration, &r) : s->f32.advance(duration, &r);
  if (refused) *refused = r ? 1 : 0;
  return steps;
}

// All four planes of the current copy, as the step holds them (float: 4 n values).
void oracle_step_read_state_f32(void* p, float* out) {
  auto* s = static_cast<StepHandle*>(p);
  std::memcpy(out, s->f32.planes(), sizeof(float) * k_state_planes * s->f32.n);
}

void oracle_step_read_state_f64(void* p, double* out) {
  auto* s = static_cast<StepHandle*>(p);
  std::memcpy(out, s->f64.planes(), sizeof(double) * k_state_planes * s->f64.n);
}

void oracle_step_prime(void* p) {  // prime_main (slang:373-386) of the state as it stands
  auto* s = static_cast<StepHandle*>(p);
  if (s->is64) s->f64.prime_records();
  else s->f32.prime_records();
}

void oracle_step_write_planes_f32(void* p, const float* planes) {  // a raw upload, for the tests
  auto* s = static_cast<StepHandle*>(p);
  std::memcpy(s->f32.planes_mut(), planes, sizeof(float) * k_state_planes * s->f32.n);
}

uint64_t oracle_step_state_hash(void* p) {
  auto* s = static_cast<StepHandle*>(p);
  return s->is64 ? 0 : s->f32.state_hash();
}

uint32_t oracle_step_group_count(void* p) {
  auto* s = static_cast<StepHandle*>(p);
  return s->is64 ? s->f64.gx * s->f64.gy : s->f32.gx * s->f32.gy;
}

// The records (8 floats each) and the ledger's 48 bytes, float instantiation.
void oracle_step_read_partials(void* p, float* out) {
  auto* s = static_cast<StepHandle*>(p);
  std::memcpy(out, s->f32.partials.data(), sizeof(Partial<float>) * s->f32.partials.size());
}

void oracle_step_read_ledger_bits(void* p, void* out48) {
  auto* s = static_cast<StepHandle*>(p);
  static_assert(sizeof(LedgerBits<float>) == 48, "the ledger is 48 bytes");
  std::memcpy(out48, &s->f32.ledger, 48);
}

// ---- the reference CPU tick in double ---------------------------------------------------------

void* oracle_solver_create(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                           double dry, uint32_t open_edges, uint32_t threads) {
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  return new (std::nothrow) SolverHandle(c, threads);
}

void oracle_solver_destroy(void* p) { delete static_cast<SolverHandle*>(p); }

// Depth and momenta (n values each); the inputs are copied (null: none).
void oracle_solver_set_state(void* p, const double* h, const double* hu, const double* hv) {
  auto* s = static_cast<SolverHandle*>(p);
  const size_t n = s->solver.n;
  std::memcpy(s->solver.h.data(), h, n * sizeof(double));
  std::memcpy(s->solver.hu.data(), hu, n * sizeof(double));
  std::memcpy(s->solver.hv.data(), hv, n * sizeof(double));
}

void oracle_solver_set_inputs(void* p, const double* bed, const double* manning,
                              const double* source) {
  auto* s = static_cast<SolverHandle*>(p);
  const size_t n = s->solver.n;
  auto copy = [n](std::vector<double>& dst, const double* src) -> const double* {
    if (src == nullptr) { dst.clear(); return nullptr; }
    dst.assign(src, src + n);
    return dst.data();
  };
  s->solver.bed = copy(s->bed, bed);
  s->solver.manning = copy(s->manning, manning);
  s->solver.source = copy(s->source, source);
}

double oracle_solver_step(void* p, double max_dt) {
  return static_cast<SolverHandle*>(p)->solver.step(max_dt);
}

uint64_t oracle_solver_advance(void* p, double duration) {
  return static_cast<SolverHandle*>(p)->solver.advance(duration);
}

void oracle_solver_get_state(void* p, double* h, double* hu, double* hv) {
  auto* s = static_cast<SolverHandle*>(p);
  const size_t n = s->solver.n;
  std::memcpy(h, s->solver.h.data(), n * sizeof(double));
  std::memcpy(hu, s->solver.hu.data(), n * sizeof(double));
  std::memcpy(hv, s->solver.hv.data(), n * sizeof(double));
}

uint64_t oracle_solver_state_hash(void* p) { return static_cast<SolverHandle*>(p)->solver.state_hash(); }

void oracle_solver_ledger(void* p, double* out5) {
  auto* s = static_cast<SolverHandle*>(p);
  out5[0] = s->solver.ledger.source_m3;
  out5[1] = s->solver.ledger.open_edge_out_m3;
  out5[2] = s->solver.ledger.roundoff_m3;
  out5[3] = s->solver.ledger.time_s;
  out5[4] = double(s->solver.ledger.steps);
}

double oracle_solver_volume(void* p) { return static_cast<SolverHandle*>(p)->solver.surface_volume_m3(); }

// ---- the adjoint's checks (wl_adjoint.hpp) ---------------------------------------------------

// `ticks` fixed-length ticks from state0 (3 planes) into out (3 planes); returns the number of
// ticks the card would have shortened.
uint32_t oracle_adj_forward(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                            double dry, uint32_t open_edges, int precision64, double dt,
                            uint32_t ticks, const double* bed, const double* src,
                            const double* state0, double* out) {
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  const size_t n = size_t(nx) * ny;
  auto run = [&](auto zero) {
    using T = decltype(zero);
    std::vector<T> b(n), s, a(3 * n), o(3 * n);
    for (size_t i = 0; i < n; ++i) b[i] = T(bed[i]);
    if (src) {
      s.resize(n);
      for (size_t i = 0; i < n; ++i) s[i] = T(src[i]);
    }
    for (size_t i = 0; i < 3 * n; ++i) a[i] = T(state0[i]);
    uint32_t lim = 0;
    for (uint32_t t = 0; t < ticks; ++t) {
      if (limited<T>(c, T(dt), a.data())) ++lim;
      forward_tick<T>(c, T(dt), b.data(), src ? s.data() : nullptr, a.data(), o.data(), nullptr);
      a.swap(o);
    }
    for (size_t i = 0; i < 3 * n; ++i) out[i] = double(a[i]);
    return lim;
  };
  return precision64 ? run(0.0) : run(0.0f);
}

// The loss and its gradients by the reverse sweep (the whole trajectory kept); returns the number
// of shortened ticks.
uint32_t oracle_adjoint(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                        double dry, uint32_t open_edges, int precision64, double dt, uint32_t ticks,
                        const double* bed, const double* src, const double* state0,
                        const uint32_t* probes, const double* targets, uint32_t n_probes,
                        double* loss, double* g_bed, double* g_src, double* g_state0) {
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  return precision64
             ? adjoint<double>(c, dt, ticks, bed, src, state0, probes, targets, n_probes, loss,
                               g_bed, g_src, g_state0)
             : adjoint<float>(c, dt, ticks, bed, src, state0, probes, targets, n_probes, loss,
                              g_bed, g_src, g_state0);
}

// The FP32 forward with the FP64 reverse sweep over it.
uint32_t oracle_adjoint_mixed(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                              double dry, uint32_t open_edges, double dt, uint32_t ticks,
                              const double* bed, const double* src, const double* state0,
                              const uint32_t* probes, const double* targets, uint32_t n_probes,
                              double* loss, double* g_bed, double* g_src) {
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  return adjoint_mixed(c, dt, ticks, bed, src, state0, probes, targets, n_probes, loss, g_bed,
                       g_src);
}

// Central differences of the FP64 replay's loss: for each listed cell, (L(p + e) - L(p - e)) / 2e
// with e = eps_bed on the bed and (when fd_src is not null and there is a source) e = rel_src *
// |source| (eps_bed where the source is 0) on the source. The replays are dealt to `threads`
// threads.
void oracle_adj_fd(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl, double dry,
                   uint32_t open_edges, double dt, uint32_t ticks, const double* bed,
                   const double* src, const double* state0, const uint32_t* probes,
                   const double* targets, uint32_t n_probes, const uint32_t* cells,
                   uint32_t n_cells, double eps_bed, double rel_src, double* fd_bed,
                   double* fd_src, uint32_t threads) {
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  const size_t n = size_t(nx) * ny;
  const uint32_t jobs = n_cells * ((src && fd_src) ? 2u : 1u);
  std::atomic<uint32_t> next{0};
  auto worker = [&]() {
    std::vector<double> b(bed, bed + n), s;
    if (src) s.assign(src, src + n);
    for (;;) {
      const uint32_t j = next.fetch_add(1);
      if (j >= jobs) break;
      const bool on_src = j >= n_cells;
      const uint32_t cell = cells[on_src ? j - n_cells : j];
      std::vector<double>& p = on_src ? s : b;
      const double base = p[cell];
      const double e = on_src ? (base != 0.0 ? rel_src * std::fabs(base) : eps_bed) : eps_bed;
      p[cell] = base + e;
      const double lp = loss_fp64(c, dt, ticks, b.data(), src ? s.data() : nullptr, state0,
                                  probes, targets, n_probes);
      p[cell] = base - e;
      const double lm = loss_fp64(c, dt, ticks, b.data(), src ? s.data() : nullptr, state0,
                                  probes, targets, n_probes);
      p[cell] = base;
      (on_src ? fd_src : fd_bed)[on_src ? j - n_cells : j] = (lp - lm) / (2.0 * e);
    }
  };
  const uint32_t nt = threads ? threads : 1u;
  std::vector<std::thread> pool;
  for (uint32_t t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
}

// The FP64 replay's loss alone.
double oracle_adj_loss64(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                         double dry, uint32_t open_edges, double dt, uint32_t ticks,
                         const double* bed, const double* src, const double* state0,
                         const uint32_t* probes, const double* targets, uint32_t n_probes) {
  const Config c = make_config(nx, ny, cell_m, gravity, cfl, dry, open_edges);
  return loss_fp64(c, dt, ticks, bed, src, state0, probes, targets, n_probes);
}

}  // extern "C"

// ---- the complete FP64 step (ws_oracle.hpp) ----------------------------------------------------
//
// Inputs come as 14 pointers, null for an empty span: bed, manning, source, ground conductivity,
// ground suction, ground capacity, carried source 0-3, carried exchange 0-3.

#include "ws_oracle.hpp"

namespace {

ws_oracle::Inputs ws_inputs(const double* const* p) {
  ws_oracle::Inputs in;
  in.bed = p[0];
  in.manning = p[1];
  in.source = p[2];
  in.ground_k = p[3];
  in.ground_s = p[4];
  in.ground_cap = p[5];
  for (int k = 0; k < 4; ++k) {
    in.carried_source[k] = p[6 + k];
    in.carried_exchange[k] = p[10 + k];
  }
  return in;
}

}  // namespace

extern "C" {

void* oracle_ws_create(uint32_t nx, uint32_t ny, double cell_m, double gravity, double cfl,
                       double dry, double rho, uint32_t open_edges, uint32_t carried,
                       const double* cc) {
  ws_oracle::Config c;
  c.nx = nx;
  c.ny = ny;
  c.cell_m = cell_m;
  c.gravity = gravity;
  c.cfl = cfl;
  c.dry = dry;
  c.rho = rho;
  c.carried = carried;
  for (uint32_t k = 0; k < carried && k < 4; ++k) c.cc[k] = {cc[3 * k], cc[3 * k + 1], cc[3 * k + 2]};
  c.west_open = open_edges & 1u;
  c.east_open = open_edges & 2u;
  c.south_open = open_edges & 4u;
  c.north_open = open_edges & 8u;
  return new (std::nothrow) ws_oracle::SolverFull(c);
}

void oracle_ws_destroy(void* p) { delete static_cast<ws_oracle::SolverFull*>(p); }

// which: 0 depth, 1 momentum x, 2 momentum y, 3 ground, 4 carried (k * n), 5 speed, 6 bed
// stress x, 7 bed stress y, 8 dissipation.
static std::vector<double>& ws_field(ws_oracle::SolverFull* s, int which) {
  switch (which) {
    case 0: return s->h;
    case 1: return s->hu;
    case 2: return s->hv;
    case 3: return s->ground;
    case 4: return s->carried;
    case 5: return s->speed;
    case 6: return s->tau_x;
    case 7: return s->tau_y;
    default: return s->dissipation;
  }
}

void oracle_ws_set(void* p, int which, const double* v) {
  auto* s = static_cast<ws_oracle::SolverFull*>(p);
  std::vector<double>& f = ws_field(s, which);
  std::memcpy(f.data(), v, f.size() * sizeof(double));
}

void oracle_ws_get(void* p, int which, double* out) {
  auto* s = static_cast<ws_oracle::SolverFull*>(p);
  const std::vector<double>& f = ws_field(s, which);
  std::memcpy(out, f.data(), f.size() * sizeof(double));
}

double oracle_ws_step(void* p, const double* const* inputs, double max_dt) {
  return static_cast<ws_oracle::SolverFull*>(p)->step(ws_inputs(inputs), max_dt);
}

uint64_t oracle_ws_advance(void* p, const double* const* inputs, double duration) {
  return static_cast<ws_oracle::SolverFull*>(p)->advance(ws_inputs(inputs), duration);
}

double oracle_ws_stable_step(void* p) { return static_cast<ws_oracle::SolverFull*>(p)->stable_step(); }

// source, open, ground, roundoff, scheme_loss, friction, time, steps, then per carried quantity
// source, from_dissipation, exchange, decayed, open (28 doubles).
void oracle_ws_ledger(void* p, double* out) {
  const ws_oracle::Ledger& l = static_cast<ws_oracle::SolverFull*>(p)->ledger;
  const double head[8] = {l.source, l.open, l.ground, l.roundoff, l.scheme_loss, l.friction,
                          l.time, double(l.steps)};
  std::memcpy(out, head, sizeof head);
  for (int k = 0; k < 4; ++k) {
    const ws_oracle::CarriedLedger& c = l.carried[k];
    const double v[5] = {c.source, c.from_dissipation, c.exchange, c.decayed, c.open};
    std::memcpy(out + 8 + 5 * k, v, sizeof v);
  }
}

uint64_t oracle_ws_hash(void* p) { return static_cast<ws_oracle::SolverFull*>(p)->state_hash(); }

void oracle_fd_exp_n(const double* x, double* out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = ws_oracle::fd_exp(x[i]);
}

void oracle_fd_log_n(const double* x, double* out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = ws_oracle::fd_log(x[i]);
}

}  // extern "C"

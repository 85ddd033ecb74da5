// ORACLE — test infrastructure only (see wl_oracle.hpp). A flat C ABI over the restatement, for
// the tests' ctypes bindings (tests/oracle.py) and bench.py's CPU-baseline leg.
#include "wl_oracle.hpp"

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

}  // extern "C"

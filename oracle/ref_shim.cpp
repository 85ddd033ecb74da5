// ORACLE — test infrastructure only. A flat C ABI over the reference's own CPU solver,
// engine::water_state::Solver (domain/water_state/include/domain/water_state/water_state.h:161-266),
// compiled from the reference's sources by oracle/build_ref.sh into oracle/_ref/libwsref.so. The
// tests use it to check the oracle's restatement (Solver64, RefStep<double>) byte for byte, and to
// time the reference's CPU tick on this host's cores. This file is this project's own code; the
// reference's sources stay where they lie and are never copied.
#include <core/jobs/job_system.h>
#include <domain/water_state/water_state.h>

#include <cstring>
#include <new>
#include <vector>

using namespace engine;

namespace {

struct Handle {
  water_state::Solver solver;
  std::vector<f64> bed, manning, source;
  jobs::JobSystem* pool = nullptr;
  explicit Handle(const water_state::Config& c) : solver(c) {}
  ~Handle() { delete pool; }
  water_state::Inputs inputs() const {
    water_state::Inputs in;
    in.bed_m = bed;
    if (!manning.empty()) in.manning = manning;
    if (!source.empty()) in.source_m_per_s = source;
    return in;
  }
};

}  // namespace

extern "C" {

void* wsref_create(u32 nx, u32 ny, double cell_m, double gravity, double cfl, double dry,
                   u32 open_edges, u32 workers) {
  water_state::Config c;
  c.nx = nx;
  c.ny = ny;
  c.cell_m = cell_m;
  c.gravity = gravity;
  c.cfl = cfl;
  c.dry_depth_m = dry;
  using water_state::Edge;
  c.edges.west = (open_edges & 1u) ? Edge::open : Edge::closed;
  c.edges.east = (open_edges & 2u) ? Edge::open : Edge::closed;
  c.edges.south = (open_edges & 4u) ? Edge::open : Edge::closed;
  c.edges.north = (open_edges & 8u) ? Edge::open : Edge::closed;
  auto* h = new (std::nothrow) Handle(c);
  if (h == nullptr) return nullptr;
  if (workers > 0) {
    jobs::JobSystemConfig jc;
    jc.performance_workers = workers;
    jc.efficiency_workers = 1;
    jc.pin_threads = false;
    h->pool = new jobs::JobSystem(jc);
  }
  return h;
}

void wsref_destroy(void* p) { delete static_cast<Handle*>(p); }

void wsref_set_state(void* p, const double* h, const double* hu, const double* hv) {
  auto* s = static_cast<Handle*>(p);
  const usize n = s->solver.cell_count();
  std::memcpy(s->solver.depth().data(), h, n * sizeof(double));
  std::memcpy(s->solver.momentum_x().data(), hu, n * sizeof(double));
  std::memcpy(s->solver.momentum_y().data(), hv, n * sizeof(double));
}

void wsref_set_inputs(void* p, const double* bed, const double* manning, const double* source) {
  auto* s = static_cast<Handle*>(p);
  const usize n = s->solver.cell_count();
  s->bed.assign(bed, bed + n);
  if (manning) s->manning.assign(manning, manning + n); else s->manning.clear();
  if (source) s->source.assign(source, source + n); else s->source.clear();
}

double wsref_step(void* p, double max_dt) {
  auto* s = static_cast<Handle*>(p);
  return s->solver.step(s->inputs(), max_dt, s->pool);
}

u64 wsref_advance(void* p, double duration) {
  auto* s = static_cast<Handle*>(p);
  return s->solver.advance(s->inputs(), duration, s->pool);
}

void wsref_get_state(void* p, double* h, double* hu, double* hv) {
  auto* s = static_cast<Handle*>(p);
  const usize n = s->solver.cell_count();
  std::memcpy(h, s->solver.depth().data(), n * sizeof(double));
  std::memcpy(hu, s->solver.momentum_x().data(), n * sizeof(double));
  std::memcpy(hv, s->solver.momentum_y().data(), n * sizeof(double));
}

u64 wsref_state_hash(void* p) { return static_cast<Handle*>(p)->solver.state_hash(); }

void wsref_ledger(void* p, double* out5) {
  const water_state::Ledger& l = static_cast<Handle*>(p)->solver.ledger();
  out5[0] = l.source_m3;
  out5[1] = l.open_edge_out_m3;
  out5[2] = l.roundoff_m3;
  out5[3] = l.time_s;
  out5[4] = static_cast<double>(l.steps);
}

double wsref_volume(void* p) { return static_cast<Handle*>(p)->solver.surface_volume_m3(); }

}  // extern "C"

// ---- the reference's complete step: ground, carried quantities, outputs, the whole ledger ------
//
// The same layout as oracle_ws_* (oracle/wl_oracle.cpp): inputs as 14 pointers (bed, manning,
// source, ground conductivity, suction, capacity, carried source 0-3, carried exchange 0-3), null
// for an empty span; fields by number (0 depth, 1 momentum x, 2 momentum y, 3 ground, 4 carried,
// 5 speed, 6 bed stress x, 7 bed stress y, 8 dissipation); the ledger as 28 doubles.

#include <core/math/deterministic.h>

namespace {

struct FullHandle {
  water_state::Solver solver;
  explicit FullHandle(const water_state::Config& c) : solver(c) {}
};

water_state::Inputs full_inputs(const water_state::Solver& s, const double* const* p) {
  const usize n = s.cell_count();
  auto span = [n](const double* q) { return q ? std::span<const f64>(q, n) : std::span<const f64>(); };
  water_state::Inputs in;
  in.bed_m = span(p[0]);
  in.manning = span(p[1]);
  in.source_m_per_s = span(p[2]);
  in.ground_conductivity_m_per_s = span(p[3]);
  in.ground_suction_m = span(p[4]);
  in.ground_capacity_m = span(p[5]);
  for (int k = 0; k < 4; ++k) {
    in.carried_source[k] = span(p[6 + k]);
    in.carried_exchange[k] = span(p[10 + k]);
  }
  return in;
}

std::span<f64> full_field(water_state::Solver& s, int which) {
  const u32 k = s.config().carried;
  switch (which) {
    case 0: return s.depth();
    case 1: return s.momentum_x();
    case 2: return s.momentum_y();
    case 3: return s.ground();
    case 4: return k ? std::span<f64>(s.carried(0).data(), usize{k} * s.cell_count())
                     : std::span<f64>();
    default: return {};
  }
}

}  // namespace

extern "C" {

void* wsref_full_create(u32 nx, u32 ny, double cell_m, double gravity, double cfl, double dry,
                        double rho, u32 open_edges, u32 carried, const double* cc) {
  water_state::Config c;
  c.nx = nx;
  c.ny = ny;
  c.cell_m = cell_m;
  c.gravity = gravity;
  c.cfl = cfl;
  c.dry_depth_m = dry;
  c.water_density = rho;
  c.carried = carried;
  for (u32 k = 0; k < carried && k < water_state::k_max_carried; ++k) {
    c.carried_config[k].decay_s = cc[3 * k];
    c.carried_config[k].per_joule = cc[3 * k + 1];
    c.carried_config[k].min_speed_m_per_s = cc[3 * k + 2];
  }
  using water_state::Edge;
  c.edges.west = (open_edges & 1u) ? Edge::open : Edge::closed;
  c.edges.east = (open_edges & 2u) ? Edge::open : Edge::closed;
  c.edges.south = (open_edges & 4u) ? Edge::open : Edge::closed;
  c.edges.north = (open_edges & 8u) ? Edge::open : Edge::closed;
  return new (std::nothrow) FullHandle(c);
}

void wsref_full_destroy(void* p) { delete static_cast<FullHandle*>(p); }

void wsref_full_set(void* p, int which, const double* v) {
  std::span<f64> f = full_field(static_cast<FullHandle*>(p)->solver, which);
  if (!f.empty()) std::memcpy(f.data(), v, f.size() * sizeof(double));
}

void wsref_full_get(void* p, int which, double* out) {
  water_state::Solver& s = static_cast<FullHandle*>(p)->solver;
  std::span<const f64> f;
  switch (which) {
    case 5: f = s.speed(); break;
    case 6: f = s.bed_stress_x(); break;
    case 7: f = s.bed_stress_y(); break;
    case 8: f = s.dissipation(); break;
    default: f = full_field(s, which); break;
  }
  if (!f.empty()) std::memcpy(out, f.data(), f.size() * sizeof(double));
}

double wsref_full_step(void* p, const double* const* inputs, double max_dt) {
  water_state::Solver& s = static_cast<FullHandle*>(p)->solver;
  return s.step(full_inputs(s, inputs), max_dt, nullptr);
}

u64 wsref_full_advance(void* p, const double* const* inputs, double duration) {
  water_state::Solver& s = static_cast<FullHandle*>(p)->solver;
  return s.advance(full_inputs(s, inputs), duration, nullptr);
}

void wsref_full_ledger(void* p, double* out) {
  const water_state::Ledger& l = static_cast<FullHandle*>(p)->solver.ledger();
  const double head[8] = {l.source_m3, l.open_edge_out_m3, l.ground_m3, l.roundoff_m3,
                          l.scheme_loss_j, l.friction_work_j, l.time_s, double(l.steps)};
  std::memcpy(out, head, sizeof head);
  for (u32 k = 0; k < 4; ++k) {
    const water_state::CarriedLedger& c = l.carried[k];
    const double v[5] = {c.source, c.from_dissipation, c.exchange, c.decayed, c.open_edge_out};
    std::memcpy(out + 8 + 5 * k, v, sizeof v);
  }
}

u64 wsref_full_hash(void* p) { return static_cast<FullHandle*>(p)->solver.state_hash(); }

void wsref_det_exp_n(const double* x, double* out, usize n) {
  for (usize i = 0; i < n; ++i) out[i] = det::exp(x[i]);
}

void wsref_det_log_n(const double* x, double* out, usize n) {
  for (usize i = 0; i < n; ++i) out[i] = det::log(x[i]);
}

}  // extern "C"

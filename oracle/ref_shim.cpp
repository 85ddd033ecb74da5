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

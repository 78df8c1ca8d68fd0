// C entry points over the reference's own per-particle functions, compiled
// from the reference's headers as they stand (no edits) against the Kokkos
// stand-in in kokkos_shim/.  Test infrastructure only: tests/golden/
// make_ref_golden.py calls them to write golden vectors, and the oracle's
// functions are checked against those vectors bit for bit.
//
// Compiled reference code (paths relative to the BioCMA-MCST tree):
//   apps/libs/simulation/public/simulation/kernels/move_kernel.hpp
//     __find_next_compartment (L62-L103), MoveFunctor::handle_move
//     (L393-L437), MoveFunctor::operator()(TagLeave) (L348-L359) and
//     handle_exit (L588-L648)
//   apps/libs/simulation/public/simulation/probability_leaving.hpp L18-L48
//   apps/libs/models/public/models/fixed_length.hpp L123-L161
//   apps/libs/models/public/models/simple_acetate.hpp L129-L250
//   apps/libs/models/public/models/utils.hpp L64-L69 (check_div)
//   apps/libs/mc/public/mc/prng/prng_extension.hpp L82-L147 (erfinv,
//     norminv) and TruncatedNormal::draw_from
//   apps/libs/simulation/src/feed_descriptor.cpp L12-L36, L100-L103
//     (FeedDescriptor::update, compiled from the source file) and
//   apps/libs/simulation/public/simulation/simulation_times.hpp L15-L18
//     (SimulatimeTimes::advance)
#include <simulation/kernels/move_kernel.hpp>
#include <simulation/feed_descriptor.hpp>
#include <simulation/simulation_times.hpp>
#include <models/fixed_length.hpp>
#include <models/simple_acetate.hpp>

#include <cstdint>
#include <vector>

namespace {
using Exec = ComputeSpace;

void set_tape(const double* v, int n) {
  auto& t = Kokkos::Impl::tape();
  t.v.assign(v, v + (n > 0 ? n : 0));
  t.pos = 0;
}

struct Domain {
  std::vector<std::size_t> nbr;
  MC::DomainState<Exec, true> st;
  Domain(uint32_t n_c, uint32_t K, const double* volume, const double* diag, const uint64_t* neighbors,
         const double* cdf, const MC::LeavingFlow* flows, uint32_t n_flows)
      : nbr(neighbors, neighbors + (std::size_t)n_c * K) {
    st.neighbors = MC::NeighborsView<Exec, true>(nbr.data(), n_c, K);
    st.cumulative_probability = MC::CumulativeProbabilityView<Exec, true>(cdf, n_c, K);
    st.diag_transition = MC::DiagonalView<Exec, true>(diag, n_c);
    st.liquid_volume = MC::VolumeView<Exec, true>(volume, n_c);
    st.leaving_flow = MC::LeavingFlowView<true>(flows, n_flows);
  }
};
}  // namespace

extern "C" {

long ref_assert_failures(void) { return refpin::assert_failures(); }
void ref_reset_assert_failures(void) { refpin::assert_failures() = 0; }

// __find_next_compartment(do_search, neighbors, cdf, i, u)
uint64_t ref_find_next(int32_t do_search, uint32_t n_c, uint32_t K, const uint64_t* neighbors, const double* cdf,
                       uint64_t i, double u) {
  std::vector<std::size_t> nbr(neighbors, neighbors + (std::size_t)n_c * K);
  MC::NeighborsView<Exec, true> nv(nbr.data(), n_c, K);
  MC::CumulativeProbabilityView<Exec, true> cv(cdf, n_c, K);
  return Simulation::KernelInline::__find_next_compartment(do_search != 0, nv, cv, i, u);
}

int32_t ref_leave_fast(float u, double volume, double flow, double dt) {
  return Simulation::KernelInline::probability_leaving<Simulation::KernelInline::fast_tag>(u, volume, flow, dt);
}

int32_t ref_leave_precise(float u, double volume, double flow, double dt) {
  return Simulation::KernelInline::probability_leaving<Simulation::KernelInline::precision_tag>(u, volume, flow, dt);
}

// MoveFunctor::handle_move on one particle at `pos`: returns its new
// position; *moved = the Move events counted.
uint64_t ref_handle_move(uint32_t n_c, uint32_t K, const double* volume, const double* diag, const uint64_t* neighbors,
                         const double* cdf, double dt, uint64_t pos, float u1, float u2, uint64_t* moved) {
  Domain d(n_c, K, volume, diag, neighbors, cdf, nullptr, 0);
  MC::ParticlePositions p("pos", 1);
  MC::ParticleStatus status("status", 1);
  MC::ParticleAges ages("ages", 1);
  p(0) = pos;
  Simulation::KernelInline::MoveFunctor f(1024, 0, dt, p, status, 1, d.st, MC::pool_type(), MC::EventContainer(),
                                          Simulation::ProbeAutogeneratedBuffer(), ages, true, false);
  f.handle_move(0, u1, u2);
  if (moved) *moved = f.events.get<MC::EventType::Move>();
  return p(0);
}

// MoveFunctor::operator()(TagLeave, idx, dead) on one particle: the age and
// status after it, the exits counted; the exit draw is `u` (the pool's frand).
uint64_t ref_leave_one(uint32_t n_flows, const uint64_t* index, const double* flow, const double* volume_at,
                       double dt, uint64_t pos, int32_t status_in, float age_in, float u, int32_t* status_out,
                       float* age_out) {
  std::vector<MC::LeavingFlow> lf(n_flows);
  for (uint32_t k = 0; k < n_flows; ++k) lf[k] = MC::LeavingFlow{index[k], flow[k], volume_at[k]};
  MC::ParticlePositions p("pos", 1);
  MC::ParticleStatus status("status", 1);
  MC::ParticleAges ages("ages", 1);
  p(0) = pos;
  status(0) = static_cast<MC::Status>(status_in);
  ages(0, 0) = age_in;
  MC::DomainState<Exec, true> st;
  st.leaving_flow = MC::LeavingFlowView<true>(lf.data(), n_flows);
  Simulation::KernelInline::MoveFunctor f(1024, 0, dt, p, status, 1, st, MC::pool_type(), MC::EventContainer(),
                                          Simulation::ProbeAutogeneratedBuffer(), ages, false, true);
  const double tape[1] = {static_cast<double>(u)};
  set_tape(tape, 1);
  std::size_t dead = 0;
  f(Simulation::KernelInline::TagLeave{}, 0, dead);
  *status_out = static_cast<int32_t>(status(0));
  *age_out = ages(0, 0);
  return dead;
}

// FixedLength::update on one particle with state x = {length, l_max} in the
// compartment whose substrate concentration is `s`.
int32_t ref_fixed_length_update(float dt, float* x, double s, float* contrib) {
  using M = Models::FixedLength;
  M::SelfParticle arr(x, 1);
  M::SelfContribs ctb(contrib, 1);
  const double c[1] = {s};
  MC::LocalConcentration conc(c, 1, 1);
  return static_cast<int32_t>(M::update(MC::pool_type(), dt, 0, arr, ctb, 0, conc));
}

void ref_fixed_length_division(float* x, float* child) {
  using M = Models::FixedLength;
  M::SelfParticle arr(x, 1);
  M::SelfParticle buf(child, 1);
  M::division(MC::pool_type(), 0, 0, arr, buf);
}

// SimpleAcetate::update with state x[9] in a compartment with glucose c0 and
// acetate c1; contributions to contribs[2].
int32_t ref_simple_acetate_update(float dt, float* x, double c0, double c1, float* contribs) {
  using M = Models::SimpleAcetate;
  M::SelfParticle arr(x, 1);
  M::SelfContribs ctb(contribs, 1);
  const double c[2] = {c0, c1};
  MC::LocalConcentration conc(c, 2, 1);
  return static_cast<int32_t>(M::update(MC::pool_type(), dt, 0, arr, ctb, 0, conc));
}

// SimpleAcetate::division with the draws on the tape: two standard normals
// (the log-normal a_p of mother and child), then two uniforms (the truncated
// normal l_max of mother and child).
void ref_simple_acetate_division(float* x, float* child, const double* tape, int32_t n_tape) {
  using M = Models::SimpleAcetate;
  M::SelfParticle arr(x, 1);
  M::SelfParticle buf(child, 1);
  set_tape(tape, n_tape);
  M::division(MC::pool_type(), 0, 0, arr, buf);
}

// SimpleAcetate::init with two uniforms on the tape (length, l_max).
void ref_simple_acetate_init(float* x, const double* tape, int32_t n_tape) {
  using M = Models::SimpleAcetate;
  M::SelfParticle arr(x, 1);
  set_tape(tape, n_tape);
  M::init(MC::pool_type(), 0, arr);
}

float ref_erfinv_f(float x) { return MC::Distributions::erfinv<float>(x); }
double ref_erfinv_d(double x) { return MC::Distributions::erfinv<double>(x); }
float ref_norminv_f(float p, float mean, float sd) { return MC::Distributions::norminv<float>(p, mean, sd); }

// TruncatedNormal<float>::draw_from with the uniform `u` as the pool's drand.
float ref_truncnorm_f(double u, float mu, float sigma, float lower, float upper) {
  set_tape(&u, 1);
  Kokkos::Random_XorShift1024<Exec> gen;
  return MC::Distributions::TruncatedNormal<float>::draw_from(gen, mu, sigma, lower, upper);
}

int32_t ref_check_div_f(float l, float lc) { return static_cast<int32_t>(Models::check_div<float>(l, lc)); }

// FeedDescriptor::update on a feed of the given kind (0 constant, 1
// Linear{f0, df = rate}, 2 Exponential{f0, alpha = rate}) at time t.
double ref_feed_flow(int32_t kind, double f0, double rate, double t, double dt) {
  Simulation::Feed::FeedDescriptor fd;
  fd.flow = f0;
  if (kind == 1)
    fd.extra = Simulation::Feed::Linear{f0, rate};
  else if (kind == 2)
    fd.extra = Simulation::Feed::Exponential{f0, rate};
  else
    fd.extra = Simulation::Feed::Constant{};
  fd.update(t, dt);
  return fd.flow;
}

// Relative time after n calls of SimulatimeTimes::advance(dt).
double ref_relative_time(double dt, uint32_t n) {
  Simulation::SimulatimeTimes times;
  for (uint32_t k = 0; k < n; ++k) times.advance(dt);
  return times.relative();
}
}


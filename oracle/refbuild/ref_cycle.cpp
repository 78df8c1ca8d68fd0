// The reference's whole particle cycle, compiled from its headers as they
// stand (no edits) against the Kokkos stand-in in kokkos_shim/: its cycle
// functors and its particle container run one main-loop cycle at a time on
// a container the caller fills, with the draws the caller hands in per
// container slot.  Test infrastructure only: tests/golden/
// make_ref_cycle_golden.py runs it beside the oracle and records where they
// agree; tests/test_ref_cycle.py checks the oracle against those records.
//
// Compiled reference code (paths relative to the BioCMA-MCST tree):
//   apps/libs/simulation/public/simulation/kernels/kernels.hpp
//     CycleFunctors: update (L53-L80), launch_model (L145-L224: the model
//     kernel, then the contribution kernel), launch_move (L112-L143: the
//     move kernel, then the leave reduction), get_host_reduction (L82-L92)
//   apps/libs/simulation/public/simulation/kernels/model_kernel.hpp
//     CycleFunctor (TagCycle team loop L180-L232: ages(i, 1) += d_t, update,
//     handle_division on Division, the overflow and dead reduction)
//   apps/libs/simulation/public/simulation/kernels/contribution_kernel.hpp
//     ContributionFunctor Tag0D / Tag3D
//   apps/libs/simulation/public/simulation/kernels/move_kernel.hpp
//     MoveFunctor TagMove (team draws, then handle_move for every slot of
//     the team) and TagLeave (ages(i, 0) += d_t, handle_exit)
//   apps/libs/mc/public/mc/particles_container.hpp
//     ParticlesContainer: handle_division (buffer), update_and_remove_inactive
//     and remove_inactive_particles (CompactParticlesFunctor through
//     parallel_scan), merge_buffer (InsertFunctor, _resize),
//     __allocate_buffer__
//   apps/libs/models/public/models/fixed_length.hpp, simple_acetate.hpp
//   apps/libs/common/src/common.cpp (Common::c_league_size, from the source
//     file)
// The parts restated here: the leaving flows of each cycle, which
// SimulationUnit::update_feed hands to the domain before the cycle
// (simulation.model.cpp L101-L108; the caller passes them), and the order in
// which SimulationUnit calls the rest, SimulationUnit::cycleProcess and
// post_cycle (apps/libs/simulation/public/simulation/simulation.hpp
// L184-L239):
//   pre_cycle (functors.update), contribs_scatter.reset(), launch_model,
//   launch_move when need_launch(), then the host reductions,
//   update_and_remove_inactive(out, dead), merge_buffer.
//
// Draws: the stand-in's random pool asks draw_for() below, which reads the
// running kernel's tag, league rank and loop index to find the container
// slot a draw belongs to: the model kernel's division draws (league *
// particles per team + index), the move kernel's team draws (two per slot of
// the team, in order: league * particles per team + index / 2) and the leave
// kernel's exit draw (its index).
// (the reference's headers take assert from other headers' includes)
#include <cassert>

#include <models/fixed_length.hpp>
#include <models/simple_acetate.hpp>
#include <simulation/kernels/kernels.hpp>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

namespace {
using Exec = ComputeSpace;
namespace KI = Simulation::KernelInline;

// xorshift1024* (Vigna, "An experimental exploration of Marsaglia's
// xorshift generators, scrambled", 2016), the generator family of the
// reference's pool (Kokkos::Random_XorShift1024_Pool), seeded through
// splitmix64 as its author recommends; for free-running runs, where the
// draws need no slot.
struct Xorshift1024 {
  uint64_t s[16];
  int p = 0;
  bool have_normal = false;
  double spare = 0.0;
  explicit Xorshift1024(uint64_t seed) {
    uint64_t z = seed;
    for (auto& w : s) {
      z += 0x9e3779b97f4a7c15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
      w = x ^ (x >> 31);
    }
  }
  uint64_t next() {
    const uint64_t s0 = s[p];
    uint64_t s1 = s[p = (p + 1) & 15];
    s1 ^= s1 << 31;
    s[p] = s1 ^ s0 ^ (s1 >> 11) ^ (s0 >> 30);
    return s[p] * 1181783497276652981ull;
  }
  // uniforms in [0, 1): 24 and 53 top bits
  double uniform_f() { return (double)(next() >> 40) * 0x1p-24; }
  double uniform_d() { return (double)(next() >> 11) * 0x1p-53; }
  // standard normal by the Box-Muller transform, pairs
  double normal() {
    if (have_normal) {
      have_normal = false;
      return spare;
    }
    double u1 = uniform_d();
    while (u1 <= 0.0) u1 = uniform_d();
    const double u2 = uniform_d();
    const double r = std::sqrt(-2.0 * std::log(u1)), a = 6.283185307179586 * u2;
    spare = r * std::sin(a);
    have_normal = true;
    return r * std::cos(a);
  }
};

double draw_stream(void* user, int kind) {
  Xorshift1024& g = *static_cast<Xorshift1024*>(user);
  if (kind == 2) return g.normal();
  if (kind == 1) return g.uniform_d();
  if (kind == 3) return (double)(g.next() >> 32);
  return g.uniform_f();
}

// Draws of one cycle, per container slot at the cycle's start.
struct StepDraws {
  uint64_t n = 0;
  std::size_t ppt_model = 0, ppt_move = 0;
  const float* move0 = nullptr;  // leave test
  const float* move1 = nullptr;  // destination
  const float* exit = nullptr;   // outlet exit
  const double* div = nullptr;   // [n][4]: the model's division draws in call order
  const int32_t* div_kind = nullptr;  // [4]: the draw kind each division draw must be
  std::size_t div_slot = SIZE_MAX;
  int div_k = 0;
  long misses = 0;
};

double draw_for(void* user, int kind) {
  StepDraws& d = *static_cast<StepDraws*>(user);
  const refpin::Ctx& c = refpin::ctx();
  if (c.tag == refpin::tag_id<KI::TagCycle>()) {
    const std::size_t slot = c.league * d.ppt_model + c.index;
    if (slot != d.div_slot) {
      d.div_slot = slot;
      d.div_k = 0;
    }
    if (slot >= d.n || d.div_k >= 4 || !d.div || kind != d.div_kind[d.div_k]) {
      ++d.misses;
      return 0.5;
    }
    return d.div[slot * 4 + (std::size_t)d.div_k++];
  }
  if (c.tag == refpin::tag_id<KI::TagMove>()) {
    const std::size_t slot = c.league * d.ppt_move + c.index / 2;
    if (kind != 0) ++d.misses;
    if (slot >= d.n) return 0.5;  // the last team draws for slots past the end
    return (c.index & 1u) ? d.move1[slot] : d.move0[slot];
  }
  if (c.tag == refpin::tag_id<KI::TagLeave>()) {
    if (kind != 0 || c.index >= d.n) {
      ++d.misses;
      return 0.5;
    }
    return d.exit[c.index];
  }
  ++d.misses;
  return 0.5;
}

struct CycleBase {
  virtual ~CycleBase() = default;
  // with `stream` set, every draw comes from it instead of the slot tables
  virtual int step(double dt, const double* conc, StepDraws& d, Xorshift1024* stream, uint64_t* stats,
                   double* exact, double* exact_abs, float* scatter) = 0;
  virtual uint64_t read(uint64_t cap, float* state, uint64_t* pos, uint8_t* status, float* age_h,
                        float* age_d) const = 0;
  virtual uint32_t n_var() const = 0;
  virtual uint32_t n_ctb() const = 0;
  virtual void set_leaving(uint32_t n, const double* flow) = 0;
  virtual uint64_t capacity() const = 0;
  // values the probe holds (Probes::get) and whether it needs exporting
  virtual uint64_t probe(int k, double* out, uint64_t max, int32_t* full) const = 0;
};

template <class M>
struct Cycle final : CycleBase {
  uint32_t n_c, K, n_s;
  std::vector<std::size_t> nbr;
  std::vector<double> vol, diag, cdf, conc;
  std::vector<MC::LeavingFlow> lf;
  KernelDispatchOptions opt;
  MC::ParticlesContainer<M> container;
  MC::kernelContribution contribs;
  MC::ContributionView scatter;
  MC::EventContainer events;
  // the functors get copies of these handles (Views share their storage):
  // leaving times, division times; inactive unless built with use_probe
  Simulation::ProbeAutogeneratedBuffer probe_leave, probe_div;
  KI::CycleFunctors<Exec, M> functors;

  static KernelDispatchOptions options(uint32_t ppt) {
    KernelDispatchOptions o;
    o.m_p_p_team_model = ppt;
    o.m_p_p_team_contribs = ppt;
    o.m_p_p_team_move = ppt;
    o.m_p_p_team_leave = ppt;
    return o;
  }

  static MC::RuntimeParameters runtime(uint64_t min_removal, double ratio) {
    MC::RuntimeParameters r;
    r.minimum_dead_particle_removal = min_removal;
    r.dead_particle_ratio_threshold = ratio;
    r.buffer_ratio = 1.0;        // a buffer as large as the container: no refused division
    r.allocation_factor = 2.5;   // the CPU build's factor
    r.shrink_ratio = 0.0;        // never shrink (contents are kept either way)
    return r;
  }

  MC::DomainState<Exec, true> domain() const {
    MC::DomainState<Exec, true> st;
    st.neighbors = MC::NeighborsView<Exec, true>(nbr.data(), n_c, K);
    st.cumulative_probability = MC::CumulativeProbabilityView<Exec, true>(cdf.data(), n_c, K);
    st.diag_transition = MC::DiagonalView<Exec, true>(diag.data(), n_c);
    st.liquid_volume = MC::VolumeView<Exec, true>(vol.data(), n_c);
    st.leaving_flow = MC::LeavingFlowView<true>(lf.data(), lf.size());
    return st;
  }

  Cycle(uint32_t n_c_, uint32_t K_, uint32_t n_s_, const double* volume, const double* out_flow,
        const uint64_t* neighbors, const double* cdf_, uint32_t n_out, const uint64_t* out_index,
        const double* out_flow_v, const double* out_volume, uint64_t n, const float* state, const uint64_t* pos,
        const float* age_h, const float* age_d, double weight, uint64_t min_removal, double ratio, uint32_t ppt)
      : n_c(n_c_), K(K_), n_s(n_s_), nbr(neighbors, neighbors + (std::size_t)n_c_ * K_),
        vol(volume, volume + n_c_), diag(out_flow, out_flow + n_c_), cdf(cdf_, cdf_ + (std::size_t)n_c_ * K_),
        conc((std::size_t)n_c_ * n_s_, 0.0), lf(leaving(n_out, out_index, out_flow_v, out_volume)),
        opt(options(ppt)), container(runtime(min_removal, ratio), n, 0), contribs("contribs", M::n_c, n_c_),
        scatter(Kokkos::Experimental::create_scatter_view(contribs)),
        functors(opt, container, MC::pool_type(), MC::KernelConcentrationType(conc.data(), n_s_, n_c_), scatter,
                 events, domain(), probe_leave, probe_div) {
    for (uint64_t i = 0; i < n; ++i) {
      for (uint32_t v = 0; v < M::n_var; ++v) container.model(i, v) = state[(std::size_t)v * n + i];
      container.position(i) = pos[i];
      container.status(i) = MC::Status::Idle;
      container.ages(i, 0) = age_h[i];
      container.ages(i, 1) = age_d[i];
    }
    container.weights(0) = static_cast<typename M::FloatType>(weight);
  }

  static std::vector<MC::LeavingFlow> leaving(uint32_t n_out, const uint64_t* index, const double* flow,
                                              const double* volume) {
    std::vector<MC::LeavingFlow> v;
    for (uint32_t o = 0; o < n_out; ++o) v.push_back(MC::LeavingFlow{index[o], flow[o], volume[o]});
    return v;
  }

  int step(double dt, const double* c_in, StepDraws& d, Xorshift1024* stream, uint64_t* stats, double* exact,
           double* exact_abs, float* scat) override {
    std::memcpy(conc.data(), c_in, conc.size() * sizeof(double));
    const std::size_t n_particle = container.n_particles();
    if (n_particle == 0) return 1;
    d.n = n_particle;
    d.ppt_model = opt.m_p_p_team_model;
    d.ppt_move = opt.m_p_p_team_move;
    if (stream)
      refpin::provider() = {&draw_stream, stream};
    else
      refpin::provider() = {&draw_for, &d};
    const uint64_t e_new0 = events.get<MC::EventType::NewParticle>(), e_exit0 = events.get<MC::EventType::Exit>(),
                   e_move0 = events.get<MC::EventType::Move>(), e_over0 = events.get<MC::EventType::Overflow>();
    // SimulationUnit::cycleProcess (simulation.hpp L184-L212)
    functors.update(dt, container, domain());  // pre_cycle
    scatter.reset();
    functors.launch_model(n_particle);
    // the contribution operands the scatter saw: each Idle particle's
    // weight * contribution at its compartment before the move, summed
    // exactly (products of two floats are exact in double; the sum in long
    // double is the reference of the comparison, not the reference's code)
    const double w = static_cast<double>(container.get_weight(0));
    std::vector<long double> ex((std::size_t)M::n_c * n_c, 0.0L), ab((std::size_t)M::n_c * n_c, 0.0L);
    for (std::size_t i = 0; i < n_particle; ++i) {
      if (container.status(i) != MC::Status::Idle) continue;
      const std::size_t p = container.position(i);
      for (std::size_t j = 0; j < M::n_c; ++j) {
        const double t = w * static_cast<double>(container.contribs(i, j));
        ex[j * n_c + p] += t;
        ab[j * n_c + p] += std::fabs(t);
      }
    }
    for (std::size_t k = 0; k < ex.size(); ++k) {
      exact[k] = static_cast<double>(ex[k]);
      exact_abs[k] = static_cast<double>(ab[k]);
    }
    for (std::size_t j = 0; j < M::n_c; ++j)
      for (std::size_t p = 0; p < n_c; ++p) scat[j * n_c + p] = contribs(j, p);
    if (functors.move_kernel.need_launch()) functors.launch_move(n_particle);
    // post_cycle (simulation.hpp L215-L239)
    const auto [host_red, host_out_counter] = functors.get_host_reduction();
    const std::size_t out = host_out_counter;
    container.update_and_remove_inactive(out, host_red.dead_total);
    container.merge_buffer();
    refpin::provider() = {};
    stats[0] = container.n_particles();
    stats[1] = events.get<MC::EventType::NewParticle>() - e_new0;
    stats[2] = events.get<MC::EventType::Exit>() - e_exit0;
    stats[3] = events.get<MC::EventType::Move>() - e_move0;
    stats[4] = events.get<MC::EventType::Overflow>() - e_over0;
    stats[5] = host_red.waiting_allocation_particle;
    stats[6] = out;
    stats[7] = container.get_inactive();
    return 0;
  }

  uint64_t read(uint64_t cap, float* state, uint64_t* pos, uint8_t* status, float* age_h,
                float* age_d) const override {
    const uint64_t n = container.n_particles();
    if (cap < n) return n;
    for (uint64_t i = 0; i < n; ++i) {
      for (uint32_t v = 0; v < M::n_var; ++v) state[(std::size_t)v * cap + i] = container.model(i, v);
      pos[i] = container.position(i);
      status[i] = static_cast<uint8_t>(container.status(i));
      age_h[i] = container.ages(i, 0);
      age_d[i] = container.ages(i, 1);
    }
    return n;
  }
  uint32_t n_var() const override { return M::n_var; }
  uint32_t n_ctb() const override { return M::n_c; }
  // the outlets' flows of the coming cycle (SimulationUnit::update_feed sets
  // them through ReactorDomain::set_leaving_flow before each cycle)
  void set_leaving(uint32_t n, const double* flow) override {
    for (uint32_t o = 0; o < n && o < lf.size(); ++o) lf[o].flow = flow[o];
  }
  uint64_t capacity() const override { return container.capacity(); }
  uint64_t probe(int k, double* out, uint64_t max, int32_t* full) const override {
    const auto& p = k == 0 ? probe_leave : probe_div;
    const auto v = p.get();
    const uint64_t n = std::min<uint64_t>(v.size(), max);
    for (uint64_t i = 0; i < n; ++i) out[i] = v[i];
    if (full) *full = p.need_export() ? 1 : 0;
    return v.size();
  }
};

struct Handle {
  std::unique_ptr<CycleBase> c;
  std::unique_ptr<Xorshift1024> stream;
  long misses = 0;
};
}  // namespace

extern "C" {

// A cycle of the reference's model `model` (3: FixedLength, 5: SimpleAcetate)
// over a domain of n_c compartments (neighbours and cumulative
// probabilities [n_c][K], volumes, out-flows) with n_out outlets, holding n
// particles (state [n_var][n] plane by plane, compartments, ages).
void* ref_cycle_new(int32_t model, uint32_t n_c, uint32_t K, uint32_t n_s, const double* volume,
                    const double* out_flow, const uint64_t* neighbors, const double* cdf, uint32_t n_out,
                    const uint64_t* out_index, const double* out_flow_v, const double* out_volume, uint64_t n,
                    const float* state, const uint64_t* pos, const float* age_h, const float* age_d, double weight,
                    uint64_t min_removal, double ratio, uint32_t particles_per_team) {
  auto* h = new Handle;
  if (model == 3)
    h->c = std::make_unique<Cycle<Models::FixedLength>>(n_c, K, n_s, volume, out_flow, neighbors, cdf, n_out,
                                                        out_index, out_flow_v, out_volume, n, state, pos, age_h,
                                                        age_d, weight, min_removal, ratio, particles_per_team);
  else if (model == 5)
    h->c = std::make_unique<Cycle<Models::SimpleAcetate>>(n_c, K, n_s, volume, out_flow, neighbors, cdf, n_out,
                                                          out_index, out_flow_v, out_volume, n, state, pos, age_h,
                                                          age_d, weight, min_removal, ratio, particles_per_team);
  else {
    delete h;
    return nullptr;
  }
  return h;
}

void ref_cycle_free(void* h) { delete static_cast<Handle*>(h); }

uint32_t ref_cycle_n_var(void* h) { return static_cast<Handle*>(h)->c->n_var(); }
uint32_t ref_cycle_n_ctb(void* h) { return static_cast<Handle*>(h)->c->n_ctb(); }
uint64_t ref_cycle_capacity(void* h) { return static_cast<Handle*>(h)->c->capacity(); }
// Probe k (0 leaving times, 1 division times): copies up to max of the
// values it holds into out, sets *full when it needs exporting, returns how
// many it holds (0 in the build without use_probe).
uint64_t ref_cycle_probe(void* h, int32_t k, double* out, uint64_t max, int32_t* full) {
  return static_cast<Handle*>(h)->c->probe(k, out, max, full);
}
long ref_cycle_misses(void* h) { return static_cast<Handle*>(h)->misses; }

// One cycle with the concentrations conc [n_c][n_s] and the draws of every
// slot of the container as it stands: move0/move1/exit [n] (the move test,
// destination and exit uniforms), div [n][4] (the model's division draws,
// in call order, of kinds div_kind[4]: 0 float uniform, 1 double uniform,
// 2 standard normal).  Out: stats[8] = {particles after, NewParticle
// events, Exit events, Move events, Overflow events, refused divisions,
// leave-reduction count, inactive after}; per contribution j and
// compartment p ([n_ctb][n_c]): the exact sum of the scatter's operands, the
// sum of their magnitudes, and the reference's float scatter itself.
int32_t ref_cycle_step(void* hv, double dt, const double* conc, const float* move0, const float* move1,
                       const float* exit_u, const double* div, const int32_t* div_kind, uint64_t* stats,
                       double* exact, double* exact_abs, float* scatter) {
  auto* h = static_cast<Handle*>(hv);
  StepDraws d;
  d.move0 = move0;
  d.move1 = move1;
  d.exit = exit_u;
  d.div = div;
  d.div_kind = div_kind;
  const int rc = h->c->step(dt, conc, d, nullptr, stats, exact, exact_abs, scatter);
  h->misses += d.misses;
  return rc;
}

// Free-running: the draws come, in the order the cycle asks for them, from
// one xorshift1024* stream seeded once with `seed` (the first call seeds
// it).  Outputs as ref_cycle_step.
int32_t ref_cycle_step_stream(void* hv, double dt, const double* conc, uint64_t seed, uint64_t* stats,
                              double* exact, double* exact_abs, float* scatter) {
  auto* h = static_cast<Handle*>(hv);
  if (!h->stream) h->stream = std::make_unique<Xorshift1024>(seed);
  StepDraws d;
  return h->c->step(dt, conc, d, h->stream.get(), stats, exact, exact_abs, scatter);
}

// Flows of the outlets (in the order ref_cycle_new took them) for the next
// cycle.
void ref_cycle_set_leaving(void* h, uint32_t n, const double* flow) {
  static_cast<Handle*>(h)->c->set_leaving(n, flow);
}

// The container: particles [0, n) into arrays of capacity cap (state
// [n_var][cap]); returns n (nothing written when cap < n).
uint64_t ref_cycle_read(void* h, uint64_t cap, float* state, uint64_t* pos, uint8_t* status, float* age_h,
                        float* age_d) {
  return static_cast<Handle*>(h)->c->read(cap, state, pos, status, age_h, age_d);
}
}

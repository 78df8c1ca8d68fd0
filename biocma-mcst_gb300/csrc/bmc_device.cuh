// bmc_device.cuh -- device-side data layout, draw source and model plugins.
//
// Layout in HBM, per scenario (one arena per kind, arrays 256-byte aligned):
//   state    F[n_var][cap]    SoA particle state (ModelType::SelfParticle)
//   pos      u32[cap]         compartment (reference ParticlePositions, u64)
//   status   u8[cap]          MC::Status
//   age_h    f32[cap]         reference ages(i,0), hydraulic time
//   age_d    f32[cap]         reference ages(i,1), time since division
//   id       u32[cap]         particle identity, keys the draws
//   child    F[n_var][cap] + u32[cap]   division buffer (children in rank order)
//   tile_*   u32[cap/1024]    per-tile counters (births, inactive, offsets)
//   bmask    u32[cap/32]      birth-request bits, slot order
//   bpos     u32[cap]         compartment of a mother when it asked to divide
//   gap/src  u32[cap]         compaction lists
// Domain and liquid state, per compartment:
//   crec     F[n_c][8]        compartment record: model rates (slots 0..6,
//                             from C) and the move threshold (slot 7 bits):
//                             leave iff draw < ceil(2^24 dt Q/V)
//   mrow     i32x2[n_c][K]    {floor(2^24 CDF(k)), neighbour(k)}: next =
//                             neighbour of the first k with draw <= thr
//   C        f64[2][n_c][n_s] double-buffered concentrations (step parity)
//   M, src   f64[n_c][n_s];   acc_hi/acc_lo i64/u64[n_c][n_acc] fixed point
#pragma once
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace bmc {

constexpr int kMaxOutlets = 8;
constexpr int kMaxSpecies = 8;
constexpr int kMaxVar = 16;
constexpr int kMaxRates = 8;
// Fixed point of the contribution sums: a value at its bound is 2^kQBits
// quanta (resolution 2^-42 of the bound).  A coarser 2^26, which keeps most
// adds to one 32-bit shared atomic (no carry into the high word), was slower
// on the batched workload (cycle 2.12 -> 2.25 ms): a warp still issues the
// second atomic whenever one of its lanes carries.
constexpr int kQBits = 42;
constexpr long long kQMax = 1LL << kQBits;  // |quantised value| bound
// A block flushes its shared-memory accumulator before it has summed more
// than 2^20 particles, so |partial| <= 2^62 and no int64 sum can overflow.
constexpr unsigned kFlushParticles = 1u << 20;
// ScalarSimulation::clearNegs threshold: scheme relative error 1e-4 times
// the species scale 5e-3 (implScalar.cpp L273-L277)
constexpr double kClearNegTol = 1e-4 * 5e-3;

enum : uint8_t { kIdle = 0, kDivision = 1, kExit = 2, kDead = 3 };

// ---------------------------------------------------------------------------
// Age step of the reference: ages are float, the time step a double, and
// `ages(i, 0) += d_t` (MoveFunctor, move_kernel.hpp L356; and
// `ages(i, 1) += d_t` of CycleFunctor for models whose FloatType is double,
// model_kernel.hpp L193, L270) rounds the sum to double, then to float:
// (float)((double)a + d).  Evaluated here on the integer pipe (the FP64
// pipe is scarce on this part): the exact sum rounded to 53 bits (nearest,
// ties to even) from a guard, round and sticky bit, then to 24 bits.
// Domain: a >= 0 finite, d >= 0 finite, d the same for a whole step.
struct AgeStep {
  unsigned long long md;  // d = md * 2^ed, md normalised to bit 52
  int ed;
  float d_rounded;  // (float)d: the result for a == 0
  int zero;         // d == 0: the age does not change
  float dl_abs;     // bound on |d - (float)d| (age_add_fast)
};

__host__ __device__ inline AgeStep age_step(double d) {
  unsigned long long b;
  memcpy(&b, &d, 8);
  AgeStep k;
  k.zero = d == 0.0;
  const int ef = (int)((b >> 52) & 0x7ffu);
  unsigned long long m = (b & ((1ull << 52) - 1ull)) | (ef ? (1ull << 52) : 0ull);
  int e = (ef ? ef : 1) - 1075;
  while (m && !(m >> 52)) {  // subnormal d: normalise
    m <<= 1;
    e -= 1;
  }
  k.md = m;
  k.ed = e;
  k.d_rounded = (float)d;
  // |d - (float)d| rounded to float, raised past its rounding error
  const double dl = d - (double)k.d_rounded;
  k.dl_abs = (float)(dl < 0.0 ? -dl : dl) * (1.0f + 0x1p-22f);
  return k;
}

__host__ __device__ inline float age_add(float a, const AgeStep& k) {
  if (k.zero) return a;
  unsigned ab;
  memcpy(&ab, &a, 4);
  if ((ab << 1) == 0u) return k.d_rounded;
  const int ef = (int)((ab >> 23) & 0xffu);
  unsigned long long ma = (unsigned long long)((ab & 0x7fffffu) | (ef ? 0x800000u : 0u)) << 29;
  int ea = (ef ? ef : 1) - 150 - 29;  // a = ma * 2^ea
  while (!(ma >> 52)) {  // subnormal a: normalise
    ma <<= 1;
    ea -= 1;
  }
  unsigned long long mx = ma, my = k.md;
  int ex = ea, ey = k.ed;
  if (ey > ex) {
    mx = k.md;
    my = ma;
    ex = k.ed;
    ey = ea;
  }
  const int sh = ex - ey;
  const unsigned long long x3 = mx << 3, y3 = my << 3;
  unsigned long long yal;
  if (sh == 0)
    yal = y3;
  else if (sh < 56)
    yal = (y3 >> sh) | (unsigned long long)((y3 << (64 - sh)) != 0ull);
  else
    yal = 1ull;
  unsigned long long s = x3 + yal;
  int e = ex;
  if (s >> 56) {
    s = (s >> 1) | (s & 1ull);
    e += 1;
  }
  unsigned long long m = s >> 3;  // round to 53 bits
  const unsigned g = (unsigned)(s & 7ull);
  if (g > 4u || (g == 4u && (m & 1ull))) {
    m += 1ull;
    if (m >> 53) {
      m >>= 1;
      e += 1;
    }
  }
  unsigned long long q = m >> 29;  // round to 24 bits
  const unsigned long long r = m & ((1ull << 29) - 1ull);
  if (r > (1ull << 28) || (r == (1ull << 28) && (q & 1ull))) {
    q += 1ull;
    if (q >> 24) {
      q >>= 1;
      e += 1;
    }
  }
  const unsigned out = ((unsigned)(e + 179) << 23) | (unsigned)(q & 0x7fffffull);
  float f;
  memcpy(&f, &out, 4);
  return f;
}

// The same sum with float operations where that is exact: s = fl(a + dh)
// with dh = (float)d, and e = the rounding error of that addition (Fast2Sum
// of the larger and the smaller operand).  The exact sum is s + e + dl with
// dl = d - dh; when |e| + |dl| stays below half an ulp of s by a margin
// (2^-20 of it, far more than the 2^-29 the rounding to 53 bits can move
// the sum), both roundings return s (when s is a power of two the float
// below it is half an ulp of s away, and the half of that counts).
// Otherwise (near a rounding tie, or s below 2^-81) age_add decides.  On ages advanced step by step this
// leaves age_add to a handful of steps in a run.
__host__ __device__ inline float age_add_fast(float a, const AgeStep& k) {
  if (k.zero) return a;
  const float dh = k.d_rounded;
  const float s = a + dh;
  const float big = a > dh ? a : dh, small = a > dh ? dh : a;
  const float e = small - (s - big);
  unsigned sb;
  memcpy(&sb, &s, 4);
  const unsigned se = sb & 0x7f800000u;  // exponent field of s (s >= 0)
  if (se >= (46u << 23) && se < (255u << 23)) {
    // half an ulp of s; below a power of two the neighbour is half as far
    const unsigned hb = se - ((sb & 0x7fffffu) == 0u ? (25u << 23) : (24u << 23));
    const unsigned mb = hb - (20u << 23);
    float h, m;
    memcpy(&h, &hb, 4);
    memcpy(&m, &mb, 4);  // 2^-20 of it
    const float thr = (h - m) - k.dl_abs;
    if ((e < 0.0f ? -e : e) < thr) return s;
  }
  return age_add(a, k);
}

// Per-scenario control block, written by the kernels (device memory).
struct Control {
  unsigned long long n_used;
  unsigned long long inactive;
  unsigned long long next_id;
  unsigned int step;
  unsigned int error;
  // counters of the current step (reset by the liquid step)
  unsigned long long req_div;
  unsigned long long exits;
  unsigned long long moves;
  unsigned long long clamped;
  // plan of the current step (written by the plan kernel)
  unsigned long long plan_n_old;
  unsigned long long plan_to_remove;
  unsigned long long plan_n_after;
  unsigned long long plan_births;
  unsigned long long plan_overflow;
  unsigned long long plan_next_id;
  unsigned long long plan_gaps;
  unsigned int plan_step;
  unsigned int plan_compact;
  // results of the last completed step
  unsigned long long last_births;
  unsigned long long last_exits;
  unsigned long long last_moves;
  unsigned long long last_overflow;
  unsigned long long last_req_div;
  unsigned int last_compacted;
  unsigned int map_cur;  // flow map the domain arrays hold (0xffffffff: none yet)
  double mass_balance[kMaxSpecies];
  // per-species sums of the liquid step (new mass, expected mass)
  double mb_new[kMaxSpecies];
  double mb_exp[kMaxSpecies];
  // 1 while the current step runs for this scenario (set by the liquid step
  // from the step limit, before the plan kernel advances the step counter)
  unsigned int cycling;
  // 1 when this launch sequence is a whole main-loop iteration (the liquid
  // step ran), so the plan kernel advances the relative time with the step
  unsigned int t_advance;
  // relative time of the main loop (Simulation::SimulationTimes::
  // relative_time, simulation_times.hpp L12-L29): the sum of the time steps
  // of the iterations so far, in order; feed schedules are evaluated at it
  double t_rel;
  // time-event probes (ScenDev::probe_buf): events counted so far, per probe
  // (kProbeLeaving, kProbeDivision), including those a full buffer dropped
  unsigned long long probe_n[2];
  // division events counted before this step (written by the plan kernel;
  // the division records of the step follow it in slot order)
  unsigned long long plan_probe_base;
  // event tallies since the host last cleared them (MC::EventContainer,
  // events.hpp L17-L26): NewParticle (every division request, refused or
  // not), Exit, Move, Death, Overflow, ChangeWeight; added by the plan kernel
  unsigned long long events[6];
};

// Probes of the reference's Simulation::Probes (probe.hpp L14-L18).
constexpr int kProbeLeaving = 0;   // ProbeType::LeavingTime: ages(i, 0) at exit
constexpr int kProbeDivision = 1;  // ProbeType::DivisionTime: ages(i, 1) at a division request

// Scenario descriptor as the kernels see it (one per scenario, device memory).
struct ScenDev {
  // particle container
  void* state;
  uint32_t* pos;
  uint8_t* status;
  float* age_h;
  float* age_d;
  uint32_t* id;
  void* child_state;
  uint32_t* child_pos;
  uint32_t* tile_births;
  uint32_t* tile_inactive;
  uint32_t* tile_boff;
  uint32_t* tile_goff;
  uint32_t* tile_soff;
  uint32_t* bmask;
  uint32_t* bpos;
  uint32_t* gap_slot;
  uint32_t* src_slot;
  unsigned long long cap;
  uint32_t n_tiles;
  uint32_t tile_base;  // first global tile of this scenario in its batch
  // domain
  const int2* mrow;
  // [n_c][16] rows of up to 8 entries: thresholds of mrow in slots 0..7
  // (padded with INT32_MAX), neighbours in slots 8..15 (padded with the last
  // one); two independent 32-byte loads give a row's answer
  const int32_t* mrow16;
  const double* volume;
  const double* out_flow;
  const uint32_t* in_ptr;
  const uint32_t* in_idx;
  const double* in_flow;
  const double* diag;
  const double* vinv;
  void* crec;
  uint32_t n_c;
  uint32_t K;
  uint32_t n_s;
  uint32_t n_ctb;
  uint32_t n_var;
  uint32_t n_acc;  // accumulator entries per compartment (1 when separable)
  uint32_t n_outlets;
  uint32_t outlet_idx[kMaxOutlets];
  uint32_t exit_thr[kMaxOutlets];  // leave the reactor iff draw > exit_thr
  double outlet_flow[kMaxOutlets];
  // feeds
  uint32_t n_feeds;
  uint32_t feed_in[kMaxOutlets];
  int32_t feed_out[kMaxOutlets];
  double feed_flow[kMaxOutlets];
  double feed_conc[kMaxOutlets * kMaxSpecies];
  // feed schedules (Simulation::Feed::FeedDescriptor::update): kind 0
  // constant (feed_flow), 1 linear f0 + t * rate, 2 exponential
  // f0 + exp(rate * t), at the relative time t; n_sched counts the feeds
  // that are not constant
  uint32_t n_sched;
  int32_t feed_kind[kMaxOutlets];
  double feed_f0[kMaxOutlets];
  double feed_rate[kMaxOutlets];
  uint32_t outlet_feed[kMaxOutlets];  // feed of each outlet
  // -logf of every draw value, (2k + 1) 2^-24 for k < 2^23 (the exit test's
  // float logarithm, from the host's C library); set with schedules
  const float* nlog;
  // liquid
  double* C;  // two buffers of n_c * n_s; the current one is C + (step & 1) * n_c * n_s
  double* M;
  double* src;
  long long* acc_hi;
  unsigned long long* acc_lo;
  int32_t q_exp[kMaxSpecies];      // e per accumulator column: quantum 2^e
  double q_scale_up[kMaxSpecies];  // 2^e: quanta -> value
  // model
  double params[16];
  double weight;
  double dt;
  unsigned long long seed;
  double dead_ratio;
  unsigned long long min_removal;
  Control* ctl;
  int32_t f64;
  uint32_t step_limit;  // 0: none; otherwise steps stop (no-op) once ctl->step reaches it
  // Flow-map cycle: n_maps domain states stored back to back; step k runs on
  // map (k / n_per_map) % n_maps, copied into the domain arrays above when
  // it changes (k_flowmap).  n_maps == 0: the domain is fixed.
  uint32_t n_maps;
  uint32_t n_per_map;
  uint32_t map_nnz_max;  // stride of the incoming-flow lists
  const int2* map_mrow;          // [n_maps][n_c * K]
  const double* map_volume;      // [n_maps][n_c]
  const double* map_vinv;        // [n_maps][n_c]
  const double* map_out_flow;    // [n_maps][n_c]
  const double* map_diag;        // [n_maps][n_c]
  const uint32_t* map_in_ptr;    // [n_maps][n_c + 1]
  const uint32_t* map_in_idx;    // [n_maps][map_nnz_max]
  const double* map_in_flow;     // [n_maps][map_nnz_max]
  const uint32_t* map_exit_thr;  // [n_maps][kMaxOutlets], for the current dt
  // gas state of every flow map, switched with it (map_g_nnz_max == 0: the
  // gas domain stays fixed while the maps cycle)
  const double* map_gvinv;       // [n_maps][n_c]
  const double* map_g_diag;      // [n_maps][n_c]
  const uint32_t* map_g_in_ptr;  // [n_maps][n_c + 1]
  const uint32_t* map_g_in_idx;  // [n_maps][map_g_nnz_max]
  const double* map_g_in_flow;   // [n_maps][map_g_nnz_max]
  const double* map_kla;         // [n_maps][n_c * n_s]
  uint32_t map_g_nnz_max;
  // Gas phase of a two-phase flow (gas == 0: liquid only): its own volumes,
  // transition (incoming lists + diagonal) and feeds, concentrations double
  // buffered like C, and the gas-liquid transfer
  //   mtr(j,s) = kla(j,s) (H(s) Cg(j,s) - C(j,s)) V(j)
  // gained by the liquid and lost by the gas in the same step.
  uint32_t gas;
  const double* gvinv;
  const uint32_t* g_in_ptr;
  const uint32_t* g_in_idx;
  const double* g_in_flow;
  const double* g_diag;
  double* Cg;              // two buffers of n_c * n_s, current one by step parity
  double* Mg;
  const double* kla;       // [n_c][n_s], 1/s
  double* mtr;             // [n_c][n_s], kg/s, of the last step
  double henry[kMaxSpecies];
  uint32_t n_gfeeds;
  uint32_t gfeed_in[kMaxOutlets];
  int32_t gfeed_out[kMaxOutlets];
  double gfeed_flow[kMaxOutlets];
  double gfeed_conc[kMaxOutlets * kMaxSpecies];
  // Time-event probes (the reference's Simulation::Probes with use_probe,
  // probe.hpp L38-L146): probe_cap values per probe (0: probes off)
  double* probe_buf[2];
  unsigned long long probe_cap;
};

// Probes::set (probe.hpp L61-L79): the event is counted; its value is kept
// while the buffer has room.
__device__ __forceinline__ void probe_set(const ScenDev& S, int k, double v) {
  const unsigned long long j = atomicAdd(&S.ctl->probe_n[k], 1ull);
  if (j < S.probe_cap) S.probe_buf[k][j] = v;
}

// A scenario whose step counter has reached its limit is left untouched.
__device__ __forceinline__ bool scen_finished(const ScenDev& S, const Control* ctl) {
  return S.step_limit != 0u && ctl->step >= S.step_limit;
}

// ---------------------------------------------------------------------------
// Draw source: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) with
// counter (particle id, seed low word, step, seed high word) and key
// (purpose, 0): one stream per (seed, particle, step, purpose).  The purpose
// is a constant at every call site, so the key schedule of the ten rounds
// folds into immediates instead of two additions a round per particle.
struct Draws {
  float u[4];
};

__device__ __forceinline__ Draws philox_draws(unsigned long long seed, uint32_t id, uint32_t step,
                                              uint32_t purpose) {
  uint32_t c0 = id, c1 = (uint32_t)seed, c2 = step, c3 = (uint32_t)(seed >> 32);
  uint32_t k0 = purpose, k1 = 0u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c0;
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  Draws d;
  // odd 24-bit integer * 2^-24: exact, in (0, 1)
  d.u[0] = (float)((c0 >> 8) | 1u) * 0x1p-24f;
  d.u[1] = (float)((c1 >> 8) | 1u) * 0x1p-24f;
  d.u[2] = (float)((c2 >> 8) | 1u) * 0x1p-24f;
  d.u[3] = (float)((c3 >> 8) | 1u) * 0x1p-24f;
  return d;
}

__device__ __forceinline__ void philox_raw(unsigned long long seed, uint32_t id, uint32_t step,
                                           uint32_t purpose, uint32_t out[4]) {
  uint32_t c0 = id, c1 = (uint32_t)seed, c2 = step, c3 = (uint32_t)(seed >> 32);
  uint32_t k0 = purpose, k1 = 0u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c0;
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// Integer form of a draw: the odd 24-bit integer x with u = x * 2^-24.
__device__ __forceinline__ uint32_t draw_int(uint32_t r) { return (r >> 8) | 1u; }


// ---------------------------------------------------------------------------
// Model plugins.  The ModelType concept of the reference
// (apps/libs/mc/public/mc/traits.hpp L67-L133) split for a GPU:
//   n_var, n_ctb, n_rates                   sizes
//   n_upd                                   leading rates update() reads
//   read_mask                               state variables update() reads
//   separable                               contributions are coef(c)*basis(x)
//   rates(c, p, r)                          per compartment, from C(:, j):
//                                           every factor of Model::update that
//                                           depends on the concentrations only
//   update(dt, x, r, basis|ctb, pf) -> st   Model::update of one particle
//                                           (pf: the parameters converted to F)
//   coef(r, j)                              contribution j per unit basis
//   division(x, child, d, p)                Model::division
//   init(x, d, p)                           Model::init
//   mass(x, p) -> double                    Model::mass
// A separable model's contribution to species j is coef_j(C) * basis(x);
// the cycle then sums one basis value per compartment and the coefficients
// are applied once per compartment.  A general model (separable = false)
// writes its n_ctb contributions per particle.  Every expression keeps the
// operation order of the CPU restatement, so both round identically.
//
// A model whose update is not a function of per-compartment factors alone,
// or that draws random numbers in update (the reference's
// Model::update(random_pool, d_t, idx, arr, contribs, position, c),
// traits.hpp L117, called at model_kernel.hpp L234-L240), declares
//   static constexpr bool uses_context = true;
//   update_ctx(dt, x, r, out, pf, ctx) -> st
// and the cycle calls update_ctx instead of update / update_general, with
// out the basis (separable) or the n_ctb contributions (general) and ctx the
// particle's four uniform draws of the step (Philox keyed by (seed, id,
// step, purpose 3)), the compartment's concentrations and its index.
struct UpdateContext {
  const float* draws;   // 4 uniforms in (0, 1)
  const double* c;      // concentrations of the particle's compartment [n_species]
  uint32_t position;    // compartment index
  uint32_t n_species;
};
template <class M, class = void>
struct has_context : std::false_type {};
template <class M>
struct has_context<M, std::void_t<decltype(M::uses_context)>> : std::integral_constant<bool, M::uses_context> {};

template <class F>
struct MonodModel {
  static constexpr int n_var = 2;
  static constexpr int n_ctb = 1;
  static constexpr int n_rates = 2;
  static constexpr int n_upd = 1;  // leading rates update() reads
  static constexpr int model_id = 1;
  static constexpr bool separable = true;
  static constexpr unsigned read_mask = 0x3u;
  // r = {mu, -(mu / Y)}
  __device__ __forceinline__ static void rates(const double* c, const double* p, F* r) {
    const F mu_max = (F)p[0], ks = (F)p[1], y = (F)p[2];
    F s = (F)c[0];
    if (s < (F)0) s = (F)0;
    const F g = s / (ks + s);
    const F mu = mu_max * g;
    r[0] = mu;
    r[1] = -(mu / y);
  }
  __device__ __forceinline__ static int update(F dt, F* x, const F* r, F& basis, const F* pf) {
    const F mdiv = pf[3];
    const F m = x[0];
    basis = m;
    const F growth = r[0] * m;
    x[0] = m + dt * growth;
    x[1] = x[1] + dt;
    return x[0] >= mdiv ? kDivision : kIdle;
  }
  __device__ __forceinline__ static F coef(const F* r, int j) {
    (void)j;
    return r[1];
  }
  __device__ __forceinline__ static void division(F* x, F* child, const float* d, const double* p) {
    (void)d;
    (void)p;
    const F half = x[0] * (F)0.5;
    x[0] = half;
    x[1] = (F)0;
    child[0] = half;
    child[1] = (F)0;
  }
  __device__ __forceinline__ static void init(F* x, const float* d, const double* p) {
    x[0] = (F)p[4] + (F)p[5] * (F)d[1];
    x[1] = (F)0;
  }
  __device__ __forceinline__ static double mass(const F* x, const double* p) {
    (void)p;
    return (double)x[0];
  }
};

template <class F>
struct OverflowModel {
  static constexpr int n_var = 6;
  static constexpr int n_ctb = 4;
  static constexpr int n_rates = 5;
  static constexpr int n_upd = 4;
  static constexpr int model_id = 2;
  static constexpr bool separable = true;
  static constexpr unsigned read_mask = 0x3u;  // mass and age; the rest is output
  // r = {mu, q_s, q_o2, q_ac, q_co2}
  __device__ __forceinline__ static void rates(const double* c, const double* p, F* r) {
    const F qs_max = (F)p[0], ks = (F)p[1], qo_max = (F)p[2], ko = (F)p[3];
    const F y_ox = (F)p[4], y_of = (F)p[5], y_ac = (F)p[6], y_o = (F)p[7];
    const F y_c = (F)p[8], y_cof = (F)p[10];
    F s = (F)c[0];
    if (s < (F)0) s = (F)0;
    F o = (F)c[1];
    if (o < (F)0) o = (F)0;
    const F q_s = qs_max * (s / (ks + s));
    const F q_cap = qo_max * (o / (ko + o));
    const F q_ox = q_s < q_cap ? q_s : q_cap;
    const F q_of = q_s - q_ox;
    r[0] = y_ox * q_ox + y_of * q_of;
    r[1] = q_s;
    r[2] = y_o * q_ox;
    r[3] = y_ac * q_of;
    r[4] = y_c * q_ox + y_cof * q_of;
  }
  __device__ __forceinline__ static int update(F dt, F* x, const F* r, F& basis, const F* pf) {
    const F mdiv = pf[9];
    const F m = x[0];
    basis = m;
    x[0] = m + dt * (r[0] * m);
    x[1] = x[1] + dt;
    x[2] = r[0];
    x[3] = r[1];
    x[4] = r[2];
    x[5] = r[3];
    return x[0] >= mdiv ? kDivision : kIdle;
  }
  // glucose and O2 consumed, acetate and CO2 produced
  __device__ __forceinline__ static F coef(const F* r, int j) {
    return j == 0 ? -r[1] : (j == 1 ? -r[2] : (j == 2 ? r[3] : r[4]));
  }
  __device__ __forceinline__ static void division(F* x, F* child, const float* d, const double* p) {
    (void)d;
    (void)p;
    const F half = x[0] * (F)0.5;
    x[0] = half;
    x[1] = (F)0;
    child[0] = half;
    child[1] = (F)0;
#pragma unroll
    for (int v = 2; v < 6; ++v) child[v] = x[v];
  }
  __device__ __forceinline__ static void init(F* x, const float* d, const double* p) {
    x[0] = (F)p[11] + (F)p[12] * (F)d[1];
#pragma unroll
    for (int v = 1; v < 6; ++v) x[v] = (F)0;
  }
  __device__ __forceinline__ static double mass(const F* x, const double* p) {
    (void)p;
    return (double)x[0];
  }
};

// The reference's FixedLength model (apps/libs/models/public/models/
// fixed_length.hpp L19-L161), float state {length, l_max}, one
// contribution -phi_s(C) per particle (basis 1).  Separable = false
// instantiates the same model through the general per-particle path.
template <bool Separable>
struct FixedLengthModelT {
  static constexpr int n_var = 2;
  static constexpr int n_ctb = 1;
  static constexpr int n_rates = 2;
  static constexpr int n_upd = 2;
  static constexpr int model_id = Separable ? 3 : 4;
  static constexpr bool separable = Separable;
  static constexpr unsigned read_mask = 0x3u;
  __device__ __forceinline__ static float lin_density() {
    const float d_m = (float)0.6e-6;
    return (float)1000 * (float)3.14159265358979323846 * d_m * d_m / (float)4.;
  }
  __device__ __forceinline__ static float l_dot_max() { return (float)(2e-6 / 3600.); }
  __device__ __forceinline__ static float phi_s_max() { return (l_dot_max() * lin_density()) / (float)0.5; }
  // r = {ldot, -phi_s}
  __device__ __forceinline__ static void rates(const double* c, const double* p, float* r) {
    (void)p;
    const float k = (float)1e-3;
    const float s = (float)c[0];
    const float g = s / (k + s);
    const float phi_s = phi_s_max() * g;
    r[0] = l_dot_max() * g;
    r[1] = -phi_s;
  }
  __device__ __forceinline__ static int update(float dt, float* x, const float* r, float& basis,
                                               const float* pf) {
    (void)pf;
    basis = 1.0f;
    x[0] += dt * r[0];
    return x[0] >= x[1] ? kDivision : kIdle;
  }
  __device__ __forceinline__ static int update_general(float dt, float* x, const float* r, float* ctb,
                                                       const float* pf) {
    (void)pf;
    x[0] += dt * r[0];
    ctb[0] = r[1];
    return x[0] >= x[1] ? kDivision : kIdle;
  }
  __device__ __forceinline__ static float coef(const float* r, int j) {
    (void)j;
    return r[1];
  }
  __device__ __forceinline__ static void division(float* x, float* child, const float* d, const double* p) {
    (void)d;
    (void)p;
    const float l_max_m = (float)2e-6;
    const float nl = x[0] / 2.F;
    x[0] = nl;
    x[1] = l_max_m;
    child[0] = nl;
    child[1] = l_max_m;
  }
  __device__ __forceinline__ static void init(float* x, const float* d, const double* p) {
    (void)p;
    const float l_max_m = (float)2e-6;
    const float l_min_m = l_max_m / (float)2.;
    x[0] = l_min_m + (l_max_m - l_min_m) * d[1];
    x[1] = l_max_m;
  }
  __device__ __forceinline__ static double mass(const float* x, const double* p) {
    (void)p;
    return (double)(x[0] * lin_density());
  }
};


// ---------------------------------------------------------------------------
// Elementary functions for the model draws, written out with IEEE basic
// operations only (no fused multiply-add under --fmad=false), so the CPU
// restatement, which writes the same steps in C, rounds identically.
//   log: x = m 2^e, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(t),
//        t = (m - 1) / (m + 1), odd series to t^27 (|t| <= 0.172)
//   exp: x = k ln2 + r (Cody-Waite split of ln2, |r| <= ln2 / 2), Taylor
//        series of e^r to r^20, times 2^k
namespace sa_math {
constexpr double kLn2Hi = 6.93147180369123816490e-01;  // upper bits of ln 2
constexpr double kLn2Lo = 1.90821492927058770002e-10;  // ln 2 - kLn2Hi
constexpr double kLn2 = 0.69314718055994530942;
constexpr double kSqrt2 = 1.41421356237309504880;
constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ double scale2(double v, int k) {
  // v * 2^k by exact powers of two (k within [-2044, 2046])
  while (k > 1000) {
    v *= 0x1p1000;
    k -= 1000;
  }
  while (k < -1000) {
    v *= 0x1p-1000;
    k += 1000;
  }
  return v * __longlong_as_double((long long)(1023 + k) << 52);
}

__device__ __forceinline__ double log_d(double x) {
  if (x != x || x < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
  if (x == 0.0) return __longlong_as_double((long long)0xfff0000000000000ull);
  if (x == __longlong_as_double(0x7ff0000000000000ll)) return x;
  int e = 0;
  if (x < 0x1p-1022) {  // subnormal: scale into the normal range
    x *= 0x1p54;
    e = -54;
  }
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  e += (int)((b >> 52) & 0x7ffull) - 1022;
  double m = __longlong_as_double((long long)((b & 0x000fffffffffffffull) | 0x3fe0000000000000ull));  // [0.5, 1)
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  const double t = (m - 1.0) / (m + 1.0);
  const double t2 = t * t;
  double sum = 1.0 / 27.0;
  for (int k = 25; k >= 1; k -= 2) sum = sum * t2 + 1.0 / (double)k;
  return ((double)e * kLn2Hi + 2.0 * t * sum) + (double)e * kLn2Lo;
}

__device__ __forceinline__ double exp_d(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000ll);
  if (x < -745.1332191019412) return 0.0;
  const double k = floor(x / kLn2 + 0.5);
  const double r = (x - k * kLn2Hi) - k * kLn2Lo;
  double s = 1.0;
  for (int n = 20; n >= 1; --n) s = 1.0 + s * r / (double)n;
  return scale2(s, (int)k);
}

// Winitzki's approximation of erfinv (a = 0.147), with the reference's
// type flow (prng_extension.hpp L79-L94): the logarithm in double, the
// terms and square roots in the distribution's type.
__device__ __forceinline__ float erfinv_f(float x) {
  const float a = 0.147f;
  const float inv_a = (float)(1. / (double)a);
  const float tmp = (float)(2 / (kPi * (double)a));
  const double ln1mx2 = log_d((1. - (double)x) * (1. + (double)x));
  const float term1 = (float)((double)tmp + 0.5 * ln1mx2);
  const float term2 = (float)((double)inv_a * ln1mx2);
  return copysignf(sqrtf(sqrtf(term1 * term1 - term2) - term1), x);
}
__device__ __forceinline__ double erfinv_d(double x) {
  const double a = 0.147;
  const double inv_a = 1. / a;
  const double tmp = 2 / (kPi * a);
  const double ln1mx2 = log_d((1. - x) * (1. + x));
  const double term1 = tmp + 0.5 * ln1mx2;
  const double term2 = inv_a * ln1mx2;
  return copysign(sqrt(sqrt(term1 * term1 - term2) - term1), x);
}
// norminv (prng_extension.hpp L137-L147): mean + sd sqrt2 clamp(erfinv(2p - 1), -5, 5)
__device__ __forceinline__ float norminv_f(float p, float mean, float sd) {
  const float z = fminf(fmaxf(erfinv_f(2.f * p - 1.f), -5.f), 5.f);
  return (float)((double)mean + (double)sd * kSqrt2 * (double)z);
}
__device__ __forceinline__ double norminv_d(double p, double mean, double sd) {
  const double z = fmin(fmax(erfinv_d(2. * p - 1.), -5.), 5.);
  return mean + sd * kSqrt2 * z;
}
// TruncatedNormal draw (prng_extension.hpp L379-L414) from the uniform u,
// with the distribution's 0.5 erfc(-z / sqrt2) at its bounds given
__device__ __forceinline__ float truncnorm_f(float u, float mu, float sd, float pl, float pu) {
  const float p = u * (pu - pl) + pl;
  return norminv_f(p, mu, sd);
}
}  // namespace sa_math

// Flow of feed f at the relative time t (FeedDescriptor::update,
// apps/libs/simulation/src/feed_descriptor.cpp L12-L36): constant, or
// f0 + t * df (Linear), or f0 + exp(alpha * t) (Exponential; exp from IEEE
// operations, sa_math::exp_d, as the CPU restatement).
__device__ __forceinline__ double feed_flow_at(const ScenDev& S, unsigned f, double t) {
  const int kind = S.feed_kind[f];
  if (kind == 1) return __dadd_rn(S.feed_f0[f], __dmul_rn(t, S.feed_rate[f]));
  if (kind == 2) return __dadd_rn(S.feed_f0[f], sa_math::exp_d(__dmul_rn(S.feed_rate[f], t)));
  return S.feed_flow[f];
}

// Exit threshold on the integer draw x (odd, u = x 2^-24) of the
// reference's exit test dt*F > -ln(u)*V with the float logarithm
// (probability_leaving<precision_tag>, probability_leaving.hpp L18-L33):
// nlog[k] = -logf((2k + 1) 2^-24) does not grow with k, so the draws that
// exit are k >= k*, and x exits iff x > 2 k*.  k* is searched from the
// previous threshold (a bracket grown by doubling steps, then bisection),
// so a flow that changes little from step to step costs a few loads; every
// loop is bounded by 24 rounds.  2^24 when no draw exits.
__device__ __forceinline__ uint32_t exit_threshold_dev(const float* __restrict__ nlog, double dt, double flow,
                                                       double volume, uint32_t thr_prev) {
  const uint32_t N = 1u << 23;
  const double lhs = __dmul_rn(dt, flow);
  auto exits = [&](uint32_t k) { return lhs > __dmul_rn((double)nlog[k], volume); };
  uint32_t k0 = thr_prev >> 1;
  uint32_t lo = 0u, hi = N;  // k* in [lo, hi]; k < lo do not exit; hi exits or hi == N
  if (k0 < N) {
    if (exits(k0)) {
      hi = k0;
      uint32_t d = 1u;
      for (int it = 0; it < 24; ++it) {
        if (hi == 0u) break;
        const uint32_t c = hi > d ? hi - d : 0u;
        if (exits(c)) {
          hi = c;
          d <<= 1;
        } else {
          lo = c + 1u;
          break;
        }
      }
    } else {
      lo = k0 + 1u;
      uint32_t d = 1u;
      for (int it = 0; it < 24; ++it) {
        const uint32_t c = lo + d - 1u;
        if (c >= N) break;
        if (exits(c)) {
          hi = c;
          break;
        }
        lo = c + 1u;
        d <<= 1;
      }
    }
  }
  for (int it = 0; it < 24 && lo < hi; ++it) {
    const uint32_t mid = lo + (hi - lo) / 2u;
    if (exits(mid))
      hi = mid;
    else
      lo = mid + 1u;
  }
  return lo >= N ? (1u << 24) : 2u * lo;
}

// The reference's SimpleAcetate model (apps/libs/models/public/models/
// simple_acetate.hpp L26-L250): float state {length, l_max, a_p, a_max,
// a_e, a_e_s, a_e_a, phi_s, phi_a}, two species (glucose, acetate), two
// contributions per particle (general path).  The update follows the
// reference's type flow (L153-L203): per compartment the concentrations c_j
// (double) and inv_j = (float)(1. / (c_j + k_j)); per particle
// D_j = (float)(((double)adm_j * c_j) * inv_j).  Division draws: two
// log-normal uptake capacities a_p = exp(log(a_e) - sigma^2/2 + sigma z)
// with log(a_e) in float (the reference's Kokkos::log of the float a_e) and
// z a standard normal drawn by inverse CDF with the reference's erfinv (the
// reference draws a Kokkos normal), and two truncated-normal l_max; init:
// length and l_max from the length distribution (the reference's init draws
// l_max from l_dist too).
struct SimpleAcetateModel {
  static constexpr int n_var = 9;
  static constexpr int n_ctb = 2;
  static constexpr int n_rates = 6;
  static constexpr int n_upd = 6;
  static constexpr int model_id = 5;
  static constexpr bool separable = false;
  static constexpr unsigned read_mask = 0xFu;  // length, l_max, a_p, a_max
  __device__ __forceinline__ static float a_max_m() { return (float)(2e-6 / 3600.); }
  __device__ __forceinline__ static float l_max_m() { return (float)2e-6; }
  __device__ __forceinline__ static float lin_density() {
    const float d_m = (float)0.6e-6;
    return (float)1000 * (float)3.14159265358979323846 * d_m * d_m / (float)4.;
  }
  // r = {c_s (two words), c_a (two words), inv_s, inv_a}
  __device__ __forceinline__ static void rates(const double* c, const double* p, float* r) {
    (void)p;
    const float k_s = (float)1e-3, k_a = (float)1e-4;
    r[0] = __int_as_float(__double2loint(c[0]));
    r[1] = __int_as_float(__double2hiint(c[0]));
    r[2] = __int_as_float(__double2loint(c[1]));
    r[3] = __int_as_float(__double2hiint(c[1]));
    r[4] = __double2float_rn(__ddiv_rn(1., __dadd_rn(c[0], (double)k_s)));
    r[5] = __double2float_rn(__ddiv_rn(1., __dadd_rn(c[1], (double)k_a)));
  }
  __device__ __forceinline__ static int update(float dt, float* x, const float* r, float& basis, const float* pf) {
    float ctb[2];
    (void)basis;
    return update_general(dt, x, r, ctb, pf);
  }
  __device__ __forceinline__ static int update_general(float dt, float* x, const float* r, float* ctb,
                                                       const float* pf) {
    (void)pf;
    const double c0 = __hiloint2double(__float_as_int(r[1]), __float_as_int(r[0]));
    const double c1 = __hiloint2double(__float_as_int(r[3]), __float_as_int(r[2]));
    const float y_s = 2.f, y_a = 3.f;
    const float lin = lin_density();
    const float adm0 = x[3], adm1 = x[3] / 3.f;
    const float d0 = __double2float_rn(__dmul_rn(__dmul_rn((double)adm0, c0), (double)r[4]));
    const float d1 = __double2float_rn(__dmul_rn(__dmul_rn((double)adm1, c1), (double)r[5]));
    float a_e = 0.f;
    // Kokkos::min(a, b) = (b < a) ? b : a
    const float u0 = (x[2] < d0) ? x[2] : d0;
    a_e += u0;
    const float pa = d0 - x[2];
    const float mask = pa < 0.f ? 1.f : 0.f;
    const float u1 = mask * ((-pa < d1) ? -pa : d1) + (1.f - mask) * 0.f;
    a_e += u1;
    x[0] += dt * a_e;
    x[4] = a_e;
    x[5] = u0;
    x[6] = u1;
    const float phi_s = -1.f * d0 * lin * y_s;
    const float phi_a = mask * (-u1 * lin * y_a) + (1.f - mask) * (pa * lin * y_s / y_a);
    x[7] = phi_s;
    x[8] = phi_a;
    ctb[0] = phi_s;
    ctb[1] = phi_a;
    return x[0] >= x[1] ? kDivision : kIdle;
  }
  __device__ __forceinline__ static float coef(const float* r, int j) {
    (void)r;
    (void)j;
    return 0.f;
  }
  __device__ __forceinline__ static void division(float* x, float* child, const float* d, const double* p) {
    (void)p;
    const float lm = l_max_m();
    x[0] = x[0] / 2.F;
#pragma unroll
    for (int v = 0; v < 4; ++v) child[v] = x[v];
#pragma unroll
    for (int v = 4; v < 9; ++v) child[v] = 0.f;
    const double sigma = 0.2;
    const float log_ae = __double2float_rn(sa_math::log_d((double)x[4]));
    const double average = (double)log_ae - sigma * sigma / 2;
    // Kokkos' normal(mean, sd) = mean + sd * z, z standard normal
    const double z1 = sa_math::norminv_d((double)d[0], 0.0, 1.0);
    const double z2 = sa_math::norminv_d((double)d[1], 0.0, 1.0);
    const float gen1 = (float)sa_math::exp_d(average + sigma * z1);
    const float gen2 = (float)sa_math::exp_d(average + sigma * z2);
    // l_max_dist: TruncatedNormal(l_max, l_max / 10, 0.7 l_max, 1.3 l_max):
    // z = -3, +3, 0.5 erfc(-z / sqrt2) rounded to float
    const float sd = (float)((double)lm / 10.);
    const float lmax1 = sa_math::truncnorm_f(d[2], lm, sd, 0x1.61de2p-10f, 0x1.ff4f1p-1f);
    const float lmax2 = sa_math::truncnorm_f(d[3], lm, sd, 0x1.61de2p-10f, 0x1.ff4f1p-1f);
    x[2] = gen1;
    x[1] = lmax1;
    child[2] = gen2;
    child[1] = lmax2;
  }
  __device__ __forceinline__ static void init(float* x, const float* d, const double* p) {
    (void)p;
    const float lm = l_max_m();
    // l_dist: TruncatedNormal(0.75 l_max, l_max / 10, 0.7 l_min, 1.3 l_max):
    // z = -4.0000005, +5.4999995
    const float mu = (float)((double)lm * 0.75), sd = (float)((double)lm / 10.);
    x[0] = sa_math::truncnorm_f(d[1], mu, sd, 0x1.09ad56p-15f, 1.0f);
    x[1] = sa_math::truncnorm_f(d[2], mu, sd, 0x1.09ad56p-15f, 1.0f);
    x[2] = a_max_m() / 2.f;
    x[3] = a_max_m();  // the mean of a_max_dist, symmetric about a_max
#pragma unroll
    for (int v = 4; v < 9; ++v) x[v] = 0.f;
  }
  __device__ __forceinline__ static double mass(const float* x, const double* p) {
    (void)p;
    return (double)(x[0] * lin_density());
  }
};

}  // namespace bmc

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

namespace bmc {

constexpr int kMaxOutlets = 8;
constexpr int kMaxSpecies = 8;
constexpr int kMaxVar = 8;
constexpr int kMaxRates = 8;
constexpr long long kQMax = 1LL << 42;  // |quantised value| bound
// A block flushes its shared-memory accumulator before it has summed more
// than 2^20 particles, so |partial| <= 2^62 and no int64 sum can overflow.
constexpr unsigned kFlushParticles = 1u << 20;
// ScalarSimulation::clearNegs threshold: scheme relative error 1e-4 times
// the species scale 5e-3 (implScalar.cpp L273-L277)
constexpr double kClearNegTol = 1e-4 * 5e-3;

enum : uint8_t { kIdle = 0, kDivision = 1, kExit = 2, kDead = 3 };

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
  unsigned int pad;
};

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
};

// A scenario whose step counter has reached its limit is left untouched.
__device__ __forceinline__ bool scen_finished(const ScenDev& S, const Control* ctl) {
  return S.step_limit != 0u && ctl->step >= S.step_limit;
}

// ---------------------------------------------------------------------------
// Draw source: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), keyed by
// the scenario seed, counter (particle id, step, purpose, 0).
struct Draws {
  float u[4];
};

__device__ __forceinline__ Draws philox_draws(unsigned long long seed, uint32_t id, uint32_t step,
                                              uint32_t purpose) {
  uint32_t c0 = id, c1 = step, c2 = purpose, c3 = 0u;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
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
  uint32_t c0 = id, c1 = step, c2 = purpose, c3 = 0u;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
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

}  // namespace bmc

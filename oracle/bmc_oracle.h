/*
 * bmc_oracle.h -- CPU restatement of the BioCMA-MCST Monte Carlo cycle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file and bmc_oracle.c are the oracle the
 * GPU path is compared against; the product (libbmc) never links, loads or
 * calls them.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use the oracle.
 *
 * What it restates (reference paths are relative to the BioCMA-MCST tree):
 *   - per-particle cycle: apps/libs/simulation/public/simulation/kernels/
 *       model_kernel.hpp L164-L268 (ages(i,1)+=dt, Model::update, division)
 *       contribution_kernel.hpp L146-L186 (S(j,pos) += w*contribs(p,j))
 *       move_kernel.hpp L62-L103 (__find_next_compartment), L393-L437
 *       (handle_move), L348-L359 + L588-L648 (TagLeave / handle_exit)
 *     apps/libs/simulation/public/simulation/probability_leaving.hpp L18-L35
 *   - division buffer, compaction, merge: apps/libs/mc/public/mc/
 *       particles_container.hpp L541-L575 (update_and_remove_inactive,
 *       handle_division), L577-L600 (merge_buffer), L737-L795
 *       (remove_inactive_particles) and L292-L383 (CompactParticlesFunctor,
 *       whose single-threaded execution order is the one restated here)
 *   - liquid step: apps/libs/simulation/src/implScalar.cpp L251-L264
 *       (performStep), apps/libs/simulation/src/simulation.model.cpp L73-L111
 *       (update_feed), ordering from apps/core/src/host_specific.cpp L257-L313
 *
 * Parity status: the reference ships no golden vectors for the cycle, the
 * move, the scatter or the liquid step (its own tests cover feed arithmetic
 * and container counts only).  The oracle is pinned against those tests, the
 * published Philox4x32-10 known-answer vectors, and hand-derived cases
 * worked from the reference source; see tests/golden/.
 */
#ifndef BMC_ORACLE_H
#define BMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_IDLE = 0, ORC_DIVISION = 1, ORC_EXIT = 2, ORC_DEAD = 3 };
enum {
  ORC_MODEL_MONOD = 1,
  ORC_MODEL_OVERFLOW = 2,
  ORC_MODEL_FIXED_LENGTH = 3,
  ORC_MODEL_FIXED_LENGTH_GENERAL = 4,
  ORC_MODEL_SIMPLE_ACETATE = 5
};
enum { ORC_DRAW_PHILOX = 0, ORC_DRAW_XORSHIFT = 1 };

/* A cell model supplied at run time as host functions (a model library's
 * bmc_udf_host_model, include/bmc.h; same layout).  x, child and r point to
 * the model's float type (double when f64 != 0, else float). */
typedef struct orc_udf_model {
  uint32_t n_var;
  uint32_t n_ctb;
  uint32_t n_rates;
  int32_t separable;
  void (*rates)(const double* c, const double* params, void* r);
  int32_t (*update)(double dt, void* x, const void* r, void* out, const double* params);
  double (*coef)(const void* r, int32_t j);
  void (*division)(void* x, void* child, const float* draws, const double* params);
  void (*init)(void* x, const float* draws, const double* params);
  double (*mass)(const void* x, const double* params);
  /* update with the particle's context (draws of purpose 3, the
   * compartment's concentrations and index), NULL when the model has none */
  int32_t (*update_ctx)(double dt, void* x, const void* r, void* out, const double* params, const float* draws,
                        const double* c, uint32_t position, uint32_t n_species);
} orc_udf_model;

#define ORC_MAX_OUTLETS 8
#define ORC_MAX_PARAMS 16

/* Every array is owned by the caller.  Particle arrays have `phys_capacity`
 * slots; `state` is SoA: state[v * phys_capacity + i], element type double
 * when f64 != 0 else float. */
typedef struct orc_state {
  /* particle container */
  uint64_t n_used;
  uint64_t phys_capacity;
  uint64_t inactive;
  uint64_t next_id;
  void* state;
  uint32_t* pos;
  uint8_t* status;
  float* age_h; /* reference ages(i,0): hydraulic time */
  float* age_d; /* reference ages(i,1): time since division */
  uint32_t* id;
  uint8_t* div_flag;     /* scratch, phys_capacity */
  uint32_t* div_pos;     /* scratch, phys_capacity */
  void* child_state;     /* scratch, n_var * phys_capacity */
  uint32_t* child_pos;   /* scratch */
  uint32_t* gap_slot;    /* scratch */
  uint32_t* src_slot;    /* scratch */

  /* model */
  int32_t model;
  int32_t f64;
  uint32_t n_var;
  uint32_t n_ctb;
  double params[ORC_MAX_PARAMS];
  double weight;

  /* domain: liquid_volume, diag_transition (out flows), neighbors, CDF */
  uint32_t n_c;
  uint32_t K;
  uint32_t n_s;
  const double* volume;
  const double* out_flow;
  const uint32_t* neighbors; /* n_c * K, row-major */
  const double* cdf;         /* n_c * K, row-major */
  uint32_t n_outlets;
  uint32_t outlet_index[ORC_MAX_OUTLETS];
  double outlet_flow[ORC_MAX_OUTLETS];
  double outlet_volume[ORC_MAX_OUTLETS];

  /* liquid scalars, layout [compartment][species] (reference LayoutLeft of
   * an n_species x n_compartments matrix) */
  double* C;
  double* M;
  double* src;      /* contributions of the last cycle (+ feed during a step) */
  double* sink;     /* per compartment */
  const double* vinv;
  const uint32_t* in_ptr;  /* incoming-flow CSR by destination column */
  const uint32_t* in_idx;
  const double* in_flow;
  /* feeds: constant flow * concentration at an inlet, optional outlet sink */
  uint32_t n_feeds;
  uint32_t feed_in[ORC_MAX_OUTLETS];
  int32_t feed_out[ORC_MAX_OUTLETS];
  double feed_flow[ORC_MAX_OUTLETS];
  double feed_conc[ORC_MAX_OUTLETS * 8]; /* [feed][species] */

  /* randomness */
  int32_t draw_mode;
  uint64_t seed;
  uint32_t step;

  /* runtime parameters (reference MC::RuntimeParameters) */
  double dead_ratio_threshold;
  uint64_t min_removal;

  /* Exact contribution sums.  Separable models (contribution j =
   * coef_j(C) * basis(particle)): each particle's basis is rounded to the
   * integer q = rint(basis * 2^-q_exp[0]), |q| <= q_max, summed exactly per
   * compartment, and src(c, j) = (weight * coef_j(c)) * total.  General
   * models: weight * contribution j of each particle is quantised with
   * q_exp[j] and summed exactly.  See orc_quantize / orc_fixed_to_double. */
  int32_t separable;
  int32_t q_exp[8];
  int64_t q_max;
  uint64_t ctb_clamped;

  /* quirk emulation: 1 = reference Tag3D contribution early return */
  int32_t quirk_tag3d;

  /* per-step outputs */
  uint64_t births;
  uint64_t exits;
  uint64_t moves;
  uint64_t overflow;
  uint64_t requested_divisions;
  int32_t compacted;
  int32_t error;

  /* run-time model: when set, it replaces the compiled-in models */
  const orc_udf_model* udf;

  /* gas phase of a two-phase flow (gas == 0: liquid only):
   * apps/libs/simulation/src/simulation.model.cpp L132-L150 (ode_step),
   * implScalar.cpp L229-L249 (performStepGL), hydro/impl_mtr.cpp L150-L166
   * (fixed kla transfer), implScalar.cpp L266-L293 (clearNegs) */
  int32_t gas;
  const double* gvinv;
  const uint32_t* g_in_ptr;
  const uint32_t* g_in_idx;
  const double* g_in_flow;
  const double* g_out_flow; /* gas diagonal = -g_out_flow */
  double* Cg;
  double* Mg;
  const double* kla;        /* [n_c][n_s] */
  double* mtr;              /* [n_c][n_s], transfer to the liquid of the last step */
  double henry[8];
  uint32_t n_gfeeds;
  uint32_t gfeed_in[ORC_MAX_OUTLETS];
  int32_t gfeed_out[ORC_MAX_OUTLETS];
  double gfeed_flow[ORC_MAX_OUTLETS];
  double gfeed_conc[ORC_MAX_OUTLETS * 8];

  /* feed schedules (Simulation::Feed::FeedDescriptor, feed_descriptor.hpp
   * L39-L100; FeedDescriptor::update, feed_descriptor.cpp L12-L36): kind 0
   * constant (feed_flow), 1 linear f0 + t * rate, 2 exponential
   * f0 + exp(rate * t), evaluated by orc_step at the relative time t_rel
   * (the sum of the time steps of the steps so far, simulation_times.hpp
   * L12-L29) */
  int32_t feed_kind[ORC_MAX_OUTLETS];
  double feed_f0[ORC_MAX_OUTLETS];
  double feed_rate[ORC_MAX_OUTLETS];
  double t_rel;

  /* time-event probes (reference Simulation::Probes, apps/libs/simulation/
   * public/simulation/probe.hpp L38-L146, with use_probe): probe_buf[0]
   * leaving times (ages(i,0) of a particle leaving through an outlet,
   * before its reset, move_kernel.hpp L629-L635), probe_buf[1] division
   * times (ages(i,1) of a particle whose update asks to divide, before the
   * division is attempted, model_kernel.hpp L245-L251), both in slot order
   * within a step; probe_n counts every event, a value is stored while its
   * index is below probe_cap (0: probes off) */
  uint64_t probe_cap;
  double* probe_buf[2];
  uint64_t probe_n[2];
} orc_state;

void orc_set_outlets(orc_state* s);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float orc_u01(uint32_t x);
void orc_draws(uint64_t seed, uint32_t id, uint32_t step, uint32_t purpose, float out[4]);

void orc_init_particles(orc_state* s, uint64_t n, uint32_t pos_lo, uint32_t pos_hi);
double orc_total_mass(const orc_state* s);

void orc_scalar_step(orc_state* s, double dt);
/* Probes::set (probe.hpp L61-L79): counts the event of probe k and stores
 * v while the buffer has room; returns 1 if stored. */
int orc_probe_set(orc_state* s, int k, double v);
/* Model::mass of every used slot into out[n_used]. */
void orc_particle_mass(const orc_state* s, double* out);
void orc_cycle(orc_state* s, double dt, int n_threads);
void orc_post_cycle(orc_state* s);
void orc_step(orc_state* s, double dt, int n_threads);
void orc_liquid_step(orc_state* s, double dt);
void orc_run(orc_state* s, double dt, uint32_t n_steps, int n_threads);
void orc_remove_inactive(orc_state* s, uint64_t to_remove);

int64_t orc_quantize(double v, int32_t e, int64_t qmax, int* clamped);
double orc_fixed_to_double(__int128 t, int32_t e);
uint32_t orc_find_next(const orc_state* s, uint32_t c, double u);
void orc_repartition(const orc_state* s, uint64_t* counts);

/* SimpleAcetate draw functions (for their accuracy tests). */
double orc_sa_log(double x);
double orc_sa_exp(double x);
double orc_sa_erfinv(double x);
float orc_sa_truncnorm(float u, float mu, float sd, float pl, float pu);


/* Pin entry points (one particle through the cycle's own functions). */
uint32_t orc_pin_find_next(uint32_t K, const double* cdf_row, const uint32_t* nbr_row, double u);
uint32_t orc_pin_move(uint32_t n_c, uint32_t K, const double* volume, const double* out_flow, const uint32_t* nbr,
                      const double* cdf, double dt, uint32_t pos, float u1, float u2, int32_t* moved);
int32_t orc_pin_leave(uint32_t n_outlets, const uint32_t* index, const double* flow, const double* volume, double dt,
                      uint32_t pos, uint8_t* status, float* age_h, float u);
int32_t orc_pin_exit_test(double dt, double flow, double volume, float u);
int32_t orc_pin_model_update(int32_t model, double dt, float* x, const double* c, float* ctb);
void orc_pin_fixed_length_division(float* x, float* child);
void orc_pin_simple_acetate_division(float* x, float* child, double z1, double z2, float u3, float u4);
void orc_pin_simple_acetate_init(float* x, float u_length, float u_lmax);
float orc_pin_erfinv_f(float x);
double orc_pin_erfinv_d(double x);
float orc_pin_norminv_f(float p, float mean, float sd);
double orc_pin_std_normal(float u);
void orc_draw_table(uint64_t seed, const uint32_t* ids, uint64_t n, uint32_t step, uint32_t purpose, float* out);
void orc_division_draw_table(uint64_t seed, const uint32_t* ids, uint64_t n, uint32_t step, double* out);
void orc_std_normal_table(const float* u, uint64_t n, double* out);
void orc_truncnorm_table(const float* u, uint64_t n, float mu, float sd, float lo, float hi, float* out);
float orc_pin_truncnorm_f(double u, float mu, float sd, float lower, float upper);
int32_t orc_logf_monotone_over_draws(uint32_t* bad_k);
double orc_feed_flow(int32_t kind, double flow, double f0, double rate, double t);

#ifdef __cplusplus
}
#endif
#endif

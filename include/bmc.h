/*
 * bmc.h -- C-ABI of the GB300 Monte Carlo cycle library (libbmc.so).
 *
 * The library replaces the BioCMA-MCST Monte Carlo cycle: the per-particle
 * model update, the compartment move and outlet exit, the contribution
 * scatter, and division / removal / compaction of the particle container,
 * plus the liquid-scalar Euler step that consumes the contributions.  Every
 * entry point takes plain pointers and sizes, returns 0 on success and a
 * negative BMC_E* code on failure (bmc_last_error() then holds a message),
 * mirroring apps/api/public/api/api_raw.h of the reference (int return
 * codes, opaque handle).  Host pointers are read during the call only.
 *
 * Reference paths below are relative to the BioCMA-MCST tree.
 */
#ifndef BMC_H
#define BMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BMC_VERSION_MAJOR 1
#define BMC_VERSION_MINOR 1

/* Return codes (reference: ApiResult::to_c_ret_code,
 * apps/api/public/api/results.hpp; ErrorCodes,
 * apps/libs/simulation/public/simulation/simulation_exception.hpp L10). */
#define BMC_OK 0
#define BMC_E_INVALID -1     /* bad argument / size mismatch */
#define BMC_E_CUDA -2        /* CUDA runtime error */
#define BMC_E_STATE -3       /* call out of order (e.g. no domain yet) */
#define BMC_E_CAPACITY -4    /* more particles than the container can hold */
#define BMC_E_DEVICE -5      /* device error word set (see bmc_step_stats.error) */
#define BMC_E_UNSUPPORTED -6 /* model / precision not compiled in */

/* Particle status, reference MC::Status (apps/libs/mc/public/mc/alias.hpp
 * L124-L130). */
#define BMC_STATUS_IDLE 0
#define BMC_STATUS_DIVISION 1
#define BMC_STATUS_EXIT 2
#define BMC_STATUS_DEAD 3

/* Compiled model plugins (the ModelType concept,
 * apps/libs/mc/public/mc/traits.hpp L67-L133).  FIXED_LENGTH restates the
 * reference's FixedLength model (apps/libs/models/public/models/
 * fixed_length.hpp); MONOD and OVERFLOW are the benchmark's Monod uptake and
 * Monod + overflow-to-acetate models written against the same concept. */
#define BMC_MODEL_MONOD 1
#define BMC_MODEL_OVERFLOW 2
#define BMC_MODEL_FIXED_LENGTH 3
/* FixedLength through the general per-particle contribution path. */
#define BMC_MODEL_FIXED_LENGTH_GENERAL 4
/* The reference's SimpleAcetate model (apps/libs/models/public/models/
 * simple_acetate.hpp): float state of 9 variables, glucose and acetate
 * uptake, two contributions per particle, log-normal and truncated-normal
 * draws at division. */
#define BMC_MODEL_SIMPLE_ACETATE 5

/* Device error word bits (copied back with the step statistics). */
#define BMC_ERR_POSITION 1u  /* compartment index out of range */
#define BMC_ERR_CLAMP 2u     /* a contribution exceeded its quantum range */
#define BMC_ERR_IDS 4u       /* particle id space (2^32) exhausted */
#define BMC_ERR_COMPACT 8u   /* compaction lists disagree (internal) */
#define BMC_ERR_TIMEOUT 16u  /* a bounded wait inside a kernel gave up (the step is void) */
#define BMC_ERR_SMEM 32u     /* the launch's shared memory is smaller than the accumulator (internal; the step is void) */

typedef struct bmc_scenario bmc_scenario;
typedef struct bmc_batch bmc_batch;

/* Model descriptor: the host-side metadata of the reference's ModelType
 * (n_var, n_c, FloatType) plus the parameter vector the device plugin reads.
 * Reference: traits.hpp L80-L100 (n_var, n_c, FloatType), and the UDF
 * metadata queries set_nvar_udf / set_nc_udf
 * (apps/libs/models/ext/udf_includes.hpp L29-L30). */
typedef struct bmc_model_desc {
  int32_t model;      /* BMC_MODEL_* */
  int32_t f64;        /* 1: double state and arithmetic, 0: float */
  uint32_t n_var;     /* must equal the plugin's n_var */
  uint32_t n_ctb;     /* must equal the plugin's contribution count */
  double params[16];  /* plugin parameters */
} bmc_model_desc;

/* Scenario descriptor: one reactor = one particle container + domain +
 * liquid scalars.  Reference: ParticlesContainer(RuntimeParameters, n, ...)
 * (apps/libs/mc/public/mc/particles_container.hpp L25-L43, L700) and
 * MC::load_tuning_constant (apps/libs/mc/src/unit.cpp L309-L343). */
typedef struct bmc_scenario_desc {
  bmc_model_desc model;
  uint32_t n_species;
  uint64_t capacity;               /* particle slots allocated on the device */
  uint64_t seed;                   /* Philox key */
  double dead_ratio_threshold;     /* BIOMC_MC_REMOVE_RATIO_THRESHOLD, 0.01 */
  uint64_t min_removal;            /* BIOMC_MC_MINIMUM_REMOVAL, 0 */
  /* Bounds that fix the quanta of the exact contribution sums: for a
   * separable model (contribution j = coef_j(C) * basis(particle)),
   * value_bound[0] bounds |basis| (the mass for the Monod models, 1 for
   * FixedLength); for a general model value_bound[j] bounds |contribution
   * j| of one particle.  Values above the bound are clamped and flagged
   * (BMC_ERR_CLAMP). */
  double value_bound[8];
} bmc_scenario_desc;

/* A liquid feed, reference Simulation::Feed::FeedDescriptor
 * (apps/libs/simulation/public/simulation/feed_descriptor.hpp L91-L100):
 * constant flow, one concentration per species at the inlet, optional
 * outlet (-1 for none) that becomes a leaving flow of the particles and a
 * sink of the liquid scalars. */
typedef struct bmc_feed {
  uint32_t inlet;
  int32_t outlet;
  double flow;
  double conc[8];
} bmc_feed;

/* Per-step statistics.  Reference: CycleReduceType {waiting_allocation,
 * dead} and the out counter returned by CycleFunctors::get_host_reduction
 * (apps/libs/simulation/public/simulation/kernels/kernels.hpp L80-L89), the
 * event tallies of MC::EventContainer (apps/libs/mc/public/mc/events.hpp
 * L17-L26) and ParticlesContainer::n_particles / get_inactive. */
typedef struct bmc_step_stats {
  uint64_t n_used;      /* slots in use (Idle + not yet removed) */
  uint64_t inactive;    /* non-Idle slots not yet removed */
  uint64_t births;      /* NewParticle events of the last step */
  uint64_t exits;       /* Exit events of the last step */
  uint64_t moves;       /* Move events of the last step */
  uint64_t overflow;    /* divisions refused for lack of room (Overflow) */
  uint64_t requested_divisions;
  uint64_t clamped;     /* contributions clamped to the quantum range (total) */
  uint64_t next_id;
  uint32_t step;
  uint32_t compacted;   /* 1 if the last step removed inactive particles */
  uint32_t error;       /* BMC_ERR_* bits, sticky */
  uint32_t pad;
  double mass_balance[8]; /* relative liquid mass-balance residual per species */
} bmc_step_stats;

/* ---- library ---------------------------------------------------------- */
int bmc_version(int32_t* major, int32_t* minor);
const char* bmc_last_error(void);
/* Number of SMs of the current device and the library's default device. */
int bmc_device_sm_count(int32_t* sm_count);

/* ---- scenario lifetime -------------------------------------------------- */
/* Replaces the construction of MC::ParticlesContainer + ReactorDomain +
 * ScalarSimulation in SimulationUnit's constructor
 * (apps/libs/simulation/src/simulation.cpp L47-L81). */
int bmc_scenario_create(const bmc_scenario_desc* desc, bmc_scenario** out);
int bmc_scenario_destroy(bmc_scenario* s);

/* Grow the particle container to at least `capacity` slots between steps
 * (ParticlesContainer::_resize on growth, apps/libs/mc/public/mc/
 * particles_container.hpp L603-L650: the live particles keep their slots;
 * the reference grows inside merge_buffer, here a caller grows when a step
 * reports overflow or when n_used nears the capacity).  Never shrinks;
 * the scenario's captured step is re-captured at its next run. */
int bmc_reserve(bmc_scenario* s, uint64_t capacity);

/* ReactorDomain::update (apps/libs/mc/src/domain.cpp L44-L74):
 * liquid volumes [n_c], neighbours [n_c*K] (row-major, std::size_t in the
 * reference), total out-flows per compartment (diag_transition) [n_c] and
 * the cumulative destination probabilities [n_c*K]. */
int bmc_domain_update(bmc_scenario* s, uint32_t n_c, uint32_t K, const double* volume,
                      const uint64_t* neighbors, const double* out_flows, const double* cdf);

/* ScalarSimulation::set_transition (apps/libs/simulation/src/implScalar.cpp
 * L323-L330): the liquid transition matrix in COO form; diagonal entries are
 * T(j,j) = -sum of out-flows. */
int bmc_set_transition_coo(bmc_scenario* s, uint32_t n, uint64_t nnz, const uint64_t* rows,
                           const uint64_t* cols, const double* values);

/* ScalarSimulation::deep_copy_concentration + set_mass
 * (implScalar.cpp L299-L320): concentrations [n_c][n_species]
 * (the reference's LayoutLeft n_species x n_c matrix), M = C * V. */
int bmc_set_concentrations(bmc_scenario* s, const double* conc);

/* Feeds (SimulationUnit::update_feed, simulation.model.cpp L73-L111, with
 * ReactorDomain::set_leaving_flow, domain.cpp L97-L108). At most 8.  The
 * feeds are constant (bmc_feed.flow) until bmc_set_feed_schedules is
 * called; setting the feeds again clears their schedules. */
int bmc_set_feeds(bmc_scenario* s, uint32_t n_feeds, const bmc_feed* feeds);

/* Time-varying feed flows, the reference's FeedDescriptor variants
 * Constant | Linear | Exponential (apps/libs/simulation/public/simulation/
 * feed_descriptor.hpp L39-L60, L91-L100; FeedDescriptor::update,
 * apps/libs/simulation/src/feed_descriptor.cpp L12-L36, L100-L103):
 * flow(t) = bmc_feed.flow (constant), f0 + t * rate (linear, rate = df in
 * m^3/s^2) or f0 + exp(rate * t) (exponential, rate = alpha in 1/s), at the
 * scenario's relative time t: 0 at creation, advanced by dt after every
 * main-loop step (bmc_step, bmc_step_read, bmc_run and batch runs; not by
 * bmc_cycle), as SimulationUnit::advance does.  Every main-loop step
 * evaluates the flows on the device, inside captured graphs and batches:
 * the inlet sources flow(t) * conc, the outlet sink flow(t), and the
 * outlet's leaving flow with its exit threshold (update_feed,
 * simulation.model.cpp L79-L108).  One schedule per feed of bmc_set_feeds,
 * same order.  A schedule on a feed with an outlet makes the library build
 * a 32 MiB table on the device (held until exit). */
#define BMC_FEED_CONSTANT 0
#define BMC_FEED_LINEAR 1
#define BMC_FEED_EXPONENTIAL 2
typedef struct bmc_feed_schedule {
  int32_t kind;  /* BMC_FEED_* */
  int32_t pad;
  double f0;     /* m^3/s */
  double rate;   /* df (linear) or alpha (exponential) */
} bmc_feed_schedule;
int bmc_set_feed_schedules(bmc_scenario* s, uint32_t n_feeds, const bmc_feed_schedule* schedules);
/* The scenario's relative time t (s) at which the next step evaluates its
 * feed schedules (Getter::relative_time, simulation.getset.cpp L154-L158). */
int bmc_feed_time(bmc_scenario* s, double* t);

/* MC::init + post_init_weight (apps/libs/mc/src/unit.cpp L102-L163,
 * L233-L306): n particles, model init, position uniform in [0, n_c) (or 0
 * when uniform_init == 0), weight = x0 * V_total / total mass.  Writes the
 * weight if weight_out is not NULL. */
int bmc_init_particles(bmc_scenario* s, uint64_t n, int32_t uniform_init, double x0,
                       double* weight_out);
int bmc_set_weight(bmc_scenario* s, double weight);

/* Upload an explicit container (n particles, SoA state [n_var][n]); used by
 * callers that hold particles already (serde load, tests). */
int bmc_set_particles(bmc_scenario* s, uint64_t n, const void* state, const uint32_t* pos,
                      const uint8_t* status, const float* age_h, const float* age_d,
                      const uint32_t* id, uint64_t next_id);

/* ---- the hot path -------------------------------------------------------- */
/* SimulationUnit::cycleProcess (apps/libs/simulation/public/simulation/
 * simulation.hpp L184-L239) with CycleFunctors::launch_model /
 * launch_move (kernels.hpp L124-L224) and post_cycle: model update,
 * contribution scatter, move, exit, division, compaction, merge.  Uses the
 * concentrations currently on the device; leaves the contributions of this
 * cycle as the sources of the next liquid step. */
int bmc_cycle(bmc_scenario* s, double dt, bmc_step_stats* stats);
/* cycleProcess for a caller that keeps its own liquid-scalar step (the
 * reference's host ScalarSimulation, SimulationUnit::cycleProcess with
 * getter concentrations in, scatter_contribute / synchro_sources out:
 * apps/libs/simulation/src/simulation.cpp L143-L160, implScalar.cpp L194):
 * concentrations [n_c][n_species] in, the cycle's contributions (sources,
 * same layout, kg/s) out; both host pointers, or both device pointers when
 * on_device != 0 (no host round trip).  Feeds are not applied (they belong
 * to the caller's liquid step); concentrations are not checked on device. */
int bmc_cycle_external(bmc_scenario* s, double dt, const double* conc, double* sources, int32_t on_device,
                       bmc_step_stats* stats);

/* One iteration of the reference main loop (apps/core/src/host_specific.cpp
 * L280-L291): update_feed, ode_step (ScalarSimulation::performStep,
 * implScalar.cpp L251-L264), clearContribution, cycleProcess. */
int bmc_step(bmc_scenario* s, double dt, bmc_step_stats* stats);

/* bmc_step followed by bmc_read_liquid(conc) with a single device
 * synchronisation: the step, the control block and the concentrations
 * [n_c][n_s] after the step travel back together (the host loop that reads
 * the field every iteration).  It is bmc_step_enqueue followed at once by
 * bmc_step_collect (the mapped host buffer below is allocated at the first
 * call); refused with BMC_E_STATE while enqueued steps are not collected. */
int bmc_step_read(bmc_scenario* s, double dt, bmc_step_stats* stats, double* conc);

/* A main loop that reads the field back every iteration, pipelined: the
 * host enqueues step k+1 before it waits for the results of step k, so the
 * device does not idle while the host handles them.  bmc_step_enqueue
 * enqueues one iteration (as bmc_step) and the transfer of its counters and
 * concentrations [n_c][n_s] into pinned host memory (mapped into the device
 * address space; allocated at the first call, freed with the scenario),
 * without waiting; at most two steps are in flight.  The transfer of a step
 * goes out with the next call on the scenario (in one launch with the
 * descriptor upload of a bmc_set_feeds between two enqueues), always before
 * anything else uses the scenario's stream.  bmc_step_collect waits for the
 * oldest enqueued step and writes its results into the stats and conc
 * buffers given to its bmc_step_enqueue (returns BMC_E_DEVICE when that step
 * set the error word).  Other stepping calls on the scenario are refused
 * (BMC_E_STATE) until every enqueued step is collected. */
int bmc_step_enqueue(bmc_scenario* s, double dt, bmc_step_stats* stats, double* conc);
int bmc_step_collect(bmc_scenario* s);

/* n_steps iterations on the device without host round trips (one captured
 * CUDA graph replayed).  Statistics are those of the last step. */
int bmc_run(bmc_scenario* s, double dt, uint32_t n_steps, bmc_step_stats* stats);

/* Launch shape of the scenario's cycle kernel: threads per block and
 * particles per thread of a compiled variant (256 x 1, 256 x 2, 256 x 4,
 * 512 x 2, 1024 x 1 stream particles through registers; 288 x 4 and 544 x 2
 * are 256 or 512 consumer threads plus a producer warp staging tiles through
 * the copy engine), resident blocks per SM (0 = as many as fit); threads and
 * ppt both 0 keep the current variant.  A new scenario starts in the
 * automatic shape, 544 x 2.  The staging shapes sum the contributions in
 * shared memory (n_compartments x accumulator columns x 8 bytes, beside
 * the stage buffers) while that fits a block, else straight into the
 * scenario's global accumulator, so every domain size runs; the
 * register-streaming shapes always sum in shared memory and are refused
 * (BMC_E_UNSUPPORTED) on a domain whose accumulator does not fit. */
int bmc_set_shape(bmc_scenario* s, uint32_t threads, uint32_t ppt, uint32_t blocks_per_sm);

/* Step budget: once the scenario's step counter reaches step_limit its
 * steps are no-ops (0 removes the limit).  Lets a batch hold scenarios that
 * need different numbers of steps (serving). */
int bmc_set_step_limit(bmc_scenario* s, uint32_t step_limit);

/* Enqueue n_steps iterations without waiting (bmc_synchronize waits). */
int bmc_run_async(bmc_scenario* s, double dt, uint32_t n_steps);
int bmc_synchronize(bmc_scenario* s);

/* ---- readback ------------------------------------------------------------ */
int bmc_read_stats(bmc_scenario* s, bmc_step_stats* stats);
/* Model::mass of each of the n_used slots, computed on the device by the
 * scenario's model (the mass column of the reference's particle dump,
 * get_properties, apps/core/public/core/post_process.hpp L96-L98). */
int bmc_read_mass(bmc_scenario* s, uint64_t max_n, double* mass, uint64_t* n_out);
/* Host buffers sized for n_used particles (state as [n_var][n_used]). */
int bmc_read_particles(bmc_scenario* s, uint64_t max_n, void* state, uint32_t* pos,
                       uint8_t* status, float* age_h, float* age_d, uint32_t* id,
                       uint64_t* n_out);
int bmc_read_liquid(bmc_scenario* s, double* conc, double* mass, double* sources);
/* MonteCarloUnit::getRepartition (apps/libs/mc/src/unit.cpp L191-L230). */
int bmc_repartition(bmc_scenario* s, uint64_t* counts);
/* bmc_repartition without any device allocation.  It has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory when
 * they ask for the counts: a program whose device memory is all handed out
 * in advance (a caching pool allocator such as PyTorch's under a fixed cap,
 * or a serving loop that admits scenarios against an HBM budget), where a
 * cudaMalloc outside that budget fails, and a program that cannot afford
 * the device-wide synchronisation cudaMalloc and cudaFree can cause while
 * other streams (a batch, another scenario) keep running.
 * The per-compartment counters live in one static device array of
 * BMC_REPARTITION_STATIC_MAX (65536) entries, 512 KiB held on every GPU
 * that loads the library until the process exits; scenarios with more
 * compartments are rejected with BMC_E_CAPACITY.  The call works on the
 * scenario's own device (made current for the call, the caller's device
 * restored after it); its first call on a device looks the array up
 * (cudaGetSymbolAddress).  Every call shares the array and clears the part
 * it uses; two calls whose work overlaps on the GPU (different streams,
 * different host threads) race.  counts is a host array of n_compartments
 * entries; the call waits for its result. */
#define BMC_REPARTITION_STATIC_MAX 65536
int bmc_repartition_static(bmc_scenario* s, uint64_t* counts);

/* Force removal of every inactive particle (ParticlesContainer::
 * force_remove_dead, particles_container.hpp L460-L465). */
int bmc_force_remove_dead(bmc_scenario* s);

/* ---- event tallies ---------------------------------------------------------- */
/* The reference's MC::EventContainer (apps/libs/mc/public/mc/events.hpp
 * L17-L26, L149): counts accumulated over every step since the last clear,
 * inside graph runs and batches too, in the reference's order.  As its
 * cycle does (model_kernel.hpp L253-L259), every division request counts as
 * a NewParticle event, refused or not (the refused ones also as Overflow);
 * Exit and Move as in move_kernel.hpp L643 and L434; Death and ChangeWeight
 * stay 0 (the cycle never sets them).  The exporter writes them as
 * records/tallies and clears them at every export (host_export_handler.cpp
 * L118-L122). */
#define BMC_EVENT_NEW_PARTICLE 0
#define BMC_EVENT_EXIT 1
#define BMC_EVENT_MOVE 2
#define BMC_EVENT_DEATH 3
#define BMC_EVENT_OVERFLOW 4
#define BMC_EVENT_CHANGE_WEIGHT 5
#define BMC_N_EVENTS 6
/* Copies the tallies into counts[BMC_N_EVENTS]; clear != 0 then sets them
 * to 0 (EventContainer::get_span, clear). */
int bmc_read_events(bmc_scenario* s, uint64_t* counts, int32_t clear);

/* ---- time-event probes ---------------------------------------------------- */
/* The reference's Simulation::Probes (apps/libs/simulation/public/simulation/
 * probe.hpp L38-L146), which its cycle fills when built with use_probe
 * (off in its default build): with capacity > 0 every step of the scenario
 * records, in double,
 *   BMC_PROBE_LEAVING_TIME: ages(i, 0) of each particle leaving through an
 *     outlet, before its reset (ProbeType::LeavingTime, move_kernel.hpp
 *     L629-L635), in the order the device's threads reach the exit, as the
 *     reference's atomic counter orders them;
 *   BMC_PROBE_DIVISION_TIME: ages(i, 1) of each particle whose update asks to
 *     divide, before the division is attempted, refused or not
 *     (ProbeType::DivisionTime, model_kernel.hpp L245-L251), in slot order
 *     within a step;
 * each into its own buffer of `capacity` values on the device.  Events after
 * a full buffer are counted but not stored (Probes::set), so once a leaving
 * buffer has filled, which values it kept can differ between runs.
 * bmc_probe_enable(s, 0) turns them off (the default); enabling empties both
 * buffers.  Graph runs and batches record too. */
#define BMC_PROBE_LEAVING_TIME 0
#define BMC_PROBE_DIVISION_TIME 1
int bmc_probe_enable(bmc_scenario* s, uint64_t capacity);
/* Probes::get and need_export: writes the number of events counted since
 * the probe was last emptied to *count, and copies the stored values
 * (min(capacity, count) of them, at most max_values) into out.  The buffer
 * needs exporting once *count >= capacity. */
int bmc_probe_read(bmc_scenario* s, int32_t probe, double* out, uint64_t max_values, uint64_t* count);
/* Probes::clear: the probe's count and values back to 0 (the exporter's
 * save_probes, apps/core/src/post_process.cpp L30-L46, clears after each
 * write). */
int bmc_probe_clear(bmc_scenario* s, int32_t probe);

/* ---- flow-map cycle ------------------------------------------------------- */
/* Several flow-map states of the same mesh (the reference's CMA case with
 * n_different_maps > 1, replayed by its FlowMapTransitionner): each map
 * carries its own volumes, neighbours, out-flows, cumulative probabilities
 * and liquid transition (arguments as bmc_domain_update and
 * bmc_set_transition_coo; n_compartments and K are the domain's).  All maps
 * stay on the device; main-loop step k runs on map (k / n_per_flowmap) %
 * n_maps, switched in on the device at the start of the step (the
 * UPDATE_HYDRO_STEP of apps/core/src/host_specific.cpp L255-L266, which
 * replaces volumes, neighbours, out-flows, probabilities and transition,
 * apps/libs/simulation/src/simulation.cpp L95-L139; concentrations follow
 * from the unchanged masses).  n_per_flowmap = floor(t_per_flowmap / dt) + 1,
 * or 1 when t_per_flowmap is 0 or there is one map (compute_n_per_flowmap,
 * apps/core/src/global_initaliser.cpp L104-L114).  While maps are set,
 * bmc_domain_update and bmc_set_transition_coo are refused; bmc_cycle
 * (cycle only) does not switch maps. */
int bmc_flowmap_add(bmc_scenario* s, const double* volume, const uint64_t* neighbors,
                    const double* out_flows, const double* cdf, uint64_t nnz, const uint64_t* rows,
                    const uint64_t* cols, const double* values);
int bmc_flowmap_period(bmc_scenario* s, double t_per_flowmap);
/* The gas state of flow map `map` (two-phase cases: the gas volumes and gas
 * transition in COO form, as bmc_gas_set, and the kla [n_c][n_s] of that
 * state, e.g. from bmc_mtr_turbulence_kla on its volumes; NULL keeps
 * bmc_gas_set's).  Once every flow map has one, each switch also replaces
 * the gas domain and kla, keeping the gas masses, as SimulationUnit::
 * updateScalarHydro and MassTransferModel::update do (apps/libs/simulation/
 * src/simulation.cpp L120-L139); until then the gas domain stays fixed.
 * bmc_gas_set drops the maps' gas states. */
int bmc_flowmap_add_gas(bmc_scenario* s, uint32_t map, const double* gas_volume, uint64_t nnz, const uint64_t* rows,
                        const uint64_t* cols, const double* values, const double* kla);
int bmc_flowmap_clear(bmc_scenario* s);

/* ---- CMA ingestion (host only) ------------------------------------------- */
/* Derivations of CmaUtils from a flow map F(i, j) (m^3/s, i -> j) in COO
 * form over n_c compartments (documentation/pages/03_cma.md, "Transition
 * Matrix" and "Cumulative probability"; the reference computes them in
 * rcmtool, which is outside its tree).  Self-flows F(i, i) and zero flows
 * are dropped, duplicate (i, j) entries summed; flows must be finite, >= 0.
 *
 * bmc_cma_derive: *K = the largest out-degree (at least 1).  With the three
 * arrays non-NULL (rows of K entries, k_cap >= K) it writes the arguments of
 * bmc_domain_update: neighbours [n_c*K] in ascending destination order,
 * padded with the last destination (the compartment itself when it has
 * none), out-flows [n_c] = sum_j F(i, j) summed in that order
 * (get_diag_transition), cumulative probabilities [n_c*K] = running sum /
 * out-flow (exactly 1 at the last destination and in the padding).
 *
 * bmc_cma_transition: *t_nnz = entry count; with the arrays non-NULL (cap >=
 * count) the liquid transition T(i, j) = F(i, j), T(i, i) = -out-flow(i)
 * (get_transition_matrix), sorted by (row, col): the arguments of
 * bmc_set_transition_coo.  Known answers:
 * apps/libs/cma_utils/tests/test_transition_matrix.cpp L7-L25. */
int bmc_cma_derive(uint32_t n_c, uint64_t nnz, const uint64_t* rows, const uint64_t* cols, const double* flows,
                   uint32_t* K, uint32_t k_cap, uint64_t* neighbors, double* out_flows, double* cdf);
int bmc_cma_transition(uint32_t n_c, uint64_t nnz, const uint64_t* rows, const uint64_t* cols,
                       const double* flows, uint64_t* t_nnz, uint64_t cap, uint64_t* t_rows, uint64_t* t_cols,
                       double* t_values);

/* kla (1/s) of the transferred species (O2) per compartment under the
 * reference's FlowmapTurbulence mass-transfer model
 * (MassTransfer::Impl::flowmap_gas_liquid_mass_transfer,
 * apps/libs/simulation/src/hydro/impl_mtr.cpp L100-L145, computed there at
 * every hydro-state update, simulation.cpp L132-L138):
 *   kla_j = 0.3 (eps_j nu)^(1/4) Sc^(-1/2) * 6 alpha_j / (db (1 - alpha_j)),
 * alpha_j = Vg_j / (Vl_j + Vg_j) the gas fraction, nu the kinematic
 * viscosity of water at 20 C (1.0023e-6 m^2/s from the reference's fit),
 * Sc = nu / 1e-9 (oxygen diffusivity, m^2/s), eps the turbulent energy
 * dissipation of the case (W/kg), db the bubble diameter (the reference's
 * MassTransferModel sets 5e-3 m).  The result is the O2 column of the kla
 * of bmc_gas_set (the model leaves the other species at 0; its Henry
 * constant for O2 is 3.181e-2).  Host only. */
int bmc_mtr_turbulence_kla(uint32_t n_c, const double* energy_dissipation, const double* liquid_volume,
                           const double* gas_volume, double bubble_diameter, double* kla);

/* Time step of a run (get_time_step, apps/core/src/global_initaliser.cpp
 * L51-L86, with CmaUtils::get_min_residence_time,
 * apps/libs/cma_utils/src/utils.cpp L47-L73): user_dt when > 0, else
 * min over the n_maps flow maps and their compartments of positive volume of
 * out_flow / volume, divided by 100.  volumes and out_flows: [n_maps*n_c].
 * BMC_E_INVALID when no compartment gives a positive value. */
int bmc_cma_time_step(double user_dt, uint32_t n_maps, uint32_t n_c, const double* volumes,
                      const double* out_flows, double* dt);

/* Field file of a CMA case (vofL.raw, turbE.raw, ...): a little-endian
 * uint32 count followed by that many little-endian float64 values (the
 * layout of the fixture apps/api/tests/data/0d/).  *n = count; values are
 * written when values is non-NULL and cap >= count. */
int bmc_cma_read_field(const char* path, uint64_t cap, double* values, uint64_t* n);

/* Case descriptor of a CMA case (the `cma_case` file of a case folder; the
 * reference hands its path to rcmtool v1.4, a crate outside its tree,
 * through get_dtransitioner, apps/core/src/global_initaliser.cpp L201-L243).
 * Layout read as the reference's one fixture holds it
 * (apps/api/tests/data/0d/cma_case, 63 bytes): four little-endian uint32
 * words, one float64, a uint64 entry count, then per entry a uint8 kind, a
 * uint32 byte length and the path of a file of the case, relative to the
 * case folder, without terminator.  Kinds in the fixture: 3 = liquid volumes
 * (./vofL.raw), 0 = liquid flow map (./flowL.raw).  The words and the float
 * are returned as stored (the fixture holds 1, 1, 1, 0 and 0.0); their
 * meaning, and the layout of cases with more compartments, are not pinned
 * by any file of the reference.  A file whose size does not match this
 * layout is refused (BMC_E_INVALID).
 * bmc_cma_read_case: words[4] (may be NULL), *t0 (may be NULL), *n_entries.
 * bmc_cma_case_entry: entry `index`: *kind and, when name is non-NULL, its
 * path NUL-terminated into name (name_cap >= path length + 1). */
int bmc_cma_read_case(const char* path, uint32_t* words, double* t0, uint32_t* n_entries);
int bmc_cma_case_entry(const char* path, uint32_t index, uint32_t* kind, char* name, uint64_t name_cap);

/* Liquid flow map file of a CMA case (flowL.raw): uint32 rows, uint32
 * columns, then the flows F(i, j) in COO form as three arrays, each a
 * uint64 length followed by its elements: row indices (uint64), column
 * indices (uint64), flows (float64, m^3/s).  The reference's fixture
 * (apps/api/tests/data/0d/flowL.raw, 32 bytes: a 1 x 1 map, three empty
 * arrays) fits this reading; it fits "uint32 n, uint32 entry count, then
 * (uint64 row, uint64 column, float64 flow) triplets" as well (one zero
 * self-flow, which gives the same domain), so the layout of larger maps is
 * not pinned.  Refused (BMC_E_INVALID): sizes that do not add up, arrays of
 * different lengths, entries outside the rows and columns.  *nnz = entry
 * count; with the three arrays non-NULL (cap >= count) the entries.  The
 * result feeds bmc_cma_derive / bmc_cma_transition. */
int bmc_cma_read_flowmap(const char* path, uint32_t* n_rows, uint32_t* n_cols, uint64_t* nnz, uint64_t cap,
                         uint64_t* rows, uint64_t* cols, double* flows);

/* ---- two-phase flow: gas phase ------------------------------------------- */
/* A gas phase on the scenario's mesh (SimulationUnit with
 * is_two_phase_flow; apps/libs/simulation/src/simulation.cpp L47-L81):
 * gas volumes [n_c], the gas transition in COO form (as
 * bmc_set_transition_coo), Henry constants [n_species] and the transfer
 * coefficients kla [n_c][n_species] (1/s; the reference's FixedKla gives one
 * value per species, its FlowmapTurbulence correlation one per compartment,
 * hydro/impl_mtr.cpp L92-L148).  Each main-loop step then computes, from the
 * step's old concentrations, mtr(j,s) = kla (H Cg - C) V_liquid
 * (fixed_kla_gas_liquid_mass_transfer, impl_mtr.cpp L150-L166), advances
 * the gas with -mtr and the liquid with +mtr (ScalarSimulation::
 * performStepGL, implScalar.cpp L229-L249; SimulationUnit::ode_step,
 * simulation.model.cpp L132-L150) and clears tiny negative liquid
 * concentrations (clearNegs, implScalar.cpp L266-L293).  Particles see the
 * liquid only.  The gas domain stays fixed while flow maps cycle, unless
 * every map has a gas state (bmc_flowmap_add_gas). */
int bmc_gas_set(bmc_scenario* s, const double* gas_volume, uint64_t nnz, const uint64_t* rows,
                const uint64_t* cols, const double* values, const double* henry, const double* kla);
int bmc_gas_set_concentrations(bmc_scenario* s, const double* conc);
/* Gas feeds (update_feed's gas_feeds, simulation.model.cpp L112-L119):
 * inlet sources flow x conc, outlet sinks; no particle exit. */
int bmc_gas_set_feeds(bmc_scenario* s, uint32_t n_feeds, const bmc_feed* feeds);
/* Gas concentrations, masses and the last step's transfer to the liquid
 * (kg/s), each [n_c][n_species] (NULL skips). */
int bmc_gas_read(bmc_scenario* s, double* conc, double* mass, double* transfer);

/* ---- batching: many scenarios advanced by one set of launches ----------- */
/* All scenarios of a batch share model and precision; each keeps its own
 * domain, liquid state, parameters, seed and step counter. */
int bmc_batch_create(bmc_scenario* const* scenarios, uint32_t n, bmc_batch** out);
/* A batch of `capacity` slots for one model and precision, all empty; a
 * serving loop fills and empties slots (bmc_batch_set_slot, NULL empties)
 * between runs without rebuilding the batch or its captured step: empty
 * slots are skipped by every kernel.  Setting a slot waits for the batch's
 * queued steps and for the scenario's own stream. */
int bmc_batch_create_slots(uint32_t capacity, int32_t model, int32_t f64, bmc_batch** out);
int bmc_batch_set_slot(bmc_batch* b, uint32_t slot, bmc_scenario* s);
int bmc_batch_destroy(bmc_batch* b);
/* Advance every scenario of the batch by n_steps (captured graph). */
int bmc_batch_run(bmc_batch* b, double dt, uint32_t n_steps);
/* Kernel shape of the batch, as bmc_set_shape (a new batch starts in the
 * automatic shape).  Used by the autotuner. */
int bmc_batch_set_shape(bmc_batch* b, uint32_t threads, uint32_t ppt, uint32_t blocks_per_sm);
int bmc_batch_synchronize(bmc_batch* b);

/* ---- runtime-loaded cell models ("udf_model") ----------------------------- */
/* A user model is a CUDA source file that defines a model struct and
 * expands BMC_DEFINE_UDF (biocma-mcst_gb300/csrc/bmc_udf.cuh); compiled with
 * nvcc into a shared library (bmc/udf.py build_udf), it carries the cycle's
 * kernels instantiated for that model.  bmc_udf_load opens it and returns
 * the model id (>= BMC_MODEL_UDF_FIRST) to put in bmc_model_desc.model.
 * Reference: UnsafeUDF::Loader::init_lib (apps/libs/models/ext/
 * udf_includes.cpp L58-L78) with the module symbols of udf_includes.hpp
 * L111-L122; path == NULL reads the library path from BIOMC_LIB_UDF as
 * Unsafe::load_udf does (apps/api/src/udf_handle.cpp L22-L38).  Loading the
 * same path again returns the same id; libraries stay loaded until exit. */
#define BMC_MODEL_UDF_FIRST 64
int bmc_udf_load(const char* path, int32_t* model_id);

/* Metadata of a loaded model: set_nvar_udf / set_nc_udf / names_udf /
 * species_udf of the reference's module (udf_includes.hpp L29-L65). */
typedef struct bmc_udf_info {
  uint32_t n_var;
  uint32_t n_ctb;
  int32_t separable;
  int32_t has_f32;    /* compiled for float state */
  int32_t has_f64;    /* compiled for double state */
  uint32_t n_names;   /* entries of names (state variables) */
  uint32_t n_species; /* entries of species */
  uint32_t pad;
  const char* names[16];  /* owned by the library */
  const char* species[8];
} bmc_udf_info;
int bmc_udf_get_info(int32_t model_id, bmc_udf_info* info);

/* Host (CPU) entry points of a loaded model, compiled from the same source
 * as its kernels, for CPU callers (initial conditions, post-processing,
 * reference computations).  x, child and r point to the model's float type
 * (float or double per f64); rates(c, params, r) fills the compartment
 * factors from one compartment's concentrations; update advances one
 * particle and writes its contribution basis (separable models) or its
 * n_ctb contributions (general models) to out; coef(r, j) is the
 * contribution of species j per unit basis. */
typedef struct bmc_udf_host_model {
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
  /* Models that update with their context (uses_context in the model
   * source): update_ctx replaces update, with the particle's four draws of
   * the step, its compartment's n_species concentrations c and the
   * compartment index; NULL for the other models. */
  int32_t (*update_ctx)(double dt, void* x, const void* r, void* out, const double* params, const float* draws,
                        const double* c, uint32_t position, uint32_t n_species);
} bmc_udf_host_model;
int bmc_udf_get_host_model(int32_t model_id, int32_t f64, bmc_udf_host_model* out);

/* ---- diagnostics ---------------------------------------------------------- */
/* Fill out[4*n] with the four uniform draws of (seed, id[k], step, purpose)
 * computed on the device (checks the draw source against the oracle). */
int bmc_debug_draws(uint64_t seed, const uint32_t* ids, uint64_t n, uint32_t step,
                    uint32_t purpose, float* out);
/* The cycle kernels' age step on n ages >= 0 computed on the device:
 * out[k] = (float)((double)ages[k] + dt), the reference's `ages(i, 0) +=
 * d_t` with float ages and a double time step (move_kernel.hpp L356),
 * evaluated by the kernels with float and integer operations. */
int bmc_debug_age_add(const float* ages, uint64_t n, double dt, float* out);
/* The cycle kernels' quantisation of float contribution values to the
 * accumulators' fixed point (the nearest multiple of 2^e, ties to even,
 * clamped to 2^42 quanta) on n values: out[2k] by the scaled conversion the
 * kernels use, out[2k + 1] from the IEEE fields (the form used when 2^-e is
 * not a float of at most 2^125). */
int bmc_debug_quantize(const float* values, uint64_t n, int32_t e, int64_t* out);
/* Self-test of the bounded barrier wait of the cycle kernels: one thread
 * waits on an mbarrier whose single arrival it makes first (arrive != 0) or
 * that nothing makes; in the second case the wait gives up after limit_ns
 * (at most 2 s) and *error_word = BMC_ERR_TIMEOUT, the bit a cycle kernel
 * sets in the step's error word when a tile copy never lands.  *waited_ns:
 * device time spent in the wait. */
int bmc_debug_wait(uint64_t limit_ns, int32_t arrive, uint32_t* error_word, uint64_t* waited_ns);
/* One main-loop iteration like bmc_step, with CUDA events recorded on the
 * scenario's stream between its six kernels; kernel_ms[0..5] receive the
 * durations of: liquid step, cycle, plan, divide, compact, merge.
 * Reference counterpart: the Kokkos-tools region timers of the cycle
 * (tools/benchs/benchmark.py L145-L229). */
int bmc_step_timed(bmc_scenario* s, double dt, bmc_step_stats* stats, float* kernel_ms);

/* One batched step like bmc_batch_run(b, dt, 1), launched without a graph
 * with CUDA events between the six kernels (kernel_ms as in
 * bmc_step_timed); waits for the step. */
int bmc_batch_step_timed(bmc_batch* b, double dt, float* kernel_ms);

/* bmc_run with CUDA events recorded on the scenario's stream before the
 * first and after the last step; *elapsed_ms receives the device time. */
int bmc_run_timed(bmc_scenario* s, double dt, uint32_t n_steps, bmc_step_stats* stats, float* elapsed_ms);

/* Select the CUDA device used by scenarios created afterwards on this host
 * thread (one process per GPU). */
int bmc_set_device(int32_t device);

/* Bytes the library has copied host->device and device->host so far. */
int bmc_transfer_bytes(uint64_t* h2d, uint64_t* d2h);

/* Number of kernels this library has launched so far (all scenarios). */
int bmc_launch_count(uint64_t* count);

#ifdef __cplusplus
}
#endif
#endif

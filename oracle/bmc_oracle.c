/*
 * bmc_oracle.c -- CPU restatement of the BioCMA-MCST Monte Carlo cycle.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  The product never links this file.
 * Reference citations for every function are in bmc_oracle.h and beside each
 * function below.  Compile with -ffp-contract=off: the GPU path is compiled
 * without multiply-add contraction, so both sides round every operation the
 * same way and integer outcomes (positions, statuses, counts) match bit for
 * bit.
 */
#include "bmc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Draw source.  The reference draws from Kokkos::Random_XorShift1024_Pool
 * (apps/libs/mc/public/mc/alias.hpp L98), which cannot be replayed outside
 * Kokkos.  Both this oracle and the GPU path use Philox4x32-10 (Salmon et al.,
 * SC'11, "Parallel random numbers: as easy as 1, 2, 3") with counter
 * (particle id, seed low word, step, seed high word) and key (purpose, 0):
 * one stream per (seed, particle, step, purpose). */

static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
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

/* Uniform float on the open interval (0,1): an odd 24-bit integer times
 * 2^-24, exactly representable, never 0 or 1. */
float orc_u01(uint32_t x) { return (float)((x >> 8) | 1u) * 0x1p-24f; }

/* The four raw 32-bit words of the stream (seed, id, step, purpose). */
static void draws_raw(uint64_t seed, uint32_t id, uint32_t step, uint32_t purpose, uint32_t r[4]) {
  uint32_t ctr[4] = {id, (uint32_t)seed, step, (uint32_t)(seed >> 32)};
  uint32_t key[2] = {purpose, 0u};
  orc_philox4x32_10(ctr, key, r);
}

void orc_draws(uint64_t seed, uint32_t id, uint32_t step, uint32_t purpose, float out[4]) {
  uint32_t r[4];
  draws_raw(seed, id, step, purpose, r);
  for (int k = 0; k < 4; ++k) out[k] = orc_u01(r[k]);
}

/* Independent stream for the free-running statistical comparison: a
 * splitmix64-seeded xorshift64* generator per (particle id, step), so that
 * the oracle does not share a single draw with the GPU path. */
static void xorshift_draws(uint64_t seed, uint32_t id, uint32_t step, uint32_t purpose, float out[4]) {
  uint64_t z = seed ^ ((uint64_t)id << 20) ^ ((uint64_t)step << 42) ^ ((uint64_t)purpose << 60);
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  if (z == 0) z = 0x2545F4914F6CDD1Dull;
  for (int k = 0; k < 4; ++k) {
    z ^= z >> 12;
    z ^= z << 25;
    z ^= z >> 27;
    uint64_t v = z * 0x2545F4914F6CDD1Dull;
    out[k] = orc_u01((uint32_t)(v >> 32));
  }
}

static inline void draws_for(const orc_state* s, uint32_t id, uint32_t purpose, float out[4]) {
  if (s->draw_mode == ORC_DRAW_XORSHIFT)
    xorshift_draws(s->seed, id, s->step, purpose, out);
  else
    orc_draws(s->seed, id, s->step, purpose, out);
}


/* ------------------------------------------------------------------------ */
/* Exact contribution sums.  v is rounded to the nearest multiple of 2^e
 * (ties to even), clamped to |q| <= qmax.  Integer sums are independent of
 * summation order, so every parallel decomposition gives the same total. */
int64_t orc_quantize(double v, int32_t e, int64_t qmax, int* clamped) {
  double x = rint(ldexp(v, -e));
  if (x > (double)qmax) {
    *clamped = 1;
    return qmax;
  }
  if (x < -(double)qmax) {
    *clamped = 1;
    return -qmax;
  }
  return (int64_t)x;
}

/* Total t (an integer number of quanta) to double, rounded once:
 * t = hi * 2^32 + lo with 0 <= lo < 2^32; hi*2^32 and lo are exact doubles
 * while |t| < 2^85, so the single addition is the only rounding. */
double orc_fixed_to_double(__int128 t, int32_t e) {
  const __int128 lo = t & (__int128)0xFFFFFFFFu;
  const __int128 hi = (t - lo) / ((__int128)1 << 32);
  const double d = (double)(int64_t)hi * 0x1p32 + (double)(uint64_t)lo;
  return ldexp(d, e);
}

/* ------------------------------------------------------------------------ */
/* Models, restated per the ModelType concept
 * (apps/libs/mc/public/mc/traits.hpp L67-L133): update returns Idle or
 * Division and writes the particle's contributions; division splits a mother
 * into mother + child.  Each model is instantiated for double and float. */

#define ORC_F double
#define ORC_SFX _f64
#include "bmc_oracle_models.inc"
#undef ORC_F
#undef ORC_SFX
#define ORC_F float
#define ORC_SFX _f32
#include "bmc_oracle_models.inc"
#undef ORC_F
#undef ORC_SFX

static int is_fixed_length(const orc_state* s) {
  return s->model == ORC_MODEL_FIXED_LENGTH || s->model == ORC_MODEL_FIXED_LENGTH_GENERAL;
}

/* Rates of compartment c into r[8] (element type of the model's float). */
static void model_rates(const orc_state* s, const double* c, void* r) {
  if (s->udf) {
    s->udf->rates(c, s->params, r);
    return;
  }
  if (s->f64) {
    double* rr = (double*)r;
    if (s->model == ORC_MODEL_MONOD) monod_rates_f64(c, s->params, rr);
    if (s->model == ORC_MODEL_OVERFLOW) overflow_rates_f64(c, s->params, rr);
  } else {
    float* rr = (float*)r;
    if (s->model == ORC_MODEL_MONOD) monod_rates_f32(c, s->params, rr);
    if (s->model == ORC_MODEL_OVERFLOW) overflow_rates_f32(c, s->params, rr);
    if (is_fixed_length(s)) fixed_length_rates(c, s->params, rr);
    if (s->model == ORC_MODEL_SIMPLE_ACETATE) simple_acetate_rates(c, s->params, rr);
  }
}

/* Contribution coefficient j of a compartment (as double). */
static double model_coef(const orc_state* s, const void* r, int j) {
  if (s->udf) return s->udf->coef(r, j);
  if (s->f64) {
    const double* rr = (const double*)r;
    if (s->model == ORC_MODEL_MONOD) return monod_coef_f64(rr, j);
    return overflow_coef_f64(rr, j);
  }
  const float* rr = (const float*)r;
  if (s->model == ORC_MODEL_MONOD) return (double)monod_coef_f32(rr, j);
  if (s->model == ORC_MODEL_OVERFLOW) return (double)overflow_coef_f32(rr, j);
  return (double)fixed_length_coef(rr, j);
}

/* Per-particle update.  Separable models return their basis (as double,
 * with *basis_is_float set when it is a float); the general FixedLength
 * writes its contribution w-free into ctb[0]. */
static int model_update(const orc_state* s, double dt, uint64_t i, const void* r, double* basis, double* ctb) {
  const uint64_t cap = s->phys_capacity;
  float ctx_draws[4];
  const double* ctx_c = NULL;
  if (s->udf && s->udf->update_ctx) {
    /* the reference's update(random_pool, d_t, idx, arr, contribs, position,
     * c): the particle's draws of the step and its compartment's
     * concentrations */
    draws_for(s, s->id[i], 3u, ctx_draws);
    ctx_c = s->C + (uint64_t)s->pos[i] * s->n_s;
  }
  if (s->udf && s->f64) {
    double* st = (double*)s->state;
    double x[16], out[16] = {0};
    for (uint32_t v = 0; v < s->n_var; ++v) x[v] = st[v * cap + i];
    const int res = ctx_c ? s->udf->update_ctx(dt, x, r, out, s->params, ctx_draws, ctx_c, s->pos[i], s->n_s)
                          : s->udf->update(dt, x, r, out, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) st[v * cap + i] = x[v];
    *basis = out[0];
    for (uint32_t j = 0; j < s->n_ctb; ++j) ctb[j] = out[j];
    return res;
  }
  if (s->udf) {
    float* st = (float*)s->state;
    float x[16], out[16] = {0};
    for (uint32_t v = 0; v < s->n_var; ++v) x[v] = st[v * cap + i];
    const int res = ctx_c ? s->udf->update_ctx((double)(float)dt, x, r, out, s->params, ctx_draws, ctx_c, s->pos[i],
                                               s->n_s)
                          : s->udf->update((double)(float)dt, x, r, out, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) st[v * cap + i] = x[v];
    *basis = (double)out[0];
    for (uint32_t j = 0; j < s->n_ctb; ++j) ctb[j] = (double)out[j];
    return res;
  }
  if (s->f64) {
    double* st = (double*)s->state;
    double x[16];
    for (uint32_t v = 0; v < s->n_var; ++v) x[v] = st[v * cap + i];
    double b = 0.0;
    int res = ORC_IDLE;
    if (s->model == ORC_MODEL_MONOD) res = monod_update_f64(dt, x, (const double*)r, &b, s->params);
    if (s->model == ORC_MODEL_OVERFLOW) res = overflow_update_f64(dt, x, (const double*)r, &b, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) st[v * cap + i] = x[v];
    *basis = b;
    return res;
  } else {
    float* st = (float*)s->state;
    float x[16];
    for (uint32_t v = 0; v < s->n_var; ++v) x[v] = st[v * cap + i];
    float b = 0.0f, cf[16] = {0};
    int res = ORC_IDLE;
    const float* rr = (const float*)r;
    const float dtf = (float)dt;
    if (s->model == ORC_MODEL_MONOD) res = monod_update_f32(dtf, x, rr, &b, s->params);
    if (s->model == ORC_MODEL_OVERFLOW) res = overflow_update_f32(dtf, x, rr, &b, s->params);
    if (s->model == ORC_MODEL_FIXED_LENGTH) res = fixed_length_update(dtf, x, rr, &b, s->params);
    if (s->model == ORC_MODEL_FIXED_LENGTH_GENERAL) res = fixed_length_update_general(dtf, x, rr, cf, s->params);
    if (s->model == ORC_MODEL_SIMPLE_ACETATE) res = simple_acetate_update_general(dtf, x, rr, cf, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) st[v * cap + i] = x[v];
    *basis = (double)b;
    for (uint32_t j = 0; j < s->n_ctb; ++j) ctb[j] = (double)cf[j];
    return res;
  }
}

static void model_division(const orc_state* s, uint64_t i, uint64_t child_slot) {
  const uint64_t cap = s->phys_capacity;
  float d[4];
  draws_for(s, s->id[i], 1u, d);
  if (s->udf) {
    const size_t fs = s->f64 ? sizeof(double) : sizeof(float);
    char* st = (char*)s->state;
    char* ch = (char*)s->child_state;
    double xb[16], yb[16]; /* storage for up to 16 values of either type */
    memset(yb, 0, sizeof(yb));
    for (uint32_t v = 0; v < s->n_var; ++v) memcpy((char*)xb + v * fs, st + (v * cap + i) * fs, fs);
    s->udf->division(xb, yb, d, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) {
      memcpy(st + (v * cap + i) * fs, (char*)xb + v * fs, fs);
      memcpy(ch + (v * cap + child_slot) * fs, (char*)yb + v * fs, fs);
    }
    return;
  }
  if (s->f64) {
    double* st = (double*)s->state;
    double* ch = (double*)s->child_state;
    double x[16], y[16] = {0};
    for (uint32_t v = 0; v < s->n_var; ++v) x[v] = st[v * cap + i];
    if (s->model == ORC_MODEL_MONOD) monod_division_f64(x, y, d, s->params);
    if (s->model == ORC_MODEL_OVERFLOW) overflow_division_f64(x, y, d, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) {
      st[v * cap + i] = x[v];
      ch[v * cap + child_slot] = y[v];
    }
  } else {
    float* st = (float*)s->state;
    float* ch = (float*)s->child_state;
    float x[16], y[16] = {0};
    for (uint32_t v = 0; v < s->n_var; ++v) x[v] = st[v * cap + i];
    if (s->model == ORC_MODEL_MONOD) monod_division_f32(x, y, d, s->params);
    if (s->model == ORC_MODEL_OVERFLOW) overflow_division_f32(x, y, d, s->params);
    if (is_fixed_length(s)) fixed_length_division(x, y, d, s->params);
    if (s->model == ORC_MODEL_SIMPLE_ACETATE) simple_acetate_division(x, y, d, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) {
      st[v * cap + i] = x[v];
      ch[v * cap + child_slot] = y[v];
    }
  }
}

static void model_init(const orc_state* s, uint64_t i, const float* d) {
  const uint64_t cap = s->phys_capacity;
  if (s->udf) {
    const size_t fs = s->f64 ? sizeof(double) : sizeof(float);
    double xb[16];
    memset(xb, 0, sizeof(xb));
    s->udf->init(xb, d, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) memcpy((char*)s->state + (v * cap + i) * fs, (char*)xb + v * fs, fs);
    return;
  }
  if (s->f64) {
    double* st = (double*)s->state;
    double x[16] = {0};
    if (s->model == ORC_MODEL_MONOD) monod_init_f64(x, d, s->params);
    if (s->model == ORC_MODEL_OVERFLOW) overflow_init_f64(x, d, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) st[v * cap + i] = x[v];
  } else {
    float* st = (float*)s->state;
    float x[16] = {0};
    if (s->model == ORC_MODEL_MONOD) monod_init_f32(x, d, s->params);
    if (s->model == ORC_MODEL_OVERFLOW) overflow_init_f32(x, d, s->params);
    if (is_fixed_length(s)) fixed_length_init(x, d, s->params);
    if (s->model == ORC_MODEL_SIMPLE_ACETATE) simple_acetate_init(x, d, s->params);
    for (uint32_t v = 0; v < s->n_var; ++v) st[v * cap + i] = x[v];
  }
}

static double model_mass(const orc_state* s, uint64_t i) {
  if (s->udf) {
    const uint64_t cap = s->phys_capacity;
    const size_t fs = s->f64 ? sizeof(double) : sizeof(float);
    double xb[16];
    for (uint32_t v = 0; v < s->n_var; ++v) memcpy((char*)xb + v * fs, (const char*)s->state + (v * cap + i) * fs, fs);
    return s->udf->mass(xb, s->params);
  }
  if (s->f64) return ((const double*)s->state)[i];
  if (is_fixed_length(s)) return (double)(((const float*)s->state)[i] * fixed_length_lin_density());
  if (s->model == ORC_MODEL_SIMPLE_ACETATE) return (double)(((const float*)s->state)[i] * sa_lin_density());
  return (double)((const float*)s->state)[i];
}

/* The SimpleAcetate draw functions, exported for their accuracy tests. */
double orc_sa_log(double x) { return sa_log(x); }
double orc_sa_exp(double x) { return sa_exp(x); }
double orc_sa_erfinv(double x) { return sa_erfinv_d(x); }
float orc_sa_truncnorm(float u, float mu, float sd, float pl, float pu) { return sa_truncnorm_f(u, mu, sd, pl, pu); }

/* ------------------------------------------------------------------------ */
/* Initialisation: apps/libs/mc/src/unit.cpp L102-L163 (InitFunctor: model
 * init, position = uniform integer in [min_c, max_c), mass reduction). */
void orc_init_particles(orc_state* s, uint64_t n, uint32_t pos_lo, uint32_t pos_hi) {
  const uint32_t span = pos_hi - pos_lo;
  for (uint64_t i = 0; i < n; ++i) {
    float d[4];
    const uint32_t pid = (uint32_t)i;
    /* step word 0xFFFFFFFF: no main-loop step draws with it */
    uint32_t r[4];
    draws_raw(s->seed, pid, 0xFFFFFFFFu, 2u, r);
    for (int k = 0; k < 4; ++k) d[k] = orc_u01(r[k]);
    model_init(s, i, d);
    s->pos[i] = pos_lo + (uint32_t)(((uint64_t)r[0] * (uint64_t)span) >> 32);
    s->status[i] = ORC_IDLE;
    s->age_h[i] = 0.0f;
    s->age_d[i] = 0.0f;
    s->id[i] = pid;
  }
  s->n_used = n;
  s->next_id = n;
  s->inactive = 0;
}

double orc_total_mass(const orc_state* s) {
  double m = 0.0;
  for (uint64_t i = 0; i < s->n_used; ++i)
    if (s->status[i] == ORC_IDLE) m += model_mass(s, i);
  return m;
}

/* Model::mass of every used slot (the mass column of the reference's
 * particle dump, apps/core/public/core/post_process.hpp L96-L98). */
void orc_particle_mass(const orc_state* s, double* out) {
  for (uint64_t i = 0; i < s->n_used; ++i) out[i] = model_mass(s, i);
}

/* ------------------------------------------------------------------------ */
/* Move: apps/libs/simulation/public/simulation/kernels/move_kernel.hpp
 * L62-L103.  First k with u <= CDF(c, k) over the K slots; the search is the
 * reference's branchless bisection (left=0, right=K-1). */
uint32_t orc_find_next(const orc_state* s, uint32_t c, double u) {
  const double* row = s->cdf + (uint64_t)c * s->K;
  int left = 0;
  int right = (int)s->K - 1;
  while (left < right) {
    const int mid = (left + right) >> 1;
    if (u > row[mid])
      left = mid + 1;
    else
      right = mid;
  }
  return s->neighbors[(uint64_t)c * s->K + (uint32_t)left];
}

/* Liquid step, apps/libs/simulation/src/implScalar.cpp L251-L264:
 *   M += dt * (C*T - C*sink + Src);  C = M * diag(1/V)
 * with T(i,j) = F(i->j) off the diagonal and T(j,j) = -sum_k F(j->k). */
void orc_scalar_step(orc_state* s, double dt) {
  const uint32_t ns = s->n_s;
  const uint64_t ne = (uint64_t)s->n_c * ns;
  if (s->gas) {
    /* transfer from the old concentrations, then the gas step with the
     * transfer lost (Sign::GasToLiquid); the liquid gains it below */
    for (uint32_t j = 0; j < s->n_c; ++j)
      for (uint32_t sp = 0; sp < ns; ++sp) {
        const uint64_t e = (uint64_t)j * ns + sp;
        s->mtr[e] = (s->kla[e] * (s->Cg[e] * s->henry[sp] - s->C[e])) * s->volume[j];
      }
    double* gsrc = (double*)calloc(ne ? ne : 1, sizeof(double));
    double* gsink = (double*)calloc(s->n_c, sizeof(double));
    for (uint32_t f = 0; f < s->n_gfeeds; ++f) {
      for (uint32_t sp = 0; sp < ns; ++sp)
        gsrc[(uint64_t)s->gfeed_in[f] * ns + sp] += s->gfeed_flow[f] * s->gfeed_conc[f * 8 + sp];
      if (s->gfeed_out[f] >= 0) gsink[s->gfeed_out[f]] += s->gfeed_flow[f];
    }
    for (uint32_t j = 0; j < s->n_c; ++j)
      for (uint32_t sp = 0; sp < ns; ++sp) {
        const uint64_t e = (uint64_t)j * ns + sp;
        double acc = 0.0;
        for (uint32_t q = s->g_in_ptr[j]; q < s->g_in_ptr[j + 1]; ++q)
          acc += s->Cg[(uint64_t)s->g_in_idx[q] * ns + sp] * s->g_in_flow[q];
        const double cg = s->Cg[e];
        acc += cg * (-s->g_out_flow[j]);
        const double dmdt = acc - cg * gsink[j] + gsrc[e] + (-1.0) * s->mtr[e];
        s->Mg[e] += dt * dmdt;
      }
    for (uint32_t j = 0; j < s->n_c; ++j)
      for (uint32_t sp = 0; sp < ns; ++sp) s->Cg[(uint64_t)j * ns + sp] = s->Mg[(uint64_t)j * ns + sp] * s->gvinv[j];
    free(gsrc);
    free(gsink);
  }
  for (uint32_t j = 0; j < s->n_c; ++j) {
    for (uint32_t sp = 0; sp < ns; ++sp) {
      double acc = 0.0;
      for (uint32_t e = s->in_ptr[j]; e < s->in_ptr[j + 1]; ++e)
        acc += s->C[(uint64_t)s->in_idx[e] * ns + sp] * s->in_flow[e];
      const double cj = s->C[(uint64_t)j * ns + sp];
      acc += cj * (-s->out_flow[j]);
      double dmdt = acc - cj * s->sink[j] + s->src[(uint64_t)j * ns + sp];
      if (s->gas) dmdt = dmdt + s->mtr[(uint64_t)j * ns + sp];
      s->M[(uint64_t)j * ns + sp] += dt * dmdt;
    }
  }
  const double tol = 1e-4 * 5e-3; /* clearNegs */
  for (uint32_t j = 0; j < s->n_c; ++j)
    for (uint32_t sp = 0; sp < ns; ++sp) {
      double c = s->M[(uint64_t)j * ns + sp] * s->vinv[j];
      if (s->gas && c < 0.0 && fabs(c) < tol) c = 0.0;
      s->C[(uint64_t)j * ns + sp] = c;
    }
}

/* ------------------------------------------------------------------------ */
/* Move of one Idle particle at compartment p, MoveFunctor::handle_move
 * (move_kernel.hpp L393-L437): leave iff probability_leaving<fast_tag>
 * (probability_leaving.hpp L35-L48), (dt * Q / V) > u1 with the float draw
 * compared in double, p_move = (dt * Q) / V given; then the bisection of
 * __find_next_compartment with u2. */
static inline uint32_t move_one(const orc_state* s, double p_move, uint32_t p, float u1, float u2, int* moved) {
  if (p_move > (double)u1) {
    *moved = 1;
    return orc_find_next(s, p, (double)u2);
  }
  *moved = 0;
  return p;
}

/* Exit test of probability_leaving<precision_tag> (probability_leaving.hpp
 * L18-L33): dt * F > -ln(u) * V with the logarithm of the float draw taken
 * in float (CommonMaths::_ln<true>, apps/libs/common/public/common/
 * maths.hpp L28-L34, i.e. Kokkos::log(float), the C library's logf on the
 * reference's host build) and the product in double. */
static inline int exit_test(double dt, double flow, double volume, float u) {
  return (dt * flow) > ((double)(-logf(u)) * volume);
}

/* TagLeave on one Idle particle at compartment p (move_kernel.hpp
 * L348-L359 and handle_exit L588-L648): age(0) += dt (float); the first
 * outlet whose index is p decides; with a non-zero flow the draw u is
 * tested, and on exit the status becomes Exit and age(0) is reset.
 * Returns 1 on exit. */
static inline int leave_one(const orc_state* s, double dt, float dtf, uint32_t p, uint8_t* status, float* age_h,
                            float u, float* age_at_exit) {
  (void)dtf;
  *age_h = (float)((double)*age_h + dt); /* ages(idx, 0) += d_t, d_t double */
  for (uint32_t o = 0; o < s->n_outlets; ++o) {
    if (s->outlet_index[o] == p) {
      if (s->outlet_flow[o] != 0.0 && exit_test(dt, s->outlet_flow[o], s->outlet_volume[o], u)) {
        *status = ORC_EXIT;
        if (age_at_exit) *age_at_exit = *age_h; /* the leaving-time probe's value */
        *age_h = 0.0f;
        return 1;
      }
      return 0;
    }
  }
  return 0;
}

/* Probes::set (probe.hpp L61-L79): the event is counted; its value is kept
 * while the buffer has room (returns 1 then). */
int orc_probe_set(orc_state* s, int k, double v) {
  const uint64_t j = s->probe_n[k]++;
  if (j < s->probe_cap) {
    s->probe_buf[k][j] = v;
    return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* One cycle over the container (reference CycleFunctors::launch_model then
 * launch_move, kernels.hpp L124-L224).  Per Idle particle:
 *   ages(i,1) += dt; status = Model::update(...)       model_kernel.hpp L193
 *   S(:, pos) += w * contribs                          contribution_kernel.hpp
 *   move: leave iff dt*Q/V > u1, next = CDF search(u2) move_kernel.hpp L393
 *   ages(i,0) += dt; exit iff dt*F > -ln(u3)*V          move_kernel.hpp L588
 * with the reference's own expressions (move_one, leave_one above).
 * Division requests are recorded here and carried out in slot order by
 * orc_post_cycle, which is where the reference's buffer order becomes
 * deterministic. */
void orc_cycle(orc_state* s, double dt, int n_threads) {
  const uint64_t n = s->n_used;
  const uint32_t ns = s->n_s;
  const uint32_t nctb = s->n_ctb;
  const uint32_t ncol = s->separable ? 1u : nctb;
  const int do_move = s->n_c > 1;
  const int do_leave = s->n_outlets > 0;
  const size_t rsz = s->f64 ? sizeof(double) : sizeof(float);
  /* the model's rates of every compartment, from the concentrations */
  char* rates = (char*)malloc((size_t)s->n_c * 8 * rsz);
  for (uint32_t c = 0; c < s->n_c; ++c) model_rates(s, s->C + (uint64_t)c * ns, rates + (size_t)c * 8 * rsz);
  double pmove_small[1];
  double* pmove = s->n_c > 1 ? (double*)malloc(sizeof(double) * s->n_c) : pmove_small;
  for (uint32_t c = 0; c < s->n_c && do_move; ++c) pmove[c] = (dt * s->out_flow[c]) / s->volume[c];
  const float dtf = (float)dt;

  /* Optional emulation of the reference's Tag3D contribution loop
   * (contribution_kernel.hpp L167-L185): a team thread walks 32 consecutive
   * particles and returns at the first non-Idle one, so the Idle particles
   * after it in that chunk do not contribute.  Off by default; used only to
   * quantify the deviation of the intended semantics from the shipped one. */
  uint8_t* contrib_ok = NULL;
  if (s->quirk_tag3d) {
    contrib_ok = (uint8_t*)malloc(n ? n : 1);
    for (uint64_t c0 = 0; c0 < n; c0 += 32) {
      int alive = 1;
      for (uint64_t i = c0; i < c0 + 32 && i < n; ++i) {
        if (s->status[i] != ORC_IDLE) alive = 0;
        contrib_ok[i] = (uint8_t)alive;
      }
    }
  }
  uint64_t moves = 0, exits = 0, reqdiv = 0;
  const size_t acc_len = (size_t)s->n_c * ncol;
  /* leaving times of this step, recorded in slot order after the loop */
  uint8_t* left = s->probe_cap && do_leave ? (uint8_t*)calloc(n ? n : 1, 1) : NULL;
  float* left_age = left ? (float*)malloc(sizeof(float) * (n ? n : 1)) : NULL;
  if (n_threads < 1) n_threads = 1;
  uint64_t clamped = 0;
#ifdef _OPENMP
  __int128* partial = (__int128*)calloc((size_t)n_threads * acc_len, sizeof(__int128));
#pragma omp parallel num_threads(n_threads) reduction(+ : moves, exits, reqdiv, clamped)
  {
    const int tid = omp_get_thread_num();
    __int128* acc = partial + (size_t)tid * acc_len;
#pragma omp for schedule(static)
    for (uint64_t i = 0; i < n; ++i) {
#else
  __int128* partial = (__int128*)calloc(acc_len, sizeof(__int128));
  {
    __int128* acc = partial;
    for (uint64_t i = 0; i < n; ++i) {
#endif
      if (s->status[i] != ORC_IDLE) continue;
      float d[4];
      draws_for(s, s->id[i], 0u, d);
      /* ages(i, 1) += d_t with d_t of the model's float type (model_kernel.hpp
       * L193, L270) */
      s->age_d[i] = s->f64 ? (float)((double)s->age_d[i] + dt) : s->age_d[i] + dtf;
      const uint32_t p0 = s->pos[i];
      double basis = 0.0, ctb[8] = {0};
      const int st = model_update(s, dt, i, rates + (size_t)p0 * 8 * rsz, &basis, ctb);
      if (st == ORC_DIVISION) {
        s->div_flag[i] = 1;
        s->div_pos[i] = p0;
        reqdiv++;
      }
      if (!contrib_ok || contrib_ok[i]) {
        int cl = 0;
        if (s->separable) {
          acc[p0] += orc_quantize(basis, s->q_exp[0], s->q_max, &cl);
          clamped += (uint64_t)cl;
        } else {
          for (uint32_t j = 0; j < nctb; ++j) {
            cl = 0;
            acc[(uint64_t)p0 * ncol + j] += orc_quantize(s->weight * ctb[j], s->q_exp[j], s->q_max, &cl);
            clamped += (uint64_t)cl;
          }
        }
      }
      uint32_t p = p0;
      if (do_move) {
        int moved = 0;
        p = move_one(s, pmove[p], p, d[0], d[1], &moved);
        moves += (uint64_t)moved;
        s->pos[i] = p;
      }
      if (do_leave) {
        const int ex = leave_one(s, dt, dtf, p, &s->status[i], &s->age_h[i], d[2], left ? &left_age[i] : NULL);
        exits += (uint64_t)ex;
        if (ex && left) left[i] = 1;
      }
    }
  }
#ifndef _OPENMP
  n_threads = 1;
#endif
  /* exact totals -> sources: separable src(c,j) = (w * coef_j(c)) * B(c) */
  for (uint32_t c = 0; c < s->n_c; ++c) {
    if (s->separable) {
      __int128 t = 0;
      for (int th = 0; th < n_threads; ++th) t += partial[(size_t)th * acc_len + c];
      const double B = orc_fixed_to_double(t, s->q_exp[0]);
      for (uint32_t sp = 0; sp < ns; ++sp) {
        double v = 0.0;
        if (sp < nctb) v = (s->weight * model_coef(s, rates + (size_t)c * 8 * rsz, (int)sp)) * B;
        s->src[(size_t)c * ns + sp] = v;
      }
    } else {
      for (uint32_t sp = 0; sp < ns; ++sp) {
        double v = 0.0;
        if (sp < nctb) {
          __int128 t = 0;
          for (int th = 0; th < n_threads; ++th) t += partial[(size_t)th * acc_len + (size_t)c * ncol + sp];
          v = orc_fixed_to_double(t, s->q_exp[sp]);
        }
        s->src[(size_t)c * ns + sp] = v;
      }
    }
  }
  s->ctb_clamped += clamped;
  free(partial);
  free(contrib_ok);
  if (left) {
    for (uint64_t i = 0; i < n; ++i)
      if (left[i]) (void)orc_probe_set(s, 0, (double)left_age[i]);
    free(left);
    free(left_age);
  }
  free(rates);
  if (pmove != pmove_small) free(pmove);
  s->moves = moves;
  s->exits = exits;
  s->requested_divisions = reqdiv;
}

/* Gap filling of remove_inactive_particles (particles_container.hpp L737-L795
 * with CompactParticlesFunctor L292-L383) in single-threaded order: the j-th
 * non-Idle slot of [0, n-r) receives the j-th Idle particle counted from the
 * end of [n-r, n). */
void orc_remove_inactive(orc_state* s, uint64_t to_remove) {
  if (to_remove == 0) return;
  if (to_remove == s->n_used) {
    s->n_used = 0;
    s->inactive = 0;
    return;
  }
  if (to_remove > s->n_used) {
    s->error = 1;
    return;
  }
  const uint64_t n = s->n_used;
  const uint64_t head = n - to_remove;
  uint64_t g = 0;
  for (uint64_t i = 0; i < head; ++i)
    if (s->status[i] != ORC_IDLE) s->gap_slot[g++] = (uint32_t)i;
  uint64_t q = 0;
  for (uint64_t i = n; i-- > head;)
    if (s->status[i] == ORC_IDLE) s->src_slot[q++] = (uint32_t)i;
  if (q != g) {
    s->error = 2;
    return;
  }
  const uint64_t cap = s->phys_capacity;
  for (uint64_t j = 0; j < g; ++j) {
    const uint64_t dst = s->gap_slot[j], src = s->src_slot[j];
    for (uint32_t v = 0; v < s->n_var; ++v) {
      if (s->f64)
        ((double*)s->state)[v * cap + dst] = ((double*)s->state)[v * cap + src];
      else
        ((float*)s->state)[v * cap + dst] = ((float*)s->state)[v * cap + src];
    }
    s->pos[dst] = s->pos[src];
    s->status[dst] = ORC_IDLE;
    s->age_h[dst] = s->age_h[src];
    s->age_d[dst] = s->age_d[src];
    s->id[dst] = s->id[src];
    s->div_flag[dst] = 0;
  }
  s->n_used = head;
  s->inactive -= to_remove;
}

/* Post-cycle (reference SimulationUnit::post_cycle, simulation.hpp L215):
 *   1. divisions in slot order, limited by free room (handle_division);
 *   2. inactive += out (+ dead); compaction when above the threshold
 *      max(min_removal, n_used * ratio) (update_and_remove_inactive);
 *   3. children appended after the live particles with ages 0
 *      (merge_buffer / InsertFunctor). */
void orc_post_cycle(orc_state* s) {
  const uint64_t n = s->n_used;
  uint64_t inactive_after = s->inactive + s->exits;
  const uint64_t ratio_thr = (uint64_t)((double)n * s->dead_ratio_threshold);
  const uint64_t threshold = s->min_removal > ratio_thr ? s->min_removal : ratio_thr;
  const int compact = inactive_after > threshold;
  const uint64_t n_after = compact ? n - inactive_after : n;
  const uint64_t room = s->phys_capacity > n_after ? s->phys_capacity - n_after : 0;

  uint64_t births = 0, overflow = 0;
  for (uint64_t i = 0; i < n; ++i) {
    if (!s->div_flag[i]) continue;
    s->div_flag[i] = 0;
    /* every request is a division-time event, refused or not */
    if (s->probe_cap) (void)orc_probe_set(s, 1, (double)s->age_d[i]);
    if (births < room) {
      model_division(s, i, births);
      s->child_pos[births] = s->div_pos[i];
      s->age_d[i] = 0.0f;
      births++;
    } else {
      overflow++;
    }
  }
  s->inactive = inactive_after;
  s->compacted = 0;
  if (compact) {
    orc_remove_inactive(s, inactive_after);
    s->compacted = 1;
  }
  const uint64_t base = s->n_used;
  const uint64_t cap = s->phys_capacity;
  for (uint64_t b = 0; b < births; ++b) {
    const uint64_t dst = base + b;
    for (uint32_t v = 0; v < s->n_var; ++v) {
      if (s->f64)
        ((double*)s->state)[v * cap + dst] = ((double*)s->child_state)[v * cap + b];
      else
        ((float*)s->state)[v * cap + dst] = ((float*)s->child_state)[v * cap + b];
    }
    s->pos[dst] = s->child_pos[b];
    s->status[dst] = ORC_IDLE;
    s->age_h[dst] = 0.0f;
    s->age_d[dst] = 0.0f;
    s->id[dst] = (uint32_t)(s->next_id + b);
  }
  s->n_used = base + births;
  s->next_id += births;
  s->births = births;
  s->overflow = overflow;
}

/* One main-loop iteration, apps/core/src/host_specific.cpp L280-L291:
 * update_feed -> ode_step -> clearContribution -> cycleProcess. */
/* Leaving flows of the particles from the feeds' outlets, in feed order
 * (the set_leaving_flow calls of update_feed, simulation.model.cpp L101-L108). */
void orc_set_outlets(orc_state* s) {
  s->n_outlets = 0;
  for (uint32_t f = 0; f < s->n_feeds; ++f) {
    if (s->feed_out[f] >= 0) {
      const uint32_t o = (uint32_t)s->feed_out[f];
      s->outlet_index[s->n_outlets] = o;
      s->outlet_flow[s->n_outlets] = s->feed_flow[f];
      s->outlet_volume[s->n_outlets] = s->volume[o];
      s->n_outlets++;
    }
  }
}

/* FeedDescriptor::update (feed_descriptor.cpp L12-L36): Linear f0 + t*df,
 * Exponential f0 + exp(alpha*t) (exp from IEEE operations, sa_exp, as the
 * device computes it; the reference calls the C library's exp). */
double orc_feed_flow(int32_t kind, double flow, double f0, double rate, double t) {
  if (kind == 1) return f0 + t * rate;
  if (kind == 2) return f0 + sa_exp(rate * t);
  return flow;
}

void orc_step(orc_state* s, double dt, int n_threads) {
  const uint32_t ns = s->n_s;
  /* update_feed at the relative time of this iteration (simulation.model.cpp
   * L73-L111): sources, sinks and the outlets' leaving flows */
  for (uint32_t f = 0; f < s->n_feeds; ++f)
    s->feed_flow[f] = orc_feed_flow(s->feed_kind[f], s->feed_flow[f], s->feed_f0[f], s->feed_rate[f], s->t_rel);
  for (uint32_t j = 0; j < s->n_c; ++j) s->sink[j] = 0.0;
  for (uint32_t f = 0; f < s->n_feeds; ++f) {
    for (uint32_t sp = 0; sp < ns; ++sp) {
      const double cf = s->feed_conc[f * 8 + sp];
      if (cf != 0.0) s->src[(uint64_t)s->feed_in[f] * ns + sp] += s->feed_flow[f] * cf;
    }
    if (s->feed_out[f] >= 0) s->sink[(uint32_t)s->feed_out[f]] += s->feed_flow[f];
  }
  orc_set_outlets(s);
  orc_scalar_step(s, dt);
  memset(s->src, 0, sizeof(double) * (size_t)s->n_c * ns);
  orc_cycle(s, dt, n_threads);
  orc_post_cycle(s);
  s->step++;
  s->t_rel += dt; /* SimulationUnit::advance */
}

/* orc_step without the cycle: the feeds, the liquid step from the sources
 * the caller left in src (the previous cycle's contributions), sources
 * cleared for the caller's next contributions, the step counter and the
 * relative time advanced.  For driving another implementation's particle
 * cycle with this liquid. */
void orc_liquid_step(orc_state* s, double dt) {
  const uint32_t ns = s->n_s;
  for (uint32_t f = 0; f < s->n_feeds; ++f)
    s->feed_flow[f] = orc_feed_flow(s->feed_kind[f], s->feed_flow[f], s->feed_f0[f], s->feed_rate[f], s->t_rel);
  for (uint32_t j = 0; j < s->n_c; ++j) s->sink[j] = 0.0;
  for (uint32_t f = 0; f < s->n_feeds; ++f) {
    for (uint32_t sp = 0; sp < ns; ++sp) {
      const double cf = s->feed_conc[f * 8 + sp];
      if (cf != 0.0) s->src[(uint64_t)s->feed_in[f] * ns + sp] += s->feed_flow[f] * cf;
    }
    if (s->feed_out[f] >= 0) s->sink[(uint32_t)s->feed_out[f]] += s->feed_flow[f];
  }
  orc_set_outlets(s);
  orc_scalar_step(s, dt);
  memset(s->src, 0, sizeof(double) * (size_t)s->n_c * ns);
  s->step++;
  s->t_rel += dt;
}

void orc_run(orc_state* s, double dt, uint32_t n_steps, int n_threads) {
  for (uint32_t k = 0; k < n_steps; ++k) orc_step(s, dt, n_threads);
}

/* Occupancy per compartment of Idle particles (MonteCarloUnit::getRepartition,
 * apps/libs/mc/src/unit.cpp L191-L230). */
void orc_repartition(const orc_state* s, uint64_t* counts) {
  for (uint32_t c = 0; c < s->n_c; ++c) counts[c] = 0;
  for (uint64_t i = 0; i < s->n_used; ++i)
    if (s->status[i] == ORC_IDLE) counts[s->pos[i]]++;
}

/* ------------------------------------------------------------------------ */
/* Pin entry points: one particle through the functions the cycle above
 * uses, so tests/test_ref_pins.py can hold them against outputs of the
 * reference's own code compiled from its headers. */
uint32_t orc_pin_find_next(uint32_t K, const double* cdf_row, const uint32_t* nbr_row, double u) {
  orc_state t;
  memset(&t, 0, sizeof(t));
  t.K = K;
  t.n_c = 1;
  t.cdf = (double*)cdf_row;
  t.neighbors = (uint32_t*)nbr_row;
  return orc_find_next(&t, 0, u);
}

uint32_t orc_pin_move(uint32_t n_c, uint32_t K, const double* volume, const double* out_flow, const uint32_t* nbr,
                      const double* cdf, double dt, uint32_t pos, float u1, float u2, int32_t* moved) {
  orc_state t;
  memset(&t, 0, sizeof(t));
  t.K = K;
  t.n_c = n_c;
  t.cdf = (double*)cdf;
  t.neighbors = (uint32_t*)nbr;
  const double p_move = (dt * out_flow[pos]) / volume[pos]; /* as orc_cycle's pmove */
  int m = 0;
  const uint32_t r = move_one(&t, p_move, pos, u1, u2, &m);
  *moved = m;
  return r;
}

int32_t orc_pin_leave(uint32_t n_outlets, const uint32_t* index, const double* flow, const double* volume, double dt,
                      uint32_t pos, uint8_t* status, float* age_h, float u) {
  orc_state t;
  memset(&t, 0, sizeof(t));
  t.n_outlets = n_outlets;
  for (uint32_t o = 0; o < n_outlets && o < ORC_MAX_OUTLETS; ++o) {
    t.outlet_index[o] = index[o];
    t.outlet_flow[o] = flow[o];
    t.outlet_volume[o] = volume[o];
  }
  if (*status != ORC_IDLE) return 0; /* TagLeave skips particles that are not Idle */
  return leave_one(&t, dt, (float)dt, pos, status, age_h, u, NULL);
}

int32_t orc_pin_exit_test(double dt, double flow, double volume, float u) { return exit_test(dt, flow, volume, u); }

/* The float models' update on one particle (state x in place) in a
 * compartment of concentrations c; the per-particle contributions to ctb. */
int32_t orc_pin_model_update(int32_t model, double dt, float* x, const double* c, float* ctb) {
  orc_state t;
  memset(&t, 0, sizeof(t));
  t.model = model;
  t.f64 = 0;
  float r[8] = {0};
  model_rates(&t, c, r);
  const float dtf = (float)dt;
  if (model == ORC_MODEL_FIXED_LENGTH || model == ORC_MODEL_FIXED_LENGTH_GENERAL)
    return fixed_length_update_general(dtf, x, r, ctb, t.params);
  if (model == ORC_MODEL_SIMPLE_ACETATE) return simple_acetate_update_general(dtf, x, r, ctb, t.params);
  return -1;
}

void orc_pin_fixed_length_division(float* x, float* child) {
  const float d[4] = {0};
  fixed_length_division(x, child, d, NULL);
}

void orc_pin_simple_acetate_division(float* x, float* child, double z1, double z2, float u3, float u4) {
  simple_acetate_division_z(x, child, z1, z2, u3, u4);
}

/* init draws d[1], d[2] are the length and l_max uniforms */
void orc_pin_simple_acetate_init(float* x, float u_length, float u_lmax) {
  const float d[4] = {0.f, u_length, u_lmax, 0.f};
  simple_acetate_init(x, d, NULL);
}

float orc_pin_erfinv_f(float x) { return sa_erfinv_f(x); }
double orc_pin_erfinv_d(double x) { return sa_erfinv_d(x); }
float orc_pin_norminv_f(float p, float mean, float sd) { return sa_norminv_f(p, mean, sd); }
double orc_pin_std_normal(float u) { return sa_std_normal(u); }

/* Draw tables of a container (the reference-cycle comparison hands them to
 * the reference's compiled cycle): out[i][0..3] = the four draws of purpose
 * `purpose` of the particle with id ids[i] at step `step`; with normals set,
 * lanes 0 and 1 are replaced by the standard normals the SimpleAcetate
 * division takes from them (sa_std_normal) and the table is double. */
void orc_draw_table(uint64_t seed, const uint32_t* ids, uint64_t n, uint32_t step, uint32_t purpose, float* out) {
  for (uint64_t i = 0; i < n; ++i) orc_draws(seed, ids[i], step, purpose, out + 4 * i);
}
/* Standard normals of the draw values u[k] by the reference's inverse-CDF
 * form (sa_std_normal), and truncated normals of the same draws
 * (orc_pin_truncnorm_f), for the distribution tests. */
void orc_std_normal_table(const float* u, uint64_t n, double* out) {
  for (uint64_t i = 0; i < n; ++i) out[i] = sa_std_normal(u[i]);
}
void orc_truncnorm_table(const float* u, uint64_t n, float mu, float sd, float lo, float hi, float* out) {
  for (uint64_t i = 0; i < n; ++i) out[i] = orc_pin_truncnorm_f((double)u[i], mu, sd, lo, hi);
}

void orc_division_draw_table(uint64_t seed, const uint32_t* ids, uint64_t n, uint32_t step, double* out) {
  for (uint64_t i = 0; i < n; ++i) {
    float d[4];
    orc_draws(seed, ids[i], step, 1u, d);
    out[4 * i + 0] = sa_std_normal(d[0]);
    out[4 * i + 1] = sa_std_normal(d[1]);
    out[4 * i + 2] = (double)d[2];
    out[4 * i + 3] = (double)d[3];
  }
}

/* TruncatedNormal<float>::draw_from (prng_extension.hpp L379-L414) with
 * the bounds' probabilities computed as the reference does, 0.5 *
 * erfc(-z / sqrt2) in double from the float z, rounded to float. */
float orc_pin_truncnorm_f(double u, float mu, float sd, float lower, float upper) {
  float zl = (lower - mu) / sd;
  zl = zl < -5e3f ? -5e3f : (zl > 0.f ? 0.f : zl);
  float zu = (upper - mu) / sd;
  zu = zu < 0.f ? 0.f : (zu > 5e3f ? 5e3f : zu);
  const float pl = (float)(0.5 * erfc((double)(-zl) / SA_SQRT2));
  const float pu = (float)(0.5 * erfc((double)(-zu) / SA_SQRT2));
  return sa_truncnorm_f((float)u, mu, sd, pl, pu);
}

/* 1 when the C library's logf is non-increasing in -logf over the draw
 * values (2k + 1) / 2^24 (the exit test is then monotone in the draw and a
 * threshold on the integer draw decides it); the first k that breaks it in
 * *bad_k otherwise. */
int32_t orc_logf_monotone_over_draws(uint32_t* bad_k) {
  float prev = logf(0x1p-24f);
  for (uint32_t k = 1; k < (1u << 23); ++k) {
    const float v = logf((float)(2u * k + 1u) * 0x1p-24f);
    if (v < prev) {
      if (bad_k) *bad_k = k;
      return 0;
    }
    prev = v;
  }
  return 1;
}

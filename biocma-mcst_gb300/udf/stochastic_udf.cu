// stochastic_udf.cu -- a cell model whose update draws random numbers and
// reads its compartment's concentrations, as the reference's
// Model::update(random_pool, d_t, idx, arr, contribs, position, c) may
// (apps/libs/mc/public/mc/traits.hpp L117; e.g. the probabilistic division
// test check_probability_division, apps/libs/models/public/models/utils.hpp
// L101-L115, draws in update).
//
// State {length, l_max} in float.  Per step: the glucose concentration of
// the particle's compartment s = max(c[0], 0) read directly; uptake factor
// g = s / (k + s); a noise factor 0.5 + draw[0] (mean 1) on the elongation
// l += dt * ldot_max * g * noise and on the glucose uptake
// -phi_s_max * g * noise (general contribution path); division when the
// length reaches l_max, or by chance with probability p_div per step
// (draw[1] < p_div).  Division halves the length.
// Parameters: [0] ldot_max m/s, [1] l_max m, [2] k kg/m3, [3] diameter m,
// [4] glucose-to-biomass yield, [5] p_div.
#include "bmc_udf.cuh"

template <class F>
struct StochasticUdf {
  static constexpr int n_var = 2;
  static constexpr int n_ctb = 1;
  static constexpr int n_rates = 1;
  static constexpr int n_upd = 0;
  static constexpr bool separable = false;
  static constexpr bool uses_context = true;
  static constexpr unsigned read_mask = 0x3u;

  BMC_UDF_FN static F lin_density(const double* p) {
    const F d_m = (F)p[3];
    return (F)1000 * (F)3.14159265358979323846 * d_m * d_m / (F)4;
  }
  // no per-compartment factor: update reads the concentrations itself
  BMC_UDF_FN static void rates(const double* c, const double* p, F* r) {
    (void)c;
    (void)p;
    r[0] = (F)0;
  }
  BMC_UDF_FN static int update_ctx(F dt, F* x, const F* r, F* ctb, const F* pf, const bmc::UpdateContext& ctx) {
    (void)r;
    const F ldot_max = pf[0], k = pf[2], yield = pf[4], p_div = pf[5];
    const F d_m = pf[3];
    const F lin = (F)1000 * (F)3.14159265358979323846 * d_m * d_m / (F)4;
    F s = (F)ctx.c[0];
    if (s < (F)0) s = (F)0;
    const F g = s / (k + s);
    const F noise = (F)0.5 + (F)ctx.draws[0];
    x[0] += dt * (ldot_max * g * noise);
    ctb[0] = -(((ldot_max * lin) / yield) * g * noise);
    const bool by_chance = (F)ctx.draws[1] < p_div;
    return (x[0] >= x[1] || by_chance) ? bmc::kDivision : bmc::kIdle;
  }
  BMC_UDF_FN static void division(F* x, F* child, const float* d, const double* p) {
    (void)d;
    const F l_max = (F)p[1];
    const F half = x[0] / (F)2;
    x[0] = half;
    x[1] = l_max;
    child[0] = half;
    child[1] = l_max;
  }
  BMC_UDF_FN static void init(F* x, const float* d, const double* p) {
    const F l_max = (F)p[1];
    const F l_min = l_max / (F)2;
    x[0] = l_min + (l_max - l_min) * (F)d[1];
    x[1] = l_max;
  }
  BMC_UDF_FN static double mass(const F* x, const double* p) { return (double)(x[0] * lin_density(p)); }
};

BMC_DEFINE_UDF(StochasticUdf, BMC_UDF_FLOAT | BMC_UDF_DOUBLE, BMC_UDF_NAMES("length", "l_max"),
               BMC_UDF_NAMES("glucose"))

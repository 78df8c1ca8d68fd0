// monod_udf.cu -- Monod uptake and growth written as a runtime-loaded model.
//
// The same model as libbmc's built-in BMC_MODEL_MONOD, with every
// expression in the same order, so a scenario run through this library gives
// bit-identical results to the built-in one.  State {mass, age}; one
// contribution (substrate uptake -(mu/Y) * mass, separable with basis mass).
// Parameters: [0] mu_max 1/s, [1] Ks kg/m3, [2] yield, [3] division mass,
// [4] initial mass low, [5] initial mass span.
#include "bmc_udf.cuh"

template <class F>
struct MonodUdf {
  static constexpr int n_var = 2;
  static constexpr int n_ctb = 1;
  static constexpr int n_rates = 2;
  static constexpr int n_upd = 1;
  static constexpr bool separable = true;
  static constexpr unsigned read_mask = 0x3u;

  // r = {mu, -(mu / Y)}
  BMC_UDF_FN static void rates(const double* c, const double* p, F* r) {
    const F mu_max = (F)p[0], ks = (F)p[1], y = (F)p[2];
    F s = (F)c[0];
    if (s < (F)0) s = (F)0;
    const F g = s / (ks + s);
    const F mu = mu_max * g;
    r[0] = mu;
    r[1] = -(mu / y);
  }
  BMC_UDF_FN static int update(F dt, F* x, const F* r, F& basis, const F* pf) {
    const F m = x[0];
    basis = m;
    const F growth = r[0] * m;
    x[0] = m + dt * growth;
    x[1] = x[1] + dt;
    return x[0] >= pf[3] ? bmc::kDivision : bmc::kIdle;
  }
  BMC_UDF_FN static F coef(const F* r, int j) {
    (void)j;
    return r[1];
  }
  BMC_UDF_FN static void division(F* x, F* child, const float* d, const double* p) {
    (void)d;
    (void)p;
    const F half = x[0] * (F)0.5;
    x[0] = half;
    x[1] = (F)0;
    child[0] = half;
    child[1] = (F)0;
  }
  BMC_UDF_FN static void init(F* x, const float* d, const double* p) {
    x[0] = (F)p[4] + (F)p[5] * (F)d[1];
    x[1] = (F)0;
  }
  BMC_UDF_FN static double mass(const F* x, const double* p) {
    (void)p;
    return (double)x[0];
  }
};

BMC_DEFINE_UDF(MonodUdf, BMC_UDF_FLOAT | BMC_UDF_DOUBLE, BMC_UDF_NAMES("mass", "age"),
               BMC_UDF_NAMES("glucose"))

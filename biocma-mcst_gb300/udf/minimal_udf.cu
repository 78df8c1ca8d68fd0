// minimal_udf.cu -- a length-growth cell model as a runtime-loaded model.
//
// Behaviour of the reference's example UDF (apps/udf_model/minimal.cpp:
// _update_udf, _division_udf, mass): uptake factor g = s / (k + s),
// elongation rate ldot = ldot_max g, glucose uptake phi_s = phi_s_max g;
// the length grows by dt*ldot / (1 + dt*ldot) (evaluated in double, as the
// reference's double literal makes it), the particle contributes -phi_s
// (written per particle: the general contribution path), and divides at
// length >= l_max into two halves.  mass = length * linear density.
// State {length, l_max} in float (the reference's UdfModel FloatType).
// Parameters: [0] ldot_max m/s, [1] l_max m, [2] k kg/m3, [3] diameter m,
// [4] glucose-to-biomass yield.
#include "bmc_udf.cuh"

template <class F>
struct MinimalUdf {
  static constexpr int n_var = 2;
  static constexpr int n_ctb = 1;
  static constexpr int n_rates = 2;
  static constexpr int n_upd = 2;
  static constexpr bool separable = false;
  static constexpr unsigned read_mask = 0x3u;

  // linear density rho * pi * d^2 / 4 with rho = 1000 kg/m3
  BMC_UDF_FN static F lin_density(const double* p) {
    const F d_m = (F)p[3];
    return (F)1000 * (F)3.14159265358979323846 * d_m * d_m / (F)4;
  }
  // r = {ldot, -phi_s}
  BMC_UDF_FN static void rates(const double* c, const double* p, F* r) {
    const F ldot_max = (F)p[0], k = (F)p[2], yield = (F)p[4];
    const F phi_s_max = (ldot_max * lin_density(p)) / yield;
    const F s = (F)c[0];
    const F g = s / (k + s);
    r[0] = ldot_max * g;
    r[1] = -(phi_s_max * g);
  }
  BMC_UDF_FN static int update_general(F dt, F* x, const F* r, F* ctb, const F* pf) {
    (void)pf;
    const F d_length = dt * r[0];
    x[0] = (F)((double)x[0] + (double)d_length / (1.0 + (double)(dt * r[0])));
    ctb[0] = r[1];
    return x[0] >= x[1] ? bmc::kDivision : bmc::kIdle;
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
  BMC_UDF_FN static double mass(const F* x, const double* p) {
    return (double)(x[0] * lin_density(p));
  }
};

BMC_DEFINE_UDF(MinimalUdf, BMC_UDF_FLOAT, BMC_UDF_NAMES("length", "l_max"), BMC_UDF_NAMES("glucose"))

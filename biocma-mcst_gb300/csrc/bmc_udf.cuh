// bmc_udf.cuh -- write a cell model as a runtime-loaded plugin.
//
// The GPU counterpart of the reference's "udf_model" (a shared library whose
// init/update/division/mass functions UnsafeUDF::Loader binds at run time,
// apps/libs/models/ext/udf_includes.hpp L27-L122).  A GPU cannot call a host
// function pointer per particle, so the plugin carries the whole cycle:
// include this header, define the model struct, and expand
//
//     BMC_DEFINE_UDF(MyModel, BMC_UDF_FLOAT | BMC_UDF_DOUBLE,
//                    BMC_UDF_NAMES("length", "l_max"), BMC_UDF_NAMES("glucose"))
//
// MyModel is a class template over the state float type F with:
//   static constexpr int n_var, n_ctb;        state variables, contributions
//   static constexpr int n_rates (<= 7);      factors per compartment
//   static constexpr int n_upd (<= n_rates);  leading factors update() reads
//   static constexpr bool separable;          contribution j = coef_j * basis
//   static constexpr unsigned read_mask;      state variables update() reads (it
//                                             must write every other one)
//   BMC_UDF_FN static void rates(const double* c, const double* params, F* r);
//   separable:  BMC_UDF_FN static int update(F dt, F* x, const F* r, F& basis, const F* pf);
//               BMC_UDF_FN static F coef(const F* r, int j);
//   general:    BMC_UDF_FN static int update_general(F dt, F* x, const F* r, F* ctb, const F* pf);
//   BMC_UDF_FN static void division(F* x, F* child, const float* draws, const double* params);
//   BMC_UDF_FN static void init(F* x, const float* draws, const double* params);
//   BMC_UDF_FN static double mass(const F* x, const double* params);
// update() returns bmc::kIdle or bmc::kDivision (Model::update's Status);
// pf holds the 16 parameters converted to F.  A model whose update draws
// random numbers or reads the compartment's concentrations directly (the
// reference's update(random_pool, d_t, idx, arr, contribs, position, c))
// declares instead of update / update_general:
//   static constexpr bool uses_context = true;
//   BMC_UDF_FN static int update_ctx(F dt, F* x, const F* r, F* out, const F* pf,
//                                    const bmc::UpdateContext& ctx);
// with out the basis (separable) or the n_ctb contributions (general), and
// ctx.draws four uniforms of the particle and step, ctx.c the n_species
// concentrations of its compartment, ctx.position the compartment.  Every
// function is compiled for the device (the kernels) and for the host
// (bmc_udf_get_host_model).
//
// Build with the library's flags (bmc/udf.py build_udf): sm_103a,
// --fmad=false, -ffp-contract=off, hidden visibility; only the entry points
// below are exported.
#pragma once
#include <cstddef>
#include <cstdint>
#include <type_traits>

#include "../../include/bmc.h"
#include "bmc_kernel_templates.cuh"

#define BMC_UDF_FN __host__ __device__ __forceinline__
#define BMC_UDF_FLOAT 1
#define BMC_UDF_DOUBLE 2
#define BMC_UDF_NAMES(...) __VA_ARGS__
#define BMC_UDF_EXPORT extern "C" __attribute__((visibility("default")))

namespace bmc {
namespace udf {

template <template <class> class M, class F>
struct HostModel {
  using Model = M<F>;
  static void rates(const double* c, const double* p, void* r) { Model::rates(c, p, static_cast<F*>(r)); }
  static int32_t update(double dt, void* x, const void* r, void* out, const double* p) {
    F pf[16];
    for (int k = 0; k < 16; ++k) pf[k] = (F)p[k];
    if constexpr (has_context<Model>::value) {
      (void)dt;
      (void)x;
      (void)r;
      (void)out;
      return -1;  // the model updates through update_ctx
    } else if constexpr (Model::separable) {
      F b = (F)0;
      const int st = Model::update((F)dt, static_cast<F*>(x), static_cast<const F*>(r), b, pf);
      *static_cast<F*>(out) = b;
      return st;
    } else {
      return Model::update_general((F)dt, static_cast<F*>(x), static_cast<const F*>(r), static_cast<F*>(out), pf);
    }
  }
  static int32_t update_ctx(double dt, void* x, const void* r, void* out, const double* p, const float* draws,
                            const double* c, uint32_t position, uint32_t n_species) {
    if constexpr (has_context<Model>::value) {
      F pf[16];
      for (int k = 0; k < 16; ++k) pf[k] = (F)p[k];
      const UpdateContext ctx{draws, c, position, n_species};
      return Model::update_ctx((F)dt, static_cast<F*>(x), static_cast<const F*>(r), static_cast<F*>(out), pf, ctx);
    } else {
      (void)dt, (void)x, (void)r, (void)out, (void)p, (void)draws, (void)c, (void)position, (void)n_species;
      return -1;
    }
  }
  static double coef(const void* r, int32_t j) {
    if constexpr (Model::separable)
      return (double)Model::coef(static_cast<const F*>(r), (int)j);
    else
      return 0.0;
  }
  static void division(void* x, void* child, const float* d, const double* p) {
    Model::division(static_cast<F*>(x), static_cast<F*>(child), d, p);
  }
  static void init(void* x, const float* d, const double* p) { Model::init(static_cast<F*>(x), d, p); }
  static double mass(const void* x, const double* p) { return Model::mass(static_cast<const F*>(x), p); }
  static void fill(bmc_udf_host_model* o) {
    o->n_var = Model::n_var;
    o->n_ctb = Model::n_ctb;
    o->n_rates = Model::n_rates;
    o->separable = Model::separable ? 1 : 0;
    o->rates = &rates;
    o->update = &update;
    o->coef = &coef;
    o->division = &division;
    o->init = &init;
    o->mass = &mass;
    o->update_ctx = has_context<Model>::value ? &update_ctx : nullptr;
  }
};

template <class F>
constexpr int precision_bit() {
  return sizeof(F) == 8 ? BMC_UDF_DOUBLE : BMC_UDF_FLOAT;
}

// Float type of the metadata queries: float when compiled, else double.
template <int P>
using FirstF = typename std::conditional<(P & BMC_UDF_FLOAT) != 0, float, double>::type;

template <template <class> class M, int P, class F>
const KernelSet* kernel_set_for() {
  if constexpr ((P & precision_bit<F>()) != 0) {
    using Model = M<F>;
    static_assert(Model::n_var >= 1 && Model::n_var <= kMaxVar, "n_var must be in [1, 16]");
    static_assert(Model::n_ctb >= 1 && Model::n_ctb <= kMaxSpecies, "n_ctb must be in [1, 8]");
    static_assert(Model::n_rates >= 1 && Model::n_rates <= 7, "n_rates must be in [1, 7]");
    static_assert(Model::n_upd >= 0 && Model::n_upd <= Model::n_rates, "n_upd must be <= n_rates");
    static const KernelSet k = kset::make_set<Model, F>(0);
    return &k;
  } else {
    return nullptr;
  }
}

template <template <class> class M, int P, class F>
int host_model_for(bmc_udf_host_model* out) {
  if constexpr ((P & precision_bit<F>()) != 0) {
    HostModel<M, F>::fill(out);
    return 0;
  } else {
    (void)out;
    return -1;
  }
}

inline uint32_t count_names(const char* const* v, uint32_t cap) {
  uint32_t n = 0;
  while (n < cap && v[n]) ++n;
  return n;
}

}  // namespace udf
}  // namespace bmc

// Entry points of a plugin (C-ABI, the only exported symbols).  The set of a
// precision that was not requested is null.  Kernel sets are built on first
// use and carry model id 0; libbmc assigns the id when it loads the plugin.
#define BMC_DEFINE_UDF(MODEL, PRECISIONS, NAMES, SPECIES)                                    \
  namespace {                                                                                \
  constexpr int bmc_udf_precisions_ = (PRECISIONS);                                          \
  static_assert(bmc_udf_precisions_ != 0, "compile at least one precision");                 \
  const char* const bmc_udf_names_[] = {NAMES, nullptr};                                     \
  const char* const bmc_udf_species_[] = {SPECIES, nullptr};                                 \
  using bmc_udf_meta_ = MODEL<bmc::udf::FirstF<bmc_udf_precisions_>>;                        \
  }                                                                                          \
  BMC_UDF_EXPORT int bmc_udf_abi(void) { return bmc::kKernelSetAbi; }                        \
  BMC_UDF_EXPORT const void* bmc_udf_kernel_set(int32_t f64) {                               \
    if (f64) return bmc::udf::kernel_set_for<MODEL, bmc_udf_precisions_, double>();          \
    return bmc::udf::kernel_set_for<MODEL, bmc_udf_precisions_, float>();                    \
  }                                                                                          \
  BMC_UDF_EXPORT size_t set_nvar_udf(void) { return (size_t)bmc_udf_meta_::n_var; }          \
  BMC_UDF_EXPORT size_t set_nc_udf(void) { return (size_t)bmc_udf_meta_::n_ctb; }            \
  BMC_UDF_EXPORT int32_t separable_udf(void) { return bmc_udf_meta_::separable ? 1 : 0; }    \
  BMC_UDF_EXPORT const char* const* names_udf(uint32_t* n) {                                 \
    *n = bmc::udf::count_names(bmc_udf_names_, 16);                                          \
    return bmc_udf_names_;                                                                   \
  }                                                                                          \
  BMC_UDF_EXPORT const char* const* species_udf(uint32_t* n) {                               \
    *n = bmc::udf::count_names(bmc_udf_species_, 8);                                         \
    return bmc_udf_species_;                                                                 \
  }                                                                                          \
  BMC_UDF_EXPORT int host_model_udf(int32_t f64, bmc_udf_host_model* out) {                  \
    if (f64) return bmc::udf::host_model_for<MODEL, bmc_udf_precisions_, double>(out);      \
    return bmc::udf::host_model_for<MODEL, bmc_udf_precisions_, float>(out);                 \
  }

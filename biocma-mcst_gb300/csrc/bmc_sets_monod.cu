// bmc_sets_monod.cu -- kernel sets of the Monod model (double and float).
#include "bmc_kernel_templates.cuh"

namespace bmc {

const KernelSet* set_monod(int f64) {
  static const KernelSet d = kset::make_set<MonodModel<double>, double>(1);
  static const KernelSet f = kset::make_set<MonodModel<float>, float>(1);
  return f64 ? &d : &f;
}

}  // namespace bmc

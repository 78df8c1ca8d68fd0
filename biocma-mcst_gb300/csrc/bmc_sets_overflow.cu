// bmc_sets_overflow.cu -- kernel sets of the Monod + overflow model (double and float).
#include "bmc_kernel_templates.cuh"

namespace bmc {

const KernelSet* set_overflow(int f64) {
  static const KernelSet d = kset::make_set<OverflowModel<double>, double>(2);
  static const KernelSet f = kset::make_set<OverflowModel<float>, float>(2);
  return f64 ? &d : &f;
}

}  // namespace bmc

// bmc_sets_fixed.cu -- kernel sets of the reference's FixedLength model (separable and general paths, float).
#include "bmc_kernel_templates.cuh"

namespace bmc {

const KernelSet* set_fixed_length(bool separable) {
  static const KernelSet sep = kset::make_set<FixedLengthModelT<true>, float>(3);
  static const KernelSet gen = kset::make_set<FixedLengthModelT<false>, float>(4);
  return separable ? &sep : &gen;
}

}  // namespace bmc

// bmc_sets_acetate.cu -- kernel set of the reference's SimpleAcetate model (float, general path).
#include "bmc_kernel_templates.cuh"

namespace bmc {

const KernelSet* set_simple_acetate() {
  static const KernelSet k = kset::make_set<SimpleAcetateModel, float>(5);
  return &k;
}

}  // namespace bmc

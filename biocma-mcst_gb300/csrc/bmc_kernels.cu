// bmc_kernels.cu -- the table of the built-in model plugins' kernel sets and
// the model-independent kernels (repartition, draw dump).
#include <cstdio>

#include "bmc_kernel_templates.cuh"

namespace bmc {


__global__ void k_repartition(const ScenDev* __restrict__ sc, unsigned long long* __restrict__ counts) {
  const ScenDev& S = *sc;
  const unsigned long long n = S.ctl->n_used;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t p = S.pos[i];
    if (S.status[i] == kIdle && p < S.n_c) atomicAdd(counts + p, 1ull);
  }
}

__global__ void k_debug_draws(unsigned long long seed, const uint32_t* __restrict__ ids, unsigned long long n,
                              uint32_t step, uint32_t purpose, float* __restrict__ out) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const Draws d = philox_draws(seed, ids[i], step, purpose);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[4 * i + k] = d.u[k];
  }
}

// Built-in kernel sets, one translation unit per model (compiled in
// parallel): bmc_sets_monod.cu, bmc_sets_overflow.cu, bmc_sets_fixed.cu.
const KernelSet* kernel_set(int model, int f64) {
  switch (model) {
    case 1:
      return set_monod(f64);
    case 2:
      return set_overflow(f64);
    case 3:
    case 4:
      return f64 ? nullptr : set_fixed_length(model == 3);
    default:
      return udf_kernel_set(model, f64);
  }
}

void launch_repartition(cudaStream_t st, const ScenDev* sc, unsigned long long* counts, int grid) {
  k_repartition<<<grid, 256, 0, st>>>(sc, counts);
}
void launch_debug_draws(cudaStream_t st, unsigned long long seed, const uint32_t* ids, unsigned long long n,
                        uint32_t step, uint32_t purpose, float* out) {
  k_debug_draws<<<256, 256, 0, st>>>(seed, ids, n, step, purpose, out);
}

}  // namespace bmc

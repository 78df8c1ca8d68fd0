// bmc_kernels.cu -- the table of the built-in model plugins' kernel sets and
// the model-independent kernels (repartition, draw dump).
#include <algorithm>
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

// The age step of the cycle kernels on n ages (a >= 0), for its test
// against (float)((double)a + dt) on the CPU.
__global__ void k_debug_age_add(const float* __restrict__ a, unsigned long long n, double dt, float* __restrict__ out) {
  const AgeStep k = age_step(dt);
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = age_add_fast(a[i], k);
}

// Export of one step's results to host memory mapped into the device
// address space: the control block (4-byte words) at dst, then the
// concentrations the step left (buffer step & 1 of C, [n_c][n_s], ne
// values) at dst + conc_offset.  Launched after the step on its stream; the
// host reads dst once an event recorded after this kernel has completed.
// With up_src set, block 0 then also copies a descriptor staged in mapped
// host memory (device address up_src) into up_dst: the upload that precedes
// the next step, in the same launch.
__global__ void k_export(const Control* __restrict__ ctl, const double* __restrict__ C, unsigned long long ne,
                         unsigned char* __restrict__ dst, unsigned long long conc_offset,
                         const unsigned* __restrict__ up_src, unsigned* __restrict__ up_dst) {
  static_assert(sizeof(Control) % 4 == 0, "control block in 4-byte words");
  static_assert(sizeof(ScenDev) % 4 == 0, "descriptor in 4-byte words");
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  if (blockIdx.x == 0) {
    const unsigned* cw = reinterpret_cast<const unsigned*>(ctl);
    unsigned* ow = reinterpret_cast<unsigned*>(dst);
    for (unsigned i = threadIdx.x; i < sizeof(Control) / 4; i += blockDim.x) ow[i] = cw[i];
    if (up_src)
      for (unsigned i = threadIdx.x; i < sizeof(ScenDev) / 4; i += blockDim.x) up_dst[i] = up_src[i];
  }
  const double* c = C + (unsigned long long)(ctl->step & 1u) * ne;
  double* oc = reinterpret_cast<double*>(dst + conc_offset);
  for (unsigned long long i = tid; i < ne; i += nth) oc[i] = c[i];
}

// Upload of a scenario descriptor staged in host memory mapped into the
// device address space: one block copies it into the device descriptor,
// stream-ordered like a copy but without a copy-engine round trip.
__global__ void k_upload_desc(const unsigned* __restrict__ src, unsigned* __restrict__ dst) {
  static_assert(sizeof(ScenDev) % 4 == 0, "descriptor in 4-byte words");
  for (unsigned i = threadIdx.x; i < sizeof(ScenDev) / 4; i += blockDim.x) dst[i] = src[i];
}

// The cycle kernels' float quantisation on n values with quantum 2^e:
// out[2k] through the scaled conversion (quantize_fast), out[2k + 1] from
// the IEEE fields (quantize_bits), for their test against each other and
// against rint(v * 2^-e) on the CPU.
__global__ void k_debug_quantize(const float* __restrict__ v, unsigned long long n, int e,
                                 long long* __restrict__ out) {
  const float sc = quantize_scale(e);
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    unsigned c = 0u, er = 0u;
    out[2 * i] = quantize_fast(v[i], e, sc, c, er);
    out[2 * i + 1] = quantize(v[i], e, c, er);
  }
}

// Self-test of the bounded wait the cycle kernels use on their mbarriers:
// one thread waits on phase 0 of a barrier expecting one arrival, which it
// makes first (`arrive` != 0: the wait succeeds) or that nothing makes (the
// wait gives up after limit_ns).  out[0]: BMC_ERR_TIMEOUT (16) when the wait
// gave up, else 0; out[1]: nanoseconds waited.
__global__ void k_debug_wait(unsigned long long limit_ns, int arrive, unsigned long long* out) {
  __shared__ unsigned long long bar;
  __shared__ unsigned abort_word;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1u);
  abort_word = 0u;
  fence_barrier_init();
  if (arrive) mbar_arrive(&bar);
  const unsigned long long t0 = global_ns();
  const bool ok = mbar_wait_for(&bar, 0u, &abort_word, limit_ns);
  out[0] = ok ? 0ull : 16ull;
  out[1] = global_ns() - t0;
}

// Built-in kernel sets, one translation unit per model (compiled in
// parallel): bmc_sets_monod.cu, bmc_sets_overflow.cu, bmc_sets_fixed.cu,
// bmc_sets_acetate.cu.
const KernelSet* kernel_set(int model, int f64) {
  switch (model) {
    case 1:
      return set_monod(f64);
    case 2:
      return set_overflow(f64);
    case 3:
    case 4:
      return f64 ? nullptr : set_fixed_length(model == 3);
    case 5:
      return f64 ? nullptr : set_simple_acetate();
    default:
      return udf_kernel_set(model, f64);
  }
}

void launch_repartition(cudaStream_t st, const ScenDev* sc, unsigned long long* counts, int grid) {
  k_repartition<<<grid, 256, 0, st>>>(sc, counts);
}
void launch_debug_wait(cudaStream_t st, unsigned long long limit_ns, int arrive, unsigned long long* out) {
  k_debug_wait<<<1, 32, 0, st>>>(limit_ns, arrive, out);
}
void launch_debug_draws(cudaStream_t st, unsigned long long seed, const uint32_t* ids, unsigned long long n,
                        uint32_t step, uint32_t purpose, float* out) {
  k_debug_draws<<<256, 256, 0, st>>>(seed, ids, n, step, purpose, out);
}
void launch_debug_age_add(cudaStream_t st, const float* a, unsigned long long n, double dt, float* out) {
  k_debug_age_add<<<256, 256, 0, st>>>(a, n, dt, out);
}

void launch_export(cudaStream_t st, const Control* ctl, const double* C, unsigned long long ne, unsigned char* dst,
                   unsigned long long conc_offset, const ScenDev* up_src, ScenDev* up_dst) {
  const unsigned blocks = (unsigned)std::min<unsigned long long>(64ull, (ne + 2047ull) / 2048ull + 1ull);
  k_export<<<blocks, 256, 0, st>>>(ctl, C, ne, dst, conc_offset, reinterpret_cast<const unsigned*>(up_src),
                                   reinterpret_cast<unsigned*>(up_dst));
}

void launch_upload_desc(cudaStream_t st, const ScenDev* src_mapped, ScenDev* dst) {
  k_upload_desc<<<1, 256, 0, st>>>(reinterpret_cast<const unsigned*>(src_mapped), reinterpret_cast<unsigned*>(dst));
}

void launch_debug_quantize(cudaStream_t st, const float* v, unsigned long long n, int e, long long* out) {
  k_debug_quantize<<<256, 256, 0, st>>>(v, n, e, out);
}

}  // namespace bmc

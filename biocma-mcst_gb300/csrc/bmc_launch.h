// bmc_launch.h -- host-side view of the kernels: one KernelSet per compiled
// model plugin and precision, plus the model-independent launchers.
//
// A KernelSet holds host launch functions only (no kernel handles), so a
// set built into a separately compiled plugin library (bmc_udf.cuh) is
// driven by libbmc exactly like a built-in one: every launch, attribute
// and occupancy query runs inside the module that owns the kernels.
#pragma once
#include <cuda_runtime.h>

#include "bmc_device.cuh"
#include "bmc_kernels.cuh"

namespace bmc {

// Version of KernelSet's layout and of the meaning of its launch arguments
// (such as the scatter forms a cycle launcher accepts); a plugin built
// against another version is refused at load time.
constexpr int kKernelSetAbi = 12;
// Threads per block of the liquid step (k_liquid): kLiquidThreads / n_species
// whole compartments per block, so a small domain still spreads over many SMs.
constexpr unsigned kLiquidThreads = 32;

// The last argument selects the instantiation with the warp-aggregated
// scatter, for launches whose domains all have at most
// kAggregateMaxCompartments compartments.
// Scatter form of a cycle launch: plain shared-memory atomics; warp-aggregated
// (every domain of the launch at most kAggregateMaxCompartments
// compartments); accumulator copies (some domain of a separable model at most
// kScatterCopyMaxCompartments compartments, tile-staging kernel only); global
// (no shared accumulator: each value goes straight to the scenario's exact
// global accumulator, for domains whose shared accumulator would not leave
// the tile-staging kernel two blocks per SM; tile-staging kernel only).
enum ScatterForm : int { kScatterPlain = 0, kScatterWarp = 1, kScatterCopied = 2, kScatterGlobal = 3 };
using CycleLaunch = void (*)(dim3, dim3, size_t, cudaStream_t, const ScenDev*, int, BatchCtl*, int scatter);
using DivideLaunch = void (*)(dim3, cudaStream_t, const ScenDev*, int, const BatchCtl*);
using CopyLaunch = void (*)(dim3, cudaStream_t, const ScenDev*, int, const BatchCtl*);
using InitLaunch = void (*)(dim3, cudaStream_t, const ScenDev*, unsigned long long, uint32_t, uint32_t,
                            double*);

using LiquidLaunch = void (*)(int, unsigned, cudaStream_t, ScenDev*, BatchCtl*, int);
using MoveThrLaunch = void (*)(int, cudaStream_t, ScenDev*);
// Sets the cycle kernel's dynamic shared-memory limit to `smem` and returns
// (cudaError_t) with the resident blocks per SM in *blocks_per_sm.
using CycleSetup = int (*)(size_t smem, int* blocks_per_sm);

// Cycle launch variants: {threads per block, particles per thread}.  0-4
// stream particles through registers (k_cycle); 5-6 stage tiles in shared
// memory through the copy engine (k_cycle_tma: consumer threads plus one
// producer warp, slots per consumer thread per tile).
constexpr int kCycleVariants = 7;
constexpr unsigned kVariantThreads[kCycleVariants] = {256, 256, 256, 512, 1024, 288, 544};
constexpr unsigned kVariantPPT[kCycleVariants] = {1, 2, 4, 2, 1, 4, 2};
// Launch shape a scenario or batch starts with: resolved per launch to the
// tile-staging 544 x 2 shape, with the shared accumulator while it and the
// stage buffers fit a block, else with the global accumulator
// (kScatterGlobal); register streaming 256 x 2 only if neither fits.
constexpr unsigned kVariantAuto = kCycleVariants;
constexpr unsigned kAutoStaged = 6, kAutoStreamed = 1;
// Domains of at most kScatterCopyMaxCompartments compartments (separable
// models) scatter into kAccCopies copies of the shared accumulator in the
// tile-staging kernel, lane l into copy l % kAccCopies: lanes of a warp
// that hit the same compartment mostly hit different copies, so their
// atomics stop serialising.  Copy stride: the compartment count rounded up to
// 16 plus 16 / kAccCopies, so the copies of one compartment (8 bytes, two
// banks each) sit in different banks.
constexpr unsigned kAccCopies = 8;
constexpr unsigned kScatterCopyMaxCompartments = 256;
__host__ __device__ constexpr unsigned scatter_stride(unsigned n_c) {
  return ((n_c + 15u) & ~15u) + 16u / kAccCopies;
}

// Compartments whose sources one k_plan block computes (grid y of k_plan:
// ceil(n_compartments / kPlanSlice) slices; slice 0 also plans the step).
constexpr unsigned kPlanSlice = 256;
using PlanLaunch = void (*)(int n_scen, unsigned slices, cudaStream_t, ScenDev*, BatchCtl*);

struct KernelSet {
  int abi;
  int model;
  bool f64;
  bool separable;
  int n_var;
  int n_ctb;
  LiquidLaunch liquid;
  PlanLaunch plan;
  CycleLaunch cycle[kCycleVariants];
  CycleSetup cycle_setup[kCycleVariants];
  unsigned cycle_extra_smem[kCycleVariants];  // stage buffers after the accumulator
  MoveThrLaunch move_thr;
  MoveThrLaunch flowmap;  // flow-map switch at the start of a step
  DivideLaunch divide;
  CopyLaunch compact;
  CopyLaunch merge;
  InitLaunch init;
  int (*last_error)();  // cudaGetLastError of the module owning the kernels
  // Model::mass of slots [0, n) into out (device memory)
  void (*mass)(cudaStream_t, const ScenDev*, unsigned long long n, double* out);
};

// Built-in sets first, then the sets of loaded plugins (bmc_udf_load).
const KernelSet* kernel_set(int model, int f64);
const KernelSet* set_monod(int f64);
const KernelSet* set_overflow(int f64);
const KernelSet* set_fixed_length(bool separable);
const KernelSet* set_simple_acetate();
const KernelSet* udf_kernel_set(int model, int f64);
void launch_repartition(cudaStream_t st, const ScenDev* sc, unsigned long long* counts, int grid);
void launch_debug_wait(cudaStream_t st, unsigned long long limit_ns, int arrive, unsigned long long* out);
void launch_debug_age_add(cudaStream_t st, const float* a, unsigned long long n, double dt, float* out);
void launch_debug_quantize(cudaStream_t st, const float* v, unsigned long long n, int e, long long* out);
// Copies a descriptor staged in mapped host memory (device address
// src_mapped) to the device descriptor (k_upload_desc).
void launch_upload_desc(cudaStream_t st, const ScenDev* src_mapped, ScenDev* dst);
// Copies a step's control block and current concentrations (ne =
// compartments * species values of C's current buffer) to mapped host memory
// (k_export); with up_src set, also a descriptor staged in mapped host memory
// into up_dst.
void launch_export(cudaStream_t st, const Control* ctl, const double* C, unsigned long long ne, unsigned char* dst,
                   unsigned long long conc_offset, const ScenDev* up_src = nullptr, ScenDev* up_dst = nullptr);
void launch_debug_draws(cudaStream_t st, unsigned long long seed, const uint32_t* ids, unsigned long long n,
                        uint32_t step, uint32_t purpose, float* out);

}  // namespace bmc

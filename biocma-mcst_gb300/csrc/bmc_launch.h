// bmc_launch.h -- host-side view of the kernels: one KernelSet per compiled
// model plugin and precision, plus the model-independent launchers.
#pragma once
#include <cuda_runtime.h>

#include "bmc_device.cuh"
#include "bmc_kernels.cuh"

namespace bmc {

using CycleLaunch = void (*)(dim3, dim3, size_t, cudaStream_t, const ScenDev*, int, BatchCtl*);
using DivideLaunch = void (*)(dim3, cudaStream_t, const ScenDev*, int, const BatchCtl*);
using CopyLaunch = void (*)(dim3, cudaStream_t, const ScenDev*, int, const BatchCtl*);
using InitLaunch = void (*)(dim3, cudaStream_t, const ScenDev*, unsigned long long, uint32_t, uint32_t,
                            double*);

using LiquidLaunch = void (*)(int, unsigned, cudaStream_t, ScenDev*, BatchCtl*, int);
using MoveThrLaunch = void (*)(int, cudaStream_t, ScenDev*);

// Cycle launch variants: {threads per block, particles per thread}.
constexpr int kCycleVariants = 5;
constexpr unsigned kVariantThreads[kCycleVariants] = {256, 256, 256, 512, 1024};
constexpr unsigned kVariantPPT[kCycleVariants] = {1, 2, 4, 2, 1};
using PlanLaunch = void (*)(int, cudaStream_t, ScenDev*, BatchCtl*);

struct KernelSet {
  int model;
  bool f64;
  bool separable;
  int n_var;
  int n_ctb;
  LiquidLaunch liquid;
  PlanLaunch plan;
  CycleLaunch cycle[kCycleVariants];
  const void* cycle_fn[kCycleVariants];  // for occupancy queries / attributes
  MoveThrLaunch move_thr;
  DivideLaunch divide;
  CopyLaunch compact;
  CopyLaunch merge;
  InitLaunch init;
};

const KernelSet* kernel_set(int model, int f64);
void launch_repartition(cudaStream_t st, const ScenDev* sc, unsigned long long* counts, int grid);
void launch_debug_draws(cudaStream_t st, unsigned long long seed, const uint32_t* ids, unsigned long long n,
                        uint32_t step, uint32_t purpose, float* out);

}  // namespace bmc

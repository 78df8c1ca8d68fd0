// bmc_kernels.cuh -- the Monte Carlo cycle kernels for sm_103a.
//
// One step of the reference main loop (apps/core/src/host_specific.cpp
// L280-L291) is six launches over a table of scenarios:
//   k_liquid      update_feed + ScalarSimulation::performStep (FP64 Euler)
//   k_cycle       fused model update + contribution scatter + move + exit
//                 (CycleFunctors::launch_model / launch_move, kernels.hpp)
//   k_plan        contributions -> sources, division / compaction plan,
//                 per-tile scans (post_cycle, simulation.hpp L215)
//   k_divide      Model::division in slot order + compaction lists
//   k_compact     gap filling (remove_inactive_particles)
//   k_merge       children appended after the live particles (merge_buffer)
// All but k_cycle are small or exit at once when nothing is to be done.
#pragma once
#include <cuda_runtime.h>

#include "bmc_device.cuh"

namespace bmc {

constexpr int kTile = 1024;  // particles per tile (scheduling and scan unit)

// Batch-wide scheduling state (device memory).
struct BatchCtl {
  unsigned int ticket;      // unused (tiles are partitioned statically)
  unsigned int total_tiles; // allocated tiles over all scenarios
  unsigned int flags;       // work of this step after the cycle (kFlag*)
  unsigned int total_live;  // tiles holding particles this step, all scenarios
  unsigned int* live_base;  // [n_scen]: first live tile of each scenario
};
constexpr unsigned kFlagDivide = 1u;   // some scenario asked for divisions
constexpr unsigned kFlagCompact = 2u;  // some scenario compacts
constexpr unsigned kFlagMerge = 4u;    // some scenario appends children

// ------------------------------------------------------------------------
// Vector loads / stores of PPT consecutive elements (streaming hints: the
// particle arrays are touched once per step, the domain data must stay in
// L1/L2).

template <class T, int N>
struct alignas(sizeof(T) * N >= 16 ? 16 : sizeof(T) * N) Pack {
  T v[N];
};

template <class T, int N>
__device__ __forceinline__ void ld_stream(const T* p, T* out) {
  constexpr int bytes = sizeof(T) * N;
  if constexpr (bytes == 16) {
    uint4 r = __ldcs(reinterpret_cast<const uint4*>(p));
    memcpy(out, &r, 16);
  } else if constexpr (bytes == 32) {
    uint4 a = __ldcs(reinterpret_cast<const uint4*>(p));
    uint4 b = __ldcs(reinterpret_cast<const uint4*>(p) + 1);
    memcpy(out, &a, 16);
    memcpy(reinterpret_cast<char*>(out) + 16, &b, 16);
  } else if constexpr (bytes == 8) {
    uint2 r = __ldcs(reinterpret_cast<const uint2*>(p));
    memcpy(out, &r, 8);
  } else if constexpr (bytes == 4) {
    unsigned r = __ldcs(reinterpret_cast<const unsigned*>(p));
    memcpy(out, &r, 4);
  } else if constexpr (bytes == 2) {
    unsigned short r = __ldcs(reinterpret_cast<const unsigned short*>(p));
    memcpy(out, &r, 2);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = p[k];
  }
}

template <class T, int N>
__device__ __forceinline__ void st_stream(T* p, const T* in) {
  constexpr int bytes = sizeof(T) * N;
  if constexpr (bytes == 16) {
    uint4 r;
    memcpy(&r, in, 16);
    __stcs(reinterpret_cast<uint4*>(p), r);
  } else if constexpr (bytes == 32) {
    uint4 a, b;
    memcpy(&a, in, 16);
    memcpy(&b, reinterpret_cast<const char*>(in) + 16, 16);
    __stcs(reinterpret_cast<uint4*>(p), a);
    __stcs(reinterpret_cast<uint4*>(p) + 1, b);
  } else if constexpr (bytes == 8) {
    uint2 r;
    memcpy(&r, in, 8);
    __stcs(reinterpret_cast<uint2*>(p), r);
  } else if constexpr (bytes == 4) {
    unsigned r;
    memcpy(&r, in, 4);
    __stcs(reinterpret_cast<unsigned*>(p), r);
  } else if constexpr (bytes == 2) {
    unsigned short r;
    memcpy(&r, in, 2);
    __stcs(reinterpret_cast<unsigned short*>(p), r);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) p[k] = in[k];
  }
}

// ------------------------------------------------------------------------
// Block reductions / scans (blockDim multiple of 32, at most 1024).

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Exclusive scan of one value per thread; returns the thread's prefix and
// writes the block total.  `sh` needs 33 words.
__device__ __forceinline__ unsigned block_exscan_u32(unsigned v, unsigned* sh, unsigned* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned w = lane < nw ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) sh[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const unsigned warp_off = wid > 0 ? sh[wid - 1] : 0u;
  const unsigned tot = sh[nw - 1];
  __syncthreads();
  *total = tot;
  return warp_off + x - v;
}

__device__ __forceinline__ unsigned long long block_exscan_u64(unsigned long long v, unsigned long long* sh,
                                                               unsigned long long* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned long long w = lane < nw ? sh[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) sh[lane] = w;
  }
  __syncthreads();
  const unsigned long long warp_off = wid > 0 ? sh[wid - 1] : 0ull;
  const unsigned long long tot = sh[nw - 1];
  __syncthreads();
  *total = tot;
  return warp_off + x - v;
}

// Exact total of a fixed-point accumulator (hi limb sums p >> 32, lo limb
// sums p & 0xffffffff) as a double, rounded once, times 2^e.
__device__ __forceinline__ double fixed_to_double(long long hi, unsigned long long lo, double scale_up) {
  const long long hi2 = hi + (long long)(lo >> 32);
  const unsigned long long lo2 = lo & 0xffffffffull;
  const double d = __dadd_rn(__dmul_rn((double)hi2, 4294967296.0), (double)lo2);
  return __dmul_rn(d, scale_up);
}

// ------------------------------------------------------------------------
// Scenario owning live tile g: the largest s with live_base[s] <= g (a
// scenario without live tiles shares its base with the next one).  `hint`
// is a scenario not after the answer (tickets grow within a block).
__device__ __forceinline__ int scen_of_live(const unsigned* live_base, int n_scen, unsigned g, int hint) {
  int s = hint < 0 ? 0 : hint;
  if (s + 1 < n_scen && g >= __ldg(live_base + s + 1)) {
    if (n_scen - s > 8) {
      int lo = s + 1, hi = n_scen - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(live_base + mid) <= g)
          lo = mid;
        else
          hi = mid - 1;
      }
      return lo;
    }
    while (s + 1 < n_scen && g >= __ldg(live_base + s + 1)) ++s;
  }
  return s;
}

// ------------------------------------------------------------------------
// Find the scenario owning global tile g (tiles are laid out scenario after
// scenario).  `hint` is a scenario index not after the answer.
__device__ __forceinline__ int scen_of_tile(const ScenDev* sc, int n_scen, unsigned g, int hint) {
  int s = hint < 0 ? 0 : hint;
  if (n_scen > 8 && (s + 1 < n_scen) && g >= sc[s + 1].tile_base) {
    int lo = s, hi = n_scen - 1;  // largest s with tile_base <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sc[mid].tile_base <= g)
        lo = mid;
      else
        hi = mid - 1;
    }
    return lo;
  }
  while (s + 1 < n_scen && g >= sc[s + 1].tile_base) ++s;
  return s;
}

}  // namespace bmc

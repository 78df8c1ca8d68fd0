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
  unsigned int ticket;      // next live tile to hand out (tile-staging cycle kernel)
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

// Global stores that do not allocate in L1: the cycle kernels write each
// particle's results once and never read them back in the launch, and
// allocating them evicted the compartment records and neighbour rows the
// kernels gather through L1 (same-box A/B against cache-streaming stores:
// FP64 512-compartment cycle 0.2015 -> 0.1897 ms, batched 1.956 -> 1.914 ms).
__device__ __forceinline__ void st_na(double* p, double v) {
  asm volatile("st.global.L1::no_allocate.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_na(float* p, float v) {
  asm volatile("st.global.L1::no_allocate.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ void st_na(uint32_t* p, uint32_t v) {
  asm volatile("st.global.L1::no_allocate.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_na(unsigned short* p, unsigned short v) {
  asm volatile("st.global.L1::no_allocate.u16 [%0], %1;" ::"l"(p), "h"(v) : "memory");
}
__device__ __forceinline__ void st_na(uint2* p, uint2 v) {
  asm volatile("st.global.L1::no_allocate.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(v.x), "r"(v.y) : "memory");
}
__device__ __forceinline__ void st_na(uint4* p, uint4 v) {
  asm volatile("st.global.L1::no_allocate.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z),
               "r"(v.w)
               : "memory");
}

template <class T, int N>
__device__ __forceinline__ void st_stream(T* p, const T* in) {
  constexpr int bytes = sizeof(T) * N;
  if constexpr (bytes == 16) {
    uint4 r;
    memcpy(&r, in, 16);
    st_na(reinterpret_cast<uint4*>(p), r);
  } else if constexpr (bytes == 32) {
    uint4 a, b;
    memcpy(&a, in, 16);
    memcpy(&b, reinterpret_cast<const char*>(in) + 16, 16);
    st_na(reinterpret_cast<uint4*>(p), a);
    st_na(reinterpret_cast<uint4*>(p) + 1, b);
  } else if constexpr (bytes == 8) {
    uint2 r;
    memcpy(&r, in, 8);
    st_na(reinterpret_cast<uint2*>(p), r);
  } else if constexpr (bytes == 4) {
    unsigned r;
    memcpy(&r, in, 4);
    st_na(reinterpret_cast<uint32_t*>(p), r);
  } else if constexpr (bytes == 2) {
    unsigned short r;
    memcpy(&r, in, 2);
    st_na(reinterpret_cast<unsigned short*>(p), r);
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

// Exclusive prefix sums over items [0, n) of a block whose size is a
// multiple of 32: item i has value v(i) (at most 2^32 / 32 per item), and
// out(i, prefix, total) receives the sum of v over [0, i) and over [0, n).
// Each warp takes a contiguous range of whole 32-item rounds and walks it
// one round at a time (lane l reads item round + l: coalesced), first for
// its total, then, with the block's warp offsets, for the prefixes.  v is
// read twice.  sh: 33 words of shared memory.
template <class V, class O>
__device__ __forceinline__ unsigned long long block_exscan_items(unsigned n, V v, O out, unsigned long long* sh) {
  const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned per = ((n + nw - 1u) / nw + 31u) & ~31u;
  const unsigned b = min(w * per, n), e = min(b + per, n);
  unsigned long long mine = 0ull;
  for (unsigned r = b; r < e; r += 32u)
    if (r + lane < e) mine += v(r + lane);
  mine = warp_sum_u64(mine);
  if (lane == 0) sh[w] = mine;
  __syncthreads();
  if (w == 0) {
    const unsigned long long own = lane < nw ? sh[lane] : 0ull;
    unsigned long long x = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if ((int)lane >= o) x += y;
    }
    if (lane < nw) sh[lane] = x - own;  // exclusive warp offsets
    if (lane == 31u) sh[32] = x;        // block total
  }
  __syncthreads();
  const unsigned long long total = sh[32];
  unsigned long long carry = sh[w];
  for (unsigned r = b; r < e; r += 32u) {
    const unsigned i = r + lane;
    const unsigned x0 = i < e ? (unsigned)v(i) : 0u;  // a round sums to < 2^32
    unsigned x = x0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if ((int)lane >= o) x += y;
    }
    if (i < e) out(i, carry + (x - x0), total);
    carry += __shfl_sync(0xffffffffu, x, 31);
  }
  __syncthreads();  // sh may be reused
  return total;
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

// ------------------------------------------------------------------------
// Asynchronous bulk copies (TMA, cp.async.bulk) into shared memory with
// mbarrier completion, and bounded waits.  Every wait gives up after
// kWaitNs of wall time (globaltimer) or when the block's abort word is set;
// the caller then records BMC_ERR_TIMEOUT and stops.
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// Makes barrier initialisation visible to the async proxy (the copy engine).
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Orders this thread's earlier shared-memory accesses before later copies
// into shared memory by the async proxy.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for phase `parity` of the barrier.  Returns false after limit_ns of
// wall time or when *abort is set (by another thread of the block).
__device__ __forceinline__ bool mbar_wait_for(unsigned long long* bar, unsigned parity, volatile unsigned* abort,
                                              unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0u) {
      if (*abort) return false;
      if (global_ns() - t0 > limit_ns) return false;
    }
  }
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  volatile unsigned* abort) {
  return mbar_wait_for(bar, parity, abort, kWaitNs);
}
// Global -> shared bulk copy of `bytes` (a multiple of 16; both addresses
// 16-byte aligned) completing on `bar` (transaction bytes).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ unsigned dynamic_smem_bytes() {
  unsigned v;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(v));
  return v;
}
__device__ __forceinline__ void consumer_sync(unsigned n_threads) {
  asm volatile("bar.sync 1, %0;" ::"r"(n_threads) : "memory");
}
// Block-level OR of v over the n_threads threads using named barrier 1.
__device__ __forceinline__ bool consumer_any(bool v, unsigned n_threads) {
  unsigned r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.or.pred p, 1, %2, q;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(r)
      : "r"((unsigned)v), "r"(n_threads)
      : "memory");
  return r != 0u;
}

// ------------------------------------------------------------------------
// Exact add of q to a shared-memory accumulator entry, kept as two 32-bit
// words {low: unsigned, high: signed}: the low word takes a 32-bit atomic
// whose old value gives the carry, the high word a second one with q >> 32
// plus the carry (skipped when 0).  Read as one 64-bit word (little endian)
// the entry is the two's-complement sum while the high word stays in int32:
// between flushes an entry takes at most kFlushParticles (2^20) particles'
// values of |q| <= 2^42 (kQMax), so every partial sum of the high adds is
// below 2^20 * (2^10 + 1) in magnitude (a warp-aggregated add of up to 32 values counts as their sum:
// below 2^30 + 2^21).  32-bit shared atomics are native; a 64-bit one took
// about 18 shared-memory wavefronts per warp instruction.
__device__ __forceinline__ void acc_add(unsigned long long* e, long long q) {
  unsigned* w = reinterpret_cast<unsigned*>(e);
  const unsigned lo = (unsigned)(unsigned long long)q;
  const unsigned old = atomicAdd(w, lo);
  const int hi = (int)(q >> 32) + (old + lo < old ? 1 : 0);
  if (hi != 0) atomicAdd(reinterpret_cast<int*>(w + 1), hi);
}

// Exact add of q to a scenario's global accumulator entry {hi, lo} (the
// entry a shared-memory flush adds to): q >> 32 (arithmetic) to hi, the low
// 32 bits of q to lo.  hi 2^32 + lo is the exact total however the values
// are grouped, and fixed_to_double folds lo's carries.  The results are not
// read back, so the adds compile to reductions.
__device__ __forceinline__ void acc_add_global(long long* hi, unsigned long long* lo, long long q) {
  const long long h = q >> 32;
  const unsigned long long l = (unsigned long long)q & 0xffffffffull;
  if (h != 0) atomicAdd(reinterpret_cast<unsigned long long*>(hi), (unsigned long long)h);
  if (l != 0) atomicAdd(lo, l);
}

// ------------------------------------------------------------------------
// Warp-aggregated scatter into the shared-memory accumulator: lanes whose
// `on` is set add q to acc[p]; lanes of one compartment are summed first and
// their leader issues one atomic, so a warp issues one atomic per distinct
// compartment instead of one per lane.  For tiny domains, where the lanes of
// a warp pile onto the same few addresses and their atomics serialise (0-D
// reactor: 8x faster cycle); with more compartments the per-key loop costs
// more than it saves.  Exact: q + 2^42 lies in [0, 2^43], split in 22-bit
// halves whose sums over 32 lanes fit 32 bits.  Whole warp converged.
__device__ __forceinline__ void warp_aggregated_add(unsigned long long* acc, uint32_t p, long long q, bool on) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long u = (unsigned long long)(q + (1ll << 42));
  const unsigned lo = (unsigned)(u & 0x3fffffull), hi = (unsigned)(u >> 22);
  unsigned todo = __ballot_sync(0xffffffffu, on);
  while (todo) {
    const int leader = __ffs((int)todo) - 1;
    const uint32_t key = __shfl_sync(0xffffffffu, p, leader);
    const unsigned grp = __ballot_sync(0xffffffffu, on && p == key);
    const bool in = (grp >> lane) & 1u;
    const unsigned slo = __reduce_add_sync(0xffffffffu, in ? lo : 0u);
    const unsigned shi = __reduce_add_sync(0xffffffffu, in ? hi : 0u);
    if ((int)lane == leader) {
      const long long tot =
          (long long)(((unsigned long long)shi << 22) + slo) - (long long)__popc(grp) * (1ll << 42);
      acc_add(acc + key, tot);
    }
    todo &= ~grp;
  }
}
// Domains up to this many compartments use the aggregated scatter.
constexpr unsigned kAggregateMaxCompartments = 4;

}  // namespace bmc

// bmc_kernel_templates.cuh -- the model-templated kernels of the Monte Carlo
// cycle and a KernelSet factory.  Included by bmc_kernels.cu (built-in
// models) and by runtime-loaded model plugins (bmc_udf.cuh), which
// instantiate the same kernels for their own model struct.
//
// Reference behaviour (BioCMA-MCST paths):
//   model + division request   apps/libs/simulation/public/simulation/kernels/
//                              model_kernel.hpp L164-L268
//   contribution scatter       contribution_kernel.hpp L146-L186
//   move                       move_kernel.hpp L62-L103, L393-L437
//   exit                       move_kernel.hpp L348-L359, L588-L648
//   leave tests                apps/libs/simulation/public/simulation/
//                              probability_leaving.hpp L18-L35
//   division / compaction /    apps/libs/mc/public/mc/particles_container.hpp
//   merge                      L541-L600, L737-L795
//   liquid step                apps/libs/simulation/src/implScalar.cpp L251
//   feeds                      apps/libs/simulation/src/simulation.model.cpp L73
#pragma once
#include <cstdio>

#include "bmc_kernels.cuh"
#include "bmc_launch.h"

namespace bmc {


// Slot of rate k in a compartment record: the NU = Model::n_upd rates the
// per-particle update reads sit just below the move threshold (slot 7), so
// that the fewest vector loads fetch both; the other rates (read once per
// compartment by k_plan) fill the record from slot 0.
template <class Model>
__host__ __device__ constexpr int rate_slot(int k) {
  return k < Model::n_upd ? 7 - Model::n_upd + k : k - Model::n_upd;
}

// Model::update of one Idle particle at compartment p0: the per-compartment
// factor form (update / update_general), or update_ctx with the particle's
// draws of the step (purpose 3) and its compartment's concentrations (the
// current buffer of the step: the liquid step wrote it, the step counter
// still holds this step) for models that declare uses_context.
template <class Model, class F>
__device__ __forceinline__ int update_separable(F dt, F* x, const F* r, F& basis, const F* pf, const ScenDev& S,
                                                uint32_t id, uint32_t step, uint32_t p0) {
  if constexpr (has_context<Model>::value) {
    const Draws d = philox_draws(S.seed, id, step, 3u);
    const size_t ne = (size_t)S.n_c * S.n_s;
    const UpdateContext ctx{d.u, S.C + ((step & 1u) ^ 1u) * ne + (size_t)p0 * S.n_s, p0, S.n_s};
    F out[1];
    const int st = Model::update_ctx(dt, x, r, out, pf, ctx);
    basis = out[0];
    return st;
  } else {
    (void)S;
    (void)id;
    (void)step;
    (void)p0;
    return Model::update(dt, x, r, basis, pf);
  }
}
template <class Model, class F>
__device__ __forceinline__ int update_general_of(F dt, F* x, const F* r, F* ctb, const F* pf, const ScenDev& S,
                                                 uint32_t id, uint32_t step, uint32_t p0) {
  if constexpr (has_context<Model>::value) {
    const Draws d = philox_draws(S.seed, id, step, 3u);
    const size_t ne = (size_t)S.n_c * S.n_s;
    const UpdateContext ctx{d.u, S.C + ((step & 1u) ^ 1u) * ne + (size_t)p0 * S.n_s, p0, S.n_s};
    return Model::update_ctx(dt, x, r, ctb, pf, ctx);
  } else {
    (void)S;
    (void)id;
    (void)step;
    (void)p0;
    return Model::update_general(dt, x, r, ctb, pf);
  }
}

// ---------------------------------------------------------------------------
// k_liquid: one thread per (compartment j, species s) entry; a block holds
// kLiquidThreads / n_species whole compartments (grid x over compartment chunks, grid
// y over scenarios).  Feeds into sources and sink, explicit Euler step
//   M(j,s) += dt (sum_i C(i,s) T(i,j) - C(j,s) sink(j) + src(j,s)),
//   C'(j,s) = M(j,s) / V(j),
// then Model::rates of each compartment of the block from C'(j,:) into its
// compartment record.  C is double-buffered by step parity (C' goes to the
// other buffer), so no block waits for another.  With do_scalar == 0 only
// the rates (and C carried to the next buffer).  Block (0, s) resets the
// step counters of scenario s; block (0, 0) the tile scheduler and flags.
template <class Model, class F>
__global__ void __launch_bounds__(kLiquidThreads) k_liquid(ScenDev* __restrict__ sc, BatchCtl* bctl, int do_scalar) {
  const ScenDev& S = sc[blockIdx.y];
  Control* ctl = S.ctl;
  static_assert(kLiquidThreads == 32, "the mass-balance sums below reduce within one warp");
  __shared__ double cs[kLiquidThreads];
  if (blockIdx.x == 0 && blockIdx.y == 0) {
    // live tiles of every scenario (ceil(n_used / 1024), none once finished)
    // and their prefix: the cycle hands out only tiles that hold particles
    __shared__ unsigned sh[33];
    const int n_scen = (int)gridDim.y;
    unsigned run = 0;
    for (int b0 = 0; b0 < n_scen; b0 += (int)blockDim.x) {
      const int s2 = b0 + (int)threadIdx.x;
      unsigned live = 0;
      if (s2 < n_scen) {
        const ScenDev& P = sc[s2];
        if (!scen_finished(P, P.ctl)) {
          const unsigned long long lt = (P.ctl->n_used + kTile - 1) / kTile;
          live = (unsigned)(lt < P.n_tiles ? lt : P.n_tiles);
        }
      }
      unsigned tot;
      const unsigned pre = block_exscan_u32(live, sh, &tot);
      if (s2 < n_scen) bctl->live_base[s2] = run + pre;
      run += tot;
    }
    if (threadIdx.x == 0) {
      bctl->live_base[n_scen] = run;
      bctl->total_live = run;
      bctl->ticket = 0u;
      bctl->flags = 0u;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->req_div = 0ull;
    ctl->exits = 0ull;
    ctl->moves = 0ull;
    ctl->cycling = scen_finished(S, ctl) ? 0u : 1u;
    ctl->t_advance = do_scalar ? 1u : 0u;
  }
  // feed schedules: the outlets' leaving flows and exit thresholds of this
  // step (SimulationUnit::update_feed -> ReactorDomain::set_leaving_flow,
  // simulation.model.cpp L90-L104), for the cycle that follows
  if (blockIdx.x == 0 && S.n_sched > 0u && threadIdx.x < S.n_outlets && !scen_finished(S, ctl)) {
    const unsigned o = threadIdx.x;
    const double fl = feed_flow_at(S, S.outlet_feed[o], ctl->t_rel);
    ScenDev& W = sc[blockIdx.y];
    W.outlet_flow[o] = fl;
    W.exit_thr[o] = exit_threshold_dev(S.nlog, S.dt, fl, S.volume[S.outlet_idx[o]], S.exit_thr[o]);
  }
  {
    // per-tile birth / inactive counters of this step start at zero (the
    // cycle's warps add to them)
    const unsigned long long lt = (ctl->n_used + kTile - 1) / kTile;
    const unsigned n_live = (unsigned)(lt < S.n_tiles ? lt : S.n_tiles);
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n_live; t += gridDim.x * blockDim.x) {
      S.tile_births[t] = 0u;
      S.tile_inactive[t] = 0u;
    }
  }
  const unsigned nsp = S.n_s;
  const unsigned cb = kLiquidThreads / nsp;  // compartments per block
  const unsigned j0 = blockIdx.x * cb;
  if (j0 >= S.n_c || scen_finished(S, ctl)) return;
  const unsigned t = threadIdx.x;
  const unsigned jl = t / nsp;
  const unsigned sp = t - jl * nsp;
  const unsigned j = j0 + jl;
  const bool active = jl < cb && j < S.n_c;
  const size_t ne = (size_t)S.n_c * nsp;
  const unsigned parity = ctl->step & 1u;
  const double* __restrict__ Cold = S.C + parity * ne;
  double* __restrict__ Cnew = S.C + (parity ^ 1u) * ne;
  double mb_new = 0.0, mb_exp = 0.0;  // this thread's mass-balance terms
  if (active) {
    const size_t e = (size_t)j * nsp + sp;
    double cn;
    if (!do_scalar) {
      cn = Cold[e];
    } else {
      // every load of the element that depends on no other, issued before
      // any store (the stores go through double pointers the compiler must
      // assume may alias these): the element's time on the step's critical
      // path is a few memory round trips, not one per operand
      const double dt = S.dt;
      double srcv = S.src[e];
      const double cj = Cold[e];
      const double mold = S.M[e];
      const double diag_j = S.diag[j];
      const double vinv_j = S.vinv[j];
      const unsigned e0 = S.in_ptr[j], e1 = S.in_ptr[j + 1];
      const double t_rel = ctl->t_rel;
      double sinkj = 0.0;
      for (unsigned f = 0; f < S.n_feeds; ++f) {
        const double ff = feed_flow_at(S, f, t_rel);
        if (S.feed_in[f] == j) {
          const double cf = S.feed_conc[f * kMaxSpecies + sp];
          if (cf != 0.0) srcv = __dadd_rn(srcv, __dmul_rn(ff, cf));
        }
        if (S.feed_out[f] == (int)j) sinkj = __dadd_rn(sinkj, ff);
      }
      double acc = 0.0;
      for (unsigned q = e0; q < e1; ++q)
        acc = __dadd_rn(acc, __dmul_rn(Cold[(size_t)S.in_idx[q] * nsp + sp], S.in_flow[q]));
      S.src[e] = srcv;
      acc = __dadd_rn(acc, __dmul_rn(cj, diag_j));
      double dmdt = __dadd_rn(__dsub_rn(acc, __dmul_rn(cj, sinkj)), srcv);
      double mt = 0.0;
      if (S.gas) {
        // gas-liquid transfer from the old concentrations
        // (fixed_kla_gas_liquid_mass_transfer, impl_mtr.cpp L150-L166), then
        // the gas step with the transfer lost (performStepGL, Sign::GasToLiquid)
        const double* __restrict__ Cgo = S.Cg + parity * ne;
        const double cg = Cgo[e];
        mt = __dmul_rn(__dmul_rn(S.kla[e], __dsub_rn(__dmul_rn(cg, S.henry[sp]), cj)), S.volume[j]);
        S.mtr[e] = mt;
        double gsrc = 0.0, gsink = 0.0;
        for (unsigned f = 0; f < S.n_gfeeds; ++f) {
          if (S.gfeed_in[f] == j) gsrc = __dadd_rn(gsrc, __dmul_rn(S.gfeed_flow[f], S.gfeed_conc[f * kMaxSpecies + sp]));
          if (S.gfeed_out[f] == (int)j) gsink = __dadd_rn(gsink, S.gfeed_flow[f]);
        }
        double gacc = 0.0;
        for (unsigned q = S.g_in_ptr[j]; q < S.g_in_ptr[j + 1]; ++q)
          gacc = __dadd_rn(gacc, __dmul_rn(Cgo[(size_t)S.g_in_idx[q] * nsp + sp], S.g_in_flow[q]));
        gacc = __dadd_rn(gacc, __dmul_rn(cg, S.g_diag[j]));
        const double gdmdt = __dsub_rn(__dadd_rn(__dsub_rn(gacc, __dmul_rn(cg, gsink)), gsrc), mt);
        const double mg = __dadd_rn(S.Mg[e], __dmul_rn(dt, gdmdt));
        S.Mg[e] = mg;
        S.Cg[(parity ^ 1u) * ne + e] = __dmul_rn(mg, S.gvinv[j]);
        dmdt = __dadd_rn(dmdt, mt);  // Sign::LiquidToGas
      }
      const double mnew = __dadd_rn(mold, __dmul_rn(dt, dmdt));
      S.M[e] = mnew;
      cn = __dmul_rn(mnew, vinv_j);
      // two-phase: tiny negative liquid concentrations are cleared
      // (ScalarSimulation::clearNegs, implScalar.cpp L266-L293)
      if (S.gas && cn < 0.0 && fabs(cn) < kClearNegTol) cn = 0.0;
      // mass-balance terms (diagnostic): new mass, expected mass
      mb_new = mnew;
      mb_exp = mold + dt * (srcv + mt - cj * sinkj);
    }
    Cnew[e] = cn;
    if (!do_scalar && S.gas) S.Cg[(parity ^ 1u) * ne + e] = S.Cg[parity * ne + e];
    cs[t] = cn;
  }
  __syncthreads();
  if (t < cb && j0 + t < S.n_c) {
    F r[kMaxRates];
    Model::rates(cs + t * nsp, S.params, r);
    F* rec = reinterpret_cast<F*>(S.crec) + (size_t)(j0 + t) * 8;
#pragma unroll
    for (int k = 0; k < Model::n_rates; ++k) rec[rate_slot<Model>(k)] = r[k];
  }
  if (do_scalar) {
    // per-species sums over the warp: lanes of one species lie nsp apart,
    // so a tree over offsets nsp, 2 nsp, 4 nsp, ... leaves species l's sum
    // in lane l (a diagnostic: its summation order is free, as the atomics
    // that add the blocks make it anyway)
    for (unsigned off = nsp; off < 32u; off <<= 1) {
      const double a = __shfl_down_sync(0xffffffffu, mb_new, off);
      const double b = __shfl_down_sync(0xffffffffu, mb_exp, off);
      if (t + off < 32u) {
        mb_new += a;
        mb_exp += b;
      }
    }
    if (t < nsp) {
      atomicAdd(&ctl->mb_new[t], mb_new);
      atomicAdd(&ctl->mb_exp[t], mb_exp);
    }
  }
}

// ---------------------------------------------------------------------------
// Quantisation of a value to the accumulator's fixed point: the nearest
// integer multiple of 2^e (ties to even), clamped to |q| <= kQMax.  Done on
// the integer pipe from the IEEE fields of v, so no FP64 instruction is
// spent per particle; the result equals rint(v * 2^-e) evaluated in double.
template <int MBITS, int EBITS, int BIAS, class U>
__device__ __forceinline__ long long quantize_bits(U bits, int e, unsigned& clamped, unsigned& err) {
  const bool neg = (bits >> (MBITS + EBITS)) & 1u;
  const int ex = (int)((bits >> MBITS) & (((U)1 << EBITS) - 1));
  const unsigned long long mant = (unsigned long long)(bits & (((U)1 << MBITS) - 1));
  long long q;
  if (ex == 0) {
    q = 0;  // zero or subnormal: far below any quantum in use
  } else if (ex == (1 << EBITS) - 1) {
    q = kQMax;  // inf / nan
    ++clamped;
    err |= 2u;
  } else {
    const unsigned long long m = mant | (1ull << MBITS);  // value = m * 2^(ex - BIAS - MBITS)
    const int sh = ex - BIAS - MBITS - e;                  // value / 2^e = m * 2^sh
    if (sh >= 0) {
      q = sh > 62 - MBITS ? kQMax + 1 : (long long)(m << sh);
    } else {
      const int r = -sh;
      if (r > MBITS + 1) {
        q = 0;  // below half a quantum
      } else {
        const unsigned long long t = m >> r;
        const unsigned long long rem = m & ((1ull << r) - 1ull);
        const unsigned long long half = 1ull << (r - 1);
        q = (long long)(t + ((rem > half || (rem == half && (t & 1ull))) ? 1ull : 0ull));
      }
    }
    if (q > kQMax) {
      q = kQMax;
      ++clamped;
      err |= 2u;
    }
  }
  return neg ? -q : q;
}

__device__ __forceinline__ long long quantize(double v, int e, unsigned& clamped, unsigned& err) {
  return quantize_bits<52, 11, 1023>((unsigned long long)__double_as_longlong(v), e, clamped, err);
}
__device__ __forceinline__ long long quantize(float v, int e, unsigned& clamped, unsigned& err) {
  return quantize_bits<23, 8, 127>((unsigned)__float_as_uint(v), e, clamped, err);
}

// 2^-e as a float when the float quantisation below may use it (a normal
// power of two no larger than 2^125), else 0.
__device__ __forceinline__ float quantize_scale(int e) {
  return (e >= -125 && e <= 126) ? __int_as_float((127 - e) << 23) : 0.0f;
}

// quantize(float) through one scaled conversion: v * 2^-e is exact (a
// power-of-two scale; a product too small to be a normal float lies below
// half a quantum, where any rounding still gives 0, as does a subnormal v
// while the scale is at most 2^125), and the conversion rounds to the
// nearest integer, ties to even: the integer quantize_bits computes, with
// the same clamping (inf saturates the conversion, NaN is caught apart).
// scale = quantize_scale(e), nonzero.
__device__ __forceinline__ long long quantize_scaled(float v, float scale, unsigned& clamped, unsigned& err) {
  long long q = __float2ll_rn(v * scale);
  if (q > kQMax || q < -kQMax || v != v) {
    q = signbit(v) ? -kQMax : kQMax;
    ++clamped;
    err |= 2u;
  }
  return q;
}
__device__ __forceinline__ long long quantize_fast(float v, int e, float scale, unsigned& clamped, unsigned& err) {
  return scale != 0.0f ? quantize_scaled(v, scale, clamped, err) : quantize(v, e, clamped, err);
}
__device__ __forceinline__ long long quantize_fast(double v, int e, float, unsigned& clamped, unsigned& err) {
  return quantize(v, e, clamped, err);
}

// Move threshold stored in slot 7 of a compartment record.
__device__ __forceinline__ uint32_t rec_move_thr(float v) { return __float_as_uint(v); }
__device__ __forceinline__ uint32_t rec_move_thr(double v) { return (uint32_t)__double_as_longlong(v); }

// 32-byte read-only loads (one request per lane instead of two; the address
// is 32-byte aligned: records start at multiples of 8 slots of an arena
// aligned to 256 bytes).
__device__ __forceinline__ void ldg_v8(const float* p, float (&v)[8]) {
  asm volatile("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "l"(p));
}
__device__ __forceinline__ void ldg_v8(const int32_t* p, int (&v)[8]) {
  asm volatile("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "l"(p));
}
__device__ __forceinline__ void ldg_v4(const double* p, double (&v)[4]) {
  asm volatile("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p));
}

// Loads the NU update rates and the move threshold of a compartment record
// (slots 7 - NU .. 7) through the read-only path with the widest aligned
// vector loads.
template <int NU, class F>
__device__ __forceinline__ uint32_t load_rec(const F* p, F* out) {
  static_assert(NU >= 0 && NU <= 7, "at most 7 update rates");
  constexpr int s0 = 7 - NU;
  if constexpr (sizeof(F) == 4) {
    if constexpr (NU <= 1) {
      // slots 6, 7
      const float2 a = __ldg(reinterpret_cast<const float2*>(p + 6));
      if constexpr (NU == 1) out[0] = a.x;
      return rec_move_thr(a.y);
    } else {
      // the whole 32-byte record
      float v[8];
      ldg_v8(p, v);
#pragma unroll
      for (int q = s0; q < 7; ++q) out[q - s0] = v[q];
      return rec_move_thr(v[7]);
    }
  } else if constexpr (NU == 0) {
    return rec_move_thr(__ldg(p + 7));
  } else if constexpr (NU == 1) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p + 6));
    out[0] = a.x;
    return rec_move_thr(a.y);
  } else {
    // slots below 4: a scalar when the first is odd, then aligned pairs;
    // slots 4..7 in one 32-byte load
    if constexpr (s0 < 4) {
      if constexpr ((s0 & 1) != 0) out[0] = __ldg(p + s0);
      constexpr int q0 = (s0 & 1) != 0 ? s0 + 1 : s0;
#pragma unroll
      for (int q = q0; q < 4; q += 2) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(p + q));
        out[q - s0] = a.x;
        out[q + 1 - s0] = a.y;
      }
    }
    double v[4];
    ldg_v4(p + 4, v);
#pragma unroll
    for (int q = (s0 > 4 ? s0 : 4); q < 7; ++q) out[q - s0] = v[q - 4];
    return rec_move_thr(v[3]);
  }
}

// Next compartment of a leaving particle: the first k of the row with
// x1 <= floor(2^24 CDF(k)) (K - 1 when none), the answer of the reference's
// bisection (move_kernel.hpp L89-L101).  Rows of up to 8 entries: two
// independent 32-byte loads of the padded thresholds and neighbours; the
// answer is the count of thresholds below x1 (they are non-decreasing);
// longer rows: the bisection over {threshold, neighbour} pairs.
__device__ __forceinline__ int next_compartment(const int2* __restrict__ mrow, const int32_t* __restrict__ row16,
                                                unsigned p0, unsigned K, int x1) {
  const int2* row = mrow + (size_t)p0 * K;
  if (K <= 8u) {
    int t[8], n[8];
    ldg_v8(row16 + (size_t)p0 * 16, t);
    ldg_v8(row16 + (size_t)p0 * 16 + 8, n);
    unsigned below = 0u;
#pragma unroll
    for (int k = 0; k < 8; ++k) below += t[k] < x1 ? 1u : 0u;
    int nb = n[0];
#pragma unroll
    for (int k = 1; k < 8; ++k) nb = below >= (unsigned)k ? n[k] : nb;
    return nb;
  }
  int nb = __ldg(row + (K - 1)).y;
  int left = 0, right = (int)K - 1;
  while (left < right) {
    const int mid = (left + right) >> 1;
    const int2 pm = __ldg(row + mid);
    if (x1 > pm.x) {
      left = mid + 1;
    } else {
      right = mid;
      nb = pm.y;
    }
  }
  return nb;
}

// ---------------------------------------------------------------------------
// k_cycle: the fused per-particle hot path.  Each block of a persistent
// grid streams a contiguous run of the live tiles (1024-slot tiles that hold
// particles, ordered scenario after scenario; k_liquid lists them).  For
// each Idle particle (draws: one Philox block, integers
// x_k = (r_k >> 8) | 1 with u_k = x_k 2^-24):
//   ages(i,1) += dt; Model::update(dt, x, rates(pos))
//   contribution basis (or contributions) -> shared-memory fixed-point
//     accumulator of the pre-move compartment (exact integer sums)
//   move:  leave iff x_0 < ceil(2^24 dt Q/V)       (<=> dt Q / V > u_0)
//          next = first k with x_1 <= floor(2^24 CDF(pos,k))
//                                                  (<=> u_1 <= CDF(pos,k))
//   exit:  ages(i,0) += dt; leave the reactor iff x_2 > floor(2^24 e^{-dt F/V})
//                                                  (<=> dt F > -ln(u_2) V)
// A division request sets a bit of the tile's birth mask; the division
// itself runs in k_divide once the slot-order ranks are known.
// Launch variants: THREADS per block, PPT consecutive particles per thread
// (THREADS * PPT divides the 1024-slot tile) and MINB resident blocks per SM
// the register budget is cut for.
template <class Model, class F, int PPT, int THREADS, int MINB, bool AGG>
__global__ void __launch_bounds__(THREADS, MINB)
    k_cycle(const ScenDev* __restrict__ sc, int n_scen, BatchCtl* __restrict__ bctl) {
  extern __shared__ unsigned long long sacc[];
  __shared__ unsigned long long s_cnt[5];
  __shared__ F s_pf[16];  // parameters of the current scenario, as F
  constexpr int NV = Model::n_var;
  constexpr int NC = Model::n_ctb;
  constexpr int NA = Model::separable ? 1 : NC;  // accumulator columns
  constexpr unsigned CH = 32u * PPT;             // slots per warp chunk
  constexpr unsigned NW = THREADS / 32;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const unsigned warp = (unsigned)tid >> 5;
  const unsigned total = bctl->total_live;
  const unsigned* live_base = bctl->live_base;
  int cur = -1;
  unsigned long long since_flush = 0;
  // per-thread counts between flushes (at most kFlushParticles slots)
  unsigned my_req = 0, my_exit = 0, my_move = 0, my_clamp = 0;
  unsigned my_err = 0;

  // flush the accumulator and the counters of scenario `cur` (whole block)
  auto flush = [&]() {
    __syncthreads();
    const ScenDev& P = sc[cur];
    const unsigned n_ent = P.n_c * NA;
    for (unsigned e = tid; e < n_ent; e += THREADS) {
      const long long p = (long long)sacc[e];
      if (p != 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(P.acc_hi + e), (unsigned long long)(p >> 32));
        atomicAdd(P.acc_lo + e, (unsigned long long)p & 0xffffffffull);
      }
    }
    if (tid < 5) s_cnt[tid] = 0ull;
    __syncthreads();
    const unsigned long long r0 = warp_sum_u64(my_req), r1 = warp_sum_u64(my_exit);
    const unsigned long long r2 = warp_sum_u64(my_move), r3 = warp_sum_u64(my_clamp);
    unsigned e4 = my_err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e4 |= __shfl_xor_sync(0xffffffffu, e4, o);
    if (lane == 0) {
      atomicAdd(&s_cnt[0], r0);
      atomicAdd(&s_cnt[1], r1);
      atomicAdd(&s_cnt[2], r2);
      atomicAdd(&s_cnt[3], r3);
      atomicOr(reinterpret_cast<unsigned*>(&s_cnt[4]), e4);
    }
    __syncthreads();
    if (tid == 0) {
      Control* c = P.ctl;
      if (s_cnt[0]) atomicAdd(&c->req_div, s_cnt[0]);
      if (s_cnt[1]) atomicAdd(&c->exits, s_cnt[1]);
      if (s_cnt[2]) atomicAdd(&c->moves, s_cnt[2]);
      if (s_cnt[3]) atomicAdd(&c->clamped, s_cnt[3]);
      const unsigned ev = *reinterpret_cast<unsigned*>(&s_cnt[4]);
      if (ev) atomicOr(&c->error, ev);
    }
    my_req = my_exit = my_move = my_clamp = 0u;
    my_err = 0u;
  };

  // static partition: block b streams the live tiles [g_begin, g_end), a
  // contiguous run, scenario segment after scenario segment; inside a
  // segment every warp streams its own 32*PPT-slot chunks with no block
  // barrier, so warps drift apart and hide each other's latency
  const unsigned g_begin = (unsigned)(((unsigned long long)total * blockIdx.x) / gridDim.x);
  const unsigned g_end = (unsigned)(((unsigned long long)total * (blockIdx.x + 1)) / gridDim.x);
  unsigned g = g_begin;
  while (g < g_end) {
    const int s = scen_of_live(live_base, n_scen, g, cur);
    const unsigned sb = __ldg(live_base + s), se = __ldg(live_base + s + 1);
    const unsigned ge = se < g_end ? se : g_end;
    const ScenDev& S = sc[s];
    const unsigned long long n_used = S.ctl->n_used;
    const unsigned long long p_lo = (unsigned long long)(g - sb) * kTile;
    unsigned long long p_hi = (unsigned long long)(ge - sb) * kTile;
    if (p_hi > n_used) p_hi = n_used;
    g = ge;

    const unsigned long long cap = S.cap;
    const unsigned n_c = S.n_c, K = S.K;
    const unsigned step = S.ctl->step;
    const unsigned long long seed = S.seed;
    const double dt = S.dt;
    const F dtF = (F)dt;
    const float dtf = (float)dt;
    const AgeStep ak = age_step(dt);
    const bool do_move = n_c > 1;
    const unsigned n_out = S.n_outlets;
    const int qe0 = S.q_exp[0];
    const float qs0 = quantize_scale(qe0);
    const F* __restrict__ crec = reinterpret_cast<const F*>(S.crec);
    const int2* __restrict__ mrow = S.mrow;
    F* __restrict__ state = reinterpret_cast<F*>(S.state);

    for (unsigned long long q0 = p_lo; q0 < p_hi; q0 += kFlushParticles) {
      const unsigned long long q1 = q0 + kFlushParticles < p_hi ? q0 + kFlushParticles : p_hi;
      if (s != cur || since_flush + (q1 - q0) > kFlushParticles) {
        if (cur >= 0) flush();
        __syncthreads();
        const unsigned n_ent = S.n_c * NA;
        for (unsigned e = tid; e < n_ent; e += THREADS) sacc[e] = 0ull;
        if (tid < 16) s_pf[tid] = (F)S.params[tid];
        cur = s;
        since_flush = 0;
        __syncthreads();
      }
      since_flush += q1 - q0;

#pragma unroll 1
      for (unsigned long long c = q0 + (unsigned long long)warp * CH; c < q1; c += (unsigned long long)NW * CH) {
        const unsigned long long first = c + (unsigned long long)lane * PPT;
        // every load of the chunk is issued before any result is needed
        uint8_t stv[PPT];
        uint32_t pv[PPT], idv[PPT];
        float ah[PPT], ad[PPT];
        F x[NV][PPT];
        ld_stream<uint8_t, PPT>(S.status + first, stv);
        ld_stream<uint32_t, PPT>(S.pos + first, pv);
        ld_stream<uint32_t, PPT>(S.id + first, idv);
        if (n_out > 0) ld_stream<float, PPT>(S.age_h + first, ah);
        ld_stream<float, PPT>(S.age_d + first, ad);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          if ((Model::read_mask >> v) & 1u) ld_stream<F, PPT>(state + (size_t)v * cap + first, x[v]);
        uint32_t p0s[PPT];  // compartments before the move
#pragma unroll
        for (int k = 0; k < PPT; ++k) p0s[k] = pv[k];
        bool idle[PPT];
        bool any = false, all = true;
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          idle[k] = (first + k < n_used) && stv[k] == kIdle;
          any |= idle[k];
          all &= idle[k];
        }
        // variables the update only writes are read solely when some slot of
        // the vector keeps its old value
        if (any && !all) {
#pragma unroll
          for (int v = 0; v < NV; ++v)
            if (!((Model::read_mask >> v) & 1u)) ld_stream<F, PPT>(state + (size_t)v * cap + first, x[v]);
        }
        unsigned bits = 0u;
        unsigned n_inact = 0u;
        bool has_q[PPT];  // tiny domains: quantised basis, scattered warp-aggregated
        long long qv[PPT];
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          has_q[k] = false;
          qv[k] = 0;
        }
        if (any) {
          bool st_changed = false;
#pragma unroll
          for (int k = 0; k < PPT; ++k) {
            if (!idle[k]) continue;
            const uint32_t p0 = pv[k];
            if (p0 >= n_c) {
              my_err |= 1u;
              continue;
            }
            uint32_t r[4];
            philox_raw(seed, idv[k], step, 0u, r);
            // ages(i, 1) += d_t in the model's float type
            if constexpr (sizeof(F) == 8)
              ad[k] = age_add_fast(ad[k], ak);
            else
              ad[k] = __fadd_rn(ad[k], dtf);
            F rr[Model::n_upd > 0 ? ((Model::n_upd + 1) & ~1) : 2];
            const uint32_t mthr = load_rec<Model::n_upd>(crec + (size_t)p0 * 8, rr);
            F xx[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) xx[v] = x[v][k];
            int st;
            if constexpr (Model::separable) {
              F basis;
              st = update_separable<Model, F>(dtF, xx, rr, basis, s_pf, S, idv[k], step, p0);
              const long long q = quantize_fast(basis, qe0, qs0, my_clamp, my_err);
              if constexpr (AGG) {
                qv[k] = q;
                has_q[k] = true;
              } else {
                acc_add(&sacc[p0], q);
              }
            } else {
              F ctb[NC];
              st = update_general_of<Model, F>(dtF, xx, rr, ctb, s_pf, S, idv[k], step, p0);
#pragma unroll
              for (int j = 0; j < NC; ++j) {
                const double val = __dmul_rn(S.weight, (double)ctb[j]);
                const long long q = quantize(val, S.q_exp[j], my_clamp, my_err);
                acc_add(&sacc[p0 * NC + j], q);
              }
            }
#pragma unroll
            for (int v = 0; v < NV; ++v) x[v][k] = xx[v];
            if (st == kDivision) {
              bits |= 1u << k;
              S.bpos[first + k] = p0;
              ++my_req;
            }
            uint32_t p = p0;
            if (do_move) {
              if (draw_int(r[0]) < mthr) {
                p = (uint32_t)next_compartment(mrow, S.mrow16, p0, K, (int)draw_int(r[1]));
                ++my_move;
              }
              pv[k] = p;
            }
            if (n_out > 0) {
              ah[k] = age_add_fast(ah[k], ak);  // ages(i, 0) += d_t (double)
              for (unsigned o = 0; o < n_out; ++o) {
                if (S.outlet_idx[o] == p) {
                  if (S.outlet_flow[o] != 0.0 && draw_int(r[2]) > S.exit_thr[o]) {
                    stv[k] = kExit;
                    if (S.probe_cap) probe_set(S, kProbeLeaving, (double)ah[k]);  // before the reset
                    ah[k] = 0.0f;
                    ++my_exit;
                    st_changed = true;
                  }
                  break;
                }
              }
            }
          }
#pragma unroll
          for (int v = 0; v < NV; ++v) st_stream<F, PPT>(state + (size_t)v * cap + first, x[v]);
          if (do_move) st_stream<uint32_t, PPT>(S.pos + first, pv);
          if (n_out > 0) st_stream<float, PPT>(S.age_h + first, ah);
          st_stream<float, PPT>(S.age_d + first, ad);
          if (st_changed) st_stream<uint8_t, PPT>(S.status + first, stv);
        }
        if constexpr (Model::separable && AGG) {
          // tiny domains: contributions (to the compartment before the move,
          // p0s) summed per compartment across the warp first
#pragma unroll
          for (int k = 0; k < PPT; ++k) warp_aggregated_add(sacc, p0s[k], qv[k], has_q[k]);
        }
#pragma unroll
        for (int k = 0; k < PPT; ++k) n_inact += (first + k < n_used && stv[k] != kIdle) ? 1u : 0u;
        // birth-request bits: slot first+k -> bit (first+k) % 32 of word (first+k) / 32
        constexpr int lanes_per_word = 32 / PPT;
        unsigned w = bits << ((lane % lanes_per_word) * PPT);
#pragma unroll
        for (int o = 1; o < lanes_per_word; o <<= 1) w |= __shfl_xor_sync(0xffffffffu, w, o);
        if (lane % lanes_per_word == 0) S.bmask[first >> 5] = w;
        const unsigned nb = __reduce_add_sync(0xffffffffu, (unsigned)__popc(bits));
        const unsigned ni = __reduce_add_sync(0xffffffffu, n_inact);
        if (lane == 0) {
          const unsigned t = (unsigned)(c / kTile);  // a chunk lies inside one tile
          if (nb) atomicAdd(S.tile_births + t, nb);
          if (ni) atomicAdd(S.tile_inactive + t, ni);
        }
      }
    }
  }
  if (cur >= 0) flush();
}

// ---------------------------------------------------------------------------
// k_cycle_tma: the same per-particle work as k_cycle, with the particle
// arrays of each 1024-slot tile staged in shared memory by the copy engine.
// A producer warp (one thread) takes live tiles: half of them as an even
// contiguous share per block, the rest from a global ticket by guided
// self-scheduling (half of an even share of what is left per grab, taken
// one run ahead: long runs of one scenario first, single tiles at the end,
// so uneven scenarios of a batch finish together), and issues bulk copies
// (cp.async.bulk, completion on a "full" mbarrier per stage) of the tile's
// read state variables, compartments, ids, ages and statuses, STAGES tiles
// ahead, with the tile's scenario and extent in the stage's meta record.
// THREADS consumer threads wait on the stage, process slots r*THREADS + tid
// from shared memory, write results straight to global memory (stores that
// do not allocate in L1), and release the stage on its "empty" mbarrier.  The loads in
// flight no longer live in registers, so the memory pipeline stays full at
// any occupancy.  Every wait is bounded; consumers vote after each wait, so
// if one gives up (BMC_ERR_TIMEOUT) all stop at the same point with their
// barriers matched, the producer issues nothing more and drains its copies
// in flight.  SCATTER (ScatterForm) chooses where the contributions are
// summed: the shared accumulator (plain, warp-aggregated or in copies,
// flushed to the scenario's global accumulator), or, for domains whose
// shared accumulator would not leave two blocks per SM, the global
// accumulator directly (the dynamic shared memory then holds the stages
// only).

__host__ __device__ constexpr unsigned popcount_c(unsigned v) { return v == 0u ? 0u : (v & 1u) + popcount_c(v >> 1); }

// Tile held by a stage of k_cycle_tma (s < 0: no tile left).
struct TileMeta {
  int s;
  unsigned n_in;
  unsigned long long base;
};

// Fields of the scenario a k_cycle_tma block is working on.
template <class F>
struct CycleScen {
  unsigned long long seed, cap;
  const F* crec;
  const int2* mrow;
  const int32_t* mrow16;
  F* state;
  unsigned n_c, K, step, n_out;
  F dtF;
  float dtf;
  AgeStep ak;
  int qe0;
  float qs0;                      // quantize_scale(qe0)
  unsigned rep_mask, rep_stride;  // accumulator copies - 1, copy stride
};

template <class Model, class F>
struct TileStage {
  static constexpr unsigned NV = Model::n_var;
  static constexpr unsigned RV = popcount_c(Model::read_mask & ((1u << NV) - 1u));
  static constexpr unsigned off_x = 0;
  static constexpr unsigned off_pos = RV * kTile * (unsigned)sizeof(F);
  static constexpr unsigned off_id = off_pos + kTile * 4u;
  static constexpr unsigned off_ad = off_id + kTile * 4u;
  static constexpr unsigned off_ah = off_ad + kTile * 4u;
  static constexpr unsigned off_st = off_ah + kTile * 4u;
  static constexpr unsigned bytes = (off_st + kTile + 127u) & ~127u;
  // rank of state variable v among the read ones
  __host__ __device__ static constexpr unsigned rank(unsigned v) { return popcount_c(Model::read_mask & ((1u << v) - 1u)); }
};

template <class Model, class F, int THREADS, int MINB, int STAGES, int SCATTER>
__global__ void __launch_bounds__(THREADS + 32, MINB)
    k_cycle_tma(const ScenDev* __restrict__ sc, int n_scen, BatchCtl* __restrict__ bctl) {
  constexpr bool AGG = SCATTER == kScatterWarp;
  constexpr bool COPIES = SCATTER == kScatterCopied;
  constexpr bool GLOBAL = SCATTER == kScatterGlobal;  // no shared accumulator
  using TS = TileStage<Model, F>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned long long* sacc = reinterpret_cast<unsigned long long*>(smem_raw);
  __shared__ unsigned long long s_full[STAGES], s_empty[STAGES];
  __shared__ unsigned long long s_cnt[5];
  __shared__ F s_pf[16];
  __shared__ unsigned s_abort;
  constexpr int NV = Model::n_var;
  constexpr int NC = Model::n_ctb;
  constexpr int NA = Model::separable ? 1 : NC;
  constexpr unsigned PPT = kTile / THREADS;
  static_assert(kTile % THREADS == 0 && THREADS % 32 == 0, "tile must split evenly");
  unsigned char* const stages = smem_raw + (dynamic_smem_bytes() - (unsigned)STAGES * TS::bytes);
  const int tid = threadIdx.x;
  const unsigned total = bctl->total_live;
  const unsigned* live_base = bctl->live_base;
  __shared__ TileMeta s_meta[STAGES];  // tile of each stage, written by the producer
  if (tid == 0) {
    for (int k = 0; k < STAGES; ++k) {
      mbar_init(&s_full[k], 1u);
      mbar_init(&s_empty[k], (unsigned)THREADS);
    }
    s_abort = 0u;
    fence_barrier_init();
  }
  __syncthreads();
  if (total == 0) return;

  if (tid >= THREADS) {
    // ---- producer -------------------------------------------------------
    if (tid != THREADS) return;
    int hint = -1;
    unsigned issued = 0;
    bool ok = true;
    // first half of the tiles: an even contiguous share per block, taken
    // without atomics; the rest from the ticket by guided self-scheduling
    const unsigned c0 = (total >> 1) / gridDim.x;
    const unsigned s0 = c0 * gridDim.x;
    unsigned next = c0 * blockIdx.x, end = next + c0;  // tiles of the current run
    unsigned pn = 0, pe = 0;                           // run taken ahead
    bool ahead = false;
    auto grab = [&]() {
      // half of an even share of what is left: long runs while much is
      // left, single tiles at the end
      const unsigned seen = s0 + atomicAdd(&bctl->ticket, 0u);
      const unsigned left = seen < total ? total - seen : 0u;
      const unsigned c = max(1u, left / (2u * gridDim.x));
      pn = s0 + atomicAdd(&bctl->ticket, c);
      pe = min(pn + c, total);
      ahead = true;
    };
    for (unsigned k = 0;; ++k) {
      const unsigned stg = k % STAGES, use = k / STAGES;
      if (use > 0 && !mbar_wait_bounded(&s_empty[stg], (use - 1u) & 1u, &s_abort)) {
        ok = false;
        break;
      }
      if (s_abort) {
        ok = false;
        break;
      }
      if (next >= end) {
        if (!ahead) grab();
        next = pn;
        end = pe;
        ahead = false;
        hint = -1;
      }
      TileMeta& m = s_meta[stg];
      if (next >= total) {
        // no tile left: the stage completes without bytes and says so
        m.s = -1;
        mbar_arrive(&s_full[stg]);
        issued = k;
        break;
      }
      const unsigned g = next++;
      const int s = scen_of_live(live_base, n_scen, g, hint);
      hint = s;
      const ScenDev& S = sc[s];
      const unsigned long long base = (unsigned long long)(g - __ldg(live_base + s)) * kTile;
      const unsigned long long n_used = S.ctl->n_used;
      const unsigned n_in = (unsigned)(n_used - base < kTile ? n_used - base : kTile);
      m.s = s;
      m.n_in = n_in;
      m.base = base;
      // whole 16-slot groups: every copy is a multiple of 16 bytes and stays
      // inside the tile (capacity is a whole number of tiles)
      const unsigned n16 = (n_in + 15u) & ~15u;
      const bool with_ah = S.n_outlets > 0;
      const unsigned tx = TS::RV * n16 * (unsigned)sizeof(F) + n16 * 13u + (with_ah ? n16 * 4u : 0u);
      unsigned char* buf = stages + stg * TS::bytes;
      fence_proxy_async();
      mbar_arrive_expect_tx(&s_full[stg], tx);
      const F* state = reinterpret_cast<const F*>(S.state);
#pragma unroll
      for (int v = 0; v < NV; ++v)
        if ((Model::read_mask >> v) & 1u)
          bulk_g2s(buf + TS::off_x + TS::rank((unsigned)v) * kTile * sizeof(F), state + (size_t)v * S.cap + base,
                   n16 * (unsigned)sizeof(F), &s_full[stg]);
      bulk_g2s(buf + TS::off_pos, S.pos + base, n16 * 4u, &s_full[stg]);
      bulk_g2s(buf + TS::off_id, S.id + base, n16 * 4u, &s_full[stg]);
      bulk_g2s(buf + TS::off_ad, S.age_d + base, n16 * 4u, &s_full[stg]);
      if (with_ah) bulk_g2s(buf + TS::off_ah, S.age_h + base, n16 * 4u, &s_full[stg]);
      bulk_g2s(buf + TS::off_st, S.status + base, n16, &s_full[stg]);
      issued = k + 1;
      // take the next run while this tile's copies land
      if (next >= end && !ahead) grab();
    }
    if (!ok) {
      s_abort = 1u;
      // copies of the last (up to STAGES) issued tiles may still be landing
      unsigned zero = 0u;
      const unsigned first = issued > (unsigned)STAGES ? issued - (unsigned)STAGES : 0u;
      for (unsigned j = first; j < issued; ++j)
        (void)mbar_wait_bounded(&s_full[j % STAGES], (j / STAGES) & 1u, &zero);
    }
    return;
  }

  // ---- consumers ----------------------------------------------------------
  const int lane = tid & 31;
  const unsigned warp = (unsigned)tid >> 5;
  int cur = -1;
  bool aborted = false;
  unsigned long long since_flush = 0;
  // per-thread counts between flushes (at most kFlushParticles slots)
  unsigned my_req = 0, my_exit = 0, my_move = 0, my_clamp = 0;
  unsigned my_err = 0;

  // fields of the current scenario, kept in shared memory (written by
  // thread 0 when the scenario changes) rather than in registers
  __shared__ CycleScen<F> sr;

  auto flush = [&]() {
    consumer_sync(THREADS);
    const ScenDev& P = sc[cur];
    const unsigned n_ent = P.n_c * NA;
    const unsigned copies = COPIES ? sr.rep_mask + 1u : 1u, cstride = sr.rep_stride;
    if (!GLOBAL && !aborted)
      for (unsigned e = tid; e < n_ent; e += THREADS) {
        unsigned long long u = sacc[e];
        for (unsigned c = 1; c < copies; ++c) u += sacc[e + c * cstride];
        const long long p = (long long)u;
        if (p != 0) {
          atomicAdd(reinterpret_cast<unsigned long long*>(P.acc_hi + e), (unsigned long long)(p >> 32));
          atomicAdd(P.acc_lo + e, (unsigned long long)p & 0xffffffffull);
        }
      }
    if (tid < 5) s_cnt[tid] = 0ull;
    consumer_sync(THREADS);
    const unsigned long long r0 = warp_sum_u64(my_req), r1 = warp_sum_u64(my_exit);
    const unsigned long long r2 = warp_sum_u64(my_move), r3 = warp_sum_u64(my_clamp);
    unsigned e4 = my_err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e4 |= __shfl_xor_sync(0xffffffffu, e4, o);
    if (lane == 0) {
      atomicAdd(&s_cnt[0], r0);
      atomicAdd(&s_cnt[1], r1);
      atomicAdd(&s_cnt[2], r2);
      atomicAdd(&s_cnt[3], r3);
      atomicOr(reinterpret_cast<unsigned*>(&s_cnt[4]), e4);
    }
    consumer_sync(THREADS);
    if (tid == 0) {
      Control* c = P.ctl;
      if (s_cnt[0]) atomicAdd(&c->req_div, s_cnt[0]);
      if (s_cnt[1]) atomicAdd(&c->exits, s_cnt[1]);
      if (s_cnt[2]) atomicAdd(&c->moves, s_cnt[2]);
      if (s_cnt[3]) atomicAdd(&c->clamped, s_cnt[3]);
      const unsigned ev = *reinterpret_cast<unsigned*>(&s_cnt[4]);
      if (ev) atomicOr(&c->error, ev);
    }
    my_req = my_exit = my_move = my_clamp = 0u;
    my_err = 0u;
  };

  for (unsigned k = 0;; ++k) {
    const unsigned stg = k % STAGES, use = k / STAGES;
    // every consumer agrees whether the stage arrived: if one wait gives up,
    // all stop here together, so their barriers stay matched
    const bool ok = mbar_wait_bounded(&s_full[stg], use & 1u, &s_abort);
    if (consumer_any(!ok, THREADS)) {
      aborted = true;
      my_err |= 16u;
      if (tid == 0) {
        s_abort = 1u;
        if (cur < 0) atomicOr(&sc[0].ctl->error, 16u);
      }
      break;
    }
    const TileMeta m = s_meta[stg];
    if (m.s < 0) break;  // no tile left
    const int s = m.s;
    const ScenDev& S = sc[s];
    const unsigned long long base = m.base;
    const unsigned n_in = m.n_in;
    if (s != cur || since_flush + n_in > kFlushParticles) {
      if (cur >= 0) flush();
      const bool copied = Model::separable && COPIES && S.n_c <= kScatterCopyMaxCompartments;
      const unsigned n_zero = copied ? kAccCopies * scatter_stride(S.n_c) : S.n_c * NA;
      // the copies must end before the stage buffers (a launch sized for one
      // accumulator would have them overwrite tiles in flight): refuse
      if constexpr (COPIES)
        if ((size_t)n_zero * 8u > (size_t)(stages - smem_raw)) {
          aborted = true;
          my_err |= 32u;  // BMC_ERR_SMEM
        }
      if (!GLOBAL && !aborted)
        for (unsigned e = tid; e < n_zero; e += THREADS) sacc[e] = 0ull;
      if (tid < 16) s_pf[tid] = (F)S.params[tid];
      cur = s;
      since_flush = 0;
      if (tid == 0) {
        sr.n_c = S.n_c;
        sr.K = S.K;
        sr.step = S.ctl->step;
        sr.seed = S.seed;
        sr.cap = S.cap;
        sr.dtF = (F)S.dt;
        sr.dtf = (float)S.dt;
        sr.ak = age_step(S.dt);
        sr.n_out = S.n_outlets;
        sr.qe0 = S.q_exp[0];
        sr.qs0 = quantize_scale(S.q_exp[0]);
        sr.crec = reinterpret_cast<const F*>(S.crec);
        sr.mrow = S.mrow;
        sr.mrow16 = S.mrow16;
        sr.state = reinterpret_cast<F*>(S.state);
        sr.rep_mask = copied ? kAccCopies - 1u : 0u;
        sr.rep_stride = copied ? scatter_stride(S.n_c) : 0u;
      }
      consumer_sync(THREADS);
    }
    since_flush += n_in;
    const unsigned char* buf = stages + stg * TS::bytes;
    const F* bx = reinterpret_cast<const F*>(buf + TS::off_x);
    const uint32_t* bpos = reinterpret_cast<const uint32_t*>(buf + TS::off_pos);
    const uint32_t* bid = reinterpret_cast<const uint32_t*>(buf + TS::off_id);
    const float* bad = reinterpret_cast<const float*>(buf + TS::off_ad);
    const float* bah = reinterpret_cast<const float*>(buf + TS::off_ah);
    const uint8_t* bst = buf + TS::off_st;
    unsigned nb_t = 0u, ni_t = 0u;
    // Models with few state variables keep the scenario fields every slot
    // reads in registers for the tile (measured: batched Monod cycle -1.6 %);
    // the others read them from shared memory each time, as more live
    // registers would spill there (measured: FP64 lattice cycle +6 %).
    constexpr bool kFieldsInRegs = Model::n_var <= 2 && !AGG;
    const unsigned long long t_seed = kFieldsInRegs ? sr.seed : 0ull;
    const unsigned t_step = kFieldsInRegs ? sr.step : 0u, t_nc = kFieldsInRegs ? sr.n_c : 0u;
    const F* const t_crec = kFieldsInRegs ? sr.crec : nullptr;
#pragma unroll 2
    for (unsigned r = 0; r < PPT; ++r) {
      const unsigned slot = r * THREADS + (unsigned)tid;
      const bool act = !aborted && slot < n_in;
      uint8_t stv = act ? bst[slot] : (uint8_t)kIdle;
      const bool idle = act && stv == kIdle;
      bool div = false;
      bool has_q = false;  // tiny domains: quantised basis, scattered warp-aggregated
      long long qv = 0;
      uint32_t qkey = 0u;
      if (idle) {
        const unsigned long long gi = base + slot;
        const uint32_t p0 = bpos[slot];
        if (p0 >= (kFieldsInRegs ? t_nc : sr.n_c)) {
          my_err |= 1u;
        } else {
          uint32_t rd[4];
          philox_raw(kFieldsInRegs ? t_seed : sr.seed, bid[slot], kFieldsInRegs ? t_step : sr.step, 0u, rd);
          // ages(i, 1) += d_t in the model's float type
          const float ad = sizeof(F) == 8 ? age_add_fast(bad[slot], sr.ak) : __fadd_rn(bad[slot], sr.dtf);
          F rr[Model::n_upd > 0 ? ((Model::n_upd + 1) & ~1) : 2];
          const uint32_t mthr = load_rec<Model::n_upd>((kFieldsInRegs ? t_crec : sr.crec) + (size_t)p0 * 8, rr);
          F xx[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v)
            if ((Model::read_mask >> v) & 1u) xx[v] = bx[TS::rank((unsigned)v) * kTile + slot];
          int st;
          if constexpr (Model::separable) {
            F basis;
            st = update_separable<Model, F>(sr.dtF, xx, rr, basis, s_pf, S, bid[slot], sr.step, p0);
            const long long q = quantize_fast(basis, sr.qe0, sr.qs0, my_clamp, my_err);
            if constexpr (AGG) {
              qv = q;
              qkey = p0;
              has_q = true;
            } else {
              if constexpr (COPIES)
                acc_add(&sacc[p0 + ((unsigned)lane & sr.rep_mask) * sr.rep_stride], q);
              else if constexpr (GLOBAL)
                acc_add_global(S.acc_hi + p0, S.acc_lo + p0, q);
              else
                acc_add(&sacc[p0], q);
            }
          } else {
            F ctb[NC];
            st = update_general_of<Model, F>(sr.dtF, xx, rr, ctb, s_pf, S, bid[slot], sr.step, p0);
#pragma unroll
            for (int j = 0; j < NC; ++j) {
              const double val = __dmul_rn(S.weight, (double)ctb[j]);
              const long long q = quantize(val, S.q_exp[j], my_clamp, my_err);
              if constexpr (GLOBAL)
                acc_add_global(S.acc_hi + (size_t)p0 * NC + j, S.acc_lo + (size_t)p0 * NC + j, q);
              else
                acc_add(&sacc[p0 * NC + j], q);
            }
          }
#pragma unroll
          for (int v = 0; v < NV; ++v) st_na(sr.state + (size_t)v * sr.cap + gi, xx[v]);
          if (st == kDivision) {
            div = true;
            S.bpos[gi] = p0;
            ++my_req;
          }
          uint32_t p = p0;
          if ((sr.n_c > 1u)) {
            if (draw_int(rd[0]) < mthr) {
              p = (uint32_t)next_compartment(sr.mrow, sr.mrow16, p0, sr.K, (int)draw_int(rd[1]));
              ++my_move;
            }
            st_na(S.pos + gi, p);
          }
          if (sr.n_out > 0) {
            float ah = age_add_fast(bah[slot], sr.ak);  // ages(i, 0) += d_t (double)
            for (unsigned o = 0; o < sr.n_out; ++o) {
              if (S.outlet_idx[o] == p) {
                if (S.outlet_flow[o] != 0.0 && draw_int(rd[2]) > S.exit_thr[o]) {
                  stv = kExit;
                  if (S.probe_cap) probe_set(S, kProbeLeaving, (double)ah);  // before the reset
                  ah = 0.0f;
                  ++my_exit;
                  S.status[gi] = kExit;
                }
                break;
              }
            }
            st_na(S.age_h + gi, ah);
          }
          st_na(S.age_d + gi, ad);
        }
      }
      if constexpr (Model::separable && AGG) warp_aggregated_add(sacc, qkey, qv, has_q);
      // birth-request word of the 32 slots this warp covers in round r
      const unsigned bits = __ballot_sync(0xffffffffu, div);
      const unsigned w0 = r * THREADS + warp * 32u;
      if (lane == 0 && w0 < n_in) S.bmask[(base + w0) >> 5] = bits;
      nb_t += (unsigned)__popc(bits);
      ni_t += __popc(__ballot_sync(0xffffffffu, act && stv != kIdle));
    }
    if (lane == 0) {
      const unsigned t = (unsigned)(base / kTile);
      if (nb_t) atomicAdd(S.tile_births + t, nb_t);
      if (ni_t) atomicAdd(S.tile_inactive + t, ni_t);
    }
    mbar_arrive(&s_empty[stg]);
  }
  if (cur >= 0) flush();
}

// ---------------------------------------------------------------------------
// k_plan: per scenario (grid x), blocks of 1024 threads over slices of
// kPlanSlice compartments (grid y):
//  1. every slice: exact accumulator totals -> sources of its compartments:
//     for a separable model src(j, s) = (w * coef_s(rates_j)) * B_j with B_j
//     the basis total of compartment j; for a general model src(j, s) =
//     total of w * ctb_s; accumulators cleared (FP64 work, spread over SMs);
// slice 0 only:
//  2. post_cycle decisions: inactive += exits; compaction iff inactive >
//     max(min_removal, n * ratio) (update_and_remove_inactive); room for
//     births = capacity - live particles after compaction;
//  3. scans of the per-tile counters (birth ranks, gap ranks ascending,
//     source ranks from the end);
//  4. control block advanced to the state after the step.
template <class Model, class F>
__global__ void __launch_bounds__(1024) k_plan(ScenDev* __restrict__ sc, BatchCtl* __restrict__ bctl) {
  const ScenDev& S = sc[blockIdx.x];
  Control* ctl = S.ctl;
  const int tid = threadIdx.x;
  __shared__ unsigned long long sh64[33];
  // (not scen_finished: slice 0 advances the step counter while the other
  // slices may still be starting)
  if (!ctl->cycling) {
    // nothing ran for this scenario: leave its state and a no-op plan
    if (blockIdx.y == 0 && tid == 0) {
      ctl->plan_births = 0ull;
      ctl->plan_overflow = 0ull;
      ctl->plan_compact = 0u;
      ctl->plan_to_remove = 0ull;
      ctl->plan_gaps = 0ull;
      ctl->plan_n_old = ctl->n_used;
      ctl->plan_n_after = ctl->n_used;
    }
    return;
  }

  const unsigned nsp = S.n_s;
  const F* rates = reinterpret_cast<const F*>(S.crec);
  // sources of this block's slice of compartments
  const unsigned jb = blockIdx.y * kPlanSlice;
  const unsigned je = min(jb + kPlanSlice, S.n_c);
  if (blockIdx.y == 0 && tid < (int)nsp && tid < kMaxSpecies) {
    const double a = ctl->mb_new[tid], b = ctl->mb_exp[tid];
    const double den = fabs(a) > 1e-300 ? fabs(a) : 1e-300;
    ctl->mass_balance[tid] = fabs(a - b) / den;
    ctl->mb_new[tid] = 0.0;
    ctl->mb_exp[tid] = 0.0;
  }
  if constexpr (Model::separable) {
    for (unsigned j = jb + tid; j < je; j += blockDim.x) {
      const double B = fixed_to_double(S.acc_hi[j], S.acc_lo[j], S.q_scale_up[0]);
      S.acc_hi[j] = 0;
      S.acc_lo[j] = 0ull;
      F rr[kMaxRates];
#pragma unroll
      for (int k = 0; k < Model::n_rates; ++k) rr[k] = rates[(size_t)j * 8 + rate_slot<Model>(k)];
      for (unsigned sp = 0; sp < nsp; ++sp) {
        double v = 0.0;
        if (sp < (unsigned)Model::n_ctb) v = __dmul_rn(__dmul_rn(S.weight, (double)Model::coef(rr, (int)sp)), B);
        S.src[(size_t)j * nsp + sp] = v;
      }
    }
  } else {
    const unsigned nc = Model::n_ctb;
    for (unsigned e = jb * nsp + tid; e < je * nsp; e += blockDim.x) {
      const unsigned j = e / nsp;
      const unsigned sp = e - j * nsp;
      double v = 0.0;
      if (sp < nc) {
        const unsigned idx = j * nc + sp;
        v = fixed_to_double(S.acc_hi[idx], S.acc_lo[idx], S.q_scale_up[sp]);
        S.acc_hi[idx] = 0;
        S.acc_lo[idx] = 0ull;
      }
      S.src[e] = v;
    }
  }
  if (blockIdx.y != 0) return;
  // The plan: every thread loads the control words it reads and computes the
  // same plan; after one barrier (every load performed) thread 0 writes it
  // back while the others go on to the scans, which need nothing from it.
  const unsigned long long n = ctl->n_used;
  const unsigned long long req = ctl->req_div;
  const unsigned long long c_exits = ctl->exits, c_moves = ctl->moves, c_next = ctl->next_id;
  const unsigned long long c_inactive = ctl->inactive;
  const unsigned c_step = ctl->step, c_tadv = ctl->t_advance;
  const double c_trel = ctl->t_rel;
  const unsigned long long inactive_after = c_inactive + c_exits;
  const unsigned long long ratio_thr = (unsigned long long)((double)n * S.dead_ratio);
  const unsigned long long thr = S.min_removal > ratio_thr ? S.min_removal : ratio_thr;
  int compact = inactive_after > thr ? 1 : 0;
  unsigned long long rm = compact ? inactive_after : 0ull;
  const bool bad_rm = rm > n;
  if (bad_rm) {
    rm = 0ull;
    compact = 0;
  }
  const unsigned long long after = n - rm;
  const unsigned long long room = S.cap > after ? S.cap - after : 0ull;
  const unsigned long long n_births = req < room ? req : room;
  __syncthreads();
  if (tid == 0) {
    if (bad_rm) ctl->error |= 8u;
    ctl->plan_n_old = n;
    ctl->plan_to_remove = rm;
    ctl->plan_n_after = after;
    ctl->plan_births = n_births;
    ctl->plan_overflow = req - n_births;
    ctl->plan_next_id = c_next;
    ctl->plan_step = c_step;
    ctl->plan_compact = (unsigned)compact;
    ctl->plan_gaps = 0ull;
    // every division request of the step is a division-time event, refused
    // or not (model_kernel.hpp L245-L251); k_divide records them in slot order
    const unsigned long long pb = ctl->probe_n[kProbeDivision];
    ctl->plan_probe_base = pb;
    if (S.probe_cap) ctl->probe_n[kProbeDivision] = pb + req;
    // the cycle's event counts (model_kernel.hpp L253-L259, move_kernel.hpp
    // L434 and L643): a division request is a NewParticle event whether or
    // not it finds room
    ctl->events[0] += req;
    ctl->events[1] += c_exits;
    ctl->events[2] += c_moves;
    ctl->events[4] += req - n_births;
    if (c_next + n_births > 0x100000000ull) ctl->error |= 4u;
    ctl->n_used = after + n_births;
    ctl->inactive = compact ? 0ull : inactive_after;
    ctl->next_id = c_next + n_births;
    if (S.n_maps > 0u) ctl->map_cur = (c_step / S.n_per_map) % S.n_maps;
    ctl->step = c_step + 1u;
    if (c_tadv) ctl->t_rel = __dadd_rn(c_trel, S.dt);  // SimulationUnit::advance
    ctl->last_births = n_births;
    ctl->last_exits = c_exits;
    ctl->last_moves = c_moves;
    ctl->last_overflow = req - n_births;
    ctl->last_req_div = req;
    ctl->last_compacted = (unsigned)compact;
    unsigned fl = 0u;
    if (req > 0ull) fl |= kFlagDivide;
    if (compact && after > 0ull && rm < n) fl |= kFlagCompact;
    if (n_births > 0ull) fl |= kFlagMerge;
    if (fl) atomicOr(&bctl->flags, fl);
  }
  const unsigned n_t = (unsigned)((n + kTile - 1) / kTile);
  const unsigned* __restrict__ births = S.tile_births;
  const unsigned* __restrict__ inact = S.tile_inactive;
  if (req > 0) {
    // birth ranks: births in earlier tiles
    block_exscan_items(
        n_t, [&](unsigned t) { return (unsigned long long)births[t]; },
        [&](unsigned t, unsigned long long pre, unsigned long long) { S.tile_boff[t] = (unsigned)pre; }, sh64);
  }
  if (compact && after > 0 && rm < n) {
    // gap offsets for tiles t <= after / kTile (ascending prefix of inactive)
    const unsigned tg_end = min((unsigned)(after / kTile) + 1u, n_t);
    block_exscan_items(
        tg_end, [&](unsigned t) { return (unsigned long long)inact[t]; },
        [&](unsigned t, unsigned long long pre, unsigned long long) { S.tile_goff[t] = (unsigned)pre; }, sh64);
    // source offsets for tiles t >= after / kTile: idle slots in later tiles
    const unsigned ts_begin = (unsigned)(after / kTile);
    auto idle = [&](unsigned i) {
      const unsigned t = ts_begin + i;
      const unsigned long long valid = min((unsigned long long)kTile, n - (unsigned long long)t * kTile);
      return valid - inact[t];
    };
    block_exscan_items(
        n_t - ts_begin, idle,
        [&](unsigned i, unsigned long long pre, unsigned long long tot) {
          S.tile_soff[ts_begin + i] = (unsigned)(tot - pre - idle(i));
        },
        sh64);
  }
}

// k_divide: (a) Model::division for the requests of this step, in slot
// order, the first `plan_births` succeeding (handle_division,
// particles_container.hpp L561-L575: mother updated in place, child into the
// buffer, ages(mother,1) = 0); (b) the compaction lists: j-th non-Idle slot
// of [0, n_after) and j-th Idle slot of [n_after, n) counted from the end
// (CompactParticlesFunctor run in slot order).  256 threads x 4 slots.
template <class Model, class F>
__global__ void __launch_bounds__(256) k_divide(const ScenDev* __restrict__ sc, int n_scen,
                                               const BatchCtl* __restrict__ bctl) {
  constexpr int NV = Model::n_var;
  __shared__ unsigned sh[33];
  if (!(bctl->flags & (kFlagDivide | kFlagCompact))) return;
  const unsigned total_tiles = bctl->total_tiles;
  const int tid = threadIdx.x;
  int s = -1;
  for (unsigned g = blockIdx.x; g < total_tiles; g += gridDim.x) {
    s = scen_of_tile(sc, n_scen, g, s);
    const ScenDev& S = sc[s];
    const Control* ctl = S.ctl;
    const unsigned long long n_old = ctl->plan_n_old;
    const unsigned t = g - S.tile_base;
    const unsigned long long base = (unsigned long long)t * kTile;
    if (base >= n_old) continue;
    const unsigned long long req = ctl->plan_births + ctl->plan_overflow;
    const bool cmp = ctl->plan_compact != 0u && ctl->plan_n_after > 0ull && ctl->plan_to_remove < n_old;
    if (req == 0ull && !cmp) continue;
    const unsigned long long first = base + (unsigned long long)tid * 4ull;
    const unsigned long long cap = S.cap;
    if (req > 0ull && S.tile_births[t] > 0u) {
      const unsigned word = S.bmask[first >> 5];
      const unsigned bits = (word >> (first & 31ull)) & 0xFu;
      unsigned tot;
      unsigned rank = S.tile_boff[t] + block_exscan_u32((unsigned)__popc(bits), sh, &tot);
      const unsigned long long births = ctl->plan_births;
      F* state = reinterpret_cast<F*>(S.state);
      F* child_state = reinterpret_cast<F*>(S.child_state);
      for (int k = 0; k < 4; ++k) {
        if (!((bits >> k) & 1u)) continue;
        const unsigned long long slot = first + k;
        if (S.probe_cap) {
          // ages(i, 1) of the request, before a division resets it
          const unsigned long long j = ctl->plan_probe_base + rank;
          if (j < S.probe_cap) S.probe_buf[kProbeDivision][j] = (double)S.age_d[slot];
        }
        if (rank < births) {
          F x[NV], y[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) x[v] = state[(size_t)v * cap + slot];
          const Draws d = philox_draws(S.seed, S.id[slot], ctl->plan_step, 1u);
          Model::division(x, y, d.u, S.params);
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            state[(size_t)v * cap + slot] = x[v];
            child_state[(size_t)v * cap + rank] = y[v];
          }
          S.child_pos[rank] = S.bpos[slot];
          S.age_d[slot] = 0.0f;
        }
        ++rank;
      }
    }
    if (cmp) {
      const unsigned long long after = ctl->plan_n_after;
      unsigned gbits = 0u, sbits = 0u;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const unsigned long long slot = first + k;
        if (slot >= n_old) continue;
        const bool idle = S.status[slot] == kIdle;
        if (slot < after && !idle) gbits |= 1u << k;
        if (slot >= after && idle) sbits |= 1u << k;
      }
      unsigned gtot, stot;
      const unsigned gpre = block_exscan_u32((unsigned)__popc(gbits), sh, &gtot);
      const unsigned spre = block_exscan_u32((unsigned)__popc(sbits), sh, &stot);
      if (gbits) {
        unsigned r = S.tile_goff[t] + gpre;
        for (int k = 0; k < 4; ++k)
          if ((gbits >> k) & 1u) S.gap_slot[r++] = (uint32_t)(first + k);
      }
      if (sbits) {
        unsigned i_loc = 0;
        for (int k = 0; k < 4; ++k) {
          if (!((sbits >> k) & 1u)) continue;
          const unsigned larger = stot - spre - i_loc - 1u;  // sources after this slot in the tile
          S.src_slot[S.tile_soff[t] + larger] = (uint32_t)(first + k);
          ++i_loc;
        }
      }
      if (t == (unsigned)(after / kTile) && tid == 0) {
        Control* c = const_cast<Control*>(ctl);
        c->plan_gaps = (unsigned long long)S.tile_goff[t] + gtot;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_compact: copy the j-th source particle into the j-th gap (all fields);
// k_merge: append the children after the live particles with ages 0 and
// fresh ids (InsertFunctor, particles_container.hpp L403-L447).
template <int NV, class F>
__global__ void __launch_bounds__(256) k_compact(const ScenDev* __restrict__ sc, int n_scen,
                                                const BatchCtl* __restrict__ bctl) {
  if (!(bctl->flags & kFlagCompact)) return;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (int s = 0; s < n_scen; ++s) {
    const ScenDev& S = sc[s];
    const Control* ctl = S.ctl;
    if (!ctl->plan_compact) continue;
    const unsigned long long gaps = ctl->plan_gaps;
    const unsigned long long cap = S.cap;
    const unsigned long long after = ctl->plan_n_after, n_old = ctl->plan_n_old;
    F* state = reinterpret_cast<F*>(S.state);
    for (unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; j < gaps; j += stride) {
      const unsigned long long dst = S.gap_slot[j], src = S.src_slot[j];
      if (dst >= after || src < after || src >= n_old) {  // lists inconsistent: record, skip
        atomicOr(&S.ctl->error, 8u);
        continue;
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) state[(size_t)v * cap + dst] = state[(size_t)v * cap + src];
      S.pos[dst] = S.pos[src];
      S.status[dst] = kIdle;
      S.age_h[dst] = S.age_h[src];
      S.age_d[dst] = S.age_d[src];
      S.id[dst] = S.id[src];
    }
  }
}

template <int NV, class F>
__global__ void __launch_bounds__(256) k_merge(const ScenDev* __restrict__ sc, int n_scen,
                                              const BatchCtl* __restrict__ bctl) {
  if (!(bctl->flags & kFlagMerge)) return;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (int s = 0; s < n_scen; ++s) {
    const ScenDev& S = sc[s];
    const Control* ctl = S.ctl;
    const unsigned long long births = ctl->plan_births;
    if (births == 0ull) continue;
    const unsigned long long after = ctl->plan_n_after;
    const unsigned long long id0 = ctl->plan_next_id;
    const unsigned long long cap = S.cap;
    F* state = reinterpret_cast<F*>(S.state);
    const F* child = reinterpret_cast<const F*>(S.child_state);
    for (unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; j < births; j += stride) {
      const unsigned long long dst = after + j;
#pragma unroll
      for (int v = 0; v < NV; ++v) state[(size_t)v * cap + dst] = child[(size_t)v * cap + j];
      S.pos[dst] = S.child_pos[j];
      S.status[dst] = kIdle;
      S.age_h[dst] = 0.0f;
      S.age_d[dst] = 0.0f;
      S.id[dst] = (uint32_t)(id0 + j);
    }
  }
}

// ---------------------------------------------------------------------------
// Set-up and diagnostics.

// Model::mass of every slot [0, n) (the mass column of the reference's
// particle dump, get_properties, apps/core/public/core/post_process.hpp
// L96-L98).
template <class Model, class F>
__global__ void k_mass(const ScenDev* __restrict__ sc, unsigned long long n, double* __restrict__ out) {
  const ScenDev& S = *sc;
  const F* state = reinterpret_cast<const F*>(S.state);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    F x[Model::n_var];
#pragma unroll
    for (int v = 0; v < Model::n_var; ++v) x[v] = state[(size_t)v * S.cap + i];
    out[i] = Model::mass(x, S.params);
  }
}

// InitFunctor (apps/libs/mc/src/unit.cpp L102-L137): model init from the
// particle's draws, position = lo + floor(u32 * span / 2^32), mass out.
template <class Model, class F>
__global__ void k_init(const ScenDev* __restrict__ sc, unsigned long long n, uint32_t lo, uint32_t span,
                       double* __restrict__ mass_out) {
  const ScenDev& S = *sc;
  constexpr int NV = Model::n_var;
  F* state = reinterpret_cast<F*>(S.state);
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t r[4];
    philox_raw(S.seed, (uint32_t)i, 0xFFFFFFFFu, 2u, r);
    float d[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) d[k] = (float)draw_int(r[k]) * 0x1p-24f;
    F x[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) x[v] = (F)0;
    Model::init(x, d, S.params);
#pragma unroll
    for (int v = 0; v < NV; ++v) state[(size_t)v * S.cap + i] = x[v];
    S.pos[i] = lo + __umulhi(r[0], span);
    S.status[i] = kIdle;
    S.age_h[i] = 0.0f;
    S.age_d[i] = 0.0f;
    S.id[i] = (uint32_t)i;
    mass_out[i] = Model::mass(x, S.params);
  }
}

// Move thresholds of every compartment for the current dt, into slot 7 of
// the compartment record: leave iff u < p = dt*Q/V, i.e. x < ceil(2^24 p)
// for the integer draw x.
template <class F>
__global__ void k_move_thr(ScenDev* __restrict__ sc) {
  const ScenDev& S = sc[blockIdx.y];
  F* rec = reinterpret_cast<F*>(S.crec);
  for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < S.n_c; c += gridDim.x * blockDim.x) {
    const double p = __ddiv_rn(__dmul_rn(S.dt, S.out_flow[c]), S.volume[c]);
    uint32_t t;
    if (p >= 1.0)
      t = (1u << 24) + 1u;
    else if (!(p > 0.0))
      t = 0u;
    else
      t = (uint32_t)ceil(__dmul_rn(p, 16777216.0));
    if constexpr (sizeof(F) == 4)
      rec[(size_t)c * 8 + 7] = __uint_as_float(t);
    else
      rec[(size_t)c * 8 + 7] = __longlong_as_double((long long)t);
  }
}

// k_flowmap: the flow-map cycle of the reference's main loop
// (host_specific.cpp L255-L266: when the transitioner advances, the next
// flow-map state replaces the domain -- volumes, neighbours, out-flows,
// cumulative probabilities, liquid transition).  At the start of step k the
// state in use is m = (k / n_per_map) % n_maps; when it differs from the one
// the domain arrays hold (ctl->map_cur, set by k_plan) it is copied in and
// the move thresholds of the compartment records are recomputed as
// k_move_thr does.  The outlet thresholds of m (computed on the host for the
// current dt) are written every step.  Grid: (blocks, scenarios).
template <class F>
__global__ void k_flowmap(ScenDev* __restrict__ sc) {
  ScenDev& S = sc[blockIdx.y];
  if (S.n_maps == 0u) return;
  const Control* ctl = S.ctl;
  if (scen_finished(S, ctl)) return;
  const unsigned m = (ctl->step / S.n_per_map) % S.n_maps;
  if (blockIdx.x == 0 && threadIdx.x < kMaxOutlets) S.exit_thr[threadIdx.x] = S.map_exit_thr[m * kMaxOutlets + threadIdx.x];
  if (m == ctl->map_cur) return;
  const unsigned n_c = S.n_c, K = S.K;
  const size_t o = (size_t)m * n_c;
  const unsigned stride = gridDim.x * blockDim.x;
  const unsigned t0 = blockIdx.x * blockDim.x + threadIdx.x;
  F* rec = reinterpret_cast<F*>(S.crec);
  for (unsigned c = t0; c < n_c; c += stride) {
    const double vol = S.map_volume[o + c], q = S.map_out_flow[o + c];
    const_cast<double*>(S.volume)[c] = vol;
    const_cast<double*>(S.vinv)[c] = S.map_vinv[o + c];
    const_cast<double*>(S.out_flow)[c] = q;
    const_cast<double*>(S.diag)[c] = S.map_diag[o + c];
    const double p = __ddiv_rn(__dmul_rn(S.dt, q), vol);
    uint32_t t;
    if (p >= 1.0)
      t = (1u << 24) + 1u;
    else if (!(p > 0.0))
      t = 0u;
    else
      t = (uint32_t)ceil(__dmul_rn(p, 16777216.0));
    if constexpr (sizeof(F) == 4)
      rec[(size_t)c * 8 + 7] = __uint_as_float(t);
    else
      rec[(size_t)c * 8 + 7] = __longlong_as_double((long long)t);
  }
  for (size_t e = t0; e < (size_t)n_c * K; e += stride) const_cast<int2*>(S.mrow)[e] = S.map_mrow[o * K + e];
  for (size_t e = t0; e < (size_t)n_c * 8; e += stride) {
    const unsigned k = (unsigned)(e & 7u);
    const size_t c = e >> 3;
    const int2* row = S.map_mrow + o * K + c * K;
    int32_t* r16 = const_cast<int32_t*>(S.mrow16) + c * 16;
    r16[k] = k < K ? row[k].x : INT32_MAX;
    r16[8 + k] = row[k < K ? k : K - 1].y;
  }
  const uint32_t* ptr = S.map_in_ptr + (size_t)m * (n_c + 1);
  for (unsigned c = t0; c <= n_c; c += stride) const_cast<uint32_t*>(S.in_ptr)[c] = ptr[c];
  const unsigned nnz = ptr[n_c];
  const size_t on = (size_t)m * S.map_nnz_max;
  for (unsigned e = t0; e < nnz; e += stride) {
    const_cast<uint32_t*>(S.in_idx)[e] = S.map_in_idx[on + e];
    const_cast<double*>(S.in_flow)[e] = S.map_in_flow[on + e];
  }
  if (S.map_g_nnz_max != 0u) {
    // the map's gas state: volumes (as inverses), transition and kla; the
    // gas masses are kept, as the liquid's (SimulationUnit::
    // updateScalarHydro and MassTransferModel::update, simulation.cpp
    // L120-L139)
    const size_t ne = (size_t)n_c * S.n_s;
    for (unsigned c = t0; c < n_c; c += stride) {
      const_cast<double*>(S.gvinv)[c] = S.map_gvinv[o + c];
      const_cast<double*>(S.g_diag)[c] = S.map_g_diag[o + c];
    }
    for (size_t e = t0; e < ne; e += stride) const_cast<double*>(S.kla)[e] = S.map_kla[(size_t)m * ne + e];
    const uint32_t* gptr = S.map_g_in_ptr + (size_t)m * (n_c + 1);
    for (unsigned c = t0; c <= n_c; c += stride) const_cast<uint32_t*>(S.g_in_ptr)[c] = gptr[c];
    const unsigned gnnz = gptr[n_c];
    const size_t gon = (size_t)m * S.map_g_nnz_max;
    for (unsigned e = t0; e < gnnz; e += stride) {
      const_cast<uint32_t*>(S.g_in_idx)[e] = S.map_g_in_idx[gon + e];
      const_cast<double*>(S.g_in_flow)[e] = S.map_g_in_flow[gon + e];
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers and the KernelSet factory.

namespace kset {
template <class Model, class F, int PPT, int THREADS, int MINB>
void launch_cycle_t(dim3 grid, dim3 block, size_t smem, cudaStream_t st, const ScenDev* sc, int n,
                    BatchCtl* b, int scatter) {
  (void)block;
  if (scatter == kScatterWarp)
    k_cycle<Model, F, PPT, THREADS, MINB, true><<<grid, THREADS, smem, st>>>(sc, n, b);
  else
    k_cycle<Model, F, PPT, THREADS, MINB, false><<<grid, THREADS, smem, st>>>(sc, n, b);
}
template <class Model, class F, int THREADS, int MINB, int STAGES>
void launch_cycle_tma_t(dim3 grid, dim3 block, size_t smem, cudaStream_t st, const ScenDev* sc, int n,
                        BatchCtl* b, int scatter) {
  (void)block;
  if (scatter == kScatterWarp)
    k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterWarp><<<grid, THREADS + 32, smem, st>>>(sc, n, b);
  else if (scatter == kScatterCopied)
    k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterCopied><<<grid, THREADS + 32, smem, st>>>(sc, n, b);
  else if (scatter == kScatterGlobal)
    k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterGlobal><<<grid, THREADS + 32, smem, st>>>(sc, n, b);
  else
    k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterPlain><<<grid, THREADS + 32, smem, st>>>(sc, n, b);
}
template <class Model, class F>
void launch_liquid_t(int n_scen, unsigned grid_x, cudaStream_t st, ScenDev* sc, BatchCtl* b, int do_scalar) {
  k_liquid<Model, F><<<dim3(grid_x, n_scen), kLiquidThreads, 0, st>>>(sc, b, do_scalar);
}
template <class Model, class F>
void launch_plan_t(int n_scen, unsigned slices, cudaStream_t st, ScenDev* sc, BatchCtl* b) {
  k_plan<Model, F><<<dim3(n_scen, slices), 1024, 0, st>>>(sc, b);
}
template <class Model, class F>
void launch_divide_t(dim3 grid, cudaStream_t st, const ScenDev* sc, int n, const BatchCtl* b) {
  k_divide<Model, F><<<grid, 256, 0, st>>>(sc, n, b);
}
template <class Model, class F>
void launch_compact_t(dim3 grid, cudaStream_t st, const ScenDev* sc, int n, const BatchCtl* b) {
  k_compact<Model::n_var, F><<<grid, 256, 0, st>>>(sc, n, b);
}
template <class Model, class F>
void launch_merge_t(dim3 grid, cudaStream_t st, const ScenDev* sc, int n, const BatchCtl* b) {
  k_merge<Model::n_var, F><<<grid, 256, 0, st>>>(sc, n, b);
}
template <class Model, class F>
void launch_init_t(dim3 grid, cudaStream_t st, const ScenDev* sc, unsigned long long n, uint32_t lo,
                   uint32_t span, double* mass) {
  k_init<Model, F><<<grid, 256, 0, st>>>(sc, n, lo, span, mass);
}
// Shared-memory limit and occupancy of both instantiations of a shape (the
// launch picks one per step); the occupancy reported is the smaller.
inline int setup_fn(const void* fn, int threads, size_t smem, int* blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, threads, smem);
}
inline int setup_pair(const void* f0, const void* f1, int threads, size_t smem, int* blocks_per_sm) {
  int b0 = 0, b1 = 0;
  int e = setup_fn(f0, threads, smem, &b0);
  if (e) return e;
  e = setup_fn(f1, threads, smem, &b1);
  *blocks_per_sm = b0 < b1 ? b0 : b1;
  return e;
}
template <class Model, class F, int PPT, int THREADS, int MINB>
int setup_cycle_t(size_t smem, int* blocks_per_sm) {
  return setup_pair(reinterpret_cast<const void*>(&k_cycle<Model, F, PPT, THREADS, MINB, false>),
                    reinterpret_cast<const void*>(&k_cycle<Model, F, PPT, THREADS, MINB, true>), THREADS, smem,
                    blocks_per_sm);
}
template <class Model, class F, int THREADS, int MINB, int STAGES>
int setup_cycle_tma_t(size_t smem, int* blocks_per_sm) {
  int b2 = 0;
  int e = setup_pair(reinterpret_cast<const void*>(&k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterPlain>),
                     reinterpret_cast<const void*>(&k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterWarp>),
                     THREADS + 32, smem, blocks_per_sm);
  if (e) return e;
  e = setup_fn(reinterpret_cast<const void*>(&k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterCopied>),
               THREADS + 32, smem, &b2);
  if (e) return e;
  if (b2 < *blocks_per_sm) *blocks_per_sm = b2;
  e = setup_fn(reinterpret_cast<const void*>(&k_cycle_tma<Model, F, THREADS, MINB, STAGES, kScatterGlobal>),
               THREADS + 32, smem, &b2);
  if (b2 < *blocks_per_sm) *blocks_per_sm = b2;
  return e;
}
inline int last_error_t() { return (int)cudaGetLastError(); }
template <class Model, class F>
void launch_mass_t(cudaStream_t st, const ScenDev* sc, unsigned long long n, double* out) {
  const unsigned long long blocks = (n + 255) / 256;
  k_mass<Model, F><<<(unsigned)(blocks < 4096 ? (blocks ? blocks : 1) : 4096), 256, 0, st>>>(sc, n, out);
}
template <class F>
void launch_move_thr_t(int n_scen, cudaStream_t st, ScenDev* sc) {
  k_move_thr<F><<<dim3(4, n_scen), 256, 0, st>>>(sc);
}
template <class F>
void launch_flowmap_t(int n_scen, cudaStream_t st, ScenDev* sc) {
  k_flowmap<F><<<dim3(8, n_scen), 256, 0, st>>>(sc);
}

template <class Model, class F>
KernelSet make_set(int model_id) {
  KernelSet k{};
  k.abi = kKernelSetAbi;
  k.n_var = Model::n_var;
  k.n_ctb = Model::n_ctb;
  k.model = model_id;
  k.f64 = sizeof(F) == 8;
  k.separable = Model::separable;
  k.cycle[0] = &launch_cycle_t<Model, F, 1, 256, 4>;
  k.cycle[1] = &launch_cycle_t<Model, F, 2, 256, 3>;
  k.cycle[2] = &launch_cycle_t<Model, F, 4, 256, 2>;
  k.cycle[3] = &launch_cycle_t<Model, F, 2, 512, 2>;
  k.cycle[4] = &launch_cycle_t<Model, F, 1, 1024, 1>;
  k.cycle_setup[0] = &setup_cycle_t<Model, F, 1, 256, 4>;
  k.cycle_setup[1] = &setup_cycle_t<Model, F, 2, 256, 3>;
  k.cycle_setup[2] = &setup_cycle_t<Model, F, 4, 256, 2>;
  k.cycle_setup[3] = &setup_cycle_t<Model, F, 2, 512, 2>;
  k.cycle_setup[4] = &setup_cycle_t<Model, F, 1, 1024, 1>;
  // staged (TMA) variants: 256 consumers with 3 stages, 512 consumers with 2
  k.cycle[5] = &launch_cycle_tma_t<Model, F, 256, 2, 3>;
  k.cycle[6] = &launch_cycle_tma_t<Model, F, 512, 2, 2>;
  k.cycle_setup[5] = &setup_cycle_tma_t<Model, F, 256, 2, 3>;
  k.cycle_setup[6] = &setup_cycle_tma_t<Model, F, 512, 2, 2>;
  for (int v = 0; v < kCycleVariants; ++v) k.cycle_extra_smem[v] = 0u;
  k.cycle_extra_smem[5] = 3u * TileStage<Model, F>::bytes;
  k.cycle_extra_smem[6] = 2u * TileStage<Model, F>::bytes;
  k.move_thr = &launch_move_thr_t<F>;
  k.flowmap = &launch_flowmap_t<F>;
  k.liquid = &launch_liquid_t<Model, F>;
  k.plan = &launch_plan_t<Model, F>;
  k.divide = &launch_divide_t<Model, F>;
  k.compact = &launch_compact_t<Model, F>;
  k.merge = &launch_merge_t<Model, F>;
  k.init = &launch_init_t<Model, F>;
  k.last_error = &last_error_t;
  k.mass = &launch_mass_t<Model, F>;
  return k;
}
}  // namespace kset

}  // namespace bmc

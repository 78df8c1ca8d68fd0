// bmc_api.cu -- the C-ABI of libbmc (declared in include/bmc.h).
//
// Host-side responsibilities: device memory of each scenario (one arena for
// the particle container, one for the domain and liquid state), the
// scenario descriptor the kernels read, the per-dt quantities (move
// probabilities on the device, the outlets' exit thresholds on the
// host), the step sequence and its CUDA graph, readback.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bmc.h"
#include "bmc_launch.h"

using bmc::BatchCtl;
using bmc::Control;
using bmc::kTile;
using bmc::ScenDev;

namespace {

thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};
std::atomic<unsigned long long> g_h2d{0}, g_d2h{0};

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define BMC_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(BMC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));      \
  } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

void count_copy(size_t n, cudaMemcpyKind kind) {
  if (kind == cudaMemcpyHostToDevice) g_h2d += n;
  if (kind == cudaMemcpyDeviceToHost) g_d2h += n;
}
cudaError_t counted_memcpy_async(void* dst, const void* src, size_t n, cudaMemcpyKind kind, cudaStream_t st) {
  count_copy(n, kind);
  return cudaMemcpyAsync(dst, src, n, kind, st);
}
cudaError_t counted_memcpy(void* dst, const void* src, size_t n, cudaMemcpyKind kind) {
  count_copy(n, kind);
  return cudaMemcpy(dst, src, n, kind);
}

// Carves 256-byte aligned arrays out of one allocation.
struct Carver {
  size_t off = 0;
  std::vector<std::pair<void**, size_t>> items;
  template <class T>
  void add(T** p, size_t n_elems) {
    items.emplace_back(reinterpret_cast<void**>(p), off);
    off = align_up(off + std::max<size_t>(n_elems, 1) * sizeof(T), 256);
  }
  void add_raw(void** p, size_t bytes) {
    items.emplace_back(p, off);
    off = align_up(off + std::max<size_t>(bytes, 1), 256);
  }
  void bind(void* base) {
    for (auto& it : items) *it.first = static_cast<char*>(base) + it.second;
  }
};

// ceil(log2(v)) computed exactly with frexp.
int ceil_log2(double v) {
  int ex = 0;
  const double m = std::frexp(v, &ex);
  return m == 0.5 ? ex - 1 : ex;
}

// {floor(2^24 CDF(k)), neighbour(k)} rows of a domain; u > CDF <=> x >
// floor(2^24 CDF) for the integer draw x = u 2^24.  Returns an error text.
const char* build_rows(uint32_t n_c, uint32_t K, const uint64_t* neighbors, const double* cdf,
                       std::vector<int2>& mrow) {
  mrow.assign((size_t)n_c * K, make_int2(0, 0));
  for (uint32_t i = 0; i < n_c; ++i) {
    int32_t prev = -2;
    for (uint32_t k = 0; k < K; ++k) {
      const size_t q = (size_t)i * K + k;
      uint32_t nb = i;
      if (neighbors) {
        if (neighbors[q] >= n_c) return "neighbor index out of range";
        nb = (uint32_t)neighbors[q];
      }
      int32_t th = 1 << 24;
      if (cdf) {
        if (!(cdf[q] == cdf[q])) return "cumulative probability is NaN";
        th = (int32_t)std::max(-1.0, std::min(16777216.0, std::floor(cdf[q] * 16777216.0)));
      }
      if (th < prev) return "cumulative probability rows must be non-decreasing";
      prev = th;
      mrow[q] = make_int2(th, (int)nb);
    }
  }
  return nullptr;
}

// Liquid transition in COO form -> incoming lists by destination column
// (sources ascending, duplicates summed) and the diagonal.
const char* build_csr(uint32_t n, uint64_t nnz, const uint64_t* rows, const uint64_t* cols, const double* values,
                      std::vector<uint32_t>& ptr, std::vector<uint32_t>& idx, std::vector<double>& val,
                      std::vector<double>& diag) {
  std::vector<std::pair<std::pair<uint32_t, uint32_t>, double>> off;
  diag.assign(n, 0.0);
  off.reserve(nnz);
  for (uint64_t k = 0; k < nnz; ++k) {
    if (rows[k] >= n || cols[k] >= n) return "transition index out of range";
    if (rows[k] == cols[k])
      diag[rows[k]] += values[k];
    else
      off.push_back({{(uint32_t)cols[k], (uint32_t)rows[k]}, values[k]});
  }
  std::stable_sort(off.begin(), off.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  ptr.assign(n + 1, 0u);
  idx.clear();
  val.clear();
  for (size_t k = 0; k < off.size(); ++k) {
    if (!idx.empty() && k > 0 && off[k].first == off[k - 1].first) {
      val.back() += off[k].second;
      continue;
    }
    idx.push_back(off[k].first.second);
    val.push_back(off[k].second);
    ptr[off[k].first.first + 1]++;
  }
  for (uint32_t j = 0; j < n; ++j) ptr[j + 1] += ptr[j];
  return nullptr;
}

// Launch status of the kernels a set just enqueued: this module's runtime
// error state and that of the module owning the kernels (a plugin may carry
// its own copy of the runtime).
cudaError_t launch_status(const bmc::KernelSet* ks) {
  const cudaError_t own = cudaGetLastError();
  const cudaError_t mod = (cudaError_t)ks->last_error();
  return own != cudaSuccess ? own : mod;
}

}  // namespace

namespace bmc {
// Error reporting for the other host translation units of the C-ABI.
int api_fail(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace bmc

struct bmc_scenario {
  bmc_scenario_desc desc{};
  const bmc::KernelSet* ks = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;  // CUDA device the scenario's memory and stream belong to
  int sm_count = 0;
  void* parena = nullptr;  // particle container
  void* darena = nullptr;  // domain + liquid
  void* tarena = nullptr;  // transition CSR
  ScenDev h{};             // host mirror of the descriptor
  ScenDev* d_desc = nullptr;
  Control* d_ctl = nullptr;
  BatchCtl* d_bctl = nullptr;
  Control* h_ctl = nullptr;  // pinned
  bool has_domain = false, has_transition = false, has_conc = false, has_weight = false;
  std::vector<double> volume;
  std::vector<bmc_feed> feeds;
  double dt = -1.0;
  // launch shape of the cycle kernel
  unsigned variant = bmc::kVariantAuto, blocks_per_sm = 0;  // requested cycle launch variant (bmc_launch.h)
  cudaGraphExec_t graph = nullptr;
  size_t graph_smem = 0;
  unsigned graph_grid = 0, graph_variant = 0;
  bool ctl_fresh = false;  // h_ctl mirrors the device control block (no work enqueued since)
  // last cycle-launch sizing (prepare_cycle), reused while its inputs stay
  unsigned prep_variant = ~0u, prep_bps = 0u, prep_grid = 0u, prep_run = 0u;
  size_t prep_in = 0, prep_out = 0;
  bool prep_global = false;
  unsigned graph_liq = 0, graph_plan = 0;
  int graph_scatter = 0;
  // flow-map cycle (host copies; device copies in marena)
  struct FlowMap {
    std::vector<int2> mrow;
    std::vector<double> vol, vinv, outf, diag;
    std::vector<uint32_t> ptr, idx;
    std::vector<double> val;
    // gas state (bmc_flowmap_add_gas): inverse volumes, transition, kla
    bool has_gas = false;
    std::vector<double> gvinv, gdiag, gval, kla;
    std::vector<uint32_t> gptr, gidx;
  };
  std::vector<FlowMap> maps;
  double t_per_map = 0.0;
  void* marena = nullptr;
  uint32_t* d_map_exit = nullptr;
  // gas phase of a two-phase flow (device arrays in garena)
  void* garena = nullptr;
  void* probe_arena = nullptr;  // time-event probe buffers (bmc_probe_enable)
  std::vector<double> gvol;
  // the gas domain given to bmc_gas_set (device copies in garena), put back
  // when the flow maps stop switching the gas
  std::vector<double> g_vinv, g_diag, g_val, g_kla;
  std::vector<uint32_t> g_ptr, g_idx;
  uint32_t* g_cur_ptr = nullptr;  // garena's transition buffers
  uint32_t* g_cur_idx = nullptr;
  double* g_cur_flow = nullptr;
  // steps enqueued by bmc_step_enqueue, collected in order by
  // bmc_step_collect: an event after each step's export and the caller's
  // buffers; pending entry k exports into slot k of h_export
  struct Pending {
    cudaEvent_t done = nullptr;
    bmc_step_stats* stats = nullptr;
    double* out = nullptr;
    size_t ne = 0;
  };
  Pending pend[2];
  unsigned pend_head = 0, pend_count = 0;
  // host memory mapped into the device address space, two slots of
  // [control block | concentrations], written by the export kernel
  unsigned char* h_export = nullptr;
  unsigned char* d_export = nullptr;
  size_t export_ne = 0, export_slot = 0, export_conc = 0;
  // pending entry whose export is not launched yet (-1: none): it goes out
  // with the next descriptor upload, or alone before anything else uses the
  // stream (settle_export)
  int export_deferred = -1;
  bool enqueuing = false;  // inside bmc_step_enqueue
  // staging of descriptor uploads in host memory mapped into the device
  // address space (a ring, each slot reused once the upload from it has
  // completed)
  static constexpr int kUpSlots = 4;
  ScenDev* h_up = nullptr;
  ScenDev* d_up = nullptr;  // device address of h_up
  cudaEvent_t up_done[kUpSlots] = {};
  unsigned up_next = 0;
};

struct bmc_batch {
  bool graph_maps = false;  // the captured graph includes the flow-map switch
  int sm_count = 0;
  Control* d_dummy_ctl = nullptr;  // control block of empty slots (a finished scenario)
  std::vector<bmc_scenario*> scen;
  const bmc::KernelSet* ks = nullptr;
  cudaStream_t stream = nullptr;
  ScenDev* d_table = nullptr;
  BatchCtl* d_bctl = nullptr;
  unsigned* d_live = nullptr;  // [n + 1] live-tile prefix
  std::vector<ScenDev> table;
  unsigned total_tiles = 0;
  unsigned variant = bmc::kVariantAuto, blocks_per_sm = 0;  // requested cycle launch variant (bmc_launch.h)
  cudaGraphExec_t graph = nullptr;
  size_t graph_smem = 0;
  unsigned graph_grid = 0, graph_variant = 0;
  unsigned run_variant = 0;  // variant of the last prepared launch
  bool run_global = false;   // ... and whether it scatters into the global accumulator
  unsigned plan_y = 1;       // k_plan slices of the last prepared launch
  unsigned graph_liq = 0, graph_plan = 0;
  int graph_scatter = 0;
  double dt = -1.0;
};

namespace {

// Variant index of (threads, particles per thread); -1 if not compiled.
int variant_of(unsigned threads, unsigned ppt) {
  for (int v = 0; v < bmc::kCycleVariants; ++v)
    if (bmc::kVariantThreads[v] == threads && bmc::kVariantPPT[v] == ppt) return v;
  return -1;
}

// Makes `dev` the calling thread's current device for one scope and puts the
// caller's device back at its end.
struct DeviceScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceScope(int dev) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    else if (err == cudaSuccess) prev = -1;
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// The host descriptor to the device, stream-ordered: staged in mapped
// pinned host memory and copied by a one-block kernel (a copy engine
// transfer of these few kilobytes between two steps costs several
// microseconds of stream time; a copy from pageable memory may also wait
// for the stream).
int upload_desc(bmc_scenario* s) {
  if (!s->h_up) {
    void* hp = nullptr;
    BMC_CUDA(cudaHostAlloc(&hp, bmc_scenario::kUpSlots * sizeof(ScenDev), cudaHostAllocMapped));
    s->h_up = static_cast<ScenDev*>(hp);
    void* dp = nullptr;
    BMC_CUDA(cudaHostGetDevicePointer(&dp, hp, 0));
    s->d_up = static_cast<ScenDev*>(dp);
    for (auto& e : s->up_done) BMC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  const unsigned k = s->up_next++ % bmc_scenario::kUpSlots;
  BMC_CUDA(cudaEventSynchronize(s->up_done[k]));  // the upload that last read the slot
  std::memcpy(s->h_up + k, &s->h, sizeof(ScenDev));
  if (s->export_deferred >= 0) {
    // the export of the step in flight and this upload in one launch
    const int q = s->export_deferred;
    s->export_deferred = -1;
    bmc::launch_export(s->stream, s->d_ctl, s->h.C, s->pend[q].ne, s->d_export + q * s->export_slot,
                       s->export_conc, s->d_up + k, s->d_desc);
    g_launches++;
    BMC_CUDA(cudaGetLastError());
    BMC_CUDA(cudaEventRecord(s->pend[q].done, s->stream));
  } else {
    bmc::launch_upload_desc(s->stream, s->d_up + k, s->d_desc);
    g_launches++;
    BMC_CUDA(cudaGetLastError());
  }
  count_copy(sizeof(ScenDev), cudaMemcpyHostToDevice);
  BMC_CUDA(cudaEventRecord(s->up_done[k], s->stream));
  return BMC_OK;
}

// Launches the export of the pending step whose export was deferred, alone.
// Every entry point that uses the scenario's stream (other than a descriptor
// upload, which takes the export along) calls it first, so the exported
// results are those the step left.
int settle_export(bmc_scenario* s) {
  if (!s || s->export_deferred < 0) return BMC_OK;
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  const int q = s->export_deferred;
  s->export_deferred = -1;
  bmc::launch_export(s->stream, s->d_ctl, s->h.C, s->pend[q].ne, s->d_export + q * s->export_slot, s->export_conc);
  g_launches++;
  BMC_CUDA(cudaGetLastError());
  BMC_CUDA(cudaEventRecord(s->pend[q].done, s->stream));
  return BMC_OK;
}

// Threshold of the reference's exit test on the integer draw x (odd, the
// draw u = x 2^-24): probability_leaving<precision_tag>
// (apps/libs/simulation/public/simulation/probability_leaving.hpp L18-L33)
// exits iff dt*F > -ln(u)*V with the logarithm of the float draw taken in
// float (CommonMaths::_ln<true>, the C library's logf on the reference's
// host build) and the product in double.  -logf(u) does not grow with u (the
// CPU tests check logf over every draw value), so the test holds exactly
// for x > thr, thr = (smallest exiting draw) - 1, found by bisection over
// the 2^23 draw values; 2^24 when no draw exits.
uint32_t exit_threshold(double dt, double flow, double volume) {
  auto exits = [&](uint32_t k) {
    const float u = (float)(2u * k + 1u) * 0x1p-24f;
    return (dt * flow) > ((double)(-logf(u)) * volume);
  };
  uint32_t lo = 0, hi = 1u << 23;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) / 2u;
    if (exits(mid))
      hi = mid;
    else
      lo = mid + 1u;
  }
  return lo == (1u << 23) ? (1u << 24) : 2u * lo;
}

// Outlets follow the feeds in order (SimulationUnit::update_feed assigns the
// leaving-flow slots in feed order), each with its exit threshold.
void derive_outlets(bmc_scenario* s) {
  s->h.n_feeds = (uint32_t)s->feeds.size();
  s->h.n_outlets = 0;
  for (size_t f = 0; f < s->feeds.size(); ++f) {
    const bmc_feed& fd = s->feeds[f];
    s->h.feed_in[f] = fd.inlet;
    s->h.feed_out[f] = fd.outlet;
    s->h.feed_flow[f] = fd.flow;
    for (int sp = 0; sp < bmc::kMaxSpecies; ++sp) s->h.feed_conc[f * bmc::kMaxSpecies + sp] = fd.conc[sp];
    if (fd.outlet >= 0) {
      const unsigned o = s->h.n_outlets++;
      s->h.outlet_idx[o] = (uint32_t)fd.outlet;
      s->h.outlet_feed[o] = (uint32_t)f;
      s->h.outlet_flow[o] = fd.flow;
      const double vol = s->volume[(size_t)fd.outlet];
      s->h.exit_thr[o] = s->dt > 0 ? exit_threshold(s->dt, fd.flow, vol) : (1u << 24);
    }
  }
}

// Flow-map tables that depend on dt: steps per map (compute_n_per_flowmap,
// apps/core/src/global_initaliser.cpp L104-L114) and each map's outlet
// thresholds (as derive_outlets, with that map's volumes).
int refresh_map_tables(bmc_scenario* s) {
  const size_t nm = s->maps.size();
  s->h.n_maps = (uint32_t)nm;
  if (nm == 0) {
    s->h.n_per_map = 1;
    return BMC_OK;
  }
  const double t = s->t_per_map;
  s->h.n_per_map = (t == 0.0 || nm == 1 || s->dt <= 0.0) ? 1u : (uint32_t)(size_t)(t / s->dt) + 1u;
  std::vector<uint32_t> thr(nm * bmc::kMaxOutlets, 0u);
  for (size_t m = 0; m < nm; ++m) {
    unsigned o = 0;
    for (const bmc_feed& fd : s->feeds) {
      if (fd.outlet < 0) continue;
      const double vol = s->maps[m].vol[(size_t)fd.outlet];
      thr[m * bmc::kMaxOutlets + o++] = s->dt > 0 ? exit_threshold(s->dt, fd.flow, vol) : (1u << 24);
    }
  }
  BMC_CUDA(counted_memcpy_async(s->d_map_exit, thr.data(), thr.size() * 4, cudaMemcpyHostToDevice, s->stream));
  return BMC_OK;
}

int set_dt(bmc_scenario* s, double dt, bool launch_pmove) {
  if (!(dt > 0.0)) return fail(BMC_E_INVALID, "dt must be > 0");
  if (dt == s->dt) return BMC_OK;
  s->dt = dt;
  s->h.dt = dt;
  derive_outlets(s);
  int rc = refresh_map_tables(s);
  if (rc) return rc;
  rc = upload_desc(s);
  if (rc) return rc;
  if (launch_pmove) {
    s->ks->move_thr(1, s->stream, s->d_desc);
    g_launches++;
    BMC_CUDA(launch_status(s->ks));
  }
  return BMC_OK;
}

size_t cycle_smem(const ScenDev& h) {
  size_t n = (size_t)h.n_c * h.n_acc;
  if (h.n_acc == 1 && h.n_c <= bmc::kScatterCopyMaxCompartments)  // copies of the accumulator
    n = std::max(n, (size_t)bmc::kAccCopies * bmc::scatter_stride(h.n_c));
  return n * sizeof(unsigned long long);
}

// *smem: in, the accumulator bytes; out, the dynamic shared memory of the
// launch (staged variants append their tile buffers, 128-byte aligned).
static int size_cycle(const bmc::KernelSet* ks, unsigned variant, unsigned bps_req, size_t* smem, int sm_count,
                      unsigned* grid_out, int* fit_out) {
  if (ks->cycle_extra_smem[variant] > 0) *smem = align_up(*smem, 128) + ks->cycle_extra_smem[variant];
  if (*smem > 227 * 1024)
    return fail(BMC_E_UNSUPPORTED, "shared accumulator (n_compartments * n_contributions) and tile buffers "
                                   "exceed the shared memory of a block for this launch shape");
  int bps = 0;
  BMC_CUDA((cudaError_t)ks->cycle_setup[variant](*smem, &bps));
  if (bps < 1) return fail(BMC_E_UNSUPPORTED, "cycle kernel cannot be resident with this shape");
  *fit_out = bps;
  if (bps_req > 0) bps = std::min<int>(bps, (int)bps_req);
  *grid_out = (unsigned)(sm_count * bps);
  return BMC_OK;
}

// Dynamic shared memory and grid of the cycle launch for the requested
// variant; resolves kVariantAuto (*run_out: the variant to launch).
// *global_out: the launch sums contributions straight into the global
// accumulator (kScatterGlobal, tile-staging variants only), chosen when the
// shared accumulator and the stage buffers do not fit one block.  Measured on
// 1e7 particles (ms per step, 10,648 compartments): the tile-staging kernel
// at one block per SM with its shared accumulator 0.321 (FP64) / 0.239
// (FP32), with the global accumulator at two blocks per SM 0.329 / 0.304,
// register streaming 0.532 / 0.360; so the shared accumulator is kept while
// it fits.  Register-streaming shapes always keep the shared accumulator.
int prepare_cycle(const bmc::KernelSet* ks, unsigned variant, unsigned bps_req, size_t* smem, int sm_count,
                  unsigned* grid_out, unsigned* run_out, bool* global_out) {
  int fit = 0;
  *global_out = false;
  const bool staged = variant == bmc::kVariantAuto || ks->cycle_extra_smem[variant] > 0;
  if (staged) {
    const unsigned v = variant == bmc::kVariantAuto ? bmc::kAutoStaged : variant;
    for (int glob = 0; glob < 2; ++glob) {
      size_t m = glob ? 0 : *smem;
      unsigned g = 0;
      if (size_cycle(ks, v, bps_req, &m, sm_count, &g, &fit) == BMC_OK) {
        *smem = m;
        *grid_out = g;
        *run_out = v;
        *global_out = glob != 0;
        return BMC_OK;
      }
      (void)cudaGetLastError();  // a refused size is not an error of the step
    }
    if (variant != bmc::kVariantAuto) return fail(BMC_E_UNSUPPORTED, "cycle kernel cannot be resident with this shape");
    variant = bmc::kAutoStreamed;
  }
  int rc = size_cycle(ks, variant, bps_req, smem, sm_count, grid_out, &fit);
  if (rc) return rc;
  *run_out = variant;
  return BMC_OK;
}

// Enqueue one step (liquid step optional) for a table of scenarios.
// Slices of k_plan (grid y): kPlanSlice compartments each.
unsigned plan_slices(const ScenDev& h) { return std::max(1u, (h.n_c + bmc::kPlanSlice - 1) / bmc::kPlanSlice); }

// Blocks along x of the liquid step: kLiquidThreads / n_species compartments
// per block.
unsigned liquid_grid(const ScenDev& h) {
  const unsigned cb = bmc::kLiquidThreads / std::max(1u, h.n_s);
  return std::max(1u, (h.n_c + cb - 1) / cb);
}

// With `maps`, the flow-map switch runs first (main-loop steps only).
int enqueue_step(const bmc::KernelSet* ks, cudaStream_t st, ScenDev* d_table, int n_scen, unsigned liq_grid,
                 unsigned plan_y, BatchCtl* d_bctl, int do_scalar, unsigned variant, unsigned grid, size_t smem,
                 int sm_count, bool maps, int scatter) {
  if (maps && do_scalar) {
    ks->flowmap(n_scen, st, d_table);
    g_launches += 1;
  }
  if (scatter == bmc::kScatterGlobal && ks->cycle_extra_smem[variant] == 0)
    return fail(BMC_E_UNSUPPORTED, "the global accumulator form needs a tile-staging launch shape");
  ks->liquid(n_scen, liq_grid, st, d_table, d_bctl, do_scalar);
  ks->cycle[variant](dim3(grid), dim3(bmc::kVariantThreads[variant]), smem, st, d_table, n_scen, d_bctl, scatter);
  ks->plan(n_scen, plan_y, st, d_table, d_bctl);
  ks->divide(dim3(sm_count * 4), st, d_table, n_scen, d_bctl);
  ks->compact(dim3(sm_count * 2), st, d_table, n_scen, d_bctl);
  ks->merge(dim3(sm_count * 2), st, d_table, n_scen, d_bctl);
  g_launches += 6;
  BMC_CUDA(launch_status(ks));
  return BMC_OK;
}

// Launches whose domains all have at most kAggregateMaxCompartments
// compartments use the cycle kernels with the warp-aggregated scatter.
bool tiny_domain(const ScenDev& h) { return h.n_c <= bmc::kAggregateMaxCompartments; }
// Domains whose separable-model scatter goes to accumulator copies.
bool copy_domain(const bmc::KernelSet* ks, const ScenDev& h) {
  return ks->separable && h.n_c <= bmc::kScatterCopyMaxCompartments;
}
int scenario_scatter(const bmc::KernelSet* ks, const ScenDev& h) {
  return tiny_domain(h) ? bmc::kScatterWarp : copy_domain(ks, h) ? bmc::kScatterCopied : bmc::kScatterPlain;
}
bool batch_tiny(const bmc_batch* b) {
  for (const bmc_scenario* m : b->scen)
    if (m && !tiny_domain(m->h)) return false;
  return true;
}
int batch_scatter(const bmc_batch* b) {
  if (b->run_global) return bmc::kScatterGlobal;
  if (batch_tiny(b)) return bmc::kScatterWarp;
  for (const bmc_scenario* m : b->scen)
    if (m && copy_domain(b->ks, m->h)) return bmc::kScatterCopied;
  return bmc::kScatterPlain;
}

bool batch_has_maps(const bmc_batch* b) {
  for (const bmc_scenario* m : b->scen)
    if (m && m->h.n_maps > 0) return true;
  return false;
}

// Refresh a batch's descriptor table for dt (uploading it when a member
// changed) and size the cycle launch.
int batch_prepare(bmc_batch* b, double dt, int* n_out, unsigned* max_nc_out, size_t* smem_out, unsigned* grid_out) {
  if (!b) return fail(BMC_E_INVALID, "null batch");
  const int n = (int)b->scen.size();
  bool table_changed = b->table.size() != (size_t)n;
  b->table.resize(n);
  int lo = table_changed ? 0 : n, hi = table_changed ? n - 1 : -1;  // changed entries
  unsigned tiles = 0, max_nc = 0, max_plan = 1;
  size_t smem = 0;
  for (int i = 0; i < n; ++i) {
    bmc_scenario* s = b->scen[i];
    ScenDev d{};
    if (s) {
      int rc = set_dt(s, dt, false);
      if (rc) return rc;
      d = s->h;
    } else {
      // empty slot: a finished scenario without compartments or tiles that
      // every kernel skips
      d.ctl = b->d_dummy_ctl;
      d.step_limit = 1u;
    }
    d.tile_base = tiles;
    tiles += d.n_tiles;
    max_nc = std::max(max_nc, liquid_grid(d));
    max_plan = std::max(max_plan, plan_slices(d));
    smem = std::max(smem, cycle_smem(d));
    if (std::memcmp(&d, &b->table[i], sizeof(ScenDev)) != 0) {
      table_changed = true;
      lo = std::min(lo, i);
      hi = std::max(hi, i);
    }
    b->table[i] = d;
  }
  if (table_changed || b->dt != dt) {
    BMC_CUDA(cudaStreamSynchronize(b->stream));
    if (hi >= lo)  // only the entries that changed (slots filled or emptied)
      BMC_CUDA(counted_memcpy_async(b->d_table + lo, b->table.data() + lo, sizeof(ScenDev) * (size_t)(hi - lo + 1),
                                    cudaMemcpyHostToDevice, b->stream));
    BatchCtl bc{0u, tiles, 0u, 0u, b->d_live};
    BMC_CUDA(counted_memcpy_async(b->d_bctl, &bc, sizeof(bc), cudaMemcpyHostToDevice, b->stream));
    b->ks->move_thr(n, b->stream, b->d_table);
    g_launches++;
    BMC_CUDA(launch_status(b->ks));
    b->dt = dt;
    b->total_tiles = tiles;
  }
  int rc = prepare_cycle(b->ks, b->variant, b->blocks_per_sm, &smem, b->sm_count, grid_out, &b->run_variant,
                         &b->run_global);
  if (rc) return rc;
  *n_out = n;
  *max_nc_out = max_nc;
  *smem_out = smem;
  b->plan_y = max_plan;
  return BMC_OK;
}

void stats_from_ctl(const Control& c, bmc_step_stats* out) {
  std::memset(out, 0, sizeof(*out));
  out->n_used = c.n_used;
  out->inactive = c.inactive;
  out->births = c.last_births;
  out->exits = c.last_exits;
  out->moves = c.last_moves;
  out->overflow = c.last_overflow;
  out->requested_divisions = c.last_req_div;
  out->clamped = c.clamped;
  out->next_id = c.next_id;
  out->step = c.step;
  out->compacted = c.last_compacted;
  out->error = c.error;
  for (int k = 0; k < 8; ++k) out->mass_balance[k] = c.mass_balance[k];
}

int read_ctl(bmc_scenario* s, bmc_step_stats* out) {
  BMC_CUDA(counted_memcpy_async(s->h_ctl, s->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  s->ctl_fresh = true;
  if (out) stats_from_ctl(*s->h_ctl, out);
  if (s->h_ctl->error) return fail(BMC_E_DEVICE, "device error word set: " + std::to_string(s->h_ctl->error));
  return BMC_OK;
}

int check_ready(bmc_scenario* s, bool need_liquid) {
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (s->pend_count > 0 && !s->enqueuing)
    return fail(BMC_E_STATE, "steps enqueued by bmc_step_enqueue are not collected yet");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set (bmc_domain_update)");
  if (!s->has_conc) return fail(BMC_E_STATE, "concentrations not set (bmc_set_concentrations)");
  if (!s->has_weight) return fail(BMC_E_STATE, "particles not initialised (bmc_init_particles / bmc_set_weight)");
  if (need_liquid && !s->has_transition) return fail(BMC_E_STATE, "transition not set (bmc_set_transition_coo)");
  return BMC_OK;
}

int set_quanta(bmc_scenario* s) {
  // Separable models accumulate one basis value per particle (column 0,
  // bounded by value_bound[0]); general models accumulate weight *
  // contribution j per particle (column j, bounded by weight *
  // value_bound[j]).  The quantum 2^e puts the bound at 2^kQBits quanta.
  const int cols = s->ks->separable ? 1 : s->ks->n_ctb;
  for (int j = 0; j < bmc::kMaxSpecies; ++j) {
    int e = 0;
    if (j < cols) {
      const double vmax = s->ks->separable ? s->desc.value_bound[j] : s->h.weight * s->desc.value_bound[j];
      if (!(vmax > 0.0) || !std::isfinite(vmax)) return fail(BMC_E_INVALID, "value bounds must be > 0");
      e = ceil_log2(vmax) - bmc::kQBits;
    }
    s->h.q_exp[j] = e;
    s->h.q_scale_up[j] = std::ldexp(1.0, e);
  }
  return BMC_OK;
}

}  // namespace

extern "C" {

int bmc_version(int32_t* major, int32_t* minor) {
  if (major) *major = BMC_VERSION_MAJOR;
  if (minor) *minor = BMC_VERSION_MINOR;
  return BMC_OK;
}

const char* bmc_last_error(void) { return g_last_error.c_str(); }

int bmc_device_sm_count(int32_t* sm_count) {
  int dev = 0;
  BMC_CUDA(cudaGetDevice(&dev));
  int n = 0;
  BMC_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  if (sm_count) *sm_count = n;
  return BMC_OK;
}

int bmc_set_device(int32_t device) {
  BMC_CUDA(cudaSetDevice(device));
  return BMC_OK;
}

int bmc_transfer_bytes(uint64_t* h2d, uint64_t* d2h) {
  if (h2d) *h2d = g_h2d.load();
  if (d2h) *d2h = g_d2h.load();
  return BMC_OK;
}

}  // extern "C"

// Particle arena of a scenario: the container arrays for `cap` slots
// (state of `state_bytes` per slot), the per-step scratch (division buffer,
// tile counters, request words, compaction lists), then the control block,
// the descriptor, the tile scheduler and its two-word live prefix.
static void carve_particles(Carver& cv, ScenDev& h, size_t state_bytes, unsigned long long cap, Control** ctl,
                            ScenDev** desc, BatchCtl** bctl, unsigned** live) {
  const unsigned n_tiles = (unsigned)(cap / kTile);
  cv.add_raw(&h.state, state_bytes * cap);
  cv.add(&h.pos, cap);
  cv.add(&h.status, cap);
  cv.add(&h.age_h, cap);
  cv.add(&h.age_d, cap);
  cv.add(&h.id, cap);
  cv.add_raw(&h.child_state, state_bytes * cap);
  cv.add(&h.child_pos, cap);
  cv.add(&h.tile_births, n_tiles);
  cv.add(&h.tile_inactive, n_tiles);
  cv.add(&h.tile_boff, n_tiles);
  cv.add(&h.tile_goff, n_tiles);
  cv.add(&h.tile_soff, n_tiles);
  cv.add(&h.bmask, cap / 32);
  cv.add(&h.bpos, cap);
  cv.add(&h.gap_slot, cap);
  cv.add(&h.src_slot, cap);
  cv.add(ctl, 1);
  cv.add(desc, 1);
  cv.add(bctl, 1);
  cv.add(live, 2);
}

extern "C" {

int bmc_launch_count(uint64_t* count) {
  if (count) *count = g_launches.load();
  return BMC_OK;
}

int bmc_scenario_create(const bmc_scenario_desc* desc, bmc_scenario** out) {
  if (!desc || !out) return fail(BMC_E_INVALID, "null argument");
  const bmc::KernelSet* ks = bmc::kernel_set(desc->model.model, desc->model.f64);
  if (!ks) return fail(BMC_E_UNSUPPORTED, "model / precision not compiled in");
  if ((int)desc->model.n_var != ks->n_var || (int)desc->model.n_ctb != ks->n_ctb)
    return fail(BMC_E_INVALID, "n_var / n_ctb do not match the compiled model");
  if (desc->n_species < (uint32_t)ks->n_ctb || desc->n_species > (uint32_t)bmc::kMaxSpecies)
    return fail(BMC_E_INVALID, "n_species must be in [n_ctb, 8]");
  if (desc->capacity == 0 || desc->capacity > 0xFFFFFFFFull - kTile)
    return fail(BMC_E_INVALID, "capacity must be in [1, 2^32 - 1024]");
  auto* s = new bmc_scenario();
  s->desc = *desc;
  s->ks = ks;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  s->device = dev;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete s;
    return fail(BMC_E_CUDA, std::string("device set-up: ") + cudaGetErrorString(e));
  }
  const unsigned long long cap = align_up(desc->capacity, kTile);
  const size_t fsz = desc->model.f64 ? 8 : 4;
  const unsigned n_tiles = (unsigned)(cap / kTile);
  ScenDev& h = s->h;
  h.cap = cap;
  h.n_tiles = n_tiles;
  h.tile_base = 0;
  Carver cv;
  Control* ctl_tmp = nullptr;
  ScenDev* desc_tmp = nullptr;
  BatchCtl* bctl_tmp = nullptr;
  unsigned* live_tmp = nullptr;
  carve_particles(cv, h, fsz * ks->n_var, cap, &ctl_tmp, &desc_tmp, &bctl_tmp, &live_tmp);
  e = cudaMalloc(&s->parena, cv.off);
  if (e != cudaSuccess) {
    cudaStreamDestroy(s->stream);
    delete s;
    return fail(BMC_E_CUDA, std::string("cudaMalloc particle arena: ") + cudaGetErrorString(e));
  }
  cv.bind(s->parena);
  s->d_ctl = ctl_tmp;
  s->d_desc = desc_tmp;
  s->d_bctl = bctl_tmp;
  h.ctl = s->d_ctl;
  h.n_var = ks->n_var;
  h.n_ctb = ks->n_ctb;
  h.n_acc = ks->separable ? 1u : (uint32_t)ks->n_ctb;
  h.n_s = desc->n_species;
  h.f64 = desc->model.f64;
  for (int k = 0; k < 16; ++k) h.params[k] = desc->model.params[k];
  h.seed = desc->seed;
  h.dead_ratio = desc->dead_ratio_threshold;
  h.min_removal = desc->min_removal;
  e = cudaMallocHost(&s->h_ctl, sizeof(Control));
  if (e == cudaSuccess) e = cudaMemsetAsync(s->parena, 0, cv.off, s->stream);
  if (e == cudaSuccess) {
    BatchCtl b{0u, n_tiles, 0u, 0u, live_tmp};
    e = counted_memcpy_async(s->d_bctl, &b, sizeof(b), cudaMemcpyHostToDevice, s->stream);
  }
  if (e == cudaSuccess) e = counted_memcpy_async(s->d_desc, &h, sizeof(ScenDev), cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cudaFree(s->parena);
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    cudaStreamDestroy(s->stream);
    delete s;
    return fail(BMC_E_CUDA, std::string("scenario set-up: ") + cudaGetErrorString(e));
  }
  *out = s;
  return BMC_OK;
}

int bmc_scenario_destroy(bmc_scenario* s) {
  if (!s) return BMC_OK;
  cudaStreamSynchronize(s->stream);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->parena) cudaFree(s->parena);
  if (s->darena) cudaFree(s->darena);
  if (s->tarena) cudaFree(s->tarena);
  if (s->marena) cudaFree(s->marena);
  if (s->garena) cudaFree(s->garena);
  if (s->probe_arena) cudaFree(s->probe_arena);
  if (s->h_ctl) cudaFreeHost(s->h_ctl);
  for (auto& q : s->pend)
    if (q.done) cudaEventDestroy(q.done);
  if (s->h_export) cudaFreeHost(s->h_export);
  for (auto& e : s->up_done)
    if (e) cudaEventDestroy(e);
  if (s->h_up) cudaFreeHost(s->h_up);
  cudaStreamDestroy(s->stream);
  delete s;
  return BMC_OK;
}

int bmc_reserve(bmc_scenario* s, uint64_t capacity) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (capacity == 0 || capacity > 0xFFFFFFFFull - kTile) return fail(BMC_E_INVALID, "capacity must be in [1, 2^32 - 1024]");
  const unsigned long long cap = align_up(capacity, kTile);
  if (cap <= s->h.cap) return BMC_OK;  // never shrinks
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  BMC_CUDA(counted_memcpy_async(s->h_ctl, s->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  const unsigned long long n = s->h_ctl->n_used;
  const size_t fsz = s->h.f64 ? 8 : 4;
  const int nv = (int)s->h.n_var;
  ScenDev h = s->h;  // old pointers stay in s->h until the copy is done
  h.cap = cap;
  h.n_tiles = (unsigned)(cap / kTile);
  Carver cv;
  Control* ctl = nullptr;
  ScenDev* desc = nullptr;
  BatchCtl* bctl = nullptr;
  unsigned* live = nullptr;
  carve_particles(cv, h, fsz * nv, cap, &ctl, &desc, &bctl, &live);
  void* arena = nullptr;
  BMC_CUDA(cudaMalloc(&arena, cv.off));
  cv.bind(arena);
  cudaError_t e = cudaMemsetAsync(arena, 0, cv.off, s->stream);
  // the n live slots of every container array, and the control block
  for (int v = 0; v < nv && e == cudaSuccess; ++v)
    e = cudaMemcpyAsync(static_cast<char*>(h.state) + (size_t)v * cap * fsz,
                        static_cast<const char*>(s->h.state) + (size_t)v * s->h.cap * fsz, n * fsz,
                        cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.pos, s->h.pos, n * 4, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.status, s->h.status, n, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.age_h, s->h.age_h, n * 4, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.age_d, s->h.age_d, n * 4, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.id, s->h.id, n * 4, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, s->d_ctl, sizeof(Control), cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cudaFree(arena);
    return fail(BMC_E_CUDA, std::string("reserve: ") + cudaGetErrorString(e));
  }
  cudaFree(s->parena);
  s->parena = arena;
  h.ctl = ctl;
  s->h = h;
  s->d_ctl = ctl;
  s->d_desc = desc;
  s->d_bctl = bctl;
  s->desc.capacity = capacity;
  // the captured step holds the old descriptor and scheduler addresses
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  s->ctl_fresh = false;
  BatchCtl b{0u, h.n_tiles, 0u, 0u, live};
  BMC_CUDA(counted_memcpy_async(s->d_bctl, &b, sizeof(b), cudaMemcpyHostToDevice, s->stream));
  int rc = upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_domain_update(bmc_scenario* s, uint32_t n_c, uint32_t K, const double* volume, const uint64_t* neighbors,
                      const double* out_flows, const double* cdf) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !volume || !out_flows || n_c == 0 || K == 0) return fail(BMC_E_INVALID, "bad domain arguments");
  if (n_c > 1 && (!neighbors || !cdf)) return fail(BMC_E_INVALID, "neighbors and cdf required when n_c > 1");
  if (!s->maps.empty()) return fail(BMC_E_STATE, "the domain follows the flow-map cycle (bmc_flowmap_clear first)");
  std::vector<int2> mrow;
  if (const char* why = build_rows(n_c, K, neighbors, cdf, mrow)) return fail(BMC_E_INVALID, why);
  std::vector<double> vol(volume, volume + n_c), outf(out_flows, out_flows + n_c), vinv(n_c), diag(n_c);
  for (uint32_t j = 0; j < n_c; ++j) {
    if (!(vol[j] > 0.0)) return fail(BMC_E_INVALID, "volumes must be > 0");
    if (!(outf[j] >= 0.0)) return fail(BMC_E_INVALID, "out flows must be >= 0");
    vinv[j] = 1.0 / vol[j];
    diag[j] = -outf[j];
  }
  ScenDev& h = s->h;
  const bool resize = !s->has_domain || h.n_c != n_c || h.K != K;
  if (resize) {
    cudaStreamSynchronize(s->stream);
    if (s->darena) cudaFree(s->darena);
    s->darena = nullptr;
    // the step graph's launch choices depend on the domain's size
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
    const size_t ne = (size_t)n_c * h.n_s, na = (size_t)n_c * h.n_acc;
    Carver cv;
    int2* p_mrow = nullptr;
    cv.add(&p_mrow, (size_t)n_c * K);
    int32_t* p_row16 = nullptr;
    cv.add(&p_row16, (size_t)n_c * 16);
    double* p_vol = nullptr;
    cv.add(&p_vol, n_c);
    double* p_out = nullptr;
    cv.add(&p_out, n_c);
    double* p_diag = nullptr;
    cv.add(&p_diag, n_c);
    double* p_vinv = nullptr;
    cv.add(&p_vinv, n_c);
    double* p_rec = nullptr;
    cv.add(&p_rec, (size_t)n_c * 8);
    cv.add(&h.C, 2 * ne);
    cv.add(&h.M, ne);
    cv.add(&h.src, ne);
    cv.add(&h.acc_hi, na);
    cv.add(&h.acc_lo, na);
    BMC_CUDA(cudaMalloc(&s->darena, cv.off));
    cv.bind(s->darena);
    h.mrow = p_mrow;
    h.mrow16 = p_row16;
    h.volume = p_vol;
    h.out_flow = p_out;
    h.diag = p_diag;
    h.vinv = p_vinv;
    h.crec = p_rec;
    BMC_CUDA(cudaMemsetAsync(s->darena, 0, cv.off, s->stream));
    s->has_conc = false;
    s->has_transition = false;
  }
  h.n_c = n_c;
  h.K = K;
  BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.volume), vol.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.out_flow), outf.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(const_cast<int2*>(h.mrow), mrow.data(), mrow.size() * sizeof(int2), cudaMemcpyHostToDevice, s->stream));
  {
    // rows of up to 8 entries: thresholds (padded with INT32_MAX) then
    // neighbours (padded with the last), 16 slots a compartment
    std::vector<int32_t> row16((size_t)n_c * 16, INT32_MAX);
    for (size_t i = 0; i < n_c; ++i)
      for (size_t k = 0; k < 8; ++k) {
        if (k < K) row16[i * 16 + k] = mrow[i * K + k].x;
        row16[i * 16 + 8 + k] = mrow[i * K + std::min<size_t>(k, K - 1)].y;
      }
    BMC_CUDA(counted_memcpy_async(const_cast<int32_t*>(h.mrow16), row16.data(), row16.size() * sizeof(int32_t),
                                  cudaMemcpyHostToDevice, s->stream));
  }
  BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.vinv), vinv.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
  if (!s->has_transition)
    BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.diag), diag.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
  s->volume = vol;
  s->has_domain = true;
  const double dt = s->dt;
  s->dt = -1.0;
  int rc = BMC_OK;
  if (dt > 0)
    rc = set_dt(s, dt, true);
  else {
    derive_outlets(s);
    rc = upload_desc(s);
  }
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_set_transition_coo(bmc_scenario* s, uint32_t n, uint64_t nnz, const uint64_t* rows, const uint64_t* cols,
                           const double* values) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || (nnz && (!rows || !cols || !values))) return fail(BMC_E_INVALID, "bad transition arguments");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  if (n != s->h.n_c) return fail(BMC_E_INVALID, "transition size differs from n_compartments");
  if (!s->maps.empty()) return fail(BMC_E_STATE, "the domain follows the flow-map cycle (bmc_flowmap_clear first)");
  std::vector<uint32_t> ptr, idx;
  std::vector<double> val, diag;
  if (const char* why = build_csr(n, nnz, rows, cols, values, ptr, idx, val, diag)) return fail(BMC_E_INVALID, why);
  cudaStreamSynchronize(s->stream);
  if (s->tarena) cudaFree(s->tarena);
  s->tarena = nullptr;
  Carver cv;
  uint32_t* p_ptr = nullptr;
  uint32_t* p_idx = nullptr;
  double* p_val = nullptr;
  cv.add(&p_ptr, n + 1);
  cv.add(&p_idx, idx.size());
  cv.add(&p_val, val.size());
  BMC_CUDA(cudaMalloc(&s->tarena, cv.off));
  cv.bind(s->tarena);
  BMC_CUDA(counted_memcpy_async(p_ptr, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice, s->stream));
  if (!idx.empty()) {
    BMC_CUDA(counted_memcpy_async(p_idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_val, val.data(), val.size() * 8, cudaMemcpyHostToDevice, s->stream));
  }
  BMC_CUDA(counted_memcpy_async(const_cast<double*>(s->h.diag), diag.data(), n * 8, cudaMemcpyHostToDevice, s->stream));
  s->h.in_ptr = p_ptr;
  s->h.in_idx = p_idx;
  s->h.in_flow = p_val;
  int rc = upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  s->has_transition = true;
  return BMC_OK;
}

int bmc_set_concentrations(bmc_scenario* s, const double* conc) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !conc) return fail(BMC_E_INVALID, "null argument");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  const size_t n_c = s->h.n_c, ns = s->h.n_s;
  std::vector<double> C(conc, conc + n_c * ns), M(n_c * ns);
  for (size_t j = 0; j < n_c; ++j) {
    for (size_t sp = 0; sp < ns; ++sp) {
      if (!(C[j * ns + sp] >= 0.0)) return fail(BMC_E_INVALID, "concentrations must be >= 0");
      M[j * ns + sp] = C[j * ns + sp] * s->volume[j];
    }
  }
  BMC_CUDA(counted_memcpy_async(s->h.C, C.data(), C.size() * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.C + C.size(), C.data(), C.size() * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.M, M.data(), M.size() * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(cudaMemsetAsync(s->h.src, 0, C.size() * 8, s->stream));
  BMC_CUDA(cudaMemsetAsync(s->h.acc_hi, 0, n_c * s->h.n_acc * 8, s->stream));
  BMC_CUDA(cudaMemsetAsync(s->h.acc_lo, 0, n_c * s->h.n_acc * 8, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  s->has_conc = true;
  return BMC_OK;
}

int bmc_set_feeds(bmc_scenario* s, uint32_t n_feeds, const bmc_feed* feeds) {
  if (!s || (n_feeds && !feeds)) return fail(BMC_E_INVALID, "null argument");
  if (n_feeds > (uint32_t)bmc::kMaxOutlets) return fail(BMC_E_INVALID, "at most 8 feeds");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  for (uint32_t f = 0; f < n_feeds; ++f) {
    if (feeds[f].inlet >= s->h.n_c || feeds[f].outlet >= (int32_t)s->h.n_c || feeds[f].outlet < -1)
      return fail(BMC_E_INVALID, "feed position out of range");
    if (!(feeds[f].flow >= 0.0)) return fail(BMC_E_INVALID, "feed flow must be >= 0");
  }
  s->feeds.assign(feeds, feeds + n_feeds);
  // new feeds are constant until bmc_set_feed_schedules says otherwise
  s->h.n_sched = 0u;
  for (int f = 0; f < bmc::kMaxOutlets; ++f) {
    s->h.feed_kind[f] = BMC_FEED_CONSTANT;
    s->h.feed_f0[f] = 0.0;
    s->h.feed_rate[f] = 0.0;
  }
  derive_outlets(s);
  int rc = refresh_map_tables(s);
  if (rc) return rc;
  // stream-ordered: the descriptor copy is staged at once, later work on
  // this stream sees it; no wait for the device
  return upload_desc(s);
}

int bmc_set_weight(bmc_scenario* s, double weight) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !(weight > 0.0)) return fail(BMC_E_INVALID, "weight must be > 0");
  s->h.weight = weight;
  int rc = set_quanta(s);
  if (rc) return rc;
  rc = upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  s->has_weight = true;
  return BMC_OK;
}

static int write_ctl_fresh(bmc_scenario* s, unsigned long long n, unsigned long long next_id,
                           unsigned long long inactive) {
  BMC_CUDA(counted_memcpy_async(s->h_ctl, s->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  Control c = *s->h_ctl;
  c.n_used = n;
  c.next_id = next_id;
  c.inactive = inactive;
  BMC_CUDA(counted_memcpy_async(s->d_ctl, &c, sizeof(Control), cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  s->ctl_fresh = false;
  return BMC_OK;
}

int bmc_init_particles(bmc_scenario* s, uint64_t n, int32_t uniform_init, double x0, double* weight_out) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  if (n > s->h.cap) return fail(BMC_E_CAPACITY, "more particles than capacity");
  if (n == 0) return fail(BMC_E_INVALID, "n must be > 0");
  double* d_mass = nullptr;
  BMC_CUDA(cudaMalloc(&d_mass, n * sizeof(double)));
  const uint32_t span = uniform_init ? s->h.n_c : 1u;
  s->ks->init(dim3(s->sm_count * 8), s->stream, s->d_desc, n, 0u, span, d_mass);
  g_launches++;
  std::vector<double> mass(n);
  cudaError_t e = launch_status(s->ks);
  if (e == cudaSuccess) e = counted_memcpy_async(mass.data(), d_mass, n * 8, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d_mass);
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("init: ") + cudaGetErrorString(e));
  double total = 0.0;
  for (uint64_t i = 0; i < n; ++i) total += mass[i];
  double vtot = 0.0;
  for (double v : s->volume) vtot += v;
  const double w = (x0 * vtot) / total;
  if (!(w > 0.0) || !std::isfinite(w)) return fail(BMC_E_INVALID, "initial weight is not positive");
  int rc = write_ctl_fresh(s, n, n, 0ull);
  if (rc) return rc;
  rc = bmc_set_weight(s, w);
  if (rc) return rc;
  if (weight_out) *weight_out = w;
  return BMC_OK;
}

int bmc_set_particles(bmc_scenario* s, uint64_t n, const void* state, const uint32_t* pos, const uint8_t* status,
                      const float* age_h, const float* age_d, const uint32_t* id, uint64_t next_id) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !state || !pos || !status || !age_h || !age_d || !id) return fail(BMC_E_INVALID, "null argument");
  if (n > s->h.cap) return fail(BMC_E_CAPACITY, "more particles than capacity");
  const size_t fsz = s->h.f64 ? 8 : 4;
  for (int v = 0; v < (int)s->h.n_var; ++v)
    BMC_CUDA(counted_memcpy_async(static_cast<char*>(s->h.state) + (size_t)v * s->h.cap * fsz,
                             static_cast<const char*>(state) + (size_t)v * n * fsz, n * fsz, cudaMemcpyHostToDevice,
                             s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.pos, pos, n * 4, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.status, status, n, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.age_h, age_h, n * 4, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.age_d, age_d, n * 4, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.id, id, n * 4, cudaMemcpyHostToDevice, s->stream));
  unsigned long long inactive = 0;
  for (uint64_t i = 0; i < n; ++i) inactive += status[i] != BMC_STATUS_IDLE;
  return write_ctl_fresh(s, n, next_id, inactive);
}

static int ensure_graph(bmc_scenario* s, unsigned grid, size_t smem, unsigned variant, int scatter) {
  const unsigned liq = liquid_grid(s->h), plan = plan_slices(s->h);
  if (s->graph && s->graph_smem == smem && s->graph_grid == grid && s->graph_variant == variant &&
      s->graph_liq == liq && s->graph_plan == plan && s->graph_scatter == scatter)
    return BMC_OK;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  cudaGraph_t g = nullptr;
  BMC_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  const unsigned long long before = g_launches.load();
  int rc = enqueue_step(s->ks, s->stream, s->d_desc, 1, liq, plan, s->d_bctl, 1, variant, grid, smem, s->sm_count,
                        s->h.n_maps > 0, scatter);
  g_launches = before;
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&s->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  s->graph_smem = smem;
  s->graph_grid = grid;
  s->graph_variant = variant;
  s->graph_liq = liq;
  s->graph_plan = plan;
  s->graph_scatter = scatter;
  return BMC_OK;
}

// prepare_cycle for a scenario, reusing the last answer while the launch
// shape and the accumulator size are unchanged (no attribute or occupancy
// query per step).
static int scenario_prepare(bmc_scenario* s, size_t* smem, unsigned* grid, unsigned* variant, int* scatter) {
  if (s->prep_variant == s->variant && s->prep_bps == s->blocks_per_sm && s->prep_in == *smem) {
    *smem = s->prep_out;
    *grid = s->prep_grid;
    *variant = s->prep_run;
    *scatter = s->prep_global ? bmc::kScatterGlobal : scenario_scatter(s->ks, s->h);
    return BMC_OK;
  }
  const size_t in = *smem;
  bool glob = false;
  int rc = prepare_cycle(s->ks, s->variant, s->blocks_per_sm, smem, s->sm_count, grid, variant, &glob);
  if (rc) return rc;
  *scatter = glob ? bmc::kScatterGlobal : scenario_scatter(s->ks, s->h);
  s->prep_global = glob;
  s->prep_run = *variant;
  s->prep_variant = s->variant;
  s->prep_bps = s->blocks_per_sm;
  s->prep_in = in;
  s->prep_out = *smem;
  s->prep_grid = *grid;
  return BMC_OK;
}

static int scenario_steps(bmc_scenario* s, double dt, uint32_t n_steps, int do_scalar, bool use_graph) {
  int rc = check_ready(s, do_scalar != 0);
  if (rc) return rc;
  rc = set_dt(s, dt, true);
  if (rc) return rc;
  s->ctl_fresh = false;
  size_t smem = cycle_smem(s->h);
  unsigned grid = 0, variant = 0;
  int scatter = 0;
  rc = scenario_prepare(s, &smem, &grid, &variant, &scatter);
  if (rc) return rc;
  if (use_graph && do_scalar) {
    rc = ensure_graph(s, grid, smem, variant, scatter);
    if (rc) return rc;
    for (uint32_t k = 0; k < n_steps; ++k) {
      BMC_CUDA(cudaGraphLaunch(s->graph, s->stream));
      g_launches += 6;
    }
    return BMC_OK;
  }
  for (uint32_t k = 0; k < n_steps; ++k) {
    rc = enqueue_step(s->ks, s->stream, s->d_desc, 1, liquid_grid(s->h), plan_slices(s->h), s->d_bctl, do_scalar,
                      variant, grid, smem, s->sm_count, s->h.n_maps > 0, scatter);
    if (rc) return rc;
  }
  return BMC_OK;
}

int bmc_cycle(bmc_scenario* s, double dt, bmc_step_stats* stats) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  int rc = scenario_steps(s, dt, 1, 0, false);
  if (rc) return rc;
  return read_ctl(s, stats);
}

int bmc_cycle_external(bmc_scenario* s, double dt, const double* conc, double* sources, int32_t on_device,
                       bmc_step_stats* stats) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !conc || !sources) return fail(BMC_E_INVALID, "null argument");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  const size_t ne = (size_t)s->h.n_c * s->h.n_s;
  const cudaMemcpyKind kin = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind kout = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  // the cycle reads the concentrations from the buffer of the step's parity:
  // both buffers get them
  BMC_CUDA(counted_memcpy_async(s->h.C, conc, ne * 8, kin, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.C + ne, conc, ne * 8, kin, s->stream));
  s->has_conc = true;
  int rc = scenario_steps(s, dt, 1, 0, false);
  if (rc) return rc;
  BMC_CUDA(counted_memcpy_async(sources, s->h.src, ne * 8, kout, s->stream));
  return read_ctl(s, stats);
}

int bmc_step(bmc_scenario* s, double dt, bmc_step_stats* stats) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  int rc = scenario_steps(s, dt, 1, 1, true);
  if (rc) return rc;
  return read_ctl(s, stats);
}

int bmc_step_read(bmc_scenario* s, double dt, bmc_step_stats* stats, double* conc) {
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (!conc) return fail(BMC_E_INVALID, "null concentrations");
  if (s->pend_count > 0) return fail(BMC_E_STATE, "steps enqueued by bmc_step_enqueue are not collected yet");
  // The pipelined pair with nothing else in flight: the step, then one small
  // kernel writing its control block and the concentration buffer it left
  // into mapped host memory, waited for at once.
  bmc_step_stats unused;
  const int rc = bmc_step_enqueue(s, dt, stats ? stats : &unused, conc);
  if (rc) return rc;
  return bmc_step_collect(s);
}

int bmc_run(bmc_scenario* s, double dt, uint32_t n_steps, bmc_step_stats* stats) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  int rc = scenario_steps(s, dt, n_steps, 1, true);
  if (rc) return rc;
  return read_ctl(s, stats);
}

int bmc_run_async(bmc_scenario* s, double dt, uint32_t n_steps) {
  if (const int rc_settle = settle_export(s)) return rc_settle; return scenario_steps(s, dt, n_steps, 1, true); }

int bmc_run_timed(bmc_scenario* s, double dt, uint32_t n_steps, bmc_step_stats* stats, float* elapsed_ms) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  int rc = check_ready(s, true);
  if (rc) return rc;
  rc = set_dt(s, dt, true);  // outside the timed region
  if (rc) return rc;
  cudaEvent_t e0, e1;
  BMC_CUDA(cudaEventCreate(&e0));
  BMC_CUDA(cudaEventCreate(&e1));
  BMC_CUDA(cudaEventRecord(e0, s->stream));
  rc = scenario_steps(s, dt, n_steps, 1, true);
  cudaEventRecord(e1, s->stream);
  if (rc == BMC_OK) rc = read_ctl(s, stats);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (elapsed_ms) *elapsed_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int bmc_synchronize(bmc_scenario* s) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_read_stats(bmc_scenario* s, bmc_step_stats* stats) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  return read_ctl(s, stats);
}

int bmc_read_particles(bmc_scenario* s, uint64_t max_n, void* state, uint32_t* pos, uint8_t* status, float* age_h,
                       float* age_d, uint32_t* id, uint64_t* n_out) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  int rc = read_ctl(s, nullptr);
  if (rc && rc != BMC_E_DEVICE) return rc;
  const uint64_t n = s->h_ctl->n_used;
  if (n_out) *n_out = n;
  if (n > max_n) return fail(BMC_E_CAPACITY, "host buffers smaller than n_used");
  const size_t fsz = s->h.f64 ? 8 : 4;
  if (state)
    for (int v = 0; v < (int)s->h.n_var; ++v)
      BMC_CUDA(counted_memcpy_async(static_cast<char*>(state) + (size_t)v * n * fsz,
                               static_cast<const char*>(s->h.state) + (size_t)v * s->h.cap * fsz, n * fsz,
                               cudaMemcpyDeviceToHost, s->stream));
  if (pos) BMC_CUDA(counted_memcpy_async(pos, s->h.pos, n * 4, cudaMemcpyDeviceToHost, s->stream));
  if (status) BMC_CUDA(counted_memcpy_async(status, s->h.status, n, cudaMemcpyDeviceToHost, s->stream));
  if (age_h) BMC_CUDA(counted_memcpy_async(age_h, s->h.age_h, n * 4, cudaMemcpyDeviceToHost, s->stream));
  if (age_d) BMC_CUDA(counted_memcpy_async(age_d, s->h.age_d, n * 4, cudaMemcpyDeviceToHost, s->stream));
  if (id) BMC_CUDA(counted_memcpy_async(id, s->h.id, n * 4, cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_read_mass(bmc_scenario* s, uint64_t max_n, double* mass, uint64_t* n_out) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  int rc = read_ctl(s, nullptr);
  if (rc && rc != BMC_E_DEVICE) return rc;
  const uint64_t n = s->h_ctl->n_used;
  if (n_out) *n_out = n;
  if (n > max_n) return fail(BMC_E_CAPACITY, "host buffer smaller than n_used");
  if (n == 0 || !mass) return BMC_OK;
  double* d = nullptr;
  BMC_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), n * sizeof(double), s->stream));
  s->ks->mass(s->stream, s->d_desc, n, d);
  g_launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = counted_memcpy_async(mass, d, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  const cudaError_t ef = cudaFreeAsync(d, s->stream);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  BMC_CUDA(e);
  return BMC_OK;
}

int bmc_read_liquid(bmc_scenario* s, double* conc, double* mass, double* sources) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  const size_t ne = (size_t)s->h.n_c * s->h.n_s;
  if (!s->ctl_fresh) {  // the step parity names the current concentration buffer
    int rc = read_ctl(s, nullptr);
    if (rc && rc != BMC_E_DEVICE) return rc;
  }
  const double* cur = s->h.C + (s->h_ctl->step & 1u) * ne;
  if (conc) BMC_CUDA(counted_memcpy_async(conc, cur, ne * 8, cudaMemcpyDeviceToHost, s->stream));
  if (mass) BMC_CUDA(counted_memcpy_async(mass, s->h.M, ne * 8, cudaMemcpyDeviceToHost, s->stream));
  if (sources) BMC_CUDA(counted_memcpy_async(sources, s->h.src, ne * 8, cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_repartition(bmc_scenario* s, uint64_t* counts) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !counts) return fail(BMC_E_INVALID, "null argument");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  unsigned long long* d = nullptr;
  BMC_CUDA(cudaMalloc(&d, s->h.n_c * 8ull));
  cudaError_t e = cudaMemsetAsync(d, 0, s->h.n_c * 8ull, s->stream);
  if (e == cudaSuccess) {
    bmc::launch_repartition(s->stream, s->d_desc, d, s->sm_count * 4);
    g_launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = counted_memcpy_async(counts, d, s->h.n_c * 8ull, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("repartition: ") + cudaGetErrorString(e));
  return BMC_OK;
}

// ---- allocation-free repartition --------------------------------------------------
// Per-compartment counters of bmc_repartition_static: one array in the
// library's static device memory, present on every GPU that loads the
// library until the process exits.  In host code the name below only
// stands in for the array; its device address on a GPU comes from
// cudaGetSymbolAddress with that GPU current, looked up once per device and
// passed to the kernel.
static __device__ __align__(256) unsigned long long g_repartition_scratch[BMC_REPARTITION_STATIC_MAX];

namespace {
std::mutex g_scratch_mu;
std::array<unsigned long long*, 64> g_scratch_ptr{};  // device address of the array, by device ordinal

}  // namespace

int bmc_repartition_static(bmc_scenario* s, uint64_t* counts) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !counts) return fail(BMC_E_INVALID, "null argument");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  if (s->h.n_c > BMC_REPARTITION_STATIC_MAX)
    return fail(BMC_E_CAPACITY, "bmc_repartition_static: " + std::to_string(s->h.n_c) +
                                    " compartments exceed the static scratch of " +
                                    std::to_string(BMC_REPARTITION_STATIC_MAX));
  const int dev = s->device;
  if (dev < 0 || dev >= (int)g_scratch_ptr.size()) return fail(BMC_E_INVALID, "device ordinal out of range");
  // the scenario's device is current for the look-up, the kernel and the copies
  DeviceScope scope(dev);
  if (scope.err != cudaSuccess)
    return fail(BMC_E_CUDA, std::string("bmc_repartition_static: device ") + cudaGetErrorString(scope.err));
  unsigned long long* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      BMC_CUDA(cudaGetSymbolAddress(&p, g_repartition_scratch));
      g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  const size_t bytes = (size_t)s->h.n_c * sizeof(unsigned long long);
  // the array keeps the previous call's counts: clear this call's range
  BMC_CUDA(cudaMemsetAsync(scratch, 0, bytes, s->stream));
  bmc::launch_repartition(s->stream, s->d_desc, scratch, s->sm_count * 4);
  g_launches++;
  BMC_CUDA(cudaGetLastError());
  BMC_CUDA(counted_memcpy_async(counts, scratch, bytes, cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_force_remove_dead(bmc_scenario* s) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  int rc = read_ctl(s, nullptr);
  if (rc) return rc;
  const uint64_t n = s->h_ctl->n_used;
  const size_t fsz = s->h.f64 ? 8 : 4;
  const int nv = (int)s->h.n_var;
  std::vector<char> st((size_t)nv * n * fsz);
  std::vector<uint32_t> pos(n), id(n);
  std::vector<uint8_t> status(n);
  std::vector<float> ah(n), ad(n);
  uint64_t got = 0;
  rc = bmc_read_particles(s, n, st.data(), pos.data(), status.data(), ah.data(), ad.data(), id.data(), &got);
  if (rc) return rc;
  uint64_t r = 0;
  for (uint64_t i = 0; i < n; ++i) r += status[i] != BMC_STATUS_IDLE;
  if (r == 0) return BMC_OK;
  const uint64_t head = n - r;
  std::vector<uint64_t> gaps, srcs;
  for (uint64_t i = 0; i < head; ++i)
    if (status[i] != BMC_STATUS_IDLE) gaps.push_back(i);
  for (uint64_t i = n; i-- > head;)
    if (status[i] == BMC_STATUS_IDLE) srcs.push_back(i);
  for (size_t j = 0; j < gaps.size(); ++j) {
    const uint64_t d = gaps[j], src = srcs[j];
    for (int v = 0; v < nv; ++v) std::memcpy(&st[((size_t)v * n + d) * fsz], &st[((size_t)v * n + src) * fsz], fsz);
    pos[d] = pos[src];
    status[d] = BMC_STATUS_IDLE;
    ah[d] = ah[src];
    ad[d] = ad[src];
    id[d] = id[src];
  }
  // repack the state with the new count as row stride
  std::vector<char> st2((size_t)nv * head * fsz);
  for (int v = 0; v < nv; ++v) std::memcpy(&st2[(size_t)v * head * fsz], &st[(size_t)v * n * fsz], head * fsz);
  return bmc_set_particles(s, head, st2.data(), pos.data(), status.data(), ah.data(), ad.data(), id.data(),
                           s->h_ctl->next_id);
}

// ---- time-event probes ---------------------------------------------------------------
}  // extern "C"

// Reads, changes and writes back the control block between steps.
template <class Fn>
static int ctl_update(bmc_scenario* s, Fn fn) {
  BMC_CUDA(counted_memcpy_async(s->h_ctl, s->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  Control c = *s->h_ctl;
  fn(c);
  *s->h_ctl = c;
  BMC_CUDA(counted_memcpy_async(s->d_ctl, &c, sizeof(Control), cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

extern "C" {

int bmc_read_events(bmc_scenario* s, uint64_t* counts, int32_t clear) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !counts) return fail(BMC_E_INVALID, "null argument");
  if (clear && s->pend_count > 0) return fail(BMC_E_STATE, "steps enqueued by bmc_step_enqueue are not collected yet");
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  int rc = read_ctl(s, nullptr);
  if (rc && rc != BMC_E_DEVICE) return rc;
  for (int k = 0; k < BMC_N_EVENTS; ++k) counts[k] = s->h_ctl->events[k];
  if (!clear) return BMC_OK;
  rc = ctl_update(s, [](Control& c) {
    for (auto& e : c.events) e = 0ull;
  });
  if (rc) return rc;
  s->ctl_fresh = false;
  return BMC_OK;
}

int bmc_probe_enable(bmc_scenario* s, uint64_t capacity) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (s->pend_count > 0) return fail(BMC_E_STATE, "steps enqueued by bmc_step_enqueue are not collected yet");
  if (capacity > (1ull << 32)) return fail(BMC_E_INVALID, "probe capacity above 2^32 values");
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  if (s->probe_arena) cudaFree(s->probe_arena);
  s->probe_arena = nullptr;
  s->h.probe_buf[0] = s->h.probe_buf[1] = nullptr;
  s->h.probe_cap = 0;
  if (capacity > 0) {
    BMC_CUDA(cudaMalloc(&s->probe_arena, 2 * capacity * sizeof(double)));
    BMC_CUDA(cudaMemsetAsync(s->probe_arena, 0, 2 * capacity * sizeof(double), s->stream));
    s->h.probe_buf[0] = static_cast<double*>(s->probe_arena);
    s->h.probe_buf[1] = s->h.probe_buf[0] + capacity;
    s->h.probe_cap = capacity;
  }
  int rc = ctl_update(s, [](Control& c) { c.probe_n[0] = c.probe_n[1] = 0ull; });
  if (rc) return rc;
  s->ctl_fresh = false;
  return upload_desc(s);
}

int bmc_probe_read(bmc_scenario* s, int32_t probe, double* out, uint64_t max_values, uint64_t* count) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !count) return fail(BMC_E_INVALID, "null argument");
  if (probe != BMC_PROBE_LEAVING_TIME && probe != BMC_PROBE_DIVISION_TIME) return fail(BMC_E_INVALID, "unknown probe");
  if (max_values > 0 && !out) return fail(BMC_E_INVALID, "null output");
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  int rc = read_ctl(s, nullptr);
  if (rc && rc != BMC_E_DEVICE) return rc;
  const uint64_t n = s->h_ctl->probe_n[probe];
  *count = n;
  const uint64_t stored = std::min<uint64_t>(std::min<uint64_t>(n, s->h.probe_cap), max_values);
  if (stored > 0) {
    BMC_CUDA(counted_memcpy_async(out, s->h.probe_buf[probe], stored * sizeof(double), cudaMemcpyDeviceToHost,
                                  s->stream));
    BMC_CUDA(cudaStreamSynchronize(s->stream));
  }
  return BMC_OK;
}

int bmc_probe_clear(bmc_scenario* s, int32_t probe) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (probe != BMC_PROBE_LEAVING_TIME && probe != BMC_PROBE_DIVISION_TIME) return fail(BMC_E_INVALID, "unknown probe");
  if (s->pend_count > 0) return fail(BMC_E_STATE, "steps enqueued by bmc_step_enqueue are not collected yet");
  DeviceScope on(s->device);
  BMC_CUDA(on.err);
  if (s->h.probe_cap > 0)
    BMC_CUDA(cudaMemsetAsync(s->h.probe_buf[probe], 0, s->h.probe_cap * sizeof(double), s->stream));
  int rc = ctl_update(s, [probe](Control& c) { c.probe_n[probe] = 0ull; });
  if (rc) return rc;
  s->ctl_fresh = false;
  return BMC_OK;
}

// ---- batching ------------------------------------------------------------------

// Stream, descriptor table, control blocks and live-tile prefix of a batch
// of n slots; empty slots point at a control block of a finished scenario.
static int batch_alloc(bmc_batch* b, uint32_t n) {
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_table, sizeof(ScenDev) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_bctl, sizeof(BatchCtl));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_live, sizeof(unsigned) * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_dummy_ctl, sizeof(Control));
  if (e == cudaSuccess) {
    Control c{};
    c.step = 1u;  // with step_limit 1: finished
    e = cudaMemcpy(b->d_dummy_ctl, &c, sizeof(Control), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    if (b->d_table) cudaFree(b->d_table);
    if (b->d_bctl) cudaFree(b->d_bctl);
    if (b->d_live) cudaFree(b->d_live);
    if (b->d_dummy_ctl) cudaFree(b->d_dummy_ctl);
    if (b->stream) cudaStreamDestroy(b->stream);
    return fail(BMC_E_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
  }
  return BMC_OK;
}

int bmc_batch_create(bmc_scenario* const* scenarios, uint32_t n, bmc_batch** out) {
  if (!scenarios || n == 0 || !out) return fail(BMC_E_INVALID, "empty batch");
  auto* b = new bmc_batch();
  b->scen.assign(scenarios, scenarios + n);
  b->ks = scenarios[0]->ks;
  for (uint32_t i = 0; i < n; ++i) {
    if (!scenarios[i] || scenarios[i]->ks != b->ks) {
      delete b;
      return fail(BMC_E_INVALID, "all scenarios of a batch must share model and precision");
    }
    int rc = check_ready(scenarios[i], true);
    if (rc) {
      delete b;
      return rc;
    }
    cudaStreamSynchronize(scenarios[i]->stream);
  }
  b->sm_count = scenarios[0]->sm_count;
  int rc = batch_alloc(b, n);
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return BMC_OK;
}

int bmc_batch_create_slots(uint32_t capacity, int32_t model, int32_t f64, bmc_batch** out) {
  if (capacity == 0 || !out) return fail(BMC_E_INVALID, "empty batch");
  const bmc::KernelSet* ks = bmc::kernel_set(model, f64);
  if (!ks) return fail(BMC_E_UNSUPPORTED, "model / precision not compiled in");
  auto* b = new bmc_batch();
  b->ks = ks;
  b->scen.assign(capacity, nullptr);
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    delete b;
    return fail(BMC_E_CUDA, "cannot query the device");
  }
  int rc = batch_alloc(b, capacity);
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return BMC_OK;
}

int bmc_batch_set_slot(bmc_batch* b, uint32_t slot, bmc_scenario* s) {
  if (!b || slot >= b->scen.size()) return fail(BMC_E_INVALID, "no such slot");
  if (s) {
    if (s->ks != b->ks) return fail(BMC_E_INVALID, "all scenarios of a batch must share model and precision");
    for (size_t i = 0; i < b->scen.size(); ++i)
      if (b->scen[i] == s && i != slot) return fail(BMC_E_INVALID, "scenario already holds another slot");
    int rc = check_ready(s, true);
    if (rc) return rc;
    BMC_CUDA(cudaStreamSynchronize(s->stream));
  }
  // the slot's previous scenario may still be in use by queued steps
  BMC_CUDA(cudaStreamSynchronize(b->stream));
  b->scen[slot] = s;
  return BMC_OK;
}

int bmc_batch_destroy(bmc_batch* b) {
  if (!b) return BMC_OK;
  cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->d_table);
  cudaFree(b->d_bctl);
  cudaFree(b->d_live);
  if (b->d_dummy_ctl) cudaFree(b->d_dummy_ctl);
  cudaStreamDestroy(b->stream);
  delete b;
  return BMC_OK;
}

int bmc_set_step_limit(bmc_scenario* s, uint32_t step_limit) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  s->h.step_limit = step_limit;
  int rc = upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_set_shape(bmc_scenario* s, uint32_t threads, uint32_t ppt, uint32_t blocks_per_sm) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (threads || ppt) {  // 0 and 0 keep the current variant (the automatic one included)
    const unsigned cur = s->variant == bmc::kVariantAuto ? bmc::kAutoStaged : s->variant;
    const unsigned th = threads ? threads : bmc::kVariantThreads[cur];
    const unsigned pp = ppt ? ppt : bmc::kVariantPPT[cur];
    const int v = variant_of(th, pp);
    if (v < 0) return fail(BMC_E_INVALID, "no compiled cycle variant with this threads x ppt");
    s->variant = (unsigned)v;
  }
  s->blocks_per_sm = blocks_per_sm;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  return BMC_OK;
}

int bmc_batch_set_shape(bmc_batch* b, uint32_t threads, uint32_t ppt, uint32_t blocks_per_sm) {
  if (!b) return fail(BMC_E_INVALID, "null batch");
  if (threads || ppt) {  // 0 and 0 keep the current variant (the automatic one included)
    const unsigned cur = b->variant == bmc::kVariantAuto ? bmc::kAutoStaged : b->variant;
    const unsigned th = threads ? threads : bmc::kVariantThreads[cur];
    const unsigned pp = ppt ? ppt : bmc::kVariantPPT[cur];
    const int v = variant_of(th, pp);
    if (v < 0) return fail(BMC_E_INVALID, "no compiled cycle variant with this threads x ppt");
    b->variant = (unsigned)v;
  }
  b->blocks_per_sm = blocks_per_sm;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  return BMC_OK;
}

int bmc_batch_run(bmc_batch* b, double dt, uint32_t n_steps) {
  if (b)
    for (bmc_scenario* m : b->scen)
      if (m) m->ctl_fresh = false;
  int n = 0;
  unsigned max_nc = 0, grid = 0;
  size_t smem = 0;
  int rc = batch_prepare(b, dt, &n, &max_nc, &smem, &grid);
  if (rc) return rc;
  const int scatter = batch_scatter(b);
  if (!b->graph || b->graph_smem != smem || b->graph_grid != grid || b->graph_variant != b->run_variant ||
      b->graph_maps != batch_has_maps(b) || b->graph_liq != max_nc || b->graph_plan != b->plan_y ||
      b->graph_scatter != scatter) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    cudaGraph_t g = nullptr;
    BMC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const unsigned long long before = g_launches.load();
    rc = enqueue_step(b->ks, b->stream, b->d_table, n, max_nc, b->plan_y, b->d_bctl, 1, b->run_variant, grid,
                      smem, b->sm_count, batch_has_maps(b), scatter);
    g_launches = before;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    b->graph_smem = smem;
    b->graph_grid = grid;
    b->graph_variant = b->run_variant;
    b->graph_maps = batch_has_maps(b);
    b->graph_liq = max_nc;
    b->graph_plan = b->plan_y;
    b->graph_scatter = scatter;
  }
  for (uint32_t k = 0; k < n_steps; ++k) {
    BMC_CUDA(cudaGraphLaunch(b->graph, b->stream));
    g_launches += 6;
  }
  return BMC_OK;
}

int bmc_batch_synchronize(bmc_batch* b) {
  if (!b) return fail(BMC_E_INVALID, "null batch");
  BMC_CUDA(cudaStreamSynchronize(b->stream));
  return BMC_OK;
}

// ---- two-phase flow: gas phase -------------------------------------------------------
// Reference: SimulationUnit with is_two_phase_flow (gas ScalarSimulation,
// apps/libs/simulation/src/simulation.cpp L47-L81, L133-L139), ode_step
// (simulation.model.cpp L132-L150: transfer, gas step, liquid step,
// clearNegs), gas feeds (simulation.model.cpp L112-L119) and the FixedKla
// transfer (hydro/impl_mtr.cpp L150-L166).

namespace {
int upload_maps(bmc_scenario* s);  // flow maps to the device (below)
}  // namespace

extern "C" {

int bmc_gas_set(bmc_scenario* s, const double* gas_volume, uint64_t nnz, const uint64_t* rows, const uint64_t* cols,
                const double* values, const double* henry, const double* kla) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !gas_volume || !henry || !kla || (nnz && (!rows || !cols || !values)))
    return fail(BMC_E_INVALID, "bad gas arguments");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set (bmc_domain_update fixes n_compartments)");
  ScenDev& h = s->h;
  const uint32_t n_c = h.n_c;
  const size_t ne = (size_t)n_c * h.n_s;
  std::vector<double> gv(gas_volume, gas_volume + n_c), gvinv(n_c);
  for (uint32_t j = 0; j < n_c; ++j) {
    if (!(gv[j] > 0.0)) return fail(BMC_E_INVALID, "gas volumes must be > 0");
    gvinv[j] = 1.0 / gv[j];
  }
  for (size_t e = 0; e < ne; ++e)
    if (!(kla[e] >= 0.0)) return fail(BMC_E_INVALID, "kla must be >= 0");
  std::vector<uint32_t> ptr, idx;
  std::vector<double> val, diag;
  if (const char* why = build_csr(n_c, nnz, rows, cols, values, ptr, idx, val, diag)) return fail(BMC_E_INVALID, why);
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  if (s->garena) cudaFree(s->garena);
  s->garena = nullptr;
  Carver cv;
  double *p_gvinv = nullptr, *p_flow = nullptr, *p_diag = nullptr, *p_kla = nullptr;
  uint32_t *p_ptr = nullptr, *p_idx = nullptr;
  cv.add(&p_gvinv, n_c);
  cv.add(&p_ptr, n_c + 1);
  cv.add(&p_idx, idx.size());
  cv.add(&p_flow, val.size());
  cv.add(&p_diag, n_c);
  cv.add(&p_kla, ne);
  cv.add(&h.Cg, 2 * ne);
  cv.add(&h.Mg, ne);
  cv.add(&h.mtr, ne);
  BMC_CUDA(cudaMalloc(&s->garena, cv.off));
  cv.bind(s->garena);
  BMC_CUDA(cudaMemsetAsync(s->garena, 0, cv.off, s->stream));
  BMC_CUDA(counted_memcpy_async(p_gvinv, gvinv.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(p_ptr, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice, s->stream));
  if (!idx.empty()) {
    BMC_CUDA(counted_memcpy_async(p_idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_flow, val.data(), val.size() * 8, cudaMemcpyHostToDevice, s->stream));
  }
  BMC_CUDA(counted_memcpy_async(p_diag, diag.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(p_kla, kla, ne * 8, cudaMemcpyHostToDevice, s->stream));
  h.gvinv = p_gvinv;
  h.g_in_ptr = p_ptr;
  h.g_in_idx = p_idx;
  h.g_in_flow = p_flow;
  h.g_diag = p_diag;
  h.kla = p_kla;
  for (int k = 0; k < bmc::kMaxSpecies; ++k) h.henry[k] = k < (int)h.n_s ? henry[k] : 0.0;
  h.gas = 1;
  s->gvol = gv;
  s->g_vinv = gvinv;
  s->g_diag = diag;
  s->g_ptr = ptr;
  s->g_idx = idx;
  s->g_val = val;
  s->g_kla.assign(kla, kla + ne);
  s->g_cur_ptr = p_ptr;
  s->g_cur_idx = p_idx;
  s->g_cur_flow = p_flow;
  // gas states of the flow maps belonged to the previous gas domain
  bool had = false;
  for (auto& m : s->maps) {
    had = had || m.has_gas;
    m.has_gas = false;
  }
  int rc = had ? upload_maps(s) : upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_gas_set_concentrations(bmc_scenario* s, const double* conc) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !conc) return fail(BMC_E_INVALID, "null argument");
  if (!s->h.gas) return fail(BMC_E_STATE, "no gas phase (bmc_gas_set)");
  const size_t n_c = s->h.n_c, ns = s->h.n_s;
  std::vector<double> C(conc, conc + n_c * ns), M(n_c * ns);
  for (size_t j = 0; j < n_c; ++j)
    for (size_t sp = 0; sp < ns; ++sp) {
      if (!(C[j * ns + sp] >= 0.0)) return fail(BMC_E_INVALID, "concentrations must be >= 0");
      M[j * ns + sp] = C[j * ns + sp] * s->gvol[j];
    }
  BMC_CUDA(counted_memcpy_async(s->h.Cg, C.data(), C.size() * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.Cg + C.size(), C.data(), C.size() * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(counted_memcpy_async(s->h.Mg, M.data(), M.size() * 8, cudaMemcpyHostToDevice, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_gas_set_feeds(bmc_scenario* s, uint32_t n_feeds, const bmc_feed* feeds) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || (n_feeds && !feeds)) return fail(BMC_E_INVALID, "null argument");
  if (n_feeds > (uint32_t)bmc::kMaxOutlets) return fail(BMC_E_INVALID, "at most 8 gas feeds");
  if (!s->h.gas) return fail(BMC_E_STATE, "no gas phase (bmc_gas_set)");
  ScenDev& h = s->h;
  for (uint32_t f = 0; f < n_feeds; ++f) {
    if (feeds[f].inlet >= h.n_c || feeds[f].outlet >= (int32_t)h.n_c || feeds[f].outlet < -1)
      return fail(BMC_E_INVALID, "gas feed position out of range");
    if (!(feeds[f].flow >= 0.0)) return fail(BMC_E_INVALID, "gas feed flow must be >= 0");
  }
  h.n_gfeeds = n_feeds;
  for (uint32_t f = 0; f < n_feeds; ++f) {
    h.gfeed_in[f] = feeds[f].inlet;
    h.gfeed_out[f] = feeds[f].outlet;
    h.gfeed_flow[f] = feeds[f].flow;
    for (int sp = 0; sp < bmc::kMaxSpecies; ++sp) h.gfeed_conc[f * bmc::kMaxSpecies + sp] = feeds[f].conc[sp];
  }
  return upload_desc(s);
}

int bmc_gas_read(bmc_scenario* s, double* conc, double* mass, double* transfer) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (!s->h.gas) return fail(BMC_E_STATE, "no gas phase (bmc_gas_set)");
  const size_t ne = (size_t)s->h.n_c * s->h.n_s;
  if (!s->ctl_fresh) {
    int rc = read_ctl(s, nullptr);
    if (rc && rc != BMC_E_DEVICE) return rc;
  }
  const double* cur = s->h.Cg + (s->h_ctl->step & 1u) * ne;
  if (conc) BMC_CUDA(counted_memcpy_async(conc, cur, ne * 8, cudaMemcpyDeviceToHost, s->stream));
  if (mass) BMC_CUDA(counted_memcpy_async(mass, s->h.Mg, ne * 8, cudaMemcpyDeviceToHost, s->stream));
  if (transfer) BMC_CUDA(counted_memcpy_async(transfer, s->h.mtr, ne * 8, cudaMemcpyDeviceToHost, s->stream));
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

}  // extern "C"

// ---- flow-map cycle -----------------------------------------------------------------

namespace {

// Uploads every map of the cycle (one arena) and sizes the current
// incoming-flow lists for the largest map; map 0 is copied in at the next
// step (map_cur reset).
int upload_maps(bmc_scenario* s) {
  ScenDev& h = s->h;
  const size_t nm = s->maps.size(), n_c = h.n_c, K = h.K;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  if (s->marena) {
    // the current incoming-flow lists lived in the map arena: a transition
    // has to be given again (bmc_set_transition_coo) before the next step
    cudaFree(s->marena);
    s->marena = nullptr;
    h.in_ptr = nullptr;
    h.in_idx = nullptr;
    h.in_flow = nullptr;
    s->has_transition = false;
  }
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  // the gas domain of bmc_gas_set back in place (a switch to a map's gas
  // state overwrites it); the maps' gas states are carved below when every
  // map has one
  if (h.gas) {
    h.g_in_ptr = s->g_cur_ptr;
    h.g_in_idx = s->g_cur_idx;
    h.g_in_flow = s->g_cur_flow;
    BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.gvinv), s->g_vinv.data(), n_c * 8, cudaMemcpyHostToDevice,
                                  s->stream));
    BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.g_diag), s->g_diag.data(), n_c * 8, cudaMemcpyHostToDevice,
                                  s->stream));
    BMC_CUDA(counted_memcpy_async(const_cast<double*>(h.kla), s->g_kla.data(), s->g_kla.size() * 8,
                                  cudaMemcpyHostToDevice, s->stream));
  }
  h.map_gvinv = h.map_g_diag = h.map_g_in_flow = h.map_kla = nullptr;
  h.map_g_in_ptr = h.map_g_in_idx = nullptr;
  h.map_g_nnz_max = 0;
  if (nm == 0) {
    h.n_maps = 0;
    h.n_per_map = 1;
    h.map_mrow = nullptr;
    h.map_volume = h.map_vinv = h.map_out_flow = h.map_diag = h.map_in_flow = nullptr;
    h.map_in_ptr = h.map_in_idx = h.map_exit_thr = nullptr;
    s->d_map_exit = nullptr;
    int rc = upload_desc(s);
    if (rc) return rc;
    BMC_CUDA(cudaStreamSynchronize(s->stream));
    return BMC_OK;
  }
  size_t nnz_max = 1;
  for (const auto& m : s->maps) nnz_max = std::max(nnz_max, m.idx.size());
  Carver cv;
  int2* p_mrow = nullptr;
  double *p_vol = nullptr, *p_vinv = nullptr, *p_out = nullptr, *p_diag = nullptr, *p_flow = nullptr;
  uint32_t *p_ptr = nullptr, *p_idx = nullptr, *p_exit = nullptr;
  cv.add(&p_mrow, nm * n_c * K);
  cv.add(&p_vol, nm * n_c);
  cv.add(&p_vinv, nm * n_c);
  cv.add(&p_out, nm * n_c);
  cv.add(&p_diag, nm * n_c);
  cv.add(&p_ptr, nm * (n_c + 1));
  cv.add(&p_idx, nm * nnz_max);
  cv.add(&p_flow, nm * nnz_max);
  cv.add(&p_exit, nm * bmc::kMaxOutlets);
  // current incoming-flow lists, large enough for every map
  uint32_t *c_ptr = nullptr, *c_idx = nullptr;
  double* c_flow = nullptr;
  cv.add(&c_ptr, n_c + 1);
  cv.add(&c_idx, nnz_max);
  cv.add(&c_flow, nnz_max);
  // gas states, when every map has one, and the current gas transition
  // lists, large enough for every map's
  const bool gas_maps =
      h.gas && std::all_of(s->maps.begin(), s->maps.end(), [](const bmc_scenario::FlowMap& m) { return m.has_gas; });
  const size_t ne = n_c * h.n_s;
  size_t gmax = 1;
  double *q_gvinv = nullptr, *q_gdiag = nullptr, *q_gflow = nullptr, *q_kla = nullptr, *cg_flow = nullptr;
  uint32_t *q_gptr = nullptr, *q_gidx = nullptr, *cg_ptr = nullptr, *cg_idx = nullptr;
  if (gas_maps) {
    for (const auto& m : s->maps) gmax = std::max(gmax, m.gidx.size());
    cv.add(&q_gvinv, nm * n_c);
    cv.add(&q_gdiag, nm * n_c);
    cv.add(&q_gptr, nm * (n_c + 1));
    cv.add(&q_gidx, nm * gmax);
    cv.add(&q_gflow, nm * gmax);
    cv.add(&q_kla, nm * ne);
    cv.add(&cg_ptr, n_c + 1);
    cv.add(&cg_idx, gmax);
    cv.add(&cg_flow, gmax);
  }
  BMC_CUDA(cudaMalloc(&s->marena, cv.off));
  cv.bind(s->marena);
  BMC_CUDA(cudaMemsetAsync(s->marena, 0, cv.off, s->stream));
  for (size_t m = 0; m < nm; ++m) {
    const auto& f = s->maps[m];
    BMC_CUDA(counted_memcpy_async(p_mrow + m * n_c * K, f.mrow.data(), n_c * K * sizeof(int2), cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_vol + m * n_c, f.vol.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_vinv + m * n_c, f.vinv.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_out + m * n_c, f.outf.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_diag + m * n_c, f.diag.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
    BMC_CUDA(counted_memcpy_async(p_ptr + m * (n_c + 1), f.ptr.data(), (n_c + 1) * 4, cudaMemcpyHostToDevice, s->stream));
    if (!f.idx.empty()) {
      BMC_CUDA(counted_memcpy_async(p_idx + m * nnz_max, f.idx.data(), f.idx.size() * 4, cudaMemcpyHostToDevice, s->stream));
      BMC_CUDA(counted_memcpy_async(p_flow + m * nnz_max, f.val.data(), f.val.size() * 8, cudaMemcpyHostToDevice, s->stream));
    }
  }
  h.map_mrow = p_mrow;
  h.map_volume = p_vol;
  h.map_vinv = p_vinv;
  h.map_out_flow = p_out;
  h.map_diag = p_diag;
  h.map_in_ptr = p_ptr;
  h.map_in_idx = p_idx;
  h.map_in_flow = p_flow;
  h.map_exit_thr = p_exit;
  h.map_nnz_max = (uint32_t)nnz_max;
  if (gas_maps) {
    for (size_t m = 0; m < nm; ++m) {
      const auto& f = s->maps[m];
      BMC_CUDA(counted_memcpy_async(q_gvinv + m * n_c, f.gvinv.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
      BMC_CUDA(counted_memcpy_async(q_gdiag + m * n_c, f.gdiag.data(), n_c * 8, cudaMemcpyHostToDevice, s->stream));
      BMC_CUDA(counted_memcpy_async(q_gptr + m * (n_c + 1), f.gptr.data(), (n_c + 1) * 4, cudaMemcpyHostToDevice,
                                    s->stream));
      if (!f.gidx.empty()) {
        BMC_CUDA(counted_memcpy_async(q_gidx + m * gmax, f.gidx.data(), f.gidx.size() * 4, cudaMemcpyHostToDevice,
                                      s->stream));
        BMC_CUDA(counted_memcpy_async(q_gflow + m * gmax, f.gval.data(), f.gval.size() * 8, cudaMemcpyHostToDevice,
                                      s->stream));
      }
      BMC_CUDA(counted_memcpy_async(q_kla + m * ne, f.kla.data(), ne * 8, cudaMemcpyHostToDevice, s->stream));
    }
    h.map_gvinv = q_gvinv;
    h.map_g_diag = q_gdiag;
    h.map_g_in_ptr = q_gptr;
    h.map_g_in_idx = q_gidx;
    h.map_g_in_flow = q_gflow;
    h.map_kla = q_kla;
    h.map_g_nnz_max = (uint32_t)gmax;
    // filled by the first step's switch to a map
    h.g_in_ptr = cg_ptr;
    h.g_in_idx = cg_idx;
    h.g_in_flow = cg_flow;
  }
  s->d_map_exit = p_exit;
  h.in_ptr = c_ptr;
  h.in_idx = c_idx;
  h.in_flow = c_flow;
  s->has_transition = true;
  // the host's view of the volumes (outlet thresholds of the fixed-domain
  // path) follows map 0 until the device switches
  s->volume = s->maps[0].vol;
  derive_outlets(s);
  int rc = refresh_map_tables(s);
  if (rc) return rc;
  const unsigned none = 0xffffffffu;
  BMC_CUDA(counted_memcpy_async(&s->d_ctl->map_cur, &none, sizeof(none), cudaMemcpyHostToDevice, s->stream));
  s->ctl_fresh = false;
  rc = upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

}  // namespace

extern "C" {

int bmc_flowmap_add(bmc_scenario* s, const double* volume, const uint64_t* neighbors, const double* out_flows,
                    const double* cdf, uint64_t nnz, const uint64_t* rows, const uint64_t* cols, const double* values) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !volume || !out_flows || (nnz && (!rows || !cols || !values)))
    return fail(BMC_E_INVALID, "bad flow-map arguments");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set (bmc_domain_update fixes n_compartments and K)");
  const uint32_t n_c = s->h.n_c, K = s->h.K;
  if (n_c > 1 && (!neighbors || !cdf)) return fail(BMC_E_INVALID, "neighbors and cdf required when n_c > 1");
  bmc_scenario::FlowMap f;
  if (const char* why = build_rows(n_c, K, neighbors, cdf, f.mrow)) return fail(BMC_E_INVALID, why);
  f.vol.assign(volume, volume + n_c);
  f.outf.assign(out_flows, out_flows + n_c);
  f.vinv.resize(n_c);
  for (uint32_t j = 0; j < n_c; ++j) {
    if (!(f.vol[j] > 0.0)) return fail(BMC_E_INVALID, "volumes must be > 0");
    if (!(f.outf[j] >= 0.0)) return fail(BMC_E_INVALID, "out flows must be >= 0");
    f.vinv[j] = 1.0 / f.vol[j];
  }
  if (const char* why = build_csr(n_c, nnz, rows, cols, values, f.ptr, f.idx, f.val, f.diag))
    return fail(BMC_E_INVALID, why);
  if (nnz == 0)
    for (uint32_t j = 0; j < n_c; ++j) f.diag[j] = -f.outf[j];
  s->maps.push_back(std::move(f));
  return upload_maps(s);
}

int bmc_flowmap_add_gas(bmc_scenario* s, uint32_t map, const double* gas_volume, uint64_t nnz, const uint64_t* rows,
                        const uint64_t* cols, const double* values, const double* kla) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !gas_volume || (nnz && (!rows || !cols || !values))) return fail(BMC_E_INVALID, "bad gas flow-map arguments");
  if (!s->h.gas) return fail(BMC_E_STATE, "no gas phase (bmc_gas_set)");
  if (map >= s->maps.size()) return fail(BMC_E_INVALID, "no such flow map (bmc_flowmap_add first)");
  const uint32_t n_c = s->h.n_c;
  const size_t ne = (size_t)n_c * s->h.n_s;
  bmc_scenario::FlowMap& f = s->maps[map];
  std::vector<double> gvinv(n_c);
  for (uint32_t j = 0; j < n_c; ++j) {
    if (!(gas_volume[j] > 0.0)) return fail(BMC_E_INVALID, "gas volumes must be > 0");
    gvinv[j] = 1.0 / gas_volume[j];
  }
  std::vector<double> k(kla ? kla : s->g_kla.data(), (kla ? kla : s->g_kla.data()) + ne);
  for (double v : k)
    if (!(v >= 0.0)) return fail(BMC_E_INVALID, "kla must be >= 0");
  std::vector<uint32_t> ptr, idx;
  std::vector<double> val, diag;
  if (const char* why = build_csr(n_c, nnz, rows, cols, values, ptr, idx, val, diag)) return fail(BMC_E_INVALID, why);
  f.gvinv = std::move(gvinv);
  f.gdiag = std::move(diag);
  f.gptr = std::move(ptr);
  f.gidx = std::move(idx);
  f.gval = std::move(val);
  f.kla = std::move(k);
  f.has_gas = true;
  return upload_maps(s);
}

int bmc_flowmap_period(bmc_scenario* s, double t_per_flowmap) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !(t_per_flowmap >= 0.0)) return fail(BMC_E_INVALID, "t_per_flowmap must be >= 0");
  s->t_per_map = t_per_flowmap;
  int rc = refresh_map_tables(s);
  if (rc) return rc;
  rc = upload_desc(s);
  if (rc) return rc;
  BMC_CUDA(cudaStreamSynchronize(s->stream));
  return BMC_OK;
}

int bmc_flowmap_clear(bmc_scenario* s) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  s->maps.clear();
  return upload_maps(s);
}

}  // extern "C"

// ---- diagnostics -----------------------------------------------------------------

int bmc_step_timed(bmc_scenario* s, double dt, bmc_step_stats* stats, float* kernel_ms) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  int rc = check_ready(s, true);
  if (rc) return rc;
  rc = set_dt(s, dt, true);
  if (rc) return rc;
  size_t smem = cycle_smem(s->h);
  unsigned grid = 0, variant = 0;
  int scatter = 0;
  rc = scenario_prepare(s, &smem, &grid, &variant, &scatter);
  if (rc) return rc;
  cudaEvent_t ev[7];
  for (auto& e : ev) BMC_CUDA(cudaEventCreate(&e));
  cudaStream_t st = s->stream;
  if (s->h.n_maps > 0) {
    s->ks->flowmap(1, st, s->d_desc);
    g_launches++;
  }
  BMC_CUDA(cudaEventRecord(ev[0], st));
  s->ks->liquid(1, liquid_grid(s->h), st, s->d_desc, s->d_bctl, 1);
  BMC_CUDA(cudaEventRecord(ev[1], st));
  s->ks->cycle[variant](dim3(grid), dim3(bmc::kVariantThreads[variant]), smem, st, s->d_desc, 1, s->d_bctl,
                        scatter);
  BMC_CUDA(cudaEventRecord(ev[2], st));
  s->ks->plan(1, plan_slices(s->h), st, s->d_desc, s->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[3], st));
  s->ks->divide(dim3(s->sm_count * 4), st, s->d_desc, 1, s->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[4], st));
  s->ks->compact(dim3(s->sm_count * 2), st, s->d_desc, 1, s->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[5], st));
  s->ks->merge(dim3(s->sm_count * 2), st, s->d_desc, 1, s->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[6], st));
  g_launches += 6;
  BMC_CUDA(launch_status(s->ks));
  rc = read_ctl(s, stats);
  for (int k = 0; k < 6 && kernel_ms; ++k) cudaEventElapsedTime(&kernel_ms[k], ev[k], ev[k + 1]);
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

int bmc_batch_step_timed(bmc_batch* b, double dt, float* kernel_ms) {
  if (b)
    for (bmc_scenario* m : b->scen)
      if (m) m->ctl_fresh = false;
  int n = 0;
  unsigned max_nc = 0, grid = 0;
  size_t smem = 0;
  int rc = batch_prepare(b, dt, &n, &max_nc, &smem, &grid);
  if (rc) return rc;
  const int sm = b->sm_count;
  cudaEvent_t ev[7];
  for (auto& e : ev) BMC_CUDA(cudaEventCreate(&e));
  cudaStream_t st = b->stream;
  const unsigned variant = b->run_variant;
  if (batch_has_maps(b)) {
    b->ks->flowmap(n, st, b->d_table);
    g_launches++;
  }
  BMC_CUDA(cudaEventRecord(ev[0], st));
  b->ks->liquid(n, max_nc, st, b->d_table, b->d_bctl, 1);
  BMC_CUDA(cudaEventRecord(ev[1], st));
  b->ks->cycle[variant](dim3(grid), dim3(bmc::kVariantThreads[variant]), smem, st, b->d_table, n, b->d_bctl,
                        batch_scatter(b));
  BMC_CUDA(cudaEventRecord(ev[2], st));
  b->ks->plan(n, b->plan_y, st, b->d_table, b->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[3], st));
  b->ks->divide(dim3(sm * 4), st, b->d_table, n, b->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[4], st));
  b->ks->compact(dim3(sm * 2), st, b->d_table, n, b->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[5], st));
  b->ks->merge(dim3(sm * 2), st, b->d_table, n, b->d_bctl);
  BMC_CUDA(cudaEventRecord(ev[6], st));
  g_launches += 6;
  BMC_CUDA(launch_status(b->ks));
  BMC_CUDA(cudaStreamSynchronize(st));
  for (int k = 0; k < 6 && kernel_ms; ++k) cudaEventElapsedTime(&kernel_ms[k], ev[k], ev[k + 1]);
  for (auto& e : ev) cudaEventDestroy(e);
  return BMC_OK;
}

int bmc_debug_draws(uint64_t seed, const uint32_t* ids, uint64_t n, uint32_t step, uint32_t purpose, float* out) {
  if (!ids || !out || n == 0) return fail(BMC_E_INVALID, "bad arguments");
  uint32_t* d_ids = nullptr;
  float* d_out = nullptr;
  BMC_CUDA(cudaMalloc(&d_ids, n * 4));
  cudaError_t e = cudaMalloc(&d_out, n * 16);
  if (e == cudaSuccess) e = counted_memcpy(d_ids, ids, n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    bmc::launch_debug_draws(0, seed, d_ids, n, step, purpose, d_out);
    g_launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = counted_memcpy(out, d_out, n * 16, cudaMemcpyDeviceToHost);
  cudaFree(d_ids);
  if (d_out) cudaFree(d_out);
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("debug draws: ") + cudaGetErrorString(e));
  return BMC_OK;
}

int bmc_debug_age_add(const float* ages, uint64_t n, double dt, float* out) {
  if (!ages || !out || n == 0 || !(dt >= 0.0)) return fail(BMC_E_INVALID, "bad arguments");
  float* d_a = nullptr;
  float* d_out = nullptr;
  BMC_CUDA(cudaMalloc(&d_a, n * 4));
  cudaError_t e = cudaMalloc(&d_out, n * 4);
  if (e == cudaSuccess) e = counted_memcpy(d_a, ages, n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    bmc::launch_debug_age_add(0, d_a, n, dt, d_out);
    g_launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = counted_memcpy(out, d_out, n * 4, cudaMemcpyDeviceToHost);
  cudaFree(d_a);
  if (d_out) cudaFree(d_out);
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("debug age add: ") + cudaGetErrorString(e));
  return BMC_OK;
}

int bmc_debug_quantize(const float* values, uint64_t n, int32_t e, int64_t* out) {
  if (!values || !out || n == 0) return fail(BMC_E_INVALID, "bad arguments");
  float* d_v = nullptr;
  long long* d_out = nullptr;
  BMC_CUDA(cudaMalloc(&d_v, n * 4));
  cudaError_t err = cudaMalloc(&d_out, n * 16);
  if (err == cudaSuccess) err = counted_memcpy(d_v, values, n * 4, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    bmc::launch_debug_quantize(0, d_v, n, e, d_out);
    g_launches++;
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = counted_memcpy(out, d_out, n * 16, cudaMemcpyDeviceToHost);
  cudaFree(d_v);
  if (d_out) cudaFree(d_out);
  if (err != cudaSuccess) return fail(BMC_E_CUDA, std::string("debug quantize: ") + cudaGetErrorString(err));
  return BMC_OK;
}

int bmc_debug_wait(uint64_t limit_ns, int32_t arrive, uint32_t* error_word, uint64_t* waited_ns) {
  if (!error_word || !waited_ns) return fail(BMC_E_INVALID, "null argument");
  if (limit_ns > 2000000000ull) return fail(BMC_E_INVALID, "limit above the kernels' own 2 s");
  unsigned long long* d = nullptr;
  BMC_CUDA(cudaMalloc(&d, 16));
  bmc::launch_debug_wait(0, limit_ns, arrive, d);
  g_launches++;
  unsigned long long h[2] = {0ull, 0ull};
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = counted_memcpy(h, d, 16, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(BMC_E_CUDA, std::string("debug wait: ") + cudaGetErrorString(e));
  *error_word = (uint32_t)h[0];
  *waited_ns = h[1];
  return BMC_OK;
}

}  // extern "C"

// ---- runtime-loaded cell models ------------------------------------------------
// Reference: UnsafeUDF::Loader::init_lib (apps/libs/models/ext/udf_includes.cpp
// L58-L78) binds a module's init/update/division/mass/names/... symbols;
// Unsafe::load_udf (apps/api/src/udf_handle.cpp L22-L38) takes the path from
// BIOMC_LIB_UDF.  Here a plugin exports its kernel sets (one per precision)
// and host entry points; a set is copied into the registry under the id the
// plugin receives.  Plugins stay loaded until exit: scenarios and graphs
// hold their launch functions.

namespace {

struct UdfEntry {
  int32_t id = 0;
  std::string path;
  void* handle = nullptr;
  bmc::KernelSet sets[2]{};  // [f64]
  bool has[2] = {false, false};
  bmc_udf_info info{};
  int (*host_model)(int32_t, bmc_udf_host_model*) = nullptr;
};

std::mutex g_udf_mu;
std::vector<UdfEntry*> g_udfs;  // never freed (see above)

UdfEntry* find_udf(int32_t id) {
  for (UdfEntry* e : g_udfs)
    if (e->id == id) return e;
  return nullptr;
}

}  // namespace

namespace bmc {
const KernelSet* udf_kernel_set(int model, int f64) {
  std::lock_guard<std::mutex> lk(g_udf_mu);
  UdfEntry* e = find_udf(model);
  if (!e || !e->has[f64 ? 1 : 0]) return nullptr;
  return &e->sets[f64 ? 1 : 0];
}
}  // namespace bmc

extern "C" {

int bmc_udf_load(const char* path, int32_t* model_id) {
  if (!model_id) return fail(BMC_E_INVALID, "model_id is null");
  std::string p;
  if (path) {
    p = path;
  } else {
    const char* env = std::getenv("BIOMC_LIB_UDF");
    if (!env) return fail(BMC_E_INVALID, "var BIOMC_LIB_UDF not found");
    p = env;
  }
  std::lock_guard<std::mutex> lk(g_udf_mu);
  for (UdfEntry* e : g_udfs)
    if (e->path == p) {
      *model_id = e->id;
      return BMC_OK;
    }
  void* h = dlopen(p.c_str(), RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    const char* why = dlerror();
    return fail(BMC_E_INVALID, std::string("cannot load model library: ") + (why ? why : p));
  }
  using AbiFn = int (*)();
  using SetFn = const void* (*)(int32_t);
  using SizeFn = size_t (*)();
  using IntFn = int32_t (*)();
  using NamesFn = const char* const* (*)(uint32_t*);
  using HostFn = int (*)(int32_t, bmc_udf_host_model*);
  auto abi = reinterpret_cast<AbiFn>(dlsym(h, "bmc_udf_abi"));
  auto kset = reinterpret_cast<SetFn>(dlsym(h, "bmc_udf_kernel_set"));
  auto nvar = reinterpret_cast<SizeFn>(dlsym(h, "set_nvar_udf"));
  auto nc = reinterpret_cast<SizeFn>(dlsym(h, "set_nc_udf"));
  auto sep = reinterpret_cast<IntFn>(dlsym(h, "separable_udf"));
  auto names = reinterpret_cast<NamesFn>(dlsym(h, "names_udf"));
  auto species = reinterpret_cast<NamesFn>(dlsym(h, "species_udf"));
  auto host = reinterpret_cast<HostFn>(dlsym(h, "host_model_udf"));
  if (!abi || !kset || !nvar || !nc || !sep || !names || !host) {
    dlclose(h);
    return fail(BMC_E_INVALID, "not a model library (missing bmc_udf_* / *_udf symbols): " + p);
  }
  if (abi() != bmc::kKernelSetAbi) {
    dlclose(h);
    return fail(BMC_E_UNSUPPORTED, "model library built against another KernelSet layout: " + p);
  }
  auto* e = new UdfEntry();
  e->id = BMC_MODEL_UDF_FIRST + (int32_t)g_udfs.size();
  e->path = p;
  e->handle = h;
  e->host_model = host;
  for (int f = 0; f < 2; ++f) {
    const auto* ks = static_cast<const bmc::KernelSet*>(kset(f));
    if (!ks) continue;
    if (ks->abi != bmc::kKernelSetAbi || ks->f64 != (f == 1) || ks->n_var != (int)nvar() ||
        ks->n_ctb != (int)nc()) {
      delete e;
      dlclose(h);
      return fail(BMC_E_UNSUPPORTED, "inconsistent kernel set in model library: " + p);
    }
    e->sets[f] = *ks;
    e->sets[f].model = e->id;
    e->has[f] = true;
  }
  if (!e->has[0] && !e->has[1]) {
    delete e;
    dlclose(h);
    return fail(BMC_E_UNSUPPORTED, "model library has no kernel set: " + p);
  }
  bmc_udf_info& in = e->info;
  in.n_var = (uint32_t)nvar();
  in.n_ctb = (uint32_t)nc();
  in.separable = sep();
  in.has_f32 = e->has[0] ? 1 : 0;
  in.has_f64 = e->has[1] ? 1 : 0;
  uint32_t n = 0;
  const char* const* v = names(&n);
  in.n_names = std::min<uint32_t>(n, 16);
  for (uint32_t k = 0; k < in.n_names; ++k) in.names[k] = v[k];
  v = species(&n);
  in.n_species = std::min<uint32_t>(n, 8);
  for (uint32_t k = 0; k < in.n_species; ++k) in.species[k] = v[k];
  g_udfs.push_back(e);
  *model_id = e->id;
  return BMC_OK;
}

int bmc_udf_get_info(int32_t model_id, bmc_udf_info* info) {
  if (!info) return fail(BMC_E_INVALID, "info is null");
  std::lock_guard<std::mutex> lk(g_udf_mu);
  UdfEntry* e = find_udf(model_id);
  if (!e) return fail(BMC_E_INVALID, "no model library loaded under this id");
  *info = e->info;
  return BMC_OK;
}

int bmc_udf_get_host_model(int32_t model_id, int32_t f64, bmc_udf_host_model* out) {
  if (!out) return fail(BMC_E_INVALID, "out is null");
  std::lock_guard<std::mutex> lk(g_udf_mu);
  UdfEntry* e = find_udf(model_id);
  if (!e) return fail(BMC_E_INVALID, "no model library loaded under this id");
  if (e->host_model(f64 ? 1 : 0, out) != 0) return fail(BMC_E_UNSUPPORTED, "precision not compiled in the model library");
  return BMC_OK;
}

}  // extern "C"

// ---- feed schedules ------------------------------------------------------------------
namespace {
std::mutex g_nlog_mu;
std::array<float*, 64> g_nlog{};  // -logf of every draw value, by device ordinal
}  // namespace

// The table the device's exit thresholds search (exit_threshold_dev):
// nlog[k] = -logf((2k + 1) 2^-24), from this process's C library, the same
// logf the host-side thresholds and the CPU restatement use.  32 MiB per
// device, made once, held until the process exits.
static int ensure_nlog(bmc_scenario* s) {
  const int dev = s->device;
  if (dev < 0 || dev >= (int)g_nlog.size()) return fail(BMC_E_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_nlog_mu);
  if (!g_nlog[dev]) {
    DeviceScope scope(dev);
    if (scope.err != cudaSuccess) return fail(BMC_E_CUDA, std::string("feed schedules: ") + cudaGetErrorString(scope.err));
    const size_t n = (size_t)1 << 23;
    std::vector<float> h(n);
    for (size_t k = 0; k < n; ++k) h[k] = -logf((float)(2u * (uint32_t)k + 1u) * 0x1p-24f);
    float* d = nullptr;
    BMC_CUDA(cudaMalloc(&d, n * sizeof(float)));
    const cudaError_t e = cudaMemcpy(d, h.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d);
      return fail(BMC_E_CUDA, std::string("feed schedules: ") + cudaGetErrorString(e));
    }
    g_h2d += n * sizeof(float);
    g_nlog[dev] = d;
  }
  s->h.nlog = g_nlog[dev];
  return BMC_OK;
}

int bmc_set_feed_schedules(bmc_scenario* s, uint32_t n_feeds, const bmc_feed_schedule* schedules) {
  if (!s || (n_feeds && !schedules)) return fail(BMC_E_INVALID, "null argument");
  if (n_feeds != (uint32_t)s->feeds.size())
    return fail(BMC_E_INVALID, "one schedule per feed of bmc_set_feeds, in the same order");
  uint32_t n_sched = 0;
  bool outlet_sched = false;
  for (uint32_t f = 0; f < n_feeds; ++f) {
    const bmc_feed_schedule& q = schedules[f];
    if (q.kind < BMC_FEED_CONSTANT || q.kind > BMC_FEED_EXPONENTIAL) return fail(BMC_E_INVALID, "unknown feed kind");
    if (!std::isfinite(q.f0) || !std::isfinite(q.rate)) return fail(BMC_E_INVALID, "schedule values must be finite");
    if (q.kind != BMC_FEED_CONSTANT) {
      ++n_sched;
      if (s->feeds[f].outlet >= 0) outlet_sched = true;
    }
  }
  if (outlet_sched) {
    const int rc = ensure_nlog(s);
    if (rc) return rc;
  }
  for (uint32_t f = 0; f < n_feeds; ++f) {
    s->h.feed_kind[f] = schedules[f].kind;
    s->h.feed_f0[f] = schedules[f].f0;
    s->h.feed_rate[f] = schedules[f].rate;
  }
  s->h.n_sched = n_sched;
  return upload_desc(s);
}

int bmc_feed_time(bmc_scenario* s, double* t) {
  if (const int rc_settle = settle_export(s)) return rc_settle;
  if (!s || !t) return fail(BMC_E_INVALID, "null argument");
  const int rc = read_ctl(s, nullptr);
  if (rc && rc != BMC_E_DEVICE) return rc;
  *t = s->h_ctl->t_rel;
  return BMC_OK;
}

// ---- pipelined main loop --------------------------------------------------------------
int bmc_step_enqueue(bmc_scenario* s, double dt, bmc_step_stats* stats, double* conc) {
  if (!s || !stats || !conc) return fail(BMC_E_INVALID, "null argument");
  if (s->pend_count >= 2) return fail(BMC_E_STATE, "two steps in flight: collect one first");
  if (!s->has_domain) return fail(BMC_E_STATE, "domain not set");
  DeviceScope on(s->device);
  const size_t ne = (size_t)s->h.n_c * s->h.n_s;
  if (s->export_ne < ne) {
    if (s->pend_count > 0) return fail(BMC_E_STATE, "the domain grew while steps are in flight");
    if (s->h_export) cudaFreeHost(s->h_export);
    s->h_export = s->d_export = nullptr;
    s->export_ne = 0;
    s->export_conc = align_up(sizeof(Control), 256);
    s->export_slot = align_up(s->export_conc + ne * sizeof(double), 256);
    void* hp = nullptr;
    BMC_CUDA(cudaHostAlloc(&hp, 2 * s->export_slot, cudaHostAllocMapped));
    s->h_export = static_cast<unsigned char*>(hp);
    void* dp = nullptr;
    BMC_CUDA(cudaHostGetDevicePointer(&dp, hp, 0));
    s->d_export = static_cast<unsigned char*>(dp);
    s->export_ne = ne;
  }
  const unsigned k = (s->pend_head + s->pend_count) % 2u;
  bmc_scenario::Pending& q = s->pend[k];
  if (!q.done) BMC_CUDA(cudaEventCreateWithFlags(&q.done, cudaEventDisableTiming));
  int rc = settle_export(s);  // the previous step's export, if still deferred
  if (rc) return rc;
  s->enqueuing = true;
  rc = scenario_steps(s, dt, 1, 1, true);
  s->enqueuing = false;
  if (rc) return rc;
  // the step's counters and concentrations go straight into slot k by a
  // small kernel (no copies), launched with the next descriptor upload when
  // one comes before anything else (bmc_set_feeds in a loop), else alone
  s->export_deferred = (int)k;
  g_d2h += sizeof(Control) + ne * sizeof(double);
  q.stats = stats;
  q.out = conc;
  q.ne = ne;
  s->pend_count++;
  return BMC_OK;
}

int bmc_step_collect(bmc_scenario* s) {
  if (!s) return fail(BMC_E_INVALID, "null scenario");
  if (s->pend_count == 0) return fail(BMC_E_STATE, "no step enqueued");
  const unsigned k = s->pend_head;
  bmc_scenario::Pending& q = s->pend[k];
  if (s->export_deferred == (int)k) {
    const int rc = settle_export(s);
    if (rc) return rc;
  }
  BMC_CUDA(cudaEventSynchronize(q.done));
  s->pend_head = (s->pend_head + 1) % 2u;
  s->pend_count--;
  const unsigned char* slot = s->h_export + k * s->export_slot;
  Control c;
  std::memcpy(&c, slot, sizeof(Control));
  std::memcpy(q.out, slot + s->export_conc, q.ne * sizeof(double));
  stats_from_ctl(c, q.stats);
  if (s->pend_count == 0) {
    *s->h_ctl = c;
    s->ctl_fresh = true;
  }
  if (c.error) return fail(BMC_E_DEVICE, "device error word set: " + std::to_string(c.error));
  return BMC_OK;
}


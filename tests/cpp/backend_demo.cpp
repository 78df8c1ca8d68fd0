// backend_demo.cpp -- the binding a maintainer adds to the reference's
// simulation core to hand its particle cycle to libbmc (class BmcBackend),
// compiled as a C++ program against include/bmc.h and linked to libbmc.so.
//
//   backend_demo <input.bin> <output.bin> [pipelined]
//
// The input holds one scenario (sizes, model descriptor, domain, liquid
// transition, concentrations, feeds, run length); the program sets it up
// through the C-ABI, runs the main loop with step_and_export (bmc_step_read
// every iteration, growth on overflow) or, with `pipelined`, with
// bmc_step_enqueue / bmc_step_collect and two steps in flight (feeds set
// again before every enqueue), then writes the per-step counters, the
// concentrations of every step and the final particles.  The test compares
// these with the Python binding's run bit for bit.
extern "C" {
#include "bmc.h"
}
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

class BmcBackend {
 public:
  explicit BmcBackend(const bmc_scenario_desc& d) { check(bmc_scenario_create(&d, &s_)); }
  ~BmcBackend() { bmc_scenario_destroy(s_); }
  BmcBackend(const BmcBackend&) = delete;
  BmcBackend& operator=(const BmcBackend&) = delete;

  // UPDATE_HYDRO_STEP: ReactorDomain::update + ScalarSimulation::set_transition
  void update_hydro(const std::vector<double>& vol, uint32_t K, const std::vector<uint64_t>& nb,
                    const std::vector<double>& out_flows, const std::vector<double>& cdf,
                    const std::vector<uint64_t>& rows, const std::vector<uint64_t>& cols,
                    const std::vector<double>& vals) {
    const uint32_t n_c = (uint32_t)vol.size();
    check(bmc_domain_update(s_, n_c, K, vol.data(), nb.data(), out_flows.data(), cdf.data()));
    check(bmc_set_transition_coo(s_, n_c, vals.size(), rows.data(), cols.data(), vals.data()));
  }
  void set_concentrations(const std::vector<double>& c) { check(bmc_set_concentrations(s_, c.data())); }
  void set_feeds(const std::vector<bmc_feed>& f) { check(bmc_set_feeds(s_, (uint32_t)f.size(), f.data())); }
  double init(uint64_t n, double x0) {
    double w = 0.0;
    check(bmc_init_particles(s_, n, 1, x0, &w));
    return w;
  }
  // one main-loop iteration with the field read back in the same
  // synchronisation; grow the container when births were refused
  bmc_step_stats step_and_export(double dt, std::vector<double>& c, double alloc_factor) {
    bmc_step_stats st{};
    check(bmc_step_read(s_, dt, &st, c.data()));
    if (st.overflow > 0) check(bmc_reserve(s_, (uint64_t)((double)(st.n_used + st.overflow) * alloc_factor)));
    return st;
  }
  // the main loop with the host's work on step k overlapped with step k+1
  // on the device: counters and fields of every step into st / c
  void run_pipelined(double dt, uint32_t n_steps, const std::vector<bmc_feed>& feeds,
                     std::vector<bmc_step_stats>& st, std::vector<std::vector<double>>& c) {
    for (uint32_t k = 0; k < n_steps; ++k) {
      check(bmc_set_feeds(s_, (uint32_t)feeds.size(), feeds.data()));
      check(bmc_step_enqueue(s_, dt, &st[k], c[k].data()));
      if (k > 0) check(bmc_step_collect(s_));
    }
    if (n_steps > 0) check(bmc_step_collect(s_));
  }
  bmc_scenario* handle() { return s_; }

 private:
  static void check(int rc) {
    if (rc != BMC_OK) throw std::runtime_error(bmc_last_error());
  }
  bmc_scenario* s_ = nullptr;
};

namespace {
struct Reader {
  FILE* f;
  template <class T>
  T get() {
    T v{};
    if (std::fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("short input");
    return v;
  }
  template <class T>
  std::vector<T> vec(size_t n) {
    std::vector<T> v(n);
    if (n && std::fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short input");
    return v;
  }
};
template <class T>
void put(FILE* f, const T* p, size_t n) {
  if (n && std::fwrite(p, sizeof(T), n, f) != n) throw std::runtime_error("short write");
}
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3 && !(argc == 4 && std::strcmp(argv[3], "pipelined") == 0)) {
    std::fprintf(stderr, "usage: %s input.bin output.bin [pipelined]\n", argv[0]);
    return 2;
  }
  const bool pipelined = argc == 4;
  try {
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) throw std::runtime_error("cannot open input");
    Reader r{in};
    bmc_scenario_desc d{};
    d = r.get<bmc_scenario_desc>();
    const uint32_t n_c = r.get<uint32_t>(), K = r.get<uint32_t>(), n_s = r.get<uint32_t>();
    const uint64_t n_particles = r.get<uint64_t>();
    const double x0 = r.get<double>(), dt = r.get<double>(), alloc = r.get<double>();
    const uint32_t n_steps = r.get<uint32_t>(), n_feeds = r.get<uint32_t>();
    const uint64_t nnz = r.get<uint64_t>();
    auto vol = r.vec<double>(n_c);
    auto nb = r.vec<uint64_t>((size_t)n_c * K);
    auto outf = r.vec<double>(n_c);
    auto cdf = r.vec<double>((size_t)n_c * K);
    auto rows = r.vec<uint64_t>(nnz);
    auto cols = r.vec<uint64_t>(nnz);
    auto vals = r.vec<double>(nnz);
    auto c0 = r.vec<double>((size_t)n_c * n_s);
    auto feeds = r.vec<bmc_feed>(n_feeds);
    std::fclose(in);

    BmcBackend backend(d);
    backend.update_hydro(vol, K, nb, outf, cdf, rows, cols, vals);
    backend.set_concentrations(c0);
    backend.set_feeds(feeds);
    const double w = backend.init(n_particles, x0);

    FILE* out = std::fopen(argv[2], "wb");
    if (!out) throw std::runtime_error("cannot open output");
    put(out, &w, 1);
    std::vector<double> c((size_t)n_c * n_s);
    if (pipelined) {
      std::vector<bmc_step_stats> sts(n_steps);
      std::vector<std::vector<double>> cs(n_steps, std::vector<double>((size_t)n_c * n_s));
      backend.run_pipelined(dt, n_steps, feeds, sts, cs);
      for (uint32_t k = 0; k < n_steps; ++k) {
        const bmc_step_stats& st = sts[k];
        const uint64_t row[6] = {st.n_used, st.births, st.exits, st.moves, st.overflow, st.error};
        put(out, row, 6);
        put(out, cs[k].data(), cs[k].size());
      }
    } else {
      for (uint32_t k = 0; k < n_steps; ++k) {
        const bmc_step_stats st = backend.step_and_export(dt, c, alloc);
        const uint64_t row[6] = {st.n_used, st.births, st.exits, st.moves, st.overflow, st.error};
        put(out, row, 6);
        put(out, c.data(), c.size());
      }
    }
    // the final particles: SoA state, compartments, statuses, ids
    bmc_step_stats st{};
    if (bmc_read_stats(backend.handle(), &st) != BMC_OK) throw std::runtime_error(bmc_last_error());
    const uint64_t n = st.n_used;
    const size_t fsz = d.model.f64 ? 8 : 4;
    std::vector<char> state((size_t)d.model.n_var * n * fsz);
    std::vector<uint32_t> pos(n), id(n);
    std::vector<uint8_t> status(n);
    uint64_t got = 0;
    if (bmc_read_particles(backend.handle(), n, state.data(), pos.data(), status.data(), nullptr, nullptr, id.data(),
                           &got) != BMC_OK)
      throw std::runtime_error(bmc_last_error());
    put(out, &n, 1);
    put(out, state.data(), state.size());
    put(out, pos.data(), n);
    put(out, status.data(), n);
    put(out, id.data(), n);
    // the run's event tallies (the exporter's records/tallies) and every
    // particle's Model::mass (the particle dump's mass column)
    uint64_t events[BMC_N_EVENTS] = {};
    if (bmc_read_events(backend.handle(), events, 0) != BMC_OK) throw std::runtime_error(bmc_last_error());
    put(out, events, BMC_N_EVENTS);
    std::vector<double> mass(n);
    if (bmc_read_mass(backend.handle(), n, mass.data(), &got) != BMC_OK) throw std::runtime_error(bmc_last_error());
    put(out, mass.data(), n);
    std::fclose(out);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "backend_demo: %s\n", e.what());
    return 1;
  }
  return 0;
}

// bmc_cma.cpp -- CMA ingestion on the host (declared in include/bmc.h):
// the per-compartment quantities the cycle reads, derived from a flow map,
// the automatic time step of a flow-map set, and the field files of a CMA
// case.  Pure host code: nothing here touches the device.
//
// Derivations (documentation/pages/03_cma.md, "Transition Matrix" and
// "Cumulative probability"; CmaUtils::get_transition_matrix,
// get_diag_transition, get_cumulative_probabilities):
//   T(i, j) = F(i, j) for i != j,  T(i, i) = -sum_{j != i} F(i, j);
//   P(I_j | L) = F(i, j) / sum_k F(i, k), accumulated over the destinations
//   of i in ascending order.
// Self-flows F(i, i) carry no particle and no scalar (the reference's
// transition test, apps/libs/cma_utils/tests/test_transition_matrix.cpp
// L7-L25: flows {{1,2},{3,4}} give {{-2,2},{3,-3}}).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#include "../../include/bmc.h"

namespace bmc {
int api_fail(int code, const std::string& msg);
}

namespace {

struct Link {
  uint32_t dst;
  double flow;
};

// Out-links of every compartment: entries with i == j or F == 0 dropped,
// duplicates of one (i, j) summed in input order, destinations ascending.
const char* gather_links(uint32_t n_c, uint64_t nnz, const uint64_t* rows, const uint64_t* cols,
                         const double* flows, std::vector<uint64_t>& ptr, std::vector<Link>& links) {
  std::vector<std::pair<std::pair<uint32_t, uint32_t>, double>> e;
  e.reserve(nnz);
  for (uint64_t k = 0; k < nnz; ++k) {
    if (rows[k] >= n_c || cols[k] >= n_c) return "flow index out of range";
    const double f = flows[k];
    if (!std::isfinite(f) || f < 0.0) return "flows must be finite and >= 0";
    if (rows[k] == cols[k] || f == 0.0) continue;
    e.push_back({{(uint32_t)rows[k], (uint32_t)cols[k]}, f});
  }
  std::stable_sort(e.begin(), e.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  ptr.assign((size_t)n_c + 1, 0u);
  links.clear();
  for (size_t k = 0; k < e.size(); ++k) {
    if (k > 0 && e[k].first == e[k - 1].first) {
      links.back().flow += e[k].second;
      continue;
    }
    links.push_back({e[k].first.second, e[k].second});
    ptr[e[k].first.first + 1]++;
  }
  for (uint32_t i = 0; i < n_c; ++i) ptr[i + 1] += ptr[i];
  return nullptr;
}

uint32_t read_u32_le(const unsigned char* b) {
  return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}

uint64_t read_u64_le(const unsigned char* b) {
  uint64_t u = 0;
  for (int k = 7; k >= 0; --k) u = (u << 8) | (uint64_t)b[k];
  return u;
}

double read_f64_le(const unsigned char* b) {
  const uint64_t u = read_u64_le(b);
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}

// Whole file into buf; false when it cannot be opened.
bool slurp(const char* path, std::vector<unsigned char>& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  buf.clear();
  unsigned char chunk[65536];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  std::fclose(f);
  return true;
}

// Entry of a case descriptor: kind byte and the path's bytes in the file.
struct CaseEntry {
  uint32_t kind;
  uint32_t len;
  size_t off;
};

// Case descriptor: 4 uint32 words, one float64, a uint64 entry count, then
// per entry a uint8 kind, a uint32 length and the path's bytes; the whole
// file and nothing more.  Returns an error message or nullptr.
const char* parse_case(const std::vector<unsigned char>& b, std::vector<CaseEntry>& out) {
  const size_t n = b.size();
  if (n < 32) return "case descriptor shorter than its 32-byte header";
  const uint64_t count = read_u64_le(b.data() + 24);
  if (count > (n - 32) / 5) return "case descriptor entry count exceeds what the file can hold";
  out.clear();
  size_t o = 32;
  for (uint64_t k = 0; k < count; ++k) {
    if (o + 5 > n) return "case descriptor ends inside an entry header";
    CaseEntry e;
    e.kind = b[o];
    e.len = read_u32_le(b.data() + o + 1);
    o += 5;
    if (e.len == 0 || e.len > n - o) return "case descriptor entry path runs past the end of the file";
    e.off = o;
    o += e.len;
    out.push_back(e);
  }
  if (o != n) return "case descriptor has bytes after its last entry";
  return nullptr;
}

}  // namespace

extern "C" {

int bmc_cma_derive(uint32_t n_c, uint64_t nnz, const uint64_t* rows, const uint64_t* cols, const double* flows,
                   uint32_t* K, uint32_t k_cap, uint64_t* neighbors, double* out_flows, double* cdf) {
  if (n_c == 0 || !K || (nnz && (!rows || !cols || !flows))) return bmc::api_fail(BMC_E_INVALID, "bad flow map");
  std::vector<uint64_t> ptr;
  std::vector<Link> links;
  if (const char* why = gather_links(n_c, nnz, rows, cols, flows, ptr, links)) return bmc::api_fail(BMC_E_INVALID, why);
  uint64_t kmax = 1;
  for (uint32_t i = 0; i < n_c; ++i) kmax = std::max<uint64_t>(kmax, ptr[i + 1] - ptr[i]);
  *K = (uint32_t)kmax;
  if (!neighbors && !out_flows && !cdf) return BMC_OK;
  if (!neighbors || !out_flows || !cdf) return bmc::api_fail(BMC_E_INVALID, "give all three output arrays or none");
  if (k_cap < kmax) return bmc::api_fail(BMC_E_INVALID, "k_cap is below the largest out-degree (K)");
  std::vector<double> cum;
  for (uint32_t i = 0; i < n_c; ++i) {
    const uint64_t b = ptr[i], deg = ptr[i + 1] - b;
    uint64_t* nb = neighbors + (size_t)i * kmax;
    double* cd = cdf + (size_t)i * kmax;
    // running sum in destination order: its last value is the out-flow,
    // so the last cumulative probability is exactly 1
    cum.resize(deg);
    double s = 0.0;
    for (uint64_t k = 0; k < deg; ++k) {
      s += links[b + k].flow;
      cum[k] = s;
    }
    out_flows[i] = s;
    for (uint64_t k = 0; k < deg; ++k) {
      nb[k] = links[b + k].dst;
      cd[k] = cum[k] / s;
    }
    const uint64_t pad = deg ? links[b + deg - 1].dst : i;
    for (uint64_t k = deg; k < kmax; ++k) {
      nb[k] = pad;
      cd[k] = 1.0;
    }
  }
  return BMC_OK;
}

int bmc_cma_transition(uint32_t n_c, uint64_t nnz, const uint64_t* rows, const uint64_t* cols, const double* flows,
                       uint64_t* t_nnz, uint64_t cap, uint64_t* t_rows, uint64_t* t_cols, double* t_values) {
  if (n_c == 0 || !t_nnz || (nnz && (!rows || !cols || !flows))) return bmc::api_fail(BMC_E_INVALID, "bad flow map");
  std::vector<uint64_t> ptr;
  std::vector<Link> links;
  if (const char* why = gather_links(n_c, nnz, rows, cols, flows, ptr, links)) return bmc::api_fail(BMC_E_INVALID, why);
  const uint64_t total = links.size() + n_c;
  *t_nnz = total;
  if (!t_rows && !t_cols && !t_values) return BMC_OK;
  if (!t_rows || !t_cols || !t_values) return bmc::api_fail(BMC_E_INVALID, "give all three output arrays or none");
  if (cap < total) return bmc::api_fail(BMC_E_INVALID, "cap is below the entry count");
  uint64_t o = 0;
  for (uint32_t i = 0; i < n_c; ++i) {
    double s = 0.0;
    for (uint64_t k = ptr[i]; k < ptr[i + 1]; ++k) s += links[k].flow;
    bool diag_done = false;
    for (uint64_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      if (!diag_done && links[k].dst > i) {
        t_rows[o] = i, t_cols[o] = i, t_values[o] = -s, ++o;
        diag_done = true;
      }
      t_rows[o] = i, t_cols[o] = links[k].dst, t_values[o] = links[k].flow, ++o;
    }
    if (!diag_done) t_rows[o] = i, t_cols[o] = i, t_values[o] = -s, ++o;
  }
  return BMC_OK;
}

int bmc_cma_time_step(double user_dt, uint32_t n_maps, uint32_t n_c, const double* volumes, const double* out_flows,
                      double* dt) {
  if (!dt) return bmc::api_fail(BMC_E_INVALID, "null dt");
  if (user_dt > 0.0) {
    *dt = user_dt;
    return BMC_OK;
  }
  if (n_maps == 0 || n_c == 0 || !volumes || !out_flows) return bmc::api_fail(BMC_E_INVALID, "no flow map");
  double m = std::numeric_limits<double>::max();
  for (size_t k = 0; k < (size_t)n_maps * n_c; ++k)
    if (volumes[k] > 0.0) m = std::min(m, out_flows[k] / volumes[k]);
  if (m == std::numeric_limits<double>::max() || m == 0.0)
    return bmc::api_fail(BMC_E_INVALID, "no time step given and impossible to estimate it with the given flow maps");
  *dt = m / 100.;
  return BMC_OK;
}

// Kinematic viscosity of water (m^2/s) at temp degrees Celsius in (0, 370):
// the sixth-degree fit (in mm^2/s) the reference takes from the Engineering
// ToolBox water-viscosity table (c_kinematic_viscosity, apps/libs/simulation/
// src/hydro/impl_mtr.cpp L56-L84), evaluated by Horner's rule and rounded to
// 1e-10 m^2/s as the reference rounds it.
static double water_kinematic_viscosity(double temp) {
  static const double lo[7] = {1.79194000343777, -0.0607310297913931, 0.00144686943485654, -0.0000234079044336466,
                               0.00000023336659710795, -0.00000000126441088087, 0.00000000000282244333};
  static const double hi[7] = {1.08486933174497,         -0.0166081298727911,       0.000136367622445752,
                               -0.00000064995487357883,  0.00000000181964246491, -0.00000000000277495333,
                               0.00000000000000178038};
  const double* c = temp < 85.0 ? lo : hi;
  double p = c[6];
  for (int k = 5; k >= 0; --k) p = p * temp + c[k];
  return std::round(p * 0.000001 * 10000000000.0) / 10000000000.0;
}

int bmc_mtr_turbulence_kla(uint32_t n_c, const double* energy_dissipation, const double* liquid_volume,
                           const double* gas_volume, double bubble_diameter, double* kla) {
  if (!energy_dissipation || !liquid_volume || !gas_volume || !kla) return bmc::api_fail(BMC_E_INVALID, "null argument");
  if (!(bubble_diameter > 0.0)) return bmc::api_fail(BMC_E_INVALID, "bubble diameter must be positive");
  const double nu = water_kinematic_viscosity(20.0);  // the reference's temperature
  const double schmidt = nu / 1e-9;                   // and oxygen diffusivity, m^2/s
  for (uint32_t j = 0; j < n_c; ++j) {
    const double vl = liquid_volume[j], vg = gas_volume[j], eps = energy_dissipation[j];
    if (!(vl > 0.0) || !(vg >= 0.0) || !(eps >= 0.0))
      return bmc::api_fail(BMC_E_INVALID, "volumes must be positive (gas: non-negative), dissipation non-negative");
    const double alpha = vg / (vl + vg);
    const double kl = 0.3 * std::pow(eps * nu, 0.25) * std::pow(schmidt, -0.5);
    const double area = 6. * alpha / (bubble_diameter * (1 - alpha));
    kla[j] = kl * area;
  }
  return BMC_OK;
}

int bmc_cma_read_field(const char* path, uint64_t cap, double* values, uint64_t* n) {
  if (!path || !n) return bmc::api_fail(BMC_E_INVALID, "null argument");
  std::vector<unsigned char> buf;
  if (!slurp(path, buf)) return bmc::api_fail(BMC_E_INVALID, std::string("cannot open ") + path);
  if (buf.size() < 4) return bmc::api_fail(BMC_E_INVALID, "field file shorter than its count");
  const uint64_t count = read_u32_le(buf.data());
  if (buf.size() != 4 + 8 * count)
    return bmc::api_fail(BMC_E_INVALID, "field file size differs from 4 + 8 * count");
  *n = count;
  if (!values) return BMC_OK;
  if (cap < count) return bmc::api_fail(BMC_E_INVALID, "cap is below the value count");
  for (uint64_t k = 0; k < count; ++k) values[k] = read_f64_le(buf.data() + 4 + 8 * k);
  return BMC_OK;
}

int bmc_cma_read_case(const char* path, uint32_t* words, double* t0, uint32_t* n_entries) {
  if (!path || !n_entries) return bmc::api_fail(BMC_E_INVALID, "null argument");
  std::vector<unsigned char> buf;
  if (!slurp(path, buf)) return bmc::api_fail(BMC_E_INVALID, std::string("cannot open ") + path);
  std::vector<CaseEntry> ent;
  const char* err = parse_case(buf, ent);
  if (err) return bmc::api_fail(BMC_E_INVALID, err);
  if (words)
    for (int k = 0; k < 4; ++k) words[k] = read_u32_le(buf.data() + 4 * k);
  if (t0) *t0 = read_f64_le(buf.data() + 16);
  *n_entries = (uint32_t)ent.size();
  return BMC_OK;
}

int bmc_cma_case_entry(const char* path, uint32_t index, uint32_t* kind, char* name, uint64_t name_cap) {
  if (!path || !kind) return bmc::api_fail(BMC_E_INVALID, "null argument");
  std::vector<unsigned char> buf;
  if (!slurp(path, buf)) return bmc::api_fail(BMC_E_INVALID, std::string("cannot open ") + path);
  std::vector<CaseEntry> ent;
  const char* err = parse_case(buf, ent);
  if (err) return bmc::api_fail(BMC_E_INVALID, err);
  if (index >= ent.size()) return bmc::api_fail(BMC_E_INVALID, "entry index out of range");
  const CaseEntry& e = ent[index];
  *kind = e.kind;
  if (!name) return BMC_OK;
  if (name_cap < (uint64_t)e.len + 1u) return bmc::api_fail(BMC_E_INVALID, "name_cap is below the path length + 1");
  std::memcpy(name, buf.data() + e.off, e.len);
  name[e.len] = '\0';
  return BMC_OK;
}

int bmc_cma_read_flowmap(const char* path, uint32_t* n_rows, uint32_t* n_cols, uint64_t* nnz, uint64_t cap,
                         uint64_t* rows, uint64_t* cols, double* flows) {
  if (!path || !n_rows || !n_cols || !nnz) return bmc::api_fail(BMC_E_INVALID, "null argument");
  std::vector<unsigned char> buf;
  if (!slurp(path, buf)) return bmc::api_fail(BMC_E_INVALID, std::string("cannot open ") + path);
  const size_t n = buf.size();
  if (n < 32) return bmc::api_fail(BMC_E_INVALID, "flow map shorter than its header and three array lengths");
  const uint32_t nr = read_u32_le(buf.data()), nc = read_u32_le(buf.data() + 4);
  // three arrays, each a uint64 length then its elements (8 bytes each)
  size_t o = 8;
  uint64_t len[3];
  size_t at[3];
  for (int a = 0; a < 3; ++a) {
    if (o + 8 > n) return bmc::api_fail(BMC_E_INVALID, "flow map ends inside an array length");
    len[a] = read_u64_le(buf.data() + o);
    o += 8;
    if (len[a] > (n - o) / 8) return bmc::api_fail(BMC_E_INVALID, "flow map array runs past the end of the file");
    at[a] = o;
    o += 8 * (size_t)len[a];
  }
  if (o != n) return bmc::api_fail(BMC_E_INVALID, "flow map size differs from its header and array lengths");
  if (len[0] != len[1] || len[1] != len[2])
    return bmc::api_fail(BMC_E_INVALID, "flow map arrays (rows, columns, flows) differ in length");
  for (uint64_t k = 0; k < len[0]; ++k) {
    const uint64_t r = read_u64_le(buf.data() + at[0] + 8 * k), c = read_u64_le(buf.data() + at[1] + 8 * k);
    if (r >= nr || c >= nc) return bmc::api_fail(BMC_E_INVALID, "flow map entry outside its rows and columns");
  }
  *n_rows = nr;
  *n_cols = nc;
  *nnz = len[0];
  if (!rows && !cols && !flows) return BMC_OK;
  if (!rows || !cols || !flows) return bmc::api_fail(BMC_E_INVALID, "give all three arrays or none");
  if (cap < len[0]) return bmc::api_fail(BMC_E_INVALID, "cap is below the entry count");
  for (uint64_t k = 0; k < len[0]; ++k) {
    rows[k] = read_u64_le(buf.data() + at[0] + 8 * k);
    cols[k] = read_u64_le(buf.data() + at[1] + 8 * k);
    flows[k] = read_f64_le(buf.data() + at[2] + 8 * k);
  }
  return BMC_OK;
}

}  // extern "C"

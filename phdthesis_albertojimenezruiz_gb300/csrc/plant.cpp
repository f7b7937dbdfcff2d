// Synthetic PV plant generator (see plant.hpp).
#include "plant.hpp"

#include <algorithm>
#include <cmath>
#include <map>

#include "symbolic.hpp"

namespace pvglu {

namespace {

// splitmix64: a small, portable, seedable generator (same stream on every
// host architecture).
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
};

struct Builder {
  int n;
  std::vector<std::map<int, double>> lin;                    // linear values
  std::vector<std::map<int, std::vector<std::pair<int, int>>>> pan;  // (panel, sign)
  explicit Builder(int n_) : n(n_), lin(n_), pan(n_) {}
  void add_lin(int r, int c, double v) {
    if (r < 0 || c < 0) return;
    lin[r][c] += v;
  }
  void touch(int r, int c) {
    if (r < 0 || c < 0) return;
    lin[r][c] += 0.0;
  }
  // Admittance g between n1 and n2 (002b:5-38), ground = -1.
  void admittance(int n1, int n2, double g) {
    add_lin(n1, n1, g);
    add_lin(n1, n2, -g);
    add_lin(n2, n1, -g);
    add_lin(n2, n2, g);
  }
  void panel_stamp(int id, int hi, int lo) {
    auto put = [&](int r, int c, int sgn) {
      if (r < 0 || c < 0) return;
      touch(r, c);
      pan[r][c].push_back({id, sgn});
    };
    put(hi, hi, +1);
    put(hi, lo, -1);
    put(lo, hi, -1);
    put(lo, lo, +1);
  }
};

}  // namespace

double panel_voc(const pvglu_panel_params& pp, double iph) {
  // Newton on I(V) = 0 from the diode-only estimate.
  double v = pp.a * std::log(iph / pp.i0 + 1.0);
  for (int it = 0; it < 100; it++) {
    double i, didv;
    pvglu_panel_iv(&pp, iph, v, &i, &didv);
    const double dv = -i / didv;
    v += dv;
    if (std::fabs(dv) < 1e-13 * std::fabs(v)) break;
  }
  return v;
}

int build_plant(const PlantConfig& cfg, Plant& P) {
  if (cfg.n_inverters <= 0 || cfg.n_strings <= 0 || cfg.n_series <= 0)
    return ERR_BAD_ARG;
  P = Plant();
  P.cfg = cfg;
  P.panel.i0 = cfg.i0;
  P.panel.a = cfg.ideality * cfg.cells * cfg.vt;
  P.panel.rs = cfg.rs;
  P.panel.rsh = cfg.rsh;
  P.voc_panel = panel_voc(P.panel, cfg.iph_stc);
  P.v_mppt = cfg.mppt_fraction * cfg.n_series * P.voc_panel;

  const int per_inv = cfg.n_strings * cfg.n_series + 3;
  const int64_t n64 = (int64_t)cfg.n_inverters * per_inv;
  if (n64 > 200000000) return ERR_TOO_LARGE;
  P.n = (int)n64;
  P.n_panels = cfg.n_inverters * cfg.n_strings * cfg.n_series;
  Builder B(P.n);
  P.b_lin.assign(P.n, 0.0);

  const int blocks_1d = (int)std::ceil(std::sqrt((double)cfg.n_inverters));
  P.extent_x = blocks_1d * cfg.n_series * cfg.pitch;
  P.extent_y = ((cfg.n_inverters + blocks_1d - 1) / blocks_1d) * cfg.n_strings * cfg.pitch;
  const double g_string = 1.0 / cfg.r_string, g_comb = 1.0 / cfg.r_combiner;

  int pid = 0;
  for (int v = 0; v < cfg.n_inverters; v++) {
    const int base = v * per_inv;
    const int comb = base + cfg.n_strings * cfg.n_series;
    const int term = comb + 1, icur = comb + 2;
    const int bx = v % blocks_1d, by = v / blocks_1d;
    for (int s = 0; s < cfg.n_strings; s++) {
      for (int p = 0; p < cfg.n_series; p++) {
        const int hi = base + s * cfg.n_series + p;
        const int lo = (p == 0) ? -1 : hi - 1;
        P.pan_hi.push_back(hi);
        P.pan_lo.push_back(lo);
        P.pan_x.push_back((bx * cfg.n_series + p + 0.5) * cfg.pitch);
        P.pan_y.push_back((by * cfg.n_strings + s + 0.5) * cfg.pitch);
        B.panel_stamp(pid, hi, lo);
        pid++;
      }
      B.admittance(base + s * cfg.n_series + cfg.n_series - 1, comb, g_string);
    }
    B.admittance(comb, term, g_comb);
    // Voltage source T_v -> ground with its own row (002b:110-125).
    B.add_lin(term, icur, -1.0);
    B.add_lin(icur, term, 1.0);
    P.b_lin[icur] += P.v_mppt;
    P.inv_combiner.push_back(comb);
    P.inv_terminal.push_back(term);
    P.inv_current.push_back(icur);
  }

  P.rowptr.assign(P.n + 1, 0);
  P.contrib_ptr.clear();
  P.contrib_ptr.push_back(0);
  for (int r = 0; r < P.n; r++) {
    for (const auto& kv : B.lin[r]) {
      P.colidx.push_back(kv.first);
      P.a_lin.push_back(kv.second);
      auto it = B.pan[r].find(kv.first);
      if (it != B.pan[r].end())
        for (const auto& ps : it->second) {
          P.contrib_panel.push_back(ps.first);
          P.contrib_sign.push_back((signed char)ps.second);
        }
      P.contrib_ptr.push_back((int)P.contrib_panel.size());
    }
    P.rowptr[r + 1] = (int)P.colidx.size();
  }
  // Node incidence of panel currents (f flows hi -> lo through the panel).
  std::vector<std::vector<std::pair<int, int>>> inc(P.n);
  for (int k = 0; k < P.n_panels; k++) {
    if (P.pan_hi[k] >= 0) inc[P.pan_hi[k]].push_back({k, +1});
    if (P.pan_lo[k] >= 0) inc[P.pan_lo[k]].push_back({k, -1});
  }
  P.inc_ptr.assign(P.n + 1, 0);
  for (int i = 0; i < P.n; i++) {
    for (const auto& ks : inc[i]) {
      P.inc_panel.push_back(ks.first);
      P.inc_sign.push_back((signed char)ks.second);
    }
    P.inc_ptr[i + 1] = (int)P.inc_panel.size();
  }
  return OK;
}

void plant_shadows(const Plant& P, const ShadowConfig& sc, uint64_t seed,
                   std::vector<double>& params) {
  SplitMix64 rng(seed * 0x2545F4914F6CDD1Dull + 0x1234567ull);
  const int ns = sc.min_shadows +
                 (int)(rng.next() % (uint64_t)(sc.max_shadows - sc.min_shadows + 1));
  params.assign(6 * (size_t)ns, 0.0);
  for (int k = 0; k < ns; k++) {
    double* c = &params[6 * (size_t)k];
    c[0] = rng.uniform(0.0, P.extent_x);
    c[1] = rng.uniform(0.0, P.extent_y);
    c[4] = rng.uniform(sc.min_depth, sc.max_depth);
    c[5] = rng.uniform(sc.min_sigma, sc.max_sigma);
    const double speed = rng.uniform(sc.min_speed, sc.max_speed);
    const double ang = rng.uniform(0.0, 6.283185307179586);
    c[2] = speed * std::cos(ang);
    c[3] = speed * std::sin(ang);
  }
}

void plant_irradiance(const Plant& P, const ShadowConfig& sc, uint64_t seed,
                      double t, double* g_out) {
  std::vector<double> sh;
  plant_shadows(P, sc, seed, sh);
  const int ns = (int)(sh.size() / 6);
  for (int i = 0; i < P.n_panels; i++)
    g_out[i] = pvglu_shadow_irradiance(P.pan_x[i], P.pan_y[i], sh.data(), ns, t, sc.g_clear);
}

}  // namespace pvglu

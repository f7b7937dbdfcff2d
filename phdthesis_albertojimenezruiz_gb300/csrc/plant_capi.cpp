// C ABI of the plant generator (include/pvglu_plant.h), host part.
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/pvglu_plant.h"
#include "plant.hpp"
#include "symbolic.hpp"

struct pvglu_plant {
  pvglu::Plant p;
  std::vector<int> contrib_sign_i, inc_sign_i;
};

extern "C" {

int pvglu_plant_create(int n_inverters, int n_strings, int n_series, pvglu_plant** out) {
  if (!out) return PVGLU_ERR_BAD_ARG;
  *out = nullptr;
  pvglu::PlantConfig cfg;
  cfg.n_inverters = n_inverters;
  cfg.n_strings = n_strings;
  cfg.n_series = n_series;
  auto* h = new pvglu_plant();
  const int rc = pvglu::build_plant(cfg, h->p);
  if (rc) {
    delete h;
    return rc;
  }
  h->contrib_sign_i.assign(h->p.contrib_sign.begin(), h->p.contrib_sign.end());
  h->inc_sign_i.assign(h->p.inc_sign.begin(), h->p.inc_sign.end());
  *out = h;
  return PVGLU_OK;
}

int pvglu_plant_destroy(pvglu_plant* p) {
  delete p;
  return PVGLU_OK;
}

int pvglu_plant_get_info(const pvglu_plant* h, pvglu_plant_info* info) {
  if (!h || !info) return PVGLU_ERR_BAD_ARG;
  const auto& p = h->p;
  info->n = p.n;
  info->n_panels = p.n_panels;
  info->nnz_a = (int64_t)p.colidx.size();
  info->n_inverters = p.cfg.n_inverters;
  info->n_strings = p.cfg.n_strings;
  info->n_series = p.cfg.n_series;
  info->voc_panel = p.voc_panel;
  info->v_mppt = p.v_mppt;
  info->extent_x = p.extent_x;
  info->extent_y = p.extent_y;
  info->panel_i0 = p.panel.i0;
  info->panel_a = p.panel.a;
  info->panel_rs = p.panel.rs;
  info->panel_rsh = p.panel.rsh;
  info->iph_stc = p.cfg.iph_stc;
  return PVGLU_OK;
}

int pvglu_plant_get_iarray(const pvglu_plant* h, const char* name, const int** data,
                           int64_t* len) {
  if (!h || !name || !data || !len) return PVGLU_ERR_BAD_ARG;
  const auto& p = h->p;
  const std::string k(name);
  const std::vector<int>* v = nullptr;
#define PVG(key, expr) if (k == key) v = &(expr);
  PVG("rowptr", p.rowptr) PVG("colidx", p.colidx) PVG("pan_hi", p.pan_hi)
  PVG("pan_lo", p.pan_lo) PVG("contrib_ptr", p.contrib_ptr)
  PVG("contrib_panel", p.contrib_panel) PVG("inc_ptr", p.inc_ptr)
  PVG("inc_panel", p.inc_panel) PVG("inv_terminal", p.inv_terminal)
  PVG("inv_current", p.inv_current) PVG("inv_combiner", p.inv_combiner)
  PVG("contrib_sign", h->contrib_sign_i) PVG("inc_sign", h->inc_sign_i)
#undef PVG
  if (!v) return PVGLU_ERR_BAD_ARG;
  *data = v->data();
  *len = (int64_t)v->size();
  return PVGLU_OK;
}

int pvglu_plant_get_darray(const pvglu_plant* h, const char* name, const double** data,
                           int64_t* len) {
  if (!h || !name || !data || !len) return PVGLU_ERR_BAD_ARG;
  const auto& p = h->p;
  const std::string k(name);
  const std::vector<double>* v = nullptr;
  if (k == "a_lin") v = &p.a_lin;
  if (k == "b_lin") v = &p.b_lin;
  if (k == "pan_x") v = &p.pan_x;
  if (k == "pan_y") v = &p.pan_y;
  if (!v) return PVGLU_ERR_BAD_ARG;
  *data = v->data();
  *len = (int64_t)v->size();
  return PVGLU_OK;
}

int pvglu_plant_irradiance(const pvglu_plant* h, int min_shadows, int max_shadows,
                           double min_depth, double max_depth, uint64_t seed, double t,
                           double* g_out) {
  if (!h || !g_out || min_shadows < 0 || max_shadows < min_shadows) return PVGLU_ERR_BAD_ARG;
  pvglu::ShadowConfig sc;
  sc.min_shadows = min_shadows;
  sc.max_shadows = max_shadows;
  sc.min_depth = min_depth;
  sc.max_depth = max_depth;
  pvglu::plant_irradiance(h->p, sc, seed, t, g_out);
  return PVGLU_OK;
}

int pvglu_plant_shadows(const pvglu_plant* h, int min_shadows, int max_shadows,
                        double min_depth, double max_depth, uint64_t seed, int* count,
                        double* params) {
  if (!h || !count || !params || min_shadows < 0 || max_shadows < min_shadows)
    return PVGLU_ERR_BAD_ARG;
  pvglu::ShadowConfig sc;
  sc.min_shadows = min_shadows;
  sc.max_shadows = max_shadows;
  sc.min_depth = min_depth;
  sc.max_depth = max_depth;
  std::vector<double> sh;
  pvglu::plant_shadows(h->p, sc, seed, sh);
  *count = (int)(sh.size() / 6);
  std::copy(sh.begin(), sh.end(), params);
  return PVGLU_OK;
}

int pvglu_plant_panel_iv(const pvglu_plant* h, int count, const double* iph, const double* v,
                         double* current, double* didv) {
  if (!h || count < 0 || !iph || !v || !current || !didv) return PVGLU_ERR_BAD_ARG;
  for (int i = 0; i < count; i++) pvglu_panel_iv(&h->p.panel, iph[i], v[i], &current[i], &didv[i]);
  return PVGLU_OK;
}

int pvglu_plant_exp_log(int count, const double* x, double* exp_out, double* log_out) {
  if (count < 0 || (count > 0 && !x)) return PVGLU_ERR_BAD_ARG;
  for (int i = 0; i < count; i++) {
    if (exp_out) exp_out[i] = pvglu_exp(x[i]);
    if (log_out) log_out[i] = pvglu_log(x[i]);
  }
  return PVGLU_OK;
}

}  // extern "C"

// C ABI of the host-only parts: errors, front end, readers, HDF5 writer.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <map>
#include <tuple>
#include "capi_util.hpp"
#include "schedule.hpp"
#include "frontend.hpp"

namespace slaph {
namespace {
thread_local std::string g_last_error;
}
void set_last_error(std::string const &m) { g_last_error = m; }
}  // namespace slaph

struct slaph_frontend {
  slaph::GlobalData gd;
  std::unique_ptr<slaph::FlatPlan> plan;
};

namespace {
void copy_str(std::string const &s, char *buf, size_t len) {
  if (!buf || len == 0) throw slaph::ArgError("null buffer");
  if (s.size() + 1 > len) throw slaph::ArgError("buffer too small for '" + s + "'");
  std::memcpy(buf, s.c_str(), s.size() + 1);
}
}  // namespace

extern "C" {

const char *slaph_last_error(void) { return slaph::g_last_error.c_str(); }

int slaph_trace_kind_arity(int kind) { return slaph::trace_kind_arity(kind); }
const char *slaph_trace_kind_name(int kind) { return slaph::trace_kind_name(kind); }

int slaph_frontend_create(const char *infile_path, int argc, const char *const *argv,
                          slaph_frontend **out) {
  return slaph::guarded(
      [&] {
        if (!infile_path || !out) throw slaph::ArgError("null argument");
        *out = nullptr;
        auto fe = std::make_unique<slaph_frontend>();
        std::vector<std::string> args;
        for (int i = 0; i < argc; ++i) args.emplace_back(argv[i] ? argv[i] : "");
        slaph::read_parameters(fe->gd, infile_path, args);
        fe->plan = std::make_unique<slaph::FlatPlan>(fe->gd);
        *out = fe.release();
      },
      SLAPH_ERR_PARSE);
}

int slaph_frontend_destroy(slaph_frontend *fe) {
  delete fe;
  return SLAPH_OK;
}

int slaph_frontend_dims(const slaph_frontend *fe, slaph_dims *out) {
  return slaph::guarded([&] {
    if (!fe || !out) throw slaph::ArgError("null argument");
    auto const &gd = fe->gd;
    if (gd.quarks.empty()) throw slaph::ArgError("no quarks defined");
    slaph_dims d{};
    d.Lt = gd.Lt;
    d.Lx = gd.Lx;
    d.Ly = gd.Ly;
    d.Lz = gd.Lz;
    d.nev = gd.number_of_eigen_vec;
    d.dilT = gd.quarks[0].number_of_dilution_T;
    d.dilE = gd.quarks[0].number_of_dilution_E;
    int n = 0;
    for (auto const &q : gd.quarks) n += q.number_of_rnd_vec;
    d.n_rnd = n;
    *out = d;
  });
}

int slaph_frontend_plan(const slaph_frontend *fe, const slaph_plan **out) {
  return slaph::guarded([&] {
    if (!fe || !out) throw slaph::ArgError("null argument");
    *out = &fe->plan->plan();
  });
}

int slaph_frontend_get_int(const slaph_frontend *fe, const char *key, int64_t *out) {
  return slaph::guarded([&] {
    if (!fe || !key || !out) throw slaph::ArgError("null argument");
    auto const &gd = fe->gd;
    std::string const k = key;
    if (k == "start_config")
      *out = gd.start_config;
    else if (k == "end_config")
      *out = gd.end_config;
    else if (k == "delta_config")
      *out = gd.delta_config;
    else if (k == "single_time_slice_combination")
      *out = gd.single_time_slice_combination;
    else if (k == "n_quarks")
      *out = static_cast<int64_t>(gd.quarks.size());
    else if (k == "nb_eigen_threads")
      *out = gd.nb_eigen_threads;
    else if (k == "iterations")
      *out = gd.iterations;
    else
      throw slaph::ArgError("unknown integer setting '" + k + "'");
  });
}

int slaph_frontend_get_double(const slaph_frontend *fe, const char *key, double *out) {
  return slaph::guarded([&] {
    if (!fe || !key || !out) throw slaph::ArgError("null argument");
    std::string const k = key;
    if (k == "alpha1")
      *out = fe->gd.alpha1;
    else if (k == "alpha2")
      *out = fe->gd.alpha2;
    else
      throw slaph::ArgError("unknown floating-point setting '" + k + "'");
  });
}

int slaph_frontend_get_str(const slaph_frontend *fe, const char *key, char *buf, size_t len) {
  return slaph::guarded([&] {
    if (!fe || !key) throw slaph::ArgError("null argument");
    auto const &gd = fe->gd;
    std::string const k = key;
    if (k == "output_path")
      copy_str(gd.path_output, buf, len);
    else if (k == "path_eigenvectors")
      copy_str(gd.path_eigenvectors, buf, len);
    else if (k == "name_eigenvectors")
      copy_str(gd.name_eigenvectors, buf, len);
    else if (k == "handling_vdaggerv")
      copy_str(gd.handling_vdaggerv, buf, len);
    else if (k == "path_vdaggerv")
      copy_str(gd.path_vdaggerv, buf, len);
    else if (k == "path_config")
      copy_str(gd.path_config, buf, len);
    else
      throw slaph::ArgError("unknown string setting '" + k + "'");
  });
}

int slaph_frontend_io_name(const slaph_frontend *fe, int config, int which, int index, char *buf,
                           size_t len) {
  return slaph::guarded([&] {
    if (!fe) throw slaph::ArgError("null argument");
    copy_str(slaph::io_name(fe->gd, config, which, index), buf, len);
  });
}

int slaph_vdaggerv_file_name(const char *path_vdaggerv, int32_t config, const slaph_vdv_op *op,
                             int32_t t, int32_t kind, char *buf, size_t len) {
  return slaph::guarded([&] {
    if (!path_vdaggerv || !op) throw slaph::ArgError("null argument");
    copy_str(slaph::vdaggerv_file_name(path_vdaggerv, config, *op, t, kind), buf, len);
  });
}

int slaph_read_eigenvectors(const char *path, int64_t dim_row, int32_t nev, double *out) {
  return slaph::guarded([&] {
    if (!path || !out || dim_row < 1 || nev < 1) throw slaph::ArgError("invalid argument");
    slaph::read_eigenvectors(path, dim_row, nev, out);
  });
}

int slaph_read_perambulator(const char *path, int32_t Lt, int32_t nev, int32_t dilT, int32_t dilE,
                            int32_t dilD, double *out) {
  return slaph::guarded([&] {
    if (!path || !out) throw slaph::ArgError("invalid argument");
    slaph::read_perambulator(path, Lt, nev, dilT, dilE, dilD, out);
  });
}

int slaph_read_random_vector(const char *path, int64_t length, double *out) {
  return slaph::guarded([&] {
    if (!path || !out || length < 1) throw slaph::ArgError("invalid argument");
    slaph::read_random_vector(path, length, out);
  });
}

int slaph_read_gauge_lime(const char *path, int32_t Lt, int32_t Lx, int32_t Ly, int32_t Lz,
                          int32_t n_dir, double *out) {
  return slaph::guarded([&] {
    if (!path || !out || Lt < 1 || Lx < 1 || Ly < 1 || Lz < 1)
      throw slaph::ArgError("invalid argument");
    slaph::read_gauge_lime(path, Lt, Lx, Ly, Lz, n_dir, out);
  });
}

int slaph_write_correlators_h5(const char *file_path, int32_t n_datasets,
                               const char *const *dataset_names, int32_t Lt, const double *data) {
  return slaph::guarded([&] {
    if (!file_path) throw slaph::ArgError("null path");
    slaph::write_correlators_h5(file_path, n_datasets, dataset_names, Lt, data);
  });
}

int64_t slaph_plan_output_doubles(const slaph_plan *plan, int32_t Lt) {
  if (!plan || Lt < 1) return -1;
  int64_t n = 0;
  for (int32_t d = 0; d < plan->n_diagrams; ++d) n += plan->diagrams[d].n_requests;
  return n * Lt * 2;
}

int slaph_plan_schedule_stats(const slaph_dims *dims, const slaph_plan *plan,
                              int32_t single_block_pair, int32_t check_layout, double *out,
                              int32_t n) {
  return slaph::guarded([&] {
    if (!dims || !plan || !out || n < 0) throw slaph::ArgError("null argument");
    slaph::Schedule const s = slaph::build_schedule(*dims, *plan, single_block_pair);
    double v[17] = {};
    v[0] = static_cast<double>(s.waves.size());
    int64_t lists = 0, uniq = 0, resid = 0, groups = 0;
    for (auto const &w : s.waves) {
      lists += static_cast<int64_t>(w.lists.size());
      uniq += static_cast<int64_t>(w.unique_lists.size());
      resid += static_cast<int64_t>(w.residual_lists.size());
      groups += static_cast<int64_t>(w.groups.size());
    }
    v[1] = static_cast<double>(lists);
    v[2] = static_cast<double>(uniq);
    v[3] = static_cast<double>(resid);
    v[4] = static_cast<double>(groups);
    v[5] = static_cast<double>(s.n_trace_entries);
    v[6] = static_cast<double>(s.n_unique_entries);
    v[7] = static_cast<double>(s.n_group_entries);
    v[8] = static_cast<double>(s.n_terms);
    v[9] = static_cast<double>(s.n_prods);
    v[10] = static_cast<double>(s.q0.size());
    v[11] = static_cast<double>(s.q1.size());
    v[12] = static_cast<double>(s.q2.size());
    v[13] = static_cast<double>(s.n_outputs);
    if (check_layout) {
      // Every value index is written by exactly one entry of one distinct
      // list; every other list reads the values of a list with its operands.
      bool ok = true;
      for (auto const &w : s.waves) {
        std::vector<uint8_t> seen(static_cast<size_t>(w.n_values), 0);
        for (int32_t l : w.unique_lists) {
          auto const &L = w.lists[l];
          int64_t const ne = static_cast<int64_t>(s.shapes[L.shape].i.size());
          for (int64_t e = 0; e < ne; ++e) {
            int64_t const k = L.val_off + e * L.stride;
            if (k < 0 || k >= w.n_values || seen[k]++) ok = false;
          }
        }
        for (auto c : seen)
          if (c != 1) ok = false;
        std::map<std::tuple<int32_t, int32_t, int32_t>, std::pair<int64_t, int32_t>> where;
        for (int32_t l : w.unique_lists) {
          auto const &L = w.lists[l];
          where[{L.shape, L.a_base, L.b_base}] = {L.val_off, L.stride};
        }
        for (auto const &L : w.lists) {
          auto it = where.find({L.shape, L.a_base, L.b_base});
          if (it == where.end() || it->second != std::make_pair(L.val_off, L.stride)) ok = false;
        }
        int64_t ge = 0;
        for (auto const &g : w.groups)
          ge += static_cast<int64_t>(s.shapes[g.shape].i.size()) * g.n_a * g.n_b;
        if (ge != w.n_group_entries || w.n_group_values != ge) ok = false;
      }
      v[14] = ok ? 1.0 : 0.0;
    }
    // The tensor-core product plan: its tiles, and (check_layout) whether it
    // computes every product of every level exactly once, into its slot,
    // from its left and right matrices.
    int64_t p_tiles = 0;
    bool p_ok = true;
    for (auto const &w : s.waves)
      for (size_t lv = 0; lv + 1 < w.prod_level_off.size(); ++lv) {
        int64_t const b = w.prod_level_off[lv], e = w.prod_level_off[lv + 1];
        slaph::ProductPlan const pp = slaph::plan_products(w.prods.data() + b, e - b, s.eds);
        p_tiles += pp.n_tiles;
        if (!check_layout) continue;
        std::vector<std::tuple<int32_t, int32_t, int32_t>> want, got;
        for (int64_t k = b; k < e; ++k) want.emplace_back(w.prods[k].a, w.prods[k].b, w.prods[k].c);
        for (auto const &g : pp.groups) {
          if (g.n_l < 1 || g.n_l > std::max(1, 64 / s.eds)) p_ok = false;
          for (int32_t u = 0; u < g.n_u; ++u) {
            int32_t const r = pp.r_slots[pp.u_list[g.u_off + u]];
            if (u > 0 && pp.u_list[g.u_off + u] <= pp.u_list[g.u_off + u - 1]) p_ok = false;
            for (int32_t l = 0; l < 4; ++l) {
              int32_t const slot = pp.out_tab[4 * (g.u_off + u) + l];
              if (slot < 0) continue;
              if (l >= g.n_l) p_ok = false;
              else got.emplace_back(g.l[l], r, slot);
            }
          }
        }
        std::sort(want.begin(), want.end());
        std::sort(got.begin(), got.end());
        if (want != got) p_ok = false;
      }
    v[15] = static_cast<double>(p_tiles);
    if (check_layout) v[16] = p_ok ? 1.0 : 0.0;
    for (int32_t i = 0; i < n && i < 17; ++i) out[i] = v[i];
  });
}

}  // extern "C"

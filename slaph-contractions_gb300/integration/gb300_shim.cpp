// gb300_shim.cpp -- the reference-side binding of the GB300 engine.
//
// A maintainer of sLapH-contractions compiles this file in place of
// src/OperatorFactory.cpp and src/Correlators.cpp and links
// libslaph_gb300.so; main/contract.cpp and every header stay unchanged.  It
// defines, against the reference's own declarations:
//
//   OperatorFactory (include/OperatorsForMesons.hpp:36-96): the constructor,
//     create_operators (src/OperatorFactory.cpp:507-520) and its three modes
//     build/write (build_vdaggerv, :220-326), read (:328-393) and liuming
//     (:395-490), and free_memory_vdaggerv.  VdaggerV is built on the GPU
//     (eigenvectors read and uploaded timeslice by timeslice, displaced
//     operators on HYP-smeared links) and copied into the class's own
//     vdaggerv blocks, so return_vdaggerv (:66-69) keeps its meaning.
//   create_momenta / create_momenta_new (:98-108): the phase table, for
//     callers such as tests/gtest/create_momenta.cpp.
//   contract (include/Correlators.hpp:41-54, src/Correlators.cpp:40-127): the
//     lookup tables flattened into slaph_plan, perambulators and random
//     vectors uploaded, the contraction on the GPU, and one HDF5 file per
//     diagram written as Diagram::write does (src/Diagram.cpp:132-147).
//
// The engine is created by create_operators (one per OperatorFactory) and
// found again by contract through the OperatorFactory it is given.  Errors of
// the engine are rethrown as std::runtime_error with the engine's message
// (which repeats the reference's own text where the reference throws).  The
// precision is SLAPH_MIXED unless the environment sets
// SLAPH_GB300_PRECISION=fp64.  C++11, like the reference.
#include "Correlators.hpp"
#include "OperatorsForMesons.hpp"
#include "Perambulator.hpp"
#include "RandomVector.hpp"
#include "global_data.hpp"
#include "typedefs.hpp"

#include "slaph_gb300.h"

#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

void ck(int rc) {
  if (rc != SLAPH_OK) throw std::runtime_error(slaph_last_error());
}

int precision_from_env() {
  char const *p = std::getenv("SLAPH_GB300_PRECISION");
  return (p && std::string(p) == "fp64") ? SLAPH_FP64 : SLAPH_MIXED;
}

// Page-locked host staging buffer from the engine (uploads at the full link
// rate), released on destruction.
struct PinnedBuffer {
  double *p = nullptr;
  size_t n = 0;
  void reserve(size_t doubles) {
    if (doubles <= n) return;
    if (p) slaph_host_free(p);
    p = nullptr;
    n = 0;
    void *q = nullptr;
    ck(slaph_host_alloc(doubles * sizeof(double), &q));
    p = static_cast<double *>(q);
    n = doubles;
  }
  ~PinnedBuffer() {
    if (p) slaph_host_free(p);
  }
};

// One engine per OperatorFactory, with what contract() needs to find again.
struct EngineState {
  slaph_engine *eng = nullptr;
  slaph_dims dims{};
  int precision = SLAPH_MIXED;
  std::vector<slaph_vdv_op> ops;
  PinnedBuffer staging;  // one eigenvector timeslice on its way to the device
  EngineState() = default;
  EngineState(EngineState const &) = delete;
  EngineState &operator=(EngineState const &) = delete;
  ~EngineState() {
    if (eng) slaph_engine_destroy(eng);
  }
};

std::mutex g_mutex;
std::map<OperatorFactory const *, std::unique_ptr<EngineState>> g_engines;

EngineState &state_of(OperatorFactory const *f) {
  std::lock_guard<std::mutex> lock(g_mutex);
  std::unique_ptr<EngineState> &s = g_engines[f];
  if (!s) s.reset(new EngineState);
  return *s;
}

// VdaggerVQuantumNumbers (include/typedefs.hpp:44-55) -> slaph_vdv_op, with
// the displacement steps passed through.
std::vector<slaph_vdv_op> flatten_operators(OperatorLookup const &lookup) {
  std::vector<slaph_vdv_op> ops;
  for (auto const &o : lookup.vdaggerv_lookup) {
    slaph_vdv_op v{};
    v.id = static_cast<int32_t>(o.id);
    for (int i = 0; i < 3; ++i) v.momentum[i] = o.momentum[i];
    if (o.displacement.size() > SLAPH_MAX_DISP)
      throw std::runtime_error("gb300 shim: more displacement steps than the engine takes");
    v.n_disp = static_cast<int32_t>(o.displacement.size());
    for (size_t k = 0; k < o.displacement.size(); ++k) {
      v.disp[2 * k] = o.displacement[k].first;
      v.disp[2 * k + 1] = o.displacement[k].second;
    }
    ops.push_back(v);
  }
  return ops;
}

// The number of random vectors: RandomVector has no count accessor, and its
// operator() checks the index (std::vector::at).
ssize_t count_random_vectors(RandomVector const &rnd, ssize_t length) {
  ssize_t n = 0;
  for (;; ++n) {
    try {
      (void)rnd(n, length - 1);
    } catch (std::out_of_range const &) {
      return n;
    }
  }
}

void mkdir_p(std::string const &path) {
  std::string cur;
  for (size_t i = 0; i <= path.size(); ++i) {
    if (i == path.size() || path[i] == '/') {
      if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
        throw std::runtime_error("cannot create directory " + cur);
    }
    if (i < path.size()) cur.push_back(path[i]);
  }
}

int trace_kind(std::string const &name) {
  for (int k = 0; k < SLAPH_TR_KINDS; ++k)
    if (name == slaph_trace_kind_name(k)) return k;
  throw std::runtime_error("gb300 shim: unknown trace " + name);
}

// The lookup tables contract() receives, flattened into slaph_plan; the
// vectors own everything the plan points to.
struct FlatPlan {
  slaph_plan plan{};
  std::vector<slaph_vdv_op> ops;
  std::vector<std::vector<int32_t>> pairs[3];
  std::vector<slaph_factor_index> factors[3];
  std::vector<int32_t> trace_ids[SLAPH_TR_KINDS];
  std::vector<std::vector<slaph_correlator_request>> requests;
  std::vector<std::string> names;
  std::vector<slaph_diagram> diagrams;

  FlatPlan(OperatorLookup const &lookup, DilutedFactorIndicesCollection const &quarks,
           TraceIndicesCollection const &traces, CorrelatorRequestsMap const &corr) {
    ops = flatten_operators(lookup);
    char const *qnames[3] = {"Q0", "Q1", "Q2"};
    for (int q = 0; q < 3; ++q) {
      auto it = quarks.find(qnames[q]);
      if (it == quarks.end()) continue;
      for (auto const &f : it->second) {
        pairs[q].emplace_back();
        for (auto const &p : f.rnd_vec_ids) {
          pairs[q].back().push_back(static_cast<int32_t>(p.first));
          pairs[q].back().push_back(static_cast<int32_t>(p.second));
        }
      }
      for (size_t i = 0; i < it->second.size(); ++i) {
        auto const &f = it->second[i];
        slaph_factor_index x{};
        x.id_vdaggerv = static_cast<int32_t>(f.id_vdaggerv);
        x.need_vdaggerv_daggering = f.need_vdaggerv_daggering ? 1 : 0;
        x.gamma = f.gamma.empty() ? 0 : f.gamma[0];
        x.n_rnd_pairs = static_cast<int32_t>(f.rnd_vec_ids.size());
        x.rnd_pairs = pairs[q][i].data();
        factors[q].push_back(x);
      }
    }
    for (auto const &t : traces) {
      int const k = trace_kind(t.first);
      for (auto const &ids : t.second) {
        if (static_cast<int>(ids.size()) != slaph_trace_kind_arity(k))
          throw std::runtime_error("gb300 shim: trace index arity mismatch");
        for (auto x : ids) trace_ids[k].push_back(static_cast<int32_t>(x));
      }
    }
    for (auto const &d : corr) {
      if (d.second.empty()) continue;  // contract() skips empty diagrams
      names.push_back(d.first);
      requests.emplace_back();
      for (auto const &r : d.second) {
        if (r.trace_requests.size() > 3)
          throw std::runtime_error("This many traces are not implemented yet.");
        slaph_correlator_request c{};
        c.n_traces = static_cast<int32_t>(r.trace_requests.size());
        for (size_t i = 0; i < r.trace_requests.size(); ++i) {
          auto const &tr = r.trace_requests[i];
          c.traces[i].kind = trace_kind(tr.tr_name);
          c.traces[i].tr_id = static_cast<int32_t>(tr.tr_id);
          c.traces[i].n_loc = static_cast<int32_t>(tr.locations.size());
          for (size_t l = 0; l < tr.locations.size() && l < 6; ++l)
            c.traces[i].loc[l] = tr.locations[l] == Location::sink ? 1 : 0;
        }
        c.dataset_name = r.hdf5_dataset_name.c_str();
        requests.back().push_back(c);
      }
    }
    for (size_t i = 0; i < names.size(); ++i) {
      slaph_diagram g{};
      g.name = names[i].c_str();
      g.n_requests = static_cast<int32_t>(requests[i].size());
      g.requests = requests[i].data();
      diagrams.push_back(g);
    }
    plan.n_vdv_ops = static_cast<int32_t>(ops.size());
    plan.vdv_ops = ops.data();
    plan.index_of_unity = lookup.index_of_unity;
    plan.need_gaugefield = lookup.need_gaugefield ? 1 : 0;
    for (int q = 0; q < 3; ++q) {
      plan.n_factors[q] = static_cast<int32_t>(factors[q].size());
      plan.factors[q] = factors[q].data();
    }
    for (int k = 0; k < SLAPH_TR_KINDS; ++k) {
      plan.n_trace_ids[k] =
          static_cast<int32_t>(trace_ids[k].size() / slaph_trace_kind_arity(k));
      plan.trace_ql_ids[k] = trace_ids[k].data();
    }
    plan.n_diagrams = static_cast<int32_t>(diagrams.size());
    plan.diagrams = diagrams.data();
  }
};

}  // namespace

// create_momenta (src/OperatorFactory.cpp:64-95): momentum[op.id][x] =
// exp(-i 2 pi (px x/Lx + py y/Ly + pz z/Lz)), site x * Ly * Lz + y * Lz + z.
void create_momenta(const ssize_t Lx, const ssize_t Ly, const ssize_t Lz,
                    const std::vector<VdaggerVQuantumNumbers> &vdaggerv_lookup,
                    array_cd_d2 &momentum) {
  const double pi2 = 2.0 * std::acos(-1.0);
  for (auto const &op : vdaggerv_lookup) {
    const double ipx = op.momentum[0] * pi2 / static_cast<double>(Lx);
    const double ipy = op.momentum[1] * pi2 / static_cast<double>(Ly);
    const double ipz = op.momentum[2] * pi2 / static_cast<double>(Lz);
    for (ssize_t x = 0; x < Lx; ++x)
      for (ssize_t y = 0; y < Ly; ++y)
        for (ssize_t z = 0; z < Lz; ++z) {
          const double arg = (ipx * x + ipy * y) + ipz * z;
          momentum[op.id][x * Ly * Lz + y * Lz + z] =
              std::complex<double>(std::cos(arg), -std::sin(arg));
        }
  }
}

// create_momenta_new (:110-140) computes the same table.
void create_momenta_new(const ssize_t Lx, const ssize_t Ly, const ssize_t Lz,
                        const std::vector<VdaggerVQuantumNumbers> &vdaggerv_lookup,
                        array_cd_d2 &momentum) {
  create_momenta(Lx, Ly, Lz, vdaggerv_lookup, momentum);
}

OperatorFactory::OperatorFactory(const ssize_t Lt, const ssize_t Lx, const ssize_t Ly,
                                 const ssize_t Lz, const ssize_t nb_ev, const ssize_t dilE,
                                 const OperatorLookup &operator_lookuptable,
                                 const std::string &handling_vdaggerv,
                                 const std::string &path_vdaggerv,
                                 const std::string &path_config,
                                 const HypPars &hyp_parameters)
    : vdaggerv(),
      momentum(),
      operator_lookuptable(operator_lookuptable),
      Lt(Lt),
      Lx(Lx),
      Ly(Ly),
      Lz(Lz),
      nb_ev(nb_ev),
      dilE(dilE),
      handling_vdaggerv(handling_vdaggerv),
      path_vdaggerv(path_vdaggerv),
      path_config(path_config),
      hyp_parameters(hyp_parameters) {
  vdaggerv.resize(boost::extents[operator_lookuptable.vdaggerv_lookup.size()][Lt]);
  // The phases are built on the device; the host table is not kept.
}

// The engine of this factory, created on its first create_operators.  The
// time dilution is an argument of contract() only (include/Correlators.hpp:
// 41-54): the engine starts with one dilution block (dilT = Lt), which VdaggerV
// does not depend on, and contract() sets the real one.
void OperatorFactory::create_operators(const std::string &filename,
                                       const RandomVector &rnd_vec, const int config) {
  is_vdaggerv_set = false;
  EngineState &s = state_of(this);
  if (!s.eng) {
    s.precision = precision_from_env();
    s.dims.Lt = static_cast<int32_t>(Lt);
    s.dims.Lx = static_cast<int32_t>(Lx);
    s.dims.Ly = static_cast<int32_t>(Ly);
    s.dims.Lz = static_cast<int32_t>(Lz);
    s.dims.nev = static_cast<int32_t>(nb_ev);
    s.dims.dilT = static_cast<int32_t>(Lt);
    s.dims.dilE = static_cast<int32_t>(dilE);
    s.dims.n_rnd = static_cast<int32_t>(count_random_vectors(rnd_vec, Lt * 4 * nb_ev));
    if (s.dims.n_rnd < 1) throw std::runtime_error("gb300 shim: no random vectors");
    s.ops = flatten_operators(operator_lookuptable);
    ck(slaph_engine_create(&s.dims, &s.eng));
    ck(slaph_engine_set_operators(s.eng, s.ops.data(), static_cast<int32_t>(s.ops.size()),
                                  operator_lookuptable.index_of_unity));
  }
  if (handling_vdaggerv == "write" || handling_vdaggerv == "build")
    build_vdaggerv(filename, config);
  else if (handling_vdaggerv == "read")
    read_vdaggerv(config);
  else if (handling_vdaggerv == "liuming")
    read_vdaggerv_liuming(config);
  else
    throw std::runtime_error("The flag handling_vdaggerv in input file is wrong!");
  // The blocks into the class's own storage, for return_vdaggerv.
  for (auto const &op : operator_lookuptable.vdaggerv_lookup)
    for (ssize_t t = 0; t < Lt; ++t) {
      Eigen::MatrixXcd &m = vdaggerv[op.id][t];
      m.resize(nb_ev, nb_ev);
      ck(slaph_vdaggerv_fetch(s.eng, static_cast<int32_t>(op.id), static_cast<int32_t>(t),
                              reinterpret_cast<double *>(m.data())));
    }
  is_vdaggerv_set = true;
}

void OperatorFactory::build_vdaggerv(const std::string &filename, const int config) {
  EngineState &s = state_of(this);
  int64_t const dim_row = 3 * Lx * Ly * Lz;
  bool const only_unity = operator_lookuptable.vdaggerv_lookup.size() == 1 &&
                          operator_lookuptable.vdaggerv_lookup[0].id ==
                              operator_lookuptable.index_of_unity;
  if (operator_lookuptable.need_gaugefield) {
    // GaugeField::read_gauge_field + smearing_hyp (:248-260), on the device
    char name[4096];
    std::snprintf(name, sizeof name, "%s/conf.%04d", path_config.c_str(), config);
    std::vector<double> U(static_cast<size_t>(Lt) * Lx * Ly * Lz * 3 * 18);
    ck(slaph_read_gauge_lime(name, static_cast<int32_t>(Lt), static_cast<int32_t>(Lx),
                             static_cast<int32_t>(Ly), static_cast<int32_t>(Lz), 3, U.data()));
    size_t const per = static_cast<size_t>(Lx) * Ly * Lz * 3 * 18;
    for (ssize_t t = 0; t < Lt; ++t)
      ck(slaph_engine_set_gauge(s.eng, static_cast<int32_t>(t), U.data() + per * t));
    if (hyp_parameters.iterations > 0)
      ck(slaph_engine_smear_gauge_hyp(s.eng, hyp_parameters.alpha1, hyp_parameters.alpha2,
                                      static_cast<int32_t>(hyp_parameters.iterations)));
  }
  if (!only_unity) {
    // "<filename>%03d" per timeslice (:274-278), read into one page-locked
    // buffer and copied to the device timeslice by timeslice.
    s.staging.reserve(static_cast<size_t>(2 * dim_row * nb_ev));
    for (ssize_t t = 0; t < Lt; ++t) {
      char name[4096];
      std::snprintf(name, sizeof name, "%s%03d", filename.c_str(), static_cast<int>(t));
      ck(slaph_read_eigenvectors(name, dim_row, static_cast<int32_t>(nb_ev), s.staging.p));
      ck(slaph_engine_set_eigenvectors(s.eng, static_cast<int32_t>(t), s.staging.p));
    }
  }
  ck(slaph_vdaggerv_build(s.eng, s.precision));
  if (handling_vdaggerv == "write") ck(slaph_vdaggerv_write(s.eng, path_vdaggerv.c_str(), config));
}

void OperatorFactory::read_vdaggerv(const int config) {
  ck(slaph_vdaggerv_read(state_of(this).eng, path_vdaggerv.c_str(), config, 0));
}

void OperatorFactory::read_vdaggerv_liuming(const int config) {
  ck(slaph_vdaggerv_read(state_of(this).eng, path_vdaggerv.c_str(), config, 1));
}

void OperatorFactory::free_memory_vdaggerv() {
  for (auto const &op : operator_lookuptable.vdaggerv_lookup)
    for (ssize_t t = 0; t < Lt; ++t) vdaggerv[op.id][t].resize(0, 0);
}

void contract(const ssize_t Lt, const ssize_t dilT, const ssize_t dilE, const ssize_t nev,
              OperatorFactory const &meson_operator, RandomVector const &randomvectors,
              Perambulator const &perambulators, OperatorLookup const &operator_lookup,
              TraceIndicesCollection const &trace_indices_map,
              CorrelatorRequestsMap const &correlator_requests_map,
              DilutedFactorIndicesCollection const &quark_lookup, std::string const output_path,
              std::string const output_filename, int single_time_slice_combination) {
  EngineState &s = state_of(&meson_operator);
  if (!s.eng)
    throw std::runtime_error("gb300 shim: create_operators must run before contract");
  if (s.dims.Lt != Lt || s.dims.nev != nev || s.dims.dilE != dilE)
    throw std::runtime_error("gb300 shim: contract sizes differ from the OperatorFactory's");
  if (s.dims.dilT != dilT) {
    ck(slaph_engine_set_time_dilution(s.eng, static_cast<int32_t>(dilT)));
    s.dims.dilT = static_cast<int32_t>(dilT);
  }
  FlatPlan const fp(operator_lookup, quark_lookup, trace_indices_map, correlator_requests_map);
  // Perambulators (Eigen column-major complex, the ABI's layout) and random
  // vectors (copied through RandomVector::operator()).
  ssize_t const length = Lt * 4 * nev;
  std::vector<std::complex<double>> noise(static_cast<size_t>(length));
  for (int32_t r = 0; r < s.dims.n_rnd; ++r) {
    Eigen::MatrixXcd const &P = perambulators[r];
    ck(slaph_engine_set_perambulator(s.eng, r, reinterpret_cast<double const *>(P.data())));
    for (ssize_t k = 0; k < length; ++k) noise[static_cast<size_t>(k)] = randomvectors(r, k);
    ck(slaph_engine_set_random_vector(s.eng, r, reinterpret_cast<double const *>(noise.data())));
  }
  std::vector<double> corr(
      static_cast<size_t>(slaph_plan_output_doubles(&fp.plan, static_cast<int32_t>(Lt))));
  ck(slaph_contract(s.eng, &fp.plan, s.precision, SLAPH_ACC_NATIVE,
                    single_time_slice_combination, corr.data()));
  // Diagram::write: <output_path>/<diagram><output_filename>, one dataset per
  // request (include/h5-wrapper.hpp:106-200).
  mkdir_p(output_path);
  size_t k = 0;
  for (auto const &d : fp.diagrams) {
    std::vector<char const *> names;
    for (int32_t i = 0; i < d.n_requests; ++i) names.push_back(d.requests[i].dataset_name);
    std::string const file = output_path + "/" + d.name + output_filename;
    ck(slaph_write_correlators_h5(file.c_str(), d.n_requests, names.data(),
                                  static_cast<int32_t>(Lt), corr.data() + 2 * k * Lt));
    k += static_cast<size_t>(d.n_requests);
  }
}

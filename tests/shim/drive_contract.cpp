// Test driver of the reference-side shim: the sequence of main/contract.cpp
// (:55-105) for one configuration, on the reference's own types (here the
// stand-in headers), with the shim's OperatorFactory and contract().
//
// The lookup tables are rebuilt in the reference's types (OperatorLookup,
// DilutedFactorIndicesCollection, TraceIndicesCollection,
// CorrelatorRequestsMap) from the engine's front end, so the shim's
// flattening is exercised in a round trip.  Inputs are read from the
// reference's file formats and names under the working directory.
//
//   drive_contract <infile> <config>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "Correlators.hpp"
#include "slaph_gb300.h"

namespace {

void ck(int rc) {
  if (rc != SLAPH_OK) throw std::runtime_error(slaph_last_error());
}

std::string io_name(slaph_frontend const *fe, int config, int which, int index) {
  char buf[4096];
  ck(slaph_frontend_io_name(fe, config, which, index, buf, sizeof buf));
  return buf;
}

std::string get_str(slaph_frontend const *fe, char const *key) {
  char buf[4096];
  ck(slaph_frontend_get_str(fe, key, buf, sizeof buf));
  return buf;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: drive_contract <infile> <config>\n");
    return 2;
  }
  try {
    int const config = std::atoi(argv[2]);
    std::string const cfg = argv[2];
    char const *args[] = {"--start_config", cfg.c_str(), "--end_config", cfg.c_str()};
    slaph_frontend *fe = nullptr;
    ck(slaph_frontend_create(argv[1], 4, args, &fe));
    slaph_dims d{};
    ck(slaph_frontend_dims(fe, &d));
    slaph_plan const *plan = nullptr;
    ck(slaph_frontend_plan(fe, &plan));

    // lookup tables in the reference's types
    OperatorLookup lookup;
    for (int32_t i = 0; i < plan->n_vdv_ops; ++i) {
      slaph_vdv_op const &o = plan->vdv_ops[i];
      DisplacementDirection disp;
      for (int32_t k = 0; k < o.n_disp; ++k) disp.push_back({o.disp[2 * k], o.disp[2 * k + 1]});
      lookup.vdaggerv_lookup.emplace_back(o.id, std::array<int, 3>{o.momentum[0], o.momentum[1],
                                                                   o.momentum[2]},
                                          disp);
    }
    lookup.index_of_unity = plan->index_of_unity;
    lookup.need_gaugefield = plan->need_gaugefield != 0;
    DilutedFactorIndicesCollection quarks;
    char const *qn[3] = {"Q0", "Q1", "Q2"};
    for (int q = 0; q < 3; ++q) {
      auto &v = quarks[qn[q]];
      for (int32_t i = 0; i < plan->n_factors[q]; ++i) {
        slaph_factor_index const &f = plan->factors[q][i];
        DilutedFactorIndex x;
        x.id_vdaggerv = f.id_vdaggerv;
        x.need_vdaggerv_daggering = f.need_vdaggerv_daggering != 0;
        x.gamma = {f.gamma};
        for (int32_t k = 0; k < f.n_rnd_pairs; ++k)
          x.rnd_vec_ids.emplace_back(f.rnd_pairs[2 * k], f.rnd_pairs[2 * k + 1]);
        v.push_back(x);
      }
    }
    TraceIndicesCollection traces;
    for (int k = 0; k < SLAPH_TR_KINDS; ++k) {
      auto &v = traces[slaph_trace_kind_name(k)];
      int const ar = slaph_trace_kind_arity(k);
      for (int32_t i = 0; i < plan->n_trace_ids[k]; ++i)
        v.emplace_back(plan->trace_ql_ids[k] + static_cast<ptrdiff_t>(i) * ar,
                       plan->trace_ql_ids[k] + static_cast<ptrdiff_t>(i + 1) * ar);
    }
    CorrelatorRequestsMap requests;
    for (int32_t g = 0; g < plan->n_diagrams; ++g) {
      slaph_diagram const &dg = plan->diagrams[g];
      auto &v = requests[dg.name];
      for (int32_t r = 0; r < dg.n_requests; ++r) {
        slaph_correlator_request const &c = dg.requests[r];
        CorrelatorRequest cr;
        cr.hdf5_dataset_name = c.dataset_name;
        for (int32_t j = 0; j < c.n_traces; ++j) {
          TraceRequest tr;
          tr.tr_name = slaph_trace_kind_name(c.traces[j].kind);
          tr.tr_id = c.traces[j].tr_id;
          for (int32_t l = 0; l < c.traces[j].n_loc; ++l)
            tr.locations.push_back(c.traces[j].loc[l] ? Location::sink : Location::source);
          cr.trace_requests.push_back(tr);
        }
        v.push_back(cr);
      }
    }

    // inputs, as main/contract.cpp:55-88 sets them up
    ssize_t const length = static_cast<ssize_t>(d.Lt) * 4 * d.nev;
    RandomVector rnd(d.n_rnd, length);
    std::vector<ssize_t> rows(d.n_rnd, length),
        cols(d.n_rnd, static_cast<ssize_t>(d.Lt / d.dilT) * d.dilE * 4);
    Perambulator peram(d.n_rnd, rows, cols);
    for (int32_t r = 0; r < d.n_rnd; ++r) {
      ck(slaph_read_random_vector(io_name(fe, config, 2, r).c_str(), length,
                                  reinterpret_cast<double *>(rnd.load(r))));
      ck(slaph_read_perambulator(io_name(fe, config, 1, r).c_str(), d.Lt, d.nev, d.dilT, d.dilE,
                                 4, reinterpret_cast<double *>(peram.load(r).data())));
    }
    double a1 = 0, a2 = 0;
    int64_t iters = 0;
    ck(slaph_frontend_get_double(fe, "alpha1", &a1));
    ck(slaph_frontend_get_double(fe, "alpha2", &a2));
    ck(slaph_frontend_get_int(fe, "iterations", &iters));
    HypPars hyp{a1, a2, static_cast<ssize_t>(iters)};
    OperatorFactory factory(d.Lt, d.Lx, d.Ly, d.Lz, d.nev, d.dilE, lookup,
                            get_str(fe, "handling_vdaggerv"), get_str(fe, "path_vdaggerv"),
                            get_str(fe, "path_config"), hyp);
    factory.create_operators(io_name(fe, config, 0, 0), rnd, config);
    contract(d.Lt, d.dilT, d.dilE, d.nev, factory, rnd, peram, lookup, traces, requests, quarks,
             get_str(fe, "output_path"), io_name(fe, config, 3, 0), -1);
    // return_vdaggerv keeps its meaning: the identity block stays the identity
    if (lookup.index_of_unity >= 0) {
      Eigen::MatrixXcd const &I = factory.return_vdaggerv(lookup.index_of_unity, 0);
      for (int i = 0; i < d.nev; ++i)
        if (I(i, i) != Complex(1.0, 0.0)) throw std::runtime_error("identity block");
    }
    std::printf("drive_contract: %d diagrams written\n", plan->n_diagrams);
    slaph_frontend_destroy(fe);
    return 0;
  } catch (std::exception const &e) {
    std::fprintf(stderr, "drive_contract: %s\n", e.what());
    return 1;
  }
}

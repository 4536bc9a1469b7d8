// Front end of the engine: infile -> GlobalData -> lookup tables.
//
// Restates, in plain C++17 without Boost or Eigen:
//   read_parameters            src/global_data.cpp:61-390
//   make_quark/operator/corr   src/global_data_input_handling_utils.cpp:133-347
//   diagram_specs              src/DiagramSpec.cpp:3-163
//   init_lookup_tables         src/init_lookup_tables.cpp:470-556
//   build_IO_names             src/global_data_build_IO_names.cpp:76-85
// The output is the set of lookup tables contract() consumes, plus a flat
// slaph_plan view of them for the C ABI.
#pragma once

#include <array>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../../include/slaph_gb300.h"

namespace slaph {

using Vec3 = std::array<int, 3>;
// (direction '>' or '<', axis 'x' 'y' 'z') pairs, include/typedefs.hpp:21
using Displacement = std::vector<std::pair<char, char>>;

struct Quark {  // include/global_data_typedefs.hpp:35-72
  std::string type;
  int number_of_rnd_vec = 0;
  std::string dilution_T;
  int number_of_dilution_T = 0;
  std::string dilution_E;
  int number_of_dilution_E = 0;
  std::string dilution_D;
  int number_of_dilution_D = 0;
  int id = 0;
  std::string path;
};

struct QuantumNumbers {  // include/global_data_typedefs.hpp:82-89
  std::vector<int> gamma;
  Displacement displacement;
  Vec3 momentum{0, 0, 0};
};

using Operators = std::vector<QuantumNumbers>;

struct CorrelatorSpec {  // Correlators_2, include/global_data_typedefs.hpp:142-150
  std::string type;
  std::vector<int> quark_numbers;
  std::vector<int> operator_numbers;
  std::string GEVP;
  std::vector<Vec3> tot_mom;
};

struct VdvQuantumNumbers {  // include/typedefs.hpp:44-55
  int id;
  Vec3 momentum;
  Displacement displacement;
};

struct OperatorLookup {  // include/typedefs.hpp:63-78
  std::vector<VdvQuantumNumbers> vdaggerv_lookup;
  int index_of_unity = -1;
  bool need_gaugefield = false;
};

struct FactorIndex {  // DilutedFactorIndex, include/typedefs.hpp:105-121
  int id_vdaggerv = 0;
  bool need_vdaggerv_daggering = false;
  std::vector<int> gamma;
  std::vector<std::pair<int, int>> rnd_vec_ids;
  bool operator==(FactorIndex const &o) const {
    return id_vdaggerv == o.id_vdaggerv &&
           need_vdaggerv_daggering == o.need_vdaggerv_daggering && gamma == o.gamma &&
           rnd_vec_ids == o.rnd_vec_ids;
  }
};

enum class Location { source = 0, sink = 1 };

struct TraceRequest {  // include/global_data.hpp:72-81
  std::string tr_name;
  int tr_id = 0;
  std::vector<Location> locations;
  bool operator==(TraceRequest const &o) const {
    return tr_name == o.tr_name && tr_id == o.tr_id && locations == o.locations;
  }
};

struct CorrelatorRequest {  // include/global_data.hpp:83-90
  std::vector<TraceRequest> trace_requests;
  std::string hdf5_dataset_name;
  // Equality ignores the dataset name, as the reference does.
  bool operator==(CorrelatorRequest const &o) const {
    return trace_requests == o.trace_requests;
  }
};

struct QuarklineSpec {  // include/DiagramSpec.hpp:8-14
  std::string name;
  int q1, q2;
  bool is_loop() const { return q1 == q2; }
};
using TraceSpec = std::vector<QuarklineSpec>;
struct DiagramSpec {
  std::pair<std::vector<int>, std::vector<int>> vertices;  // (source, sink)
  std::vector<TraceSpec> traces;
};

// diagram_specs, src/DiagramSpec.cpp:3-163
std::map<std::string, DiagramSpec> const &diagram_specs();

// Trace-kind name <-> enum slaph_trace_kind.
int trace_kind_from_name(std::string const &name);
char const *trace_kind_name(int kind);
int trace_kind_arity(int kind);

struct GlobalData {  // include/global_data.hpp:104-160
  int Lx = 0, Ly = 0, Lz = 0, Lt = 0;
  int number_of_eigen_vec = 0;
  int start_config = -1, end_config = 0, delta_config = 1;
  long nb_eigen_threads = 1;
  std::string path_eigenvectors = ".";
  std::string name_eigenvectors = "eigenvector";
  std::string path_output = "../../contractions";
  std::string path_config;
  std::string name_lattice;
  std::string handling_vdaggerv = "build";
  std::string path_vdaggerv;
  double alpha1 = 0, alpha2 = 0;
  long iterations = 0;
  int single_time_slice_combination = -1;

  std::vector<Quark> quarks;
  std::vector<Operators> operator_list;
  std::vector<CorrelatorSpec> correlator_list;
  std::map<int, int> momentum_cutoff{{0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 4}};

  OperatorLookup operator_lookuptable;
  std::map<std::string, std::vector<FactorIndex>> quarkline_lookuptable;
  std::map<std::string, std::vector<std::vector<int>>> trace_indices_map;
  std::map<std::string, std::vector<CorrelatorRequest>> correlator_requests_map;
};

// Parses an infile (boost::program_options config-file syntax) plus
// "--key value" command-line overrides and builds the lookup tables.
// Throws std::runtime_error with the reference's message texts.
void read_parameters(GlobalData &gd, std::string const &infile,
                     std::vector<std::string> const &args);

// Individual parsers (exposed for tests).
Quark make_quark(std::string const &s);
Operators make_operator_list(std::string const &s);
CorrelatorSpec make_correlator(std::string const &s);
void init_lookup_tables(GlobalData &gd);

// Dataset name, src/init_lookup_tables.cpp:196-211.
std::string build_hdf5_dataset_name(std::string const &corr_type,
                                    std::vector<std::string> const &quark_types,
                                    std::vector<QuantumNumbers> const &qn);

std::string io_name(GlobalData const &gd, int config, int which, int index);

// Owner of a flattened slaph_plan view over a GlobalData's lookup tables.
class FlatPlan {
 public:
  explicit FlatPlan(GlobalData const &gd);
  slaph_plan const &plan() const { return plan_; }

 private:
  slaph_plan plan_{};
  std::vector<slaph_vdv_op> vdv_;
  std::vector<std::vector<int32_t>> rnd_storage_[3];
  std::vector<slaph_factor_index> factors_[3];
  std::vector<int32_t> trace_ids_[SLAPH_TR_KINDS];
  std::vector<std::vector<slaph_correlator_request>> requests_;
  std::vector<std::string> names_;
  std::vector<std::string> dataset_names_;
  std::vector<slaph_diagram> diagrams_;
};

}  // namespace slaph

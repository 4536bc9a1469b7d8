// Test stand-in for the reference's include/OperatorsForMesons.hpp: class
// OperatorFactory with the reference's constructor, public interface
// (create_operators, free_memory_vdaggerv, return_vdaggerv :59-69), private
// members and private builders, and the create_momenta declarations
// (:98-108).  The reference-side shim defines the member functions.
#pragma once
#include <Eigen/Dense>
#include <boost/multi_array.hpp>

#include "RandomVector.hpp"
#include "global_data.hpp"
#include "typedefs.hpp"

typedef boost::multi_array<Eigen::MatrixXcd, 2> array_Xcd_d2_eigen;
typedef boost::multi_array<Complex, 2> array_cd_d2;

class OperatorFactory {
 public:
  OperatorFactory(const ssize_t Lt, const ssize_t Lx, const ssize_t Ly, const ssize_t Lz,
                  const ssize_t nb_ev, const ssize_t dilE,
                  const OperatorLookup &operator_lookuptable,
                  const std::string &handling_vdaggerv, const std::string &path_vdaggerv,
                  const std::string &path_config, const HypPars &hyp_parameters);
  ~OperatorFactory(){};

  void create_operators(const std::string &filename, const RandomVector &rnd_vec,
                        const int config);
  void free_memory_vdaggerv();

  inline const Eigen::MatrixXcd &return_vdaggerv(const ssize_t index, const ssize_t t) const {
    return vdaggerv[static_cast<size_t>(index)][t];
  }

 private:
  array_Xcd_d2_eigen vdaggerv;
  array_cd_d2 momentum;

  const OperatorLookup operator_lookuptable;
  const ssize_t Lt, Lx, Ly, Lz;
  const ssize_t nb_ev, dilE;
  bool is_vdaggerv_set = false;
  std::string handling_vdaggerv;
  std::string path_vdaggerv;
  std::string path_config;
  HypPars hyp_parameters;

  void build_vdaggerv(const std::string &filename, const int config);
  void read_vdaggerv(const int config);
  void read_vdaggerv_liuming(const int config);
};

void create_momenta(const ssize_t Lx, const ssize_t Ly, const ssize_t Lz,
                    const std::vector<VdaggerVQuantumNumbers> &vdaggerv_lookup,
                    array_cd_d2 &momentum);

void create_momenta_new(const ssize_t Lx, const ssize_t Ly, const ssize_t Lz,
                        const std::vector<VdaggerVQuantumNumbers> &vdaggerv_lookup,
                        array_cd_d2 &momentum);

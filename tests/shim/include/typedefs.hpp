// Test stand-in for the reference's include/typedefs.hpp: the types the
// reference-side shim reads (VdaggerVQuantumNumbers :44-55, OperatorLookup
// :57-77, DilutedFactorIndex :105-121, DilutedFactorIndicesCollection :136),
// with the reference's member names and types.
#pragma once
#include <sys/types.h>

#include <array>
#include <complex>
#include <map>
#include <string>
#include <utility>
#include <vector>

using Complex = std::complex<double>;
using DisplacementDirection = std::vector<std::pair<char, char>>;

struct VdaggerVQuantumNumbers {
  ssize_t id;
  std::array<int, 3> momentum;
  DisplacementDirection displacement;
  VdaggerVQuantumNumbers(const ssize_t id, std::array<int, 3> const &momentum,
                         DisplacementDirection const &displacement)
      : id(id), momentum(momentum), displacement(displacement) {}
};

struct OperatorLookup {
  std::vector<VdaggerVQuantumNumbers> vdaggerv_lookup;
  int index_of_unity;
  bool need_gaugefield = false;
};

struct DilutedFactorIndex {
  ssize_t id_vdaggerv;
  bool need_vdaggerv_daggering;
  std::vector<int> gamma;
  std::vector<std::pair<ssize_t, ssize_t>> rnd_vec_ids;
};

using DilutedFactorIndicesCollection = std::map<std::string, std::vector<DilutedFactorIndex>>;
using Indices = std::vector<ssize_t>;

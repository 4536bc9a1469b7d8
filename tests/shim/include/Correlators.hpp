// Test stand-in for the reference's include/Correlators.hpp: the declaration
// of contract() (:41-54) and the headers it brings in.
#pragma once
#include "OperatorsForMesons.hpp"
#include "Perambulator.hpp"
#include "global_data.hpp"
#include "typedefs.hpp"

#include <string>

void contract(const ssize_t Lt, const ssize_t dilT, const ssize_t dilE, const ssize_t nev,
              OperatorFactory const &meson_operator, RandomVector const &randomvectors,
              Perambulator const &perambulators, OperatorLookup const &operator_lookup,
              TraceIndicesCollection const &trace_indices_map,
              CorrelatorRequestsMap const &correlator_requests_map,
              DilutedFactorIndicesCollection const &quark_lookup, std::string const output_path,
              std::string const output_filename, int single_time_slice_combination);

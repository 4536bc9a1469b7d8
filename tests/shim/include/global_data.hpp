// Test stand-in for the reference's include/global_data.hpp and
// global_data_typedefs.hpp: the request types contract() receives
// (Location, TraceRequest, CorrelatorRequest, TraceIndicesCollection,
// CorrelatorRequestsMap) and HypPars, with the reference's member names.
#pragma once
#include "typedefs.hpp"

enum class Location { source, sink };

struct TraceRequest {
  std::string tr_name;
  ssize_t tr_id;
  std::vector<Location> locations;
};

struct CorrelatorRequest {
  std::vector<TraceRequest> trace_requests;
  std::string hdf5_dataset_name;
};

typedef std::map<std::string, std::vector<Indices>> TraceIndicesCollection;
typedef std::map<std::string, std::vector<CorrelatorRequest>> CorrelatorRequestsMap;

struct HypPars {
  double alpha1;
  double alpha2;
  ssize_t iterations;
};

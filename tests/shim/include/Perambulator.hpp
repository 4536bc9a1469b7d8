// Test stand-in for the reference's include/Perambulator.hpp: the class with
// its constructor and operator[](entity) (:44) returning the re-sorted
// column-major Eigen::MatrixXcd.  The test driver fills it through load().
#pragma once
#include <Eigen/Dense>

#include "typedefs.hpp"

class Perambulator {
 public:
  Perambulator(const ssize_t nb_entities, const std::vector<ssize_t> &size_rows,
               const std::vector<ssize_t> &size_cols)
      : peram(static_cast<size_t>(nb_entities)) {
    for (ssize_t i = 0; i < nb_entities; i++)
      peram[static_cast<size_t>(i)].resize(size_rows[static_cast<size_t>(i)],
                                           size_cols[static_cast<size_t>(i)]);
  }
  inline const Eigen::MatrixXcd &operator[](const ssize_t entity) const {
    return peram.at(static_cast<size_t>(entity));
  }
  Eigen::MatrixXcd &load(const ssize_t entity) { return peram.at(static_cast<size_t>(entity)); }

 private:
  std::vector<Eigen::MatrixXcd> peram;
};

// Test stand-in for the reference's include/RandomVector.hpp: the class with
// its constructor and operator()(entity, entry) (:38, a checked access).  The
// test driver fills it with load(), which the shim does not use.
#pragma once
#include "typedefs.hpp"

class RandomVector {
 public:
  RandomVector(const ssize_t nb_entities, const ssize_t length)
      : vec(static_cast<size_t>(nb_entities * length)), length(length) {}
  inline Complex operator()(const ssize_t entity, const ssize_t entry) const {
    return vec.at(static_cast<size_t>(entity * length + entry));
  }
  Complex *load(const ssize_t entity) { return vec.data() + entity * length; }

 private:
  std::vector<Complex> vec;
  const ssize_t length;
};

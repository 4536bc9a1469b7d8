// Error plumbing of the C ABI: typed exceptions inside the library, int status
// codes plus a thread-local message at the boundary.  The message texts follow
// the reference's exceptions where the reference throws.
#pragma once

#include <stdexcept>
#include <string>

#include "../../../include/slaph_gb300.h"

namespace slaph {

struct Error : std::runtime_error {
  int code;
  Error(int c, std::string const &m) : std::runtime_error(m), code(c) {}
};
struct ArgError : Error {
  explicit ArgError(std::string const &m) : Error(SLAPH_ERR_ARG, m) {}
};
struct IoError : Error {
  explicit IoError(std::string const &m) : Error(SLAPH_ERR_IO, m) {}
};
struct StateError : Error {
  explicit StateError(std::string const &m) : Error(SLAPH_ERR_STATE, m) {}
};
struct EmptyError : Error {
  explicit EmptyError(std::string const &m) : Error(SLAPH_ERR_EMPTY, m) {}
};
struct UnsupportedError : Error {
  explicit UnsupportedError(std::string const &m) : Error(SLAPH_ERR_UNSUPPORTED, m) {}
};
struct CudaError : Error {
  explicit CudaError(std::string const &m) : Error(SLAPH_ERR_CUDA, m) {}
};
struct NoMemError : Error {
  explicit NoMemError(std::string const &m) : Error(SLAPH_ERR_NOMEM, m) {}
};
struct TimeoutError : Error {
  explicit TimeoutError(std::string const &m) : Error(SLAPH_ERR_TIMEOUT, m) {}
};

void set_last_error(std::string const &m);

// Runs f, mapping exceptions to status codes and the thread-local message.
template <typename F>
int guarded(F &&f, int fallback = SLAPH_ERR_ARG) {
  try {
    f();
    return SLAPH_OK;
  } catch (Error const &e) {
    set_last_error(e.what());
    return e.code;
  } catch (std::bad_alloc const &) {
    set_last_error("host allocation failed");
    return SLAPH_ERR_NOMEM;
  } catch (std::exception const &e) {
    set_last_error(e.what());
    return fallback;
  }
}

// Readers and writer of io.cpp.
void read_eigenvectors(char const *path, int64_t dim_row, int32_t nev, double *out);
void read_perambulator(char const *path, int32_t Lt, int32_t nev, int32_t dilT, int32_t dilE,
                       int32_t dilD, double *out);
void read_random_vector(char const *path, int64_t length, double *out);
void read_gauge_lime(char const *path, int32_t Lt, int32_t Lx, int32_t Ly, int32_t Lz,
                     int32_t n_dir, double *out);
void write_correlators_h5(char const *file_path, int32_t n, char const *const *names, int32_t Lt,
                          double const *data);
std::string vdaggerv_file_name(char const *path, int32_t config, slaph_vdv_op const &op,
                               int32_t t, int32_t kind);
void write_vdaggerv_file(std::string const &name, double const *block, int64_t nev);
void read_vdaggerv_file(std::string const &name, double *out, int64_t n_doubles);

}  // namespace slaph

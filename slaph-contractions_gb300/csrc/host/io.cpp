// Input staging and correlator output in the reference's file formats.
//
//  slaph_read_eigenvectors    EigenVector::read_eigen_vector, src/EigenVector.cpp:35-76
//  slaph_read_perambulator    Perambulator::read_perambulator, src/Perambulator.cpp:12-71
//  slaph_read_random_vector   RandomVector::read_random_vector, src/RandomVector.cpp:87-113
//  slaph_read_gauge_lime      GaugeField::read_gauge_field + map_timeslice_to_eigen,
//                             src/GaugeField.cpp:108-149,762-928
//  slaph_write_correlators_h5 WriteHDF5Correlator, include/h5-wrapper.hpp:106-200
//  slaph_vdaggerv_file_name   VdaggerV file names of OperatorFactory's "write",
//                             "read" and "liuming" modes, src/OperatorFactory.cpp:
//                             225-237,302-312,328-490
//
// The HDF5 writer emits the same on-disk subset the reference's HDF5 C++ calls
// produce (superblock v0, one root group as a v1 B-tree of symbol-table nodes,
// contiguous datasets of compound {re f64, im f64}), written directly because
// no HDF5 library is present.
#include <algorithm>
#include <complex>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <stdexcept>
#include <string>
#include <vector>

#include "capi_util.hpp"

namespace slaph {

void read_eigenvectors(char const *path, int64_t dim_row, int32_t nev, double *out) {
  FILE *fp = std::fopen(path, "rb");
  if (!fp) throw IoError(std::string("Eigenvector file does not exist! ") + path);
  for (int32_t c = 0; c < nev; ++c) {
    size_t const n = std::fread(out + 2 * dim_row * c, sizeof(double), 2 * dim_row, fp);
    if (n != static_cast<size_t>(2 * dim_row)) {
      std::fclose(fp);
      throw IoError(std::string("Problem while reading Eigenvectors! ") + path);
    }
  }
  std::fclose(fp);
}

void read_perambulator(char const *path, int32_t Lt, int32_t nev, int32_t dilT, int32_t dilE,
                       int32_t dilD, double *out) {
  if (Lt < 1 || nev < 1 || dilT < 1 || dilE < 1 || dilD < 1 || Lt % dilT)
    throw ArgError("invalid perambulator sizes");
  int64_t const rows = 4LL * nev * Lt;
  int64_t const nblk = Lt / dilT;
  int64_t const cols = nblk * dilE * dilD;
  std::vector<double> buf(static_cast<size_t>(2 * rows * cols));
  FILE *fp = std::fopen(path, "rb");
  if (!fp) throw IoError(std::string("failed to open file to read perambulator: ") + path);
  size_t const n = std::fread(buf.data(), 2 * sizeof(double), rows * cols, fp);
  std::fclose(fp);
  if (n != static_cast<size_t>(rows * cols))
    throw IoError("Failed to read perambulator. Expected size " + std::to_string(rows * cols) +
                  " and got " + std::to_string(n));
  // File rows are (t, ev, dirac) with dirac fastest, columns (block, ev, dirac)
  // with dirac fastest; the matrix wants rows (t, dirac, ev) and columns
  // (block, dirac, ev) with ev fastest (src/Perambulator.cpp:53-64).
  for (int64_t t1 = 0; t1 < Lt; ++t1)
    for (int64_t ev1 = 0; ev1 < nev; ++ev1)
      for (int64_t d1 = 0; d1 < 4; ++d1) {
        int64_t const row_file = 4 * nev * t1 + 4 * ev1 + d1;
        int64_t const row = 4 * nev * t1 + nev * d1 + ev1;
        for (int64_t b = 0; b < nblk; ++b)
          for (int64_t ev2 = 0; ev2 < dilE; ++ev2)
            for (int64_t d2 = 0; d2 < dilD; ++d2) {
              int64_t const col_file = dilD * dilE * b + dilD * ev2 + d2;
              int64_t const col = dilE * dilD * b + dilE * d2 + ev2;
              double const *src = &buf[2 * (row_file * cols + col_file)];
              double *dst = out + 2 * (row + rows * col);
              dst[0] = src[0];
              dst[1] = src[1];
            }
      }
}

void read_random_vector(char const *path, int64_t length, double *out) {
  FILE *fp = std::fopen(path, "rb");
  if (!fp) throw IoError(std::string("failed to open file to read random vector: ") + path);
  size_t const n = std::fread(out, 2 * sizeof(double), length, fp);
  std::fclose(fp);
  if (n != static_cast<size_t>(length))
    throw IoError(std::string("not all data could be read from random vector file ") + path);
}

// LIME container (records of a 144-byte big-endian header: magic 0x456789ab,
// version, flags, data length, 128-byte type; data padded to 8 bytes) holding
// an ILDG gauge field: "ildg-binary-data" of big-endian doubles, sites with x
// fastest and t slowest, per site the links in direction order x, y, z, t,
// each 3x3 complex row-major.  Written out as the reference's GaugeField keeps
// them: per timeslice [site x Ly Lz + y Lz + z][dir][a + 3 b] (column-major
// link), spatial directions 0..2 and, with n_dir == 4, the temporal link as
// direction 3.
void read_gauge_lime(char const *path, int32_t Lt, int32_t Lx, int32_t Ly, int32_t Lz,
                     int32_t n_dir, double *out) {
  if (n_dir != 3 && n_dir != 4) throw ArgError("n_dir must be 3 or 4");
  FILE *fp = std::fopen(path, "rb");
  if (!fp) throw IoError(std::string("Could not open file ") + path);
  auto be64 = [](uint8_t const *p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v = (v << 8) | p[i];
    return v;
  };
  int64_t const V3 = static_cast<int64_t>(Lx) * Ly * Lz;
  int64_t const sites = V3 * Lt;
  uint64_t const want = static_cast<uint64_t>(sites) * 72 * sizeof(double);
  bool found = false;
  uint64_t len = 0;
  for (;;) {
    uint8_t hdr[144];
    if (std::fread(hdr, 1, 144, fp) != 144) break;
    uint64_t const magic = (static_cast<uint64_t>(hdr[0]) << 24) | (hdr[1] << 16) |
                           (hdr[2] << 8) | hdr[3];
    if (magic != 0x456789abULL) {
      std::fclose(fp);
      throw IoError(std::string("not a LIME file: ") + path);
    }
    len = be64(hdr + 8);
    std::string const type(reinterpret_cast<char const *>(hdr + 16),
                           strnlen(reinterpret_cast<char const *>(hdr + 16), 128));
    if (type == "ildg-binary-data") {
      found = true;
      break;
    }
    if (std::fseek(fp, static_cast<long>((len + 7) / 8 * 8), SEEK_CUR) != 0) break;
  }
  if (!found) {
    std::fclose(fp);
    throw IoError(std::string("no ildg-binary-data record found in file ") + path);
  }
  if (len != want) {
    std::fclose(fp);
    if (len == want / 2) throw UnsupportedError("Single precision read!");
    throw IoError(std::string("Probably wrong lattice size or precision in file ") + path);
  }
  std::vector<uint8_t> site(72 * sizeof(double));
  for (int64_t t = 0; t < Lt; ++t)
    for (int64_t z = 0; z < Lz; ++z)
      for (int64_t y = 0; y < Ly; ++y)
        for (int64_t x = 0; x < Lx; ++x) {
          if (std::fread(site.data(), 1, site.size(), fp) != site.size()) {
            std::fclose(fp);
            throw IoError(std::string("LIME read error while reading file ") + path);
          }
          int64_t const s = x * Ly * Lz + y * Lz + z;
          for (int k = 0; k < 4; ++k) {  // file directions x, y, z, t
            if (k == 3 && n_dir == 3) continue;
            double *link = out + ((t * V3 + s) * n_dir + k) * 18;
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j)
                for (int c = 0; c < 2; ++c) {
                  uint64_t const bits = be64(site.data() + 8 * (((k * 3 + i) * 3 + j) * 2 + c));
                  double v;
                  std::memcpy(&v, &bits, sizeof v);
                  link[2 * (i + 3 * j) + c] = v;
                }
          }
        }
  std::fclose(fp);
}

namespace {

// Little-endian byte sink with patchable fields.
struct Buf {
  std::vector<uint8_t> b;
  size_t pos() const { return b.size(); }
  void u8(uint8_t v) { b.push_back(v); }
  void u16(uint16_t v) {
    for (int i = 0; i < 2; ++i) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
  }
  void u32(uint32_t v) {
    for (int i = 0; i < 4; ++i) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
  }
  void u64(uint64_t v) {
    for (int i = 0; i < 8; ++i) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
  }
  void bytes(void const *p, size_t n) {
    auto const *c = static_cast<uint8_t const *>(p);
    b.insert(b.end(), c, c + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() {
    while (b.size() % 8) b.push_back(0);
  }
  void put64(size_t at, uint64_t v) {
    for (int i = 0; i < 8; ++i) b[at + i] = static_cast<uint8_t>(v >> (8 * i));
  }
  void put32(size_t at, uint32_t v) {
    for (int i = 0; i < 4; ++i) b[at + i] = static_cast<uint8_t>(v >> (8 * i));
  }
};

constexpr uint64_t kUndef = ~0ULL;
constexpr int kLeafK = 4;       // group leaf node K: at most 2K entries per SNOD
constexpr int kInternalK = 16;  // group internal node K: at most 2K children

// One header message: type, payload; payload padded to 8 bytes.
void message(Buf &o, uint16_t type, Buf const &payload, uint8_t flags = 0) {
  Buf p = payload;
  p.pad8();
  o.u16(type);
  o.u16(static_cast<uint16_t>(p.b.size()));
  o.u8(flags);
  o.zeros(3);
  o.bytes(p.b.data(), p.b.size());
}

// Version-1 object header around a list of (type, payload, flags).
void object_header(Buf &o, std::vector<std::tuple<uint16_t, Buf, uint8_t>> const &msgs) {
  Buf body;
  for (auto const &m : msgs) message(body, std::get<0>(m), std::get<1>(m), std::get<2>(m));
  o.u8(1);
  o.u8(0);
  o.u16(static_cast<uint16_t>(msgs.size()));
  o.u32(1);
  o.u32(static_cast<uint32_t>(body.b.size()));
  o.zeros(4);
  o.bytes(body.b.data(), body.b.size());
}

Buf f64_member_type() {
  Buf t;
  t.u8(0x11);  // version 1, class 1 (floating point)
  t.u8(0x20);  // little endian, no padding, implied mantissa msb
  t.u8(63);    // sign bit location
  t.u8(0);
  t.u32(8);
  t.u16(0);     // bit offset
  t.u16(64);    // precision
  t.u8(52);     // exponent location
  t.u8(11);     // exponent size
  t.u8(0);      // mantissa location
  t.u8(52);     // mantissa size
  t.u32(1023);  // exponent bias
  return t;
}

Buf complex_type() {
  Buf t;
  t.u8(0x16);  // version 1, class 6 (compound)
  t.u16(2);    // two members
  t.u8(0);
  t.u32(16);
  char const *names[2] = {"re", "im"};
  for (int m = 0; m < 2; ++m) {
    t.bytes(names[m], 2);
    t.zeros(6);        // name + NUL padded to 8
    t.u32(8 * m);      // byte offset
    t.u8(0);           // dimensionality
    t.zeros(3 + 4 + 4 + 16);
    Buf mt = f64_member_type();
    t.bytes(mt.b.data(), mt.b.size());
  }
  return t;
}

}  // namespace

void write_correlators_h5(char const *file_path, int32_t n, char const *const *names, int32_t Lt,
                          double const *data) {
  if (n < 0 || Lt < 1 || (n > 0 && (!names || !data))) throw ArgError("invalid h5 write args");
  // Links of an HDF5 group B-tree are kept sorted by name (strcmp order).
  std::vector<int32_t> order(n);
  for (int32_t i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(),
            [&](int32_t a, int32_t b) { return std::strcmp(names[a], names[b]) < 0; });
  for (int32_t i = 1; i < n; ++i)
    if (std::strcmp(names[order[i - 1]], names[order[i]]) == 0)
      throw ArgError(std::string("duplicate dataset name ") + names[order[i]]);

  Buf o;
  // Superblock v0.
  o.bytes("\x89HDF\r\n\x1a\n", 8);
  o.u8(0);
  o.u8(0);
  o.u8(0);
  o.u8(0);
  o.u8(0);
  o.u8(8);
  o.u8(8);
  o.u8(0);
  o.u16(kLeafK);
  o.u16(kInternalK);
  o.u32(0);
  o.u64(0);       // base address
  o.u64(kUndef);  // free-space info
  size_t const eof_at = o.pos();
  o.u64(0);       // end of file, patched
  o.u64(kUndef);  // driver info
  // Root group symbol table entry.
  o.u64(0);
  size_t const root_hdr_at = o.pos();
  o.u64(0);
  o.u32(1);
  o.u32(0);
  size_t const root_scratch_at = o.pos();
  o.u64(0);
  o.u64(0);

  // Local heap: "" at 0, then names, each NUL-terminated and padded to 8.
  Buf heap_data;
  heap_data.zeros(8);
  std::vector<uint64_t> name_off(n);
  for (int32_t k = 0; k < n; ++k) {
    int32_t const i = order[k];
    name_off[k] = heap_data.pos();
    heap_data.bytes(names[i], std::strlen(names[i]) + 1);
    heap_data.pad8();
  }
  size_t const heap_at = o.pos();
  o.bytes("HEAP", 4);
  o.u8(0);
  o.zeros(3);
  o.u64(heap_data.pos());
  o.u64(kUndef);
  o.u64(heap_at + 32);
  o.bytes(heap_data.b.data(), heap_data.b.size());

  // Dataset headers and data.
  std::vector<uint64_t> hdr_addr(n);
  for (int32_t k = 0; k < n; ++k) {
    int32_t const i = order[k];
    o.pad8();
    hdr_addr[k] = o.pos();
    Buf space;
    space.u8(1);
    space.u8(1);
    space.u8(1);
    space.zeros(5);
    space.u64(static_cast<uint64_t>(Lt));
    space.u64(static_cast<uint64_t>(Lt));
    Buf fill;
    fill.u8(2);
    fill.u8(2);
    fill.u8(2);
    fill.u8(1);
    fill.u32(0);
    Buf layout;
    layout.u8(3);
    layout.u8(1);
    size_t const data_addr_field = 2;
    layout.u64(0);
    layout.u64(static_cast<uint64_t>(16) * Lt);
    size_t const hdr_start = o.pos();
    object_header(o, {{0x1, space, 0}, {0x3, complex_type(), 1}, {0x5, fill, 1}, {0x8, layout, 0}});
    // The layout message is the last one; patch its data address after the
    // header is emitted.
    size_t const layout_payload = o.pos() - 24;
    o.pad8();
    uint64_t const data_at = o.pos();
    o.put64(layout_payload + data_addr_field, data_at);
    (void)hdr_start;
    o.bytes(data + 2 * static_cast<size_t>(Lt) * i, 16 * static_cast<size_t>(Lt));
  }

  // Symbol-table nodes (leaves) of up to 2*kLeafK entries each.
  struct Child {
    uint64_t addr;
    uint64_t max_name;  // heap offset of the largest name below
  };
  std::vector<Child> level;
  for (int32_t s = 0; s < n || (s == 0 && n == 0); s += 2 * kLeafK) {
    int32_t const cnt = std::min<int32_t>(2 * kLeafK, n - s);
    o.pad8();
    uint64_t const at = o.pos();
    o.bytes("SNOD", 4);
    o.u8(1);
    o.u8(0);
    o.u16(static_cast<uint16_t>(std::max(cnt, 0)));
    for (int32_t e = 0; e < 2 * kLeafK; ++e) {
      if (e < cnt) {
        o.u64(name_off[s + e]);
        o.u64(hdr_addr[s + e]);
        o.u32(0);
        o.u32(0);
        o.zeros(16);
      } else {
        o.zeros(40);
      }
    }
    level.push_back({at, cnt > 0 ? name_off[s + cnt - 1] : 0});
    if (n == 0) break;
  }
  // B-tree levels of up to 2*kInternalK children per node.
  int node_level = 0;
  uint64_t root_btree = 0;
  while (true) {
    std::vector<Child> parents;
    for (size_t s = 0; s < level.size(); s += 2 * kInternalK) {
      size_t const cnt = std::min<size_t>(2 * kInternalK, level.size() - s);
      o.pad8();
      uint64_t const at = o.pos();
      o.bytes("TREE", 4);
      o.u8(0);
      o.u8(static_cast<uint8_t>(node_level));
      o.u16(static_cast<uint16_t>(cnt));
      o.u64(kUndef);
      o.u64(kUndef);
      o.u64(0);  // key 0: empty name
      for (size_t c = 0; c < cnt; ++c) {
        o.u64(level[s + c].addr);
        o.u64(level[s + c].max_name);
      }
      // Unused entries of a full-size node.
      for (size_t c = cnt; c < 2 * kInternalK; ++c) {
        o.u64(0);
        o.u64(0);
      }
      parents.push_back({at, level[s + cnt - 1].max_name});
    }
    ++node_level;
    if (parents.size() == 1) {
      root_btree = parents[0].addr;
      break;
    }
    level = parents;
  }
  // Root group object header: symbol table message.
  o.pad8();
  uint64_t const root_hdr = o.pos();
  Buf stab;
  stab.u64(root_btree);
  stab.u64(heap_at);
  object_header(o, {{0x11, stab, 0}});
  o.pad8();
  o.put64(root_hdr_at, root_hdr);
  o.put64(root_scratch_at, root_btree);
  o.put64(root_scratch_at + 8, heap_at);
  o.put64(eof_at, o.pos());

  FILE *fp = std::fopen(file_path, "wb");
  if (!fp) throw IoError(std::string("cannot create ") + file_path);
  size_t const w = std::fwrite(o.b.data(), 1, o.b.size(), fp);
  int const rc = std::fclose(fp);
  if (w != o.b.size() || rc != 0) throw IoError(std::string("short write to ") + file_path);
}

// ---------------------------------------------------------------- VdaggerV files
// Momentum digits as std::to_string of each component, concatenated
// (src/OperatorFactory.cpp:306-308, 352-354).
static std::string momentum_string(int32_t const m[3], int sign) {
  return std::to_string(sign * m[0]) + std::to_string(sign * m[1]) + std::to_string(sign * m[2]);
}

std::string vdaggerv_file_name(char const *path, int32_t config, slaph_vdv_op const &op,
                               int32_t t, int32_t kind) {
  char buf[64];
  std::string const p = path ? path : "";
  switch (kind) {
    case SLAPH_VDV_FILE_WRITE: {
      // "/%s/cnfg%04d/" + "operators.%04d.p_%s.d_%s.t_%03d" (:225-226, 309-311);
      // the displacement string is to_string(DisplacementDirection)
      // (include/global_data_typedefs.hpp:108-117): "000" or the pairs.
      std::string d;
      for (int i = 0; i < op.n_disp; ++i) {
        d.push_back(op.disp[2 * i]);
        d.push_back(op.disp[2 * i + 1]);
      }
      if (op.n_disp == 0) d = "000";
      std::snprintf(buf, sizeof buf, "/cnfg%04d/operators.%04d.p_", config, config);
      std::string out = "/" + p + buf + momentum_string(op.momentum, 1) + ".d_" + d;
      std::snprintf(buf, sizeof buf, ".t_%03d", t);
      return out + buf;
    }
    case SLAPH_VDV_FILE_READ: {
      // "/%s/cnfg%04d/operators.%04d" + ".p_" + momentum + "_.t_%03d" (:332-356):
      // no displacement, and not the name the "write" mode produces.
      std::snprintf(buf, sizeof buf, "/cnfg%04d/operators.%04d.p_", config, config);
      std::string out = "/" + p + buf + momentum_string(op.momentum, 1);
      std::snprintf(buf, sizeof buf, "_.t_%03d", t);
      return out + buf;
    }
    case SLAPH_VDV_FILE_LIUMING_MINUS:
    case SLAPH_VDV_FILE_LIUMING_PLUS: {
      // "/%s/VdaggerV." + "p<x>p<y>p<z>.conf%04d", first with -p (:400-427).
      int const sg = kind == SLAPH_VDV_FILE_LIUMING_MINUS ? -1 : 1;
      std::string out = "/" + p + "/VdaggerV.";
      for (int i = 0; i < 3; ++i) out += "p" + std::to_string(sg * op.momentum[i]);
      std::snprintf(buf, sizeof buf, ".conf%04d", config);
      return out + buf;
    }
    default:
      throw ArgError("unknown VdaggerV file kind " + std::to_string(kind));
  }
}

void write_vdaggerv_file(std::string const &name, double const *block, int64_t nev) {
  // write_vdaggerv (src/OperatorFactory.cpp:144-168): nev x nev complex,
  // column-major, native doubles.  The directory is created as build_vdaggerv
  // does in "write" mode (:229-237).
  std::filesystem::path const dir = std::filesystem::path(name).parent_path();
  std::error_code ec;
  if (!dir.empty()) std::filesystem::create_directories(dir, ec);
  std::FILE *fp = std::fopen(name.c_str(), "wb");
  if (!fp) throw IoError("Can't open " + name);
  size_t const n = static_cast<size_t>(2 * nev * nev);
  size_t const w = std::fwrite(block, sizeof(double), n, fp);
  int const rc = std::fclose(fp);
  if (w != n || rc != 0) throw IoError("Problems while write to " + name);
}

void read_vdaggerv_file(std::string const &name, double *out, int64_t n_doubles) {
  std::FILE *fp = std::fopen(name.c_str(), "rb");
  if (!fp) throw IoError("Can't open " + name);
  size_t const r = std::fread(out, sizeof(double), static_cast<size_t>(n_doubles), fp);
  std::fclose(fp);
  if (r != static_cast<size_t>(n_doubles)) throw IoError("Problems while reading from " + name);
}

}  // namespace slaph

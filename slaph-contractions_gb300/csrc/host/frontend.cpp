// Front end: infile parsing and lookup-table construction.  See frontend.hpp
// for the reference functions each part restates.
#include "frontend.hpp"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace slaph {

namespace {

std::string trim(std::string const &s) {
  size_t b = s.find_first_not_of(" \t\r\n");
  if (b == std::string::npos) return "";
  size_t e = s.find_last_not_of(" \t\r\n");
  return s.substr(b, e - b + 1);
}

// boost::split with is_any_of(sep) keeps empty tokens.
std::vector<std::string> split(std::string const &s, char sep) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : s) {
    if (c == sep) {
      out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(c);
    }
  }
  out.push_back(cur);
  return out;
}

// Strict integer conversion in the manner of boost::lexical_cast<int>.
int to_int(std::string const &s) {
  if (s.empty()) throw std::runtime_error("bad lexical cast: empty string to int");
  size_t pos = 0;
  long v = 0;
  try {
    v = std::stol(s, &pos);
  } catch (...) {
    throw std::runtime_error("bad lexical cast: '" + s + "' to int");
  }
  if (pos != s.size() || s[0] == ' ' || s[0] == '+')
    throw std::runtime_error("bad lexical cast: '" + s + "' to int");
  return static_cast<int>(v);
}

double to_double(std::string const &s) {
  size_t pos = 0;
  double v = 0;
  try {
    v = std::stod(s, &pos);
  } catch (...) {
    throw std::runtime_error("bad lexical cast: '" + s + "' to double");
  }
  if (pos != s.size()) throw std::runtime_error("bad lexical cast: '" + s + "' to double");
  return v;
}

int norm2(Vec3 const &v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
Vec3 neg(Vec3 const &v) { return {-v[0], -v[1], -v[2]}; }
Vec3 add(Vec3 const &a, Vec3 const &b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }

// src/global_data_input_handling_utils.cpp:40-52: strips "p(" / "P(" and ")".
Vec3 vec3_from_string(std::string in) {
  in.erase(0, 2);
  if (!in.empty()) in.erase(in.end() - 1);
  auto tok = split(in, ',');
  if (tok.size() < 3) throw std::runtime_error("bad 3-vector '" + in + "'");
  return {to_int(tok[0]), to_int(tok[1]), to_int(tok[2])};
}

// src/global_data_input_handling_utils.cpp:54-66: all integer 3-vectors with
// |p|^2 == p, components running from -p to p, first component slowest.
void all_momenta_with_norm(int p, std::vector<Vec3> &out) {
  for (int a = -p; a < p + 1; ++a)
    for (int b = -p; b < p + 1; ++b)
      for (int c = -p; c < p + 1; ++c)
        if (a * a + b * b + c * c == p) out.push_back({a, b, c});
}

std::string ints_to_string(std::vector<int> const &v) {
  std::string r;
  for (int x : v) r += std::to_string(x);
  return r;
}
std::string vec_to_string(Vec3 const &v) {
  return std::to_string(v[0]) + std::to_string(v[1]) + std::to_string(v[2]);
}
std::string disp_to_string(Displacement const &d) {
  if (d.empty()) return "000";
  std::string r;
  for (auto const &p : d) {
    r.push_back(p.first);
    r.push_back(p.second);
  }
  return r;
}

template <typename T>
int unique_push_back(std::vector<T> &v, T const &e) {
  auto it = std::find(v.begin(), v.end(), e);
  if (it == v.end()) {
    v.push_back(e);
    return static_cast<int>(v.size()) - 1;
  }
  return static_cast<int>(it - v.begin());
}

std::map<std::string, DiagramSpec> make_diagram_specs() {
  std::map<std::string, DiagramSpec> m;
  using V = std::vector<int>;
  auto spec = [](V so, V si, std::vector<TraceSpec> tr) {
    DiagramSpec d;
    d.vertices = {so, si};
    d.traces = tr;
    return d;
  };
  m["C1"] = spec({0}, {}, {{{"Q1", 0, 0}}});
  m["C20"] = spec({0}, {1}, {{{"Q1", 0, 1}, {"Q1", 1, 0}}});
  m["C2c"] = spec({0}, {1}, {{{"Q0", 0, 1}, {"Q2", 1, 0}}});
  m["C20V"] = spec({0}, {1}, {{{"Q1", 0, 0}}, {{"Q1", 1, 1}}});
  m["C30"] = spec({0, 2}, {1}, {{{"Q1", 0, 1}, {"Q1", 1, 2}, {"Q1", 2, 0}}});
  m["C3c"] = spec({0, 2}, {1}, {{{"Q1", 0, 1}, {"Q0", 1, 2}, {"Q2", 2, 0}}});
  m["C30V"] = spec({0, 1}, {2}, {{{"Q1", 0, 1}, {"Q1", 1, 0}}, {{"Q1", 2, 2}}});
  m["C40B"] = spec({0, 3}, {1, 2},
                   {{{"Q1", 3, 0}, {"Q1", 0, 1}, {"Q1", 1, 2}, {"Q1", 2, 3}}});
  m["C4cB"] = spec({0, 3}, {1, 2},
                   {{{"Q2", 3, 0}, {"Q0", 0, 1}, {"Q2", 1, 2}, {"Q0", 2, 3}}});
  m["C40C"] = spec({0, 2}, {1, 3},
                   {{{"Q1", 3, 0}, {"Q1", 0, 1}, {"Q1", 1, 2}, {"Q1", 2, 3}}});
  m["C4cC"] = spec({0, 2}, {1, 3},
                   {{{"Q2", 3, 0}, {"Q0", 0, 1}, {"Q2", 1, 2}, {"Q0", 2, 3}}});
  m["C40D"] = spec({0, 2}, {1, 3},
                   {{{"Q1", 0, 1}, {"Q1", 1, 0}}, {{"Q1", 2, 3}, {"Q1", 3, 2}}});
  m["C4cD"] = spec({0, 2}, {1, 3},
                   {{{"Q0", 0, 1}, {"Q2", 1, 0}}, {{"Q0", 2, 3}, {"Q2", 3, 2}}});
  m["C40V"] = spec({0, 1}, {2, 3},
                   {{{"Q1", 0, 1}, {"Q1", 1, 0}}, {{"Q1", 2, 3}, {"Q1", 3, 2}}});
  m["C4cV"] = spec({0, 1}, {2, 3},
                   {{{"Q0", 0, 1}, {"Q2", 1, 0}}, {{"Q0", 2, 3}, {"Q2", 3, 2}}});
  m["C6cC"] = spec({0, 2, 4}, {1, 3, 5},
                   {{{"Q2", 5, 0},
                     {"Q0", 0, 1},
                     {"Q2", 1, 2},
                     {"Q0", 2, 3},
                     {"Q2", 3, 4},
                     {"Q0", 4, 5}}});
  m["C6cD"] = spec({0, 2, 4}, {1, 3, 5},
                   {{{"Q0", 0, 1}, {"Q2", 1, 0}},
                    {{"Q0", 2, 3}, {"Q2", 3, 2}},
                    {{"Q0", 4, 5}, {"Q2", 5, 4}}});
  m["C6cCD"] = spec({0, 2, 4}, {1, 3, 5},
                    {{{"Q2", 3, 0}, {"Q0", 0, 1}, {"Q2", 1, 2}, {"Q0", 2, 3}},
                     {{"Q0", 4, 5}, {"Q2", 5, 4}}});
  return m;
}

char const *const kTraceNames[SLAPH_TR_KINDS] = {
    "trQ1", "trQ1Q1", "trQ0Q2", "trQ1Q1Q1", "trQ1Q0Q2", "trQ1Q1Q1Q1", "trQ2Q0Q2Q0",
    "trQ2Q0Q2Q0Q2Q0"};
int const kTraceArity[SLAPH_TR_KINDS] = {1, 2, 2, 3, 3, 4, 4, 6};

}  // namespace

std::map<std::string, DiagramSpec> const &diagram_specs() {
  static std::map<std::string, DiagramSpec> const specs = make_diagram_specs();
  return specs;
}

int trace_kind_from_name(std::string const &name) {
  for (int k = 0; k < SLAPH_TR_KINDS; ++k)
    if (name == kTraceNames[k]) return k;
  return -1;
}
char const *trace_kind_name(int kind) {
  return (kind >= 0 && kind < SLAPH_TR_KINDS) ? kTraceNames[kind] : nullptr;
}
int trace_kind_arity(int kind) {
  return (kind >= 0 && kind < SLAPH_TR_KINDS) ? kTraceArity[kind] : -1;
}

// src/global_data_input_handling_utils.cpp:133-157 and quark_check :159-192.
Quark make_quark(std::string const &s) {
  auto tok = split(s, ':');
  if (tok.size() != 9)
    throw std::runtime_error("the argument ('" + s +
                             "') for option 'quarks.quark' is invalid");
  Quark q;
  q.type = tok[0];
  q.number_of_rnd_vec = to_int(tok[1]);
  q.dilution_T = tok[2];
  q.number_of_dilution_T = to_int(tok[3]);
  q.dilution_E = tok[4];
  q.number_of_dilution_E = to_int(tok[5]);
  q.dilution_D = tok[6];
  q.number_of_dilution_D = to_int(tok[7]);
  q.path = tok[8];
  if (q.type != "u" && q.type != "d" && q.type != "s" && q.type != "c")
    throw std::runtime_error("quarks.quark.type must be u, d, s or c");
  if (q.number_of_rnd_vec < 1)
    throw std::runtime_error("quarks.quark.number_of_rnd_vec must be greater than 0");
  if (q.dilution_T != "TI" && q.dilution_T != "TB" && q.dilution_T != "TF")
    throw std::runtime_error("quarks.quark.dilution_T must be TI, TB, TF");
  if (q.number_of_dilution_T < 1)
    throw std::runtime_error(
        "quarks.quark.number_of_dilution_T must be greater than 0 and smaller than the "
        "temporal extent");
  if (q.dilution_E != "EI" && q.dilution_E != "EB" && q.dilution_E != "EF")
    throw std::runtime_error("quarks.quark.dilution_E must be EI, EB or EF");
  if (q.number_of_dilution_E < 1)
    throw std::runtime_error(
        "quarks.quark.number_of_dilution_E must be greater than 0 and smaller than "
        "number of eigen vectors");
  if (q.dilution_D != "DI" && q.dilution_D != "DB" && q.dilution_D != "DF")
    throw std::runtime_error("quarks.quark.dilution_D must be DI, DB or DF");
  if (q.number_of_dilution_D < 1 || q.number_of_dilution_D > 4)
    throw std::runtime_error(
        "quarks.quark.number_of_dilution_D must be greater than 0 and smaller than 5");
  return q;
}

// src/global_data_input_handling_utils.cpp:215-275.  Individual operators are
// separated by ':'; each is a '.'-separated list of g<int>, d0 | d<disp>,
// p(<x>,<y>,<z>) | p<n>[,<n>...].
Operators make_operator_list(std::string const &s) {
  Operators ops;
  for (auto const &op_t : split(s, ':')) {
    std::vector<int> gammas;
    std::vector<Displacement> disp_dirs;
    std::vector<std::vector<Vec3>> mom_vec;
    for (auto str : split(op_t, '.')) {
      if (str.compare(0, 1, "g") == 0) {
        gammas.push_back(to_int(str.substr(1)));
      } else if (str.compare(0, 1, "d") == 0) {
        if (str.compare(1, 1, "0") == 0) {
          disp_dirs.push_back(Displacement());
        } else if (str.compare(1, 1, "<") == 0 || str.compare(1, 1, ">") == 0) {
          auto tokens = split(str.substr(1), ',');
          disp_dirs.resize(tokens.size());
          for (size_t c = 0; c < tokens.size(); ++c) {
            Displacement d;
            for (auto const &dir : split(tokens[c], '|')) {
              if (dir.size() < 2)
                throw std::runtime_error(
                    "Something wrong with the displacement in the operator definition!");
              d.push_back({dir[0], dir[1]});
            }
            disp_dirs[c] = d;
          }
        } else {
          throw std::runtime_error(
              "Something wrong with the displacement in the operator definition!");
        }
      } else if (str.compare(0, 1, "p") == 0) {
        if (str.compare(1, 1, "(") == 0) {
          mom_vec.resize(1);
          mom_vec[0].push_back(vec3_from_string(str));
        } else {
          auto tokens = split(str.substr(1), ',');
          mom_vec.resize(tokens.size());
          for (size_t c = 0; c < tokens.size(); ++c)
            all_momenta_with_norm(to_int(tokens[c]), mom_vec[c]);
        }
      } else {
        throw std::runtime_error("There is something wrong with the operators!");
      }
    }
    for (auto const &moms : mom_vec)
      for (auto const &mom : moms)
        for (auto const &d : disp_dirs) ops.push_back({gammas, d, mom});
  }
  return ops;
}

// src/global_data_input_handling_utils.cpp:302-347.
CorrelatorSpec make_correlator(std::string const &s) {
  CorrelatorSpec c;
  for (auto t : split(s, ':')) {
    if (t.compare(0, 1, "C") == 0) {
      c.type = t;
    } else if (t.compare(0, 1, "Q") == 0) {
      c.quark_numbers.push_back(to_int(t.substr(1)));
    } else if (t.compare(0, 2, "Op") == 0) {
      c.operator_numbers.push_back(to_int(t.substr(2)));
    } else if (t.compare(0, 1, "G") == 0) {
      c.GEVP = t;
    } else if (t.compare(0, 1, "P") == 0) {
      if (t.compare(1, 1, "(") == 0) {
        c.tot_mom.push_back(vec3_from_string(t));
      } else {
        for (auto const &tok : split(t.substr(1), ','))
          all_momenta_with_norm(to_int(tok), c.tot_mom);
      }
    } else {
      throw std::runtime_error(
          "There is something wrong with the correlators in the input file!");
    }
  }
  return c;
}

std::string build_hdf5_dataset_name(std::string const &corr_type,
                                    std::vector<std::string> const &quark_types,
                                    std::vector<QuantumNumbers> const &qn) {
  std::string name = corr_type + "_";
  for (auto const &qt : quark_types) name += qt;
  for (auto const &op : qn) {
    name += "_p" + vec_to_string(op.momentum);
    name += ".d" + disp_to_string(op.displacement);
    name += ".g" + ints_to_string(op.gamma);
  }
  return name;
}

namespace {

// src/init_lookup_tables.cpp:42-163.  The sink cartesian product takes its
// lengths from the *source* vertices (:78-82); this is kept as is, since it
// decides which sink operators are reachable.
void quantum_numbers_of_correlator(CorrelatorSpec const &corr,
                                   std::vector<Operators> const &operator_list,
                                   std::vector<std::vector<QuantumNumbers>> &out,
                                   std::map<int, int> const &momentum_cutoff) {
  std::vector<Operators const *> qn_op;
  for (int op_number : corr.operator_numbers) {
    if (op_number < 0 || op_number >= static_cast<int>(operator_list.size())) {
      std::ostringstream oss;
      oss << "Operator with ID " << op_number
          << " which is used in [correlator_lists] is not defined. Please adjust your "
             "parameter file.";
      throw std::runtime_error(oss.str());
    }
    qn_op.push_back(&operator_list[op_number]);
  }
  auto const spec_it = diagram_specs().find(corr.type);
  if (spec_it == diagram_specs().end())
    throw std::runtime_error("Unknown diagram type '" + corr.type + "'");
  auto const &vertices = spec_it->second.vertices;
  auto op_at = [&](int vertex) -> Operators const & {
    if (vertex >= static_cast<int>(qn_op.size()))
      throw std::runtime_error("Too few operators given for correlator " + corr.type);
    return *qn_op[vertex];
  };

  std::vector<long> len_so, len_si;
  for (int v : vertices.first) len_so.push_back(static_cast<long>(op_at(v).size()));
  for (int v : vertices.first) len_si.push_back(static_cast<long>(op_at(v).size()));
  auto product_size = [](std::vector<long> const &l) {
    long n = 1;
    for (long x : l) n *= x;
    return n;
  };
  // CartesianProduct (include/CartesianProduct.hpp): first index fastest.
  auto combination = [](std::vector<long> const &l, long i) {
    std::vector<long> c(l.size());
    for (size_t j = 0; j < l.size(); ++j) {
      c[j] = i % l[j];
      i /= l[j];
    }
    return c;
  };

  size_t const n_so = vertices.first.size(), n_si = vertices.second.size();
  std::vector<QuantumNumbers> qn_so(n_so), qn_si(n_si), qn_all(n_so + n_si);
  long const n_prod_so = product_size(len_so), n_prod_si = product_size(len_si);
  for (long iso = 0; iso < n_prod_so; ++iso) {
    auto idx = combination(len_so, iso);
    for (size_t j = 0; j < n_so; ++j) {
      auto const &ops = op_at(vertices.first[j]);
      qn_so[j] = ops.at(idx[j]);
      qn_all[vertices.first[j]] = qn_so[j];
    }
    Vec3 p_so{0, 0, 0};
    int sum_norm_sq = 0;
    for (auto const &q : qn_so) {
      p_so = add(p_so, q.momentum);
      sum_norm_sq += norm2(q.momentum);
    }
    if (!corr.tot_mom.empty() &&
        std::find(corr.tot_mom.begin(), corr.tot_mom.end(), p_so) == corr.tot_mom.end())
      continue;
    auto cut = momentum_cutoff.find(norm2(p_so));
    if (cut == momentum_cutoff.end())
      throw std::runtime_error("map::at: no momentum cutoff for |P|^2 = " +
                               std::to_string(norm2(p_so)));
    if (sum_norm_sq > cut->second) continue;

    if (n_si == 0) {
      out.push_back(qn_so);
    } else {
      for (long isi = 0; isi < n_prod_si; ++isi) {
        auto jdx = combination(len_si, isi);
        for (size_t j = 0; j < n_si; ++j) {
          auto const &ops = op_at(vertices.second[j]);
          qn_si[j] = ops.at(jdx[j]);
          qn_all[vertices.second[j]] = qn_si[j];
        }
        Vec3 p_si{0, 0, 0};
        for (auto const &q : qn_si) p_si = add(p_si, q.momentum);
        if (p_so == neg(p_si)) out.push_back(qn_all);
      }
    }
  }
}

// src/init_lookup_tables.cpp:235-264.
void build_vdaggerv_lookup(std::vector<std::vector<QuantumNumbers>> const &qns,
                           std::vector<VdvQuantumNumbers> &lookup,
                           std::vector<std::vector<std::pair<int, bool>>> &vdv_indices) {
  for (auto const &qn_vec : qns) {
    std::vector<std::pair<int, bool>> row;
    for (auto const &qn : qn_vec) {
      auto it = std::find_if(lookup.begin(), lookup.end(), [&](VdvQuantumNumbers const &v) {
        return v.displacement == qn.displacement &&
               (v.momentum == qn.momentum || v.momentum == neg(qn.momentum));
      });
      if (it == lookup.end()) {
        lookup.push_back({static_cast<int>(lookup.size()), qn.momentum, qn.displacement});
        row.emplace_back(static_cast<int>(lookup.size()) - 1, false);
      } else {
        bool const dagger =
            qn.momentum != Vec3{0, 0, 0} && it->momentum == neg(qn.momentum);
        row.emplace_back(static_cast<int>(it - lookup.begin()), dagger);
      }
    }
    vdv_indices.push_back(row);
  }
}

// src/init_lookup_tables.cpp:294-335.
std::vector<std::pair<int, int>> rnd_vec_ids(std::vector<Quark> const &quarks, int id_q1,
                                             int id_q2, bool is_loop) {
  if (id_q1 < 0 || id_q2 < 0 || id_q1 >= static_cast<int>(quarks.size()) ||
      id_q2 >= static_cast<int>(quarks.size()))
    throw std::runtime_error("Quark index out of range in correlator definition");
  int s1 = 0, s2 = 0;
  for (int i = 0; i < id_q1; ++i) s1 += quarks[i].number_of_rnd_vec;
  for (int i = 0; i < id_q2; ++i) s2 += quarks[i].number_of_rnd_vec;
  int const e1 = s1 + quarks[id_q1].number_of_rnd_vec;
  int const e2 = s2 + quarks[id_q2].number_of_rnd_vec;
  if (quarks[id_q1].number_of_rnd_vec < 1 || quarks[id_q2].number_of_rnd_vec < 1 ||
      (id_q1 == id_q2 && quarks[id_q1].number_of_rnd_vec < 2))
    throw std::runtime_error(
        "There are not enough random vectors for charged correlators");
  std::vector<std::pair<int, int>> out;
  if (!is_loop) {
    for (int i = s1; i < e1; ++i)
      for (int j = s2; j < e2; ++j)
        if (i != j) out.emplace_back(i, j);
  } else {
    for (int i = s1; i < e1; ++i) out.emplace_back(i, i);
  }
  return out;
}

struct TraceRequestFactory {  // src/init_lookup_tables.cpp:370-393
  std::string name;
  std::vector<int> vertices;
  std::vector<Location> locations;
  TraceRequest make(std::vector<std::vector<int>> &tr_lookup,
                    std::vector<int> const &ql_ids) const {
    std::vector<int> ids;
    for (int v : vertices) ids.push_back(ql_ids.at(v));
    int const tr_id = unique_push_back(tr_lookup, ids);
    return {name, tr_id, locations};
  }
};

// src/init_lookup_tables.cpp:397-462.
std::vector<TraceRequestFactory> make_trace_request_factories(DiagramSpec const &spec) {
  std::vector<TraceRequestFactory> f;
  for (auto const &trace : spec.traces) {
    std::string name = "tr";
    std::vector<int> vertices;
    int previous_q2 = -1;
    for (auto const &ql : trace) {
      name += ql.name;
      vertices.push_back(ql.q1);
      if (previous_q2 >= 0 && ql.q1 != previous_q2)
        throw std::runtime_error(
            "Inconsistency in quark line definitions of the diagrams. This is not a "
            "user error but needs to be fixed by a developer.");
      previous_q2 = ql.q2;
    }
    if (vertices[0] != trace.back().q2)
      throw std::runtime_error(
          "This trace does not end with the vertex that it started with. This "
          "inconsistency needs to be fixed by a developer.");
    std::vector<Location> locations;
    for (int v : vertices) {
      auto const &so = spec.vertices.first, &si = spec.vertices.second;
      if (std::find(so.begin(), so.end(), v) != so.end())
        locations.push_back(Location::source);
      else if (std::find(si.begin(), si.end(), v) != si.end())
        locations.push_back(Location::sink);
      else
        throw std::runtime_error(
            "The vertex was not found in the list, this needs to be fixed by a "
            "developer.");
    }
    f.push_back({name, vertices, locations});
  }
  return f;
}

}  // namespace

// src/init_lookup_tables.cpp:470-556.
void init_lookup_tables(GlobalData &gd) {
  for (char const *q : {"Q0", "Q1", "Q2"}) gd.quarkline_lookuptable[q];
  for (int k = 0; k < SLAPH_TR_KINDS; ++k) gd.trace_indices_map[kTraceNames[k]];

  for (auto const &corr : gd.correlator_list) {
    std::vector<std::vector<QuantumNumbers>> qns;
    quantum_numbers_of_correlator(corr, gd.operator_list, qns, gd.momentum_cutoff);

    std::vector<std::string> quark_types;
    for (int id : corr.quark_numbers) {
      if (id < 0 || id >= static_cast<int>(gd.quarks.size()))
        throw std::runtime_error("Quark index out of range in correlator definition");
      quark_types.push_back(gd.quarks[id].type);
    }

    std::vector<std::vector<std::pair<int, bool>>> vdv_indices;
    build_vdaggerv_lookup(qns, gd.operator_lookuptable.vdaggerv_lookup, vdv_indices);

    auto const &spec = diagram_specs().at(corr.type);
    size_t ql_size = 0;
    for (auto const &tr : spec.traces) ql_size += tr.size();
    std::vector<int> ql_ids(ql_size, 0);
    auto const factories = make_trace_request_factories(spec);

    for (size_t d = 0; d < qns.size(); ++d) {
      for (auto const &trace_spec : spec.traces) {
        for (auto const &ql : trace_spec) {
          if (ql.q1 >= static_cast<int>(corr.quark_numbers.size()) ||
              ql.q2 >= static_cast<int>(corr.quark_numbers.size()))
            throw std::runtime_error("Too few quarks given for correlator " + corr.type);
          auto const ric = rnd_vec_ids(gd.quarks, corr.quark_numbers[ql.q1],
                                       corr.quark_numbers[ql.q2], ql.is_loop());
          // build_Quarkline_lookup_one_qn, src/init_lookup_tables.cpp:348-368:
          // the operator of a quark line is the one at its q2 vertex.
          auto const &qn = qns[d][ql.q2];
          FactorIndex cand{vdv_indices[d][ql.q2].first, vdv_indices[d][ql.q2].second,
                           qn.gamma, ric};
          ql_ids[ql.q2] = unique_push_back(gd.quarkline_lookuptable[ql.name], cand);
        }
      }
      CorrelatorRequest req;
      req.hdf5_dataset_name = build_hdf5_dataset_name(corr.type, quark_types, qns[d]);
      for (auto const &f : factories)
        req.trace_requests.push_back(f.make(gd.trace_indices_map[f.name], ql_ids));
      unique_push_back(gd.correlator_requests_map[corr.type], req);
    }
  }

  bool found = false;
  for (auto const &op : gd.operator_lookuptable.vdaggerv_lookup)
    if (op.momentum == Vec3{0, 0, 0} && op.displacement.empty()) {
      gd.operator_lookuptable.index_of_unity = op.id;
      found = true;
    }
  if (!found) gd.operator_lookuptable.index_of_unity = -1;
  gd.operator_lookuptable.need_gaugefield = false;
  for (auto const &op : gd.operator_lookuptable.vdaggerv_lookup)
    if (!op.displacement.empty()) {
      gd.operator_lookuptable.need_gaugefield = true;
      break;
    }
}

namespace {

// Options known to read_parameters (src/global_data.cpp:72-194).
enum class OptKind { Int, Long, Str, Dbl, List };
struct OptDef {
  char const *name;
  OptKind kind;
};
OptDef const kOptions[] = {
    {"nb_eigen_threads", OptKind::Long},
    {"output_path", OptKind::Str},
    {"path_config", OptKind::Str},
    {"lattice", OptKind::Str},
    {"Lt", OptKind::Int},
    {"Lx", OptKind::Int},
    {"Ly", OptKind::Int},
    {"Lz", OptKind::Int},
    {"alpha1", OptKind::Dbl},
    {"alpha2", OptKind::Dbl},
    {"iterations", OptKind::Long},
    {"number_of_eigen_vec", OptKind::Int},
    {"path_eigenvectors", OptKind::Str},
    {"name_eigenvectors", OptKind::Str},
    {"handling_vdaggerv", OptKind::Str},
    {"path_vdaggerv", OptKind::Str},
    {"quarks.quark", OptKind::List},
    {"operator_lists.operator_list", OptKind::List},
    {"correlator_lists.correlator_list", OptKind::List},
    {"start_config", OptKind::Int},
    {"end_config", OptKind::Int},
    {"delta_config", OptKind::Int},
    {"momentum_cutoff_0", OptKind::Int},
    {"single_time_slice_combination", OptKind::Int},
};

OptDef const *find_option(std::string const &name) {
  for (auto const &o : kOptions)
    if (name == o.name) return &o;
  return nullptr;
}

}  // namespace

void read_parameters(GlobalData &gd, std::string const &infile,
                     std::vector<std::string> const &args) {
  // Values given on the command line win over the config file; the config file
  // wins over defaults (boost::program_options store semantics).
  std::map<std::string, std::vector<std::string>> cli, cfg;
  for (size_t i = 0; i < args.size(); ++i) {
    std::string a = args[i];
    std::string key, value;
    if (a.rfind("--", 0) == 0) {
      a = a.substr(2);
      auto eq = a.find('=');
      if (eq != std::string::npos) {
        key = a.substr(0, eq);
        value = a.substr(eq + 1);
      } else {
        key = a;
        if (i + 1 >= args.size())
          throw std::runtime_error("the required argument for option '--" + key +
                                   "' is missing");
        value = args[++i];
      }
    } else {
      throw std::runtime_error("unrecognised command-line token '" + a + "'");
    }
    if (key == "input" || key == "i") continue;
    if (!find_option(key)) throw std::runtime_error("unrecognised option '--" + key + "'");
    cli[key].push_back(value);
  }

  std::ifstream ifs(infile);
  if (!ifs) throw std::runtime_error("CANNOT open input file: " + infile);
  std::string line, section;
  while (std::getline(ifs, line)) {
    auto hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    line = trim(line);
    if (line.empty()) continue;
    if (line.front() == '[') {
      if (line.back() != ']') throw std::runtime_error("invalid section line: " + line);
      section = trim(line.substr(1, line.size() - 2));
      continue;
    }
    auto eq = line.find('=');
    if (eq == std::string::npos)
      throw std::runtime_error("the options configuration file contains an invalid line '" +
                               line + "'");
    std::string key = trim(line.substr(0, eq));
    if (!section.empty()) key = section + "." + key;
    std::string value = trim(line.substr(eq + 1));
    OptDef const *opt = find_option(key);
    if (!opt) throw std::runtime_error("unrecognised option '" + key + "'");
    if (opt->kind != OptKind::List && cfg.count(key))
      throw std::runtime_error("option '" + key + "' cannot be specified more than once");
    cfg[key].push_back(value);
  }

  auto lookup = [&](std::string const &k) -> std::vector<std::string> const * {
    if (cli.count(k)) return &cli.at(k);
    if (cfg.count(k)) return &cfg.at(k);
    return nullptr;
  };
  auto get_int = [&](char const *k, int &dst) {
    if (auto v = lookup(k)) dst = to_int(v->back());
  };
  auto get_long = [&](char const *k, long &dst) {
    if (auto v = lookup(k)) dst = to_int(v->back());
  };
  auto get_str = [&](char const *k, std::string &dst) {
    if (auto v = lookup(k)) dst = v->back();
  };
  auto get_dbl = [&](char const *k, double &dst) {
    if (auto v = lookup(k)) dst = to_double(v->back());
  };
  get_long("nb_eigen_threads", gd.nb_eigen_threads);
  get_str("output_path", gd.path_output);
  get_str("path_config", gd.path_config);
  get_str("lattice", gd.name_lattice);
  get_int("Lt", gd.Lt);
  get_int("Lx", gd.Lx);
  get_int("Ly", gd.Ly);
  get_int("Lz", gd.Lz);
  get_dbl("alpha1", gd.alpha1);
  get_dbl("alpha2", gd.alpha2);
  get_long("iterations", gd.iterations);
  get_int("number_of_eigen_vec", gd.number_of_eigen_vec);
  get_str("path_eigenvectors", gd.path_eigenvectors);
  get_str("name_eigenvectors", gd.name_eigenvectors);
  get_str("handling_vdaggerv", gd.handling_vdaggerv);
  get_str("path_vdaggerv", gd.path_vdaggerv);
  get_int("start_config", gd.start_config);
  get_int("end_config", gd.end_config);
  get_int("delta_config", gd.delta_config);
  get_int("momentum_cutoff_0", gd.momentum_cutoff[0]);
  get_int("single_time_slice_combination", gd.single_time_slice_combination);

  // src/global_data_input_handling.cpp:19-148: checks of lattice, configs, nev.
  if (gd.Lt < 1)
    throw std::runtime_error(
        "input file error: option \"Lt\" is mendatory and its value must be an integer "
        "greater than 0!");
  if (gd.Lx < 1 || gd.Ly < 1 || gd.Lz < 1)
    throw std::runtime_error(
        "input file error: options \"Lx\", \"Ly\", \"Lz\" are mandatory and their values "
        "must be integers greater than 0!");
  if (gd.start_config < 0)
    throw std::runtime_error(
        "input file error: option \"start config\" is mandatory and its value must be an "
        "integer greater or equal 0!");
  if (gd.end_config < 0 || gd.end_config < gd.start_config)
    throw std::runtime_error(
        "input file error: option \"end_config\" is mandatory, its value must be an "
        "integer greater than 0, and it must be larger than start config!");
  if (gd.delta_config < 0)
    throw std::runtime_error(
        "input file error: option \"delta_config\" is mandatory and its value must be an "
        "integer greater than 0!");
  if (gd.number_of_eigen_vec < 1)
    throw std::runtime_error(
        "input file error: option \"number_of_eigen_vec\" is mandatory and its value must "
        "be an integer greater than 0!");

  gd.quarks.clear();
  if (auto v = lookup("quarks.quark"))
    for (auto const &s : *v) gd.quarks.push_back(make_quark(s));
  for (size_t i = 0; i < gd.quarks.size(); ++i) gd.quarks[i].id = static_cast<int>(i);
  gd.operator_list.clear();
  if (auto v = lookup("operator_lists.operator_list"))
    for (auto const &s : *v) gd.operator_list.push_back(make_operator_list(s));
  gd.correlator_list.clear();
  if (auto v = lookup("correlator_lists.correlator_list"))
    for (auto const &s : *v) gd.correlator_list.push_back(make_correlator(s));

  init_lookup_tables(gd);
}

namespace {
std::string fmt(char const *f, ...) {
  char buf[4096];
  va_list ap;
  va_start(ap, f);
  vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}
}  // namespace

// src/global_data_build_IO_names.cpp:7-85; the gauge configuration as
// GaugeField::read_gauge_field names it (src/GaugeField.cpp:765-766).
std::string io_name(GlobalData const &gd, int config, int which, int index) {
  if (which == 0)
    return fmt("%s/%s.%04d.", gd.path_eigenvectors.c_str(), gd.name_eigenvectors.c_str(),
               config);
  if (which == 3) return fmt("_cnfg%04d.h5", config);
  if (which == 4) return fmt("%s/conf.%04d", gd.path_config.c_str(), config);
  if (which != 1 && which != 2) throw std::runtime_error("io_name: unknown kind");
  int j = 0;
  for (auto const &q : gd.quarks) {
    for (int r = 0; r < q.number_of_rnd_vec; ++r, ++j) {
      if (j != index) continue;
      if (which == 2)
        return fmt("%s/cnfg%04d/rnd_vec_%02d/randomvector.rndvecnb%02d.%s.nbev%04d.%04d",
                   q.path.c_str(), config, r, r, q.type.c_str(), gd.number_of_eigen_vec,
                   config);
      return fmt(
          "%s/cnfg%04d/rnd_vec_%02d/"
          "perambulator.rndvecnb%02d.%s.Tso%c%04d.Vso%c%04d.Dso%c%1d.TsiF%04d.SsiF%04d."
          "DsiF4.CsiF3.smeared0.%05d",
          q.path.c_str(), config, r, r, q.type.c_str(), q.dilution_T.back(),
          gd.Lt / q.number_of_dilution_T, q.dilution_E.back(), q.number_of_dilution_E,
          q.dilution_D.back(), q.number_of_dilution_D, gd.Lt, gd.Lx * gd.Ly * gd.Lz,
          config);
    }
  }
  throw std::runtime_error("io_name: random vector index out of range");
}

FlatPlan::FlatPlan(GlobalData const &gd) {
  for (auto const &op : gd.operator_lookuptable.vdaggerv_lookup) {
    slaph_vdv_op o{};
    o.id = op.id;
    for (int i = 0; i < 3; ++i) o.momentum[i] = op.momentum[i];
    if (op.displacement.size() > SLAPH_MAX_DISP)
      throw std::runtime_error("displacement longer than SLAPH_MAX_DISP");
    o.n_disp = static_cast<int32_t>(op.displacement.size());
    for (size_t i = 0; i < op.displacement.size(); ++i) {
      o.disp[2 * i] = op.displacement[i].first;
      o.disp[2 * i + 1] = op.displacement[i].second;
    }
    vdv_.push_back(o);
  }
  plan_.n_vdv_ops = static_cast<int32_t>(vdv_.size());
  plan_.vdv_ops = vdv_.data();
  plan_.index_of_unity = gd.operator_lookuptable.index_of_unity;
  plan_.need_gaugefield = gd.operator_lookuptable.need_gaugefield ? 1 : 0;

  char const *qnames[3] = {"Q0", "Q1", "Q2"};
  for (int q = 0; q < 3; ++q) {
    auto it = gd.quarkline_lookuptable.find(qnames[q]);
    if (it == gd.quarkline_lookuptable.end()) continue;
    rnd_storage_[q].resize(it->second.size());
    for (size_t i = 0; i < it->second.size(); ++i) {
      auto const &fi = it->second[i];
      auto &st = rnd_storage_[q][i];
      for (auto const &p : fi.rnd_vec_ids) {
        st.push_back(p.first);
        st.push_back(p.second);
      }
    }
    for (size_t i = 0; i < it->second.size(); ++i) {
      auto const &fi = it->second[i];
      slaph_factor_index f{};
      f.id_vdaggerv = fi.id_vdaggerv;
      f.need_vdaggerv_daggering = fi.need_vdaggerv_daggering ? 1 : 0;
      f.gamma = fi.gamma.empty() ? 0 : fi.gamma[0];
      f.n_rnd_pairs = static_cast<int32_t>(fi.rnd_vec_ids.size());
      f.rnd_pairs = rnd_storage_[q][i].data();
      factors_[q].push_back(f);
    }
    plan_.n_factors[q] = static_cast<int32_t>(factors_[q].size());
    plan_.factors[q] = factors_[q].data();
  }

  for (int k = 0; k < SLAPH_TR_KINDS; ++k) {
    auto it = gd.trace_indices_map.find(kTraceNames[k]);
    int const ar = kTraceArity[k];
    if (it != gd.trace_indices_map.end())
      for (auto const &ids : it->second) {
        if (static_cast<int>(ids.size()) != ar)
          throw std::runtime_error("trace index arity mismatch");
        for (int x : ids) trace_ids_[k].push_back(x);
      }
    plan_.n_trace_ids[k] = static_cast<int32_t>(trace_ids_[k].size() / ar);
    plan_.trace_ql_ids[k] = trace_ids_[k].data();
  }

  size_t n_diag = 0, n_req = 0;
  for (auto const &d : gd.correlator_requests_map)
    if (!d.second.empty()) {
      ++n_diag;
      n_req += d.second.size();
    }
  names_.reserve(n_diag);
  dataset_names_.reserve(n_req);
  requests_.reserve(n_diag);
  for (auto const &d : gd.correlator_requests_map) {
    if (d.second.empty()) continue;
    names_.push_back(d.first);
    requests_.emplace_back();
    for (auto const &r : d.second) {
      slaph_correlator_request cr{};
      if (r.trace_requests.size() > 3)
        throw std::runtime_error("This many traces are not implemented yet.");
      cr.n_traces = static_cast<int32_t>(r.trace_requests.size());
      for (size_t i = 0; i < r.trace_requests.size(); ++i) {
        auto const &tr = r.trace_requests[i];
        cr.traces[i].kind = trace_kind_from_name(tr.tr_name);
        if (cr.traces[i].kind < 0) throw std::runtime_error("unknown trace " + tr.tr_name);
        cr.traces[i].tr_id = tr.tr_id;
        cr.traces[i].n_loc = static_cast<int32_t>(tr.locations.size());
        for (size_t l = 0; l < tr.locations.size() && l < 6; ++l)
          cr.traces[i].loc[l] = static_cast<int32_t>(tr.locations[l]);
      }
      dataset_names_.push_back(r.hdf5_dataset_name);
      cr.dataset_name = dataset_names_.back().c_str();
      requests_.back().push_back(cr);
    }
  }
  for (size_t i = 0; i < names_.size(); ++i) {
    slaph_diagram dg{};
    dg.name = names_[i].c_str();
    dg.n_requests = static_cast<int32_t>(requests_[i].size());
    dg.requests = requests_[i].data();
    diagrams_.push_back(dg);
  }
  plan_.n_diagrams = static_cast<int32_t>(diagrams_.size());
  plan_.diagrams = diagrams_.data();
}

}  // namespace slaph

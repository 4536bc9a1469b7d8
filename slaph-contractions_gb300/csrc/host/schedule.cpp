// Symbolic replay of contract(): builds the flat work lists of schedule.hpp.
#include "schedule.hpp"

#include <algorithm>
#include <climits>
#include <atomic>
#include <cstdlib>
#include <exception>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_set>

#include "capi_util.hpp"

namespace slaph {

namespace {

// A DilutedFactor without data: random-vector pair and used-index mask.
struct SymE {
  int32_t r1, r2;
  uint16_t used;
  bool operator<(SymE const &o) const {
    return std::tie(r1, r2, used) < std::tie(o.r1, o.r2, o.used);
  }
};

// Concrete list: entry e lives in matrix slot base + e.  Product slots are
// encoded as -(local + 1) until the factor slot count is final.  t: the
// timeslice of the list's first factor (of its left operand for a product).
struct ListRef {
  int32_t shape;
  int32_t base;
  int32_t level;
  int32_t t;
};

struct ProdTemplate {
  int32_t out_shape;
  std::vector<std::pair<int32_t, int32_t>> pairs;
};

char const *const kMulEmpty =
    "vector<DilutedFactor> operator*(vector<DilutedFactor>, vector<DilutedFactor>) has an "
    "empty result.";
char const *const kTrEmpty2 =
    "vector<DilutedTrace> factor_to_trace(vector<DilutedFactor>, vector<DilutedFactor>) has an "
    "empty result. Not enough random vectors?";
char const *const kTrEmpty1 =
    "vector<DilutedTrace> factor_to_trace(vector<DilutedFactor>) has an empty result.";
char const *const kIpEmpty =
    "compcomp_t inner_product(vector<DilutedTrace>, vector<DilutedTrace>) has an empty "
    "result. Not enough random vectors?";

inline uint64_t pack2(int64_t a, int64_t b) {
  return (static_cast<uint64_t>(static_cast<uint32_t>(a)) << 32) | static_cast<uint32_t>(b);
}

// Memo from 64-bit keys: open addressing with linear probing in a
// power-of-two table at most half full (the symbolic replay looks keys up
// some 10^8 times per plan; a node-based map spends most of that time in cache
// misses).
template <typename V>
class Memo64 {
 public:
  V const *find(uint64_t key) const {
    if (n_ == 0) return nullptr;
    for (size_t i = slot_of(key);; i = (i + 1) & mask_) {
      Slot const &s = slots_[i];
      if (!s.used) return nullptr;
      if (s.key == key) return &s.val;
    }
  }
  // Inserts a key that is not present.
  void emplace(uint64_t key, V const &val) {
    if (2 * (n_ + 1) > slots_.size()) grow();
    insert(key, val);
  }
  void clear() {
    if (n_ == 0) return;
    for (auto &s : slots_) s.used = false;
    n_ = 0;
  }

 private:
  struct Slot {
    uint64_t key;
    V val;
    bool used;
  };
  std::vector<Slot> slots_;
  size_t n_ = 0, mask_ = 0;

  size_t slot_of(uint64_t k) const {
    // 64-bit mixing (the finaliser of MurmurHash3)
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return static_cast<size_t>(k) & mask_;
  }
  void insert(uint64_t key, V const &val) {
    size_t i = slot_of(key);
    while (slots_[i].used) i = (i + 1) & mask_;
    slots_[i] = Slot{key, val, true};
    ++n_;
  }
  void grow() {
    std::vector<Slot> old;
    old.swap(slots_);
    slots_.assign(old.empty() ? 1024 : 2 * old.size(), Slot{0, V{}, false});
    mask_ = slots_.size() - 1;
    n_ = 0;
    for (auto const &s : old)
      if (s.used) insert(s.key, s.val);
  }
};

class Builder {
 public:
  Builder(slaph_dims const &d, slaph_plan const &p) : dims_(d), plan_(p) {
    s_.dims = d;
    s_.eds = 4 * d.dilE;
    s_.n_vdv = p.n_vdv_ops;
    block_size_ = d.dilT;
  }

  Schedule run(int single_block_pair) {
    int const Lt = dims_.Lt;
    int const nb = Lt / block_size_;
    int const n_bp = nb * (nb + 1) / 2;
    std::vector<int64_t> offset(plan_.n_diagrams);
    int64_t total = 0;
    for (int d = 0; d < plan_.n_diagrams; ++d) {
      offset[d] = total;
      total += plan_.diagrams[d].n_requests;
    }
    s_.n_outputs = total;
    // Per diagram, its requests' trace references numbered by (kind, trace
    // id, locations): equal references give the same trace list within a
    // slice pair, so each is resolved once per slice pair, at its first use
    // in request order (the order in which lists are created is unchanged).
    std::vector<std::vector<int32_t>> ref_of(plan_.n_diagrams);
    std::vector<int32_t> n_refs(plan_.n_diagrams, 0);
    for (int d = 0; d < plan_.n_diagrams; ++d) {
      auto const &dg = plan_.diagrams[d];
      std::map<std::array<int32_t, 9>, int32_t> ids;
      for (int i = 0; i < dg.n_requests; ++i) {
        auto const &req = dg.requests[i];
        if (req.n_traces < 1 || req.n_traces > 3) continue;  // rejected below
        for (int k = 0; k < req.n_traces; ++k) {
          auto const &r = req.traces[k];
          std::array<int32_t, 9> key{r.kind, r.tr_id, r.n_loc, 0, 0, 0, 0, 0, 0};
          for (int l = 0; l < std::min(std::max(r.n_loc, 0), 6); ++l) key[3 + l] = r.loc[l];
          ref_of[d].push_back(ids.emplace(key, static_cast<int32_t>(ids.size())).first->second);
        }
      }
      n_refs[d] = static_cast<int32_t>(ids.size());
    }
    for (int b = 0; b < n_bp; ++b) {
      if (single_block_pair >= 0 && b != single_block_pair) continue;
      begin_wave(b);
      auto const slices = slice_pairs(b, nb);
      w_.terms.reserve(static_cast<size_t>(total) * slices.size());
      tlist_memo_.resize(slices.size());
      for (int d = 0; d < plan_.n_diagrams; ++d) {
        auto const &dg = plan_.diagrams[d];
        std::vector<int32_t> ref_list(n_refs[d]);
        for (size_t spi = 0; spi < slices.size(); ++spi) {
          auto const &sp = slices[spi];
          int const dt = std::abs((sp.second - sp.first - Lt) % Lt);
          std::fill(ref_list.begin(), ref_list.end(), -1);
          size_t pos = 0;
          for (int i = 0; i < dg.n_requests; ++i) {
            auto const &req = dg.requests[i];
            if (req.n_traces < 1 || req.n_traces > 3)
              throw UnsupportedError("This many traces are not implemented yet.");
            Term t{};
            t.n = req.n_traces;
            for (int k = 0; k < req.n_traces; ++k) {
              int32_t &id = ref_list[ref_of[d][pos++]];
              if (id < 0) id = trace_list(req.traces[k], sp.first, sp.second, tlist_memo_[spi]);
              t.list[k] = id;
            }
            if (req.n_traces > 1) check_inner_product(t);
            t.out = static_cast<int32_t>(offset[d] + i);
            t.dt = dt;
            w_.terms.push_back(t);
          }
        }
      }
      end_wave();
    }
    finish();
    return std::move(s_);
  }

 private:
  slaph_dims dims_;
  slaph_plan const &plan_;
  Schedule s_;
  int block_size_;
  int32_t n_factor_slots_ = 0;

  std::vector<std::vector<SymE>> shapes_;
  std::map<std::vector<SymE>, int32_t> shape_ids_;
  Memo64<int32_t> fshape_memo_;     // (type, ql) -> shape
  Memo64<int32_t> ptemplate_memo_;  // (shapeL, shapeR) -> template
  std::vector<ProdTemplate> ptemplates_;
  Memo64<int32_t> tshape_memo_;     // (shapeL, shapeR|-1) -> trace shape
  std::vector<int32_t> tshape_ip_checked_;
  std::unordered_set<uint64_t> ip_checked_;  // shape tuples already checked

  Memo64<ListRef> flist_memo_;  // factor lists, global
  // product lists of the wave, by the timeslice of the left operand (the key
  // decides it; a slice pair's lookups stay within two small tables)
  std::vector<Memo64<ListRef>> plist_memo_;
  // trace lists of the wave, one memo per slice pair (a slice pair's lookups
  // stay within its own small table)
  std::vector<Memo64<int32_t>> tlist_memo_;
  std::vector<int32_t> list_shape_;                   // trace list -> trace shape (wave)
  std::map<std::tuple<int, int, int>, int32_t> q0m_memo_, q1r_memo_;
  std::map<std::tuple<int, int, int, int>, int32_t> q2m_memo_;

  Wave w_;
  int32_t wave_prod_slots_ = 0;
  std::vector<std::pair<int32_t, ProdInst>> wave_prods_;  // (level, product)

  int blk(int t) const { return t / block_size_; }

  // DilutionScheme::operator[] and BlockIterator (include/dilution-iterator.hpp:
  // 21-191, 306-356) for DilutionType::block.
  std::vector<std::pair<int, int>> slice_pairs(int i, int nb) const {
    int bsnk = 0, bsrc = 0;
    for (int j = 0; j < i; ++j) {
      ++bsnk;
      if (bsnk == nb) {
        ++bsrc;
        bsnk = bsrc;
      }
    }
    int const bs = block_size_;
    std::vector<std::pair<int, int>> out;
    for (int s = bsrc * bs; s < (bsrc + 1) * bs; ++s)
      for (int k = bsnk * bs; k < (bsnk + 1) * bs; ++k) out.emplace_back(s, k);
    if (bsrc != bsnk)
      for (int s = bsnk * bs; s < (bsnk + 1) * bs; ++s)
        for (int k = bsrc * bs; k < (bsrc + 1) * bs; ++k) out.emplace_back(s, k);
    return out;
  }

  void begin_wave(int b) {
    w_ = Wave{};
    w_.block_pair = b;
    wave_prod_slots_ = 0;
    wave_prods_.clear();
    plist_memo_.assign(static_cast<size_t>(dims_.Lt), Memo64<ListRef>{});
    tlist_memo_.clear();  // sized per wave by run()
    list_shape_.clear();
  }

  void end_wave() {
    std::stable_sort(wave_prods_.begin(), wave_prods_.end(),
                     [](auto const &x, auto const &y) { return x.first < y.first; });
    int32_t level = -1;
    for (size_t k = 0; k < wave_prods_.size(); ++k) {
      while (level < wave_prods_[k].first) {
        w_.prod_level_off.push_back(static_cast<int64_t>(k));
        ++level;
      }
      w_.prods.push_back(wave_prods_[k].second);
    }
    w_.prod_level_off.push_back(static_cast<int64_t>(wave_prods_.size()));
    w_.n_prod_slots = wave_prod_slots_;
    double const e = s_.eds;
    w_.flops_products = 8.0 * e * e * e * w_.prods.size();
    double tr2 = 0, tr1 = 0;
    for (auto const &l : w_.lists) {
      double const n = static_cast<double>(s_.shapes[l.shape].i.size());
      (l.b_base == INT32_MIN ? tr1 : tr2) += n;
    }
    w_.flops_traces = 8.0 * e * e * tr2 + 2.0 * e * tr1;
    w_.n_trace_entries = static_cast<int64_t>(tr1 + tr2);
    s_.waves.push_back(std::move(w_));
  }

  void finish() {
    s_.n_factor_slots = n_factor_slots_;
    auto fix = [&](int32_t slot) {
      return slot >= 0 ? slot : n_factor_slots_ + (-slot - 1);
    };
    for (auto &w : s_.waves) {
      for (auto &p : w.prods) {
        p.a = fix(p.a);
        p.b = fix(p.b);
        p.c = fix(p.c);
      }
      for (auto &l : w.lists) {
        l.a_base = fix(l.a_base);
        if (l.b_base != INT32_MIN) l.b_base = fix(l.b_base);
        else l.b_base = -1;
      }
    }
    // Waves are grouped independently, in parallel.
    {
      std::atomic<size_t> next{0};
      std::exception_ptr err;
      std::mutex mu;
      size_t const nw = s_.waves.size();
      unsigned const hw = std::max(1u, std::thread::hardware_concurrency());
      std::vector<std::thread> pool;
      for (unsigned k = 0; k < std::min<size_t>(hw, nw); ++k)
        pool.emplace_back([&] {
          for (size_t i; (i = next++) < nw;) {
            try {
              group_lists(s_.waves[i]);
            } catch (...) {
              std::lock_guard<std::mutex> g(mu);
              if (!err) err = std::current_exception();
            }
          }
        });
      for (auto &t : pool) t.join();
      if (err) std::rethrow_exception(err);
    }
    for (auto &w : s_.waves) {
      s_.n_unique_entries += unique_entries(w);
      s_.n_group_entries += w.n_group_entries;
      s_.max_prod_slots = std::max(s_.max_prod_slots, w.n_prod_slots);
      s_.max_values = std::max(s_.max_values, w.n_values);
      s_.max_terms = std::max<int64_t>(s_.max_terms, static_cast<int64_t>(w.terms.size()));
      s_.max_lists = std::max<int64_t>(s_.max_lists, static_cast<int64_t>(w.lists.size()));
      s_.flops_products += w.flops_products;
      s_.flops_traces += w.flops_traces;
      s_.n_terms += static_cast<int64_t>(w.terms.size());
      s_.n_trace_entries += w.n_trace_entries;
      s_.n_prods += static_cast<int64_t>(w.prods.size());
    }
    double const nev = dims_.nev, dilE = dims_.dilE;
    s_.flops_factors = 8.0 * (s_.q0m.size() * 4.0 * nev * nev + s_.q0.size() * 4.0 * nev * dilE +
                              s_.q1r.size() * 4.0 * nev * nev +
                              s_.q1.size() * 16.0 * dilE * dilE * nev +
                              s_.q2m.size() * 16.0 * dilE * nev * nev +
                              s_.q2.size() * 64.0 * dilE * dilE * nev);
  }

  int64_t unique_entries(Wave const &w) const {
    int64_t n = 0;
    for (int32_t l : w.unique_lists) n += static_cast<int64_t>(s_.shapes[w.lists[l].shape].i.size());
    return n;
  }

  // Merges lists with equal operands, finds the dense trace groups and lays
  // out the trace values: group values first (entry-major, B group, A group),
  // then the residual lists one after another.
  void group_lists(Wave &w) {
    int64_t const n = static_cast<int64_t>(w.lists.size());
    // Lists in order of (shape, a_base, b_base, index), sorted as compact
    // records (the keys next to the index, not behind it).
    struct ListKey {
      int32_t shape, a, b, k;
      bool operator<(ListKey const &o) const {
        return std::tie(shape, a, b, k) < std::tie(o.shape, o.a, o.b, o.k);
      }
    };
    std::vector<int32_t> ord(n);
    {
      std::vector<ListKey> keys(n);
      for (int64_t k = 0; k < n; ++k) {
        auto const &l = w.lists[k];
        keys[k] = {l.shape, l.a_base, l.b_base, static_cast<int32_t>(k)};
      }
      std::sort(keys.begin(), keys.end());
      for (int64_t p = 0; p < n; ++p) ord[p] = keys[p].k;
    }
    auto key = [&](int32_t k) {
      auto const &l = w.lists[k];
      return std::make_tuple(l.shape, l.a_base, l.b_base);
    };
    // canonical[k]: the lowest-numbered list with the operands of list k.
    std::vector<int32_t> canonical(n);
    std::vector<int32_t> uniq;  // canonical lists in key order
    for (int64_t p = 0; p < n; ++p) {
      if (p > 0 && key(ord[p]) == key(ord[p - 1])) {
        canonical[ord[p]] = canonical[ord[p - 1]];
      } else {
        canonical[ord[p]] = ord[p];
        uniq.push_back(ord[p]);
      }
    }
    // Runs of equal (shape, a_base) among the two-matrix lists: the B set of
    // each A group, in increasing b_base.  A groups with equal (shape, B set)
    // form a complete bipartite set.
    struct Run {
      int32_t shape, a;
      int64_t begin, end;  // into uniq
      uint64_t hash;
    };
    std::vector<Run> runs;
    for (int64_t p = 0; p < static_cast<int64_t>(uniq.size());) {
      auto const &l = w.lists[uniq[p]];
      int64_t q = p;
      uint64_t h = 1469598103934665603ULL;
      while (q < static_cast<int64_t>(uniq.size()) && w.lists[uniq[q]].shape == l.shape &&
             w.lists[uniq[q]].a_base == l.a_base) {
        h = (h ^ static_cast<uint32_t>(w.lists[uniq[q]].b_base)) * 1099511628211ULL;
        ++q;
      }
      if (l.b_base >= 0) runs.push_back({l.shape, l.a_base, p, q, h});
      p = q;
    }
    auto same_set = [&](Run const &x, Run const &y) {
      if (x.shape != y.shape || x.end - x.begin != y.end - y.begin || x.hash != y.hash)
        return false;
      for (int64_t u = 0; u < x.end - x.begin; ++u)
        if (w.lists[uniq[x.begin + u]].b_base != w.lists[uniq[y.begin + u]].b_base)
          return false;
      return true;
    };
    // Runs in order of (shape, B-set hash, B-set size), ties in run order.
    struct RunKey {
      int32_t shape, k;
      uint64_t hash;
      int64_t size;
      bool operator<(RunKey const &o) const {
        return std::tie(shape, hash, size, k) < std::tie(o.shape, o.hash, o.size, o.k);
      }
    };
    std::vector<int32_t> run_ord(runs.size());
    {
      std::vector<RunKey> keys(runs.size());
      for (size_t k = 0; k < runs.size(); ++k)
        keys[k] = {runs[k].shape, static_cast<int32_t>(k), runs[k].hash,
                   runs[k].end - runs[k].begin};
      std::sort(keys.begin(), keys.end());
      for (size_t p = 0; p < keys.size(); ++p) run_ord[p] = keys[p].k;
    }
    std::vector<char> in_group(n, 0);
    w.groups.clear();
    w.group_bases.clear();
    int64_t val = 0;
    for (size_t p = 0; p < run_ord.size();) {
      size_t q = p + 1;
      while (q < run_ord.size() && same_set(runs[run_ord[p]], runs[run_ord[q]])) ++q;
      Run const &r0 = runs[run_ord[p]];
      int32_t const n_a = static_cast<int32_t>(q - p);
      int32_t const n_b = static_cast<int32_t>(r0.end - r0.begin);
      if (n_a >= kMinGroupA && n_b >= kMinGroupB) {
        TraceGroup g{};
        g.shape = r0.shape;
        g.n_a = n_a;
        g.n_b = n_b;
        g.a_off = static_cast<int64_t>(w.group_bases.size());
        std::vector<int32_t> members(run_ord.begin() + p, run_ord.begin() + q);
        std::sort(members.begin(), members.end(),
                  [&](int32_t x, int32_t y) { return runs[x].a < runs[y].a; });
        for (int32_t m : members) w.group_bases.push_back(runs[m].a);
        g.b_off = static_cast<int64_t>(w.group_bases.size());
        for (int64_t u = r0.begin; u < r0.end; ++u)
          w.group_bases.push_back(w.lists[uniq[u]].b_base);
        g.val_base = val;
        int64_t const n_e = static_cast<int64_t>(s_.shapes[g.shape].i.size());
        int64_t const plane = static_cast<int64_t>(n_a) * n_b;
        for (int32_t ia = 0; ia < n_a; ++ia) {
          Run const &r = runs[members[ia]];
          for (int64_t u = r.begin; u < r.end; ++u) {
            auto &l = w.lists[uniq[u]];
            l.val_off = val + (u - r.begin) * n_a + ia;
            l.stride = static_cast<int32_t>(plane);
            in_group[uniq[u]] = 1;
          }
        }
        val += n_e * plane;
        w.n_group_entries += n_e * plane;
        w.groups.push_back(g);
      }
      p = q;
    }
    w.n_group_values = val;
    w.unique_lists.clear();
    w.residual_lists.clear();
    for (int64_t k = 0; k < n; ++k) {
      if (canonical[k] != k) continue;
      w.unique_lists.push_back(static_cast<int32_t>(k));
      if (in_group[k]) continue;
      w.residual_lists.push_back(static_cast<int32_t>(k));
      auto &l = w.lists[k];
      l.val_off = val;
      l.stride = 1;
      val += static_cast<int64_t>(s_.shapes[l.shape].i.size());
    }
    for (int64_t k = 0; k < n; ++k)
      if (canonical[k] != k) {
        w.lists[k].val_off = w.lists[canonical[k]].val_off;
        w.lists[k].stride = w.lists[canonical[k]].stride;
      }
    w.n_values = val;
  }

  slaph_factor_index const &op(int type, int ql) const {
    if (ql < 0 || ql >= plan_.n_factors[type])
      throw ArgError("quark line index out of range in trace lookup");
    return plan_.factors[type][ql];
  }

  int32_t vdv_code(slaph_factor_index const &o) const {
    if (o.id_vdaggerv < 0 || o.id_vdaggerv >= plan_.n_vdv_ops)
      throw ArgError("VdaggerV id out of range");
    if (o.gamma < 0 || o.gamma > 15) throw ArgError("gamma index out of range");
    return 2 * o.id_vdaggerv + (o.need_vdaggerv_daggering ? 1 : 0);
  }

  int32_t shape_id(std::vector<SymE> const &v) {
    auto it = shape_ids_.find(v);
    if (it != shape_ids_.end()) return it->second;
    int32_t const id = static_cast<int32_t>(shapes_.size());
    shapes_.push_back(v);
    shape_ids_.emplace(v, id);
    return id;
  }

  template <typename K, typename V>
  int32_t intern(std::map<K, int32_t> &memo, K const &key, std::vector<V> &vec, V const &val) {
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
    int32_t const id = static_cast<int32_t>(vec.size());
    vec.push_back(val);
    memo.emplace(key, id);
    return id;
  }

  // DilutedFactorFactory<Q>::operator[](key).at(ql): one entry per rnd pair,
  // in the order of the lookup table (src/DilutedFactorFactory.cpp:65,131,202).
  ListRef factor_list(int type, int a, int b, int c, int ql) {
    uint64_t const key = (static_cast<uint64_t>(type) << 62) |
                         (static_cast<uint64_t>(a & 0x3FF) << 52) |
                         (static_cast<uint64_t>(b & 0x3FF) << 42) |
                         (static_cast<uint64_t>(c & 0x3FF) << 32) | static_cast<uint32_t>(ql);
    if (ListRef const *hit = flist_memo_.find(key)) return *hit;
    auto const &o = op(type, ql);
    int32_t const vdv = vdv_code(o);
    int32_t const base = n_factor_slots_;
    std::vector<SymE> entries;
    for (int k = 0; k < o.n_rnd_pairs; ++k) {
      int const r1 = o.rnd_pairs[2 * k], r2 = o.rnd_pairs[2 * k + 1];
      if (r1 < 0 || r2 < 0 || r1 >= dims_.n_rnd || r2 >= dims_.n_rnd)
        throw ArgError("random vector index out of range");
      int32_t const slot = n_factor_slots_++;
      if (type == 0) {  // key {t}
        int32_t const m = intern(q0m_memo_, std::make_tuple(a, vdv, r2), s_.q0m, Q0MInst{a, vdv, r2});
        s_.q0.push_back({a, m, r1, o.gamma, slot});
      } else if (type == 1) {  // key {t, b}
        int32_t const r = intern(q1r_memo_, std::make_tuple(a, vdv, r1), s_.q1r, Q1RInst{a, vdv, r1});
        s_.q1.push_back({a, b, r, r2, o.gamma, slot});
      } else {  // key {b1, t, b2}: a = t, b = b1, c = b2
        int32_t const m =
            intern(q2m_memo_, std::make_tuple(a, b, r1, vdv), s_.q2m, Q2MInst{a, b, r1, vdv});
        s_.q2.push_back({a, c, m, r2, o.gamma, slot});
      }
      entries.push_back({r1, r2, 0});
    }
    uint64_t const skey = pack2(type, ql);
    int32_t shape;
    if (int32_t const *hit = fshape_memo_.find(skey)) {
      shape = *hit;
    } else {
      shape = shape_id(entries);
      fshape_memo_.emplace(skey, shape);
    }
    ListRef ref{shape, base, 0, a};
    flist_memo_.emplace(key, ref);
    return ref;
  }
  ListRef q0(int t, int ql) { return factor_list(0, t, 0, 0, ql); }
  ListRef q1(int t, int b, int ql) { return factor_list(1, t, b, 0, ql); }
  ListRef q2(int b1, int t, int b2, int ql) { return factor_list(2, t, b1, b2, ql); }

  // operator*(vector<DF>, vector<DF>), src/DilutedFactor.cpp:6-51.
  ProdTemplate const &product_template(int32_t sl, int32_t sr) {
    uint64_t const key = pack2(sl, sr);
    if (int32_t const *hit = ptemplate_memo_.find(key)) return ptemplates_[*hit];
    ProdTemplate t;
    std::vector<SymE> out;
    auto const &L = shapes_[sl];
    auto const &R = shapes_[sr];
    for (size_t x = 0; x < L.size(); ++x)
      for (size_t y = 0; y < R.size(); ++y) {
        if (!(L[x].r2 == R[y].r1 && L[x].r1 != R[y].r2)) continue;
        if ((L[x].used & R[y].used) != 0u) continue;
        t.pairs.emplace_back(static_cast<int32_t>(x), static_cast<int32_t>(y));
        out.push_back({L[x].r1, R[y].r2,
                       static_cast<uint16_t>(L[x].used | R[y].used | (1u << L[x].r2))});
      }
    if (out.empty()) throw EmptyError(kMulEmpty);
    t.out_shape = shape_id(out);
    int32_t const id = static_cast<int32_t>(ptemplates_.size());
    ptemplates_.push_back(std::move(t));
    ptemplate_memo_.emplace(key, id);
    return ptemplates_[id];
  }

  // multiply<1,1> memo (include/DilutedFactor.hpp:164-187), per wave.
  ListRef multiply(ListRef const &l, ListRef const &r) {
    uint64_t const key = pack2(l.base, r.base);
    Memo64<ListRef> &memo = plist_memo_[static_cast<size_t>(l.t)];
    if (ListRef const *hit = memo.find(key)) return *hit;
    ProdTemplate const &t = product_template(l.shape, r.shape);
    int32_t const level = std::max(l.level, r.level) + 1;
    int32_t const base = -(wave_prod_slots_ + 1);
    for (auto const &pr : t.pairs) {
      int32_t const slot = -(wave_prod_slots_ + 1);
      ++wave_prod_slots_;
      int32_t const a = l.base >= 0 ? l.base + pr.first : l.base - pr.first;
      int32_t const b = r.base >= 0 ? r.base + pr.second : r.base - pr.second;
      wave_prods_.push_back({level, ProdInst{a, b, slot}});
    }
    ListRef ref{t.out_shape, base, level, l.t};
    memo.emplace(key, ref);
    return ref;
  }

  // factor_to_trace(L, R) / factor_to_trace(F), src/DilutedTrace.cpp:84-165.
  int32_t trace_shape(int32_t sl, int32_t sr) {
    uint64_t const key = pack2(sl, sr);
    if (int32_t const *hit = tshape_memo_.find(key)) return *hit;
    TraceShape ts;
    auto const &L = shapes_[sl];
    if (sr >= 0) {
      auto const &R = shapes_[sr];
      for (size_t x = 0; x < L.size(); ++x)
        for (size_t y = 0; y < R.size(); ++y) {
          if (!(L[x].r2 == R[y].r1 && L[x].r1 == R[y].r2)) continue;
          if ((L[x].used & R[y].used) != 0u) continue;
          ts.i.push_back(static_cast<int32_t>(x));
          ts.j.push_back(static_cast<int32_t>(y));
          ts.mask.push_back(static_cast<uint16_t>(L[x].used | R[y].used | (1u << L[x].r2) |
                                                  (1u << L[x].r1)));
        }
      if (ts.i.empty()) throw EmptyError(kTrEmpty2);
    } else {
      for (size_t x = 0; x < L.size(); ++x) {
        if (L[x].r1 != L[x].r2) continue;
        ts.i.push_back(static_cast<int32_t>(x));
        ts.j.push_back(-1);
        ts.mask.push_back(static_cast<uint16_t>(L[x].used | (1u << L[x].r1)));
      }
      if (ts.i.empty()) throw EmptyError(kTrEmpty1);
    }
    int32_t const id = static_cast<int32_t>(s_.shapes.size());
    s_.shapes.push_back(std::move(ts));
    tshape_memo_.emplace(key, id);
    return id;
  }

  int32_t new_list(int32_t shape, ListRef const &a, ListRef const *b) {
    TraceList tl;
    tl.shape = shape;
    tl.a_base = a.base;
    tl.b_base = b ? b->base : INT32_MIN;
    tl.stride = 1;
    tl.val_off = w_.n_values;
    w_.n_values += static_cast<int64_t>(s_.shapes[shape].i.size());
    w_.lists.push_back(tl);
    list_shape_.push_back(shape);
    return static_cast<int32_t>(w_.lists.size()) - 1;
  }
  int32_t to_trace(ListRef const &l, ListRef const &r) {
    return new_list(trace_shape(l.shape, r.shape), l, &r);
  }
  int32_t to_trace(ListRef const &f) { return new_list(trace_shape(f.shape, -1), f, nullptr); }

  // DilutedTrace*Factory::build for one trace id, src/DilutedTraceFactory.cpp.
  int32_t build_trace(int kind, int const *k, int const *c) {
    switch (kind) {
      case SLAPH_TR_Q1:
        return to_trace(q1(k[0], blk(k[0]), c[0]));
      case SLAPH_TR_Q1Q1:
        return to_trace(q1(k[0], blk(k[1]), c[0]), q1(k[1], blk(k[0]), c[1]));
      case SLAPH_TR_Q0Q2:
        return to_trace(q0(k[1], c[1]), q2(blk(k[1]), k[0], blk(k[1]), c[0]));
      case SLAPH_TR_Q1Q1Q1: {
        ListRef const p = multiply(q1(k[0], blk(k[1]), c[0]), q1(k[1], blk(k[2]), c[1]));
        return to_trace(p, q1(k[2], blk(k[0]), c[2]));
      }
      case SLAPH_TR_Q1Q0Q2: {
        ListRef const p = multiply(q0(k[0], c[2]), q2(blk(k[0]), k[0], blk(k[1]), c[0]));
        return to_trace(p, q1(k[1], blk(k[2]), c[1]));
      }
      case SLAPH_TR_Q1Q1Q1Q1: {
        ListRef const p1 = multiply(q1(k[0], blk(k[1]), c[0]), q1(k[1], blk(k[2]), c[1]));
        ListRef const p2 = multiply(q1(k[2], blk(k[3]), c[2]), q1(k[3], blk(k[0]), c[3]));
        return to_trace(p1, p2);
      }
      case SLAPH_TR_Q2Q0Q2Q0: {
        int const b0 = blk(k[0]), b2 = blk(k[2]);
        ListRef const p1 = multiply(q0(k[0], c[0]), q2(b0, k[1], b2, c[1]));
        ListRef const p2 = multiply(q0(k[2], c[2]), q2(b2, k[3], b0, c[3]));
        return to_trace(p1, p2);
      }
      case SLAPH_TR_Q2Q0Q2Q0Q2Q0: {
        int const b1 = blk(k[1]), b3 = blk(k[3]), b5 = blk(k[5]);
        ListRef p = multiply(q2(b5, k[0], b1, c[1]), q0(k[1], c[2]));
        p = multiply(p, q2(b1, k[2], b3, c[3]));
        p = multiply(p, q0(k[3], c[4]));
        p = multiply(p, q2(b3, k[4], b5, c[5]));
        return to_trace(p, q0(k[5], c[0]));
      }
      default:
        throw ArgError("unknown trace kind");
    }
  }

  int32_t trace_list(slaph_trace_request const &r, int src, int snk, Memo64<int32_t> &memo) {
    static int const arity[SLAPH_TR_KINDS] = {1, 2, 2, 3, 3, 4, 4, 6};
    if (r.kind < 0 || r.kind >= SLAPH_TR_KINDS) throw ArgError("unknown trace kind");
    if (r.tr_id < 0 || r.tr_id >= plan_.n_trace_ids[r.kind] || r.tr_id >= (1 << 24))
      throw ArgError("trace id out of range");
    if (r.n_loc != arity[r.kind]) throw ArgError("trace request location count mismatch");
    // The reference memoises by the tuple of times (include/DilutedTraceFactory.hpp:
    // 44-57); a pattern of source/sink locations gives that tuple from (src, snk).
    int pattern = 0;
    if (src != snk)
      for (int l = 0; l < r.n_loc; ++l) pattern |= (r.loc[l] ? 1 : 0) << l;
    uint64_t const key = (static_cast<uint64_t>(r.kind) << 61) |
                         (static_cast<uint64_t>(r.tr_id) << 37) |
                         (static_cast<uint64_t>(src & 0x3FF) << 27) |
                         (static_cast<uint64_t>(snk & 0x3FF) << 17) |
                         static_cast<uint64_t>(src == snk ? 0 : pattern);
    if (int32_t const *hit = memo.find(key)) return *hit;
    int k[6];
    for (int l = 0; l < r.n_loc; ++l) k[l] = r.loc[l] == 0 ? src : snk;
    int const *c = plan_.trace_ql_ids[r.kind] + static_cast<int64_t>(r.tr_id) * arity[r.kind];
    int32_t const id = build_trace(r.kind, k, c);
    memo.emplace(key, id);
    return id;
  }

  // inner_product must have at least one summand (src/DilutedTrace.cpp:37-41,
  // 75-79).  Masks depend only on the trace shapes, so the check is memoised.
  void check_inner_product(Term const &t) {
    int32_t key[3] = {0, 0, 0};
    for (int k = 0; k < t.n; ++k) key[k] = list_shape_[t.list[k]];
    if (key[0] >= (1 << 21) || key[1] >= (1 << 21) || key[2] >= (1 << 21))
      throw UnsupportedError("more than 2^21 trace shapes");
    uint64_t const packed = (static_cast<uint64_t>(t.n == 3 ? 1 : 0) << 63) |
                            (static_cast<uint64_t>(key[0]) << 42) |
                            (static_cast<uint64_t>(key[1]) << 21) | static_cast<uint64_t>(key[2]);
    if (ip_checked_.count(packed)) return;
    auto const &a = s_.shapes[key[0]].mask;
    auto const &b = s_.shapes[key[1]].mask;
    bool any = false;
    if (t.n == 2) {
      for (auto x : a)
        for (auto y : b) any = any || (x & y) == 0;
    } else {
      auto const &c = s_.shapes[key[2]].mask;
      for (auto x : a)
        for (auto y : b)
          for (auto z : c) any = any || (x & y & z) == 0;
    }
    if (!any) throw EmptyError(kIpEmpty);
    ip_checked_.insert(packed);
  }
};

}  // namespace

Schedule build_schedule(slaph_dims const &dims, slaph_plan const &plan, int single_block_pair) {
  if (dims.Lt < 1 || dims.dilT < 1 || dims.Lt % dims.dilT != 0 || dims.dilE < 1 || dims.nev < 1)
    throw ArgError("invalid dims for the contraction schedule");
  if (dims.Lt > 1024) throw UnsupportedError("Lt above 1024 is not supported");
  if (dims.n_rnd > 16) throw UnsupportedError("at most 16 random vectors (16-bit used masks)");
  Builder b(dims, plan);
  return b.run(single_block_pair);
}

ProductPlan plan_products(ProdInst const *prods, int64_t n, int32_t eds) {
  ProductPlan pp;
  int32_t const per_group = eds > 0 && eds <= 64 ? std::max(1, 64 / eds) : 1;
  // left matrices (by first appearance) with their (right index, slot)
  // lists; right matrices numbered by first appearance
  std::map<int32_t, int32_t> lidx, ridx;
  std::vector<int32_t> l_slot;
  std::vector<std::vector<std::pair<int32_t, int32_t>>> lr;
  for (int64_t k = 0; k < n; ++k) {
    ProdInst const &pi = prods[k];
    auto li = lidx.emplace(pi.a, static_cast<int32_t>(l_slot.size()));
    if (li.second) {
      l_slot.push_back(pi.a);
      lr.emplace_back();
    }
    auto ri = ridx.emplace(pi.b, static_cast<int32_t>(pp.r_slots.size()));
    if (ri.second) pp.r_slots.push_back(pi.b);
    lr[li.first->second].push_back({ri.first->second, pi.c});
  }
  int32_t const n_l = static_cast<int32_t>(l_slot.size());
  std::vector<std::vector<int32_t>> inv(pp.r_slots.size());
  for (int32_t li = 0; li < n_l; ++li) {
    std::sort(lr[li].begin(), lr[li].end());
    for (auto const &rc : lr[li]) inv[rc.first].push_back(li);
  }
  std::vector<char> used(n_l, 0);
  std::vector<int32_t> cnt(n_l, 0), touched;
  for (int32_t li = 0; li < n_l; ++li) {
    if (used[li]) continue;
    std::vector<int32_t> mem{li};
    used[li] = 1;
    while (static_cast<int32_t>(mem.size()) < per_group) {
      touched.clear();
      for (int32_t m : mem)
        for (auto const &rc : lr[m])
          for (int32_t l2 : inv[rc.first])
            if (!used[l2] && cnt[l2]++ == 0) touched.push_back(l2);
      int32_t best = -1;
      for (int32_t l2 : touched)
        if (best < 0 || cnt[l2] > cnt[best] || (cnt[l2] == cnt[best] && l2 < best)) best = l2;
      for (int32_t l2 : touched) cnt[l2] = 0;
      if (best < 0) break;
      mem.push_back(best);
      used[best] = 1;
    }
    std::vector<int32_t> uni;
    for (int32_t m : mem)
      for (auto const &rc : lr[m]) uni.push_back(rc.first);
    std::sort(uni.begin(), uni.end());
    uni.erase(std::unique(uni.begin(), uni.end()), uni.end());
    ProductGroup g{};
    for (int x = 0; x < 4; ++x) g.l[x] = -1;
    g.n_l = static_cast<int32_t>(mem.size());
    for (int32_t x = 0; x < g.n_l; ++x) g.l[x] = l_slot[mem[x]];
    g.n_u = static_cast<int32_t>(uni.size());
    if (pp.u_list.size() + uni.size() > 0x7fffffffULL)
      throw UnsupportedError("product GEMM lists above 2^31");
    g.u_off = static_cast<int32_t>(pp.u_list.size());
    for (int32_t u : uni) {
      pp.u_list.push_back(u);
      for (int x = 0; x < 4; ++x) {
        int32_t slot = -1;
        if (x < g.n_l) {
          auto const &v = lr[mem[x]];
          auto it = std::lower_bound(v.begin(), v.end(), std::make_pair(u, INT32_MIN));
          if (it != v.end() && it->first == u) slot = it->second;
        }
        pp.out_tab.push_back(slot);
      }
    }
    pp.n_tiles += (static_cast<int64_t>(eds) * g.n_u + 79) / 80;
    pp.groups.push_back(g);
  }
  return pp;
}

}  // namespace slaph

// C ABI of the host search driver (include/rils_rols_host.h).
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>

#include "../../../include/rils_rols_gb300.h"
#include "../../../include/rils_rols_host.h"
#include "../common/error.h"
#include "encode.h"
#include "parallel.h"
#include "search.h"

struct rrh_model {
  rrh::Search search;
  rrg_context* ctx = nullptr;  // owned; created on first use of the device backend
  bool graph = false;          // device rounds as CUDA graphs (rrh_set_graph)
  bool column_cache = true;    // factor columns kept across rounds (rrh_set_column_cache)
  rrh_model(bool c, int mfc, int ms, double cp, int mc, double ss, bool v, int rs) : search(c, mfc, ms, cp, mc, ss, v, rs) {}
  ~rrh_model() {
    if (ctx) rrg_context_destroy(ctx);
  }
};

namespace {

// ---- default backend: the device path of include/rils_rols_gb300.h ----
void* dev_dataset_create(void* self, const double* X, const double* y, int64_t n, int32_t d) {
  rrh_model* m = static_cast<rrh_model*>(self);
  if (!m->ctx) {
    if (rrg_context_create(0, &m->ctx) != RRG_OK) return nullptr;
    if (m->graph) rrg_context_set_graph(m->ctx, 1);
    if (!m->column_cache) rrg_context_set_column_cache(m->ctx, 0);
  }
  rrg_dataset* ds = nullptr;
  if (rrg_dataset_create(m->ctx, X, y, n, d, &ds) != RRG_OK) return nullptr;
  return ds;
}
int32_t dev_eval(void* ds, const rrg_batch* b, int32_t p, rrg_result* r, double* c) {
  return rrg_eval(static_cast<rrg_dataset*>(ds), b, p, r, c);
}
int32_t dev_predict(void* ds, const rrg_batch* b, double* v) { return rrg_predict(static_cast<rrg_dataset*>(ds), b, v); }
void dev_dataset_destroy(void* ds) { rrg_dataset_destroy(static_cast<rrg_dataset*>(ds)); }

rrh_backend device_backend(rrh_model* m) {
  rrh_backend be;
  be.self = m;
  be.dataset_create = dev_dataset_create;
  be.eval = dev_eval;
  be.predict = dev_predict;
  be.dataset_destroy = dev_dataset_destroy;
  return be;
}

int32_t put(const std::string& s, char* out, int32_t cap) {
  if ((int64_t)s.size() + 1 > cap) return -(int32_t)(s.size() + 1);
  std::memcpy(out, s.c_str(), s.size() + 1);
  return (int32_t)s.size();
}

template <typename F>
int32_t guarded(F&& f) {
  try {
    return f();
  } catch (const std::exception& e) {
    rrc::set_error(e.what());
    return RRG_E_INVALID;
  }
}

rrh::BatchBuilder g_encoded;  // holds the last rrh_encode result

}  // namespace

extern "C" {

rrh_model* rrh_create(int32_t classification, int32_t max_fit_calls, int32_t max_seconds, double complexity_penalty,
                      int32_t max_complexity, double sample_size, int32_t verbose, int32_t random_state) {
  try {
    rrh_model* m = new rrh_model(classification != 0, max_fit_calls, max_seconds, complexity_penalty, max_complexity,
                                 sample_size, verbose != 0, random_state);
    m->search.set_backend(device_backend(m));
    return m;
  } catch (const std::exception& e) {
    rrc::set_error(e.what());
    return nullptr;
  }
}

void rrh_destroy(rrh_model* m) { delete m; }

int32_t rrh_set_backend(rrh_model* m, const rrh_backend* be) {
  if (!m) return RRG_E_INVALID;
  m->search.set_backend(be ? *be : device_backend(m));
  return RRG_OK;
}

int32_t rrh_set_graph(rrh_model* m, int32_t on) {
  if (!m) return RRG_E_INVALID;
  m->graph = on != 0;
  return m->ctx ? rrg_context_set_graph(m->ctx, on) : RRG_OK;
}

int32_t rrh_set_column_cache(rrh_model* m, int32_t on) {
  if (!m) return RRG_E_INVALID;
  m->column_cache = on != 0;
  return m->ctx ? rrg_context_set_column_cache(m->ctx, on) : RRG_OK;
}

int32_t rrh_set_precision(rrh_model* m, int32_t p) {
  if (!m || (p != RRG_PLAIN_FP64 && p != RRG_MIXED && p != RRG_MIXED_CERTIFIED)) return RRG_E_INVALID;
  m->search.set_precision(p);
  return RRG_OK;
}

int32_t rrh_fit(rrh_model* m, const double* X, const double* y, int32_t n, int32_t d) {
  if (!m || !X || !y || n <= 0 || d <= 0) {
    rrc::set_error("rrh_fit: invalid arguments");
    return RRG_E_INVALID;
  }
  return guarded([&] {
    m->search.fit(X, y, n, d);
    return (int32_t)RRG_OK;
  });
}

int32_t rrh_predict(rrh_model* m, const double* X, int32_t n, int32_t d, double* out) {
  if (!m || !X || !out || n <= 0 || d <= 0) {
    rrc::set_error("rrh_predict: invalid arguments");
    return RRG_E_INVALID;
  }
  return guarded([&] {
    m->search.predict(X, n, d, out);
    return (int32_t)RRG_OK;
  });
}

int32_t rrh_model_string(const rrh_model* m, char* buf, int32_t cap) { return put(m->search.model_string(), buf, cap); }
int32_t rrh_model_prefix(const rrh_model* m, char* buf, int32_t cap) { return put(m->search.model_prefix(), buf, cap); }
double rrh_best_time(const rrh_model* m) { return m->search.best_time(); }
double rrh_total_time(const rrh_model* m) { return m->search.total_time(); }
int32_t rrh_fit_calls(const rrh_model* m) { return m->search.fit_calls(); }
int64_t rrh_counter(const rrh_model* m, int32_t which) { return m->search.counter(which); }

int32_t rrh_candidates(const char* tree, int32_t local_search, int32_t d, int32_t classification, char* out,
                       int32_t cap) {
  return guarded([&] {
    rrh::CandidateGen g;
    std::vector<int> feats(d);
    for (int i = 0; i < d; ++i) feats[i] = i;
    g.setup_nodes(feats, classification != 0);
    auto c = g.all_candidates(rrh::from_prefix(tree), local_search != 0);
    std::string s;
    for (auto& f : c) s += rrh::to_string(f) + "\t" + rrh::to_prefix(f) + "\n";
    return put(s, out, cap);
  });
}

int32_t rrh_rewrite(const char* tree, int32_t what, char* out, int32_t cap) {
  return guarded([&] {
    rrh::Arena a;
    rrh::Flat f = rrh::from_prefix(tree);
    if (what == 5) {
      std::string s;
      for (auto& g : rrh::tune_factors(f, a)) s += rrh::to_string(g) + "\t" + rrh::to_prefix(g) + "\n";
      return put(s, out, cap);
    }
    rrh::Node* t = rrh::thaw(f, a);
    if (what == 1) rrh::expand(t, a);
    if (what == 2) rrh::simplify(t);
    if (what == 3) rrh::normalize_factor_constants(t, rrh::NONE, false);
    if (what == 4) {
      int it_max = 5;
      while (it_max > 0) {
        const int sz = rrh::size(t);
        rrh::expand(t, a);
        rrh::normalize_factor_constants(t, rrh::NONE, false);
        rrh::simplify(t);
        if (rrh::size(t) == sz) break;
        it_max--;
      }
    }
    rrh::Flat g = rrh::freeze(t);
    return put(rrh::to_string(g) + "\t" + rrh::to_prefix(g) + "\t" + std::to_string(rrh::size(t)), out, cap);
  });
}

int32_t rrh_encode(const char* trees, int32_t mode, rrg_batch* out) {
  return guarded([&] {
    g_encoded.clear();
    std::istringstream in(trees);
    std::string line;
    std::vector<std::string> lines;
    while (std::getline(in, line))
      if (!line.empty()) lines.push_back(line);
    // parse and split on the host threads, encode in order
    std::vector<std::vector<rrh::Flat>> parts(lines.size());
    rrh::parallel_slices(lines.size(), 32, [&](size_t b, size_t e) {
      rrh::Arena a;
      for (size_t i = b; i < e; ++i) {
        rrh::Flat f = rrh::from_prefix(lines[i]);
        if (mode == RRG_TUNED) {
          a.reset();
          parts[i] = rrh::tune_factors(f, a);
        } else {
          parts[i] = std::vector<rrh::Flat>{f};
        }
      }
    });
    std::vector<const std::vector<rrh::Flat>*> ptrs(parts.size());
    for (size_t i = 0; i < parts.size(); ++i) ptrs[i] = &parts[i];
    g_encoded.add_all(ptrs, mode == RRG_TUNED ? RRG_TUNED : RRG_UNTUNED);
    *out = g_encoded.view();
    return (int32_t)RRG_OK;
  });
}

int32_t rrh_rebuild(const char* tree, const double* coefs, int32_t n_coefs, char* out, int32_t cap) {
  return guarded([&] {
    rrh::Arena a;
    auto factors = rrh::tune_factors(rrh::from_prefix(tree), a);
    if ((int)factors.size() + 1 != n_coefs) throw std::runtime_error("rrh_rebuild: coefficient count mismatch");
    rrh::Flat g = rrh::rebuild(factors, coefs);
    return put(rrh::to_string(g) + "\t" + rrh::to_prefix(g), out, cap);
  });
}

}  // extern "C"

// ORACLE (test infrastructure only): a harness around the reference's own,
// unmodified sources so that this repository can pin its oracle and its
// product against them.  Built by oracle/build_ref.sh into oracle/_ref/ from
// the sources where they lie (rils_rols_cpp/node.cpp, rils_rols_cpp.cpp),
// against the self-written Eigen subset in oracle/eigen_shim/.
//
// The reference's class keeps its hot-path members private
// (rils_rols_cpp/rils_rols_cpp.cpp:88-643); the harness re-opens them for
// testing by compiling the translation unit with `private` spelled `public`.
// Nothing here changes what the reference computes.
#include <algorithm>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <memory>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include <pybind11/pybind11.h>
#include <pybind11/numpy.h>

#define private public
#include "rils_rols_cpp.cpp"
#undef private

namespace {

using std::shared_ptr;
using std::string;
using std::vector;

struct Tok {
  const char* p;
};

node_type op_of(const string& s) {
  static const std::pair<const char*, node_type> tab[] = {
      {"add", node_type::PLUS},  {"sub", node_type::MINUS}, {"mul", node_type::MULTIPLY},
      {"div", node_type::DIVIDE}, {"sin", node_type::SIN},  {"cos", node_type::COS},
      {"ln", node_type::LN},     {"exp", node_type::EXP},   {"sqrt", node_type::SQRT},
      {"sqr", node_type::SQR},   {"pow", node_type::POW},   {"lt", node_type::LESS_THAN},
      {"gt", node_type::GREATER_THAN}, {"eq", node_type::EQUAL}, {"ne", node_type::NOT_EQUAL},
      {"min", node_type::MIN},   {"max", node_type::MAX}};
  for (auto& e : tab)
    if (s == e.first) return e.second;
  return node_type::NONE;
}

const char* name_of(node_type t) {
  switch (t) {
    case node_type::PLUS: return "add";
    case node_type::MINUS: return "sub";
    case node_type::MULTIPLY: return "mul";
    case node_type::DIVIDE: return "div";
    case node_type::SIN: return "sin";
    case node_type::COS: return "cos";
    case node_type::LN: return "ln";
    case node_type::EXP: return "exp";
    case node_type::SQRT: return "sqrt";
    case node_type::SQR: return "sqr";
    case node_type::POW: return "pow";
    case node_type::LESS_THAN: return "lt";
    case node_type::GREATER_THAN: return "gt";
    case node_type::EQUAL: return "eq";
    case node_type::NOT_EQUAL: return "ne";
    case node_type::MIN: return "min";
    case node_type::MAX: return "max";
    default: return "?";
  }
}

// prefix form: tokens separated by single spaces; x<i> variable, c:<double> constant
shared_ptr<node> parse(std::istringstream& in) {
  string t;
  if (!(in >> t)) throw std::runtime_error("truncated tree");
  if (t[0] == 'x') return std::make_shared<node>(std::atoi(t.c_str() + 1));
  if (t.rfind("c:", 0) == 0) return std::make_shared<node>(std::strtod(t.c_str() + 2, nullptr));
  node_type ty = op_of(t);
  if (ty == node_type::NONE) throw std::runtime_error("bad token " + t);
  auto n = std::make_shared<node>(ty);
  n->set_left(parse(in));
  if (get_arity(ty) == 2) n->set_right(parse(in));
  return n;
}

shared_ptr<node> parse_tree(const char* s) {
  std::istringstream in(s);
  return parse(in);
}

void emit_prefix(const node* n, string& out) {
  char buf[64];
  if (!out.empty()) out += ' ';
  if (n->get_type() == node_type::VAR) {
    std::snprintf(buf, sizeof buf, "x%d", n->get_var_index());
    out += buf;
  } else if (n->get_type() == node_type::CONST) {
    std::snprintf(buf, sizeof buf, "c:%.17g", n->get_const_value());
    out += buf;
  } else {
    out += name_of(n->get_type());
    emit_prefix(n->get_left(), out);
    if (n->get_arity() == 2) emit_prefix(n->get_right(), out);
  }
}

int put(const string& s, char* out, int cap) {
  if ((int)s.size() + 1 > cap) return -(int)s.size() - 1;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return (int)s.size();
}

vector<Eigen::ArrayXd> cols_of(const double* Xcol, int n, int d) {
  vector<Eigen::ArrayXd> X(d);
  for (int j = 0; j < d; ++j) {
    X[j].resize(n);
    for (int i = 0; i < n; ++i) X[j][i] = Xcol[(size_t)j * n + i];
  }
  return X;
}

Eigen::ArrayXd arr_of(const double* y, int n) {
  Eigen::ArrayXd a(n);
  for (int i = 0; i < n; ++i) a[i] = y[i];
  return a;
}

rils_rols make_rr(int classification, int d) {
  rils_rols rr(classification != 0, 1 << 30, 1 << 30, 0.001, 50, 1.0, false, 0);
  vector<int> feats(d);
  std::iota(feats.begin(), feats.end(), 0);
  rr.setup_nodes(feats);
  return rr;
}

}  // namespace

extern "C" {

// Full fit through the reference's fit_inner (rils_rols_cpp.cpp:772-859) on a
// row-major X (the layout get_x receives, :675-698).  Writes the model string
// and returns the number of fitness calls, or a negative value on overflow.
int ref_fit(const double* X_rowmajor, const double* y, int n, int d, int classification,
            int max_fit_calls, int max_seconds, double cp, int max_complexity, double sample_size,
            int random_state, char* model_out, int cap, double* pred_out) {
  vector<Eigen::ArrayXd> Xe(d);
  for (int j = 0; j < d; ++j) Xe[j].resize(n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) Xe[j][i] = X_rowmajor[(size_t)i * d + j];
  Eigen::ArrayXd ye = arr_of(y, n);
  rils_rols rr(classification != 0, max_fit_calls, max_seconds, cp, max_complexity, sample_size, false,
               random_state);
  rr.fit_inner(Xe, ye);
  if (pred_out) {
    Eigen::ArrayXd p = rr.predict_inner(Xe);
    for (int i = 0; i < n; ++i) pred_out[i] = p[i];
  }
  string prefix;
  emit_prefix(rr.final_solution.get(), prefix);
  string s = rr.get_model_string() + "\n" + prefix;
  if (put(s, model_out, cap) < 0) return -1;
  return rr.get_fit_calls();
}

// One candidate through tune_constants (:445-518) and fitness (:520-541), or
// fitness alone when tuned == 0.  out3 = (1-R2 or loss, RMSE, size).
int ref_tune_fitness(const double* Xcol, const double* y, int n, int d, const char* tree, int tuned,
                     int classification, double* out3, char* tree_out, int cap) {
  try {
    auto X = cols_of(Xcol, n, d);
    auto ya = arr_of(y, n);
    rils_rols rr = make_rr(classification, d);
    shared_ptr<node> t = parse_tree(tree);
    shared_ptr<node> sol = tuned ? rr.tune_constants(t, X, ya) : t;
    auto f = rr.fitness(sol, X, ya);
    out3[0] = std::get<0>(f);
    out3[1] = std::get<1>(f);
    out3[2] = std::get<2>(f);
    string prefix;
    emit_prefix(sol.get(), prefix);
    return put(sol->to_string() + "\n" + prefix, tree_out, cap);
  } catch (const std::exception& e) {
    return put(string("ERROR ") + e.what(), tree_out, cap), -2;
  }
}

// Candidate generation (:348-443).  Output: one candidate per line, each line
// "<to_string>\t<prefix form>".
int ref_candidates(const char* tree, int local_search, int d, int classification, char* out, int cap) {
  try {
    rils_rols rr = make_rr(classification, d);
    vector<Eigen::ArrayXd> X;
    Eigen::ArrayXd y;
    auto c = rr.all_candidates(parse_tree(tree), X, y, local_search != 0);
    string s;
    for (auto& nd : c) {
      string p;
      emit_prefix(&nd, p);
      s += nd.to_string() + "\t" + p + "\n";
    }
    return put(s, out, cap);
  } catch (const std::exception& e) {
    return put(string("ERROR ") + e.what(), out, cap), -2;
  }
}

// Tree rewriting primitives (node.cpp:140-374, node.h:255-322).
//   what = 0: to_string; 1: expand; 2: simplify; 3: normalize_factor_constants(NONE,false);
//          4: the candidate clean-up loop of all_candidates (:413-425);
//          5: expand+simplify then extract_non_constant_factors + the factor filter of
//             tune_constants (:448-473), one factor per line.
// Output: "<to_string>\t<prefix>\t<size>" (what 0-4) or factor lines (what 5).
int ref_rewrite(const char* tree, int what, char* out, int cap) {
  try {
    shared_ptr<node> t = parse_tree(tree);
    if (what == 1) t->expand();
    if (what == 2) t->simplify();
    if (what == 3) t->normalize_factor_constants(node_type::NONE, false);
    if (what == 4) {
      int it_max = 5;
      while (it_max > 0) {
        const auto size = t->size();
        t->expand();
        t->normalize_factor_constants(node_type::NONE, false);
        t->simplify();
        if (t->size() == size) break;
        it_max--;
      }
    }
    if (what == 5) {
      t->expand();
      t->simplify();
      vector<node*> all_factors;
      t->extract_non_constant_factors(all_factors);
      string s;
      for (auto f : all_factors) {
        node* g = f;
        if (f->is<node_type::CONST>()) continue;
        if (f->get_arity() == 2 && f->get_left()->is<node_type::CONST>() && f->get_right()->is<node_type::CONST>())
          continue;
        if (f->is<node_type::MULTIPLY>() || f->is<node_type::PLUS>() || f->is<node_type::MINUS>()) {
          if (f->get_left()->is<node_type::CONST>()) g = f->get_right();
          else if (f->get_right()->is<node_type::CONST>()) g = f->get_left();
        }
        if (g == f && f->is<node_type::DIVIDE>() && f->get_right()->is<node_type::CONST>()) g = f->get_left();
        string p;
        emit_prefix(g, p);
        s += g->to_string() + "\t" + p + "\n";
      }
      return put(s, out, cap);
    }
    string p;
    emit_prefix(t.get(), p);
    return put(t->to_string() + "\t" + p + "\t" + std::to_string(t->size()), out, cap);
  } catch (const std::exception& e) {
    return put(string("ERROR ") + e.what(), out, cap), -2;
  }
}

}  // extern "C"

// Host search driver; see search.h.
#include "parallel.h"
#include "search.h"

#include "../common/rr_sum.h"

#include <algorithm>
#include <cmath>
#include <iostream>
#include <numeric>
#include <random>
#include <stdexcept>
#include <tuple>

namespace rrh {

// ------------------------------------------------------------ glibc rand ----
void GlibcRand::seed(unsigned s) {
  if (s == 0) s = 1;
  tab_[0] = (uint32_t)s;
  long word = (long)s;
  for (int i = 1; i < 31; ++i) {
    long hi = word / 127773;
    long lo = word % 127773;
    word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    tab_[i] = (uint32_t)word;
  }
  f_ = 3;
  b_ = 0;
  for (int k = 0; k < 310; ++k) next();
}

int GlibcRand::next() {
  uint32_t val = tab_[f_] += tab_[b_];
  int result = (int)(val >> 1);
  ++f_;
  if (f_ >= 31) {
    f_ = 0;
    ++b_;
  } else {
    ++b_;
    if (b_ >= 31) b_ = 0;
  }
  return result;
}

// ------------------------------------------------------- candidate gen ----
namespace {
constexpr double kPi = 3.14159265358979323846;  // node.h:11

// BFS order of the subtrees of the subtree at t[0..n) (node.h:351-377)
void bfs_positions(const FNode* t, std::vector<size_t>& pos) {
  pos.clear();
  pos.push_back(0);
  for (size_t i = 0; i < pos.size(); ++i) {
    size_t p = pos[i];
    int ar = arity_of(t[p].type);
    if (ar >= 1) {
      size_t lp = p + 1;
      pos.push_back(lp);
      if (ar == 2) pos.push_back(lp + subtree_len(t, lp));
    }
  }
}

Flat sub(const FNode* t, size_t p) { return Flat(t + p, t + p + subtree_len(t, p)); }
}  // namespace

void CandidateGen::setup_nodes(const std::vector<int>& rel_feat, bool classification) {
  // appended, never cleared (rils_rols_cpp.cpp:121-148)
  for (uint8_t op : {PLUS, MINUS, MULTIPLY, DIVIDE, SIN, COS, LN, EXP, SQRT, SQR})
    allowed_.push_back(FNode{op, -1, 0.0});
  for (double c : {-1., 0., 0.5, 1., 2., kPi, 10.}) allowed_.push_back(FNode{CONST, -1, c});
  for (int v : rel_feat) allowed_.push_back(FNode{VAR, v, 0.0});
  if (classification)
    for (uint8_t op : {LESS_THAN, GREATER_THAN, EQUAL, NOT_EQUAL, MIN, MAX}) allowed_.push_back(FNode{op, -1, 0.0});
}

void CandidateGen::add_const_finetune(const FNode* t, size_t, std::vector<Flat>& out) {
  if (t[0].type != CONST) return;
  const double v = t[0].val;
  if (v == 0.0) {
    out.push_back(leaf_const(-1.0));
    out.push_back(leaf_const(1.0));
  } else {
    for (double m : {-1., 0.01, 0.1, 0.2, 0.5, 0.8, 0.9, 0., 1., 1.1, 1.2, 2., kPi, 5., 10., 20., 50., 100.})
      out.push_back(leaf_const(v * m));
  }
}

void CandidateGen::add_change_to_subtree(const FNode* t, size_t, std::vector<Flat>& out) {
  int ar = arity_of(t[0].type);
  std::vector<size_t> pos;
  if (ar >= 1) {
    const FNode* l = t + 1;
    bfs_positions(l, pos);
    for (size_t p : pos) out.push_back(sub(l, p));
  }
  if (ar >= 2) {
    const FNode* r = t + 1 + subtree_len(t, 1);
    bfs_positions(r, pos);
    for (size_t p : pos) out.push_back(sub(r, p));
  }
}

void CandidateGen::add_change_to_var_or_1(const FNode* t, size_t, std::vector<Flat>& out) {
  for (const FNode& a : allowed_) {
    if (a.type != VAR) continue;
    if (t[0].type == VAR && t[0].var == a.var) continue;
    out.push_back(Flat{a});
  }
  out.push_back(leaf_const(1.0));
}

void CandidateGen::add_change_unary_applied(const FNode* t, size_t n, std::vector<Flat>& out) {
  for (const FNode& a : allowed_) {
    if (arity_of(a.type) != 1 || !is_allowed_left(a.type, t[0].type)) continue;
    out.push_back(make_unary(a.type, t, n));
  }
}

void CandidateGen::add_change_unary_to_another(const FNode* t, size_t, std::vector<Flat>& out) {
  if (arity_of(t[0].type) != 1) return;
  const FNode* child = t + 1;
  const size_t cn = subtree_len(t, 1);
  for (const FNode& a : allowed_) {
    if (arity_of(a.type) != 1 || a.type == t[0].type) continue;
    if (!is_allowed_left(a.type, child[0].type)) continue;
    out.push_back(make_unary(a.type, child, cn));
  }
}

void CandidateGen::add_change_binary_applied(const FNode* t, size_t n, std::vector<Flat>& out) {
  std::vector<size_t> pos;
  bfs_positions(t, pos);
  std::vector<std::pair<const FNode*, size_t>> args;
  args.reserve(pos.size() + allowed_.size());
  for (size_t p : pos) args.emplace_back(t + p, subtree_len(t, p));
  for (const FNode& a : allowed_)
    if (a.type == VAR || a.type == CONST) args.emplace_back(&a, 1);
  for (const FNode& b : allowed_) {
    if (arity_of(b.type) != 2) continue;
    for (auto& g : args) {
      if (is_allowed_left(b.type, t[0].type)) out.push_back(make_binary(b.type, t, n, g.first, g.second));
      if (!symmetric_of(b.type) && is_allowed_left(b.type, g.first[0].type))
        out.push_back(make_binary(b.type, g.first, g.second, t, n));
    }
  }
}

void CandidateGen::add_change_binary_to_another(const FNode* t, size_t, std::vector<Flat>& out) {
  if (arity_of(t[0].type) != 2) return;
  const FNode* l = t + 1;
  const size_t ln = subtree_len(t, 1);
  const FNode* r = l + ln;
  const size_t rn = subtree_len(r, 0);
  for (const FNode& b : allowed_) {
    if (arity_of(b.type) != 2 || b.type == t[0].type) continue;
    if (is_allowed_left(b.type, l[0].type)) out.push_back(make_binary(b.type, l, ln, r, rn));
    if (!symmetric_of(b.type) && is_allowed_left(b.type, r[0].type)) out.push_back(make_binary(b.type, r, rn, l, ln));
  }
}

void CandidateGen::change_candidates(const FNode* t, size_t n, std::vector<Flat>& out) {
  // rils_rols_cpp.cpp:332-346
  add_const_finetune(t, n, out);
  add_change_to_subtree(t, n, out);
  add_change_to_var_or_1(t, n, out);
  add_change_unary_applied(t, n, out);
  add_change_unary_to_another(t, n, out);
  add_change_binary_applied(t, n, out);
  add_change_binary_to_another(t, n, out);
}

void CandidateGen::perturb_candidates(const FNode* t, size_t n, std::vector<Flat>& out) {
  // rils_rols_cpp.cpp:318-330
  add_change_to_subtree(t, n, out);
  add_change_to_var_or_1(t, n, out);
  if (t[0].type == VAR) add_change_unary_applied(t, n, out);
  add_change_unary_to_another(t, n, out);
  if (t[0].type == VAR || t[0].type == CONST) add_change_binary_applied(t, n, out);
  add_change_binary_to_another(t, n, out);
}

namespace {
// a candidate's to_string key with its hash, computed on the slice threads so
// that the order-keeping de-duplication below only compares
struct KeyRef {
  const std::string* s;
  size_t h;
  bool operator==(const KeyRef& o) const { return h == o.h && *s == *o.s; }
};
struct KeyRefHash {
  size_t operator()(const KeyRef& k) const { return k.h; }
};
}  // namespace

std::vector<Flat> CandidateGen::all_candidates(const Flat& S, bool local_search) {
  // The candidates of one subtree position are those of change/perturb on
  // that subtree spliced into S; positions are visited in breadth-first
  // order, the root's candidates taken whole (rils_rols_cpp.cpp:348-411).
  // Positions are independent, so they are generated on the host threads and
  // concatenated in position order, which is the sequential order.
  std::vector<size_t> pos{0};
  for (size_t i = 0; i < pos.size(); ++i) {
    const size_t p = pos[i];
    const int ar = arity_of(S[p].type);
    if (ar >= 1) {
      const size_t lp = p + 1;
      pos.push_back(lp);
      if (ar >= 2) pos.push_back(lp + subtree_len(S.data(), lp));
    }
  }
  std::vector<std::vector<Flat>> unit(pos.size());
  std::vector<std::vector<std::string>> ukey(pos.size());
  parallel_slices(pos.size(), 1, [&](size_t b, size_t e) {
    std::vector<Flat> cands;
    for (size_t i = b; i < e; ++i) {
      const size_t p = pos[i], len = subtree_len(S.data(), p);
      cands.clear();
      if (local_search) change_candidates(S.data() + p, len, cands);
      else perturb_candidates(S.data() + p, len, cands);
      auto& out = unit[i];
      auto& keys = ukey[i];
      out.reserve(cands.size());
      keys.resize(cands.size());
      for (size_t c = 0; c < cands.size(); ++c) {
        if (p == 0) {
          out.push_back(std::move(cands[c]));
        } else {
          Flat f;
          f.reserve(S.size() - len + cands[c].size());
          f.insert(f.end(), S.begin(), S.begin() + p);
          f.insert(f.end(), cands[c].begin(), cands[c].end());
          f.insert(f.end(), S.begin() + p + len, S.end());
          out.push_back(std::move(f));
        }
        to_string(out.back().data(), out.back().size(), keys[c]);
      }
    }
  });
  // first de-duplication by to_string, keeping the first occurrence
  std::hash<std::string> hs;
  std::unordered_set<KeyRef, KeyRefHash> seen;
  std::vector<Flat> all;
  size_t raw = 0;
  for (auto& u : unit) raw += u.size();
  all.reserve(raw);
  seen.reserve(raw);
  for (size_t i = 0; i < unit.size(); ++i)
    for (size_t c = 0; c < unit[i].size(); ++c)
      if (seen.insert(KeyRef{&ukey[i][c], hs(ukey[i][c])}).second) all.push_back(std::move(unit[i][c]));
  // clean-up loop (rils_rols_cpp.cpp:413-425), each candidate on its own, on
  // the host threads, with the key of the cleaned candidate
  std::vector<std::string> key2(all.size());
  std::vector<size_t> hash2(all.size());
  parallel_slices(all.size(), 32, [&](size_t b, size_t e) {
    Arena arena;
    for (size_t i = b; i < e; ++i) {
      Flat& f = all[i];
      arena.reset();
      Node* t = thaw(f, arena);
      int it_max = 5;
      while (it_max > 0) {
        const int sz = size(t);
        expand(t, arena);
        normalize_factor_constants(t, NONE, false);
        simplify(t);
        if (size(t) == sz) break;
        it_max--;
      }
      f.clear();
      freeze_into(t, f);
      to_string(f.data(), f.size(), key2[i]);
      hash2[i] = hs(key2[i]);
    }
  });
  std::vector<Flat> filtered;
  filtered.reserve(all.size());
  seen.clear();
  for (size_t i = 0; i < all.size(); ++i)
    if (seen.insert(KeyRef{&key2[i], hash2[i]}).second) filtered.push_back(std::move(all[i]));
  return filtered;
}

// -------------------------------------------------------------- search ----
Search::Search(bool classification, int max_fit_calls, int max_seconds, double complexity_penalty,
               int max_complexity, double sample_size, bool verbose, int random_state)
    : max_fit_calls_(max_fit_calls),
      max_seconds_(max_seconds),
      random_state_(random_state),
      complexity_penalty_(complexity_penalty),
      sample_size_(sample_size),
      max_complexity_(max_complexity),
      classification_(classification),
      verbose_(verbose) {
  reset();
}

Search::~Search() {
  if (dataset_ && backend_.dataset_destroy) backend_.dataset_destroy(dataset_);
}

void Search::reset() {
  main_it_ = 0;
  last_improved_it_ = 0;
  fit_calls_ = 0;
  ls_calls_ = 0;
  start_time_ = std::chrono::high_resolution_clock::now();
  checked_perts_.clear();
  skipped_perts_ = 0;
  total_perts_ = 0;
  rand_.seed((unsigned)random_state_);
}

bool Search::finished() const {
  using namespace std::chrono;
  return fit_calls_ >= max_fit_calls_ ||
         duration_cast<seconds>(high_resolution_clock::now() - start_time_).count() > max_seconds_;
}

bool Search::check_skip(const std::string& s) {
  total_perts_++;
  if (checked_perts_.count(s)) {
    skipped_perts_++;
    return true;
  }
  checked_perts_.insert(s);
  return false;
}

double Search::fitness_value(const Fit& f) const {
  return (1 + f.loss) * (1 + f.rmse) * (1 + f.size * complexity_penalty_);
}

int Search::compare_fitness(const Fit& f1, const Fit& f2) const {
  const int s1 = f1.size, s2 = f2.size;
  if ((s1 > max_complexity_ || s2 > max_complexity_) && s1 != s2) return s1 - s2;
  const double v1 = fitness_value(f1), v2 = fitness_value(f2);
  if (v1 < v2) return -1;
  if (v1 > v2) return 1;
  return 0;
}

namespace {
bool dominates(const Fit& p, const Fit& f) { return p.loss <= f.loss && p.rmse <= f.rmse && p.size <= f.size; }
bool is_dominated(const std::vector<Fit>& pareto, const Fit& f) {
  for (const auto& p : pareto)
    if (dominates(p, f)) return true;
  return false;
}
void add_to_pareto(std::vector<Fit>& pareto, const Fit& f) {
  if (is_dominated(pareto, f)) return;
  for (int i = (int)pareto.size() - 1; i >= 0; i--)
    if (dominates(f, pareto[i])) pareto.erase(pareto.begin() + i);
  pareto.push_back(f);
}
}  // namespace

void Search::print_state(const Fit& curr) const {
  std::cout << "it=" << main_it_ << "\tfit_calls=" << fit_calls_ << "\tls_calls=" << ls_calls_;
  if (classification_) {
    std::cout << "\tcurr_LOSS=" << curr.loss << "\tcurr_size=" << curr.size;
    std::cout << "\tfinal_LOSS=" << final_fitness_.loss << "\tfinal_size=" << final_fitness_.size;
  } else {
    std::cout << "\tcurr_R2=" << (1 - curr.loss) << "\tcurr_RMSE=" << curr.rmse << "\tcurr_size=" << curr.size;
    std::cout << "\tfinal_R2=" << (1 - final_fitness_.loss) << "\tfinal_RMSE=" << final_fitness_.rmse
              << "\tfinal_size=" << final_fitness_.size;
  }
  std::cout << "\tchecks_skip=" << skipped_perts_ << "/" << total_perts_ << "\tsol=" << to_string(final_solution_)
            << std::endl
            << std::endl;
}

void Search::run_batch(std::vector<rrg_result>& res, std::vector<double>& coefs) {
  if (!backend_.eval) throw std::runtime_error("no fitness backend installed");
  rrg_batch b = bb_.view();
  res.assign(b.n_cand, rrg_result{});
  coefs.assign(bb_.n_coefs() > 0 ? bb_.n_coefs() : 1, 0.0);
  const auto t0 = std::chrono::steady_clock::now();
  int32_t st = backend_.eval(dataset_, &b, precision_, res.data(), coefs.data());
  backend_ns_ += std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
  if (st != RRG_OK) throw std::runtime_error(std::string("fitness backend failed: ") + rrg_last_error());
  ++n_rounds_;
  n_scored_ += b.n_cand;
}

std::vector<Fit> Search::score_untuned(const std::vector<const Flat*>& trees) {
  bb_.clear();
  std::vector<Flat> one(1);
  for (const Flat* t : trees) {
    one[0] = *t;
    bb_.add(one, RRG_UNTUNED);
  }
  std::vector<rrg_result> res;
  std::vector<double> coefs;
  run_batch(res, coefs);
  std::vector<Fit> out(trees.size());
  for (size_t i = 0; i < trees.size(); ++i) out[i] = Fit{res[i].loss, res[i].rmse, res[i].size};
  return out;
}

std::vector<Search::Tuned> Search::score_tuned(const std::vector<const Flat*>& trees) {
  bb_.clear();
  std::vector<Tuned> out(trees.size());
  // the factor split of tune_constants (expand, simplify, top-level factors)
  // of every candidate, on the host threads; encoded in candidate order
  parallel_slices(trees.size(), 32, [&](size_t b, size_t e) {
    Arena arena;
    for (size_t i = b; i < e; ++i) {
      arena.reset();
      out[i].factors = tune_factors(*trees[i], arena);
    }
  });
  {
    std::vector<const std::vector<Flat>*> parts(trees.size());
    for (size_t i = 0; i < trees.size(); ++i) parts[i] = &out[i].factors;
    bb_.add_all(parts, RRG_TUNED);
  }
  std::vector<rrg_result> res;
  std::vector<double> coefs;
  run_batch(res, coefs);
  const auto& cands = bb_.cands();
  for (size_t i = 0; i < trees.size(); ++i) {
    const int nc = (int)out[i].factors.size() + 1;
    out[i].coefs.assign(coefs.begin() + cands[i].coef_offset, coefs.begin() + cands[i].coef_offset + nc);
    out[i].fit = Fit{res[i].loss, res[i].rmse, res[i].size};
    if (!(res[i].flags & RRG_F_NONFINITE) && res[i].size != rebuilt_size(out[i].factors, out[i].coefs.data()))
      throw std::runtime_error("device and host disagree on the rebuilt tree size");
  }
  return out;
}

std::vector<int> Search::relevant_features(const std::vector<std::vector<double>>& X,
                                           const std::vector<double>& y) const {
  const int feat_cnt = (int)X.size();
  std::vector<int> rel(feat_cnt);
  if (feat_cnt <= max_feat_) {
    std::iota(rel.begin(), rel.end(), 0);
    return rel;
  }
  // R2(X[i], y) (rils_rols_cpp.cpp:40-45, 753-770), sums in the fixed CSUM order
  std::vector<std::tuple<double, int>> by_r2;
  for (int i = 0; i < feat_cnt; ++i) {
    const auto& a = X[i];
    const double avg = rr_csum(a.data(), (long)a.size()) / (double)a.size();
    rr_csum_acc acc;
    rr_csum_init(&acc);
    for (size_t r = 0; r < a.size(); ++r) rr_csum_add(&acc, (a[r] - y[r]) * (a[r] - y[r]));
    const double ssr = rr_csum_total(&acc);
    rr_csum_init(&acc);
    for (size_t r = 0; r < a.size(); ++r) rr_csum_add(&acc, (a[r] - avg) * (a[r] - avg));
    const double sst = rr_csum_total(&acc);
    by_r2.emplace_back(1 - ssr / sst, i);
  }
  std::sort(by_r2.begin(), by_r2.end(), std::greater<>());
  rel.clear();
  for (int i = 0; i < max_feat_; ++i) rel.push_back(std::get<1>(by_r2[i]));
  return rel;
}

Flat Search::local_search(const Flat& passed) {
  std::vector<Fit> pareto;
  ls_calls_++;
  bool improved = true;
  Tuned t0 = std::move(score_tuned({&passed})[0]);
  Flat curr = rebuild(t0.factors, t0.coefs.data());
  fit_calls_++;
  Fit curr_fit = t0.fit;
  while (improved && !finished()) {
    improved = false;
    std::vector<Flat> perts = gen_.all_candidates(curr, true);
    std::vector<const Flat*> ptrs;
    ptrs.reserve(perts.size());
    for (auto& p : perts) ptrs.push_back(&p);
    std::vector<Tuned> scored = score_tuned(ptrs);
    for (size_t j = 0; j < perts.size(); ++j) {
      if (finished()) break;
      fit_calls_++;
      const Fit f = scored[j].fit;
      if (verbose_ && fit_calls_ % 10000 == 0) print_state(curr_fit);
      if (!is_dominated(pareto, f) && compare_fitness(f, curr_fit) < 0) {
        improved = true;
        Flat t = rebuild(scored[j].factors, scored[j].coefs.data());
        arena_.reset();
        Node* nt = thaw(t, arena_);
        int it_max = 5;
        while (it_max > 0) {
          const int sz = size(nt);
          expand(nt, arena_);
          simplify(nt);
          if (sz == size(nt)) break;
          it_max--;
        }
        t = freeze(nt);
        const Fit f2 = score_untuned({&t})[0];
        fit_calls_++;
        curr = std::move(t);
        curr_fit = f2;
        add_to_pareto(pareto, f2);
      }
    }
  }
  return curr;
}

void Search::fit(const double* X, const double* y, int n, int d) {
  std::vector<std::vector<double>> Xe(d, std::vector<double>(n));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) Xe[j][i] = X[(size_t)i * d + j];
  std::vector<double> ye(y, y + n);
  fit_inner(Xe, ye);
}

void Search::fit_inner(const std::vector<std::vector<double>>& X_all, const std::vector<double>& y_all) {
  using namespace std::chrono;
  reset();
  const int sample_cnt = int(sample_size_ * y_all.size());
  std::vector<int> selected(y_all.size());
  std::iota(selected.begin(), selected.end(), 0);
  std::shuffle(selected.begin(), selected.end(), std::default_random_engine(random_state_));
  const int d = (int)X_all.size();
  std::vector<std::vector<double>> X(d, std::vector<double>(sample_cnt));
  std::vector<double> y(sample_cnt);
  for (int ix = 0; ix < sample_cnt; ++ix) {
    const int i = selected[ix];
    for (int j = 0; j < d; ++j) X[j][ix] = X_all[j][i];
    y[ix] = y_all[i];
  }
  std::vector<int> rel_feat = relevant_features(X, y);
  gen_.setup_nodes(rel_feat, classification_);

  std::vector<double> Xcol((size_t)d * sample_cnt);
  for (int j = 0; j < d; ++j) std::copy(X[j].begin(), X[j].end(), Xcol.begin() + (size_t)j * sample_cnt);
  if (dataset_ && backend_.dataset_destroy) backend_.dataset_destroy(dataset_);
  dataset_ = backend_.dataset_create ? backend_.dataset_create(backend_.self, Xcol.data(), y.data(), sample_cnt, d)
                                     : nullptr;
  if (!dataset_) throw std::runtime_error(std::string("cannot create the fitness dataset: ") + rrg_last_error());

  final_solution_ = leaf_const(0.0);
  final_fitness_ = score_untuned({&final_solution_})[0];
  fit_calls_++;
  bool improved = true;
  std::string key;
  while (!finished()) {
    main_it_ += 1;
    Flat start_solution = final_solution_;
    if (!improved) {
      std::vector<Flat> all_perts = gen_.all_candidates(final_solution_, false);
      const int i1 = rand_.next() % (int)all_perts.size();
      std::vector<Flat> all_2 = gen_.all_candidates(all_perts[i1], false);
      const int i2 = rand_.next() % (int)all_2.size();
      start_solution = all_2[i2];
      if (verbose_) std::cout << "Randomized to " << to_string(start_solution) << std::endl;
    }
    improved = false;
    std::vector<Flat> all_perts = gen_.all_candidates(start_solution, false);
    if (verbose_) std::cout << "Checking " << all_perts.size() << " perturbations of starting solution." << std::endl;
    std::vector<std::string> keys(all_perts.size());
    std::vector<const Flat*> todo;
    std::vector<int> slot(all_perts.size(), -1);
    for (size_t i = 0; i < all_perts.size(); ++i) {
      keys[i] = to_string(all_perts[i]);
      if (!checked_perts_.count(keys[i])) {
        slot[i] = (int)todo.size();
        todo.push_back(&all_perts[i]);
      }
    }
    std::vector<Fit> fits;
    if (!todo.empty()) fits = score_untuned(todo);
    std::vector<std::pair<double, int>> r2_by_perts;
    for (size_t i = 0; i < all_perts.size(); ++i) {
      if (finished()) break;
      if (check_skip(keys[i])) continue;
      fit_calls_++;
      r2_by_perts.emplace_back(fits[slot[i]].loss, (int)i);
    }
    std::sort(r2_by_perts.begin(), r2_by_perts.end(),
              [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first < b.first; });
    for (size_t i = 0; i < r2_by_perts.size(); ++i) {
      if (finished()) break;
      const int pi = r2_by_perts[i].second;
      checked_perts_.insert(keys[pi]);
      Flat ls_pert = local_search(all_perts[pi]);
      const Fit ls_fit = score_untuned({&ls_pert})[0];
      fit_calls_++;
      if (compare_fitness(ls_fit, final_fitness_) < 0) {
        improved = true;
        final_solution_ = ls_pert;
        final_fitness_ = ls_fit;
        if (verbose_) print_state(final_fitness_);
        best_time_ = duration_cast<milliseconds>(high_resolution_clock::now() - start_time_).count() / 1000.0;
      }
    }
  }
  total_time_ = duration_cast<milliseconds>(high_resolution_clock::now() - start_time_).count() / 1000.0;
}

void Search::predict(const double* X, int n, int d, double* out) {
  std::vector<double> Xcol((size_t)d * n), zeros(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) Xcol[(size_t)j * n + i] = X[(size_t)i * d + j];
  void* ds = backend_.dataset_create(backend_.self, Xcol.data(), zeros.data(), n, d);
  if (!ds) throw std::runtime_error(std::string("cannot create the prediction dataset: ") + rrg_last_error());
  bb_.clear();
  std::vector<Flat> one{final_solution_};
  bb_.add(one, RRG_UNTUNED);
  rrg_batch b = bb_.view();
  int32_t st = backend_.predict(ds, &b, out);
  backend_.dataset_destroy(ds);
  if (st != RRG_OK) throw std::runtime_error(std::string("prediction failed: ") + rrg_last_error());
  if (classification_)
    for (int i = 0; i < n; ++i) out[i] = out[i] >= 0.5 ? 1.0 : 0.0;
}

int64_t Search::counter(int which) const {
  switch (which) {
    case 0: return ls_calls_;
    case 1: return main_it_;
    case 2: return n_rounds_;
    case 3: return n_scored_;
    case 4: return skipped_perts_;
    case 5: return total_perts_;
    case 6: return backend_ns_;
    default: return -1;
  }
}

}  // namespace rrh

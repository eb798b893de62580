// Host search driver: iterated local search of RILS-ROLS with the fitness of
// every local-search round scored in one batched backend call.
// Follows rils_rols_cpp/rils_rols_cpp.cpp:88-881 (class rils_rols).
#pragma once
#include <chrono>
#include <cstdint>
#include <string>
#include <unordered_set>
#include <vector>

#include "../../../include/rils_rols_host.h"
#include "encode.h"
#include "expr.h"

namespace rrh {

// glibc's srand()/rand() (TYPE_3 additive feedback generator, degree 31,
// separation 3, 310 discarded outputs), kept per model so that no other
// caller of rand() in the process can change the search.
class GlibcRand {
 public:
  void seed(unsigned s);
  int next();

 private:
  int f_ = 3, b_ = 0;
  uint32_t tab_[31];
};

struct Fit {
  double loss = 0, rmse = 0;
  int size = 0;
};

// Candidate generation of the local search and of the perturbation step
// (rils_rols_cpp.cpp:121-148, 163-443).
class CandidateGen {
 public:
  void setup_nodes(const std::vector<int>& rel_feat, bool classification);
  // all_candidates(solution, local_search) with both de-duplication passes
  std::vector<Flat> all_candidates(const Flat& solution, bool local_search);

 private:
  void change_candidates(const FNode* t, size_t n, std::vector<Flat>& out);
  void perturb_candidates(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_const_finetune(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_change_to_subtree(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_change_to_var_or_1(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_change_unary_applied(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_change_unary_to_another(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_change_binary_applied(const FNode* t, size_t n, std::vector<Flat>& out);
  void add_change_binary_to_another(const FNode* t, size_t n, std::vector<Flat>& out);
  std::vector<FNode> allowed_;
  Arena arena_;
};

class Search {
 public:
  Search(bool classification, int max_fit_calls, int max_seconds, double complexity_penalty, int max_complexity,
         double sample_size, bool verbose, int random_state);
  ~Search();
  void set_backend(const rrh_backend& be) { backend_ = be; }
  void set_precision(int p) { precision_ = p; }
  // X row-major n x d
  void fit(const double* X, const double* y, int n, int d);
  void predict(const double* X, int n, int d, double* out);
  std::string model_string() const { return to_string(final_solution_); }
  std::string model_prefix() const { return to_prefix(final_solution_); }
  double best_time() const { return best_time_; }
  double total_time() const { return total_time_; }
  int fit_calls() const { return fit_calls_; }
  int64_t counter(int which) const;

 private:
  struct Tuned {
    Fit fit;
    std::vector<Flat> factors;
    std::vector<double> coefs;
  };
  void reset();
  bool finished() const;
  bool check_skip(const std::string& s);
  std::vector<int> relevant_features(const std::vector<std::vector<double>>& X, const std::vector<double>& y) const;
  void fit_inner(const std::vector<std::vector<double>>& X_all, const std::vector<double>& y_all);
  Flat local_search(const Flat& passed);
  double fitness_value(const Fit& f) const;
  int compare_fitness(const Fit& a, const Fit& b) const;
  void print_state(const Fit& curr) const;

  // batched scoring (no fit_calls accounting; the replay does that)
  std::vector<Fit> score_untuned(const std::vector<const Flat*>& trees);
  std::vector<Tuned> score_tuned(const std::vector<const Flat*>& trees);
  void run_batch(std::vector<rrg_result>& res, std::vector<double>& coefs);

  // parameters (rils_rols_cpp.cpp:92-94)
  int max_fit_calls_, max_seconds_, random_state_, max_feat_ = 200;
  double complexity_penalty_, sample_size_, max_complexity_;
  bool classification_, verbose_;
  // state (rils_rols_cpp.cpp:97-104)
  int main_it_ = 0, last_improved_it_ = 0, fit_calls_ = 0, ls_calls_ = 0, skipped_perts_ = 0, total_perts_ = 0;
  std::unordered_set<std::string> checked_perts_;
  std::chrono::high_resolution_clock::time_point start_time_;
  Flat final_solution_;
  Fit final_fitness_;
  double best_time_ = 0, total_time_ = 0;
  GlibcRand rand_;
  CandidateGen gen_;
  // backend
  rrh_backend backend_{};
  void* dataset_ = nullptr;
  int precision_ = RRG_PLAIN_FP64;
  BatchBuilder bb_;
  Arena arena_;
  int64_t n_rounds_ = 0, n_scored_ = 0;
  int64_t backend_ns_ = 0;  // wall time inside the fitness backend (device rounds)
};

}  // namespace rrh

// Flattening of candidate trees into the postfix code of the C ABI
// (include/rils_rols_gb300.h, enum rrg_op) and the tune_constants split of a
// candidate into top-level factors (rils_rols_cpp.cpp:445-475) and its rebuild
// from the fitted coefficients (rils_rols_cpp.cpp:488-517).
#pragma once
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/rils_rols_gb300.h"
#include "expr.h"

namespace rrh {

// tune_constants, first half: expand + simplify a copy of `cand`, split it
// into top-level +/- terms and keep the non-constant part of each term
// (rils_rols_cpp.cpp:448-473).  The free term 1.0 is implicit.
std::vector<Flat> tune_factors(const Flat& cand, Arena& arena);

// tune_constants, second half: sum of coef[i]*factor[i] with the drop
// (|c| < 1e-12) and snap (|c-1| < 1e-12) rules; coefs has factors.size()+1
// entries, the free term last (rils_rols_cpp.cpp:488-517).
Flat rebuild(const std::vector<Flat>& factors, const double* coefs);

// Node count of the rebuilt tree without building it.
int rebuilt_size(const std::vector<Flat>& factors, const double* coefs);

// One candidate's postfix code with constant-pool indices local to it, as
// encoded on its own (any thread); BatchBuilder::merge pools the constants.
struct EncodedCand {
  std::vector<uint32_t> code;
  std::vector<double> consts;
  std::vector<int32_t> n_nodes;  // per factor
  int stack_need = 0;
  int mode = 0;
};
void encode_local(const std::vector<Flat>& factors, int mode, Arena& arena,
                  std::unordered_map<const Node*, int>& depth, EncodedCand& out);

// Accumulates candidates into one rrg_batch.
class BatchBuilder {
 public:
  void clear();
  // every candidate of `cands` (the same mode), encoded on the host threads
  // and appended in order
  void add_all(const std::vector<const std::vector<Flat>*>& cands, int mode);
  int merge(const EncodedCand& e);
  // mode RRG_TUNED: `factors` are the non-constant factors; RRG_UNTUNED:
  // factors has exactly one entry, the whole tree.  Returns the candidate
  // index; sets *too_large if the candidate cannot be encoded.
  int add(const std::vector<Flat>& factors, int mode);
  rrg_batch view() const;
  int n_cand() const { return (int)cands_.size(); }
  int n_coefs() const { return n_coefs_; }
  const std::vector<rrg_cand>& cands() const { return cands_; }

 private:
  int const_index(double v);
  std::vector<rrg_cand> cands_;
  std::vector<rrg_factor> factors_;
  std::vector<uint32_t> code_;
  std::vector<double> consts_;
  std::unordered_map<uint64_t, int> const_map_;
  int n_coefs_ = 0;
  Arena arena_;
  std::unordered_map<const Node*, int> depth_;
  EncodedCand scratch_;
};

}  // namespace rrh

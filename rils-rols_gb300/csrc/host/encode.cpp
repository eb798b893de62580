// Candidate flattening and the tune_constants split/rebuild; see encode.h.
#include "encode.h"

#include <cstring>
#include <stdexcept>

namespace rrh {

std::vector<Flat> tune_factors(const Flat& cand, Arena& arena) {
  Node* t = thaw(cand, arena);
  expand(t, arena);
  simplify(t);
  std::vector<Node*> all;
  extract_non_constant_factors(t, all);
  std::vector<Flat> out;
  out.reserve(all.size());
  for (Node* f : all) {
    if (f->type == CONST) continue;
    if (f->arity() == 2 && f->l->type == CONST && f->r->type == CONST) continue;
    if (f->type == MULTIPLY || f->type == PLUS || f->type == MINUS) {
      if (f->l->type == CONST) { out.push_back(freeze(f->r)); continue; }
      if (f->r->type == CONST) { out.push_back(freeze(f->l)); continue; }
    }
    if (f->type == DIVIDE && f->r->type == CONST) { out.push_back(freeze(f->l)); continue; }
    out.push_back(freeze(f));
  }
  return out;
}

Flat rebuild(const std::vector<Flat>& factors, const double* coefs) {
  const size_t m = factors.size();
  Flat ols;
  bool have = false;
  for (size_t i = 0; i <= m; ++i) {
    const double c = coefs[i];
    if (value_zero(c)) continue;
    Flat term;
    if (i == m) {
      term = leaf_const(c * 1.0);
    } else if (value_one(c)) {
      term = factors[i];
    } else {
      FNode k{CONST, -1, c};
      term = make_binary(MULTIPLY, &k, 1, factors[i].data(), factors[i].size());
    }
    if (!have) {
      ols = std::move(term);
      have = true;
    } else {
      ols = make_binary(PLUS, ols.data(), ols.size(), term.data(), term.size());
    }
  }
  if (!have) ols = leaf_const(0.0);
  return ols;
}

int rebuilt_size(const std::vector<Flat>& factors, const double* coefs) {
  const size_t m = factors.size();
  int total = 0, kept = 0;
  for (size_t i = 0; i <= m; ++i) {
    if (value_zero(coefs[i])) continue;
    ++kept;
    if (i == m) total += 1;
    else if (value_one(coefs[i])) total += (int)factors[i].size();
    else total += 2 + (int)factors[i].size();
  }
  return kept == 0 ? 1 : total + kept - 1;
}

// ------------------------------------------------------------- batches ----
void BatchBuilder::clear() {
  cands_.clear();
  factors_.clear();
  code_.clear();
  consts_.clear();
  const_map_.clear();
  n_coefs_ = 0;
}

int BatchBuilder::const_index(double v) {
  uint64_t bits;
  std::memcpy(&bits, &v, sizeof bits);
  auto it = const_map_.find(bits);
  if (it != const_map_.end()) return it->second;
  int idx = (int)consts_.size();
  consts_.push_back(v);
  const_map_.emplace(bits, idx);
  return idx;
}

namespace {

struct Emitter {
  std::vector<uint32_t>& code;
  std::unordered_map<const Node*, int> depth;
  BatchBuilder* bb;
  int (BatchBuilder::*cidx)(double);

  static bool leaf(const Node* n) { return n->type == CONST || n->type == VAR; }

  // operator -> (base, swap operands)
  static void base_of(uint8_t t, int& base, bool& swap) {
    swap = false;
    switch (t) {
      case PLUS: base = RRG_ADD; break;
      case MINUS: base = RRG_SUB; break;
      case MULTIPLY: base = RRG_MUL; break;
      case DIVIDE: base = RRG_DIV; break;
      case POW: base = RRG_POW; break;
      case LESS_THAN: base = RRG_LT; break;
      case GREATER_THAN: base = RRG_LT; swap = true; break;  // a > b  <=>  b < a
      case EQUAL: base = RRG_EQ; break;
      case NOT_EQUAL: base = RRG_NE; break;
      case MIN: base = RRG_MIN; break;
      case MAX: base = RRG_MAX; break;
      default: throw std::runtime_error("unsupported binary operator in candidate");
    }
  }
  static bool commutative(int base) { return base == RRG_ADD || base == RRG_MUL || base == RRG_EQ || base == RRG_NE; }

  int D(const Node* n) {
    auto it = depth.find(n);
    if (it != depth.end()) return it->second;
    int d;
    int ar = n->arity();
    if (ar == 0) {
      d = 0;
    } else if (ar == 1) {
      d = D(n->l);
    } else {
      int base;
      bool swap;
      base_of(n->type, base, swap);
      const Node* a = swap ? n->r : n->l;
      const Node* b = swap ? n->l : n->r;
      if (leaf(b)) d = D(a);
      else if (leaf(a)) d = D(b);
      else if (D(a) >= D(b)) d = std::max(D(a), 1 + D(b));
      else d = std::max(D(b), 1 + D(a));
    }
    depth.emplace(n, d);
    return d;
  }

  uint32_t leaf_arg(const Node* n) {
    return n->type == VAR ? (uint32_t)n->var : (uint32_t)(bb->*cidx)(n->val);
  }

  void emit(const Node* n, bool push) {
    int ar = n->arity();
    if (ar == 0) {
      int op = n->type == VAR ? (push ? RRG_OP_PSV : RRG_OP_LDV) : (push ? RRG_OP_PSC : RRG_OP_LDC);
      code.push_back(RRG_INSN(op, leaf_arg(n)));
      return;
    }
    if (ar == 1) {
      emit(n->l, push);
      int op;
      switch (n->type) {
        case SIN: op = RRG_OP_SIN; break;
        case COS: op = RRG_OP_COS; break;
        case LN: op = RRG_OP_LN; break;
        case EXP: op = RRG_OP_EXP; break;
        case SQRT: op = RRG_OP_SQRT; break;
        case SQR: op = RRG_OP_SQR; break;
        default: throw std::runtime_error("unsupported unary operator in candidate");
      }
      code.push_back(RRG_INSN(op, 0));
      return;
    }
    int base;
    bool swap;
    base_of(n->type, base, swap);
    const Node* a = swap ? n->r : n->l;  // left operand of `base`
    const Node* b = swap ? n->l : n->r;  // right operand of `base`
    int src, dir;
    uint32_t arg = 0;
    if (leaf(b)) {
      emit(a, push);
      src = b->type == VAR ? RRG_SRC_V : RRG_SRC_C;
      arg = leaf_arg(b);
      dir = RRG_DIR_R;
    } else if (leaf(a)) {
      emit(b, push);
      src = a->type == VAR ? RRG_SRC_V : RRG_SRC_C;
      arg = leaf_arg(a);
      dir = RRG_DIR_N;
    } else if (D(a) >= D(b)) {
      emit(a, push);
      emit(b, true);
      src = RRG_SRC_S;
      dir = RRG_DIR_N;
    } else {
      emit(b, push);
      emit(a, true);
      src = RRG_SRC_S;
      dir = RRG_DIR_R;
    }
    if (commutative(base)) dir = RRG_DIR_N;
    code.push_back(RRG_INSN(RRG_BIN_OP(base, src, dir), arg));
  }
};

}  // namespace

int BatchBuilder::encode_factor(const Flat& f, int slot) {
  arena_.reset();
  Node* t = thaw(f, arena_);
  Emitter e{code_, {}, this, &BatchBuilder::const_index};
  int d = e.D(t);
  e.emit(t, false);
  code_.push_back(RRG_INSN(RRG_OP_EMIT, slot));
  return d;
}

int BatchBuilder::add(const std::vector<Flat>& factors, int mode) {
  rrg_cand c;
  std::memset(&c, 0, sizeof c);
  c.code_offset = (int32_t)code_.size();
  c.first_factor = (int32_t)factors_.size();
  c.n_factors = (int32_t)factors.size();
  c.mode = mode;
  c.coef_offset = mode == RRG_TUNED ? n_coefs_ : 0;
  c.stack_need = 0;
  if (mode == RRG_TUNED && (int)factors.size() + 1 > RRG_MAX_TERMS)
    throw std::runtime_error("candidate has more than RRG_MAX_TERMS terms");
  if (mode == RRG_UNTUNED && factors.size() != 1) throw std::runtime_error("untuned candidate needs one program");
  for (size_t i = 0; i < factors.size(); ++i) {
    int d = encode_factor(factors[i], (int)i);
    if (d > c.stack_need) c.stack_need = d;
    factors_.push_back(rrg_factor{(int32_t)factors[i].size(), 0});
  }
  if (c.stack_need > RRG_MAX_STACK) throw std::runtime_error("candidate exceeds RRG_MAX_STACK spill depth");
  c.code_len = (int32_t)code_.size() - c.code_offset;
  if (mode == RRG_TUNED) n_coefs_ += (int)factors.size() + 1;
  cands_.push_back(c);
  return (int)cands_.size() - 1;
}

rrg_batch BatchBuilder::view() const {
  rrg_batch b;
  b.n_cand = (int32_t)cands_.size();
  b.n_factors = (int32_t)factors_.size();
  b.n_code = (int32_t)code_.size();
  b.n_consts = (int32_t)consts_.size();
  b.cands = cands_.data();
  b.factors = factors_.data();
  b.code = code_.data();
  b.consts = consts_.data();
  return b;
}

}  // namespace rrh

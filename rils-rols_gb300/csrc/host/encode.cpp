// Candidate flattening and the tune_constants split/rebuild; see encode.h.
#include "encode.h"
#include "parallel.h"

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
  std::unordered_map<const Node*, int>& depth;
  std::vector<double>& pool;  // constants of this candidate; code holds local indices

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
    if (n->type == VAR) return (uint32_t)n->var;
    pool.push_back(n->val);
    return (uint32_t)(pool.size() - 1);
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

void encode_local(const std::vector<Flat>& factors, int mode, Arena& arena,
                  std::unordered_map<const Node*, int>& depth, EncodedCand& out) {
  out.code.clear();
  out.consts.clear();
  out.n_nodes.clear();
  out.stack_need = 0;
  out.mode = mode;
  if (mode == RRG_TUNED && (int)factors.size() + 1 > RRG_MAX_TERMS)
    throw std::runtime_error("candidate has more than RRG_MAX_TERMS terms");
  if (mode == RRG_UNTUNED && factors.size() != 1) throw std::runtime_error("untuned candidate needs one program");
  for (size_t i = 0; i < factors.size(); ++i) {
    arena.reset();
    depth.clear();
    Node* t = thaw(factors[i], arena);
    Emitter e{out.code, depth, out.consts};
    const int d = e.D(t);
    e.emit(t, false);
    out.code.push_back(RRG_INSN(RRG_OP_EMIT, (uint32_t)i));
    out.stack_need = std::max(out.stack_need, d);
    out.n_nodes.push_back((int32_t)factors[i].size());
  }
  if (out.stack_need > RRG_MAX_STACK) throw std::runtime_error("candidate exceeds RRG_MAX_STACK spill depth");
}

int BatchBuilder::merge(const EncodedCand& e) {
  rrg_cand c;
  std::memset(&c, 0, sizeof c);
  c.code_offset = (int32_t)code_.size();
  c.first_factor = (int32_t)factors_.size();
  c.n_factors = (int32_t)e.n_nodes.size();
  c.mode = e.mode;
  c.coef_offset = e.mode == RRG_TUNED ? n_coefs_ : 0;
  c.stack_need = e.stack_need;
  for (uint32_t w : e.code) {
    const int op = (int)(w & 0xffu);
    const bool cst = op == RRG_OP_LDC || op == RRG_OP_PSC ||
                     (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_C);
    code_.push_back(cst ? RRG_INSN(op, (uint32_t)const_index(e.consts[w >> 8])) : w);
  }
  for (int32_t nn : e.n_nodes) factors_.push_back(rrg_factor{nn, 0});
  c.code_len = (int32_t)code_.size() - c.code_offset;
  if (e.mode == RRG_TUNED) n_coefs_ += c.n_factors + 1;
  cands_.push_back(c);
  return (int)cands_.size() - 1;
}

int BatchBuilder::add(const std::vector<Flat>& factors, int mode) {
  encode_local(factors, mode, arena_, depth_, scratch_);
  return merge(scratch_);
}

void BatchBuilder::add_all(const std::vector<const std::vector<Flat>*>& cands, int mode) {
  std::vector<EncodedCand> enc(cands.size());
  parallel_slices(cands.size(), 32, [&](size_t b, size_t e) {
    Arena arena;
    std::unordered_map<const Node*, int> depth;
    for (size_t i = b; i < e; ++i) encode_local(*cands[i], mode, arena, depth, enc[i]);
  });
  for (const EncodedCand& e : enc) merge(e);
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

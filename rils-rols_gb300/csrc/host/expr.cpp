// Expression-tree IR of the RILS-ROLS search (host side); see expr.h.
#include "expr.h"

#include <climits>
#include <limits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>

namespace rrh {

namespace {
// EPS of node.h:14 is pow(10, -12), evaluated at run time there as well.
const double kEpsRt = std::pow(10.0, -12);
}  // namespace

bool value_zero(double v) { return std::fabs(v) < kEpsRt; }
bool value_one(double v) { return std::fabs(v - 1) < kEpsRt; }

// ---------------------------------------------------------------- arena ----
Node* Arena::make(uint8_t type, int32_t var, double val, Node* l, Node* r) {
  if (blocks_.empty()) {
    blocks_.push_back(static_cast<Node*>(::operator new(sizeof(Node) * kBlock)));
    cur_ = 0;
    used_ = 0;
  }
  if (used_ == kBlock) {
    ++cur_;
    if (cur_ == blocks_.size()) blocks_.push_back(static_cast<Node*>(::operator new(sizeof(Node) * kBlock)));
    used_ = 0;
  }
  Node* n = blocks_[cur_] + used_++;
  n->type = type;
  n->var = var;
  n->val = val;
  n->l = l;
  n->r = r;
  return n;
}

void Arena::reset() {
  cur_ = 0;
  used_ = 0;
}

Arena::~Arena() {
  for (Node* b : blocks_) ::operator delete(b);
}

// ----------------------------------------------------------- flat trees ----
Flat leaf_const(double v) { return Flat{FNode{CONST, -1, v}}; }
Flat leaf_var(int i) { return Flat{FNode{VAR, i, 0.0}}; }

Flat make_unary(uint8_t op, const FNode* a, size_t na) {
  Flat f;
  f.reserve(na + 1);
  f.push_back(FNode{op, -1, 0.0});
  f.insert(f.end(), a, a + na);
  return f;
}

Flat make_binary(uint8_t op, const FNode* a, size_t na, const FNode* b, size_t nb) {
  Flat f;
  f.reserve(na + nb + 1);
  f.push_back(FNode{op, -1, 0.0});
  f.insert(f.end(), a, a + na);
  f.insert(f.end(), b, b + nb);
  return f;
}

size_t subtree_len(const FNode* t, size_t p) {
  size_t need = 1, q = p;
  while (need > 0) {
    need += arity_of(t[q].type);
    --need;
    ++q;
  }
  return q - p;
}

namespace {

// (int)std::round(v) as x86-64 performs it (cvttsd2si): out-of-range values
// become INT_MIN.  The reference's text keys are reproduced on every host.
int x86_int(double r) {
  if (!(r > -2147483649.0 && r < 2147483648.0)) return INT_MIN;
  return static_cast<int>(r);
}

void append_const(double v, std::string& o) {
  if (std::fabs(std::round(v) - v) < kEpsRt) {
    o += std::to_string(x86_int(std::round(v)));
  } else if (std::isnan(v)) {
    o += std::signbit(v) ? "-nan" : "nan";  // glibc's %f spelling of a NaN
  } else {
    char buf[512];
    std::snprintf(buf, sizeof buf, "%f", v);
    o += buf;
  }
}

size_t ts(const FNode* t, size_t p, std::string& o) {
  const FNode& n = t[p];
  auto bin = [&](const char* pre, const char* mid, const char* post) {
    o += pre;
    size_t q = ts(t, p + 1, o);
    o += mid;
    q = ts(t, q, o);
    o += post;
    return q;
  };
  auto un = [&](const char* pre, const char* post) {
    o += pre;
    size_t q = ts(t, p + 1, o);
    o += post;
    return q;
  };
  switch (n.type) {
    case CONST: append_const(n.val, o); return p + 1;
    case VAR: o += 'x'; o += std::to_string(n.var); return p + 1;
    case PLUS: return bin("(", "+", ")");
    case MINUS: return bin("(", "-", ")");
    case MULTIPLY: return bin("(", "*", ")");
    case DIVIDE: return bin("(", "/", ")");
    case SIN: return un("sin(", ")");
    case COS: return un("cos(", ")");
    case LN: return un("ln(", ")");
    case EXP: return un("exp(", ")");
    case SQRT: return un("sqrt(", ")");
    case SQR: return un("((", ")**2)");
    case POW: return bin("pow(", ",", ")");
    // node.h:286-293 prints '<' for all four comparison operators
    case LESS_THAN: case GREATER_THAN: case EQUAL: case NOT_EQUAL: return bin("(", "<", ")");
    case MIN: return bin("MIN(", ", ", ")");
    case MAX: return bin("MAX(", ", ", ")");
    default: o += "*****UNKNOWN*****"; return p + subtree_len(t, p);
  }
}

const char* prefix_name(uint8_t t) {
  static const char* names[N_OPS] = {"?", "c", "x", "add", "sub", "mul", "div", "sin", "cos", "ln",
                                     "exp", "sqrt", "sqr", "pow", "lt", "gt", "eq", "ne", "min", "max"};
  return t < N_OPS ? names[t] : "?";
}

}  // namespace

void to_string(const FNode* t, size_t n, std::string& out) {
  if (n) ts(t, 0, out);
}

std::string to_string(const Flat& f) {
  std::string s;
  s.reserve(f.size() * 8);
  to_string(f.data(), f.size(), s);
  return s;
}

std::string to_prefix(const Flat& f) {
  std::string s;
  char buf[64];
  for (size_t i = 0; i < f.size(); ++i) {
    if (i) s += ' ';
    if (f[i].type == CONST) {
      std::snprintf(buf, sizeof buf, "c:%.17g", f[i].val);
      s += buf;
    } else if (f[i].type == VAR) {
      s += 'x';
      s += std::to_string(f[i].var);
    } else {
      s += prefix_name(f[i].type);
    }
  }
  return s;
}

Flat from_prefix(const std::string& s) {
  // whitespace-separated tokens, scanned in place (a round encodes thousands
  // of trees, so no stream or per-token string for operators and constants)
  auto is_space = [](char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; };
  Flat f;
  size_t need = 1;
  const char* p = s.c_str();
  const char* const end = p + s.size();
  for (;;) {
    while (p < end && is_space(*p)) ++p;
    if (p == end) break;
    const char* q = p;
    while (q < end && !is_space(*q)) ++q;
    const size_t len = (size_t)(q - p);
    if (need == 0) throw std::runtime_error("trailing tokens in tree: " + s);
    if (p[0] == 'x') {
      f.push_back(FNode{VAR, std::stoi(std::string(p + 1, len - 1)), 0.0});
    } else if (len >= 2 && p[0] == 'c' && p[1] == ':') {
      // strtod stops at the whitespace that ends the token
      f.push_back(FNode{CONST, -1, std::strtod(p + 2, nullptr)});
    } else {
      uint8_t op = NONE;
      for (uint8_t t = PLUS; t < N_OPS; ++t) {
        const char* nm = prefix_name(t);
        if (std::strlen(nm) == len && std::memcmp(nm, p, len) == 0) op = t;
      }
      if (op == NONE) throw std::runtime_error("bad token in tree: " + std::string(p, len));
      f.push_back(FNode{op, -1, 0.0});
    }
    need += arity_of(f.back().type);
    --need;
    p = q;
  }
  if (need != 0) throw std::runtime_error("truncated tree: " + s);
  return f;
}

// -------------------------------------------------------- pointer trees ----
namespace {
Node* thaw_rec(const FNode* t, size_t& p, Arena& a) {
  const FNode& f = t[p++];
  Node* n = a.make(f.type, f.var, f.val);
  int ar = arity_of(f.type);
  if (ar >= 1) n->l = thaw_rec(t, p, a);
  if (ar >= 2) n->r = thaw_rec(t, p, a);
  return n;
}
}  // namespace

Node* thaw(const FNode* t, size_t n, Arena& a) {
  if (n == 0) return nullptr;
  size_t p = 0;
  return thaw_rec(t, p, a);
}

void freeze_into(const Node* t, Flat& out) {
  out.push_back(FNode{t->type, t->var, t->val});
  int ar = t->arity();
  if (ar >= 1) freeze_into(t->l, out);
  if (ar >= 2) freeze_into(t->r, out);
}

Flat freeze(const Node* t) {
  Flat f;
  f.reserve(32);
  freeze_into(t, f);
  return f;
}

int size(const Node* t) {
  int ar = t->arity();
  if (ar == 0) return 1;
  if (ar == 1) return 1 + size(t->l);
  return 1 + size(t->l) + size(t->r);
}

Node* deep_copy(const Node* t, Arena& a) {
  Node* n = a.make(t->type, t->var, t->val);
  int ar = t->arity();
  if (ar >= 1) n->l = deep_copy(t->l, a);
  if (ar >= 2) n->r = deep_copy(t->r, a);
  return n;
}

namespace {
inline bool is_pm(const Node* n) { return n->type == PLUS || n->type == MINUS; }
// node.h:130-139: take over every field of `src`
inline void take(Node* dst, const Node* src) {
  dst->type = src->type;
  dst->var = src->var;
  dst->val = src->val;
  dst->l = src->l;
  dst->r = src->r;
}
inline void set_const(Node* n, double v) {
  n->type = CONST;
  n->val = v;
  n->l = nullptr;
  n->r = nullptr;
}
}  // namespace

void expand(Node* t, Arena& a) {
  int ar = t->arity();
  if (ar == 0) return;
  if (ar == 1) {
    expand(t->l, a);
    return;
  }
  expand(t->l, a);
  expand(t->r, a);
  if (t->type != MULTIPLY) return;
  Node* L = t->l;
  Node* R = t->r;
  if (is_pm(L)) {
    if (is_pm(R)) {
      // (t1+-t2)*(t3+-t4) = t1*t3 +- t1*t4 +- t2*t3 +- t2*t4  (node.cpp:329-338)
      Node* f1 = a.make(MULTIPLY, -1, 0.0, deep_copy(L->l, a), deep_copy(R->l, a));
      Node* f2 = a.make(MULTIPLY, -1, 0.0, deep_copy(L->l, a), deep_copy(R->r, a));
      Node* f3 = a.make(MULTIPLY, -1, 0.0, deep_copy(L->r, a), deep_copy(R->l, a));
      Node* f4 = a.make(MULTIPLY, -1, 0.0, deep_copy(L->r, a), deep_copy(R->r, a));
      Node* nl = a.make(R->type, -1, 0.0, f1, f2);
      Node* nr = a.make(R->type, -1, 0.0, f3, f4);
      t->type = L->type;
      t->var = -1;
      t->val = 0.0;
      t->l = nl;
      t->r = nr;
    } else {
      // node.cpp:361-363: the right product is built from the NEW left node's
      // right operand (a copy of t3), giving (t1*t3)*(t3*t3).
      Node* nl = a.make(MULTIPLY, -1, 0.0, deep_copy(L->l, a), deep_copy(R, a));
      Node* nr = a.make(MULTIPLY, -1, 0.0, deep_copy(nl->r, a), deep_copy(R, a));
      t->l = nl;
      t->r = nr;
      t->type = nl->type;
    }
  } else if (is_pm(R)) {
    // node.cpp:368-370: the right product copies the NEW left product,
    // giving (t1*t2)*((t1*t2)*t3).
    Node* nl = a.make(MULTIPLY, -1, 0.0, deep_copy(L, a), deep_copy(R->l, a));
    Node* nr = a.make(MULTIPLY, -1, 0.0, deep_copy(nl, a), deep_copy(R->r, a));
    t->l = nl;
    t->r = nr;
    t->type = nr->type;
  }
}

namespace {
double fold_raw(uint8_t type, double a, double b) {
  switch (type) {
    case PLUS: return a + b;
    case MINUS: return a - b;
    case MULTIPLY: return a * b;
    case DIVIDE: return a / b;
    case POW: return std::pow(a, b);
    case LESS_THAN: return a < b ? 1 : 0;
    case GREATER_THAN: return a > b ? 1 : 0;
    case EQUAL: return a == b ? 1 : 0;
    case NOT_EQUAL: return a != b ? 1 : 0;
    case MIN: return a < b ? a : b;
    case MAX: return a > b ? a : b;
    default: throw std::runtime_error("constant folding: unknown binary opcode");
  }
}
// A NaN made by an invalid operation on non-NaN operands gets the sign of the
// x86-64 default NaN, so that folded constants print alike on every host.
double fold(uint8_t type, double a, double b) {
  const double r = fold_raw(type, a, b);
  if (std::isnan(r) && !std::isnan(a) && !std::isnan(b)) return -std::numeric_limits<double>::quiet_NaN();
  return r;
}
}  // namespace

void simplify(Node* t) {
  int ar = t->arity();
  if (ar == 0) return;
  if (ar == 1) {
    simplify(t->l);
    return;
  }
  simplify(t->l);
  simplify(t->r);
  Node* L = t->l;
  Node* R = t->r;
  const uint8_t ty = t->type;
  if (L->type == CONST && R->type == CONST) {
    set_const(t, fold(ty, L->val, R->val));
    return;
  }
  if (L->type == CONST) {
    if (ty == PLUS || ty == MINUS) {
      if (value_zero(L->val)) {
        take(t, R);
      } else if (is_pm(R)) {
        if (R->l->type == CONST) {
          if (ty == PLUS) L->val += R->l->val; else L->val -= R->l->val;
          take(R, R->r);
        } else if (R->r->type == CONST) {
          if (ty == PLUS) {
            if (R->type == PLUS) L->val += R->r->val; else L->val -= R->r->val;
          } else {
            if (R->type == PLUS) L->val -= R->r->val; else L->val += R->r->val;
          }
          take(R, R->l);
        }
      }
    } else if (ty == MULTIPLY) {
      if (value_zero(L->val)) {
        set_const(t, 0.0);
      } else if (value_one(L->val)) {
        take(t, R);
      } else if (R->type == MULTIPLY) {
        if (R->l->type == CONST) {
          L->val *= R->l->val;
          take(R, R->r);
        } else if (R->r->type == CONST) {
          L->val *= R->r->val;
          take(R, R->l);
        }
      }
    } else if (ty == DIVIDE && value_zero(L->val)) {
      set_const(t, 0.0);
    }
  } else if (R->type == CONST) {
    if (ty == PLUS || ty == MINUS) {
      if (value_zero(R->val)) {
        take(t, L);
      } else if (is_pm(L)) {
        if (L->l->type == CONST) {
          if (ty == PLUS) L->l->val += R->val; else L->l->val -= R->val;
          R->val = 0;
        } else if (L->r->type == CONST) {
          if (L->type == PLUS) R->val += L->r->val; else R->val -= L->r->val;
          L->r->val = 0;
        }
      }
    } else if (ty == MULTIPLY) {
      if (value_one(R->val)) {
        take(t, L);
      } else if (value_zero(R->val)) {
        set_const(t, 0.0);
      } else if (L->type == MULTIPLY) {
        if (L->l->type == CONST) {
          R->val *= L->l->val;
          take(L, L->r);
        } else if (L->r->type == CONST) {
          R->val *= L->r->val;
          take(L, L->l);
        }
      }
    }
  }
}

void normalize_factor_constants(Node* t, uint8_t parent, bool inside) {
  (void)parent;
  if (t->type == CONST) {
    t->val = 1;
  } else if (!inside && is_pm(t)) {
    normalize_factor_constants(t->l, t->type, false);
    normalize_factor_constants(t->r, t->type, false);
  } else if (!inside) {
    if (t->type == MULTIPLY) {
      normalize_factor_constants(t->l, t->type, true);
      normalize_factor_constants(t->r, t->type, true);
    } else if (t->type == DIVIDE) {
      normalize_factor_constants(t->r, t->type, true);
    }
  }
}

void extract_non_constant_factors(Node* t, std::vector<Node*>& out) {
  if (is_pm(t)) {
    extract_non_constant_factors(t->l, out);
    extract_non_constant_factors(t->r, out);
  } else if (t->type != CONST) {
    out.push_back(t);
  }
}

bool is_allowed_left(uint8_t self, uint8_t child) {
  switch (self) {
    case EXP: case LN: return !(child == EXP || child == LN);
    case POW: return child != POW;
    case COS: case SIN: return !(child == COS || child == SIN);
    default: return true;
  }
}

}  // namespace rrh

// Expression-tree IR of the RILS-ROLS search, host side.
//
// Mirrors the node type of the reference (rils_rols_cpp/node.h:16-331,
// rils_rols_cpp/node.cpp) with the same operator set, the same rewriting
// rules (expand, simplify, normalize_factor_constants), the same text form
// (to_string, which is also the de-duplication key of the search) and the
// same node count (size).  Two representations are used:
//   * Flat  - a tree stored in prefix order in one vector (value semantics,
//             cheap to copy, splice and hash); candidates and search state
//             live in this form;
//   * Node  - a pointer tree in an Arena, used where the rewriting rules
//             mutate a tree in place.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace rrh {

// Operator codes, in the order of the reference enum (node.h:16-38).
enum Op : uint8_t {
  NONE = 0, CONST, VAR, PLUS, MINUS, MULTIPLY, DIVIDE, SIN, COS, LN, EXP, SQRT, SQR, POW,
  LESS_THAN, GREATER_THAN, EQUAL, NOT_EQUAL, MIN, MAX, N_OPS
};

// node.h:40-56 (arity) and node.h:58-68 (symmetry)
inline int arity_of(uint8_t t) {
  switch (t) {
    case CONST: case VAR: return 0;
    case SIN: case COS: case LN: case EXP: case SQRT: case SQR: return 1;
    default: return 2;
  }
}
inline bool symmetric_of(uint8_t t) { return !(t == MINUS || t == DIVIDE || t == POW); }

// |v| < 1e-12 and |v-1| < 1e-12 (node.h:13-14, 333-339)
constexpr double kEps = 1e-12;
bool value_zero(double v);
bool value_one(double v);

struct FNode {
  uint8_t type;
  int32_t var;
  double val;
};
using Flat = std::vector<FNode>;

struct Node {
  uint8_t type;
  int32_t var;
  double val;
  Node* l;
  Node* r;
  int arity() const { return arity_of(type); }
};

// Bump allocator for pointer trees; reset() frees everything at once.
class Arena {
 public:
  Node* make(uint8_t type, int32_t var = -1, double val = 0.0, Node* l = nullptr, Node* r = nullptr);
  void reset();
  ~Arena();

 private:
  std::vector<Node*> blocks_;
  size_t used_ = 0;
  size_t cur_ = 0;
  static constexpr size_t kBlock = 4096;
};

// --- flat trees ------------------------------------------------------------
Flat leaf_const(double v);
Flat leaf_var(int i);
Flat make_unary(uint8_t op, const FNode* a, size_t na);
Flat make_binary(uint8_t op, const FNode* a, size_t na, const FNode* b, size_t nb);
// number of nodes of the subtree that starts at position p
size_t subtree_len(const FNode* t, size_t p);
inline int flat_size(const Flat& f) { return (int)f.size(); }

// text form of node.h:255-301; appended to `out`
void to_string(const FNode* t, size_t n, std::string& out);
std::string to_string(const Flat& f);

// prefix token form used by tests and tools: "add x0 c:2.5"
std::string to_prefix(const Flat& f);
Flat from_prefix(const std::string& s);  // throws std::runtime_error

// --- pointer trees -----------------------------------------------------------
Node* thaw(const FNode* t, size_t n, Arena& a);
inline Node* thaw(const Flat& f, Arena& a) { return thaw(f.data(), f.size(), a); }
Flat freeze(const Node* t);
void freeze_into(const Node* t, Flat& out);
int size(const Node* t);
Node* deep_copy(const Node* t, Arena& a);

// node.cpp:340-374 (including its one-sided distribution, which reuses the
// freshly built left product when forming the right one)
void expand(Node* t, Arena& a);
// node.cpp:152-296
void simplify(Node* t);
// node.cpp:312-327
void normalize_factor_constants(Node* t, uint8_t parent, bool inside_factor);
// node.cpp:140-147
void extract_non_constant_factors(Node* t, std::vector<Node*>& out);
// node.cpp:97-118: may a node of type `self` take `child` as its left operand
bool is_allowed_left(uint8_t self, uint8_t child);

}  // namespace rrh

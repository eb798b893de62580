// Rounds over the shared factor table: the mixed round (FP32 table, pair
// sums, solve, residual pass) and the FP64 scoring of candidate lists
// (FP64 table, direct column-pivoted QR per candidate).
//
// A candidate's tuned form is a sum of top-level factors
// (tune_constants, rils_rols_cpp.cpp:448-475); candidates of one round share
// most factors, so factor programs are de-duplicated on the host (same
// instructions, same constant values) and each distinct factor is evaluated
// once per round.  The arithmetic of every factor value is that of the
// per-candidate paths, so sharing changes no result.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../common/error.h"
#include "../common/rr_sum.h"
#include "common.cuh"
#include "ftable.cuh"
#include "mixed.cuh"
#include "plain.cuh"
#include "qr_chunk.cuh"
#include "rescore.cuh"
#include "runtime.cuh"
#include "tune.cuh"

using namespace rrd;

namespace {

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  rrc::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

#define RRG_CUDA(call)                              \
  do {                                              \
    if (!cuda_ok((call), #call)) return RRG_E_CUDA; \
  } while (0)

// pair indices of cross pairs while the pair map is built (then their rank)
constexpr int32_t kCrossTag = 1 << 30;
// most slots a column arena holds (the bookkeeping scans them)
constexpr int64_t kCacheSlotsMax = 1 << 16;
// pair cache: slots of the pair array (8 bytes each); registry size at which
// the factor ids start afresh
constexpr int64_t kPairSlots = 1 << 22;
constexpr size_t kRegistryMax = (size_t)1 << 19;
// mixed rounds with fewer candidates decide their second half on the host
constexpr int64_t kAsyncMinCands = 64;
// FP64 column arena: slots of the scratch budget's half for the FP64 table
int64_t fp64_cache_slots(size_t scratch_bytes, int64_t n_pad) {
  const double col8 = 8.0 * (double)n_pad;
  const int64_t fcap =
      std::min<int64_t>(kCacheSlotsMax, std::max<int64_t>(2 * RRG_MAX_TERMS, (int64_t)(scratch_bytes / 3 / col8)));
  return std::min<int64_t>(kCacheSlotsMax, std::max<int64_t>(fcap, (int64_t)(scratch_bytes / 2 / col8)));
}
// rows from which rounds keep their columns: below, evaluating a column
// costs less than the bookkeeping of finding it (a 569-row classifier
// search ran 0.46 ms per round slower with the cache)
constexpr int64_t kCacheMinRows = 8192;

bool const_arg(int op) {
  if (op == RRG_OP_LDC || op == RRG_OP_PSC) return true;
  if (op >= RRG_OP_BIN) return (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_C;
  return false;
}

// Sections of one upload, each 256-byte aligned, copied into one pinned
// buffer and sent with one host-to-device copy.
struct Packer {
  std::vector<std::pair<const void*, size_t>> parts;
  std::vector<size_t> offs;
  size_t total = 0;
  size_t add(const void* p, size_t bytes) {
    const size_t off = total;
    parts.push_back({p, bytes});
    offs.push_back(off);
    total = (size_t)round_up((int64_t)(total + bytes), 256);
    return off;
  }
  // `round`: the context's round sequence number.  The previous round has
  // completed before a round is submitted, so a pinned buffer waits only when
  // it already fed a copy earlier in this round (that copy may be queued).
  rrg_status send(HostBuf& h, DevBuf& d, cudaStream_t st, uint64_t round) {
    if (h.used_in == round) RRG_CUDA(cudaStreamSynchronize(st));
    h.used_in = round;
    if (!h.reserve(std::max<size_t>(total, 256)) || !d.reserve(std::max<size_t>(total, 256))) {
      rrc::set_error("factor table: staging allocation failed");
      return RRG_E_OOM;
    }
    char* hp = static_cast<char*>(h.ptr);
    for (size_t i = 0; i < parts.size(); ++i)
      if (parts[i].first && parts[i].second) std::memcpy(hp + offs[i], parts[i].first, parts[i].second);
    if (total) RRG_CUDA(cudaMemcpyAsync(d.ptr, h.ptr, total, cudaMemcpyHostToDevice, st));
    return RRG_OK;
  }
  template <class T>
  T* at(DevBuf& d, size_t off) const {
    return reinterpret_cast<T*>(static_cast<char*>(d.ptr) + off);
  }
};

int cand_factors(const rrg_cand& cd) { return cd.mode == RRG_TUNED ? cd.n_factors : 1; }

// ----------------------------------------------- shared subexpressions ----
// Factor programs parsed back into trees: every distinct sin / cos / ln /
// exp / pow subtree of a sub-round becomes a table column of its own,
// evaluated once, and the programs that contain it read that column.
struct PNode {
  int8_t kind;  // 0 feature, 1 constant, 3 unary, 4 binary
  int8_t op;    // unary opcode or binary base
  int32_t arg;  // feature or constant index
  int32_t a, b; // children
};

bool parse_program(const uint32_t* code, int len, std::vector<PNode>& nd, int32_t& root) {
  std::vector<int32_t> st;
  auto leaf = [&](int8_t kind, uint32_t arg) {
    nd.push_back(PNode{kind, 0, (int32_t)arg, -1, -1});
    return (int32_t)nd.size() - 1;
  };
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    if (op == RRG_OP_LDV || op == RRG_OP_PSV) {
      st.push_back(leaf(0, arg));
    } else if (op == RRG_OP_LDC || op == RRG_OP_PSC) {
      st.push_back(leaf(1, arg));
    } else if (op >= RRG_OP_SIN && op <= RRG_OP_SQR) {
      if (st.empty()) return false;
      const int32_t x = st.back();
      nd.push_back(PNode{3, (int8_t)op, 0, x, -1});
      st.back() = (int32_t)nd.size() - 1;
    } else if (op == RRG_OP_EMIT) {
      if (st.size() != 1) return false;
      root = st.back();
      return true;
    } else if (op >= RRG_OP_BIN) {
      const int kk = op - RRG_OP_BIN;
      const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
      if (st.empty()) return false;
      const int32_t tos = st.back();
      st.pop_back();
      int32_t other;
      if (src == RRG_SRC_S) {
        if (st.empty()) return false;
        other = st.back();
        st.pop_back();
      } else {
        other = leaf(src == RRG_SRC_V ? 0 : 1, arg);
      }
      nd.push_back(PNode{4, (int8_t)base, 0, dir == RRG_DIR_N ? other : tos, dir == RRG_DIR_N ? tos : other});
      st.push_back((int32_t)nd.size() - 1);
    } else {
      return false;
    }
  }
  return false;
}

bool shared_root(const PNode& n) {
  return (n.kind == 3 && (n.op == RRG_OP_SIN || n.op == RRG_OP_COS || n.op == RRG_OP_LN || n.op == RRG_OP_EXP)) ||
         (n.kind == 4 && n.op == RRG_POW);
}

struct TableProgs {
  std::vector<uint32_t> code;      // column programs, contiguous, in column order
  std::vector<int2> meta;          // [column] (code offset, length)
  std::vector<int32_t> stack;      // [column] spill depth
  std::vector<int32_t> level_end;  // columns of level L end at level_end[L] (levels ascending)
  std::vector<int32_t> fcol;       // [local factor] table column
};

// Postfix encoder with the operand-source superinstructions and Sethi-Ullman
// ordering; a node marked as a table column is read as a leaf.
struct Encoder {
  const std::vector<PNode>& nd;
  const std::vector<int32_t>& col_of;  // [node] table column, -1 when computed inline
  int32_t root = -1;
  std::vector<int32_t> memo;
  std::vector<uint32_t>* out = nullptr;
  int sp = 0, maxsp = 0;
  Encoder(const std::vector<PNode>& n, const std::vector<int32_t>& c) : nd(n), col_of(c), memo(n.size(), -1) {}
  bool leaf(int32_t m) const { return nd[m].kind <= 1 || (m != root && col_of[m] >= 0); }
  int need(int32_t m) {
    if (leaf(m)) return 0;
    if (m != root && memo[m] >= 0) return memo[m];
    const PNode& n = nd[m];
    int v;
    if (n.kind == 3) {
      v = need(n.a);
    } else if (leaf(n.b)) {
      v = need(n.a);
    } else if (leaf(n.a)) {
      v = need(n.b);
    } else {
      const int na = need(n.a), nb = need(n.b);
      v = na >= nb ? std::max(na, nb + 1) : std::max(nb, na + 1);
    }
    if (m != root) memo[m] = v;
    return v;
  }
  void src_of(int32_t m, int& src, uint32_t& arg) const {
    if (nd[m].kind == 0) { src = RRG_SRC_V; arg = (uint32_t)nd[m].arg; }
    else if (nd[m].kind == 1) { src = RRG_SRC_C; arg = (uint32_t)nd[m].arg; }
    else { src = kSrcT; arg = (uint32_t)col_of[m]; }
  }
  void emit(int32_t m, bool live) {
    if (leaf(m)) {
      int src;
      uint32_t arg;
      src_of(m, src, arg);
      int op = src == RRG_SRC_V ? (live ? RRG_OP_PSV : RRG_OP_LDV)
                                : (src == RRG_SRC_C ? (live ? RRG_OP_PSC : RRG_OP_LDC) : (live ? kOpPST : kOpLDT));
      if (live) maxsp = std::max(maxsp, ++sp);
      out->push_back(RRG_INSN(op, arg));
      return;
    }
    const PNode& n = nd[m];
    if (n.kind == 3) {
      emit(n.a, live);
      out->push_back(RRG_INSN(n.op, 0));
      return;
    }
    int src;
    uint32_t arg;
    if (leaf(n.b)) {
      emit(n.a, live);
      src_of(n.b, src, arg);
      out->push_back(RRG_INSN(RRG_BIN_OP(n.op, src, RRG_DIR_R), arg));
    } else if (leaf(n.a)) {
      emit(n.b, live);
      src_of(n.a, src, arg);
      out->push_back(RRG_INSN(RRG_BIN_OP(n.op, src, RRG_DIR_N), arg));
    } else if (need(n.a) >= need(n.b)) {
      emit(n.a, live);
      emit(n.b, true);
      out->push_back(RRG_INSN(RRG_BIN_OP(n.op, RRG_SRC_S, RRG_DIR_N), 0));
      --sp;
    } else {
      emit(n.b, live);
      emit(n.a, true);
      out->push_back(RRG_INSN(RRG_BIN_OP(n.op, RRG_SRC_S, RRG_DIR_R), 0));
      --sp;
    }
  }
  int encode(int32_t r, std::vector<uint32_t>& dst) {
    root = r;
    out = &dst;
    sp = maxsp = 0;
    emit(r, false);
    dst.push_back(RRG_INSN(RRG_OP_EMIT, 0));
    return maxsp;
  }
};

// Table programs of the local factors (programs in lcode / lmeta).  A
// transcendental subtree becomes a column of its own only when it occurs at
// least twice (a column costs a write and a read per use); share = false
// keeps every factor a single program.
bool build_table_programs(const std::vector<uint32_t>& lcode, const std::vector<int2>& lmeta, const double* consts,
                          TableProgs& tp, bool share = true) {
  const int32_t nfl = (int32_t)lmeta.size();
  std::vector<PNode> nd;
  nd.reserve(lcode.size() + 16);
  std::vector<int32_t> froot(nfl);
  for (int32_t l = 0; l < nfl; ++l)
    if (!parse_program(lcode.data() + lmeta[l].x, lmeta[l].y, nd, froot[l])) return false;
  // structural class of every node, bottom-up (children precede parents):
  // equal classes are equal subtrees (features by index, constants by bits)
  struct ClassKey {
    uint64_t arg;
    int32_t a, b;
    int8_t kind, op;
    bool operator==(const ClassKey& o) const {
      return arg == o.arg && a == o.a && b == o.b && kind == o.kind && op == o.op;
    }
  };
  struct ClassHash {
    size_t operator()(const ClassKey& k) const {
      uint64_t h = k.arg * 0x9e3779b97f4a7c15ull;
      h ^= ((uint64_t)(uint32_t)k.a << 32 | (uint32_t)k.b) + 0x7f4a7c159e3779b9ull + (h << 6) + (h >> 2);
      h ^= ((uint64_t)(uint8_t)k.kind << 8 | (uint8_t)k.op) + (h << 6) + (h >> 2);
      return (size_t)(h ^ (h >> 29));
    }
  };
  std::unordered_map<ClassKey, int32_t, ClassHash> classes;
  classes.reserve(nd.size() + 16);
  std::vector<int32_t> cls(nd.size());
  for (size_t i = 0; i < nd.size(); ++i) {
    const PNode& n = nd[i];
    ClassKey k{0, -1, -1, n.kind, 0};
    if (n.kind == 0) {
      k.arg = (uint64_t)n.arg;
    } else if (n.kind == 1) {
      std::memcpy(&k.arg, consts + n.arg, sizeof k.arg);
    } else {
      k.op = n.op;
      k.a = cls[n.a];
      if (n.kind == 4) k.b = cls[n.b];
    }
    cls[i] = classes.emplace(k, (int32_t)classes.size()).first->second;
  }
  // occurrences of every transcendental subtree
  std::vector<int32_t> uses(classes.size(), 0);
  if (share)
    for (size_t i = 0; i < nd.size(); ++i)
      if (shared_root(nd[i])) ++uses[cls[i]];
  // shared subtrees and their levels (1 + the deepest shared subtree inside)
  std::vector<int32_t> aux_index(classes.size(), -1);
  std::vector<int32_t> aux_node, aux_level, aux_of(nd.size(), -1), lvl(nd.size(), 0);
  for (size_t i = 0; i < nd.size(); ++i) {
    const PNode& n = nd[i];
    int inner = 0;
    if (n.kind >= 3) inner = std::max(inner, lvl[n.a]);
    if (n.kind == 4) inner = std::max(inner, lvl[n.b]);
    lvl[i] = inner;
    if (share && shared_root(n) && uses[cls[i]] >= 2) {
      int32_t id = aux_index[cls[i]];
      if (id < 0) {
        id = (int32_t)aux_node.size();
        aux_index[cls[i]] = id;
        aux_node.push_back((int32_t)i);
        aux_level.push_back(inner + 1);
      }
      aux_of[i] = id;
      lvl[i] = aux_level[id];
    }
  }
  // column order: shared subtrees by level, then the factors not aliased to one
  const int n_aux = (int)aux_node.size();
  const int max_level = n_aux ? *std::max_element(aux_level.begin(), aux_level.end()) : 0;
  std::vector<int32_t> aux_col(n_aux, -1);
  std::vector<int32_t> col_nodes;  // node encoded for each column
  tp.level_end.clear();
  for (int L = 1; L <= max_level; ++L) {
    for (int a = 0; a < n_aux; ++a)
      if (aux_level[a] == L) {
        aux_col[a] = (int32_t)col_nodes.size();
        col_nodes.push_back(aux_node[a]);
      }
    tp.level_end.push_back((int32_t)col_nodes.size());
  }
  tp.fcol.assign(nfl, -1);
  for (int32_t l = 0; l < nfl; ++l) {
    const int32_t r = froot[l];
    if (aux_of[r] >= 0) {
      tp.fcol[l] = aux_col[aux_of[r]];
    } else {
      tp.fcol[l] = (int32_t)col_nodes.size();
      col_nodes.push_back(r);
    }
  }
  tp.level_end.push_back((int32_t)col_nodes.size());
  std::vector<int32_t> col_of(nd.size(), -1);
  for (size_t i = 0; i < nd.size(); ++i)
    if (aux_of[i] >= 0) col_of[i] = aux_col[aux_of[i]];
  Encoder enc(nd, col_of);
  tp.code.clear();
  tp.meta.assign(col_nodes.size(), make_int2(0, 0));
  tp.stack.assign(col_nodes.size(), 0);
  for (size_t c = 0; c < col_nodes.size(); ++c) {
    const int off = (int)tp.code.size();
    tp.stack[c] = enc.encode(col_nodes[c], tp.code);
    tp.meta[c] = make_int2(off, (int)tp.code.size() - off);
  }
  return true;
}

// Slots of one sub-round's table columns in a column arena (colcache.h):
// the factors found in the cache are read where they are; the others, and
// the shared columns their programs read, are evaluated into slots taken for
// them.  `ep` holds the evaluated programs in table order (levels ascending)
// with their table reads renumbered to slots, `ewcol` the slot each writes.
struct CachePlan {
  TableProgs ep;
  std::vector<int32_t> ewcol;
  std::vector<int32_t> ecol;     // [evaluated program] its table column
  std::vector<int32_t> fslot;    // [local factor] slot
  std::vector<int32_t> mprog;    // local factors evaluated (not found)
  std::vector<int32_t> scratch;  // slots of shared columns (this sub-round only)
  int64_t hits = 0;
  int64_t arena = 0;             // slots the arena must hold
  bool kept = false;             // the cache was used (slots scattered)
};

bool table_ref(uint32_t w) {
  const int op = (int)(w & 0xffu);
  return op == kOpLDT || op == kOpPST || (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == kSrcT);
}

// Starts a sub-round of `cc`.  When the shared columns do not fit next to
// the factors, tp is rebuilt without them; false when even then the
// factors do not fit (the caller's sub-rounds are sized so that they do).
// keep = false bypasses the cache (small datasets, where evaluating a
// column costs less than looking it up): every column is evaluated into
// slot = its table column, and whatever the cache held is forgotten.
bool plan_columns(ColumnCache& cc, bool keep, const std::vector<uint32_t>& lcode, const std::vector<int2>& lmeta,
                  const double* consts, TableProgs& tp, CachePlan& out) {
  const int32_t nfl = (int32_t)lmeta.size();
  out = CachePlan();
  if (!keep) {
    if (cc.size() > 0) cc.reset(cc.limit());
    const int32_t nc = (int32_t)tp.meta.size();
    out.ep = tp;
    out.ewcol.resize(nc);
    out.ecol.resize(nc);
    for (int32_t c = 0; c < nc; ++c) out.ewcol[c] = out.ecol[c] = c;
    out.fslot = tp.fcol;
    for (int32_t l = 0; l < nfl; ++l) out.mprog.push_back(l);
    out.arena = nc;
    return true;
  }
  out.kept = true;
  cc.begin();
  std::vector<uint64_t> hash(nfl);
  std::vector<int32_t> fhit(nfl, -1);
  auto prog = [&](int32_t l) { return FactorProg{lcode.data() + lmeta[l].x, lmeta[l].y, consts}; };
  for (int32_t l = 0; l < nfl; ++l) {
    hash[l] = prog(l).hash();
    fhit[l] = cc.find(prog(l), hash[l]);
    out.hits += fhit[l] >= 0 ? 1 : 0;
  }
  std::vector<int32_t> slot_of;
  std::vector<uint8_t> need, is_fac;
  int64_t n_new = 0;
  auto plan = [&]() {
    const int32_t nc = (int32_t)tp.meta.size();
    slot_of.assign(nc, -1);
    is_fac.assign(nc, 0);
    need.assign(nc, 0);
    for (int32_t l = 0; l < nfl; ++l) {
      is_fac[tp.fcol[l]] = 1;
      if (fhit[l] >= 0) slot_of[tp.fcol[l]] = fhit[l];
      else need[tp.fcol[l]] = 1;
    }
    // a program reads columns of lower levels only (lower numbers)
    for (int32_t c = nc - 1; c >= 0; --c) {
      if (!need[c]) continue;
      for (int pc = 0; pc < tp.meta[c].y; ++pc) {
        const uint32_t w = tp.code[tp.meta[c].x + pc];
        if (table_ref(w) && slot_of[w >> 8] < 0) need[w >> 8] = 1;
      }
    }
    n_new = 0;
    for (int32_t c = 0; c < nc; ++c) n_new += need[c] ? 1 : 0;
    return n_new <= cc.available();
  };
  if (!plan()) {
    if (!build_table_programs(lcode, lmeta, consts, tp, false) || !plan()) return false;
  }
  std::vector<int32_t> taken;
  if (!cc.take(n_new, taken)) return false;
  const int32_t nc = (int32_t)tp.meta.size();
  size_t t = 0;
  for (int32_t c = 0; c < nc; ++c)
    if (need[c]) {
      slot_of[c] = taken[t++];
      if (!is_fac[c]) out.scratch.push_back(slot_of[c]);
    }
  out.fslot.resize(nfl);
  for (int32_t l = 0; l < nfl; ++l) {
    out.fslot[l] = slot_of[tp.fcol[l]];
    if (fhit[l] < 0) {
      cc.insert(prog(l), hash[l], out.fslot[l]);
      out.mprog.push_back(l);
    }
  }
  TableProgs& ep = out.ep;
  for (size_t L = 0, c0 = 0; L < tp.level_end.size(); c0 = tp.level_end[L++]) {
    for (int32_t c = (int32_t)c0; c < tp.level_end[L]; ++c) {
      if (!need[c]) continue;
      const int off = (int)ep.code.size();
      for (int pc = 0; pc < tp.meta[c].y; ++pc) {
        uint32_t w = tp.code[tp.meta[c].x + pc];
        if (table_ref(w)) w = (w & 0xffu) | ((uint32_t)slot_of[w >> 8] << 8);
        ep.code.push_back(w);
      }
      ep.meta.push_back(make_int2(off, tp.meta[c].y));
      ep.stack.push_back(tp.stack[c]);
      out.ewcol.push_back(slot_of[c]);
      out.ecol.push_back(c);
    }
    ep.level_end.push_back((int32_t)ep.meta.size());
  }
  out.arena = cc.size();
  return true;
}

}  // namespace

void build_factor_table(const rrg_cand* cands, int32_t n_cand, const uint32_t* code, const double* consts,
                        FactorTable& ft) {
  ft.code.clear();
  ft.meta.clear();
  ft.stack.clear();
  ft.occ.clear();
  ft.ids.clear();
  ft.cand_off.assign((size_t)n_cand + 1, 0);
  // factors are equal when their words are, except that a constant operand
  // is compared by its value (two candidates may hold the same constant at
  // different pool indices): a 64-bit hash of that sequence picks the
  // candidates, a word-by-word comparison decides
  auto const_bits = [&](uint32_t w) {
    uint64_t b;
    std::memcpy(&b, consts + (w >> 8), sizeof b);
    return b;
  };
  auto same = [&](const uint32_t* a, const uint32_t* b, int len) {
    for (int i = 0; i < len; ++i) {
      const uint32_t wa = a[i], wb = b[i];
      const int oa = (int)(wa & 0xffu);
      if (oa != (int)(wb & 0xffu)) return false;
      if (const_arg(oa) ? const_bits(wa) != const_bits(wb) : wa != wb) return false;
    }
    return true;
  };
  std::unordered_map<uint64_t, int32_t> index;  // hash -> latest factor with it
  std::vector<int32_t> next_same;               // earlier factors with the same hash
  index.reserve((size_t)n_cand * 2 + 16);
  for (int32_t c = 0; c < n_cand; ++c) {
    ft.cand_off[c] = (int32_t)ft.ids.size();
    const rrg_cand& cd = cands[c];
    int32_t start = cd.code_offset;
    const int32_t end = cd.code_offset + cd.code_len;
    int sp = 0, depth = 0;
    uint64_t h = 0x9e3779b97f4a7c15ull;
    for (int32_t pc = start; pc < end; ++pc) {
      const uint32_t w = code[pc];
      const int op = (int)(w & 0xffu);
      if (op == RRG_OP_EMIT) {
        const int len = pc - start;
        auto it = index.find(h);
        int32_t id = it == index.end() ? -1 : it->second;
        while (id >= 0 && !(ft.meta[id].y == len + 1 && same(ft.code.data() + ft.meta[id].x, code + start, len)))
          id = next_same[id];
        if (id < 0) {
          id = (int32_t)ft.meta.size();
          next_same.push_back(it == index.end() ? -1 : it->second);
          index[h] = id;
          int2 mt;
          mt.x = (int)ft.code.size();
          mt.y = len + 1;
          ft.code.insert(ft.code.end(), code + start, code + pc);
          ft.code.push_back(RRG_INSN(RRG_OP_EMIT, 0));
          ft.meta.push_back(mt);
          ft.stack.push_back(depth);
          ft.occ.push_back(0);
        }
        ft.occ[id] += 1;
        ft.ids.push_back(id);
        start = pc + 1;
        sp = 0;
        depth = 0;
        h = 0x9e3779b97f4a7c15ull;
        continue;
      }
      const uint64_t v = const_arg(op) ? (const_bits(w) ^ ((uint64_t)op << 56)) : (uint64_t)w;
      h = (h ^ v) * 0x100000001b3ull;
      h ^= h >> 29;
      if (op == RRG_OP_PSV || op == RRG_OP_PSC) depth = std::max(depth, ++sp);
      else if (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_S) --sp;
    }
  }
  ft.cand_off[n_cand] = (int32_t)ft.ids.size();
}

// --------------------------------------------------------- mixed round ----
rrg_status rrg_context::run_mixed(const rrg_dataset* ds, const std::vector<int32_t>& cands, bool certify) {
  const int32_t n_cand = (int32_t)host_cands.size();
  // the mixed kernels take up to kMixedMaxM factors of spill depth <= kMixedStackCap
  std::vector<int32_t> mixed, routed;
  for (int32_t c : cands) {
    const rrg_cand& cd = host_cands[c];
    const int m = cand_factors(cd);
    bool ok = m <= kMixedMaxM;
    for (int s = 0; s < m && ok; ++s) {
      const int32_t id = ft.ids[ft.cand_off[c] + s];
      ok = ft.stack[id] <= kMixedStackCap && ft.meta[id].y <= kFacCodeSmem;
    }
    (ok ? mixed : routed).push_back(c);
  }
  last_plain_routed = (int64_t)routed.size();
  const int n_super = pair_row_blocks(ds->n_pad);
  const int fb_cap = std::max(1, n_cand);
  const size_t back_bytes = sizeof(int32_t) * (fb_cap + 1 + kFbReasons) + (size_t)fb_cap;
  if (!d_terms.reserve(sizeof(MixedTerm) * fb_cap) || !d_sse1.reserve(sizeof(double) * fb_cap) ||
      !d_cert_e.reserve(sizeof(double) * fb_cap) ||
      !d_probe.reserve(sizeof(ProbeOut) * fb_cap) || !d_nanrow.reserve(sizeof(int64_t) * fb_cap) ||
      !d_partial.reserve(sizeof(double) * (size_t)fb_cap * n_super) || !d_fallback.reserve(back_bytes) ||
      !h_fallback.reserve(back_bytes)) {
    rrc::set_error("mixed round: scratch allocation failed");
    return RRG_E_OOM;
  }
  std::vector<int32_t> fb_all;
  const size_t col_bytes = sizeof(float2) * (size_t)ds->n_pad;
  const int64_t cap_f =
      std::min<int64_t>(kCacheSlotsMax, std::max<int64_t>(16, (int64_t)(table_budget_bytes / col_bytes)));
  std::vector<int32_t> lid(ft.meta.size(), -1), lf;
  size_t pos = 0;
  while (pos < mixed.size()) {
    lf.clear();
    size_t end = pos;
    while (end < mixed.size()) {
      const int32_t c = mixed[end];
      const int m = cand_factors(host_cands[c]);
      int fresh = 0;
      for (int s = 0; s < m; ++s) fresh += lid[ft.ids[ft.cand_off[c] + s]] < 0 ? 1 : 0;
      if (end > pos && (int64_t)lf.size() + fresh > cap_f) break;
      for (int s = 0; s < m; ++s) {
        const int32_t g = ft.ids[ft.cand_off[c] + s];
        if (lid[g] < 0) {
          lid[g] = (int32_t)lf.size();
          lf.push_back(g);
        }
      }
      ++end;
    }
    // one sub-round (the table budget holds the whole round): its second
    // half is decided on the device, with no read-back.  A round of few
    // candidates reads its flags back instead (unless rounds run as graphs,
    // whose captures need the device-decided form and its buffers): on a
    // recorded 1M-row search the 2416 one-candidate rounds took 0.26 s so
    // against 0.45 s with the device-decided lane's launches
    const bool async = async_rounds && pos == 0 && end == mixed.size() &&
                       (graph_rounds || capturing || (int64_t)(end - pos) >= kAsyncMinCands);
    bool async_done = false;
    const rrg_status st = mixed_subround(ds, mixed.data() + pos, (int32_t)(end - pos), lf, lid, certify, fb_all,
                                         async, &async_done);
    for (int32_t g : lf) lid[g] = -1;
    if (st != RRG_OK) return st;
    pos = end;
  }
  last_fallback = (int64_t)fb_all.size();
  rrg_status st = RRG_OK;
  if (!routed.empty()) st = run_fp64_table(ds, routed, 0u);
  if (st == RRG_OK && !fb_all.empty()) {
    std::sort(fb_all.begin(), fb_all.end());
    st = run_fp64_table(ds, fb_all, RRG_F_QR_FALLBACK);
  }
  return st;
}

rrg_status rrg_context::mixed_subround(const rrg_dataset* ds, const int32_t* list, int32_t cnt,
                                       const std::vector<int32_t>& lf, const std::vector<int32_t>& lid,
                                       bool certify, std::vector<int32_t>& fb_all, bool async,
                                       bool* async_done) {
  if (async_done) *async_done = false;
  const DevData dd = ds->view();
  const int32_t nfl = (int32_t)lf.size();
  // local programs, contiguous in local id order
  std::vector<uint32_t> lcode;
  std::vector<int2> lmeta(nfl);
  for (int32_t i = 0; i < nfl; ++i) {
    const int2 mt = ft.meta[lf[i]];
    lmeta[i] = make_int2((int)lcode.size(), mt.y);
    lcode.insert(lcode.end(), ft.code.begin() + mt.x, ft.code.begin() + mt.x + mt.y);
  }
  // table columns: shared transcendental subtrees (by level), then factors
  TableProgs tp;
  const char* hb = static_cast<const char*>(h_batch.ptr);
  const double* consts64 = reinterpret_cast<const double*>(hb + off_d);
  if (!build_table_programs(lcode, lmeta, consts64, tp)) {
    rrc::set_error("mixed round: a factor program could not be parsed");
    return RRG_E_INVALID;
  }
  // shared columns on top of the factors must fit the table budget
  if ((double)tp.meta.size() * sizeof(float2) * (double)ds->n_pad > (double)table_budget_bytes)
    build_table_programs(lcode, lmeta, consts64, tp, false);
  // Column cache: the factor columns an earlier round on this dataset left
  // in the arena are read again; the others, and the shared columns their
  // programs read, are evaluated into free or least recently used slots (the
  // shared ones for this sub-round only).  Every kernel below addresses the
  // arena by slot; the re-scoring lane keeps the table's own column numbers
  // for its FP64 table.
  const size_t col_bytes = sizeof(float2) * (size_t)ds->n_pad;
  const int64_t climit =
      std::min<int64_t>(kCacheSlotsMax, std::max<int64_t>(16, (int64_t)(table_budget_bytes / col_bytes)));
  if (fcache.limit() != climit || fcache_npad != ds->n_pad) {
    fcache.reset(climit);
    fcache_npad = ds->n_pad;
  }
  fcache.bind(ds->uid);
  CachePlan cp;
  if (!plan_columns(fcache, cache_on && ds->n >= kCacheMinRows, lcode, lmeta, consts64, tp, cp)) {
    rrc::set_error("mixed round: the column cache has no room for the sub-round");
    return RRG_E_OOM;
  }
  // scratch slots go back to the free list when this sub-round is enqueued
  struct GiveBack {
    ColumnCache& cc;
    std::vector<int32_t>& s;
    ~GiveBack() { cc.give_back(s); }
  } give_back{fcache, cp.scratch};
  const int32_t ncol = (int32_t)tp.meta.size();
  for (int32_t c = 0; c < ncol; ++c)
    if (tp.stack[c] > kMixedStackCap || tp.meta[c].y > kFacCodeSmem) {
      rrc::set_error("mixed round: a table program exceeds the evaluator's limits");
      return RRG_E_INVALID;
    }
  const TableProgs& ep = cp.ep;
  const std::vector<int32_t>& ewcol = cp.ewcol;
  const std::vector<int32_t>& fslot = cp.fslot;
  const std::vector<int32_t>& mprog = cp.mprog;
  const int32_t ne = (int32_t)ep.meta.size();
  last_cache_hits += cp.hits;
  last_cache_evals += ne;
  // rows per thread of each evaluated program.  It fixes the order of the
  // factor's three self sums, so for a factor it is decided by the factor's
  // own program (not by the shared columns its table program happens to
  // read in this sub-round): a factor's sums are then the same bits in every
  // round, kept or evaluated again.
  std::vector<uint8_t> elight(ne);
  {
    std::vector<int32_t> fac_of(ncol, -1);
    for (int32_t l = 0; l < nfl; ++l) fac_of[tp.fcol[l]] = l;
    for (int32_t e = 0; e < ne; ++e) {
      const int32_t l = fac_of[cp.ecol[e]];
      elight[e] = l >= 0 ? fac_light(lmeta[l].y, ft.stack[lf[l]]) : fac_light(ep.meta[e].y, ep.stack[e]);
    }
  }
  // evaluator groups per level, of at most `gmax` factors: consecutive
  // columns of one rows-per-thread class whose programs fit the shared
  // buffer; per level the light groups first, then the others.  The group
  // size is a launch shape only (each factor is evaluated and summed alone):
  // the tuner's TK_FAC_GROUP.
  struct GroupSet {
    std::vector<int2> groups;
    std::vector<int32_t> level_groups;  // groups of level L end at level_groups[L]
    std::vector<int32_t> level_light;   // ... of which the first level_light[L] are light
    std::vector<int32_t> feat_off{0};   // [group + 1]: the features each group reads (staged form)
    std::vector<int32_t> feat;
    int32_t slots = 0;                  // most features one group reads
    size_t off = 0, off_foff = 0, off_feat = 0;
  };
  auto build_groups = [&](int gmax, GroupSet& gs) {
    for (size_t L = 0, c0 = 0; L < ep.level_end.size(); ++L) {
      const int32_t c1 = ep.level_end[L];
      std::vector<int2> heavy;
      int32_t n_light = 0;
      for (int32_t i = (int32_t)c0; i < c1;) {
        const bool light = elight[i] != 0;
        int32_t j = i, words = 0;
        while (j < c1 && j - i < gmax && words + ep.meta[j].y <= kFacCodeSmem && (elight[j] != 0) == light)
          words += ep.meta[j++].y;
        if (light) {
          gs.groups.push_back(make_int2(i, j - i));
          ++n_light;
        } else {
          heavy.push_back(make_int2(i, j - i));
        }
        i = j;
      }
      gs.groups.insert(gs.groups.end(), heavy.begin(), heavy.end());
      gs.level_light.push_back(n_light);
      gs.level_groups.push_back((int32_t)gs.groups.size());
      c0 = c1;
    }
    // the features each group's programs read, ascending
    std::vector<uint8_t> used(std::max(1, ds->d));
    for (const int2& g : gs.groups) {
      std::fill(used.begin(), used.end(), 0);
      for (int32_t c = g.x; c < g.x + g.y; ++c)
        for (int pc = 0; pc < ep.meta[c].y; ++pc) {
          const uint32_t w = ep.code[ep.meta[c].x + pc];
          const int op = (int)(w & 0xffu);
          if (op == RRG_OP_LDV || op == RRG_OP_PSV || (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_V))
            used[w >> 8] = 1;
        }
      int32_t k = 0;
      for (int32_t j = 0; j < ds->d; ++j)
        if (used[j]) {
          gs.feat.push_back(j);
          ++k;
        }
      gs.slots = std::max(gs.slots, k);
      gs.feat_off.push_back((int32_t)gs.feat.size());
    }
  };
  bool gtrial = false;
  int gvals[4] = {tune_pick(TK_FAC_GROUP, 0, ds->n, &gtrial), 0, 0, 0};
  gtrial = gtrial && !capturing && (int64_t)ne * ds->n >= kTuneMinWork;
  const int ngv = gtrial ? tune_variants(TK_FAC_GROUP, 0, gvals) : 1;
  std::vector<GroupSet> gsets(ngv);
  for (int v = 0; v < ngv; ++v) build_groups(std::min(gvals[v], kFacGroupMax), gsets[v]);
  // row chunks of fac_chunk(d) rows (the self sums' partials are per chunk);
  // pair sums and the residual pass use kPairRows blocks
  const int32_t n_self = 3 * ne;
  int chunk = fac_chunk(ds->d);
  if ((ds->n_pad + chunk - 1) / chunk > 65535) chunk = (int)round_up((ds->n_pad + 65534) / 65535, kFacStep);
  const int64_t n_chunks64 = (ds->n_pad + chunk - 1) / chunk;
  const int n_chunks = (int)n_chunks64;
  const int n_super = pair_row_blocks(ds->n_pad);
  const size_t n_slots = (size_t)std::max<int64_t>(1, cp.arena);
  if (!d_F.grow_keep(col_bytes * n_slots, d_F.cap) ||
      !d_P.reserve(sizeof(float2) * (size_t)n_chunks * std::max(1, n_self)) ||
      !d_cfnan.grow_keep(sizeof(unsigned long long) * n_slots, d_cfnan.cap) ||
      !d_cself.grow_keep(sizeof(double) * 3 * n_slots, d_cself.cap) ||
      !d_cprobe.grow_keep(sizeof(FacProbe) * n_slots, d_cprobe.cap)) {
    rrc::set_error("mixed round: factor table allocation failed");
    return RRG_E_OOM;
  }
  // the table programs go up first and the evaluator starts; the host builds
  // the pair map while it runs
  Packer pkt;
  const size_t o_tcode = pkt.add(tp.code.data(), sizeof(uint32_t) * tp.code.size());
  const size_t o_ecode = pkt.add(ep.code.data(), sizeof(uint32_t) * std::max<size_t>(1, ep.code.size()));
  const size_t o_emeta = pkt.add(ep.meta.data(), sizeof(int2) * std::max<size_t>(1, ep.meta.size()));
  const size_t o_ewcol = pkt.add(ewcol.data(), sizeof(int32_t) * std::max<size_t>(1, ewcol.size()));
  for (GroupSet& gs : gsets) {
    gs.off = pkt.add(gs.groups.data(), sizeof(int2) * gs.groups.size());
    gs.off_foff = pkt.add(gs.feat_off.data(), sizeof(int32_t) * gs.feat_off.size());
    gs.off_feat = pkt.add(gs.feat.data(), sizeof(int32_t) * std::max<size_t>(1, gs.feat.size()));
  }
  rrg_status pst = pkt.send(h_ftp, d_ftp, stream, round_seq);
  if (pst != RRG_OK) return pst;
  float2* F = static_cast<float2*>(d_F.ptr);
  float2* Pself = static_cast<float2*>(d_P.ptr);  // [chunk][3 ne]
  unsigned long long* fnan = static_cast<unsigned long long*>(d_cfnan.ptr);
  double* cself = static_cast<double*>(d_cself.ptr);
  FacProbe* cprobe = static_cast<FacProbe*>(d_cprobe.ptr);
  uint32_t* status = static_cast<uint32_t*>(d_status.ptr);
  const int32_t* d_ewcol = pkt.at<const int32_t>(d_ftp, o_ewcol);
  if (!cp.kept)
    RRG_CUDA(cudaMemsetAsync(fnan, 0x7f, sizeof(unsigned long long) * std::max(1, ne), stream));
  else if (!launch_fill_slots(d_ewcol, ne, fnan, 1, 0x7f7f7f7f7f7f7f7full, stream))
    return RRG_E_CUDA;

  cudaEvent_t t0 = mark_begin();
  FacEvalArgs fa;
  fa.ds = dd;
  fa.code = pkt.at<const uint32_t>(d_ftp, o_ecode);
  fa.meta = pkt.at<const int2>(d_ftp, o_emeta);
  fa.wcol = d_ewcol;
  fa.K = dev.consts32;
  fa.Klo = dev.consts32lo;
  fa.chunk = chunk;
  fa.F = F;
  fa.P = Pself;
  fa.n_pairs = n_self;
  fa.fnan = fnan;
  fa.status = status;
  fa.stage = 0;
  fa.stage_slots = 0;
  // X and y staged in shared memory by tensor copies (the tuner's
  // TK_FAC_STAGE, per feature count): possible when every group's features
  // and y fit the shared memory of one block and the tensor maps encode
  const int stage_bucket = std::min(std::max(ds->d, 1), 64);
  bool strial = false;
  const bool stage_pick = tune_pick(TK_FAC_STAGE, stage_bucket, ds->n, &strial) == 2;
  auto can_stage = [&](const GroupSet& gs) {
    return chunk % kTmaRows == 0 && gs.slots <= kFacStageMax &&
           fac_eval_smem_staged(chunk, gs.slots) <= (size_t)227 * 1024;
  };
  const bool maps_ok = fac_stage_maps(fa, dd);
  // one launch per level: a level reads the columns of the levels before it
  auto eval_all = [&](const GroupSet& gs, bool stage) {
    fa.stage = stage ? 1 : 0;
    fa.stage_slots = gs.slots;
    fa.gfeat = pkt.at<const int32_t>(d_ftp, gs.off_feat);
    for (size_t L = 0, g0 = 0; L < gs.level_groups.size(); ++L) {
      const int gl = (int)g0 + gs.level_light[L];
      fa.groups = pkt.at<const int2>(d_ftp, gs.off) + g0;
      fa.gfeat_off = pkt.at<const int32_t>(d_ftp, gs.off_foff) + g0;
      bool ok = launch_fac_eval(fa, gl - (int)g0, n_chunks, true, stream);
      fa.groups = pkt.at<const int2>(d_ftp, gs.off) + gl;
      fa.gfeat_off = pkt.at<const int32_t>(d_ftp, gs.off_foff) + gl;
      ok = ok && launch_fac_eval(fa, gs.level_groups[L] - gl, n_chunks, false, stream);
      if (!ok) return false;
      launches += (gl > (int)g0) + (gs.level_groups[L] > gl);
      g0 = gs.level_groups[L];
    }
    return true;
  };
  int gbest = 0;  // the group set in use
  if (gtrial) {
    // the first round of this row class: every group size timed on the
    // real launches (a repeat rewrites the same columns and sums)
    float ms[4];
    for (int v = 0; v < ngv; ++v) {
      bool ok = true;
      const bool st = stage_pick && maps_ok && can_stage(gsets[v]);
      const rrg_status ts = time_trial([&] { ok = eval_all(gsets[v], st); }, ms[v]);
      if (!ok) return RRG_E_CUDA;
      if (ts != RRG_OK) return ts;
      if (ms[v] < ms[gbest]) gbest = v;
    }
    tune_store(TK_FAC_GROUP, 0, ds->n, gvals, ms, ngv);
  }
  const bool stage_ok = maps_ok && can_stage(gsets[gbest]);
  if (strial && !capturing && stage_ok && (int64_t)ne * ds->n >= kTuneMinWork) {
    // the first round of this feature count: reading X from global memory
    // and staging it, both timed on the real launches
    int vals[2] = {1, 2};
    float ms[2];
    for (int v = 0; v < 2; ++v) {
      bool ok = true;
      const rrg_status ts = time_trial([&] { ok = eval_all(gsets[gbest], vals[v] == 2); }, ms[v]);
      if (!ok) return RRG_E_CUDA;
      if (ts != RRG_OK) return ts;
    }
    tune_store(TK_FAC_STAGE, stage_bucket, ds->n, vals, ms, 2);
  } else if (!gtrial && !eval_all(gsets[0], stage_pick && stage_ok)) {
    return RRG_E_CUDA;
  }
  // Pair map: self pairs by slot (entries -2 - p into the slots' self
  // sums); cross pairs oriented so that `a` is the rarer factor (its
  // partners are then the widely shared ones, hot in L2) and kept across
  // rounds like the columns (the pair cache, keyed by the two factors'
  // registry ids; a pair's sum is the same bits in either orientation):
  // only the pairs not found are summed, into their slots of the pair array.
  auto prog_of = [&](int32_t l) { return FactorProg{lcode.data() + lmeta[l].x, lmeta[l].y, consts64}; };
  const bool keepp = cp.kept;
  std::vector<uint32_t> fid;
  if (keepp) {
    if (freg.size() > kRegistryMax) {
      freg.clear();
      pairc.clear();
    }
    if (pairc.limit() != kPairSlots) pairc.reset(kPairSlots);
    pairc.bind(ds->uid);
    pairc.begin();
    fid.resize(nfl);
    for (int32_t l = 0; l < nfl; ++l) {
      const FactorProg fp = prog_of(l);
      fid[l] = freg.id(fp, fp.hash());
    }
  } else if (pairc.size() > 0) {
    pairc.reset(pairc.limit());  // the pair array is rewritten from slot 0 below
  }
  std::unordered_map<uint64_t, int32_t> cmap;
  cmap.reserve((size_t)cnt * 4 + 16);
  std::vector<std::pair<int32_t, int32_t>> cross;  // (a, b) local factors, oriented
  std::vector<int32_t> pair_of((size_t)cnt * kMixedE, -1), cand_fac((size_t)cnt * kMixedMaxM, 0);
  std::vector<int32_t> cand_col((size_t)cnt * kMixedMaxM, 0), cand_slot((size_t)cnt * kMixedMaxM, 0);
  auto cross_id = [&](int32_t x, int32_t y) {
    const int32_t gx = lf[x], gy = lf[y];
    if (!(ft.occ[gx] < ft.occ[gy] || (ft.occ[gx] == ft.occ[gy] && gx < gy))) std::swap(x, y);
    const uint64_t key = ((uint64_t)(uint32_t)x << 32) | (uint32_t)y;
    auto it = cmap.find(key);
    if (it != cmap.end()) return it->second;
    const int32_t id = (int32_t)cross.size();
    cmap.emplace(key, id);
    cross.push_back({x, y});
    return id;
  };
  constexpr int Gn = GramSize<kMixedMaxM>::G;
  for (int32_t li = 0; li < cnt; ++li) {
    const int32_t c = list[li];
    const int m = cand_factors(host_cands[c]);
    int32_t l[kMixedMaxM];
    for (int s = 0; s < m; ++s) {
      l[s] = lid[ft.ids[ft.cand_off[c] + s]];
      cand_fac[(size_t)li * kMixedMaxM + s] = fslot[l[s]];
      cand_col[(size_t)li * kMixedMaxM + s] = tp.fcol[l[s]];
      cand_slot[(size_t)li * kMixedMaxM + s] = fslot[l[s]];
    }
    // self sums by slot (entries -2 - p, p into the slots' self sums);
    // cross pairs numbered from kCrossTag until their order is known
    int32_t* po = pair_of.data() + (size_t)li * kMixedE;
    int e = 0;
    for (int i = 0; i < kMixedMaxM; ++i)
      for (int j = i; j < kMixedMaxM; ++j, ++e)
        if (i < m && j < m) po[e] = l[i] == l[j] ? -2 - 3 * fslot[l[i]] : kCrossTag + cross_id(l[i], l[j]);
    for (int i = 0; i < m; ++i) {
      po[Gn + i] = -2 - (3 * fslot[l[i]] + 1);
      po[Gn + kMixedMaxM + i] = -2 - (3 * fslot[l[i]] + 2);
    }
  }
  // slots of the cross pairs; the pairs to sum (not found)
  const int32_t n_cross = (int32_t)cross.size();
  std::vector<int32_t> cslot(n_cross), miss;
  if (keepp) {
    std::vector<uint64_t> pkey(n_cross);
    for (int32_t k = 0; k < n_cross; ++k) {
      const uint32_t ia = fid[cross[k].first], ib = fid[cross[k].second];
      pkey[k] = ((uint64_t)std::min(ia, ib) << 32) | std::max(ia, ib);
      cslot[k] = pairc.find(pkey[k]);
      if (cslot[k] < 0) miss.push_back(k);
    }
    std::vector<int32_t> got;
    if (!pairc.take((int64_t)miss.size(), got)) {
      rrc::set_error("mixed round: the pair cache has no room for the sub-round");
      return RRG_E_OOM;
    }
    for (size_t i = 0; i < miss.size(); ++i) {
      cslot[miss[i]] = got[i];
      pairc.insert(pkey[miss[i]], got[i]);
    }
  } else {
    for (int32_t k = 0; k < n_cross; ++k) cslot[k] = k;
    miss.resize(n_cross);
    std::iota(miss.begin(), miss.end(), 0);
  }
  const int32_t n_miss = (int32_t)miss.size();
  last_pair_hits += n_cross - n_miss;
  last_pair_evals += n_miss;
  for (int32_t& p : pair_of)
    if (p >= kCrossTag) p = cslot[p - kCrossTag];
  // the pairs to sum by (a's slot, b's slot); units = runs of equal a
  std::vector<int32_t> order(miss), partner(n_miss), omap(n_miss);
  auto slot_pair = [&](int32_t k) { return std::make_pair(fslot[cross[k].first], fslot[cross[k].second]); };
  std::sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return slot_pair(x) < slot_pair(y); });
  for (int32_t i = 0; i < n_miss; ++i) {
    partner[i] = fslot[cross[order[i]].second];
    omap[i] = cslot[order[i]];
  }
  // units of at most `maxp` partners (a launch shape only: each pair's sum
  // is formed alone; the tuner's TK_PAIR_UNIT)
  auto build_units = [&](int maxp, std::vector<int4>& units) {
    for (int32_t k = 0; k < n_miss;) {
      const int32_t a = fslot[cross[order[k]].first];
      int32_t e = k;
      while (e < n_miss && fslot[cross[order[e]].first] == a) ++e;
      for (int32_t s0 = k; s0 < e; s0 += maxp) units.push_back(make_int4(a, s0, std::min(e, s0 + maxp), 0));
      k = e;
    }
  };
  bool ptrial = false;
  int pvals[4] = {tune_pick(TK_PAIR_UNIT, 0, ds->n, &ptrial), 0, 0, 0};
  ptrial = ptrial && !capturing && (int64_t)n_miss * ds->n >= kTuneMinWork;
  const int npv = ptrial ? tune_variants(TK_PAIR_UNIT, 0, pvals) : 1;
  std::vector<std::vector<int4>> usets(npv);
  for (int v = 0; v < npv; ++v) build_units(pvals[v], usets[v]);
  const size_t n_pslots = (size_t)std::max<int64_t>(1, keepp ? pairc.size() : n_cross);
  if (!d_Pc.reserve(sizeof(float2) * (size_t)n_super * std::max(1, n_miss)) ||
      !d_psum.grow_keep(sizeof(double) * n_pslots, d_psum.cap)) {
    rrc::set_error("mixed round: factor table allocation failed");
    return RRG_E_OOM;
  }
  // probe programs: the factors evaluated in this sub-round (their records
  // go to their slots)
  std::vector<uint32_t> pcode;
  std::vector<int2> pmeta;
  std::vector<int32_t> pslot;
  for (int32_t l : mprog) {
    pmeta.push_back(make_int2((int)pcode.size(), lmeta[l].y));
    pcode.insert(pcode.end(), lcode.begin() + lmeta[l].x, lcode.begin() + lmeta[l].x + lmeta[l].y);
    pslot.push_back(fslot[l]);
  }
  Packer pk;
  const size_t o_code = pk.add(pcode.data(), sizeof(uint32_t) * std::max<size_t>(1, pcode.size()));
  const size_t o_meta = pk.add(pmeta.data(), sizeof(int2) * std::max<size_t>(1, pmeta.size()));
  const size_t o_pslot = pk.add(pslot.data(), sizeof(int32_t) * std::max<size_t>(1, pslot.size()));
  const size_t o_ccol = pk.add(cand_col.data(), sizeof(int32_t) * cand_col.size());
  const size_t o_cslot = pk.add(cand_slot.data(), sizeof(int32_t) * cand_slot.size());
  std::vector<size_t> o_units(npv);
  for (int v = 0; v < npv; ++v) o_units[v] = pk.add(usets[v].data(), sizeof(int4) * usets[v].size());
  const size_t o_partner = pk.add(partner.data(), sizeof(int32_t) * std::max<size_t>(1, partner.size()));
  const size_t o_omap = pk.add(omap.data(), sizeof(int32_t) * std::max<size_t>(1, omap.size()));
  const size_t o_pair = pk.add(pair_of.data(), sizeof(int32_t) * pair_of.size());
  const size_t o_list = pk.add(list, sizeof(int32_t) * cnt);
  const size_t o_cfac = pk.add(cand_fac.data(), sizeof(int32_t) * cand_fac.size());
  const size_t o_list2 = pk.add(nullptr, sizeof(int32_t) * cnt);  // filled after the solve
  pst = pk.send(h_ft, d_ft, stream, round_seq);
  if (pst != RRG_OK) return pst;
  const uint32_t* d_code = pk.at<const uint32_t>(d_ft, o_code);
  const int2* d_meta = pk.at<const int2>(d_ft, o_meta);
  const int32_t* d_list = pk.at<const int32_t>(d_ft, o_list);
  const int32_t* d_cfac = pk.at<const int32_t>(d_ft, o_cfac);
  int32_t* d_list2 = pk.at<int32_t>(d_ft, o_list2);
  float2* Pcross = static_cast<float2*>(d_Pc.ptr);  // [row block][cross pairs]
  double* psum = static_cast<double*>(d_psum.ptr);
  const int32_t* d_cslot = pk.at<const int32_t>(d_ft, o_cslot);
  const int fb_cap = std::max(1, (int)host_cands.size());
  const size_t back_bytes = sizeof(int32_t) * (fb_cap + 1 + kFbReasons) + (size_t)fb_cap;
  int32_t* fallback = static_cast<int32_t*>(d_fallback.ptr);
  uint32_t* reasons = reinterpret_cast<uint32_t*>(fallback + fb_cap + 1);
  uint8_t* pass2 = reinterpret_cast<uint8_t*>(fallback + fb_cap + 1 + kFbReasons);
  RRG_CUDA(cudaMemsetAsync(d_fallback.ptr, 0, back_bytes, stream));
  RRG_CUDA(cudaMemsetAsync(d_cert_e.ptr, 0xff, sizeof(double) * fb_cap, stream));  // NaN: no check
  mark_end(P_GRAM, t0);
  phase_bytes[P_GRAM] += (double)ds->n * 8.0 * (double)(ds->d + 1 + ne);
  t0 = mark_begin();
  PairArgs pa;
  pa.F = F;
  pa.n_pad = ds->n_pad;
  pa.partner = pk.at<const int32_t>(d_ft, o_partner);
  pa.P = Pcross;
  pa.n_pairs = n_miss;
  pa.cross0 = 0;
  auto pair_all = [&](int v) {
    pa.units = pk.at<const int4>(d_ft, o_units[v]);
    pa.n_units = (int32_t)usets[v].size();
    return launch_pair_sum(pa, n_super, stream);
  };
  if (ptrial) {
    // every unit size timed on the real launch (a repeat rewrites the same sums)
    float ms[4];
    for (int v = 0; v < npv; ++v) {
      bool ok = true;
      const rrg_status ts = time_trial([&] { ok = pair_all(v); }, ms[v]);
      if (!ok) return RRG_E_CUDA;
      if (ts != RRG_OK) return ts;
      ++launches;
    }
    tune_store(TK_PAIR_UNIT, 0, ds->n, pvals, ms, npv);
  } else if (!pair_all(0)) {
    return RRG_E_CUDA;
  }
  mark_end(P_PAIRS, t0);
  phase_bytes[P_PAIRS] += (double)ds->n * 8.0 * (double)nfl;
  t0 = mark_begin();
  if (!launch_pair_reduce(Pself, n_self, n_chunks, 0, n_self, cself, stream, d_ewcol) ||
      !launch_pair_reduce(Pcross, n_miss, n_super, 0, n_miss, psum, stream, nullptr,
                          pk.at<const int32_t>(d_ft, o_omap)) ||
      !launch_fac_probe(d_code, d_meta, (int32_t)mprog.size(), dev.consts, dev.consts32, dev.consts32lo, dd, cprobe,
                        stream, pk.at<const int32_t>(d_ft, o_pslot)) ||
      !launch_cand_probe(dev.cands, d_list, cnt, d_cfac, nullptr, cprobe, fnan,
                         static_cast<ProbeOut*>(d_probe.ptr), static_cast<int64_t*>(d_nanrow.ptr), stream)) {
    cuda_ok(cudaGetLastError(), "mixed round launch");
    return RRG_E_CUDA;
  }
  SolveArgs sa;
  sa.b = dev;
  sa.ds = dd;
  sa.list = d_list;
  sa.n_list = cnt;
  sa.pair_of = pk.at<const int32_t>(d_ft, o_pair);
  sa.psum = psum;
  sa.pself = cself;
  sa.coefs = static_cast<double*>(d_coefs.ptr);
  sa.terms = static_cast<MixedTerm*>(d_terms.ptr);
  sa.res = static_cast<rrg_result*>(d_res.ptr);
  sa.fallback = fallback;
  sa.fallback_cap = fb_cap;
  sa.sse1 = static_cast<double*>(d_sse1.ptr);
  sa.pass2 = pass2;
  sa.probe = static_cast<const ProbeOut*>(d_probe.ptr);
  sa.reasons = reasons;
  sa.nanrow = static_cast<const int64_t*>(d_nanrow.ptr);
  sa.cert_e = static_cast<double*>(d_cert_e.ptr);
  sa.rank_tol = 1e-11;
  sa.fallback_tol = 1e-7;
  sa.pass2_tol = 1e-8;
  sa.cert_tol = cert_tol;
  sa.certify = certify ? 1 : 0;
  if (!launch_solve(sa, stream)) {
    cuda_ok(cudaGetLastError(), "mixed solve launch");
    return RRG_E_CUDA;
  }
  mark_end(P_SOLVE, t0);
  launches += 7;
  if (async && cnt <= 65535) {
    // ------------------------------------------------------------------
    // Second half decided on the device: no read-back before the results.
    // The residual-pass list is compacted from the solve's flags; the FP64
    // re-scoring lane evaluates, from the round's own table programs, only
    // the columns its candidates read, decides the certain sentinels, and
    // factorises the rest with the list form of the cluster QR.  Every value
    // is computed by the same arithmetic as the host-driven path.
    // ------------------------------------------------------------------
    const size_t col8 = sizeof(double) * (size_t)ds->n_pad;
    const size_t n_all = host_cands.size();
    static const int kBucketCols[kQrBuckets] = {4, 8, 16, RRG_MAX_TERMS + 1};
    int bucket_cap[kQrBuckets] = {0, 0, 0, 0}, bucket_wide[kQrBuckets] = {0, 0, 0, 0};
    for (int32_t li = 0; li < cnt; ++li) {
      const rrg_cand& cd = host_cands[list[li]];
      if (cd.mode != RRG_TUNED) continue;
      const int cols = cd.n_factors + 2;
      const int q = cols <= 4 ? 0 : (cols <= 8 ? 1 : (cols <= 16 ? 2 : 3));
      ++bucket_cap[q];
      bucket_wide[q] = std::max(bucket_wide[q], cols);
    }
    // working columns of the QR: each bucket factorises up to qbatch[q] of
    // its candidates at a time (in order, as many batches as its capacity
    // needs), the buckets sharing half the scratch budget in proportion to
    // their capacities
    const int64_t nch = (ds->n + RR_CHUNK - 1) / RR_CHUNK;
    // (room for one candidate per bucket is set aside first, so that the
    // rounded-down shares and that minimum stay within the half together)
    double slot_need = 0.0, slot_min = 0.0;
    for (int q = 0; q < kQrBuckets; ++q) {
      slot_need += (double)bucket_cap[q] * kBucketCols[q] * (double)col8;
      if (bucket_cap[q]) slot_min += (double)kBucketCols[q] * (double)col8;
    }
    const double room = std::max(0.0, (double)scratch_budget_bytes / 2 - slot_min);
    const double share = slot_need > 0.0 ? std::min(1.0, room / slot_need) : 1.0;
    int qbatch[kQrBuckets] = {0, 0, 0, 0};
    size_t m_cols = 0, q_bytes = 0;
    for (int q = 0; q < kQrBuckets; ++q) {
      if (!bucket_cap[q]) continue;
      qbatch[q] = std::max(1, std::min(bucket_cap[q], (int)((double)bucket_cap[q] * share)));
      m_cols += (size_t)qbatch[q] * kBucketCols[q];
      q_bytes += (size_t)round_up((int64_t)qr_chunk_scratch_bytes(qbatch[q], ds->n, kBucketCols[q]), 256);
    }
    const bool fits = (double)m_cols * (double)col8 <= (double)scratch_budget_bytes / 2 &&
                      (double)ncol * (double)col8 <= (double)scratch_budget_bytes / 2;
    if (fits) {
      // FP64 column cache: a factor column it holds is copied into the
      // lane's table when a re-scored candidate reads it (kept[col] = its
      // slot); the factor columns the lane evaluates are stored into it when
      // the next round starts (which ones, the device decides: the lane's
      // marks are read back with the round's results)
      std::vector<int32_t> kept(std::max(1, ncol), -1);
      const bool keep64 = cache_on && ds->n >= kCacheMinRows;
      int64_t n_kept = 0;
      if (keep64) {
        const int64_t pl = fp64_cache_slots(scratch_budget_bytes, ds->n_pad);
        if (pcache.limit() != pl || pcache_npad != ds->n_pad) {
          pcache.reset(pl);
          pcache_npad = ds->n_pad;
        }
        pcache.bind(ds->uid);
        pcache.begin();
        for (int32_t l = 0; l < nfl; ++l) {
          const FactorProg fp{lcode.data() + lmeta[l].x, lmeta[l].y, consts64};
          const int32_t sl = pcache.find(fp, fp.hash());
          if (sl >= 0) {
            kept[tp.fcol[l]] = sl;
            ++n_kept;
          }
        }
      }
      // host records of the lane: one-column pseudo-candidates of the table
      // programs, the shared-column closure of every column (a kept column's
      // own closure is not needed), placements of the round's candidates
      // (factor columns through cand_col)
      std::vector<rrg_cand> fc(std::max(1, ncol));
      std::vector<PlainCand> fpc(std::max(1, ncol));
      std::vector<int32_t> dep_off(ncol + 1, 0), deps;
      std::vector<std::vector<int32_t>> closure(ncol);
      for (int32_t i = 0; i < ncol; ++i) {
        rrg_cand& p = fc[i];
        p.code_offset = tp.meta[i].x;
        p.code_len = tp.meta[i].y;
        p.first_factor = 0;
        p.n_factors = 1;
        p.mode = RRG_UNTUNED;
        p.coef_offset = 0;
        p.stack_need = tp.stack[i];
        p.reserved = 0;
        fpc[i] = PlainCand{i, 0, 0, 1, 0};
        std::vector<int32_t>& cl = closure[i];
        for (int pc = 0; pc < tp.meta[i].y; ++pc) {
          const uint32_t w = tp.code[tp.meta[i].x + pc];
          const int op = (int)(w & 0xffu);
          const bool tref = op == kOpLDT || op == kOpPST ||
                            (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == kSrcT);
          if (!tref) continue;
          const int32_t a = (int32_t)(w >> 8);
          cl.push_back(a);
          if (kept[a] < 0) cl.insert(cl.end(), closure[a].begin(), closure[a].end());  // a is of a lower level
        }
        std::sort(cl.begin(), cl.end());
        cl.erase(std::unique(cl.begin(), cl.end()), cl.end());
        dep_off[i + 1] = dep_off[i] + (int32_t)cl.size();
        deps.insert(deps.end(), cl.begin(), cl.end());
      }
      std::vector<int32_t> li_of(n_all, -1);
      std::vector<PlainCand> pcs(std::max<size_t>(1, n_all));
      for (int32_t li = 0; li < cnt; ++li) {
        const int32_t c = list[li];
        const rrg_cand& cd = host_cands[c];
        li_of[c] = li;
        pcs[c] = PlainCand{(int64_t)li * kMixedMaxM, 0, 0, cd.mode == RRG_TUNED ? cd.n_factors + 1 : 1, 0};
      }
      const int32_t n_levels = (int32_t)tp.level_end.size();
      Packer pf;
      const size_t o_fc = pf.add(fc.data(), sizeof(rrg_cand) * fc.size());
      const size_t o_fpc = pf.add(fpc.data(), sizeof(PlainCand) * fpc.size());
      const size_t o_doff = pf.add(dep_off.data(), sizeof(int32_t) * dep_off.size());
      const size_t o_deps = pf.add(deps.data(), sizeof(int32_t) * std::max<size_t>(1, deps.size()));
      const size_t o_liof = pf.add(li_of.data(), sizeof(int32_t) * li_of.size());
      const size_t o_pcs = pf.add(pcs.data(), sizeof(PlainCand) * pcs.size());
      const size_t o_lend = pf.add(tp.level_end.data(), sizeof(int32_t) * tp.level_end.size());
      const size_t o_kept = pf.add(kept.data(), sizeof(int32_t) * kept.size());
      pst = pf.send(h_fbpack, d_fbpack, stream, round_seq);
      if (pst != RRG_OK) return pst;
      const int nb_res = (int)((ds->n + RR_CHUNK - 1) / RR_CHUNK);
      const int nbx = (int)std::max<int64_t>(1, std::min<int64_t>(16, (ds->n + 32767) / 32768));
      const size_t stat_words = 2 + kFbReasons + (size_t)n_levels;
      if (!d_rlist2.reserve(sizeof(int32_t) * (cnt + 1)) || !d_fbneed.reserve(std::max(1, ncol)) ||
          !d_fbcols.reserve(sizeof(int32_t) * (ncol + n_levels + 1)) ||
          !d_fbF64.reserve(col8 * std::max(1, ncol)) || !d_fbcst.reserve(sizeof(ColStat) * std::max(1, ncol)) ||
          !d_fbgram.reserve(sizeof(double) * (size_t)cnt * nbx * (kGramCols * (kGramCols + 1) / 2)) ||
          !d_fbblist.reserve(sizeof(int32_t) * ((size_t)kQrBuckets * cnt + kQrBuckets)) ||
          !d_fbM.reserve(col8 * std::max<size_t>(1, m_cols)) || !d_qrs.reserve(std::max<size_t>(256, q_bytes)) ||
          !h_fbstat.reserve(sizeof(int32_t) * stat_words)) {
        rrc::set_error("mixed round: re-scoring lane allocation failed");
        return RRG_E_OOM;
      }
      int32_t* list2 = static_cast<int32_t*>(d_rlist2.ptr);
      int32_t* count2 = list2 + cnt;
      uint8_t* need = static_cast<uint8_t*>(d_fbneed.ptr);
      int32_t* lvl_cols = static_cast<int32_t*>(d_fbcols.ptr);
      int32_t* lvl_count = lvl_cols + ncol;
      double* F64 = static_cast<double*>(d_fbF64.ptr);
      ColStat* cst = static_cast<ColStat*>(d_fbcst.ptr);
      double* gpart = static_cast<double*>(d_fbgram.ptr);
      int32_t* blist = static_cast<int32_t*>(d_fbblist.ptr);
      int32_t* bcount = blist + (size_t)kQrBuckets * cnt;
      double* Mq = static_cast<double*>(d_fbM.ptr);
      const int32_t* d_ccol = pk.at<const int32_t>(d_ft, o_ccol);
      PlainCand* d_pcs = pf.at<PlainCand>(d_fbpack, o_pcs);
      const int32_t* fb_count = fallback;  // fallback[0]: entries queued so far
      const int32_t* fb_list = fallback + 1;
      double* coefs = static_cast<double*>(d_coefs.ptr);
      rrg_result* res = static_cast<rrg_result*>(d_res.ptr);
      double* sse = static_cast<double*>(d_partial.ptr);
      // residual pass of the mixed candidates whose one-pass SSE is not
      // accurate enough, over the device-compacted list
      if (!launch_pass2_compact(d_list, cnt, pass2, list2, count2, stream)) {
        cuda_ok(cudaGetLastError(), "residual list launch");
        return RRG_E_CUDA;
      }
      ResidArgs ra;
      ra.b = dev;
      ra.ds = dd;
      ra.F = F;
      ra.mlist = d_list;
      ra.list2 = list2;
      ra.n2 = cnt;
      ra.n2_dev = count2;
      ra.cand_col = d_cslot;
      ra.terms = static_cast<const MixedTerm*>(d_terms.ptr);
      ra.n_chunks = n_super;
      ra.sse = sse;
      t0 = mark_begin();
      if (!launch_ftab_resid(ra, stream, 16 * sm_count) ||
          (certify && !launch_cert_resid(d_list, list2, cnt, sse, n_super, static_cast<const double*>(d_cert_e.ptr),
                                         dd, cert_tol, fallback, fb_cap, reasons, stream, count2))) {
        cuda_ok(cudaGetLastError(), "mixed residual launch");
        return RRG_E_CUDA;
      }
      mark_end(P_RESID, t0);
      t0 = mark_begin();
      finalize_kernel<<<(cnt + 127) / 128, 128, 0, stream>>>(dev, dd, d_list, 0, cnt, sse, n_super,
                                                             static_cast<const double*>(d_coefs.ptr), res, 0u,
                                                             static_cast<const double*>(d_sse1.ptr));
      mark_end(P_FINAL, t0);
      launches += 3 + (certify ? 1 : 0);
      // FP64 re-scoring lane over fallback[1 .. 1 + fallback[0])
      t0 = mark_begin();
      RRG_CUDA(cudaMemsetAsync(need, 0, std::max(1, ncol), stream));
      RRG_CUDA(cudaMemsetAsync(cst, 0, sizeof(ColStat) * std::max(1, ncol), stream));
      RRG_CUDA(cudaMemsetAsync(bcount, 0, sizeof(int32_t) * kQrBuckets, stream));
      DevBatch fdev = dev;
      fdev.cands = pf.at<const rrg_cand>(d_fbpack, o_fc);
      fdev.code = pkt.at<const uint32_t>(d_ftp, o_tcode);
      fdev.n_cand = ncol;
      fdev.n_code = (int32_t)tp.code.size();
      clear_results_kernel<<<(cnt + 255) / 256, 256, 0, stream>>>(fb_list, cnt, res, fb_count);
      const int32_t* d_kept = pf.at<const int32_t>(d_fbpack, o_kept);
      if (!launch_rescore_mark(dev.cands, fallback, cnt, pf.at<const int32_t>(d_fbpack, o_liof), d_ccol,
                               pf.at<const int32_t>(d_fbpack, o_doff), pf.at<const int32_t>(d_fbpack, o_deps),
                               n_kept ? d_kept : nullptr, need, stream) ||
          !launch_rescore_levels(need, pf.at<const int32_t>(d_fbpack, o_lend), n_levels, lvl_cols, lvl_count,
                                 stream) ||
          (n_kept && !launch_lane_copy(need, d_kept, ncol, static_cast<const double*>(d_F64.ptr),
                                       static_cast<const ColStat*>(d_ccst.ptr), F64, cst, ds->n_pad, stream))) {
        cuda_ok(cudaGetLastError(), "re-scoring list launch");
        return RRG_E_CUDA;
      }
      last_cache64_hits += n_kept;
      bool wave_trial = false;
      int waves = tune_pick(TK_EVAL_WAVES, 0, ds->n, &wave_trial);
      const int max_nbc = (int)std::max<int64_t>(1, (ds->n + 1023) / 1024);
      auto eval_level = [&](int32_t L, int wv) {
        const int32_t lo = L == 0 ? 0 : tp.level_end[L - 1];
        table_eval_list_kernel<<<std::max(1, wv * sm_count), 256, plain_eval_smem(), stream>>>(
            fdev, dd, pf.at<const PlainCand>(d_fbpack, o_fpc), lvl_cols + lo, lvl_count + L, max_nbc, F64, status,
            cst);
      };
      if (wave_trial && !capturing && n_levels > 0) {
        // the first round of this row class: read the per-level counts back
        // once and time every shape on the widest level (re-evaluating a
        // level rewrites the same columns and statistics)
        std::vector<int32_t> hc(n_levels);
        RRG_CUDA(cudaMemcpyAsync(hc.data(), lvl_count, sizeof(int32_t) * n_levels, cudaMemcpyDeviceToHost, stream));
        RRG_CUDA(cudaStreamSynchronize(stream));
        int32_t widest = 0;
        for (int32_t L = 1; L < n_levels; ++L)
          if (hc[L] > hc[widest]) widest = L;
        if ((int64_t)hc[widest] * ds->n >= kTuneMinWork) {
          for (int32_t L = 0; L < widest; ++L) eval_level(L, waves);  // the columns the widest level reads
          int vals[4];
          float ms[4];
          const int nv = tune_variants(TK_EVAL_WAVES, 0, vals);
          for (int v = 0; v < nv; ++v) {
            rrg_status ts = time_trial([&] { eval_level(widest, vals[v]); }, ms[v]);
            if (ts != RRG_OK) return ts;
          }
          tune_store(TK_EVAL_WAVES, 0, ds->n, vals, ms, nv);
          waves = tune_pick(TK_EVAL_WAVES, 0, ds->n, &wave_trial);
        }
      }
      for (int32_t L = 0; L < n_levels; ++L) eval_level(L, waves);
      sentinel_classify_kernel<<<(cnt + 127) / 128, 128, 0, stream>>>(dev, fb_list, 0, cnt, d_pcs, d_ccol, cst,
                                                                     ds->n, coefs, res, status + kStatusSentinel,
                                                                     fb_count);
      nan_gram_kernel<<<dim3(nbx, cnt), 256, 0, stream>>>(fb_list, cnt, d_pcs, d_ccol, cst, F64, ds->n, ds->n_pad,
                                                          gpart, fb_count);
      nan_gram_decide_kernel<<<(cnt + 127) / 128, 128, 0, stream>>>(dev, fb_list, cnt, d_pcs, d_ccol, cst, nbx, gpart,
                                                                    coefs, res, status + kStatusSentinel, fb_count);
      if (!launch_rescore_buckets(dev.cands, fallback, cnt, d_pcs, blist, bcount, stream)) {
        cuda_ok(cudaGetLastError(), "re-scoring bucket launch");
        return RRG_E_CUDA;
      }
      mark_end(P_PLAIN_EVAL, t0);
      launches += n_levels + 6;
      // the QR of every bucket, side by side on the side streams: the chunked
      // passes over the bucket's list, qbatch[q] candidates per batch
      t0 = mark_begin();
      RRG_CUDA(cudaEventRecord(fork_ev, stream));
      int used = 0;
      size_t m_off = 0, q_off = 0;
      for (int q = 0; q < kQrBuckets; ++q) {
        if (!qbatch[q]) continue;
        cudaStream_t sq = side[used % kSide];
        if (used < kSide) RRG_CUDA(cudaStreamWaitEvent(sq, fork_ev, 0));
        for (int32_t t0b = 0; t0b < bucket_cap[q]; t0b += qbatch[q]) {
          QrJob jb{};
          jb.b = dev;
          jb.ds = dd;
          jb.pc = d_pcs;
          jb.list = blist + (size_t)q * cnt;
          jb.list_off = t0b;
          jb.n_list = qbatch[q];
          jb.dcount = bcount + q;
          jb.A = F64;
          jb.colmap = d_ccol;
          jb.M = Mq + m_off * ds->n_pad;
          jb.slot_cols = kBucketCols[q];
          jb.coefs = coefs;
          jb.res = res;
          jb.status = status;
          jb.count_bytes = 1;
          jb.max_cols = kBucketCols[q];
          jb.max_steps = bucket_wide[q] - 1;
          qr_chunk_bind(jb, static_cast<char*>(d_qrs.ptr) + q_off);
          if (!launch_qr_chunked(jb, qr_blocks(kBucketCols[q], (int64_t)qbatch[q] * nch), sq, &launches)) {
            cuda_ok(cudaGetLastError(), "QR launch");
            return RRG_E_CUDA;
          }
        }
        m_off += (size_t)qbatch[q] * kBucketCols[q];
        q_off += (size_t)round_up((int64_t)qr_chunk_scratch_bytes(qbatch[q], ds->n, kBucketCols[q]), 256);
        ++used;
      }
      for (int i = 0; i < std::min(used, (int)kSide); ++i) {
        RRG_CUDA(cudaEventRecord(join_ev[i], side[i]));
        RRG_CUDA(cudaStreamWaitEvent(stream, join_ev[i], 0));
      }
      mark_end(P_PLAIN_QR, t0);
      t0 = mark_begin();
      plain_resid_kernel<<<dim3(nb_res, cnt), 256, 0, stream>>>(dev, dd, d_pcs, fb_list, 0, F64, coefs, sse, d_ccol,
                                                               fb_count);
      mark_end(P_PLAIN_RESID, t0);
      t0 = mark_begin();
      finalize_kernel<<<(cnt + 127) / 128, 128, 0, stream>>>(dev, dd, fb_list, 0, cnt, sse, nb_res, coefs, res,
                                                             RRG_F_QR_FALLBACK, nullptr, fb_count);
      mark_end(P_FINAL, t0);
      launches += 2;
      // statistics for rrg_last_round_stats: re-scored count, residual-pass
      // count, reasons, columns evaluated per level
      int32_t* hs = static_cast<int32_t*>(h_fbstat.ptr);
      RRG_CUDA(cudaMemcpyAsync(hs, fallback, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
      RRG_CUDA(cudaMemcpyAsync(hs + 1, count2, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
      RRG_CUDA(cudaMemcpyAsync(hs + 2, reasons, sizeof(uint32_t) * kFbReasons, cudaMemcpyDeviceToHost, stream));
      if (n_levels)
        RRG_CUDA(cudaMemcpyAsync(hs + 2 + kFbReasons, lvl_count, sizeof(int32_t) * n_levels, cudaMemcpyDeviceToHost,
                                 stream));
      if (keep64) {
        // the lane's marks, and the factor programs whose columns it may
        // evaluate, for the store into the cache when the next round starts
        if (!h_fbneed.reserve((size_t)std::max(1, ncol))) {
          rrc::set_error("mixed round: staging allocation failed");
          return RRG_E_OOM;
        }
        RRG_CUDA(cudaMemcpyAsync(h_fbneed.ptr, need, (size_t)std::max(1, ncol), cudaMemcpyDeviceToHost, stream));
        LaneStore& ls = lane_store;
        ls.valid = true;
        ls.uid = ds->uid;
        ls.n_pad = ds->n_pad;
        ls.code.clear();
        ls.meta.clear();
        ls.col.clear();
        const double* pool = consts64;
        ls.consts.assign(pool, pool + std::max(0, dev.n_consts));
        for (int32_t l = 0; l < nfl; ++l) {
          if (kept[tp.fcol[l]] >= 0) continue;
          ls.meta.push_back(make_int2((int)ls.code.size(), lmeta[l].y));
          ls.code.insert(ls.code.end(), lcode.begin() + lmeta[l].x, lcode.begin() + lmeta[l].x + lmeta[l].y);
          ls.col.push_back(tp.fcol[l]);
        }
      }
      fbstat_pending = true;
      fbstat_levels = n_levels;
      fbstat_rows = (double)ds->n;
      fbstat_d = ds->d;
      RRG_CUDA(cudaGetLastError());
      if (async_done) *async_done = true;
      return RRG_OK;
    }
  }
  // residual-pass flags (and the fallback list so far) back to the host
  RRG_CUDA(cudaMemcpyAsync(h_fallback.ptr, d_fallback.ptr, back_bytes, cudaMemcpyDeviceToHost, stream));
  RRG_CUDA(cudaStreamSynchronize(stream));
  const int32_t* hf = static_cast<const int32_t*>(h_fallback.ptr);
  const uint8_t* hp2 = reinterpret_cast<const uint8_t*>(hf + fb_cap + 1 + kFbReasons);
  std::vector<int32_t> list2;
  for (int32_t li = 0; li < cnt; ++li)
    if (hp2[list[li]]) list2.push_back(li);
  last_pass2 += (int64_t)list2.size();
  double* sse = static_cast<double*>(d_partial.ptr);
  if (!list2.empty()) {
    if (!h_mlist.reserve(sizeof(int32_t) * list2.size())) {
      rrc::set_error("mixed round: staging allocation failed");
      return RRG_E_OOM;
    }
    std::memcpy(h_mlist.ptr, list2.data(), sizeof(int32_t) * list2.size());
    RRG_CUDA(cudaMemcpyAsync(d_list2, h_mlist.ptr, sizeof(int32_t) * list2.size(), cudaMemcpyHostToDevice, stream));
    ResidArgs ra;
    ra.b = dev;
    ra.ds = dd;
    ra.F = F;
    ra.mlist = d_list;
    ra.list2 = d_list2;
    ra.n2 = (int32_t)list2.size();
    ra.n2_dev = nullptr;
    ra.cand_col = d_cslot;
    ra.terms = static_cast<const MixedTerm*>(d_terms.ptr);
    ra.n_chunks = n_super;
    ra.sse = sse;
    t0 = mark_begin();
    if (!launch_ftab_resid(ra, stream) ||
        (certify && !launch_cert_resid(d_list, d_list2, ra.n2, sse, n_super, static_cast<const double*>(d_cert_e.ptr),
                                       dd, cert_tol, fallback, fb_cap, reasons, stream))) {
      cuda_ok(cudaGetLastError(), "mixed residual launch");
      return RRG_E_CUDA;
    }
    mark_end(P_RESID, t0);
    launches += certify ? 2 : 1;
  }
  t0 = mark_begin();
  finalize_kernel<<<(cnt + 127) / 128, 128, 0, stream>>>(dev, dd, d_list, 0, cnt, sse, n_super,
                                                         static_cast<const double*>(d_coefs.ptr),
                                                         static_cast<rrg_result*>(d_res.ptr), 0u,
                                                         static_cast<const double*>(d_sse1.ptr));
  mark_end(P_FINAL, t0);
  ++launches;
  if (certify && !list2.empty()) {
    // the residual-pass checks may have queued more
    RRG_CUDA(cudaMemcpyAsync(h_fallback.ptr, d_fallback.ptr, sizeof(int32_t) * (fb_cap + 1 + kFbReasons),
                             cudaMemcpyDeviceToHost, stream));
    RRG_CUDA(cudaStreamSynchronize(stream));
  }
  const uint32_t* hr = reinterpret_cast<const uint32_t*>(hf + fb_cap + 1);
  for (int i = 0; i < kFbReasons; ++i) last_reasons[i] += hr[i];
  const int32_t nf = std::min(hf[0], fb_cap);
  fb_all.insert(fb_all.end(), hf + 1, hf + 1 + nf);
  RRG_CUDA(cudaGetLastError());
  return RRG_OK;
}

// ------------------------------------------------- FP64 over the table ----
// The listed candidates (absolute indices) scored by the plain FP64 path's
// arithmetic: their distinct factors evaluated once into an FP64 table, then
// per candidate the direct column-pivoted QR on [factors | 1 | y] (one block
// each), the rebuilt sum's residual and the fitness.  `ft` must describe the
// round's batch.
rrg_status rrg_context::run_fp64_table(const rrg_dataset* ds, const std::vector<int32_t>& list_in,
                                       uint32_t flags_or) {
  if (list_in.empty()) return RRG_OK;
  // candidates ordered by the QR kernel's column bucket, so that each launch
  // uses the smallest register footprint its candidates allow
  auto bucket = [&](int32_t c) {
    const rrg_cand& cd = host_cands[c];
    return plain_qr_bucket(cd.mode == RRG_TUNED ? cd.n_factors + 2 : 2);
  };
  const char* hb = static_cast<const char*>(h_batch.ptr);
  std::vector<int32_t> list(list_in);
  // widest bucket first: its blocks are the longest, so they start first
  std::stable_sort(list.begin(), list.end(), [&](int32_t x, int32_t y) { return bucket(x) > bucket(y); });
  const DevData dd = ds->view();
  const size_t col8 = sizeof(double) * (size_t)ds->n_pad;
  // factors per FP64 table (shared subtree columns come on top: keep room)
  const int64_t fcap =
      std::min<int64_t>(kCacheSlotsMax, std::max<int64_t>(2 * RRG_MAX_TERMS, (int64_t)(scratch_budget_bytes / 3 / col8)));
  const int64_t mcap = std::max<int64_t>(2 * RRG_MAX_TERMS + 2, (int64_t)(scratch_budget_bytes / 2 / col8));
  // FP64 column arena: the table's half of the scratch budget
  const int64_t plimit = fp64_cache_slots(scratch_budget_bytes, ds->n_pad);
  const int nb_res = (int)((ds->n + RR_CHUNK - 1) / RR_CHUNK);
  const size_t n_all = host_cands.size();
  if (!d_partial.reserve(sizeof(double) * n_all * (size_t)nb_res)) {
    rrc::set_error("FP64 round: scratch allocation failed");
    return RRG_E_OOM;
  }
  std::vector<int32_t> lid(ft.meta.size(), -1), lf;
  size_t pos = 0;
  while (pos < list.size()) {
    // candidates whose distinct factors fit the FP64 table
    lf.clear();
    size_t end = pos;
    while (end < list.size()) {
      const int32_t c = list[end];
      const int m = cand_factors(host_cands[c]);
      int fresh = 0;
      for (int s = 0; s < m; ++s) fresh += lid[ft.ids[ft.cand_off[c] + s]] < 0 ? 1 : 0;
      if (end > pos && (int64_t)lf.size() + fresh > fcap) break;
      for (int s = 0; s < m; ++s) {
        const int32_t g = ft.ids[ft.cand_off[c] + s];
        if (lid[g] < 0) {
          lid[g] = (int32_t)lf.size();
          lf.push_back(g);
        }
      }
      ++end;
    }
    const int32_t nfl = (int32_t)lf.size();
    const int32_t ng = (int32_t)(end - pos);
    // table columns (shared transcendental subtrees by level, then the
    // factors), each a one-factor untuned pseudo-candidate writing its column;
    // FP64 values are the same computed inline or through a shared column
    std::vector<uint32_t> lcode;
    std::vector<int2> lmeta(nfl);
    for (int32_t i = 0; i < nfl; ++i) {
      const int2 mt = ft.meta[lf[i]];
      lmeta[i] = make_int2((int)lcode.size(), mt.y);
      lcode.insert(lcode.end(), ft.code.begin() + mt.x, ft.code.begin() + mt.x + mt.y);
    }
    TableProgs tp;
    const double* consts64 = reinterpret_cast<const double*>(hb + off_d);
    if (!build_table_programs(lcode, lmeta, consts64, tp)) {
      rrc::set_error("FP64 round: a factor program could not be parsed");
      return RRG_E_INVALID;
    }
    // Column cache (as in the mixed rounds): FP64 columns of earlier rounds
    // on this dataset are read again, the others evaluated into slots of the
    // FP64 arena; the QR, sentinel and residual kernels address it by slot.
    if (pcache.limit() != plimit || pcache_npad != ds->n_pad) {
      pcache.reset(plimit);
      pcache_npad = ds->n_pad;
    }
    pcache.bind(ds->uid);
    CachePlan cp;
    if (!plan_columns(pcache, cache_on && ds->n >= kCacheMinRows, lcode, lmeta, consts64, tp, cp)) {
      rrc::set_error("FP64 round: the column cache has no room for the table");
      return RRG_E_OOM;
    }
    struct GiveBack {
      ColumnCache& cc;
      std::vector<int32_t>& s;
      ~GiveBack() { cc.give_back(s); }
    } give_back{pcache, cp.scratch};
    const TableProgs& ep = cp.ep;
    const int32_t ne = (int32_t)ep.meta.size();
    last_cache64_hits += cp.hits;
    last_cache64_evals += ne;
    const std::vector<uint32_t>& fcode = ep.code;
    std::vector<rrg_cand> fc(std::max(1, ne));
    std::vector<PlainCand> fpc(std::max(1, ne));
    for (int32_t i = 0; i < ne; ++i) {
      rrg_cand& p = fc[i];
      p.code_offset = ep.meta[i].x;
      p.code_len = ep.meta[i].y;
      p.first_factor = 0;
      p.n_factors = 1;
      p.mode = RRG_UNTUNED;
      p.coef_offset = 0;
      p.stack_need = ep.stack[i];
      p.reserved = 0;
      if (ep.stack[i] > RRG_MAX_STACK) {
        rrc::set_error("FP64 round: a table program exceeds the spill stack");
        return RRG_E_INVALID;
      }
      fpc[i] = PlainCand{cp.ewcol[i], 0, 0, 1, 0};
    }
    // column map and QR working columns; QR sub-batches by the M budget
    std::vector<int32_t> colmap;
    std::vector<PlainCand> pcs(std::max<size_t>(1, n_all));
    std::vector<std::pair<int32_t, int32_t>> subs;  // [first, end) positions in the group list
    int64_t mcol = 0, mcols_max = 1;
    int32_t sub0 = 0;
    for (int32_t i = 0; i < ng; ++i) {
      const int32_t c = list[pos + i];
      const rrg_cand& cd = host_cands[c];
      const int m = cand_factors(cd);
      const int32_t k = cd.mode == RRG_TUNED ? cd.n_factors + 1 : 1;
      const int64_t need = cd.mode == RRG_TUNED ? k + 1 : 0;
      if (i > sub0 && (mcol + need > mcap || i - sub0 >= 65535)) {
        subs.push_back({sub0, i});
        sub0 = i;
        mcol = 0;
      }
      PlainCand& p = pcs[c];
      p.a_col = (int64_t)colmap.size();
      p.m_col = mcol;
      p.s_off = 0;
      p.k = k;
      p.pad = 0;
      mcol += need;
      mcols_max = std::max(mcols_max, mcol);
      for (int s = 0; s < m; ++s) colmap.push_back(cp.fslot[lid[ft.ids[ft.cand_off[c] + s]]]);
    }
    subs.push_back({sub0, ng});
    Packer pk;
    const size_t o_fcode = pk.add(fcode.data(), sizeof(uint32_t) * std::max<size_t>(1, fcode.size()));
    const size_t o_ewcol = pk.add(cp.ewcol.data(), sizeof(int32_t) * std::max<size_t>(1, cp.ewcol.size()));
    const size_t o_fc = pk.add(fc.data(), sizeof(rrg_cand) * fc.size());
    const size_t o_fpc = pk.add(fpc.data(), sizeof(PlainCand) * fpc.size());
    const size_t o_cmap = pk.add(colmap.data(), sizeof(int32_t) * std::max<size_t>(1, colmap.size()));
    const size_t o_pcs = pk.add(pcs.data(), sizeof(PlainCand) * pcs.size());
    const size_t o_list = pk.add(list.data() + pos, sizeof(int32_t) * ng);
    rrg_status pst = pk.send(h_ft64, d_ft64, stream, round_seq);
    if (pst != RRG_OK) return pst;
    const size_t n_slots = (size_t)std::max<int64_t>(1, cp.arena);
    if (!d_F64.grow_keep(col8 * n_slots, d_F64.cap) || !d_M.reserve(col8 * mcols_max) ||
        !d_ccst.grow_keep(sizeof(ColStat) * n_slots, d_ccst.cap)) {
      rrc::set_error("FP64 round: table allocation failed");
      return RRG_E_OOM;
    }
    double* F64 = static_cast<double*>(d_F64.ptr);
    double* M = static_cast<double*>(d_M.ptr);
    const int32_t* d_list = pk.at<const int32_t>(d_ft64, o_list);
    const PlainCand* d_pcs = pk.at<const PlainCand>(d_ft64, o_pcs);
    const int32_t* d_cmap = pk.at<const int32_t>(d_ft64, o_cmap);
    double* coefs = static_cast<double*>(d_coefs.ptr);
    rrg_result* res = static_cast<rrg_result*>(d_res.ptr);
    uint32_t* status = static_cast<uint32_t*>(d_status.ptr);
    double* partial = static_cast<double*>(d_partial.ptr);
    clear_results_kernel<<<(ng + 255) / 256, 256, 0, stream>>>(d_list, ng, res);
    // distinct factors, FP64, the plain evaluator (bit-identical values)
    DevBatch fdev = dev;
    fdev.cands = pk.at<const rrg_cand>(d_ft64, o_fc);
    fdev.code = pk.at<const uint32_t>(d_ft64, o_fcode);
    fdev.n_cand = ne;
    fdev.n_code = (int32_t)fcode.size();
    // column statistics of the table (by slot, kept with the columns),
    // gathered by the evaluator, then the candidates whose QR outcome is
    // certainly the all-NaN sentinel (their QR and residual work is skipped)
    ColStat* cst = static_cast<ColStat*>(d_ccst.ptr);
    static_assert(sizeof(ColStat) == 2 * sizeof(unsigned long long), "ColStat is two words");
    if (!cp.kept)
      RRG_CUDA(cudaMemsetAsync(cst, 0, sizeof(ColStat) * (size_t)std::max(1, ne), stream));
    else if (!launch_fill_slots(pk.at<const int32_t>(d_ft64, o_ewcol), ne, reinterpret_cast<unsigned long long*>(cst),
                                2, 0ull, stream))
      return RRG_E_CUDA;
    cudaEvent_t t0 = mark_begin();
    // one launch (or several of at most 65535 columns) per level; blocks per
    // column from the tuner's SM waves (any value gives the same columns)
    bool wave_trial = false;
    int waves = tune_pick(TK_EVAL_WAVES, 0, ds->n, &wave_trial);
    size_t wave_level = 0;  // a trial times the widest level
    for (size_t L = 0, c0 = 0, widest = 0; L < ep.level_end.size(); c0 = ep.level_end[L++])
      if ((size_t)ep.level_end[L] - c0 > widest) {
        widest = (size_t)ep.level_end[L] - c0;
        wave_level = L;
      }
    for (size_t L = 0, c0 = 0; L < ep.level_end.size(); ++L) {
      const int32_t c1 = ep.level_end[L];
      const int32_t nl = c1 - (int32_t)c0;
      auto eval_level = [&](int wv) {
        const int nb = (int)std::max<int64_t>(
            1, std::min<int64_t>(((int64_t)wv * sm_count + nl - 1) / std::max(1, nl), (ds->n + 1023) / 1024));
        for (int32_t f0 = (int32_t)c0; f0 < c1; f0 += 65535) {
          const int32_t nfb = std::min<int32_t>(65535, c1 - f0);
          plain_eval_kernel<<<dim3(nb, nfb), 256, plain_eval_smem(), stream>>>(
              fdev, dd, pk.at<const PlainCand>(d_ft64, o_fpc), nullptr, f0, F64, status, cst);
          ++launches;
        }
      };
      if (wave_trial && !capturing && L == wave_level && (int64_t)nl * ds->n >= kTuneMinWork) {
        // re-evaluating a level rewrites the same columns: time every shape
        int vals[4];
        float ms[4];
        const int nv = tune_variants(TK_EVAL_WAVES, 0, vals);
        for (int v = 0; v < nv; ++v) {
          rrg_status ts = time_trial([&] { eval_level(vals[v]); }, ms[v]);
          if (ts != RRG_OK) return ts;
        }
        tune_store(TK_EVAL_WAVES, 0, ds->n, vals, ms, nv);
        wave_trial = false;
        waves = tune_pick(TK_EVAL_WAVES, 0, ds->n, &wave_trial);
      } else {
        eval_level(waves);
      }
      c0 = c1;
    }
    sentinel_classify_kernel<<<(ng + 127) / 128, 128, 0, stream>>>(dev, d_list, 0, ng,
                                                                   pk.at<PlainCand>(d_ft64, o_pcs), d_cmap, cst,
                                                                   ds->n, coefs, res, status + kStatusSentinel);
    {
      // NaN columns beyond column 0: the Gram certificate of the finite columns
      const int nbx = (int)std::max<int64_t>(1, std::min<int64_t>(16, (ds->n + 32767) / 32768));
      const size_t gbytes = sizeof(double) * (size_t)ng * nbx * (kGramCols * (kGramCols + 1) / 2);
      if (!d_gram.reserve(gbytes)) {
        rrc::set_error("FP64 round: scratch allocation failed");
        return RRG_E_OOM;
      }
      double* gpart = static_cast<double*>(d_gram.ptr);
      for (int32_t g0 = 0; g0 < ng; g0 += 65535) {
        const int32_t gn = std::min<int32_t>(65535, ng - g0);
        nan_gram_kernel<<<dim3(nbx, gn), 256, 0, stream>>>(d_list + g0, gn, d_pcs, d_cmap, cst, F64, ds->n,
                                                           ds->n_pad, gpart + (size_t)g0 * nbx *
                                                                                  (kGramCols * (kGramCols + 1) / 2));
      }
      nan_gram_decide_kernel<<<(ng + 127) / 128, 128, 0, stream>>>(dev, d_list, ng, pk.at<PlainCand>(d_ft64, o_pcs),
                                                                   d_cmap, cst, nbx, gpart, coefs, res,
                                                                   status + kStatusSentinel);
      launches += 2;
    }
    mark_end(P_PLAIN_EVAL, t0);
    phase_bytes[P_PLAIN_EVAL] += (double)ds->n * 8.0 * (double)(ds->d + ne);
    launches += 2;
    for (const auto& sb : subs) {
      const int32_t ns = sb.second - sb.first;
      if (ns <= 0) continue;
      // one factorisation per register bucket of the sub-batch, side by side
      // on the side streams: one block per candidate while the rows fit one
      // chunk, otherwise the chunked passes over the whole GPU (same bits)
      struct QrRun {
        int32_t b0, b1;
        int bk, wide;
        size_t off;
      };
      std::vector<QrRun> runs;
      const bool chunked = ds->n > RR_CHUNK;
      size_t qbytes = 0;
      for (int32_t b0 = sb.first; b0 < sb.second;) {
        const int bk = bucket(list[pos + b0]);
        int32_t b1 = b0;
        int wide = 2;
        while (b1 < sb.second && bucket(list[pos + b1]) == bk) {
          const rrg_cand& cd = host_cands[list[pos + b1]];
          if (cd.mode == RRG_TUNED) wide = std::max(wide, cd.n_factors + 2);
          ++b1;
        }
        runs.push_back({b0, b1, bk, wide, qbytes});
        if (chunked) qbytes += (size_t)round_up((int64_t)qr_chunk_scratch_bytes(b1 - b0, ds->n, bk), 256);
        b0 = b1;
      }
      if (chunked && !d_qrs.reserve(std::max<size_t>(qbytes, 256))) {
        rrc::set_error("FP64 round: QR scratch allocation failed");
        return RRG_E_OOM;
      }
      t0 = mark_begin();
      RRG_CUDA(cudaEventRecord(fork_ev, stream));
      int used = 0;
      for (const QrRun& r : runs) {
        cudaStream_t s = side[used % kSide];
        if (used < kSide) RRG_CUDA(cudaStreamWaitEvent(s, fork_ev, 0));
        bool ok;
        if (!chunked) {
          ok = launch_plain_qr(r.bk, r.b1 - r.b0, s, dev, dd, d_pcs, d_list, r.b0, F64, M, coefs, res, status, d_cmap);
          ++launches;
        } else {
          QrJob jb{};
          jb.b = dev;
          jb.ds = dd;
          jb.pc = d_pcs;
          jb.list = d_list;
          jb.list_off = r.b0;
          jb.n_list = r.b1 - r.b0;
          jb.dcount = nullptr;
          jb.A = F64;
          jb.colmap = d_cmap;
          jb.M = M;
          jb.slot_cols = 0;
          jb.coefs = coefs;
          jb.res = res;
          jb.status = status;
          jb.count_bytes = 1;
          jb.max_cols = r.bk;
          jb.max_steps = r.wide - 1;
          qr_chunk_bind(jb, static_cast<char*>(d_qrs.ptr) + r.off);
          ok = launch_qr_chunked(jb, qr_blocks(r.bk, (int64_t)jb.n_list * jb.nch), s, &launches);
        }
        if (!ok) {
          cuda_ok(cudaGetLastError(), "QR launch");
          return RRG_E_CUDA;
        }
        ++used;
      }
      for (int i = 0; i < std::min(used, (int)kSide); ++i) {
        RRG_CUDA(cudaEventRecord(join_ev[i], side[i]));
        RRG_CUDA(cudaStreamWaitEvent(stream, join_ev[i], 0));
      }
      mark_end(P_PLAIN_QR, t0);
      t0 = mark_begin();
      plain_resid_kernel<<<dim3(nb_res, ns), 256, 0, stream>>>(dev, dd, d_pcs, d_list, sb.first, F64, coefs, partial,
                                                               d_cmap);
      mark_end(P_PLAIN_RESID, t0);
      t0 = mark_begin();
      finalize_kernel<<<(ns + 127) / 128, 128, 0, stream>>>(dev, dd, d_list, sb.first, sb.second, partial, nb_res,
                                                            coefs, res, flags_or, nullptr);
      mark_end(P_FINAL, t0);
      launches += 3;
    }
    RRG_CUDA(cudaGetLastError());
    for (int32_t g : lf) lid[g] = -1;
    pos = end;
  }
  return RRG_OK;
}

// The factor columns the previous round's re-scoring lane evaluated, from its
// FP64 table into FP64 cache slots (the table is rewritten only by the next
// lane, later on the same stream).  Called when a round starts; a store for
// another dataset, or after the cache was cleared, is dropped.
rrg_status rrg_context::store_lane_columns() {
  if (!lane_store.valid) return RRG_OK;
  LaneStore& ls = lane_store;
  ls.valid = false;
  if (!cache_on || pcache.uid() != ls.uid || pcache_npad != ls.n_pad || ls.col.empty()) return RRG_OK;
  const uint8_t* need = static_cast<const uint8_t*>(h_fbneed.ptr);
  pcache.begin();
  std::vector<int32_t> fsel;
  std::vector<uint64_t> hsel;
  for (size_t f = 0; f < ls.col.size(); ++f) {
    if (need[ls.col[f]] != kNeedEval) continue;
    const FactorProg fp{ls.code.data() + ls.meta[f].x, ls.meta[f].y, ls.consts.data()};
    const uint64_t h = fp.hash();
    if (pcache.find(fp, h) >= 0) continue;  // stored meanwhile
    fsel.push_back((int32_t)f);
    hsel.push_back(h);
  }
  const int64_t k = std::min<int64_t>((int64_t)fsel.size(), pcache.available());
  if (k <= 0) return RRG_OK;
  std::vector<int32_t> slots;
  if (!pcache.take(k, slots)) return RRG_OK;
  std::vector<int32_t> pairs(2 * (size_t)k);
  for (int64_t i = 0; i < k; ++i) {
    const int32_t f = fsel[i];
    pcache.insert(FactorProg{ls.code.data() + ls.meta[f].x, ls.meta[f].y, ls.consts.data()}, hsel[i], slots[i]);
    pairs[2 * i] = ls.col[f];
    pairs[2 * i + 1] = slots[i];
  }
  const size_t col8 = sizeof(double) * (size_t)ls.n_pad;
  const size_t n_slots = (size_t)pcache.size();
  if (!d_F64.grow_keep(col8 * n_slots, d_F64.cap) || !d_ccst.grow_keep(sizeof(ColStat) * n_slots, d_ccst.cap) ||
      !h_store.reserve(sizeof(int32_t) * pairs.size()) || !d_store.reserve(sizeof(int32_t) * pairs.size())) {
    rrc::set_error("column cache: allocation failed");
    return RRG_E_OOM;
  }
  std::memcpy(h_store.ptr, pairs.data(), sizeof(int32_t) * pairs.size());
  RRG_CUDA(cudaMemcpyAsync(d_store.ptr, h_store.ptr, sizeof(int32_t) * pairs.size(), cudaMemcpyHostToDevice, stream));
  if (!launch_cache_store(static_cast<const int32_t*>(d_store.ptr), (int32_t)k, static_cast<const double*>(d_fbF64.ptr),
                          static_cast<const ColStat*>(d_fbcst.ptr), static_cast<double*>(d_F64.ptr),
                          static_cast<ColStat*>(d_ccst.ptr), ls.n_pad, stream))
    return RRG_E_CUDA;
  ++launches;
  return RRG_OK;
}

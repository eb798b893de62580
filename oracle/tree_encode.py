"""ORACLE - test infrastructure only (tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py).  Nothing of the product imports this module.

The oracle's own path from a candidate tree to the batch that
oracle/rrg_oracle.c scores, written independently of the product's host
library, so that the CPU baseline and the oracle side of the parity tests
never run the product's tree code:

  parse        prefix form ("add x0 mul c:2.5 sin x1"), the token syntax of
               the C ABI's trees;
  expand       node::expand, rils_rols_cpp/node.cpp:344-374, quirks included:
               (t1 +- t2) * t3 becomes (t1*t3) * (t3*t3), and t1 * (t2 +- t3)
               becomes (t1*t2) * ((t1*t2)*t3), because the second product is
               built from the freshly assigned left operand and the node keeps
               the type of that product (MULTIPLY);
  simplify     node::simplify, node.cpp:152-296 (constant folding and the
               0 / 1 / nested-constant rules, in the reference's branch order);
  factors      tune_constants' split into top-level non-constant factors and
               its filter (rils_rols_cpp.cpp:445-475, extract_non_constant_factors
               node.cpp:140-147); the free term is added by the scorer;
  encode       postfix programs in the C ABI's code words
               (include/rils_rols_gb300.h: rrg_op), one program per factor,
               children in Sethi-Ullman order with plain spill-stack operands.

The result of tune_constants + fitness does not depend on the evaluation
order of a tree's nodes (every node is one IEEE operation on its children's
values), so any valid postfix order gives the reference's values.

Python's float arithmetic is IEEE binary64 with round-to-nearest, the same
as the reference's doubles; the operations that raise in Python (division by
zero, pow domain and range errors) are done through numpy float64 scalars,
whose pow is the C library's.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

# node_type (rils_rols_cpp/node.h:16-38)
NONE, CONST, VAR, PLUS, MINUS, MUL, DIV, SIN, COS, LN, EXP, SQRT, SQR, POW, LT, GT, EQ, NE, MIN, MAX = range(20)
UNARY_TYPES = (SIN, COS, LN, EXP, SQRT, SQR)
TOKENS = {"add": PLUS, "sub": MINUS, "mul": MUL, "div": DIV, "sin": SIN, "cos": COS, "ln": LN, "exp": EXP,
          "sqrt": SQRT, "sqr": SQR, "pow": POW, "lt": LT, "gt": GT, "eq": EQ, "ne": NE, "min": MIN, "max": MAX}
NAMES = {v: k for k, v in TOKENS.items()}
EPS = 1e-12  # pow(10, -PRECISION), node.h:13-14


def arity_of(t: int) -> int:
    """get_arity, node.h:40-56 (NONE counts as binary there)"""
    if t in (CONST, VAR):
        return 0
    if t in UNARY_TYPES:
        return 1
    return 2


def value_zero(v: float) -> bool:
    return abs(v) < EPS


def value_one(v: float) -> bool:
    return abs(v - 1) < EPS


def _div(a: float, b: float) -> float:
    with np.errstate(all="ignore"):
        return float(np.float64(a) / np.float64(b))


def _pow(a: float, b: float) -> float:
    with np.errstate(all="ignore"):
        return float(np.power(np.float64(a), np.float64(b)))


def fold(t: int, a: float, b: float) -> float:
    """The constant folding of node::simplify, node.cpp:162-190"""
    if t == PLUS:
        return a + b
    if t == MINUS:
        return a - b
    if t == MUL:
        return a * b  # overflow gives inf (Python float multiplication does not raise)
    if t == DIV:
        return _div(a, b)
    if t == POW:
        return _pow(a, b)
    if t == LT:
        return 1.0 if a < b else 0.0
    if t == GT:
        return 1.0 if a > b else 0.0
    if t == EQ:
        return 1.0 if a == b else 0.0
    if t == NE:
        return 1.0 if a != b else 0.0
    if t == MIN:
        return a if a < b else b
    if t == MAX:
        return a if a > b else b
    raise ValueError(f"constant folding: no rule for node type {t}")


class Node:
    """A tree node with the reference's field set (node.h:70-77).  Children
    are shared references, as the reference's shared_ptr members are."""
    __slots__ = ("type", "arity", "left", "right", "value", "var")

    def __init__(self, t: int, left: "Node | None" = None, right: "Node | None" = None, value: float = 0.0,
                 var: int = -1):
        self.type = t
        self.arity = arity_of(t)
        self.left = left
        self.right = right
        self.value = value
        self.var = var

    # node.h:130-139
    def update_with(self, src: "Node") -> None:
        self.left, self.right, self.arity = src.left, src.right, src.arity
        self.value, self.var, self.type = src.value, src.var, src.type

    # node.h:196-201
    def set_type(self, t: int) -> None:
        self.type = t
        self.arity = arity_of(t)

    # node.h:215-221
    def set_const_value(self, v: float) -> None:
        self.set_type(CONST)
        self.value = v
        self.left = None
        self.right = None

    def size(self) -> int:
        """node.h:311-322"""
        if self.arity == 0:
            return 1
        if self.arity == 1:
            return 1 + self.left.size()
        return 1 + self.left.size() + self.right.size()

    def prefix(self) -> str:
        """Prefix form, constants with 17 significant digits."""
        out: list[str] = []

        def rec(n: Node):
            if n.type == VAR:
                out.append(f"x{n.var}")
            elif n.type == CONST:
                out.append("c:" + _g17(n.value))
            else:
                out.append(NAMES[n.type])
                rec(n.left)
                if n.arity == 2:
                    rec(n.right)

        rec(self)
        return " ".join(out)

    # --------------------------------------------------------- expand ----
    def expand(self) -> None:
        """node::expand, node.cpp:344-374"""
        if self.arity == 0:
            return
        if self.arity == 1:
            self.left.expand()
            return
        self.left.expand()
        self.right.expand()
        if self.type != MUL:
            return
        if self.left.type in (PLUS, MINUS):
            if self.right.type in (PLUS, MINUS):
                self.update_with(_binomial(self.left, self.right))
            else:
                self.left = make_copy(MUL, self.left.left, self.right)
                # the right product takes the new left product's right operand
                self.right = make_copy(MUL, self.left.right, self.right)
                self.set_type(self.left.type)
        elif self.right.type in (PLUS, MINUS):
            self.left = make_copy(MUL, self.left, self.right.left)
            # the right product takes the new left product as its left operand
            self.right = make_copy(MUL, self.left, self.right.right)
            self.set_type(self.right.type)

    # ------------------------------------------------------- simplify ----
    def simplify(self) -> None:
        """node::simplify, node.cpp:152-296"""
        if self.arity == 0:
            return
        if self.arity == 1:
            self.left.simplify()
            return
        L, R, t = self.left, self.right, self.type
        L.simplify()
        R.simplify()
        L, R = self.left, self.right
        if L.type == CONST and R.type == CONST:
            self.value = fold(t, L.value, R.value)
            self.arity = 0
            self.type = CONST
            self.left = None
            self.right = None
        elif L.type == CONST:
            if t in (PLUS, MINUS):
                if value_zero(L.value):
                    self.update_with(R)  # 0 + t = t and 0 - t = t
                elif R.type in (PLUS, MINUS):
                    if R.left.type == CONST:
                        L.value = L.value + R.left.value if t == PLUS else L.value - R.left.value
                        R.update_with(R.right)
                    elif R.right.type == CONST:
                        if t == PLUS:
                            L.value = L.value + R.right.value if R.type == PLUS else L.value - R.right.value
                        else:
                            L.value = L.value - R.right.value if R.type == PLUS else L.value + R.right.value
                        R.update_with(R.left)
            elif t == MUL:
                if value_zero(L.value):
                    self.set_const_value(0.0)
                elif value_one(L.value):
                    self.update_with(R)
                elif R.type == MUL:
                    if R.left.type == CONST:
                        L.value = _mul(L.value, R.left.value)
                        R.update_with(R.right)
                    elif R.right.type == CONST:
                        L.value = _mul(L.value, R.right.value)
                        R.update_with(R.left)
            elif t == DIV and value_zero(L.value):
                self.set_const_value(0.0)
        elif R.type == CONST:
            if t in (PLUS, MINUS):
                if value_zero(R.value):
                    self.update_with(L)
                elif L.type in (PLUS, MINUS):
                    if L.left.type == CONST:
                        L.left.value = L.left.value + R.value if t == PLUS else L.left.value - R.value
                        R.value = 0.0
                    elif L.right.type == CONST:
                        R.value = R.value + L.right.value if L.type == PLUS else R.value - L.right.value
                        L.right.value = 0.0
            elif t == MUL:
                if value_one(R.value):
                    self.update_with(L)
                elif value_zero(R.value):
                    self.set_const_value(0.0)
                elif L.type == MUL:
                    if L.left.type == CONST:
                        R.value = _mul(R.value, L.left.value)
                        L.update_with(L.right)
                    elif L.right.type == CONST:
                        R.value = _mul(R.value, L.right.value)
                        L.update_with(L.left)


def _mul(a: float, b: float) -> float:
    return a * b


def _g17(v: float) -> str:
    s = "%.17g" % v
    return s


def deep_copy(n: Node) -> Node:
    """node::node_copy, node.h:141-148"""
    c = Node(n.type, None, None, n.value, n.var)
    c.arity = n.arity
    if n.left is not None:
        c.left = deep_copy(n.left)
    if n.right is not None:
        c.right = deep_copy(n.right)
    return c


def make_copy(t: int, left: Node, right: Node | None = None) -> Node:
    """create_node_ptr, node.h:334-337: a new node over deep copies"""
    return Node(t, deep_copy(left), deep_copy(right) if right is not None else None)


def _binomial(L: Node, R: Node) -> Node:
    """binomial_mult, node.cpp:332-342"""
    f1 = make_copy(MUL, L.left, R.left)
    f2 = make_copy(MUL, L.left, R.right)
    f3 = make_copy(MUL, L.right, R.left)
    f4 = make_copy(MUL, L.right, R.right)
    return Node(L.type, Node(R.type, f1, f2), Node(R.type, f3, f4))


def parse(tree: str) -> Node:
    toks = tree.split()
    pos = 0

    def rec() -> Node:
        nonlocal pos
        if pos >= len(toks):
            raise ValueError(f"truncated tree: {tree!r}")
        t = toks[pos]
        pos += 1
        if t[0] == "x":
            return Node(VAR, var=int(t[1:]))
        if t.startswith("c:"):
            return Node(CONST, value=float(t[2:]))
        ty = TOKENS.get(t)
        if ty is None:
            raise ValueError(f"unknown token {t!r}")
        left = rec()
        right = rec() if arity_of(ty) == 2 else None
        return Node(ty, left, right)

    root = rec()
    if pos != len(toks):
        raise ValueError(f"trailing tokens in {tree!r}")
    return root


def top_level_factors(n: Node, out: list[Node]) -> None:
    """extract_non_constant_factors, node.cpp:140-147"""
    if n.type in (PLUS, MINUS):
        top_level_factors(n.left, out)
        top_level_factors(n.right, out)
    elif n.type != CONST:
        out.append(n)


def tuned_factors(tree: Node) -> list[Node]:
    """The factors tune_constants fits (rils_rols_cpp.cpp:448-473), free term
    excluded; the tree is expanded and simplified in place, as there."""
    tree.expand()
    tree.simplify()
    found: list[Node] = []
    top_level_factors(tree, found)
    out = []
    for f in found:
        if f.type == CONST:
            continue
        if f.arity == 2 and f.left.type == CONST and f.right.type == CONST:
            continue
        if f.type in (MUL, PLUS, MINUS):
            if f.left.type == CONST:
                out.append(f.right)
                continue
            if f.right.type == CONST:
                out.append(f.left)
                continue
        if f.type == DIV and f.right.type == CONST:
            out.append(f.left)
            continue
        out.append(f)
    return out


# ------------------------------------------------------------ programs ----
# code words of include/rils_rols_gb300.h
OP_LDV, OP_LDC, OP_PSV, OP_PSC, OP_EMIT, OP_BIN = 1, 2, 3, 4, 11, 16
UNARY_OP = {SIN: 5, COS: 6, LN: 7, EXP: 8, SQRT: 9, SQR: 10}
BIN_BASE = {PLUS: 0, MINUS: 1, MUL: 2, DIV: 3, POW: 4, LT: 5, EQ: 6, NE: 7, MIN: 8, MAX: 9}
SRC_S, DIR_N, DIR_R = 0, 0, 1
MAX_STACK = 16
MAX_TERMS = 64


def _word(op: int, arg: int = 0) -> int:
    return (op & 0xFF) | (arg << 8)


def _bin_word(base: int, direction: int) -> int:
    return _word(OP_BIN + 8 * base + 2 * SRC_S + direction)


def _need(n: Node, memo: dict) -> int:
    """spill-stack slots the subtree needs (Sethi-Ullman)"""
    if n.arity == 0:
        return 0
    k = id(n)
    if k in memo:
        return memo[k]
    if n.arity == 1:
        v = _need(n.left, memo)
    else:
        a, b = _need(n.left, memo), _need(n.right, memo)
        v = max(a, b + 1) if a >= b else max(b, a + 1)
    memo[k] = v
    return v


class _Prog:
    def __init__(self, consts: list[float]):
        self.code: list[int] = []
        self.consts = consts
        self.sp = 0
        self.depth = 0
        self.memo: dict = {}

    def emit(self, n: Node, live: bool) -> None:
        if n.arity == 0:
            if live:
                self.sp += 1
                self.depth = max(self.depth, self.sp)
            if n.type == VAR:
                self.code.append(_word(OP_PSV if live else OP_LDV, n.var))
            else:
                self.code.append(_word(OP_PSC if live else OP_LDC, len(self.consts)))
                self.consts.append(n.value)
            return
        if n.arity == 1:
            self.emit(n.left, live)
            self.code.append(_word(UNARY_OP[n.type]))
            return
        if n.type == GT:
            # a > b is b < a (node.cpp:61-68)
            base, first, second = BIN_BASE[LT], n.right, n.left
        else:
            base, first, second = BIN_BASE[n.type], n.left, n.right
        # TOS = op(first, second)
        if _need(first, self.memo) >= _need(second, self.memo):
            self.emit(first, live)
            self.emit(second, True)
            self.code.append(_bin_word(base, DIR_N))  # TOS = op(spilled first, TOS second)
        else:
            self.emit(second, live)
            self.emit(first, True)
            self.code.append(_bin_word(base, DIR_R))  # TOS = op(TOS first, spilled second)
        self.sp -= 1


class CandStruct(C.Structure):
    _fields_ = [("code_offset", C.c_int32), ("code_len", C.c_int32), ("first_factor", C.c_int32),
                ("n_factors", C.c_int32), ("mode", C.c_int32), ("coef_offset", C.c_int32),
                ("stack_need", C.c_int32), ("reserved", C.c_int32)]


class FactorStruct(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("reserved", C.c_int32)]


class BatchStruct(C.Structure):
    _fields_ = [("n_cand", C.c_int32), ("n_factors", C.c_int32), ("n_code", C.c_int32), ("n_consts", C.c_int32),
                ("cands", C.POINTER(CandStruct)), ("factors", C.POINTER(FactorStruct)),
                ("code", C.POINTER(C.c_uint32)), ("consts", C.POINTER(C.c_double))]


CAND_DT = np.dtype([(n, np.int32) for n, _ in CandStruct._fields_])
FACT_DT = np.dtype([(n, np.int32) for n, _ in FactorStruct._fields_])
UNTUNED, TUNED = 0, 1


@dataclass
class OracleBatch:
    """An rrg_batch (include/rils_rols_gb300.h) made by this module."""
    cands: np.ndarray
    factors: np.ndarray
    code: np.ndarray
    consts: np.ndarray
    n_coefs: int

    def __len__(self) -> int:
        return len(self.cands)

    def struct(self) -> BatchStruct:
        b = BatchStruct()
        b.n_cand, b.n_factors = len(self.cands), len(self.factors)
        b.n_code, b.n_consts = len(self.code), len(self.consts)
        b.cands = self.cands.ctypes.data_as(C.POINTER(CandStruct))
        b.factors = self.factors.ctypes.data_as(C.POINTER(FactorStruct))
        b.code = self.code.ctypes.data_as(C.POINTER(C.c_uint32))
        b.consts = self.consts.ctypes.data_as(C.POINTER(C.c_double))
        return b


def encode(trees: list[str], tuned: bool = True) -> OracleBatch:
    """Candidates in prefix form -> the batch oracle/rrg_oracle.c scores:
    tuned = tune_constants + fitness (rils_rols_cpp.cpp:445-541), untuned =
    fitness of the tree as given (:520-541)."""
    cands, factors, code, consts = [], [], [], []
    coef_off = 0
    for tree in trees:
        root = parse(tree)
        facs = tuned_factors(root) if tuned else [root]
        if tuned and len(facs) + 1 > MAX_TERMS:
            raise ValueError(f"{len(facs)} factors exceed the batch format's {MAX_TERMS - 1}: {tree!r}")
        start, depth = len(code), 0
        first = len(factors)
        for slot, f in enumerate(facs):
            p = _Prog(consts)
            p.emit(f, False)
            p.code.append(_word(OP_EMIT, slot))
            if p.depth > MAX_STACK:
                raise ValueError(f"a factor needs {p.depth} spill slots (at most {MAX_STACK}): {tree!r}")
            code.extend(p.code)
            depth = max(depth, p.depth)
            factors.append((f.size(), 0))
        cands.append((start, len(code) - start, first, len(facs), TUNED if tuned else UNTUNED,
                      coef_off if tuned else 0, depth, 0))
        if tuned:
            coef_off += len(facs) + 1
    return OracleBatch(np.array(cands, dtype=CAND_DT).reshape(-1), np.array(factors, dtype=FACT_DT).reshape(-1),
                       np.array(code, dtype=np.uint32), np.array(consts, dtype=np.float64), coef_off)


def rewrite(tree: str, what: int) -> str:
    """Prefix forms of the rewriting steps, for pinning against the
    reference's own: 1 expand, 2 simplify, 5 the tuned factors (one per line)."""
    root = parse(tree)
    if what == 1:
        root.expand()
    elif what == 2:
        root.simplify()
    elif what == 5:
        return "".join(f.prefix() + "\n" for f in tuned_factors(root))
    return root.prefix()

"""Host tree IR and candidate generation against the reference (golden vectors
produced by the reference's own node.cpp / rils_rols_cpp.cpp, tests/golden/)."""
import ctypes as C
import hashlib

BUF = C.create_string_buffer(1 << 26)


def _call(fn, *args):
    r = fn(*args, BUF, len(BUF))
    assert r >= 0, BUF.value[:200]
    return BUF.value.decode()


def test_rewrite_primitives(golden, lib):
    # to_string, expand, simplify, normalize_factor_constants, clean-up loop, tune_constants factors
    for case in golden("rewrite"):
        for what, want in enumerate(case["out"]):
            got = _call(lib.rrh_rewrite, case["tree"].encode(), what)
            assert got == want, (case["tree"], what)


def test_candidate_lists(golden, lib):
    # all_candidates (rils_rols_cpp.cpp:348-443): same candidates, same order, same text keys
    for case in golden("candidates"):
        got = _call(lib.rrh_candidates, case["tree"].encode(), case["local_search"], case["d"],
                    case["classification"])
        lines = got.split("\n")
        assert lines[:5] == case["head"], case["tree"]
        assert len(lines) - 1 == case["count"], case["tree"]
        assert hashlib.sha256(got.encode()).hexdigest() == case["sha256"], case["tree"]


def test_expand_quirk(lib):
    # node.cpp:361-363: (t1+t2)*t3 expands to (t1*t3)*(t3*t3) (the right product
    # is built from the freshly built left product's right operand)
    got = _call(lib.rrh_rewrite, b"mul add x0 x1 x2", 1)
    assert got.split("\t")[0] == "((x0*x2)*(x2*x2))"
    got = _call(lib.rrh_rewrite, b"mul x0 add x1 x2", 1)
    assert got.split("\t")[0] == "((x0*x1)*((x0*x1)*x2))"


def test_to_string_quirks(lib):
    # node.h:286-293 prints '<' for >, ==, !=; constants within 1e-12 of an integer print as ints
    got = _call(lib.rrh_rewrite, b"gt x0 c:2.0000000000001", 0)
    assert got.split("\t")[0] == "(x0<2)"
    got = _call(lib.rrh_rewrite, b"ne x0 c:2.00001", 0)
    assert got.split("\t")[0] == "(x0<2.000010)"
    got = _call(lib.rrh_rewrite, b"eq x0 c:3.0000000000000004", 0)
    assert got.split("\t")[0] == "(x0<3)"


def test_malformed_tree_is_an_error(lib):
    assert lib.rrh_rewrite(b"add x0", 0, BUF, len(BUF)) != 0
    assert lib.rrh_rewrite(b"frob x0", 0, BUF, len(BUF)) != 0

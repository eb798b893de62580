"""The oracle's own tree encoder (oracle/tree_encode.py, written apart from the
product's host library) against the reference: its rewriting steps against
the reference's expand / simplify / factor split (golden rewrite.json), and
its batches scored by oracle/rrg_oracle.c against the reference's
tune_constants + fitness (golden fitness.json), bit for bit."""
import numpy as np
import pytest

from oracle import pyoracle, tree_encode


def test_rewrites_match_reference(golden):
    for case in golden("rewrite"):
        for what in (0, 1, 2):
            want = case["out"][what].split("\t")[1]
            assert tree_encode.rewrite(case["tree"], what) == want, (case["tree"], what)
        want5 = "".join(line.split("\t")[1] + "\n" for line in case["out"][5].split("\n") if line)
        assert tree_encode.rewrite(case["tree"], 5) == want5, case["tree"]


def test_expand_quirks():
    # node.cpp:361-369: the second product is built from the new left product
    assert tree_encode.rewrite("mul add x0 x1 x2", 1) == "mul mul x0 x2 mul x2 x2"
    assert tree_encode.rewrite("mul x0 add x1 x2", 1) == "mul mul x0 x1 mul mul x0 x1 x2"


@pytest.mark.parametrize("name", ["toy", "rand257x3", "cls120x4", "tiny3x2"])
def test_oracle_encoder_fitness_matches_reference(golden, name):
    spec = golden("fitness")[name]
    ods = pyoracle.OracleDataset(np.array(spec["X"]), np.array(spec["y"]))
    trees = [c["tree"] for c in spec["cases"]]
    for tuned, key in ((True, "tuned"), (False, "untuned")):
        out = ods.evaluate(tree_encode.encode(trees, tuned=tuned))
        for i, case in enumerate(spec["cases"]):
            got = [out["loss"][i], out["rmse"][i], int(out["size"][i])]
            assert got == case[key]["fit"], (name, key, case["tree"], got, case[key]["fit"])


def test_oracle_encoder_agrees_with_product_encoder(golden, lib):
    # the same scores whichever encoder made the batch (the product's programs
    # use superinstructions and shared-operand forms, the oracle's plain ones)
    from rils_rols_gb300.fitness import encode
    spec = golden("fitness")["rand257x3"]
    ods = pyoracle.OracleDataset(np.array(spec["X"]), np.array(spec["y"]))
    trees = [c["tree"] for c in spec["cases"]]
    a = ods.evaluate(tree_encode.encode(trees))
    b = ods.evaluate(encode(trees))
    for f in ("loss", "rmse", "size", "rank"):
        assert np.array_equal(a[f], b[f], equal_nan=True), f
    for x, y in zip(a["coefs"], b["coefs"]):
        assert np.array_equal(x, y, equal_nan=True)


def test_malformed_trees_raise():
    for bad in ("add x0", "frob x0", "x0 x1"):
        with pytest.raises(ValueError):
            tree_encode.encode([bad])

"""The benchmark's local-search rounds: the committed list
(tests/golden/ls_rounds_regression_1m.txt.gz, made by the reference's own
all_candidates through tests/golden/make_workload.py) is what the product's
candidate generator gives for the same models, round by round, and the
oracle's own encoder takes every candidate."""
import gzip

from oracle import tree_encode
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import candidates

from conftest import GOLDEN


def load_rounds():
    rounds = {}
    for line in gzip.open(GOLDEN / "ls_rounds_regression_1m.txt.gz", "rt").read().splitlines():
        r, tree = line.split("\t")
        rounds.setdefault(int(r), []).append(tree)
    return [rounds[k] for k in sorted(rounds)]


def test_rounds_match_product_generator(lib):
    rounds = load_rounds()
    assert len(rounds) == len(synth.REGRESSION_1M_TRAJECTORY)
    for model, want in zip(synth.REGRESSION_1M_TRAJECTORY, rounds):
        assert candidates(model, 5, local_search=True) == want, model


def test_oracle_encoder_takes_every_candidate():
    trees = [t for r in load_rounds() for t in r]
    b = tree_encode.encode(trees)
    assert len(b) == len(trees) == 7083
    assert int(b.cands["stack_need"].max()) <= tree_encode.MAX_STACK

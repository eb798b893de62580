"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is downloaded or copied: every input is generated here from a seed.
Trees are in the prefix token form of the C ABI ("add x0 mul c:2.5 sin x1").
"""
from __future__ import annotations

import math
import random

import numpy as np

UNARY = ("sin", "cos", "ln", "exp", "sqrt")
BINARY = ("add", "sub", "mul", "div")
CLS_BINARY = ("lt", "gt", "eq", "ne", "min", "max")


def random_tree(rng: np.random.Generator, size: int, d: int, unary=UNARY, binary=BINARY,
                const_range=(-5.0, 5.0), p_var: float = 0.5) -> str:
    """A random expression tree with exactly `size` nodes: operators drawn
    uniformly from unary + binary, leaves x_j or U(const_range) constants."""
    out: list[str] = []

    def leaf():
        if rng.random() < p_var:
            out.append(f"x{int(rng.integers(d))}")
        else:
            out.append(f"c:{float(rng.uniform(*const_range))!r}")

    def rec(s: int):
        if s == 1:
            leaf()
            return
        ops = unary + (binary if s >= 3 else ())
        op = ops[int(rng.integers(len(ops)))]
        out.append(op)
        if op in unary:
            rec(s - 1)
        else:
            left = int(rng.integers(1, s - 1))
            rec(left)
            rec(s - 1 - left)

    rec(size)
    return " ".join(out)


def eval_tree(tree: str, X: np.ndarray) -> np.ndarray:
    """FP64 numpy evaluation of a prefix tree (columns of X are features)."""
    toks = tree.split()
    pos = 0
    fns1 = {"sin": np.sin, "cos": np.cos, "ln": np.log, "exp": np.exp, "sqrt": np.sqrt, "sqr": np.square}
    fns2 = {"add": np.add, "sub": np.subtract, "mul": np.multiply, "div": np.divide, "pow": np.power,
            "lt": lambda a, b: (a < b) * 1.0, "gt": lambda a, b: (a > b) * 1.0, "eq": lambda a, b: (a == b) * 1.0,
            "ne": lambda a, b: (a != b) * 1.0, "min": lambda a, b: np.where(a < b, a, b),
            "max": lambda a, b: np.where(a > b, a, b)}

    def rec():
        nonlocal pos
        t = toks[pos]
        pos += 1
        if t[0] == "x":
            return X[:, int(t[1:])].astype(np.float64)
        if t.startswith("c:"):
            return np.full(X.shape[0], float(t[2:]))
        if t in fns1:
            return fns1[t](rec())
        a = rec()
        b = rec()
        return fns2[t](a, b)

    with np.errstate(all="ignore"):
        return rec()


def toy_example(seed: int = 12345, samples: int = 200):
    """The two-feature toy problem with y = sin(x1) - 78.8 ln(x2) + 4 x1 + 3.31 x2,
    x ~ integer U[1, 100], split 75/25 the way sklearn's train_test_split does
    with random_state=seed (a permutation of a numpy RandomState)."""
    r = random.Random(seed)
    x1 = [r.randint(1, 100) for _ in range(samples)]
    x2 = [r.randint(1, 100) for _ in range(samples)]
    X = np.array(list(zip(x1, x2)), dtype=np.float64)
    y = np.array([math.sin(a) - 78.8 * math.log(b) + 4 * a + 3.31 * b for a, b in zip(x1, x2)])
    n_test = int(math.ceil(0.25 * samples))
    n_train = int(math.floor(0.75 * samples))
    perm = np.random.RandomState(seed).permutation(samples)
    test, train = perm[:n_test], perm[n_test:n_test + n_train]
    return X[train], X[test], y[train], y[test]


def finite_target(rng, X, size, tries=1000):
    for _ in range(tries):
        t = random_tree(rng, size, X.shape[1])
        v = eval_tree(t, X)
        if np.all(np.isfinite(v)) and np.std(v) > 1e-6:
            return t, v
    raise RuntimeError("could not draw a finite target tree")


def batched_fitness(n: int = 100_000, d: int = 10, n_trees: int = 8192, seed: int = 12345,
                    min_size: int = 3, max_size: int = 50):
    """8192 random candidate trees (sizes U{3..50}) over +,-,*,/,sin,cos,ln,exp,sqrt;
    X ~ N(0,1); y = a random 15-node tree + N(0, (0.01 std y)^2)."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d))
    ty, y = finite_target(rng, X, 15)
    y = y + rng.normal(0.0, 0.01 * np.std(y), n)
    trees = [random_tree(rng, int(rng.integers(min_size, max_size + 1)), d) for _ in range(n_trees)]
    return X, y, trees, ty


def regression_1m(n: int = 1_000_000, seed: int = 12345):
    """d=5, X ~ U(-3,3), y = 2.5 x1 x2 - sin(x3)/(1+x4^2) + 0.7 exp(0.3 x5) + N(0, (0.005 std y)^2)."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3.0, 3.0, (n, 5))
    y = 2.5 * X[:, 0] * X[:, 1] - np.sin(X[:, 2]) / (1 + X[:, 3] ** 2) + 0.7 * np.exp(0.3 * X[:, 4])
    y = y + rng.normal(0.0, 0.005 * np.std(y), n)
    return X, y


def classifier(n: int = 569, d: int = 30, seed: int = 12345, flip: float = 0.05):
    """d correlated lognormal features (pairwise correlation 0.5); labels = (random
    10-node tree > 0) with `flip` of them flipped."""
    rng = np.random.default_rng(seed)
    cov = np.full((d, d), 0.5) + 0.5 * np.eye(d)
    Z = rng.multivariate_normal(np.zeros(d), cov, size=n)
    X = np.exp(Z)
    for _ in range(1000):
        t = random_tree(rng, 10, d)
        v = eval_tree(t, X)
        lab = (v > 0).astype(np.float64)
        if np.all(np.isfinite(v)) and 0.1 < lab.mean() < 0.9:
            break
    flips = rng.random(n) < flip
    lab[flips] = 1.0 - lab[flips]
    return X, lab, t


def serving_stream(n_jobs: int = 1000, rate: float = 5.0, seed: int = 12345, n_min: int = 200,
                   n_max: int = 1_000_000, d_max: int = 20):
    """Poisson arrivals (mean `rate`/s) of fit jobs: n log-uniform in [n_min, n_max],
    d uniform in [1, d_max], X ~ N(0,1), y = random 5-25-node tree + 1% noise."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for j in range(n_jobs):
        t += rng.exponential(1.0 / rate)
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        d = int(rng.integers(1, d_max + 1))
        jobs.append({"id": j, "arrival": t, "n": n, "d": d, "seed": int(rng.integers(1 << 31)),
                     "size": int(rng.integers(5, 26))})
    return jobs


def serving_job_data(job: dict):
    rng = np.random.default_rng(job["seed"])
    X = rng.standard_normal((job["n"], job["d"]))
    _, y = finite_target(rng, X, job["size"])
    y = y + rng.normal(0.0, 0.01 * np.std(y), job["n"])
    return X, y


# Intermediate models of a search on the 1M-row regression problem (prefix
# form), from a single product term to the full generating formula; the
# local-search rounds around them are the benchmark's candidate batches.
REGRESSION_1M_TRAJECTORY = [
    "mul c:2.5 mul x0 x1",
    "add mul c:2.5 mul x0 x1 c:1.1",
    "add mul c:2.5 mul x0 x1 mul c:0.7 exp mul c:0.3 x4",
    "add mul c:2.48 mul x0 x1 mul c:0.93 exp x4",
    "add add mul c:2.49 mul x0 x1 mul c:0.71 exp mul c:0.29 x4 mul c:-0.98 sin x2",
    "add add mul c:2.5 mul x0 x1 mul c:0.7 exp mul c:0.3 x4 mul c:-1 div sin x2 add c:1 sqr x3",
    "add add mul c:2.5 mul x0 x1 mul c:0.7 exp mul c:0.3 x4 div sin x2 sqr x3",
    "sub add mul c:2.5 mul x0 x1 mul c:0.7 exp mul c:0.3 x4 div sin x2 add c:1 mul x3 x3",
]


def ls_round_batch(d: int = 5, trajectory=None) -> list[str]:
    """Local-search candidates (tuned fitness inputs) of every model in the
    trajectory, concatenated in round order."""
    from .fitness import candidates
    out = []
    for t in trajectory or REGRESSION_1M_TRAJECTORY:
        out.extend(candidates(t, d, local_search=True))
    return out

"""scikit-learn style estimators with the interface of the reference's
`rils_rols.rils_rols` module (rils_rols/rils_rols.py:16-190):
RILSROLSRegressor and RILSROLSBinaryClassifier, same constructor arguments,
fit / predict / score / model_string / fit_report_string, predict_proba for
the classifier, and sample_size = 0 for automatic sample-size tuning.

The search runs in the host driver of librils_rols_gb300.so through the
module `rils_rols_cpp` of this package (the reference's pybind11 module
name), and every candidate fitness is computed by the GB300 device path.

Differences a caller can see:
  * pandas is optional (anything with `.values` is converted), and so are
    scikit-learn (get_params / set_params come from a small base class when
    it is missing; the auto-tuning split then uses a seeded permutation) and
    sympy (without it the simplified model is the raw model string);
  * the constructor prints its arguments only when verbose;
  * `precision` selects the arithmetic: "plain" (FP64, the reference's
    numbers, default) or "mixed" (certified mixed precision);
  * bad input raises instead of ending the process.
"""
from __future__ import annotations

import inspect
import threading
import time
from math import inf

import numpy as np

import rils_rols_cpp

try:  # optional: scikit-learn's estimator base
    from sklearn.base import BaseEstimator as _EstimatorBase
except ImportError:  # pragma: no cover - exercised where sklearn is absent
    class _EstimatorBase:
        """get_params / set_params over the constructor's named arguments."""

        @classmethod
        def _param_names(cls):
            sig = inspect.signature(cls.__init__)
            return [p for p in sig.parameters if p != "self"]

        def get_params(self, deep=True):
            return {k: getattr(self, k) for k in self._param_names()}

        def set_params(self, **params):
            for k, v in params.items():
                setattr(self, k, v)
            return self


def _as_array(X) -> np.ndarray:
    if hasattr(X, "values") and not isinstance(X, np.ndarray):
        X = X.values
    return np.asarray(X, dtype=np.float64)


def r2_score(y, yp) -> float:
    """1 - SS_res / SS_tot (scikit-learn's r2_score for one output)."""
    y, yp = np.asarray(y, dtype=np.float64), np.asarray(yp, dtype=np.float64)
    ss_res = float(np.sum((y - yp) ** 2))
    ss_tot = float(np.sum((y - np.mean(y)) ** 2))
    if ss_tot == 0.0:
        return 1.0 if ss_res == 0.0 else 0.0
    return 1.0 - ss_res / ss_tot


def accuracy_score(y, yp) -> float:
    return float(np.mean(np.asarray(y) == np.asarray(yp)))


def binarize(yp):
    """Class 1 where the model value exceeds 0.5 (rils_rols/utils.py:33-35)."""
    return (np.asarray(yp) > 0.5) * 1


def proba(yp):
    """[1 - s, s] with s the logistic of the value (rils_rols/utils.py:37-39)."""
    s = 1.0 / (1.0 + np.exp(-np.asarray(yp, dtype=np.float64)))
    return np.vstack([1 - s, s]).T


def _split(X, y, train_size, random_state):
    """A train share of the rows; scikit-learn's train_test_split when present."""
    try:
        from sklearn.model_selection import train_test_split
        Xs, _, ys, _ = train_test_split(X, y, train_size=train_size, random_state=random_state)
        return Xs, ys
    except ImportError:
        idx = np.random.RandomState(random_state).permutation(len(X))[: int(round(train_size * len(X)))]
        return X[idx], y[idx]


def _simplify(model: str, timeout_s: float = 2.0):
    """sympy's simplify(ratio=1) when it finishes within the timeout, else
    sympify; the raw string when sympy is absent."""
    try:
        import sympy
    except ImportError:
        return model
    box = {}

    def work():
        try:
            box["v"] = sympy.simplify(sympy.sympify(model), ratio=1)
        except Exception as e:  # noqa: BLE001 - fall back below
            box["e"] = e

    t = threading.Thread(target=work, daemon=True)
    t.start()
    t.join(timeout_s)
    if "v" in box:
        return box["v"]
    try:
        return sympy.sympify(model)
    except Exception:  # noqa: BLE001
        return model


def _complexity(expr) -> int:
    try:
        from sympy import preorder_traversal
        return sum(1 for _ in preorder_traversal(expr))
    except ImportError:
        return len(str(expr))


class RILSROLSBase(_EstimatorBase):
    def __init__(self, classification=None, max_fit_calls=100000, max_time=100, complexity_penalty=0.001,
                 max_complexity=50, sample_size=1, verbose=False, random_state=0, precision="plain"):
        if verbose:
            print(f"Calling with max_fit_calls={max_fit_calls} max_time={max_time} "
                  f"complexity_penalty={complexity_penalty} max_complexity={max_complexity} "
                  f"sample_size={sample_size} verbose={verbose} random_state={random_state}")
        self.classification = classification
        self.max_fit_calls = max_fit_calls
        self.max_time = max_time
        self.complexity_penalty = complexity_penalty
        self.max_complexity = max_complexity
        self.sample_size = sample_size
        self.verbose = verbose
        self.random_state = random_state
        self.precision = precision
        self.rr_cpp = None
        self.model = None
        self.model_simp = None
        self._backend = None

    def set_backend(self, backend) -> None:
        """Score fitness with another rrh_backend (None: the GB300 device path)."""
        self._backend = backend

    # -- fit -------------------------------------------------------------
    def fit(self, X, y):
        """rils_rols/rils_rols.py:50-89: sample_size 0 tunes the share of rows
        on a 10% sample with 1% of the budget, then fits."""
        X, y = _as_array(X), _as_array(y).reshape(-1)
        if self.sample_size == 0:
            if self.verbose:
                print("Automatically tuning sample size:")
            if len(X) <= 10000:
                self.sample_size = 1
            else:
                start = time.time()
                total_calls = self.max_fit_calls
                self.max_fit_calls = total_calls / 100
                best = 1
                used = 0
                for ss in (0.1,):
                    Xs, ys = _split(X, y, ss, self.random_state)
                    self.sample_size = 1  # the sample is already drawn
                    self.fit_inner(Xs, ys)
                    used += self.max_fit_calls
                    r2_sample = r2_score(ys, RILSROLSBase.predict(self, Xs))
                    r2_all = r2_score(y, RILSROLSBase.predict(self, X))
                    if self.verbose:
                        print(f"Sample size {ss} --> R2={r2_all} R2_sample={r2_sample}")
                    if abs(r2_all - r2_sample) < 0.01:
                        best = ss
                        break
                self.sample_size = best
                self.max_time -= time.time() - start
                self.max_fit_calls = total_calls - used
        elif self.sample_size < 0 or self.sample_size > 1:
            raise ValueError("Sample size parameter must belong to interval (0, 1], while value 0 means it is "
                             "automatically tuned.")
        self.fit_inner(X, y)
        return self

    def fit_inner(self, X, y):
        X, y = _as_array(X), _as_array(y).reshape(-1)
        if X.ndim != 2:
            raise ValueError("X must be a 2-D array (rows x features)")
        self.rr_cpp = rils_rols_cpp.rils_rols(bool(self.classification), int(self.max_fit_calls),
                                              int(self.max_time), float(self.complexity_penalty),
                                              int(self.max_complexity), float(self.sample_size),
                                              bool(self.verbose), int(self.random_state))
        if self._backend is not None:
            self.rr_cpp.set_backend(self._backend)
        self.rr_cpp.set_precision(self.precision)
        n, d = X.shape
        self.rr_cpp.fit(np.ascontiguousarray(X).reshape(-1), y, n, d)
        self.model = self.rr_cpp.get_model_string()
        self.best_time = self.rr_cpp.get_best_time()
        self.total_time = self.rr_cpp.get_total_time()
        self.fit_calls = self.rr_cpp.get_fit_calls()
        self.model_simp = self.model if self.classification else _simplify(self.model)
        return self.model, self.model_simp

    # -- use -------------------------------------------------------------
    def check_model(self):
        if self.model is None or self.rr_cpp is None:
            raise RuntimeError("Cannot predict because model is not build yet. First call fit().")

    def predict(self, X):
        self.check_model()
        X = _as_array(X)
        if X.ndim == 1:
            X = X[:, None]
        n, d = X.shape
        return self.rr_cpp.predict(np.ascontiguousarray(X).reshape(-1), n, d)

    def model_string(self):
        self.check_model()
        return self.model_simp

    def fit_report_string(self):
        self.check_model()
        return (f"maxTime={self.max_time}\tmaxFitCalls={self.max_fit_calls}\tseed={self.random_state}\t"
                f"sizePenalty={self.complexity_penalty}\tmaxComplexity={self.max_complexity}\t"
                f"sampleShare={self.sample_size}\ttotalTime={self.total_time:.1f}\tbestTime={self.best_time}\t"
                f"fitCalls={self.fit_calls}\tsimpSize={_complexity(self.model_simp)}\texpr={self.model}\t"
                f"exprSimp={self.model_simp}")


class RILSROLSRegressor(RILSROLSBase):
    def __init__(self, max_fit_calls=100000, max_time=100, complexity_penalty=0.001, max_complexity=50,
                 sample_size=1, verbose=False, random_state=0, precision="plain"):
        super().__init__(False, max_fit_calls, max_time, complexity_penalty, max_complexity, sample_size, verbose,
                         random_state, precision)

    def score(self, X, y):
        return r2_score(_as_array(y).reshape(-1), self.predict(X))


class RILSROLSBinaryClassifier(RILSROLSBase):
    def __init__(self, max_fit_calls=100000, max_time=100, complexity_penalty=0.001, max_complexity=50,
                 sample_size=1, verbose=False, random_state=0, precision="plain"):
        super().__init__(True, max_fit_calls, max_time, complexity_penalty, max_complexity, sample_size, verbose,
                         random_state, precision)

    def check_binary_targets(self, y):
        y = _as_array(y).reshape(-1)
        if np.any((y != 0) & (y != 1)):
            raise ValueError("The classifier works only for binary targets, so allowed target values are 0 or 1.")

    def predict(self, X):
        return binarize(super().predict(X))

    def predict_proba(self, X):
        return proba(self.predict(X))

    def score(self, X, y):
        self.check_binary_targets(y)
        return accuracy_score(_as_array(y).reshape(-1), self.predict(X))

    def fit(self, X, y):
        self.check_binary_targets(y)
        return super().fit(X, y)

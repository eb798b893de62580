"""Estimators with the interface of the reference's `rils_rols` package,
scored by the GB300 fitness path."""
from .rils_rols import RILSROLSBase, RILSROLSBinaryClassifier, RILSROLSRegressor

__all__ = ["RILSROLSBase", "RILSROLSRegressor", "RILSROLSBinaryClassifier"]

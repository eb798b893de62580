"""GB300 fitness path of RILS-ROLS: batched expression evaluation, OLS refit and
penalised R2/RMSE fitness as sm_103a CUDA kernels behind a C ABI, with the
reference's search driver on the host."""
from ._lib import load  # noqa: F401

"""libkriging_gb300 -- GB300-native (sm_103a) libKriging likelihood path.

Drop-in for pylibkriging's ``Kriging`` and ``NestedKriging`` on the likelihood path: covariance build, blocked
Cholesky and triangular solves (FP64, or split-bf16 tensor-core products), concentrated log-likelihood with its
one-pass adjoint theta-gradient, the L-BFGS-B fit (multistart and NestedKriging submodel evaluations batched into
single GPU launches), the Vecchia likelihood and predict.  All compute goes through the C ABI of
``include/libkriging_gb300.h``.
"""
from ._lib import LibKrigingError, header_symbols
from ._lib import load as _load_library
from .kriging import (Kriging, Optim, VecchiaShard, check_chol_rcond, get_num_nugget, set_num_nugget,
                      vecchia_sets)
from .nested import NestedKriging


def load(filename=None):
    """load() returns the ctypes handle of the GPU library; load(filename) reads a saved model, as pylibkriging's
    module-level load does (pylibkriging.cpp:28-37, Kriging files only)."""
    if filename is None:
        return _load_library()
    return Kriging.load(filename)


__all__ = ["Kriging", "NestedKriging", "Optim", "VecchiaShard", "vecchia_sets", "set_num_nugget", "get_num_nugget",
           "check_chol_rcond", "LibKrigingError", "load", "header_symbols"]

"""GB300-native Multivariate Cauchy Estimator step path.

The per-step term propagation of the reference's ``CauchyEstimator::step``
(natsnyder1/CauchyFriendly) runs as sm_103a FP64 kernels in libmce_gb300.so,
reached through the C ABI in include/mce_c_api.h.  This package holds the
build recipe, the ctypes binding, the estimator mirrors and the seeded
synthetic workloads.
"""
from .estimator import (  # noqa: F401
    BatchedCauchyEstimator, CauchyEstimator, RelativeSystem2D, autotune_configure, autotune_table, max_shape)

__all__ = ["BatchedCauchyEstimator", "CauchyEstimator", "RelativeSystem2D", "max_shape"]

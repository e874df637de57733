"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/mce_c_api.h declares (no device calls here)."""
import ctypes

from cauchyfriendly_gb300 import _lib, build


def test_library_exports_every_declared_symbol():
    build.build()
    lib = ctypes.CDLL(build.LIB)
    names = _lib.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the binding declares a signature for each of them
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_reference_rand_constants_match_oracle_draws():
    import numpy as np
    import oracle
    lib = _lib.load()
    root = np.zeros(3)
    bp = np.zeros(10)
    rc = lib.mce_draw_reference_constants(7, 3, 10, 8, root.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          bp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == 0
    r2, b2 = oracle.draw_reference_constants(7, 3, 10)
    assert np.array_equal(root, r2) and np.array_equal(bp, b2)


def test_create_without_gpu_fails_loudly():
    import numpy as np
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from cauchyfriendly_gb300 import CauchyEstimator
    with pytest.raises(_lib.MceError):
        CauchyEstimator(np.eye(3), np.ones(3) * 0.1, np.zeros(3), 5, 3, 0, 1, 1)

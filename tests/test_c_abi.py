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


def test_invalid_arguments_return_status_without_device():
    import ctypes as ct
    import numpy as np
    lib = _lib.load()
    st = ct.c_int(0)
    dp = ct.POINTER(ct.c_double)
    A0 = np.eye(3)
    z = np.zeros(3)
    steps = np.array([5], np.int32)
    # d out of range
    h = lib.mce_batch_create(1, 9, 0, 1, 1, steps.ctypes.data_as(ct.POINTER(ct.c_int)), A0.ctypes.data_as(dp),
                             z.ctypes.data_as(dp), z.ctypes.data_as(dp), None, None, 0, ct.byref(st))
    assert not h and st.value == -1
    # more hyperplanes than the build supports (the reference caps at 31, this build at 24)
    steps = np.array([40], np.int32)
    h = lib.mce_batch_create(1, 3, 0, 1, 1, steps.ctypes.data_as(ct.POINTER(ct.c_int)), A0.ctypes.data_as(dp),
                             z.ctypes.data_as(dp), z.ctypes.data_as(dp), None, None, 0, ct.byref(st))
    assert not h and st.value == -3
    assert "31" in _lib.last_error()
    steps = np.array([24], np.int32)  # 26 hyperplanes
    h = lib.mce_batch_create(1, 3, 0, 1, 1, steps.ctypes.data_as(ct.POINTER(ct.c_int)), A0.ctypes.data_as(dp),
                             z.ctypes.data_as(dp), z.ctypes.data_as(dp), None, None, 0, ct.byref(st))
    assert not h and st.value == -3
    assert "24" in _lib.last_error()
    # NULL handle
    assert lib.mce_step(None, 0.0, None, None, None, None, 0.0, None, None) == -1


def test_autotune_entry_points_without_device():
    lib = _lib.load()
    assert lib.mce_autotune_table(None, None, 0) == 0
    assert lib.mce_autotune_table(None, None, 4) < 0
    assert lib.mce_autotune_configure(2) < 0
    assert lib.mce_autotune_kernel_name(3) == b"gtable_eval"
    assert lib.mce_autotune_kernel_name(99) == b""

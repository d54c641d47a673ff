"""The C-ABI library loads and exports every function include/sf_capi.h
declares (no GPU needed: only symbol lookup, no compute calls)."""
import ctypes

import pytest

import sfgb


def test_header_declares_the_boundary():
    names = sfgb.header_symbols()
    for required in ("sf_plan_create", "sf_correlate", "sf_covariance_eig", "sf_beamform",
                     "sf_run_adaptive", "sf_run_lambda_gpu", "sf_run_corr_beam"):
        assert required in names


def test_library_exports_every_header_symbol():
    if not sfgb.LIB_PATH.exists():
        pytest.skip("libsfgb.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(str(sfgb.LIB_PATH))
    missing = [n for n in sfgb.header_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # every header symbol has a ctypes signature in the binding
    assert set(sfgb.header_symbols()) <= set(sfgb._SIGS)


def test_no_device_error_is_loud():
    """Without a GPU, creating a plan fails with a clear error (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        sfgb.Plan(1, 1, 8, 4, 4, 1, 1)

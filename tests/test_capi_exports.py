"""The C-ABI library loads and exports every function include/pnjl_cuda.h declares (no
compute call: this runs without a GPU)."""
import ctypes
import os

import pytest

from julia_relaxtime_gb300 import _capi


def _built():
    return os.path.exists(_capi.LIB_PATH)


def test_header_declares_the_boundary():
    names = _capi.declared_functions()
    for required in ("pnjl_init", "pnjl_destroy", "pnjl_set_nodes", "pnjl_eval_batch", "pnjl_solve_batch",
                     "pnjl_solve_batch_device", "pnjl_last_error", "pnjl_thermo_batch"):
        assert required in names
    assert set(names) == set(_capi.SIGNATURES), set(names) ^ set(_capi.SIGNATURES)


@pytest.mark.skipif(not _built(), reason="libpnjl_cuda.so not built (run __graft_entry__.build())")
def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_capi.LIB_PATH)
    missing = [n for n in _capi.declared_functions() if not hasattr(lib, n)]
    assert not missing


@pytest.mark.skipif(not _built(), reason="libpnjl_cuda.so not built")
def test_host_only_entry_points():
    L = _capi.lib()
    p = _capi.pnjl_params()
    assert L.pnjl_params_default(ctypes.byref(p)) == 0
    assert p.Lambda == pytest.approx(602.3 / 197.327)
    assert L.pnjl_params_default(None) == _capi.PNJL_ERR_INVALID_ARGUMENT
    assert L.pnjl_destroy(None) == 0
    assert L.pnjl_last_error(None) == b"null context"


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_capi, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_capi, "_lib", None)
    with pytest.raises(_capi.CudaLibraryError):
        _capi.lib()

"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
and exports every entry point include/rectv_gb300.h declares (no GPU calls)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "rectv_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rectv_[a-z_]+)\s*\(", txt)))


def test_header_declares_reference_replacements():
    syms = header_symbols()
    for name in ("rectv_create", "rectv_run", "rectv_check_adjoints", "rectv_free", "rectv_last_error"):
        assert name in syms


def test_library_exports_every_header_symbol(lib_built):
    lib = ctypes.CDLL(lib_built)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(lib_built):
    from rectv_gpu_gb300 import _lib
    assert set(header_symbols()) == set(_lib.SIGNATURES)
    lib = _lib.load()
    assert lib.rectv_version().decode().startswith("rectv_gb300")
    assert lib.rectv_last_error().decode() == ""


def test_null_handle_errors_are_reported(lib_built):
    from rectv_gpu_gb300 import _lib
    lib = _lib.load()
    assert lib.rectv_free(None) == 1
    assert "null handle" in lib.rectv_last_error().decode()
    assert lib.rectv_iterate(None, 1) == 1
    with pytest.raises(_lib.RectvError):
        _lib.check(lib.rectv_set_verbose(None, 0))


def test_solver_signature_matches_reference():
    import inspect
    from rectv_gpu_gb300 import Solver
    sig = inspect.signature(Solver.recon)
    positional = [k for k, v in sig.parameters.items() if v.kind != inspect.Parameter.KEYWORD_ONLY]
    assert positional == ["self", "data", "theta", "phi", "rot_center", "lambda0", "lambda1", "niter", "titer"]
    extras = [k for k, v in sig.parameters.items() if v.kind == inspect.Parameter.KEYWORD_ONLY]
    assert extras == ["init"] and sig.parameters["init"].default is None
    d = {k: v.default for k, v in sig.parameters.items()}
    assert d["rot_center"] is None and d["lambda0"] == 1e-3 and d["lambda1"] == 1
    assert d["niter"] == 1 and d["titer"] == 1
    sig = inspect.signature(Solver.adjoint_tests)
    assert list(sig.parameters) == ["self", "data", "theta", "phi", "lambda1", "rot_center"]


def test_library_is_sm103a_only(lib_built):
    from rectv_gpu_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]

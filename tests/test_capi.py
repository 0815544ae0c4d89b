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
    return sorted(set(re.findall(r"\b(rectv_[a-z0-9_]+)\s*\(", txt)))


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


def test_estimate_bytes_is_host_arithmetic(lib_built):
    """rectv_estimate_bytes needs no GPU: the sizes the engine admits jobs by
    (config 3: about 94.5 GB, measured on the GPU: 94.4 GB)."""
    from rectv_gpu_gb300 import _lib
    from rectv_gpu_gb300.rectv import estimate_bytes
    c3 = estimate_bytes(1024, 2880, 16, 64, 16)
    assert 90e9 < c3 < 100e9
    assert estimate_bytes(512, 1440, 16, 32, 8) < estimate_bytes(512, 1440, 16, 64, 8)
    # fewer than 8 time samples take the FP32 scatter with full periodic planes
    assert estimate_bytes(256, 720, 4, 8, 8) > 0
    with pytest.raises(_lib.RectvError):
        estimate_bytes(64, 128, 8, 4, 8)  # nzp > nz


def test_direction_grouping_is_host_logic(lib_built):
    """Which USFFT path a geometry takes (build_dir_plan, no GPU): scans that
    return to their angles every half-turn share sample positions; the
    reference test's angles and calibrated measured angles keep the per-ray
    kernels."""
    import numpy as np
    from rectv_gpu_gb300 import _lib, plan_directions
    from rectv_gpu_gb300.phantom import scan_angles
    # 2880 angles over 8 half-turns (the foam example's linspace without the end point)
    assert plan_directions(scan_angles(2880, 8), 1024) == (360, 8)
    assert plan_directions(scan_angles(1440, 8), 512) == (180, 8)
    # the reference test's angles (tests/test_adjoint.py: linspace with the end point)
    assert plan_directions(np.linspace(0, 8 * np.pi, 2400).astype(np.float32), 504)[0] == 0
    # measured angles scaled by a calibration factor (examples/tao/tao.py: 0.9977)
    th = (np.linspace(0, 16 * np.pi, 1440, endpoint=False) * 0.9977).astype(np.float32)
    assert plan_directions(th, 1024) == (0, 1)
    # two rays per direction: below the default 2.5, taken with min_group = 1
    assert plan_directions(scan_angles(90, 2), 64) == (0, 2)
    assert plan_directions(scan_angles(90, 2), 64, min_group=1.0) == (45, 2)
    # theta and theta + pi are one direction (opposite orientation)
    th = np.array([0.3, 0.3 + np.pi, 0.3 + 2 * np.pi, 1.1, 1.1 + np.pi, 1.1 + 3 * np.pi], np.float32)
    assert plan_directions(th, 256) == (2, 3)
    with pytest.raises(_lib.RectvError):
        plan_directions(th, 1)


def test_engine_without_gpu_reports_an_error(lib_built):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from rectv_gpu_gb300 import _lib
    from rectv_gpu_gb300.engine import Engine
    with pytest.raises(_lib.RectvError):
        Engine(budget_bytes=1e9)

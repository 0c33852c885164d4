"""The C ABI: the shared library loads (no GPU needed) and exports every function that
include/fdga.h declares; the Python binding covers exactly that set; argument validation that
precedes any device work returns an error status instead of aborting."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fdga.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fdga_[A-Za-z0-9_]+)\s*\(", src)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for core in ("fdga_create", "fdga_iterate", "fdga_residual", "fdga_solve", "fdga_solve_newton", "fdga_jvp",
                 "fdga_dchi_dU", "fdga_batch_iterate", "fdga_bubble_noalloc", "fdga_susceptibility"):
        assert core in names


def test_library_exports_every_declared_function():
    from fdgasolver import _lib
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_exactly_the_header():
    from fdgasolver import _lib
    assert sorted(_lib.EXPORTS) == declared_functions()


def test_invalid_arguments_return_errors():
    from fdgasolver import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    bad = _lib.fdga_config()  # all zero: invalid dimensions
    assert lib.fdga_create(ctypes.byref(bad), ctypes.byref(h)) != 0
    assert lib.fdga_create_error()
    assert lib.fdga_iterate(None, 0, 1, 1) != 0
    assert lib.fdga_set_option(None, b"k3_tensor_cores", 1) != 0
    v = ctypes.c_double()
    assert lib.fdga_query(None, b"state_len", ctypes.byref(v)) != 0

"""The C-ABI library loads and exports every entry point declared in include/*.h.

No GPU needed: nothing here launches a kernel (argument validation returns
before any CUDA call).
"""

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from fluidimage_gb300 import _lib, build

    build.build()
    return _lib.load()


def declared_functions():
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = header.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(fi_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for name in names:
        assert hasattr(lib, name), name


def test_bindings_cover_the_header():
    from fluidimage_gb300 import _lib

    assert set(declared_functions()) == set(_lib._SIGNATURES)


def test_struct_layouts_match(lib):
    from fluidimage_gb300 import _lib

    sizes = (C.c_int64 * 3)()
    assert lib.fi_abi_sizes(sizes) == 0
    assert list(sizes) == [C.sizeof(_lib.PivPassArgs), C.sizeof(_lib.FixArgs),
                           C.sizeof(_lib.TpsPlan)]


def test_invalid_arguments_are_rejected_on_the_host(lib):
    from fluidimage_gb300 import _lib

    assert lib.fi_piv_pass(None, None) == -1
    assert b"null args" in lib.fi_last_error()
    args = _lib.PivPassArgs()
    args.n = 20
    assert lib.fi_piv_pass(C.byref(args), None) == -1
    assert b"not supported" in lib.fi_last_error()
    assert lib.fi_fix(None, None) == -1
    assert lib.fi_images_min(None, None, 0, 10, None, None) == -1
    with pytest.raises(_lib.CudaLibError, match="bad arguments"):
        _lib.check(lib.fi_tps_members(None, 0, None, None, 0, 0, None, None, None, None, None,
                                      None, None, None, None))
    assert lib.fi_gaussian_filter(None, None, None, 0, 1, 1, 1, None, 1, None) == -1
    assert b"null pointer" in lib.fi_last_error()
    buf = C.create_string_buffer(64)
    assert lib.fi_gaussian_filter(buf, buf, buf, 7, 1, 1, 1, buf, 1, None) == -1
    assert b"bad dtype" in lib.fi_last_error()
    assert lib.fi_sharpen_combine(buf, buf, 0, 0, 1.0, buf, None) == -1
    assert b"bad arguments" in lib.fi_last_error()


def test_version(lib):
    assert lib.fi_version().startswith(b"fluidimage_gb300")


def test_tc_pass_argument_checks(lib):
    """fi_piv_pass_tc refuses window sizes other than 32 and unknown forms before any
    CUDA call."""
    from fluidimage_gb300 import _lib as L

    a = L.PivPassArgs()
    a.n = 16
    assert lib.fi_piv_pass_tc(C.byref(a), 1, None, None) == -1
    assert b"window size" in lib.fi_last_error()
    a.n = 32
    assert lib.fi_piv_pass_tc(C.byref(a), 7, None, None) == -1
    assert b"bad form" in lib.fi_last_error()
    assert lib.fi_piv_pass_tc(None, 1, None, None) == -1

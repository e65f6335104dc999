"""The C-ABI library loads on a machine without a GPU and exports every entry point that
include/wbc.h declares, with the signatures the Python binding expects. No compute calls."""

import ctypes
import re
import subprocess

import pytest

from tests.conftest import ROOT

HEADER = ROOT / "include" / "wbc.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wbc_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from warpbiocell_gb300 import _build, _lib

    if not _build.library_path().exists():
        _build.build()
    return _lib.load()


def test_header_declares_the_boundary():
    names = declared_functions()
    assert "wbc_contact_substep" in names and "wbc_sor_sweeps" in names and "wbc_deposit" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    from warpbiocell_gb300 import _build

    out = subprocess.run(["nm", "-D", "--defined-only", str(_build.library_path())], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (wbc_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for name in declared_functions():
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)


def test_binding_covers_every_declared_symbol():
    from warpbiocell_gb300 import _lib

    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_host_only_entry_points_work_without_a_gpu(lib):
    assert lib.wbc_version() >= 1
    assert lib.wbc_device_count() >= 0
    assert lib.wbc_scan_workspace_bytes(1 << 20) >= 4 * ((1 << 20) // 4096)
    # argument validation happens before any CUDA call
    assert lib.wbc_rng_init(0, None, 10, None) == -1
    assert lib.wbc_deposit(None, 0, None, None, None, None) == -1


def test_status_codes_match_the_header():
    from warpbiocell_gb300 import _lib

    defines = dict(re.findall(r"#define (WBC_(?:OK|ERR_[A-Z]+))\s+\(?(-?\d+)\)?", HEADER.read_text()))
    assert set(defines) >= {"WBC_OK", "WBC_ERR_INVALID", "WBC_ERR_CAPACITY", "WBC_ERR_CUDA", "WBC_ERR_TIMEOUT",
                            "WBC_ERR_WORKSPACE"}
    for name, value in defines.items():
        assert getattr(_lib, name) == int(value), name


def test_status_codes_map_to_the_reference_exceptions(lib):
    from warpbiocell_gb300 import _lib

    _lib.check(_lib.WBC_OK, "ok")
    with pytest.raises(ValueError):  # parameter problems are ValueError, as in the reference's dataclasses
        _lib.check(_lib.WBC_ERR_INVALID, "wbc_x")
    for rc in (_lib.WBC_ERR_CUDA, _lib.WBC_ERR_WORKSPACE, _lib.WBC_ERR_TIMEOUT):
        with pytest.raises(_lib.LibraryError):
            _lib.check(rc, "wbc_x")
    assert issubclass(_lib.LibraryError, RuntimeError)


def test_noalloc_scan_limit_is_reported_before_any_device_work(lib):
    # The size check comes first, so the (never dereferenced) host addresses are not touched.
    buf = (ctypes.c_int32 * 2)()
    addr = ctypes.addressof(buf)
    rc = lib.wbc_division_scan_noalloc((1 << 25) + 1, addr, addr, addr, None)
    assert rc == -1
    assert b"WBC_NOALLOC_SCAN_MAX_CELLS" in lib.wbc_last_error()

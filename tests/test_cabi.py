"""The C-ABI library builds, loads, and exports every function the public
header declares (no GPU needed: only host-side entry points are called)."""
import pathlib

from slamtb_gb300 import _build, _native

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "slamtb_gb300.h"


def test_library_exports_every_header_symbol():
    _build.build()
    lib = _native.lib()
    names = _native.header_symbols(HEADER.read_text())
    assert len(names) >= 9
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # every header symbol has a ctypes signature
    assert not [n for n in names if n not in _native._SIGNATURES]


def test_host_only_entry_points():
    lib = _native.lib()
    assert b"sm_103a" in lib.stb_version()
    small = lib.stb_icp_workspace_bytes(100, 10, 10)
    big = lib.stb_icp_workspace_bytes(640 * 480, 480, 640)
    assert 0 < small < big
    assert big >= 8 * 640 * 480

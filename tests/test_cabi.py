"""The C ABI without a GPU: the library builds, loads and exports every
function the public header declares; the header's constants and struct
layouts match the Python mirror; every entry point turns bad arguments into
a status code and a "Check failed:" message before any device work."""
import ctypes
import pathlib

import pytest

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


# Entry points whose arguments are all checked on the host before any device
# work: every one of them turns null pointers and empty or invalid sizes into
# a status code and a "Check failed:" message (the reference's error prefix,
# error.hpp) without touching memory.
_CHECKED = sorted(n for n, (res, args) in _native._SIGNATURES.items()
                  if res is ctypes.c_int and args
                  and not n.startswith(("stb_profile_", "stb_set_")))
# A batch of zero twists is an empty operation, as for an empty torch tensor.
_EMPTY_OK = {"stb_exp_rt_to_matrix", "stb_exp_rt_to_matrix_backward", "stb_matrix_to_exp_rt"}


def test_wait_test_limits_setter():
    """The test hook of the bounded waits refuses a negative count of phantom
    arrivals and restores its defaults with (0, 0)."""
    lib = _native.lib()
    assert lib.stb_set_wait_test_limits(0, -1) == _native.STB_EINVAL
    assert lib.stb_last_error().startswith(b"Check failed: ")
    assert lib.stb_set_wait_test_limits(0, 0) == _native.STB_OK


def _arguments(args, size):
    out = []
    for a in args:
        if a in (ctypes.c_float, ctypes.c_double):
            out.append(0.0)
        elif a in (ctypes.c_void_p, ctypes.c_char_p):
            out.append(None)
        else:
            out.append(size)
    return out


@pytest.mark.parametrize("size", [0, 4])
def test_entry_points_reject_bad_arguments(size):
    lib = _native.lib()
    errors = (_native.STB_EINVAL, _native.STB_EDEVICE, _native.STB_EDTYPE)
    assert len(_CHECKED) >= 25
    for name in _CHECKED:
        rc = getattr(lib, name)(*_arguments(_native._SIGNATURES[name][1], size))
        if size == 0 and name in _EMPTY_OK:
            assert rc == _native.STB_OK, name
            continue
        assert rc in errors, (name, rc)
        msg = lib.stb_last_error()
        assert msg.startswith(b"Check failed: "), (name, msg)
        with pytest.raises(RuntimeError, match="^Check failed: "):
            _native.check(rc)


def test_host_tensors_are_refused():
    """No CPU fallback: host tensors raise, as the reference's device checks
    do for the wrong device (error.hpp:12-37)."""
    import torch
    from slamtb_gb300.camera import KCamera
    from slamtb_gb300.registration import ICPOdometry
    kcam = KCamera(torch.tensor([[50.0, 0, 8], [0, 50, 6], [0, 0, 1]]))
    pts, nrm = torch.rand(12, 16, 3), torch.rand(12, 16, 3)
    mask = torch.ones(12, 16, dtype=torch.bool)
    with pytest.raises(RuntimeError, match="Expected a gpu tensor"):
        ICPOdometry(3).estimate(kcam, pts.view(-1, 3), nrm.view(-1, 3), mask.view(-1),
                                target_points=pts, target_normals=nrm, target_mask=mask)
    # the _cslamtb shim names the source points first, as the reference's
    # device checks start from them (correspondence_map.cu:71-79)
    from slamtb_gb300 import processing
    from slamtb_gb300._cslamtb import CorrespondenceMap, ICPJacobian
    k = kcam.matrix
    merge = torch.full((12, 16), 0x0FFFFFFF7F800000, dtype=torch.int64)
    with pytest.raises(RuntimeError, match="^Check failed: source points: Expected a gpu"):
        CorrespondenceMap.compute_correspondence_map(
            pts.view(-1, 3), nrm.view(-1, 3), mask.view(-1), torch.eye(4), pts, nrm, mask, k,
            merge, 0.1, 0.5)
    with pytest.raises(RuntimeError, match="^Check failed: source points: Expected a gpu"):
        ICPJacobian.estimate_geometric(pts.view(-1, 3), mask.view(-1), torch.eye(4), pts, nrm,
                                       k, merge, torch.zeros(192, 6, 6), torch.zeros(192, 6),
                                       torch.zeros(192))
    for fn, args in ((processing.estimate_normals, (pts, mask)),
                     (processing.erode_mask, (mask,)),
                     (processing.bilateral_depth_filter, (pts[..., 2].contiguous(), mask))):
        with pytest.raises(RuntimeError, match="Expected a gpu tensor"):
            fn(*args)


def _python_name(name):
    """Header constant -> its name in slamtb_gb300._native."""
    for prefix in ("STB_ST_", "STB_RES_", "STB_HIST_", "STB_OPT_"):
        if name.startswith(prefix):
            return name[len("STB_"):]
    return name


def test_header_constants_match_the_python_mirror():
    """Every integer #define of the header (status codes, element types,
    status bits, result and history layouts) has the same value in
    slamtb_gb300._native."""
    import re
    defs = re.findall(r"^#define (STB_\w+) (0x[0-9a-fA-F]+|\d+)u?\b", HEADER.read_text(),
                      re.M)
    assert len(defs) >= 31 and ("STB_OPT_DW_SOLVE", "0x100") in defs
    mismatched = [(n, int(v, 0), getattr(_native, _python_name(n), None)) for n, v in defs
                  if getattr(_native, _python_name(n), None) != int(v, 0)]
    assert not mismatched, mismatched


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """The ctypes mirrors of stb_level and stb_level_params have the size
    and field offsets that a C compiler gives the header's structs."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"stb_level": _native.StbLevel, "stb_level_params": _native.StbLevelParams}
    lines = ['#include <stdio.h>', '#include "slamtb_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(HEADER.parent), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out.splitlines()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)

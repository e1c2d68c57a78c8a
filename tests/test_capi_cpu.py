"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/sptrsv_gb300.h (host-only checks, no GPU work)."""
from __future__ import annotations

import ctypes
import re

from conftest import ROOT


def _declared_functions():
    text = (ROOT / "include" / "sptrsv_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sptrsv_\w+)\s*\(", text, flags=re.M))
    return names


def test_header_declares_reference_entry_points():
    names = _declared_functions()
    for required in ("sptrsv_syncfree_cuda", "sptrsv_gb300_analyser", "sptrsv_gb300_executor",
                     "sptrsv_gb300_create", "sptrsv_gb300_analyse", "sptrsv_gb300_solve", "sptrsv_gb300_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    names = _declared_functions()
    assert len(names) >= 15
    for name in sorted(names):
        assert hasattr(built_lib, name), f"{name} declared but not exported"


def test_binding_covers_header():
    from sptrsv_gb300 import _lib
    assert _declared_functions() == set(_lib.SIGNATURES)


def test_status_strings_and_version(built_lib):
    from sptrsv_gb300 import _lib
    assert built_lib.sptrsv_gb300_version() == 101
    for code in range(-9, 1):
        s = _lib.status_string(code)
        assert s and s != "unknown status"
    assert _lib.status_string(-42) == "unknown status"


def test_invalid_arguments_rejected_on_host(built_lib):
    from sptrsv_gb300 import _lib
    assert built_lib.sptrsv_gb300_create(None) == _lib.ERR_INVALID
    assert built_lib.sptrsv_gb300_destroy(None) == _lib.ERR_INVALID
    assert built_lib.sptrsv_gb300_set_option(None, 0, 0) == _lib.ERR_INVALID
    # m != n is reported before any device work, with the reference's -1
    rc = built_lib.sptrsv_gb300_syncfree_host(None, None, None, 3, 4, 0, 0, 1, 3, None, None, None, None, None,
                                              None, None)
    assert rc == _lib.ERR_NOT_SQUARE == -1


def test_build_targets_sm103a_only():
    import build as pkg_build
    assert pkg_build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_option_constants_match_header():
    """Every SPTRSV_OPTION_* value in the header has the same number in the binding."""
    import re
    from sptrsv_gb300 import _lib
    text = (ROOT / "include" / "sptrsv_gb300.h").read_text()
    opts = {m.group(1): int(m.group(2)) for m in re.finditer(r"SPTRSV_OPTION_([A-Z_]+)\s*=\s*(\d+)", text)}
    assert len(opts) >= 20
    for name, value in opts.items():
        assert getattr(_lib, f"OPTION_{name}") == value, name
    assert sorted(opts.values()) == list(range(len(opts)))


def test_info_struct_layout_matches_header(tmp_path):
    """The ctypes mirror of sptrsv_info has the C struct's size and every field at the
    C offset (a plain C program compiled against the header prints them)."""
    import shutil
    import subprocess
    from sptrsv_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    fields = [name for name, _ in _lib.Info._fields_]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sptrsv_gb300.h"', "int main(void) {",
             '  printf("size %zu\\n", sizeof(sptrsv_info));']
    lines += [f'  printf("{f} %zu\\n", offsetof(sptrsv_info, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src = tmp_path / "info_layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "info_layout"
    subprocess.run([cc, "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                        text=True).stdout.splitlines())
    assert int(out.pop("size")) == ctypes.sizeof(_lib.Info)
    for f in fields:
        assert int(out[f]) == getattr(_lib.Info, f).offset, f


def test_enum_and_define_constants_match_header():
    """Every SPTRSV_* enumerator and numeric #define in the header (statuses, layouts,
    element types, schedules, substitution and lane-mode constants, the no-alloc size)
    has the same value in the binding, named without the SPTRSV_ prefix."""
    import re
    from sptrsv_gb300 import _lib
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "sptrsv_gb300.h").read_text(), flags=re.S)
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"\bSPTRSV_([A-Z0-9_]+)\s*=\s*(-?\d+)", text)}
    consts.update({m.group(1): int(m.group(2))
                   for m in re.finditer(r"#define\s+SPTRSV_([A-Z0-9_]+)\s+\(?(-?\d+)\)?\s*$", text, flags=re.M)})
    consts.pop("GB300_VERSION", None)
    assert {"OK", "ERR_UNSUPPORTED", "LAYOUT_COL_MAJOR", "DTYPE_F32", "SCHED_LEVELSET", "OPT_WARP_AUTO"} <= set(consts)
    for name, value in consts.items():
        assert getattr(_lib, name) == value, name

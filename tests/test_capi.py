"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares.  No compute calls (CPU only)."""
import ctypes
import glob
import os
import re

import pytest

from fluxvortex_gb300 import _capi, build
from tests.conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(fvx_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    lib = _capi.load()
    assert b"sm_103a" in lib.fvx_version()


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(build.build())
    declared = _declared()
    assert len(declared) >= 10
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_table_covers_header():
    declared = _declared()
    assert set(_capi.SIGNATURES) >= declared, declared - set(_capi.SIGNATURES)


def test_argument_errors_are_reported_without_device_work():
    lib = _capi.load()
    # unknown leg set: rejected before any CUDA call
    st = lib.fvx_segments_collapsed(None, 0, None, None, None, None, None, None, None, 0.0, 0,
                                    7, None, None, None, 0, None)
    assert st == _capi.FVX_ERR_ARG
    assert b"leg set" in lib.fvx_last_error()
    st = lib.fvx_particle_pairs(9, 0, 0, None, None, 1, None, None, None, 1, None, None, None,
                                0, None)
    assert st == _capi.FVX_ERR_ARG
    with pytest.raises(_capi.FvxError):
        _capi.check(st)


def test_scratch_query_is_host_only():
    lib = _capi.load()
    assert lib.fvx_segments_collapsed_scratch_bytes(0, 10, 0) == 0
    assert lib.fvx_particle_pairs_scratch_bytes(0, 0, 0, 10) == 0


def test_structs_match_the_header_layout(tmp_path):
    """The ctypes mirrors of FlutterParams / FlutterState / FvxSurfaces have the C layout
    (sizes and field offsets from a C program compiled against the header)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    from fluxvortex_gb300._capi import Surfaces
    from fluxvortex_gb300.flutter import _Params, _State
    fields = {"FlutterParams": _Params, "FlutterState": _State, "FvxSurfaces": Surfaces}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fluxvortex_gb300.h"',
             'int main(void) {']
    for cname, cls in fields.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.splitlines():
        cname, what, val = line.split()
        got[(cname, what)] = int(val)
    for cname, cls in fields.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)

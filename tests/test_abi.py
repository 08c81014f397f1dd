"""The C ABI: libttfld builds for sm_103a, loads, exports every entry point
declared in include/ttfld.h, and the ctypes mirrors of its structs have the
C compiler's layout.  No compute call is made (no GPU needed)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ttfld.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ttfld_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libttfld():
    from ttcode_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_the_boundary():
    fns = declared_functions()
    for must in ("ttfld_create", "ttfld_solve_with_sor", "ttfld_fill_evalues", "ttfld_diff",
                 "ttfld_coupled_energy_eqs", "ttfld_diffusion", "ttfld_adjust_sor_param",
                 "ttfld_fill_sor_matrix", "ttfld_upload", "ttfld_download"):
        assert must in fns


def test_library_exports_every_declared_symbol(libttfld):
    missing = [f for f in declared_functions() if not hasattr(libttfld, f)]
    assert not missing, missing


def test_ffi_export_list_matches_header():
    from ttcode_gb300 import _ffi
    assert sorted(_ffi.EXPORTS) == declared_functions()


def test_abi_version_and_status_strings(libttfld):
    # host-only calls: no device is touched
    assert libttfld.ttfld_abi_version() == 2
    libttfld.ttfld_status_string.restype = ctypes.c_char_p
    assert libttfld.ttfld_status_string(-7).startswith(b"non-positive Q")


def test_null_arguments_are_rejected_without_a_device(libttfld):
    assert libttfld.ttfld_create(None, None, None, None, 0) == -1
    assert libttfld.ttfld_destroy(None) == -1
    assert libttfld.ttfld_solve_with_sor(None, 0, None) == -1


def test_struct_layout_matches_c():
    from ttcode_gb300 import _ffi
    structs = {"ttfld_dims": _ffi.Dims, "ttfld_metrics": _ffi.Metrics, "ttfld_params": _ffi.Params,
               "ttfld_solve_opts": _ffi.SolveOpts, "ttfld_solve_stats": _ffi.SolveStats,
               "ttfld_step_stats": _ffi.StepStats, "ttfld_energy": _ffi.Energy,
               "ttfld_raddif_params": _ffi.RaddifParams, "ttfld_opacity_table": _ffi.OpacityTable}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-std=c11", "-o", exe, c], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(l.split() for l in out if l.strip())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_field_ids_match_header():
    from ttcode_gb300 import _ffi
    src = open(HEADER).read()
    body = src[src.index("enum ttfld_field"):]
    body = body[:body.index("};")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    val = -1
    ids = {}
    for tok in body[body.index("{") + 1:].split(","):
        tok = tok.strip()
        if not tok:
            continue
        if "=" in tok:
            name, v = [t.strip() for t in tok.split("=")]
            val = int(v)
        else:
            name = tok
            val += 1
        ids[name.replace("TTFLD_", "")] = val
    assert ids == _ffi.FIELDS

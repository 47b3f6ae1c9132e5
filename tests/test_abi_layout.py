"""The ctypes mirrors of the C ABI's option and result structs against the
header: a small C program compiled against include/bmfp.h prints sizeof and
offsetof of every field, and each ctypes Structure must agree. A field added
to the header and not to _capi.py (or in another order) shifts every field
after it, which the library would read as garbage without an error."""
import ctypes
import json
import shutil
import subprocess

import pytest

from conftest import ROOT
from block_matrix_format_performance_gb300 import _capi

STRUCTS = {
    "bmfp_solver_options": _capi.SolverOptions,
    "bmfp_solve_info": _capi.SolveInfo,
    "bmfp_server_options": _capi.ServerOptions,
    "bmfp_server_stats": _capi.ServerStats,
}


def _c_layout(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "bmfp.h"', "int main(void) {", 'printf("{");']
    first = True
    for cname, cls in STRUCTS.items():
        sep = "" if first else ","
        first = False
        lines.append(f'printf("{sep}\\"{cname}\\": {{\\"size\\": %zu", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf(", \\"{f}\\": %zu", offsetof({cname}, {f}));')
        lines.append('printf("}");')
    lines += ['printf("}\\n");', "return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", f"{ROOT}/include", str(src), "-o", str(exe)], check=True)
    return json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_structs_match_the_header(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, cls in STRUCTS.items():
        c = layout[cname]
        assert ctypes.sizeof(cls) == c["size"], cname
        for f, _ in cls._fields_:
            assert getattr(cls, f).offset == c[f], (cname, f)

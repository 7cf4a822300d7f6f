"""The Python binding's ctypes structures against the C header: every struct
the binding mirrors has the size and field offsets that include/emv.h gives
it, as compiled by the host C compiler (a layout slip would pass garbage
across the C ABI without any error)."""
import os
import shutil
import subprocess

import pytest

import steiner_edge_linear_gb300 as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PAIRS = [(E._Stp, "emv_stp"), (E._Graph, "emv_graph"), (E._Timing, "emv_timing"), (E._Result, "emv_result"),
         (E._Instance, "emv_instance"), (E._BatchStats, "emv_batch_stats"), (E._ServerOpts, "emv_server_opts"),
         (E._ServerStats, "emv_server_stats")]


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    d = tmp_path_factory.mktemp("abi")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "emv.h"', "int main(void) {"]
    for cls, cname in PAIRS:
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'    printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["    return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(d / "layout")
    subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True, timeout=60).stdout
    return {tuple(line.split()[:2]): int(line.split()[2]) for line in out.splitlines()}


@pytest.mark.parametrize("cls,cname", PAIRS, ids=[c for _, c in PAIRS])
def test_ctypes_struct_matches_header(c_layout, cls, cname):
    import ctypes

    assert ctypes.sizeof(cls) == c_layout[(cname, "size")], cname
    for f in cls._fields_:
        assert getattr(cls, f[0]).offset == c_layout[(cname, f[0])], (cname, f[0])

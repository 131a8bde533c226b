"""The ctypes mirrors in zeroslam_gb300/ba.py against the C structs of
include/zeroslam_ba.h: a small C program compiled here prints sizeof and
every member's offsetof, which must equal the ctypes layout (a mismatch
would pass garbage across the boundary without an error). CPU only."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {  # C struct -> ctypes class in zeroslam_gb300.ba
    "zs_ba_options": "Options",
    "zs_ba_problem": "Problem",
    "zs_ba_report": "Report",
    "zs_ba_batch_report": "BatchReport",
    "zs_ba_adjoint_report": "AdjointReport",
    "zs_map_cull_input": "MapCullInput",
    "zs_cull_report": "CullReport",
    "zs_map_optimise_input": "MapOptimiseInput",
    "zs_map_optimise_report": "MapOptimiseReport",
    "zs_ba_attempt": "Attempt",
}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_ctypes_layout_matches_header(tmp_path):
    from zeroslam_gb300 import ba

    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "zeroslam_ba.h"', "int main(void) {"]
    for cs, py in STRUCTS.items():
        cls = getattr(ba, py)
        lines.append(f'    printf("{cs} size %zu\\n", sizeof({cs}));')
        for name, _ in cls._fields_:
            lines.append(f'    printf("{cs} {name} %zu\\n", offsetof({cs}, {name}));')
    lines.append('    printf("zs_match size %zu\\n", sizeof(zs_match));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for row in filter(None, out):
        cs, field, v = row.split()
        got[(cs, field)] = int(v)
    import ctypes

    for cs, py in STRUCTS.items():
        cls = getattr(ba, py)
        assert got[(cs, "size")] == ctypes.sizeof(cls), cs
        for name, _ in cls._fields_:
            assert got[(cs, name)] == getattr(cls, name).offset, (cs, name)
    assert got[("zs_match", "size")] == ba.MATCH_DTYPE.itemsize


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_oracle_ctypes_layout(tmp_path):
    """The same check for the oracle's own structs (oracle/ba_oracle.h)."""
    import ctypes

    from oracle import oracle as om

    structs = {"zso_problem": om._Problem, "zso_report": om.Report, "zso_cull_map": om._CullMap}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "ba_oracle.h"', "int main(void) {"]
    for cs, cls in structs.items():
        lines.append(f'    printf("{cs} size %zu\\n", sizeof({cs}));')
        for name, _ in cls._fields_:
            lines.append(f'    printf("{cs} {name} %zu\\n", offsetof({cs}, {name}));')
    lines.append('    printf("zso_match size %zu\\n", sizeof(zso_match));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "oracle"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {(r.split()[0], r.split()[1]): int(r.split()[2]) for r in out if r}
    for cs, cls in structs.items():
        assert got[(cs, "size")] == ctypes.sizeof(cls), cs
        for name, _ in cls._fields_:
            assert got[(cs, name)] == getattr(cls, name).offset, (cs, name)
    assert got[("zso_match", "size")] == om.MATCH_DTYPE.itemsize

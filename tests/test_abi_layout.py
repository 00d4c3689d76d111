"""The ctypes mirrors of the C ABI's structs (spoa_gb300/__init__.py) have the
layout the header gives them: a C program compiled against
include/spoa_gb300.h prints every field's offset and each struct's size,
and the mirrors must agree field by field (CPU; needs gcc)."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

import spoa_gb300 as sg
from conftest import ROOT

STRUCTS = [("spoa_gb300_batch_desc", sg._BatchDesc),
           ("spoa_gb300_batch_result", sg._BatchResult),
           ("spoa_gb300_server_desc", sg._ServerDesc)]


def _c_layout():
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "spoa_gb300.h"',
             "int main(void) {"]
    for cname, mirror in STRUCTS:
        lines.append(f'  printf("{cname} . %zu\\n", sizeof({cname}));')
        for field, _ in mirror._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as tmp:
        src, exe = os.path.join(tmp, "layout.c"), os.path.join(tmp, "layout")
        with open(src, "w") as fh:
            fh.write("\n".join(lines) + "\n")
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        s, f, v = line.split()
        layout[(s, f)] = int(v)
    return layout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_ctypes_mirrors_match_the_header():
    layout = _c_layout()
    for cname, mirror in STRUCTS:
        assert layout[(cname, ".")] == ctypes.sizeof(mirror), cname
        for field, _ in mirror._fields_:
            assert layout[(cname, field)] == getattr(mirror, field).offset, (cname, field)

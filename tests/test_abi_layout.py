"""The ctypes structures of the Python binding against the C header: the same
fields in the same order at the same offsets, and the same sizes, as the C
compiler lays them out (CPU only: gcc compiles a probe of include/pcgpu.h)."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

import primecount_gb300 as pcg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {"pcg_opts": pcg.Opts, "pcg_stats": pcg.Stats, "pcg_tuning": pcg.Tuning, "pcg_i128": pcg.I128}


def c_layout():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pcgpu.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "probe.c"), os.path.join(d, "probe")
        open(src, "w").write("\n".join(lines) + "\n")
        subprocess.run([cc, "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    lay = {}
    for line in out.split("\n"):
        if line.strip():
            s, f, v = line.split()
            lay[(s, f)] = int(v)
    return lay


def test_struct_fields_and_offsets_match_header():
    lay = c_layout()
    for cname, py in STRUCTS.items():
        assert ctypes.sizeof(py) == lay[(cname, "size")], cname
        for f, _ in py._fields_:
            assert getattr(py, f).offset == lay[(cname, f)], (cname, f)


def test_header_fields_all_bound():
    # every field the header declares in pcg_opts / pcg_stats / pcg_tuning is in the binding
    import re
    h = open(os.path.join(ROOT, "include", "pcgpu.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    for cname, py in STRUCTS.items():
        if cname == "pcg_i128":
            continue
        body = re.search(r"typedef struct \{([^{}]*)\} %s;" % cname, h).group(1)
        names = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            first, *rest = [p.strip() for p in decl.split(",")]
            names.append(re.split(r"[\s*]+", first)[-1])
            names += rest
        assert names == [f for f, _ in py._fields_], cname

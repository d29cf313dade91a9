"""The ctypes mirrors of the C ABI's structs (go-melt_gb300/_native.py) against
include/gomelt.h: for every struct both declare, the size and the offset of
every field, as a C compiler lays them out (gcc on the header; no GPU)."""

import ctypes as C
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_structs():
    with open(os.path.join(ROOT, "include", "gomelt.h")) as f:
        return set(re.findall(r"^\}\s*(gm_\w+)\s*;", f.read(), flags=re.M))


def _mirrors():
    import _native as N

    out = {}
    for name in dir(N):
        cls = getattr(N, name)
        if isinstance(cls, type) and issubclass(cls, C.Structure) and name.startswith("gm_"):
            out[name] = cls
    return out


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_ctypes_structs_match_the_header():
    structs = _header_structs()
    mirrors = {k: v for k, v in _mirrors().items() if k in structs}
    assert len(mirrors) >= 20, sorted(mirrors)
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gomelt.h"', "int main(void) {"]
    for name, cls in sorted(mirrors.items()):
        lines.append(f'  printf("{name} sizeof %zu\\n", sizeof({name}));')
        for fname, *_ in cls._fields_:
            cname = "in" if fname == "in_" else fname
            lines.append(f'  printf("{name} {fname} %zu\\n", offsetof({name}, {cname}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines) + "\n")
        r = subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    bad = []
    for line in out:
        if not line:
            continue
        name, field, val = line.split()
        cls = mirrors[name]
        py = C.sizeof(cls) if field == "sizeof" else getattr(cls, field).offset
        if py != int(val):
            bad.append(f"{name}.{field}: C {val}, ctypes {py}")
    assert not bad, bad

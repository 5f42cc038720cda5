"""The ctypes mirrors of include/fjgpu.h (fjmodels_gb300/_abi.py) against the header itself:
every structure's size and every field's offset, from a C program compiled against the
header on this host.  A field added on one side only would otherwise shift the rest of a
structure the library reads."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from fjmodels_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _structures():
    return sorted((n, t) for n, t in vars(A).items()
                  if isinstance(t, type) and issubclass(t, C.Structure) and n.startswith("fj_"))


def test_every_mirror_is_checked():
    names = [n for n, _ in _structures()]
    assert "fj_model_config" in names and "fj_model_result" in names and len(names) >= 8


def test_layout_matches_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fjgpu.h"', "int main(void) {"]
    expect = []
    for name, t in _structures():
        lines.append(f'    printf("%zu\\n", sizeof({name}));')
        expect.append((name, "sizeof", C.sizeof(t)))
        for f in t._fields_:
            lines.append(f'    printf("%zu\\n", offsetof({name}, {f[0]}));')
            expect.append((name, f[0], getattr(t, f[0]).offset))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert len(got) == len(expect)
    bad = [(n, f, e, g) for (n, f, e), g in zip(expect, got) if e != g]
    assert not bad, bad

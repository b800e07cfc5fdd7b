"""The ctypes mirrors of the C ABI's structures (scamp_gb300/_lib.py) against
include/scamp_gb300.h: a small C program compiled with the host compiler
prints every field's offset and each structure's size, which must equal
ctypes' layout.  CPU only."""
import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import REPO

from scamp_gb300 import _lib


def _c_layout(tmp_path, struct, fields):
    src = tmp_path / ("%s.c" % struct)
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "scamp_gb300.h"',
             "int main(void) {",
             '  printf("size %%zu\\n", sizeof(%s));' % struct]
    for f in fields:
        lines.append('  printf("%s %%zu\\n", offsetof(%s, %s));' % (f, struct, f))
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / struct
    subprocess.run([shutil.which("gcc") or "gcc", "-std=c11", "-I", os.path.join(REPO, "include"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict((k, int(v)) for k, v in (line.split() for line in out.splitlines()))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
@pytest.mark.parametrize("struct,mirror", [("scamp_c_args", _lib.CArgs),
                                           ("scamp_c_result", _lib.CResult)])
def test_ctypes_mirror_matches_header(tmp_path, struct, mirror):
    names = [f[0] for f in mirror._fields_]
    got = _c_layout(tmp_path, struct, names)
    assert got["size"] == ctypes.sizeof(mirror), struct
    for name in names:
        assert got[name] == getattr(mirror, name).offset, (struct, name)

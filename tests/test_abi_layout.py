"""The ctypes mirror of include/kura.h has the C layout: every struct's size and every
field's offset, as a C compiler lays them out (compiled here with gcc, no GPU needed)."""
import ctypes
import json
import os
import shutil
import subprocess

import pytest

from kuramoto_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "kura_config": native.Config,
    "kura_stats": native.Stats,
    "kura_instance": native.Instance,
    "kura_multi_stats": native.MultiStats,
    "kura_callbacks": native.Callbacks,
}


def test_ctypes_mirror_matches_c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kura.h"', "int main(void) {", 'printf("{");']
    first = True
    for cname, cls in STRUCTS.items():
        sep = "" if first else ","
        first = False
        lines.append('printf("%s\\"%s\\": {\\"size\\": %%zu", sizeof(%s));' % (sep, cname, cname))
        for fname, _ in cls._fields_:
            lines.append('printf(", \\"%s\\": %%zu", offsetof(%s, %s));' % (fname, cname, fname))
        lines.append('printf("}");')
    lines += ['printf("}\\n");', "return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    for cname, cls in STRUCTS.items():
        c = got[cname]
        assert ctypes.sizeof(cls) == c["size"], cname
        for fname, _ in cls._fields_:
            assert getattr(cls, fname).offset == c[fname], (cname, fname)

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


def _kind_c(t):
    t = t.replace("const", "").strip()
    if "*" in t:
        return "ptr"
    return {"int": "i32", "int32_t": "i32", "int64_t": "i64", "uint64_t": "u64", "float": "f32",
            "double": "f64", "void": None}[t]


def _kind_ct(t):
    if t is None:
        return None
    simple = {ctypes.c_int32: "i32", ctypes.c_int64: "i64", ctypes.c_uint64: "u64", ctypes.c_float: "f32",
              ctypes.c_double: "f64"}
    if t in simple:
        return simple[t]
    return "ptr"  # c_void_p, c_char_p, POINTER(...)


def test_ctypes_signatures_match_the_header():
    """Every function the mirror binds has the header's parameter count and kinds (32/64-bit
    integer, float, double, pointer) and return kind."""
    import re
    text = open(os.path.join(ROOT, "include", "kura.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    text = " ".join(text.split())
    protos = {}
    for ret, name, params in re.findall(r"((?:const )?\w+\s*\**)\s*(kura_\w+)\s*\(([^()]*)\)\s*;", text):
        ps = [] if params.strip() in ("", "void") else [p.strip() for p in params.split(",")]
        kinds = [_kind_c(re.sub(r"\b\w+$", "", p).strip() or p) for p in ps]
        protos[name] = (_kind_c(ret), kinds)
    L = native.lib()
    checked = 0
    for name, (ret, kinds) in protos.items():
        f = getattr(L, name)
        if f.argtypes is None:  # not bound by the mirror (called with explicit types elsewhere)
            continue
        assert [_kind_ct(a) for a in f.argtypes] == kinds, name
        assert _kind_ct(f.restype) == ret, name
        checked += 1
    assert checked >= 30, (checked, sorted(protos))

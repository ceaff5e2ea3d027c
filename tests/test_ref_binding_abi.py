"""The ctypes structures of both bindings -- the product's (phd_code_gb300._lib) and the
reference-side one (tests/ref_binding.py, also printed in INTEGRATION.md) -- against
include/phdflux.h itself: sizeof and every field offset, read from a C program compiled
with the host compiler.  A structure that drifts from the header (a field added on one
side only) fails here, before any device call could write past a caller's buffer."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

import phd_code_gb300._lib as L
import ref_binding as RB

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {"phd_mesh": L.PhdMesh, "phd_clock": L.PhdClock, "phd_params": L.PhdParams, "phd_geom32": L.PhdGeom32,
           "phd_geom32_out": L.PhdGeom32Out, "phd_launch": L.PhdLaunch, "phd_handover32": L.PhdHandover32,
           "phd_adj_index": L.PhdAdjIndex}


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def layout(tmp_path_factory):
    inc = _cuda_include()
    cc = shutil.which("gcc") or shutil.which("cc")
    if inc is None or cc is None:
        pytest.skip("no host compiler or CUDA headers")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "phdflux.h"', "int main(void) {"]
    for name, cls in STRUCTS.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("  return 0; }")
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "abi.c", d / "abi"
    src.write_text("\n".join(lines) + "\n")
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), "-I", inc, str(src), "-o", str(exe)])
    out = {}
    for ln in subprocess.check_output([str(exe)]).decode().split("\n"):
        if ln.strip():
            s, f, v = ln.split()
            out[(s, f)] = int(v)
    return out


def _check(cls, cname, layout):
    assert C.sizeof(cls) == layout[(cname, "sizeof")], cname
    for f, _ in cls._fields_:
        assert getattr(cls, f).offset == layout[(cname, f)], (cname, f)


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_product_binding_matches_header(cname, layout):
    _check(STRUCTS[cname], cname, layout)


def test_reference_binding_matches_header(layout):
    _check(RB.PhdMesh, "phd_mesh", layout)
    _check(RB.PhdClock, "phd_clock", layout)
    _check(RB.PhdParams, "phd_params", layout)


def test_integration_document_matches_header(layout):
    """The structures INTEGRATION.md prints for a maintainer, executed as written."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", text, re.S)
    ns = {"C": C}
    found = set()
    for b in blocks:
        for m in re.finditer(r"^class (Phd\w+)\(C\.Structure\):[^\n]*\n(?:    .*\n|\n)+", b, re.M):
            exec(m.group(0), ns)
            found.add(m.group(1))
    assert {"PhdMesh", "PhdClock"} <= found
    names = {"PhdMesh": "phd_mesh", "PhdClock": "phd_clock", "PhdParams": "phd_params"}
    for cls_name in found:
        _check(ns[cls_name], names[cls_name], layout)

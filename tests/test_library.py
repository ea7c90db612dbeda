"""The C-ABI library builds, loads and exports every entry point that include/ttgb300.h declares
(no compute: these run without a GPU)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ttgb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ttgb_[A-Za-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built():
    from torchtt_gb300 import build
    return build.build()


def test_header_declares_the_abi():
    syms = declared_symbols()
    assert "ttgb_amen_solve" in syms and "ttgb_local_product" in syms
    assert len(syms) >= 17


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s+(ttgb_[A-Za-z0-9_]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_ctypes_binding_covers_the_header(built):
    from torchtt_gb300 import _lib
    assert sorted(_lib.EXPORTED) == declared_symbols()
    L = _lib.lib()
    assert L.ttgb_version() == 103
    p = _lib.AmenParams()
    L.ttgb_default_params(p)
    # defaults of torchtt/solvers.py:211
    assert (p.nswp, p.eps, p.rmax, p.max_full, p.kickrank, p.kick2, p.local_iterations, p.resets) == \
        (22, 1e-10, 32768, 500, 4, 0, 40, 2)


def test_sm103a_only(built):
    """The shared object carries sm_103a code (cuobjdump is not used: the ELF notes list the arch)."""
    from torchtt_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_ctypes_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of ttgb_tt, ttgb_amen_params and ttgb_stats have the C compiler's size and
    field offsets (a binding with a stale layout would read or overrun the wrong bytes)."""
    import ctypes
    from torchtt_gb300 import _lib
    mirrors = {"ttgb_tt": _lib.TTDesc, "ttgb_amen_params": _lib.AmenParams, "ttgb_stats": _lib.Stats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "ttgb300.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {" ".join(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln.strip()}
    for cname, cls in mirrors.items():
        assert got[cname + " size"] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got["%s %s" % (cname, f)] == getattr(cls, f).offset, (cname, f)

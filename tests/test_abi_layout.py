"""The ctypes mirrors of the C ABI structs (partensor-toolbox_gb300/_lib.py) against the layout
the C compiler gives include/ptg.h: every struct's size and every field's offset, checked on
this host with gcc (no GPU).  A mismatch would corrupt every options or result struct that
crosses the boundary."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (C typedef in include/ptg.h, ctypes class in _lib.py)
PAIRS = [("ptg_cpd_options", "CpdOptions"), ("ptg_cpd_result", "CpdResult"),
         ("ptg_cpd_instance", "CpdInstance"), ("ptg_sweep_trace", "SweepTrace"), ("ptg_stats", "Stats"),
         ("ptg_gtc_options", "GtcOptions"), ("ptg_gtc_result", "GtcResult")]


def test_ctypes_structs_match_c_layout(pkg, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ptg.h"', "int main(void) {"]
    for cname, pyname in PAIRS:
        cls = getattr(pkg._lib, pyname)
        lines.append(f'printf("{pyname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{pyname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    checked = 0
    for line in out.splitlines():
        pyname, field, value = line.split()
        cls = getattr(pkg._lib, pyname)
        got = ctypes.sizeof(cls) if field == "size" else getattr(cls, field).offset
        assert got == int(value), (pyname, field, got, int(value))
        checked += 1
    assert checked == sum(1 + len(getattr(pkg._lib, p)._fields_) for _, p in PAIRS)


def test_context_option_errors_without_gpu(pkg):
    """ptg_ctx_set_option rejects a NULL context before touching a device."""
    lib = pkg._lib.load()
    rc = lib.ptg_ctx_set_option(None, pkg._lib.PTG_OPT_GTC_ROWS, 0)
    assert rc == pkg._lib.PTG_ERR_INVALID
    assert b"NULL" in lib.ptg_last_error()

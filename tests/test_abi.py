"""The C-ABI boundary without a GPU: the library loads, exports every entry
point the header declares, the ctypes layouts equal the C layouts, and the
host-only entry points work."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "qsft_gb300.h")


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from qsft_gb300 import _lib
    return _lib.load()


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qsft_[a-z_0-9]+)\s*\(", src)))


def test_exports_every_declared_symbol(lib):
    from qsft_gb300 import _lib
    declared = header_functions()
    assert declared, "no declarations parsed"
    assert sorted(_lib.SYMBOLS) == declared
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (qsft_\w+)", out))
    assert set(declared) <= exported


def test_struct_layouts_match_header(tmp_path):
    from qsft_gb300._lib import QsftCtrl, QsftJob, QsftPlan
    fields = {"qsft_job": QsftJob, "qsft_ctrl": QsftCtrl, "qsft_plan": QsftPlan}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qsft_gb300.h"', 'int main(void){']
    for cname, ct in fields.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in ct._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    got = dict()
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, ct in fields.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(ct)
        for f, _ in ct._fields_:
            assert got[(cname, f)] == getattr(ct, f).offset, (cname, f)


def test_host_entry_points(lib):
    from qsft_gb300._lib import QsftJob
    assert lib.qsft_abi_version() == 1
    assert lib.qsft_built_arch() == 103
    assert lib.qsft_status_string(0) == b"ok"
    jobs = (QsftJob * 2)()
    for j, (q, n, b, C) in enumerate([(4, 20, 7, 3), (20, 10, 3, 3)]):
        jobs[j].q, jobs[j].n, jobs[j].b, jobs[j].C = q, n, b, C
        jobs[j].R, jobs[j].P, jobs[j].B = 2, n + 1, q ** b
    tb, ts, tl = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    ks = ctypes.c_int32()
    assert lib.qsft_workspace_layout(jobs, 2, ctypes.byref(tb), ctypes.byref(ts), ctypes.byref(tl),
                                     ctypes.byref(ks)) == 0
    assert tb.value == 3 * 16384 + 3 * 8000
    assert jobs[1].off_bin == 3 * 16384
    assert jobs[0].table_cap == 131072 and jobs[1].table_cap == 65536
    assert ks.value == 32
    # invalid shape is rejected, not crashed on
    jobs[0].q = 1
    assert lib.qsft_workspace_layout(jobs, 2, ctypes.byref(tb), ctypes.byref(ts), ctypes.byref(tl),
                                     ctypes.byref(ks)) == -1


def test_gpu_entry_points_reject_bad_arguments_without_launching(lib):
    """Argument checks run before any CUDA call, so they are safe on a CPU host."""
    assert lib.qsft_gwht(4, 1, 3, None, None, 1, None) == -1          # q < 2
    assert lib.qsft_gwht(4, 4, 12, None, None, 1, None) == -3         # q^b too large
    assert lib.qsft_gwht(3, 4, 3, None, None, 1, None) == -1          # bad precision... null data
    assert lib.qsft_eval_points(4, 40, 10, 5, None, 10, None, None, None, None) == -1
    assert lib.qsft_rs_decode(5, 3, 17, 100, None, None, 1, None, None) == -1   # t > 16
    assert lib.qsft_add_bins(4, None, None, -1, None) == -1
    assert lib.qsft_eval_cosets(None, None) == -1
    assert lib.qsft_peel_iteration(None, 1, None) == -1

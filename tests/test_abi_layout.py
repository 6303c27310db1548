"""The Python front-end's ctypes structures against the C header's layout: a C
probe compiled from include/busseq_gb300.h prints every struct's size and each
field's offset, which must equal the ctypes ones (a drift would pass wrong
values through every call without an error)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

import busseq_gpu_gb300 as bq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C struct name -> (ctypes structure, C field names in declaration order)
STRUCTS = {
    "busseq_dims": bq.Dims,
    "busseq_options": bq.Options,
    "busseq_estimates": bq.Estimates,
    "busseq_preserved": bq.Preserved,
    "busseq_state": bq.State,
    "busseq_log_ratios": bq.LogRatios,
    "busseq_sim_params": bq.SimParams,
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "busseq_gb300.h"', "int main(void) {"]
    for name, st in STRUCTS.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in st._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines += ["  return 0;", "}"]
    src = d / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(d / "probe")
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe], stdout=subprocess.PIPE, text=True, check=True).stdout
    lay = {}
    for line in out.splitlines():
        a, b, v = line.split()
        lay[(a, b)] = int(v)
    return lay


@pytest.mark.parametrize("name", sorted(STRUCTS))
def test_ctypes_structures_match_the_header(c_layout, name):
    st = STRUCTS[name]
    assert C.sizeof(st) == c_layout[(name, "size")], name
    for f, _ in st._fields_:
        assert getattr(st, f).offset == c_layout[(name, f)], (name, f)

"""CPU tests of the drop-in boundary: the C-ABI library builds, loads and
exports every entry point include/satsuma2_xcorr.h declares, with struct layouts
identical to the reference's wire structs.  No compute call (no GPU here)."""
import ctypes
import os
import re
import subprocess

import pytest

import satsuma2_gb300 as sg
from satsuma2_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "satsuma2_xcorr.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return sg.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xc_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_what_binding_exports():
    assert set(declared_functions()) == set(sg.EXPORTS)


def test_library_exports_every_symbol(lib):
    out = subprocess.check_output(["nm", "-D", "--defined-only", sg.LIB_PATH]).decode()
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [f for f in declared_functions() if f not in syms]
    assert not missing, missing
    for f in declared_functions():
        assert hasattr(lib, f)


def test_struct_layouts():
    # t_result (analysis/WorkQueue.h:23-33) and t_pair (:17-22) sizes on LP64
    assert sg.RESULT_DTYPE.itemsize == 72
    assert sg.RESULT_DTYPE.fields["prob"][1] == 56
    assert ctypes.sizeof(sg.Pair) == 64
    assert ctypes.sizeof(sg.Params) == 72


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "satsuma2_xcorr.h"\n'
                   '_Static_assert(sizeof(xc_result) == 72, "t_result");\n'
                   '_Static_assert(sizeof(xc_block) == 28, "t_pair");\n'
                   'int main(void) { return 0; }\n')
    subprocess.check_call(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                           str(src), "-o", str(tmp_path / "t")])


def test_version(lib):
    assert b"sm_103a" in lib.xc_version()


def test_no_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sg.XCError) as e:
        sg.XCorr()
    assert e.value.code == -2   # XC_ERR_CUDA, never a CPU fallback

"""CPU-only checks of the C-ABI library: it builds for sm_103a, loads, and
exports every entry point include/sanepic_gpu.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

import sanepic_gb300 as sg
from sanepic_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "sanepic_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(sg_[a-z_]+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def test_header_matches_python_mirror():
    assert declared_symbols() == sorted(sg.EXPORTS)


def test_library_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_struct_layouts_match_header():
    # sizes of the by-value structs shared with C (LP64)
    assert ctypes.sizeof(sg.SgDesc) == 8 * 4 + 4 + 4 + 8 + 4 + 4
    assert ctypes.sizeof(sg.SgDet) == 24
    assert ctypes.sizeof(sg.SgReport) == 4 + 4 + 8 * 6 + 8 + 8 + 8
    # precond, stop_crit, maxiter, refresh_every, verbose, x0, use_graph,
    # on_iteration, user (natural alignment, LP64)
    assert ctypes.sizeof(sg.SgSolveOpts) == 64


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError):
        sg.load_library(str(tmp_path / "nope.so"))


def test_noalloc_rejects_oversized_group_before_any_cuda_call(libpath):
    # a filter group larger than INT_MAX tiles (and not larger than ntiles)
    # cannot be narrowed to the kernel's int: refused as an argument error,
    # before any CUDA call (this runs without a GPU)
    sg.load_library(libpath)
    rc = sg.noise_filter_noalloc(16, 16, 16, 4096, 1 << 40, (1 << 31) + 5, None)
    assert rc == sg.SG_ERR_ARG
    # sizes outside [256, 131072] are refused before any CUDA call too
    assert sg.noise_filter_noalloc(16, 16, 16, 1 << 18, 1, 1, None) == sg.SG_ERR_UNSUPPORTED
    assert sg.noise_filter_noalloc(0, 16, 16, 4096, 1, 1, None) == sg.SG_ERR_ARG

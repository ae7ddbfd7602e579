"""C-ABI checks that need no GPU: the library builds, loads and exports every entry point that
include/gbturbo.h declares; the Python binding binds exactly those."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import PKG, ROOT


def declared():
    txt = open(os.path.join(ROOT, "include", "gbturbo.h")).read()
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_expected_entry_points(gbturbo):
    assert declared() == sorted(gbturbo.EXPORTED)


def test_library_builds_and_exports_all_symbols():
    import build as pkg_build
    lib = pkg_build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    syms = set(re.findall(r"\sT\s(gb_\w+)", out))
    missing = [s for s in declared() if s not in syms]
    assert not missing, missing


def test_library_loads_without_gpu(gbturbo):
    L = gbturbo.load()
    for name in declared():
        assert hasattr(L, name)
    # a call that needs no device: the error string of the calling thread
    assert isinstance(L.gb_last_error(), bytes)
    # argument checks fail before any CUDA call
    h = ctypes.c_void_p()
    assert L.gb_solver_create(None, 0, 0, ctypes.byref(h)) == -1


def test_case_reader_parity_with_oracle_options(meshgen, tmp_path, oracle_mod):
    """the oracle (C) reads the same files; both agree on the level count"""
    case = meshgen.rotor_passage(IM=17, JM=17, KM=65, options={"multigrid": "Y", "coarse_iter": "3"})
    meshgen.write_case(case, str(tmp_path))
    o = oracle_mod.Oracle(str(tmp_path))
    assert o.dims(1)[3] == 2
    assert o.dims(2)[:3] == (9, 9, 33)


def test_warm_start_entry_points_check_their_arguments_without_gpu(gbturbo):
    """the gb_ws_* group and gb_start_from_fine_state reject null handles and buffers before any
    CUDA call"""
    L = gbturbo.load()
    f = ctypes.POINTER(ctypes.c_float)
    assert L.gb_ws_create(0, None) == -1
    assert L.gb_ws_add_solves(None, None, None) == -1
    assert L.gb_ws_train(None, 10, 1024, ctypes.c_float(1e-3), None) == -1
    assert L.gb_ws_apply(None, None, None, None, None, None) == -1
    assert L.gb_ws_get_params(None, None) == -1
    assert L.gb_ws_set_norm(None, None) == -1
    assert L.gb_ws_forward(None, None, 0, None) == -1
    assert L.gb_ws_forward_backward(None, None, None, 0, None, None) == -1
    assert L.gb_ws_benchmark(None, 1024, 1, None, None, None, None) == -1
    assert L.gb_ws_samples(None) == -1
    assert L.gb_start_from_fine_state(None) == -1
    assert L.gb_ws_destroy(None) == 0
    assert b"null" in L.gb_last_error()

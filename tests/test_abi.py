"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/glphase_gpu.h; argument errors come back as status codes
without touching a GPU."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from glphase_gb300 import build, native
    build.build()
    return native.load()


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "glphase_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(glp_[a-z0-9_]+)\s*\(", hdr)))


def test_header_declares_expected_entry_points():
    from glphase_gb300 import native
    assert declared_symbols() == sorted(native.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_null_context_errors(lib):
    assert lib.glp_set_lanes_per_sample(None, 4) == 1
    assert lib.glp_set_evals_per_lane(None, 2) == 1
    assert lib.glp_set_block_sites(None, 4) == 1
    assert lib.glp_get_block_sites(None, None) == 1
    assert lib.glp_get_counters(None, None, 0) == 1
    assert lib.glp_kernel_times(None, 0, None, None) == 1
    assert lib.glp_get_stats(None, None, None, None) == 1
    assert lib.glp_last_error(None) == b"null context"
    assert lib.glp_run_generation(None, None) == 1
    assert lib.glp_set_tran(None, None, 0) == 1
    assert lib.glp_vq_train(None, None, 0, 16, None, 0, 10, None) == 1
    assert lib.glp_vq_pack(None, None, 0, 0, None, 16, 4, None) == 1
    assert lib.glp_server_create(None, 1 << 30, 0, None) == 1
    assert lib.glp_server_submit(None, None, None, 1, None) == 1
    assert lib.glp_server_tick(None, None, None) == 1
    assert lib.glp_server_poll(None, 1, None, None, None) == 1
    assert lib.glp_server_stats(None, None, None, None) == 1
    assert lib.glp_server_release(None, 1) == 1
    lib.glp_server_destroy(None)


def test_shim_header_compiles():
    """include/hmmlike_cuda_shim.hpp compiles as plain C++ against the C ABI."""
    import subprocess, tempfile
    src = '#include "hmmlike_cuda_shim.hpp"\nint main(){return 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "t.cpp")
        open(f, "w").write(src)
        subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I",
                        os.path.join(ROOT, "include"), f], check=True)


def test_header_compiles_as_c99():
    """include/glphase_gpu.h is a C header: strict C99, no C++ constructs, so
    a C caller (or a cgo / FFI binding generator) can include it."""
    import subprocess, tempfile
    src = ('#include "glphase_gpu.h"\n'
           'int main(void) { glp_generation_args a = {0}; glp_ctx *c = 0; (void)a; (void)c;\n'
           '  return GLP_REQ_DONE == 2 ? 0 : 1; }\n')
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "t.c")
        open(f, "w").write(src)
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-fsyntax-only", "-I", os.path.join(ROOT, "include"), f], check=True)

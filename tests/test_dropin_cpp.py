"""The C++ drop-in for the reference's device API (namespace HMMLikeCUDA).

* The reference's own header src/hmmLike.h declares the functions extern;
  a translation unit compiled against it, unchanged, links against the
  out-of-line shim include/hmmlike_cuda_shim.cpp and libglphase_gpu.so in
  place of src/hmmLike.cu and runs the call sequence of HMMLike
  (src/hmmLike.cpp:45-111).  Built where the reference tree exists; without
  a device it must stop at CheckDevice with the shim's std::runtime_error.
* The reference's own host driver, src/hmmLike.cpp (class HMMLike) with
  src/glPack.cpp, src/glVQ.cpp and src/sampler.cpp, compiled unchanged
  against the same header and shim (GSL and the Boost-based
  src/olivier/utils.hpp replaced by oracle/ref_shim's stand-ins), running
  the planted-parent case of src/testing/cuda_tests.cpp:205-322 through
  HMMLike's constructor and RunHMMOnSamples.  Built where the reference
  tree exists; without a device HMMLike's constructor must see CheckDevice's
  std::runtime_error, with one the planted haplotypes must be found.
* On the GPU, a C++ driver of every HMMLikeCUDA function -- size errors,
  calls before SetDevice, the planted-parent run of
  src/testing/cuda_tests.cpp:205-322 -- linked the same way.
"""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

REF_SRC = "/root/reference/src"
LIBDIR = os.path.join(ROOT, "glphase_gb300")
INC = os.path.join(ROOT, "include")
DROPIN = os.path.join(ROOT, "tests", "dropin")


def _lib():
    from glphase_gb300 import native as nat
    path = nat.lib_path()
    if not os.path.exists(path):
        pytest.skip("libglphase_gpu.so is not built")
    return path


def _build(d, sources, extra, std):
    exe = os.path.join(d, "a.out")
    cmd = (["g++", f"-std={std}", "-O1", "-I", INC] + extra + ["-o", exe] + sources +
           ["-L", LIBDIR, "-lglphase_gpu", f"-Wl,-rpath,{LIBDIR}"])
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "hmmLike.h")),
                    reason="the reference tree is not present")
def test_reference_header_links_to_shim():
    _lib()
    cccl = "/usr/local/cuda/include/cccl"
    with tempfile.TemporaryDirectory() as d:
        exe = _build(d, [os.path.join(DROPIN, "reference_header_driver.cpp"),
                         os.path.join(INC, "hmmlike_cuda_shim.cpp")],
                     ["-I", REF_SRC, "-I", cccl, "-I", "/usr/local/cuda/include"], "c++17")
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    if out.returncode == 3:  # no device: the reference's HMMLike would see this exception
        assert "no sm_103 device" in out.stdout
    else:
        assert out.returncode == 0, out.stdout + out.stderr


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "hmmLike.cpp")),
                    reason="the reference tree is not present")
def test_reference_host_driver_links_to_shim():
    _lib()
    cccl = "/usr/local/cuda/include/cccl"
    shim = os.path.join(ROOT, "oracle", "ref_shim")
    srcs = [os.path.join(REF_SRC, f) for f in ("hmmLike.cpp", "glPack.cpp", "glVQ.cpp",
                                               "sampler.cpp")]
    with tempfile.TemporaryDirectory() as d:
        # C++17 for the CUDA toolkit's thrust headers, which hmmLike.hpp includes
        exe = _build(d, [os.path.join(DROPIN, "reference_hmmlike_driver.cpp"),
                         os.path.join(INC, "hmmlike_cuda_shim.cpp")] + srcs,
                     ["-w", "-I", shim, "-I", REF_SRC, "-I", cccl, "-I",
                      "/usr/local/cuda/include"], "c++17")
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    if out.returncode == 3:  # no device: what the reference's own caller would see
        assert "no sm_103 device" in out.stdout
    else:
        assert out.returncode == 0, out.stdout + out.stderr
        assert "MISSING" not in out.stdout


@pytest.mark.gpu
def test_shim_cpp_driver_planted_parents():
    _lib()
    with tempfile.TemporaryDirectory() as d:
        exe = _build(d, [os.path.join(DROPIN, "shim_planted_test.cpp"),
                         os.path.join(INC, "hmmlike_cuda_shim.cpp")], ["-Wall"], "c++11")
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 failure(s)" in out.stdout

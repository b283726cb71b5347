"""The kNN tract-length run logic of the device (glphase_gb300/csrc/
glp_tract.h: tract_word per 64-site word, tract_join in site order, as
knn_tract_dist_kernel runs them) compiled for the host with g++ and checked
against the oracle's Haplotype::MaxTractLen restatement, which the
reference's own haplotype.cpp pins: common sites minus the longest run of
agreeing common sites, for every word shape the kernel meets -- all sites
common (the six-step run finder), part of them common (the loop over
disagreements), no disagreement, disagreements at bits 0 and 63, ragged last
words."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = r'''
#include "glp_tract.h"
extern "C" uint32_t tract_dist(const uint64_t *a, const uint64_t *b, const uint64_t *m,
                               uint32_t wn) {
  glp::Tract r{0, 0, 0, 0};
  for (uint32_t w = 0; w < wn; ++w)
    r = glp::tract_join(r, glp::tract_word((a[w] ^ b[w]) & m[w], m[w]));
  return r.len - r.best;
}
'''


@pytest.fixture(scope="module")
def tract_lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("tract")
    src, lib = d / "tract.cpp", d / "libtract.so"
    src.write_text(SRC)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-Wno-unknown-pragmas",
                    "-I", os.path.join(ROOT, "glphase_gb300", "csrc"), str(src), "-o", str(lib)],
                   check=True)
    L = C.CDLL(str(lib))
    p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
    L.tract_dist.restype = C.c_uint32
    L.tract_dist.argtypes = [p, p, p, C.c_uint32]
    return L


def _words(rng, wn, kind):
    if kind == "dense":
        return rng.integers(0, 2**64, wn, dtype=np.uint64)
    x = np.zeros(wn, np.uint64)  # a few disagreements a word, bits 0 and 63 included
    for w in range(wn):
        for b in rng.choice([0, 63, *rng.integers(0, 64, 3)], size=int(rng.integers(0, 4))):
            x[w] |= np.uint64(1) << np.uint64(b)
    return x


def test_device_tract_runs_match_oracle(tract_lib, oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(13)
    full = np.uint64(2**64 - 1)
    for t in range(3000):
        wn = int(rng.integers(1, 9))
        kind = "dense" if t % 4 == 0 else "sparse"
        a = rng.integers(0, 2**64, wn, dtype=np.uint64)
        b = a ^ _words(rng, wn, kind)
        if t % 3 == 0:
            m = np.full(wn, full)
        elif t % 3 == 1:
            m = rng.integers(0, 2**64, wn, dtype=np.uint64) | _words(rng, wn, "sparse")
        else:  # all common but a ragged last word
            m = np.full(wn, full)
            m[-1] = np.uint64((1 << int(rng.integers(1, 64))) - 1)
        ncommon = sum(bin(int(x)).count("1") for x in m)
        assert tract_lib.tract_dist(a, b, m, wn) == ncommon - O.max_tract(a, b, m), t

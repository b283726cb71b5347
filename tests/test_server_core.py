"""The request server's scheduling (glphase_gb300/csrc/glp_server_core.h,
the host logic behind glp_server_*) built with the host C++ compiler and run
against a fake launcher (tests/server_core_test.cpp): admission in arrival
order under the budget, the per-request generation arguments (annealing
penalty, buffer exchange, kick-start range), launch grouping by emission
source or per request, retirement and release.  No GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_server_core(tmp_path):
    exe = str(tmp_path / "server_core_test")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-ffp-contract=off",
                    os.path.join(ROOT, "tests", "server_core_test.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr

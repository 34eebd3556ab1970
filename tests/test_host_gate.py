"""The solve server's gate on block-solve batches (elastic_gb300/csrc/
elx_gate.h), checked on the host: tests/gate_check.cpp built with the
system C++ compiler and run (its cases are listed in its header)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_batch_gate(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "gate_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-pthread", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "elastic_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "gate_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "gate_check: ok" in r.stdout

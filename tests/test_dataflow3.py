"""The tile dataflow graph of the 3D sweeps (pfast_gb300/csrc/dataflow3.h), on the CPU: a
small C++ driver (tests/native/dataflow3_check.cpp) is compiled with g++ and runs the
dataflow kernel's counter protocol under random concurrent schedules on grids from 1x1x1 to
5x2x3 tiles.  Every item must run exactly once, after all of its dependencies, never beside
a face neighbour's item, and no counter may fall below zero."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_dataflow_graph_and_counter_protocol(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "dataflow3_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "pfast_gb300", "csrc"),
                    os.path.join(HERE, "native", "dataflow3_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-2000:]
    lines = out.stdout.split()
    assert "FAIL" not in out.stdout and out.stdout.count("ok ") == 27


def test_autotuner_policy():
    """The 3D autotuner's choice (pfast_gb300/csrc/tune_policy.h), compiled with g++ by
    tests/native/tune_policy_check.cpp: the candidates each schedule / tile-shape option allows
    (per diagonal when the grid does not fit the dataflow kernel), the untuned default
    (dataflow from two sources per SM), and the fastest mean once all allowed are timed."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "tune_policy_check")
        subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "pfast_gb300", "csrc"),
                        os.path.join(HERE, "native", "tune_policy_check.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout
    assert "FAIL" not in out.stdout and out.stdout.count("ok ") == 19

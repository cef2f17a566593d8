"""Admission policy of the request server (pfast_gb300/csrc/serve_policy.h), on the CPU:
a small C++ driver (tests/native/serve_policy_check.cpp) is compiled with g++ and its
decisions checked."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def lines(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("policy") / "serve_policy_check")
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "pfast_gb300", "csrc"),
                    os.path.join(HERE, "native", "serve_policy_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return {l.split()[0]: l.split()[1:] for l in out.splitlines()}


def test_alone_request_takes_the_budget(lines):
    # 100 fixed + 50 per source in 1000 bytes: 18 sources at once
    assert lines["alone"] == ["1", "18", "1000", "1000"]


def test_waiting_requests_share_the_budget(lines):
    # budget 1000, 2 slots: each gets a 500-byte share -> 8 sources; a third waits for a slot
    assert lines["shares"] == ["1", "8", "2", "8", "-1", "1000"]


def test_bounded_bypass(lines):
    # 3 and 4 overtake 2; then 2 blocks admission until it fits (5 may not overtake it);
    # once 2 runs (910 bytes), 5 (20 bytes) fits beside it
    assert lines["bypass"] == ["1", "3", "4", "-1", "2", "5"]


def test_resident_reservations_and_feasibility(lines):
    # 600 reserved, a second 600 refused; the request gets the free 400: 100 fixed + 3 sources
    assert lines["reserve"] == ["1", "0", "1", "3", "1000", "0"]

"""The library's host sampler of the reference's glibc label stream
(eddy_host.cpp: the TYPE_3 generator drawn a block of words at a time, and
the rejection sampler of main.cu:538-573) against glibc's own rand() as the
oracle draws it (or_glibc_labels), compiled and run on the CPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "eddy-gpu_gb300", "csrc")


@pytest.fixture(scope="module")
def sampler(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("glibc") / "glibc_stream")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    "-I", CSRC, os.path.join(HERE, "glibc_stream_main.cpp"),
                    os.path.join(CSRC, "eddy_host.cpp"), "-o", out], check=True)
    return out


@pytest.mark.parametrize("n,n1,R", [(2, 1, 20), (40, 15, 30), (1000, 400, 12), (1031, 500, 6)])
def test_library_stream_matches_glibc(sampler, oracle_lib, n, n1, R):
    r = subprocess.run([sampler, str(n), str(n1), str(R)], capture_output=True, text=True, check=True)
    lines = r.stdout.split("\n")
    got = np.array([[int(ch) for ch in ln] for ln in lines[:R]], np.uint8)
    assert lines[R] == "copy ok"
    labels0 = np.array([0 if s % 3 == 0 else 1 for s in range(n)], np.uint8)
    want = oracle_lib.glibc_labels(n, n1, labels0, R, reset=True)
    assert np.array_equal(got, want)

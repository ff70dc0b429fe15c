"""CPU: the descriptor producer's float-float exp and atan2
(skylens-stream-rs_gb300/csrc/fmath_cr.h) against the double functions
rounded to float, compiled for the host from the same source the kernels use.
Each result must be identical: the float-float value is returned only when its
rounding is settled by its error bound, else the double function is used.
(Every float in (-87, 88) and 10^9 random atan2 arguments were checked the
same way once; these runs take a strided subset and 4 * 10^6 arguments.)"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "skylens-stream-rs_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("fmath") / "fmath_check")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-o", exe,
                           os.path.join(HERE, "fmath_check.cpp"), "-lm"])
    return exe


def run(exe, mode, arg):
    r = subprocess.run([exe, str(mode), str(arg)], capture_output=True, text=True, timeout=600)
    bad, n = map(int, r.stdout.split()[-2:])
    return bad, n, r.stdout


def test_expf_equals_double_rounded(checker):
    bad, n, out = run(checker, 0, 257)  # about 8.7 M floats spread over the whole range
    assert n > 8_000_000 and bad == 0, out


def test_atan2f_equals_double_rounded(checker):
    bad, n, out = run(checker, 1, 4_000_000)
    assert n == 4_000_000 and bad == 0, out

"""The tree's monopoles are differences of 192-bit fixed-point prefix sums
(gravhopper_gb300/csrc/fixed192.cuh).  Its host build must give, for any range of
values, the exact sum of the values truncated to multiples of 2^lsb, rounded to the
nearest double (ties to even): checked here with exact rational arithmetic over
values spread across many binades, with both signs and zeros."""
import os
import shutil
import struct
import subprocess
from fractions import Fraction

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "fixed192_check.cpp")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("fixed192") / "fixed192_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, SRC], check=True)
    return exe


def _f(bits):
    return struct.unpack("<d", struct.pack("<Q", int(bits, 16)))[0]


def _trunc(x, lsb):
    q = Fraction(x) / Fraction(2) ** lsb
    t = q.numerator // q.denominator if q >= 0 else -((-q.numerator) // q.denominator)
    return Fraction(t) * Fraction(2) ** lsb


@pytest.mark.parametrize("seed,emin,emax,mbits", [(1, -40, 40, 52), (2, -5, 60, 52), (3, -300, -200, 52),
                                                  (4, 0, 1, 52), (5, -60, 37, 52), (6, 0, 60, 3), (7, 0, 60, 1)])
def test_fixed_point_range_sums_exact(checker, seed, emin, emax, mbits):
    """(mbits 1 and 3: two- and four-bit significands over 60 binades, so that range
    sums often land exactly halfway between two doubles.)"""
    out = subprocess.run([checker, "3000", "400", str(seed), str(emin), str(emax), str(mbits)],
                         capture_output=True, text=True, timeout=300, check=True).stdout.split("\n")
    lsb = int(out[0].split()[1])
    vals = [_trunc(_f(line.split()[1]), lsb) for line in out[1:] if line.startswith("v ")]
    prefix = [Fraction(0)]
    for x in vals:
        prefix.append(prefix[-1] + x)
    checked = 0
    for line in out:
        if not line.startswith("r "):
            continue
        _, s, e, bits = line.split()
        exact = prefix[int(e)] - prefix[int(s)]
        assert _f(bits) == float(exact), (s, e)
        checked += 1
    assert checked == 400

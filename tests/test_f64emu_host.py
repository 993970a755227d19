"""The integer-pipe FP64 inverse cube (gravhopper_gb300/csrc/f64emu.cuh) is pure
integer arithmetic apart from its FP32 rsqrt seed, so its host build must reproduce
the IEEE expression 1.0 / s / sqrt(s) of gravhopper/_jbgrav.c:166 bit for bit.
The check program runs random, boundary and near-midpoint inputs; with the seed
perturbed well beyond the FP32 approximation's error the range checks send inputs
to the native path, and no confirmed result may differ."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "f64emu_check.cpp")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("f64emu") / "f64emu_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, SRC], check=True)
    return exe


def _run(exe, cases, seed, perturb):
    r = subprocess.run([exe, str(cases), str(seed), str(perturb)], capture_output=True, text=True, timeout=300)
    total, wrong, fallback, out_of_range = map(int, r.stdout.split()[-4:])
    return r.returncode, total, wrong, fallback, out_of_range, r.stdout


def test_inverse_cube_bit_exact(checker):
    rc, total, wrong, fallback, out_of_range, log = _run(checker, 8_000_000, 11, 0)
    assert total >= 8_000_000
    assert wrong == 0 and out_of_range == 0, log
    assert fallback == 0, log  # an accurate seed never needs the native path
    assert rc == 0


@pytest.mark.parametrize("perturb", [22, 20, 16, 12])
def test_inverse_cube_robust_to_seed_error(checker, perturb):
    rc, total, wrong, fallback, out_of_range, log = _run(checker, 2_000_000, perturb, perturb)
    assert wrong == 0 and out_of_range == 0, log
    if perturb >= 22:
        assert fallback == 0, log
    assert rc == 0

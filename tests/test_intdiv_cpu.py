"""The integer-pipe binary64 division, square root and multiplication of the FP64 path
(fvleg_2d_gb300/csrc/cato_intdiv.cuh), compiled for the host with g++ and compared bit for bit
with the host's IEEE division, square root and multiplication (tests/intdiv_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("intdiv") / "intdiv_check")
    subprocess.run([gxx, "-O2", "-std=c++17", os.path.join(HERE, "intdiv_check.cpp"), "-o", exe],
                   check=True)
    return exe


def test_division_sqrt_and_product_bit_exact(checker):
    r = subprocess.run([checker, "1000000"], capture_output=True, text=True, timeout=600)
    lines = {ln.split()[0]: ln.split() for ln in r.stdout.splitlines() if " tested " in ln}
    assert set(lines) == {"div_random", "div_structured", "sqrt", "scale", "seeds", "mul"}, r.stdout
    for fam, f in lines.items():
        tested, fallback, bad = int(f[2]), int(f[4]), int(f[6])
        assert bad == 0, r.stdout
        assert tested > 1_000_000, (fam, r.stdout)
    # the full-range family sends the out-of-range quotients to the hardware instruction
    assert int(lines["div_random"][4]) > 0
    assert int(lines["seeds"][4]) == 0
    assert int(lines["mul"][4]) > 0  # subnormal and overflowing products take the hardware
    assert r.returncode == 0, r.stdout

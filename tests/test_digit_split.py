"""The closed-form digit split of the complex128 split products against the carry loop it
replaced, bit for bit, on 1 M host values per digit count (tests/digit_split_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(__file__)


def test_closed_form_digits_match_the_carry_loop(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "digit_split_check"
    subprocess.run([cxx, "-O2", "-o", str(exe), os.path.join(HERE, "digit_split_check.cpp")],
                   check=True)
    r = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "S=7 mismatches 0" in r.stdout

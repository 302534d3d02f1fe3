"""The short-chain pow of the device step control (csrc/fvm_pow.h), compiled for the host
with the same operations the device runs, against long double pow: within 1.5 ulp over
seeded arguments in its domain (x > 0 including subnormals, |y log2 x| < 1000)."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_pow_pos_accuracy(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "pow_accuracy"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", f"-I{ROOT / 'finitevolumemethod.jl_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "native" / "pow_accuracy.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    worst = float(out.split()[1])
    assert worst <= 1.5, out

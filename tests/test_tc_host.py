"""CPU check of the tensor-core vertical pass's host side: digit tiles, digit
table and error bound built by tc_build (tcvert.cu), replayed in exact
arithmetic by tests/tc_emul.cpp against the reference's double sums."""
import os
import subprocess

import pytest

from conftest import ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(ROOT, "imageworsener_gb300")
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def emul(tmp_path_factory, gpulib):   # gpulib: the library is built (loading it needs no GPU)
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not found")
    exe = str(tmp_path_factory.mktemp("tc") / "tc_emul")
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f"-I{LIBDIR}/csrc", f"-I{CUDA_INC}",
                        os.path.join(HERE, "tc_emul.cpp"), "-o", exe, f"-L{LIBDIR}", "-limagew_gb300",
                        f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


# (n_in, n_out, family code, p1): Lanczos3 at large and small factors, an odd
# factor, Mitchell (cubic family), and a few columns' worth of every channel
@pytest.mark.parametrize("args", [("8192", "256"), ("4096", "1000"), ("1000", "77"), ("777", "100"),
                                  ("3000", "97", "37", "0.333333333333", "96"), ("1500", "40", "49", "5", "64")])
def test_digit_sums_exact_and_within_bound(emul, args):
    r = subprocess.run([emul, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "violations=0" in r.stdout and "nonint=0" in r.stdout and "over2^24=0" in r.stdout, r.stdout

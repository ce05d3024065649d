"""Invariants of the quantisation tables (CPU): the library's own build_quant,
linked from libimagew_gb300.so by a small C++ checker
(tests/quant_tables_check.cpp).  The re-evaluation of the fast form steps
its bracket search from a coarse start table and reads one record per
bracket; this checks that the edges it steps over are ordered, that a
stepped search from any start lands where a binary search does, and that
every record equals the table entries it restates, over colour spaces,
depths, colour counts and dither families."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_quant_tables_invariants(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from imageworsener_gb300 import LIB_PATH, load
    load()   # builds the library if it is missing
    libdir = os.path.dirname(LIB_PATH)
    exe = str(tmp_path / "quant_tables_check")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "imageworsener_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "quant_tables_check.cpp"), "-L" + libdir, "-limagew_gb300",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr

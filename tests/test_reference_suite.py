"""The oracle pinned to the reference's own regression files: every line of
the reference's tests/runtest whose input and output are PNG or PNM/PAM is
replayed (tests/refsuite.py) and its output compared, value for value, with
the file in the reference's tests/expected/.

The same replay through the reference's own imagew, built here from its
sources, shows that the harness (PNG decoding, PNM/PAM stand-ins) is
faithful: a file that the reference itself does not reproduce would point at
the harness or at the machine, not at the oracle.

Runs where the reference's sources are present (tests skip elsewhere); the
GPU library is checked against the oracle by the GPU tests.
"""
import collections
import os
import subprocess

import pytest

import refsuite
from conftest import ROOT

TDIR = refsuite.reference_tests_dir()
pytestmark = pytest.mark.skipif(TDIR is None, reason="the reference's regression suite is not on this machine")

REF_CLI = os.path.join(ROOT, "oracle", "_ref", "imagew_ref")
ORACLE_CLI = os.path.join(ROOT, "oracle", "_build", "imagew_cli_oracle")
MIN_MATCHED = 156   # of the 196 lines: 4 more run through the library API below, 36 are other formats


def _make(target: str, path: str) -> str:
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), target], capture_output=True, text=True)
    if r.returncode or not os.path.exists(path):
        pytest.skip(f"{target} not buildable here: {r.stderr[-300:]}")
    return path


def _replay(exe: str, tmp_path) -> tuple[collections.Counter, list]:
    counts, bad = collections.Counter(), []
    for c in refsuite.cases(TDIR):
        status, detail = refsuite.run_case(exe, c, TDIR, str(tmp_path))
        counts[status] += 1
        if status in ("differ", "failed"):
            bad.append((c.name, c.source, c.options, detail))
    return counts, bad


def test_runtest_script_expanded():
    cmds = refsuite.runtest_commands(os.path.join(TDIR, "runtest"))
    assert len(cmds) >= 190
    names = {os.path.basename(c[1]) for c in cmds}
    # loop bodies expanded for every value; variables substituted
    for n in ("png-p4t.png", "us-lanczos8.png", "ds-gaussian.png", "dither-sierralite.png", "pam2.pam"):
        assert n in names
    scale = [c for c in cmds if os.path.basename(c[1]) == "cc-6.png"][0]
    assert scale[2:] == ["-zipcmprlevel", "-1", "-width", "35", "-height", "35", "-filter", "catrom", "-cc", "6"]


def test_png_decoder_reads_every_suite_image():
    """Every PNG input and expected file decodes; palette and colour-key
    images come out with an alpha channel where the reference's reader gives
    one."""
    from pngread import read_png
    n = 0
    for sub in ("srcimg", "expected"):
        for name in sorted(os.listdir(os.path.join(TDIR, sub))):
            if name.endswith(".png"):
                g = read_png(os.path.join(TDIR, sub, name))
                assert g.samples.shape == (g.height, g.width, g.channels)
                assert int(g.samples.max(initial=0)) < (1 << g.bit_depth)
                n += 1
    assert n > 150
    s, maxval, _ = refsuite.png_as_read(os.path.join(TDIR, "srcimg", "p4t.png"))
    assert s.shape[-1] == 4 and maxval == 255
    s, maxval, _ = refsuite.png_as_read(os.path.join(TDIR, "srcimg", "g2t.png"))
    assert s.shape[-1] == 2 and maxval == 255 and set(s[..., 1].ravel()) <= {0, 255}
    s, maxval, _ = refsuite.png_as_read(os.path.join(TDIR, "srcimg", "g4.png"))
    assert s.shape[-1] == 1 and maxval == 15


def test_reference_cli_reproduces_its_expected_files(tmp_path):
    exe = _make("refcli", REF_CLI)
    counts, bad = _replay(exe, tmp_path)
    assert not bad, f"{len(bad)} lines differ: {bad[:5]}"
    assert counts["match"] >= MIN_MATCHED, counts


def test_oracle_cli_reproduces_reference_expected_files(tmp_path):
    exe = _make("cli", ORACLE_CLI)
    counts, bad = _replay(exe, tmp_path)
    assert not bad, f"{len(bad)} lines differ: {bad[:5]}"
    assert counts["match"] >= MIN_MATCHED, counts


def _api_lines(lib) -> list:
    import numpy as np
    from imageworsener_gb300.iwapi import run_job
    bad = []
    for name, job in refsuite.api_jobs(TDIR, lib).items():
        r = run_job(lib, job)
        want = refsuite.png_values(os.path.join(TDIR, "expected", name))
        if not r.ok or not np.array_equal(want, refsuite.result_values(r)):
            bad.append((name, r.error))
    return bad


def test_reference_core_reproduces_library_api_lines(reference):
    """The lines a PNM/PAM file cannot carry (per-channel sBIT in and out, the
    input's background label as the background), through the library API:
    the reference core built here reproduces its files, so the jobs are
    faithful."""
    assert not _api_lines(reference)


def test_oracle_reproduces_library_api_lines(oracle):
    assert not _api_lines(oracle)

"""The imagew_gb300 command-line tool (imageworsener_gb300/cli): PNM/PAM files
in and out, options as the reference's imagew.  Output files must be
byte-identical to the reference's.

  * on any machine, the CLI linked against the CPU oracle is checked against
    golden digests of files written by the reference's own imagew
    (tests/golden/cli_cases.json for sizes, filters, depths, dithers and
    crops; tests/golden/cli_cases_ext.json adding relative sizes,
    translation, channel offsets, per-channel depths / colour counts /
    dithers, grayscale formulas, colour spaces, backgrounds, reorientation,
    PBM output and the other switches; tests/golden/make_cli_golden.py), and
    malformed inputs are refused;
  * where the reference sources exist, a further random grid is compared
    with the reference CLI directly;
  * on a GPU, the product build (linked against libimagew_gb300) is checked
    against the same golden digests.
"""
import json
import os
import subprocess

import pytest

import iwcli
from conftest import ROOT, GOLDEN

ORACLE_CLI = os.path.join(ROOT, "oracle", "_build", "imagew_cli_oracle")
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "imagew_ref")
GPU_CLI = os.path.join(ROOT, "imageworsener_gb300", "imagew_gb300")


GOLDEN_FILES = ["cli_cases.json", "cli_cases_ext.json"]


def _golden(name="cli_cases.json"):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def oracle_cli():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "cli"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ORACLE_CLI


@pytest.mark.parametrize("name", GOLDEN_FILES)
def test_cli_oracle_matches_reference_golden(oracle_cli, tmp_path, name):
    bad = []
    cases = _golden(name)
    for c in cases:
        rc, digest = iwcli.run_case(oracle_cli, c, str(tmp_path))
        if (rc == 0) != (c["rc"] == 0) or digest != c["sha256"]:
            bad.append((c["seed"], c["kind"], c["out"], c["args"], rc))
    assert not bad, f"{len(bad)} of {len(cases)} cases differ: {bad[:5]}"


def test_cli_oracle_matches_reference_cli_random(oracle_cli, tmp_path):
    if not os.path.exists(REF_CLI):
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refcli"], capture_output=True, text=True)
        if r.returncode or not os.path.exists(REF_CLI):
            pytest.skip("reference CLI not buildable on this machine")
    bad = []
    for seed in range(1000, 1150):
        c = iwcli.case(seed) if seed % 2 else iwcli.case_ext(seed)
        a = iwcli.run_case(REF_CLI, c, str(tmp_path))
        b = iwcli.run_case(oracle_cli, c, str(tmp_path))
        if (a[0] == 0) != (b[0] == 0) or a[1] != b[1]:
            bad.append((seed, c["kind"], c["out"], c["args"], a[0], b[0]))
    assert not bad, f"{len(bad)} cases differ: {bad[:5]}"


@pytest.mark.parametrize("content", [b"", b"P9\n1 1\n255\n\0", b"P6\n0 5\n255\n", b"P6\n4 4\n70000\n" + b"\0" * 96,
                                     b"P5\n4 4\n255\n\0\0", b"P3\n1 1\n255\n0 0 0\n", b"P7\nWIDTH 2\nHEIGHT 2\nDEPTH 5\nMAXVAL 255\nENDHDR\n" + b"\0" * 20])
def test_cli_refuses_malformed_input(oracle_cli, tmp_path, content):
    inp = tmp_path / "bad.ppm"
    inp.write_bytes(content)
    out = tmp_path / "out.ppm"
    r = subprocess.run([oracle_cli, "-noinfo", "-w", "2", str(inp), str(out)], capture_output=True)
    assert r.returncode != 0
    assert not out.exists()
    assert b"imagew error" in r.stderr


@pytest.mark.parametrize("args", [["-infmt", "ppm"], ["-infmt", "png"], ["-outfmt", "png"], ["-intent", "d"],
                                  ["-cs", "gamma"], ["-gsf", "w1,2"], ["-noopt", "x"], ["-reorient", "spin"],
                                  ["-s", "50"], ["-sampletype", "z"], ["-compress", "x"], ["-density", "x"]])
def test_cli_refuses_like_reference(oracle_cli, tmp_path, args):
    """Option values and format requests the reference's imagew refuses (a
    forced PPM/PGM/PBM input format, other formats, unknown names)."""
    inp = tmp_path / "in.ppm"
    iwcli.write_input(str(inp), "ppm8", 9, 7, 2)
    r = subprocess.run([oracle_cli, "-noinfo", *args, str(inp), str(tmp_path / "out.pam")], capture_output=True)
    assert r.returncode != 0
    assert not (tmp_path / "out.pam").exists()


def test_cli_help_and_version(oracle_cli):
    for opt in ("-help", "-version"):
        r = subprocess.run([oracle_cli, opt], capture_output=True, text=True)
        assert r.returncode == 0 and "imagew" in r.stdout


def test_cli_usage_errors(oracle_cli, tmp_path):
    assert subprocess.run([oracle_cli], capture_output=True).returncode != 0
    assert subprocess.run([oracle_cli, "-filter", "nosuch", "a.ppm", "b.ppm"], capture_output=True).returncode != 0
    inp = tmp_path / "in.ppm"
    iwcli.write_input(str(inp), "ppm8", 8, 8, 1)
    r = subprocess.run([oracle_cli, "-noinfo", str(inp), str(tmp_path / "out.xyz")], capture_output=True)
    assert r.returncode != 0 and b"Unknown output format" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN_FILES)
def test_cli_gpu_matches_reference_golden(gpulib, tmp_path, name):
    """The product build: iw_process_image() on the GPU, same files."""
    assert os.path.exists(GPU_CLI), "imagew_gb300 is built with the library"
    bad = []
    cases = _golden(name)
    for c in cases:
        rc, digest = iwcli.run_case(GPU_CLI, c, str(tmp_path))
        if (rc == 0) != (c["rc"] == 0) or digest != c["sha256"]:
            bad.append((c["seed"], c["kind"], c["out"], c["args"], rc))
    assert not bad, f"{len(bad)} of {len(cases)} cases differ: {bad[:5]}"

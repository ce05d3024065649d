"""The reference's regression suite replayed from committed fixtures
(tests/golden/refsuite*, made by tests/golden/make_refsuite_golden.py from
the reference's tests/runtest, srcimg/ and expected/), so that it runs where
the reference tree is absent -- on the GPU machine in particular:

  * the GPU build's command-line tool (imagew_gb300, linked against
    libimagew_gb300.so) on every replayable line (marker gpu), and the four
    lines that need library calls through the GPU library;
  * the same with the oracle-linked tool and the oracle library on the CPU,
    which checks the fixtures themselves.

Each output is compared with the expected file as exact sample fractions
(SHA-256 of the float64 RGBA values) and, for PNM/PAM outputs, byte for byte.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import refsuite
from conftest import ROOT, GOLDEN
from imageworsener_gb300.iwapi import Job, run_job

FIX = os.path.join(GOLDEN, "refsuite")
ORACLE_CLI = os.path.join(ROOT, "oracle", "_build", "imagew_cli_oracle")


def _load():
    with open(os.path.join(GOLDEN, "refsuite.json")) as f:
        return json.load(f)


def values_digest(v: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(v, dtype="<f8").tobytes() + repr(v.shape).encode()).hexdigest()


def replay(exe: str, tmp) -> tuple[int, list, int]:
    """(lines matched, lines that differ or fail, lines skipped)."""
    matched, bad, skipped = 0, [], 0
    for c in _load()["lines"]:
        out_ext = "pam" if c["ext"] == "png" else c["ext"]
        out = os.path.join(str(tmp), "%s.%s" % (c["name"].rsplit(".", 1)[0], out_ext))
        if os.path.exists(out):
            os.remove(out)
        extra = ["-outfmt", "pam"] if c["ext"] == "png" else []
        r = subprocess.run([exe, "-noinfo", "-nowarn", *c["options"], *extra, os.path.join(FIX, c["input"]), out],
                           capture_output=True, timeout=120)
        if r.returncode or not os.path.exists(out):
            msg = r.stderr.decode(errors="replace").strip()
            if c["ext"] == "png" and "requires equal bit depths" in msg:
                skipped += 1   # per-channel output depths: a PAM file holds one (a library line covers it)
                continue
            bad.append((c["name"], "failed: " + msg[-200:]))
            continue
        if "file_sha256" in c:
            with open(out, "rb") as f:
                if hashlib.sha256(f.read()).hexdigest() != c["file_sha256"]:
                    bad.append((c["name"], "file bytes"))
                    continue
        if values_digest(refsuite.pnm_values(out)) != c["values_sha256"]:
            bad.append((c["name"], "sample values"))
            continue
        matched += 1
    return matched, bad, skipped


def api_replay(lib) -> list:
    data = _load()
    arrays = np.load(os.path.join(GOLDEN, "refsuite_api.npz"))
    bad = []

    def conv(a):
        if isinstance(a, list):
            return tuple(conv(x) for x in a)
        if isinstance(a, dict) and "bytes" in a:
            return a["bytes"].encode()
        return a

    for k, c in enumerate(data["api"]):
        calls = [conv(x) for x in c["calls"]]
        job = Job(c["imgtype"], c["bit_depth"], c["width"], c["height"], arrays[f"in{k}"].tobytes(), calls=calls)
        r = run_job(lib, job)
        if not r.ok or values_digest(refsuite.result_values(r)) != c["values_sha256"]:
            bad.append((c["name"], r.error))
    return bad


def test_fixtures_cover_the_suite():
    data = _load()
    assert len(data["lines"]) >= 156 and len(data["api"]) == 4
    assert all(os.path.exists(os.path.join(FIX, c["input"])) for c in data["lines"])


def test_oracle_cli_replays_fixtures(tmp_path):
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "cli"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    matched, bad, skipped = replay(ORACLE_CLI, tmp_path)
    assert not bad, f"{len(bad)} lines differ: {bad[:6]}"
    assert matched >= 156 and skipped <= 1


def test_oracle_library_replays_fixture_api_lines(oracle):
    assert not api_replay(oracle)


@pytest.mark.gpu
def test_gpu_cli_replays_reference_suite(gpulib, tmp_path):
    """All replayable lines of the reference's regression suite through the
    GPU build's command-line tool: none may differ."""
    from imageworsener_gb300 import build
    exe = build.build_cli()
    matched, bad, skipped = replay(exe, tmp_path)
    assert not bad, f"{len(bad)} lines differ: {bad[:6]}"
    assert matched >= 156 and skipped <= 1


@pytest.mark.gpu
def test_gpu_library_replays_fixture_api_lines(gpulib):
    assert not api_replay(gpulib)

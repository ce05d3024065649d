"""Generates tests/golden/refsuite/ and tests/golden/refsuite.json: the
reference's own regression suite (its tests/runtest lines with PNG or PNM/PAM
input and output, inputs from tests/srcimg, outputs from tests/expected) in a
form that travels without the reference tree, so the GPU build's
command-line tool can replay it on any machine.

For every replayable line (tests/refsuite.py decides which, and how):
  * the input as the PNM/PAM file the tool reads (a PNG input decoded the
    way the reference's PNG reader hands it over; one file per source image);
  * the options (with the exact size for non-square pixel densities);
  * the SHA-256 of the expected output's exact sample fractions
    (refsuite.expected_values: float64, RGBA) and, for PNM/PAM outputs, of
    the expected file's bytes.
The four lines that need library calls a PNM/PAM file cannot carry are kept
as library jobs (raw input samples in refsuite_api.npz, calls in the JSON).

    python tests/golden/make_refsuite_golden.py    (needs the reference tree)
"""
import hashlib
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import refsuite  # noqa: E402

OUT_DIR = os.path.join(HERE, "refsuite")


def values_digest(v: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(v, dtype="<f8").tobytes() + repr(v.shape).encode()).hexdigest()


def _jsonable(a):
    if isinstance(a, (list, tuple)):
        return [_jsonable(x) for x in a]
    if isinstance(a, bytes):
        return {"bytes": a.decode()}
    if isinstance(a, (np.integer,)):
        return int(a)
    if isinstance(a, (np.floating,)):
        return float(a)
    return a


if __name__ == "__main__":
    tdir = refsuite.reference_tests_dir()
    if tdir is None:
        sys.exit("the reference's tests/ folder was not found (REFSRC / oracle/Makefile)")
    from imageworsener_gb300.iwapi import IWLib
    oracle_so = os.path.join(ROOT, "oracle", "_build", "liboracle_iw.so")
    if not os.path.exists(oracle_so):
        sys.exit("build the oracle first: make -C oracle port")
    if os.path.isdir(OUT_DIR):
        shutil.rmtree(OUT_DIR)
    os.makedirs(OUT_DIR)
    lines, skipped = [], {}
    with tempfile.TemporaryDirectory() as tmp:
        for c in refsuite.cases(tdir):
            if c.skip:
                skipped[c.name] = c.skip
                continue
            try:
                inp, opts = refsuite.prepare_input(c, tdir, tmp)
            except refsuite.Unsupported as e:
                skipped[c.name] = str(e)
                continue
            base = os.path.splitext(os.path.basename(c.source))[0] + os.path.splitext(inp)[1]
            dst = os.path.join(OUT_DIR, base)
            if os.path.exists(dst):
                with open(dst, "rb") as f1, open(inp, "rb") as f2:
                    assert f1.read() == f2.read(), base
            else:
                shutil.copyfile(inp, dst)
            entry = {"name": c.name, "input": base, "options": list(opts), "ext": c.ext,
                     "values_sha256": values_digest(refsuite.expected_values(c, tdir))}
            if c.ext != "png":
                with open(os.path.join(tdir, "expected", c.name), "rb") as f:
                    entry["file_sha256"] = hashlib.sha256(f.read()).hexdigest()
            lines.append(entry)
    api = []
    arrays = {}
    for k, (name, job) in enumerate(sorted(refsuite.api_jobs(tdir, IWLib(oracle_so)).items())):
        arrays[f"in{k}"] = np.frombuffer(job.pixels, np.uint8)
        want = refsuite.png_values(os.path.join(tdir, "expected", name))
        api.append({"name": name, "imgtype": job.imgtype, "bit_depth": job.bit_depth, "width": job.width,
                    "height": job.height, "calls": _jsonable(list(job.calls)), "values_sha256": values_digest(want)})
    np.savez_compressed(os.path.join(HERE, "refsuite_api.npz"), **arrays)
    with open(os.path.join(HERE, "refsuite.json"), "w") as f:
        json.dump({"lines": lines, "api": api, "skipped": skipped}, f, indent=0)
    size = sum(os.path.getsize(os.path.join(OUT_DIR, n)) for n in os.listdir(OUT_DIR))
    print(f"{len(lines)} tool lines, {len(api)} library lines, {len(skipped)} skipped; "
          f"{len(os.listdir(OUT_DIR))} input files, {size} bytes")
